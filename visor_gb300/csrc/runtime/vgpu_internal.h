/*
 * vgpu_internal.h - library-internal runtime entry points (not exported) used
 * by the serving engine: command lists whose device storage is stream-ordered
 * from a memory pool, and a submission split at the point where the host
 * needs the pair totals.
 */
#ifndef VGPU_INTERNAL_H
#define VGPU_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#include "visor_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Build a list (no copy commands) with its device buffers allocated from
   `pool` (cudaMemPool_t) in order on `stream` (cudaStream_t); pair totals land
   in the caller's pinned h_totals (at least one word per job). */
int vgpu_list_build_pooled(vgpu_list *l, void *pool, void *stream, uint32_t *h_totals,
                           size_t h_totals_cap);
/* Destroy a pooled list; its device buffers are freed in order on its stream. */
void vgpu_list_destroy_pooled(vgpu_list *l);
/* Uploads, triangle setup and tile-count scans of every job; queues the copy of
   the pair totals to the host.  Returns without waiting. */
int vgpu_list_phase_a(vgpu_queue *q, vgpu_list *l);
/* After phase A has completed on the device: size the binning storage, then
   clears, binning, raster and downloads.  Returns without waiting. */
int vgpu_list_phase_b(vgpu_queue *q, vgpu_list *l);
/* Grow the queue's binning storage to hold `pairs` tile pairs and `tiles` bin tiles. */
int vgpu_queue_reserve_binning(vgpu_queue *q, uint64_t pairs, uint32_t tiles);
/* CUDA device ordinal the runtime uses. */
int vgpu_device_ordinal(void);
/* Bytes of binning storage the queue holds (pairs, sort, tile ranges, scratch). */
uint64_t vgpu_queue_binning_bytes(const vgpu_queue *q);
/* Bin tiles the queue's tile arrays hold (16 bytes each). */
uint32_t vgpu_queue_tile_capacity(const vgpu_queue *q);

#ifdef __cplusplus
}
#endif

#endif
