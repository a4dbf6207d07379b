/*
 * vgpu_noalloc.h - library-internal declaration of the allocation-free submit
 * (not exported; the ICD wraps it as visor_gb300_queue_submit_noalloc).
 */
#ifndef VGPU_NOALLOC_H
#define VGPU_NOALLOC_H

#include "visor_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * vgpu_submit with every per-call binning buffer (tile pairs, sort ping-pong,
 * tile ranges, histograms) in one fixed device array instead of queue memory
 * that grows on demand.  Makes no device allocation.  Needs a list that
 * vgpu_submit has built once; a job over 1,048,576 tile pairs or 131,072 bin
 * tiles is rejected with VGPU_ERROR_OUT_OF_DEVICE_MEMORY.  The array is shared:
 * calls that overlap in time, on any queue, race.
 */
int vgpu_submit_noalloc(vgpu_queue *q, vgpu_list *l);

#ifdef __cplusplus
}
#endif

#endif
