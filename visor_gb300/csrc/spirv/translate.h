/*
 * SPIR-V -> CUDA C++ translator (replaces the reference's SPIR-V -> LLVM JIT,
 * spirv_compile.cpp:645-2432).
 *
 * vkCreateShaderModule parses a module (vst_parse); vkCreateGraphicsPipelines
 * translates a vertex/fragment pair into CUDA device code (vst_translate) that
 * NVRTC compiles together with the stage kernels.  The generated code keeps the
 * reference JIT's operation order for every op it lowers (CreateDot for dot
 * products and interpolation, 0.0f-seeded matrix products, select-based
 * FMax/FMin/FClamp, a*(1/sqrt(dot)) for Normalize) so results are bit-identical
 * to the reference's CPU path; ops the reference lowers incorrectly
 * (ShiftLeftLogical, Cross, MatrixInverse) get their SPIR-V meaning.
 */
#ifndef VISOR_SPIRV_TRANSLATE_H
#define VISOR_SPIRV_TRANSLATE_H

#include <stdint.h>

#include <string>
#include <vector>

namespace vst
{
struct Module;

/* Parse and validate a module; returns nullptr and sets err on failure. */
Module *parse(const uint32_t *words, size_t count, std::string &err);
void destroy(Module *m);
/* execution model of the named entry point (0 vertex, 4 fragment, -1 missing) */
int entry_model(const Module *m, const char *name);

struct Binding
{
  uint32_t set, binding;
};

struct Result
{
  std::string source;            /* CUDA C++ defining VGX_K, VGX_LOD_SLOT, VGX_LOD_TEX, vgx_vs, vgx_fs */
  std::vector<Binding> textures; /* VgxDraw::tex[i] <- (set, binding) */
  std::vector<Binding> ubos;     /* VgxDraw::ubo[i] <- (set, binding) */
  uint32_t k = 0;                /* interpolated float slots */
  int lod_slot = -1;
};

bool translate(const Module *vs, const char *vs_entry, const Module *fs, const char *fs_entry,
               Result &out, std::string &err);
}    // namespace vst

#endif
