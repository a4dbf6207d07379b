/*
 * visor_spirv.h - SPIR-V 1.0 modules for the scenes' shader pairs.
 *
 * No GLSL front end exists on this toolchain, so the project emits the
 * configurations' shaders directly as SPIR-V words, in the form a GLSL 450
 * compiler produces for them (gl_PerVertex output block, push-constant block
 * with ColMajor/MatrixStride/Offset member decorations, combined image
 * sampler at set 0 binding 0), restricted to the opcodes the reference's
 * compiler handles (spirv_compile.cpp:1037-1892).
 */
#ifndef VISOR_SPIRV_H
#define VISOR_SPIRV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

enum { VSPV_STAGE_VERTEX = 0, VSPV_STAGE_FRAGMENT = 4 };

/*
 * Emit the module of one stage of a VSC_SHADER_* pair.  Returns the number of
 * 32-bit words written (the full length when `words` is NULL or `capacity` is
 * too small, so callers can size the buffer), or 0 for an unknown shader.
 */
size_t vspv_emit(uint32_t shader, uint32_t stage, uint32_t *words, size_t capacity);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif
