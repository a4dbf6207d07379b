/*
 * Force-included portability shim for building the reference's CPU draw path
 * (baldurk/visor, written for MSVC) with g++ on Linux.  TEST INFRASTRUCTURE:
 * it lets oracle/Makefile compile the reference's unmodified sources.
 *
 * - MSVC __declspec spellings map to GCC attributes.
 * - abs(float) resolves to the float overload, as with MSVC's headers.
 * - sprintf_s(char (&)[N], ...) forwards to snprintf.
 * - BC4Mode/BC5Mode are declared before decompress.h uses them.
 * - microprofile.h is skipped (MICROPROFILE_ONCE) and its macros are given
 *   here: scopes compile out, counters feed visor_ref_counter_add so the
 *   oracle can read the reference's own rasterizer/* counters.
 */
#pragma once

#ifdef __cplusplus
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

/* MSVC's headers give the global abs() float overloads (the reference calls
   abs(float) in sample_cube_wrapped, texture_sampling.cpp:189-191); with
   libstdc++ the global abs is the int one unless std::abs is brought in. */
using std::abs;

template <size_t N, typename... Args>
int sprintf_s(char (&buf)[N], const char *fmt, Args... args)
{
  return snprintf(buf, N, fmt, args...);
}

enum BC4Mode
{
  BC4_UNORM = 0,
  BC4_SNORM = 1
};
enum BC5Mode
{
  BC5_UNORM = 0,
  BC5_SNORM = 1
};
extern "C" void visor_ref_counter_add(const char *name, long long count);
#else
void visor_ref_counter_add(const char *name, long long count);
#endif

#define __declspec(x) __declspec_##x
#define __declspec_align(n) __attribute__((aligned(n)))
#define __declspec_thread thread_local
#define __declspec_dllexport __attribute__((visibility("default")))

#define MICROPROFILE_ENABLED 0
#define MICROPROFILE_ONCE 1
#define MICROPROFILE_DECLARE(var)
#define MICROPROFILE_DEFINE(var, group, name, color)
#define MICROPROFILE_SCOPE(var) do {} while(0)
#define MICROPROFILE_SCOPEI(group, name, color) do {} while(0)
#define MICROPROFILE_COUNTER_SET(name, count) do {} while(0)
#ifdef VISOR_REF_NO_COUNTERS
#define MICROPROFILE_COUNTER_ADD(name, count) do {} while(0)
#else
#define MICROPROFILE_COUNTER_ADD(name, count) visor_ref_counter_add(name, count)
#endif
#define MicroProfileOnThreadCreate(name) do {} while(0)
#define MicroProfileFlip(ctx) do {} while(0)
#define MicroProfileShutdown() do {} while(0)
