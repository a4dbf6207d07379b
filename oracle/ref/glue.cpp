/*
 * Glue that turns the reference's own CPU draw path (compiled unmodified from
 * its sources by oracle/Makefile) into a callable oracle.  TEST INFRASTRUCTURE.
 *
 * The reference JIT-compiles SPIR-V with LLVM 6 (spirv_compile.cpp), which is
 * not buildable here.  This file provides the five functions of
 * spirv_compile.h instead: CompileFunction recognises the project's emitted
 * modules by their OpSourceExtension tag and GetFuncPointer returns C++
 * restatements of those shaders with the reference's VertexShader /
 * FragmentShader signatures (precompiled.h:52-55).  The restatements follow
 * the reference JIT's lowering order (spirv_compile.cpp:423-431, 572-627,
 * 629-643, 1470-1476, 1535-1545, 1635-1647, 2179-2224); texture sampling goes
 * through the reference's real sample_tex_wrapped.
 *
 * wsi.cpp calls Win32 GDI and is not built; its entry points, referenced by
 * the ICD tables in icd_interface.cpp, are stubbed here.
 */
#include "precompiled.h"

#include <chrono>
#include <string>

#include "gpu.h"
#include "spirv_compile.h"
#include "visor_driver.h"
#include "visor_scene.h"

/* ---- counters fed by the shim's MICROPROFILE_COUNTER_ADD ---------------- */

static std::atomic<long long> g_counters[6];

extern "C" void visor_ref_counter_add(const char *name, long long count)
{
  /* rasterizer/triangles/in|out, pixels/tested|written, depth/passed, draws/in */
  if(name[0] != 'r')
    return;
  const char *n = name + 11;
  int idx = -1;
  if(!strcmp(n, "triangles/in")) idx = 0;
  else if(!strcmp(n, "triangles/out")) idx = 1;
  else if(!strcmp(n, "pixels/tested")) idx = 2;
  else if(!strcmp(n, "pixels/written")) idx = 3;
  else if(!strcmp(n, "depth/passed")) idx = 4;
  else if(!strcmp(n, "draws/in")) idx = 5;
  if(idx >= 0)
    g_counters[idx] += count;
}

/* ---- shader runtime helpers (restated: they live in the LLVM TU) -------- */

/* Attribute fetch with the semantics of GetVertexAttributeData, spirv_compile.cpp:572-627 */
static float4 attr_fetch(const GPUState &state, uint32_t vertexIndex, uint32_t loc)
{
  float4 out(0.0f, 0.0f, 0.0f, 1.0f);
  const auto &a = state.pipeline->vattrs[loc];
  const byte *ptr = state.vbs[a.vb].buffer->bytes + state.vbs[a.vb].offset + a.offset +
                    (VkDeviceSize)a.stride * vertexIndex;
  float f[4];
  uint32_t u;
  switch(a.format)
  {
    case VK_FORMAT_R32G32B32A32_SFLOAT: memcpy(f, ptr, 16); out.w = f[3]; /* fall through */
    case VK_FORMAT_R32G32B32_SFLOAT: memcpy(f, ptr, 12); out.z = f[2];    /* fall through */
    case VK_FORMAT_R32G32_SFLOAT: memcpy(f, ptr, 8); out.y = f[1];        /* fall through */
    case VK_FORMAT_R32_SFLOAT: memcpy(f, ptr, 4); out.x = f[0]; break;
    case VK_FORMAT_R8G8B8A8_UNORM:
      memcpy(&u, ptr, 4);
      out.x = float((u & 0x000000ff) >> 0) / 255.0f;
      out.y = float((u & 0x0000ff00) >> 8) / 255.0f;
      out.z = float((u & 0x00ff0000) >> 16) / 255.0f;
      out.w = float((u & 0xff000000) >> 24) / 255.0f;
      break;
    default: break;
  }
  return out;
}

/* column-major mat4 * vec4 accumulated from 0.0f, as Float4x4TimesVec4 (:423-431) */
static float4 mat_vec(const float *m, const float4 &v)
{
  float4 out;
  for(int r = 0; r < 4; r++)
  {
    out.v[r] = 0.0f;
    for(int c = 0; c < 4; c++)
      out.v[r] = out.v[r] + m[c * 4 + r] * v.v[c];
  }
  return out;
}

/* four-lane CreateDot of the barycentrics with (v0, v1, v2, 0) (:629-643, :2200-2214) */
static float bary_dot(const float4 &b, float a0, float a1, float a2)
{
  float acc = b.x * a0;
  acc = acc + b.y * a1;
  acc = acc + b.z * a2;
  acc = acc + b.w * 0.0f;
  return acc;
}

static void vs_lambert_impl(const GPUState &state, uint32_t idx, VertexCacheEntry &out, bool alpha)
{
  float mvp[16];
  memcpy(mvp, state.pushconsts + 0, 64);
  float4 pos = attr_fetch(state, idx, 0);
  float4 nrm = attr_fetch(state, idx, 1);
  float4 uv = attr_fetch(state, idx, 2);
  out.position = mat_vec(mvp, float4(pos.x, pos.y, pos.z, 1.0f));
  out.interps[0] = float4(nrm.x, nrm.y, nrm.z, nrm.x);
  out.interps[1] = float4(uv.x, uv.y, uv.x, uv.x);
  if(alpha)
  {
    float4 a = attr_fetch(state, idx, 3);
    out.interps[2] = float4(a.x, a.x, a.x, a.x);
  }
}

static void vs_lambert(const GPUState &s, uint32_t i, VertexCacheEntry &o) { vs_lambert_impl(s, i, o, false); }
static void vs_lambert_alpha(const GPUState &s, uint32_t i, VertexCacheEntry &o) { vs_lambert_impl(s, i, o, true); }

static void vs_color(const GPUState &state, uint32_t idx, VertexCacheEntry &out)
{
  out.position = attr_fetch(state, idx, 0);
  out.interps[0] = attr_fetch(state, idx, 1);
}

static void fs_lambert_impl(const GPUState &state, const float4 &bary, const VertexCacheEntry tri[3],
                            float4 &out, bool alpha)
{
  float n[3], uv[2];
  for(int i = 0; i < 3; i++)
    n[i] = bary_dot(bary, tri[0].interps[0].v[i], tri[1].interps[0].v[i], tri[2].interps[0].v[i]);
  for(int i = 0; i < 2; i++)
    uv[i] = bary_dot(bary, tri[0].interps[1].v[i], tri[1].interps[1].v[i], tri[2].interps[1].v[i]);
  /* Normalize: a * (1 / sqrt(dot(a, a))), :1635-1647 */
  float sq = n[0] * n[0];
  sq = sq + n[1] * n[1];
  sq = sq + n[2] * n[2];
  float inv = 1.0f / sqrtf(sq);
  float nn[3] = {n[0] * inv, n[1] * inv, n[2] * inv};
  float light[4];
  memcpy(light, state.pushconsts + 64, 16);
  float d = nn[0] * light[0];
  d = d + nn[1] * light[1];
  d = d + nn[2] * light[2];
  float lam = d > 0.0f ? d : 0.0f; /* FMax: select(a > b, a, b), :1535-1545 */
  /* ImageSampleImplicitLod -> GetDescriptorImage(set 0, binding 0) -> sample_tex_wrapped (:1842-1886, :560-564) */
  VkImage img = state.sets[0]->binds[0].data.imageInfo.imageView->image;
  float4 t;
  sample_tex_wrapped(uv[0], uv[1], img, 0, t);
  if(!alpha)
  {
    out = float4(t.x * lam, t.y * lam, t.z * lam, t.w * lam);
  }
  else
  {
    float a = bary_dot(bary, tri[0].interps[2].x, tri[1].interps[2].x, tri[2].interps[2].x);
    out = float4(t.x * lam, t.y * lam, t.z * lam, a);
  }
}

static void fs_lambert(const GPUState &s, float, const float4 &b, const VertexCacheEntry tri[3], float4 &o)
{
  fs_lambert_impl(s, b, tri, o, false);
}
static void fs_lambert_alpha(const GPUState &s, float, const float4 &b, const VertexCacheEntry tri[3], float4 &o)
{
  fs_lambert_impl(s, b, tri, o, true);
}
/* samplerCube at the interpolated normal: ImageSampleImplicitLod on a Dim=Cube image
   lowers to sample_cube_wrapped (spirv_compile.cpp:1842-1886, 896) */
extern "C" void sample_cube_wrapped(float x, float y, float z, VkImage tex, float4 &out);
static void fs_cube(const GPUState &state, float, const float4 &b, const VertexCacheEntry tri[3], float4 &o)
{
  float n[3];
  for(int i = 0; i < 3; i++)
    n[i] = bary_dot(b, tri[0].interps[0].v[i], tri[1].interps[0].v[i], tri[2].interps[0].v[i]);
  VkImage img = state.sets[0]->binds[0].data.imageInfo.imageView->image;
  sample_cube_wrapped(n[0], n[1], n[2], img, o);
}
static void fs_color(const GPUState &, float, const float4 &b, const VertexCacheEntry tri[3], float4 &o)
{
  for(int i = 0; i < 4; i++)
    o.v[i] = bary_dot(b, tri[0].interps[0].v[i], tri[1].interps[0].v[i], tri[2].interps[0].v[i]);
}

/* ---- spirv_compile.h replacement ----------------------------------------- */

struct LLVMFunction
{
  Shader fn;
};

void InitLLVM() {}
void ShutdownLLVM() {}

LLVMFunction *CompileFunction(const uint32_t *pCode, size_t codeSize)
{
  static const struct
  {
    const char *tag;
    Shader fn;
  } table[] = {
      {"visor_shader:lambert_tex.vert", (Shader)&vs_lambert},
      {"visor_shader:lambert_tex.frag", (Shader)&fs_lambert},
      {"visor_shader:lambert_tex_alpha.vert", (Shader)&vs_lambert_alpha},
      {"visor_shader:lambert_tex_alpha.frag", (Shader)&fs_lambert_alpha},
      {"visor_shader:color.vert", (Shader)&vs_color},
      {"visor_shader:color.frag", (Shader)&fs_color},
      {"visor_shader:cube.frag", (Shader)&fs_cube},
  };
  size_t i = 5;
  while(i < codeSize)
  {
    uint32_t op = pCode[i] & 0xffff, wc = pCode[i] >> 16;
    if(wc == 0)
      break;
    if(op == 4 /* OpSourceExtension */)
    {
      const char *s = (const char *)&pCode[i + 1];
      for(const auto &e : table)
        if(!strcmp(s, e.tag))
          return new LLVMFunction{e.fn};
    }
    i += wc;
  }
  return NULL;
}

Shader GetFuncPointer(LLVMFunction *func, const char *) { return func ? func->fn : NULL; }
void DestroyFunction(LLVMFunction *func) { delete func; }

/* ---- wsi.cpp entry points (Win32-only in the reference) ------------------ */

VKAPI_ATTR VkResult VKAPI_CALL vkGetPhysicalDeviceSurfaceSupportKHR(VkPhysicalDevice, uint32_t, VkSurfaceKHR, VkBool32 *s)
{
  *s = VK_FALSE;
  return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL vkGetPhysicalDeviceSurfaceFormatsKHR(VkPhysicalDevice, VkSurfaceKHR, uint32_t *n, VkSurfaceFormatKHR *)
{
  *n = 0;
  return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL vkGetPhysicalDeviceSurfaceCapabilitiesKHR(VkPhysicalDevice, VkSurfaceKHR, VkSurfaceCapabilitiesKHR *)
{
  return VK_ERROR_EXTENSION_NOT_PRESENT;
}
VKAPI_ATTR VkResult VKAPI_CALL vkGetPhysicalDeviceSurfacePresentModesKHR(VkPhysicalDevice, VkSurfaceKHR, uint32_t *n, VkPresentModeKHR *)
{
  *n = 0;
  return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL vkCreateSwapchainKHR(VkDevice, const VkSwapchainCreateInfoKHR *, const VkAllocationCallbacks *, VkSwapchainKHR *)
{
  return VK_ERROR_EXTENSION_NOT_PRESENT;
}
VKAPI_ATTR void VKAPI_CALL vkDestroySwapchainKHR(VkDevice, VkSwapchainKHR, const VkAllocationCallbacks *) {}
VKAPI_ATTR VkResult VKAPI_CALL vkGetSwapchainImagesKHR(VkDevice, VkSwapchainKHR, uint32_t *n, VkImage *)
{
  *n = 0;
  return VK_SUCCESS;
}
VKAPI_ATTR VkResult VKAPI_CALL vkAcquireNextImageKHR(VkDevice, VkSwapchainKHR, uint64_t, VkSemaphore, VkFence, uint32_t *)
{
  return VK_ERROR_EXTENSION_NOT_PRESENT;
}
VKAPI_ATTR VkResult VKAPI_CALL vkQueuePresentKHR(VkQueue, const VkPresentInfoKHR *)
{
  return VK_ERROR_EXTENSION_NOT_PRESENT;
}

/* ---- C entry points for the tests ---------------------------------------- */

extern "C" VKAPI_ATTR PFN_vkVoidFunction VKAPI_CALL vk_icdGetInstanceProcAddr(VkInstance instance,
                                                                              const char *pName);

/*
 * InitTextureCache (texture_sampling.cpp:19-32) relinks the thread's LRU list
 * but does not reset tcache_data[0].prev or tcache_data[7].next, so a second
 * call on the same thread can leave a cycle that CacheCoord walks forever.
 * Call it at most once per thread.  For the same reason the threaded mode
 * (vkCreateInstance -> InitRasterThreads -> InitTextureCache) must run in a
 * process that has not used the serial mode.
 */
static void init_texture_cache_once()
{
  static thread_local bool done = false;
  if(!done)
  {
    InitTextureCache();
    done = true;
  }
}

/*
 * Render a scene through the reference ICD's Vulkan entry points.
 * threaded = 0: serial FIFO oracle mode (no raster threads, main-thread texture cache).
 * threaded = 1: the reference as shipped (vkCreateInstance starts 7 raster threads).
 * counters (6): tris_in, tris_out, tested, covered, shaded, draws.
 * submit_seconds: wall time of vkQueueSubmit (after uploads and pipeline creation).
 */
extern "C" __attribute__((visibility("default"))) int visor_ref_render(
    const vsc_scene *scene, uint8_t **colors, float **depths, long long *counters, int threaded,
    double *submit_seconds)
{
  for(auto &c : g_counters)
    c = 0;
  void *inst = NULL;
  if(!threaded)
  {
    VK_LOADER_DATA *i = new VK_LOADER_DATA;
    set_loader_magic_value(i);
    init_texture_cache_once();
    inst = i;
  }
  vsd_context *ctx = NULL;
  int rc = vsd_create((vsd_get_proc_fn)&vk_icdGetInstanceProcAddr, inst, &ctx);
  if(rc)
    return rc;
  vsd_scene *s = NULL;
  rc = vsd_upload(ctx, scene, 0, &s);
  if(rc)
    return rc;
  for(auto &c : g_counters)
    c = 0;
  auto t0 = std::chrono::steady_clock::now();
  rc = vsd_submit(s);
  auto t1 = std::chrono::steady_clock::now();
  if(submit_seconds)
    *submit_seconds = std::chrono::duration<double>(t1 - t0).count();
  if(rc)
    return rc;
  for(uint32_t t = 0; t < scene->num_targets; t++)
    if(colors && colors[t])
      vsd_read_target(s, t, colors[t], depths ? depths[t] : NULL);
  if(counters)
    for(int i = 0; i < 6; i++)
      counters[i] = g_counters[i];
  vsd_release(s);
  vsd_destroy(ctx);
  if(!threaded)
    delete(VK_LOADER_DATA *)inst;
  return 0;
}

/*
 * Time `steps` submissions of the scene's command buffer (after one untimed
 * warm-up submission) inside one instance.  The reference's raster threads are
 * started by vkCreateInstance and cannot be restarted in the same process
 * after vkDestroyInstance (rasterizer.cpp:86-98 leaves kill set), so the
 * threaded mode is timed in one instance lifetime per process.
 */
extern "C" __attribute__((visibility("default"))) int visor_ref_time(const vsc_scene *scene,
                                                                     int threaded, int steps,
                                                                     double *seconds)
{
  void *inst = NULL;
  if(!threaded)
  {
    VK_LOADER_DATA *i = new VK_LOADER_DATA;
    set_loader_magic_value(i);
    init_texture_cache_once();
    inst = i;
  }
  vsd_context *ctx = NULL;
  int rc = vsd_create((vsd_get_proc_fn)&vk_icdGetInstanceProcAddr, inst, &ctx);
  if(rc)
    return rc;
  vsd_scene *s = NULL;
  rc = vsd_upload(ctx, scene, 0, &s);
  if(rc)
    return rc;
  rc = vsd_submit(s);
  for(int k = 0; k < steps && !rc; k++)
  {
    auto t0 = std::chrono::steady_clock::now();
    rc = vsd_submit(s);
    auto t1 = std::chrono::steady_clock::now();
    seconds[k] = std::chrono::duration<double>(t1 - t0).count();
  }
  vsd_release(s);
  vsd_destroy(ctx);
  if(!threaded)
    delete(VK_LOADER_DATA *)inst;
  return rc;
}
