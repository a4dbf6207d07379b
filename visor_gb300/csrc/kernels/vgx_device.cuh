/*
 * vgx_device.cuh - device-side runtime helpers the translated shaders call.
 *
 * Compiled by NVRTC together with the shaders of a pipeline (see
 * vgx_stage.cuh) with --fmad=false: every float expression below keeps the
 * reference's binary32 operation order, which is what makes the results
 * bit-identical to the reference's CPU draw path.
 */
#ifndef VGX_DEVICE_CUH
#define VGX_DEVICE_CUH

/* float(byte) / 255.0f for every byte value, filled by each block's prologue. */
__shared__ float vgx_unorm8[256];

__device__ __forceinline__ void vgx_init_unorm8()
{
  for(u32 i = threadIdx.x; i < 256; i += blockDim.x)
    vgx_unorm8[i] = __fdiv_rn((float)i, 255.0f);
}

/*
 * Vertex attribute fetch with the semantics of GetVertexAttributeData
 * (spirv_compile.cpp:572-627): default (0,0,0,1); 32-bit formats copy as many
 * lanes as they have; RGBA8 UNORM decodes byte/255.  Reads outside the bound
 * buffer return the default instead of faulting.
 */
__device__ __forceinline__ float4 vgx_fetch(const VgxDraw &D, u32 loc, u32 index)
{
  float4 out = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
  if(loc >= VGX_MAX_ATTRS)
    return out;
  const VgxAttr a = D.attrs[loc];
  if(a.format == VGX_FMT_NONE || a.binding >= VGX_MAX_VB)
    return out;
  u64 off = (u64)a.offset + (u64)a.stride * (u64)index;
  u32 size = a.format == VGX_FMT_RGBA32 ? 16u : a.format == VGX_FMT_RGB32 ? 12u
             : a.format == VGX_FMT_RG32 ? 8u : 4u;
  if(off + size > D.vb_bytes[a.binding])
    return out;
  const u32 *p = (const u32 *)(D.vb[a.binding] + off);
  switch(a.format)
  {
    case VGX_FMT_RGBA32: out.w = __uint_as_float(__ldg(p + 3)); /* fall through */
    case VGX_FMT_RGB32: out.z = __uint_as_float(__ldg(p + 2));  /* fall through */
    case VGX_FMT_RG32: out.y = __uint_as_float(__ldg(p + 1));   /* fall through */
    case VGX_FMT_R32: out.x = __uint_as_float(__ldg(p + 0)); break;
    case VGX_FMT_RGBA8_UNORM:
    {
      u32 u = __ldg(p);
      out.x = vgx_unorm8[u & 0xffu];
      out.y = vgx_unorm8[(u >> 8) & 0xffu];
      out.z = vgx_unorm8[(u >> 16) & 0xffu];
      out.w = vgx_unorm8[u >> 24];
      break;
    }
    default: break;
  }
  return out;
}

__device__ __forceinline__ float4 vgx_texel(const u8 *base, u32 width, int x, int y)
{
  u32 t = __ldg((const u32 *)(base + ((u64)y * width + (u32)x) * 4u));
  return make_float4(vgx_unorm8[t & 0xffu], vgx_unorm8[(t >> 8) & 0xffu],
                     vgx_unorm8[(t >> 16) & 0xffu], vgx_unorm8[t >> 24]);
}

/*
 * Bilinear, repeat, no half-texel offset: sample_tex_wrapped
 * (texture_sampling.cpp:139-184) in its exact operation order.  Where
 * u - floor(u) rounds to 1.0 the reference reads past the row; this path (and
 * the oracle) wraps that texel.  Indices are clamped so NaN/inf coordinates
 * cannot address outside the image.
 */
__device__ __forceinline__ float4 vgx_bilinear(const u8 *base, u32 W, u32 H, float u, float v)
{
  u = u - floorf(u);
  v = v - floorf(v);
  u = u * (float)W;
  v = v * (float)H;
  int iu0 = (int)u;
  int iv0 = (int)v;
  int iu1 = iu0 + 1;
  int iv1 = iv0 + 1;
  if(iu1 >= (int)W)
    iu1 -= W;
  if(iv1 >= (int)H)
    iv1 -= H;
  float fu = u - (float)iu0;
  float fv = v - (float)iv0;
  float inv_fu = 1.0f - fu;
  float inv_fv = 1.0f - fv;
  if(iu0 >= (int)W)
    iu0 -= W;
  if(iv0 >= (int)H)
    iv0 -= H;
  iu0 = min(max(iu0, 0), (int)W - 1);
  iv0 = min(max(iv0, 0), (int)H - 1);
  iu1 = min(max(iu1, 0), (int)W - 1);
  iv1 = min(max(iv1, 0), (int)H - 1);
  float4 TL = vgx_texel(base, W, iu0, iv0);
  float4 TR = vgx_texel(base, W, iu1, iv0);
  float4 BL = vgx_texel(base, W, iu0, iv1);
  float4 BR = vgx_texel(base, W, iu1, iv1);
  float4 top, bottom, out;
  top.x = TL.x * inv_fu + TR.x * fu;
  top.y = TL.y * inv_fu + TR.y * fu;
  top.z = TL.z * inv_fu + TR.z * fu;
  top.w = TL.w * inv_fu + TR.w * fu;
  bottom.x = BL.x * inv_fu + BR.x * fu;
  bottom.y = BL.y * inv_fu + BR.y * fu;
  bottom.z = BL.z * inv_fu + BR.z * fu;
  bottom.w = BL.w * inv_fu + BR.w * fu;
  out.x = top.x * inv_fv + bottom.x * fv;
  out.y = top.y * inv_fv + bottom.y * fv;
  out.z = top.z * inv_fv + bottom.z * fv;
  out.w = top.w * inv_fv + bottom.w * fv;
  return out;
}

/* Project specification (no reference counterpart): log2 from the exponent
   bits and 2/ln2 * (s + s^3/3 + s^5/5), s = (m-1)/(m+1); same order as the oracle. */
__device__ __forceinline__ float vgx_log2(float x)
{
  if(!(x > 0.0f))
    return -128.0f;
  if(x > 3.0e38f)
    return 128.0f;
  u32 bits = __float_as_uint(x);
  int e = (int)((bits >> 23) & 0xffu) - 127;
  float m = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float poly = s + s * s2 * (1.0f / 3.0f) + s * s2 * s2 * 0.2f;
  return (float)e + poly * 2.88539008f;
}

/* Project specification: per-triangle LOD from uv area (mip 0 texels) over the doubled pixel area. */
__device__ __forceinline__ float vgx_lod(float u0, float v0, float u1, float v1, float u2, float v2,
                                         u32 width, u32 height, int area2)
{
  float du1 = u1 - u0, dv1 = v1 - v0, du2 = u2 - u0, dv2 = v2 - v0;
  float cr = du1 * dv2 - du2 * dv1;
  float auv = fabsf(cr) * (float)width * (float)height;
  float apx = (float)(area2 < 0 ? -area2 : area2);
  return 0.5f * vgx_log2(auv / apx);
}

__device__ __forceinline__ float4 vgx_sample(const VgxDraw &D, u32 slot, float u, float v, float lod)
{
  if(slot >= VGX_MAX_TEX || D.tex[slot].base == 0)
    return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const VgxTex &t = D.tex[slot];
  const u8 *base = (const u8 *)t.base;
  if(t.filter == VGX_FILTER_TRILINEAR && t.mips > 1)
  {
    float maxl = (float)(t.mips - 1);
    if(!(lod > 0.0f))
      lod = 0.0f;
    if(lod > maxl)
      lod = maxl;
    int l0 = (int)lod;
    float f = lod - (float)l0;
    int l1 = l0 + 1 < (int)t.mips ? l0 + 1 : l0;
    u32 w0 = max(t.width >> l0, 1u), h0 = max(t.height >> l0, 1u);
    float4 c0 = vgx_bilinear(base + t.mip_offset[l0], w0, h0, u, v);
    if(f > 0.0f)
    {
      u32 w1 = max(t.width >> l1, 1u), h1 = max(t.height >> l1, 1u);
      float4 c1 = vgx_bilinear(base + t.mip_offset[l1], w1, h1, u, v);
      float g = 1.0f - f;
      c0.x = c0.x * g + c1.x * f;
      c0.y = c0.y * g + c1.y * f;
      c0.z = c0.z * g + c1.z * f;
      c0.w = c0.w * g + c1.w * f;
    }
    return c0;
  }
  if(t.filter == VGX_FILTER_NEAREST)
  {
    u = u - floorf(u);
    v = v - floorf(v);
    int iu = (int)(u * (float)t.width);
    int iv = (int)(v * (float)t.height);
    if(iu >= (int)t.width)
      iu -= t.width;
    if(iv >= (int)t.height)
      iv -= t.height;
    iu = min(max(iu, 0), (int)t.width - 1);
    iv = min(max(iv, 0), (int)t.height - 1);
    return vgx_texel(base, t.width, iu, iv);
  }
  return vgx_bilinear(base, t.width, t.height, u, v);
}

/* Four-lane CreateDot (spirv_compile.cpp:629-643) of the barycentrics with
   (v0, v1, v2, 0): the fragment-input interpolation of :2200-2214. */
__device__ __forceinline__ float vgx_interp(const float *b, float a0, float a1, float a2)
{
  float acc = b[0] * a0;
  acc = acc + b[1] * a1;
  acc = acc + b[2] * a2;
  acc = acc + b[3] * 0.0f;
  return acc;
}

#endif
