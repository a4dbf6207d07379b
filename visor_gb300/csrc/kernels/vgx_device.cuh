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
 * buffer return the default instead of faulting.  A binding whose bit is set in
 * D.instance_rate (Vulkan draw parameters only) steps by the instance index.
 */
__device__ __forceinline__ float4 vgx_fetch(const VgxDraw &D, u32 loc, u32 vertex, u32 instance)
{
  float4 out = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
  if(loc >= VGX_MAX_ATTRS)
    return out;
  const VgxAttr a = D.attrs[loc];
  if(a.format == VGX_FMT_NONE || a.binding >= VGX_MAX_VB)
    return out;
  const u32 index = ((D.instance_rate >> a.binding) & 1u) ? instance : vertex;
  u64 off = (u64)a.offset + (u64)a.stride * (u64)index;
  u32 size = a.format == VGX_FMT_RGBA32 ? 16u : a.format == VGX_FMT_RGB32 ? 12u
             : a.format == VGX_FMT_RG32 ? 8u : 4u;
  if(off + size > D.vb_bytes[a.binding])
    return out;
  const u32 *p = (const u32 *)(D.vb[a.binding] + off);
  const u64 addr = D.vb[a.binding] + off;
  /* one wide load where the address is aligned and the wider read stays in the buffer */
  if(a.format != VGX_FMT_RGBA8_UNORM && a.format != VGX_FMT_R32 && (addr & 15u) == 0 &&
     off + 16 <= D.vb_bytes[a.binding])
  {
    const float4 v = __ldg((const float4 *)p);
    out.x = v.x;
    if(a.format != VGX_FMT_R32)
      out.y = v.y;
    if(a.format == VGX_FMT_RGB32 || a.format == VGX_FMT_RGBA32)
      out.z = v.z;
    if(a.format == VGX_FMT_RGBA32)
      out.w = v.w;
    return out;
  }
  if(a.format == VGX_FMT_RG32 && (addr & 7u) == 0)
  {
    const float2 v = __ldg((const float2 *)p);
    out.x = v.x;
    out.y = v.y;
    return out;
  }
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

#if VGX_TEX_BLOCKS
/* RGB565 channel to 8 bits with the block decompressor's rounding (texture_sampling.cpp:93-118
   uses 3rdparty/decompress.c): t = 255v + 2^(n-1), (t + t/2^n) / 2^n */
__device__ __forceinline__ u32 vgx_bc_expand(u32 v, u32 bits)
{
  const u32 t = v * 255u + (1u << (bits - 1));
  return (t + (t >> bits)) >> bits;
}

/*
 * Texel (x, y) of a BC2/BC3 image as RGBA bytes (R in the low byte): 16-byte
 * 4x4 blocks stored row by row, width/4 a row.  Bytes 8..15 hold two RGB565
 * endpoints and 2-bit palette indices; BC2 keeps the three-colour palette of
 * BC1 when c0 <= c1, BC3 always uses four colours.  BC2 alpha: explicit 4 bits
 * x 17; BC3 alpha: two endpoints and 3-bit indices into 8 (a0 > a1) or 6 + {0,
 * 255} interpolated values, divisions truncating.  Compiled only into the
 * raster variants of jobs that bind a block-compressed texture (VGX_TEX_BLOCKS).
 */
__device__ __forceinline__ u32 vgx_bc_texel(const u8 *base, u32 width, u32 fmt, int x, int y)
{
  const u8 *blk = base + ((u64)(y >> 2) * (width >> 2) + (u32)(x >> 2)) * 16u;
  uint4 b;
  if(((u64)blk & 15u) == 0)
  {
    b = __ldg((const uint4 *)blk);
  }
  else
  {
    u32 w[4];
#pragma unroll
    for(int k = 0; k < 4; k++)
      w[k] = (u32)__ldg(blk + 4 * k) | ((u32)__ldg(blk + 4 * k + 1) << 8) |
             ((u32)__ldg(blk + 4 * k + 2) << 16) | ((u32)__ldg(blk + 4 * k + 3) << 24);
    b = make_uint4(w[0], w[1], w[2], w[3]);
  }
  const u32 i = (u32)((y & 3) * 4 + (x & 3));
  const u32 c0 = b.z & 0xffffu, c1 = b.z >> 16;
  const u32 code = (b.w >> (2 * i)) & 3u;
  const bool four = fmt == VGX_TEX_BC3 || c0 > c1;
  u32 rgb = 0;
#pragma unroll
  for(int ch = 0; ch < 3; ch++)
  {
    const u32 sh = ch == 0 ? 11u : ch == 1 ? 5u : 0u, bits = ch == 1 ? 6u : 5u;
    const u32 a = vgx_bc_expand((c0 >> sh) & ((1u << bits) - 1u), bits);
    const u32 e = vgx_bc_expand((c1 >> sh) & ((1u << bits) - 1u), bits);
    u32 v;
    if(code == 0)
      v = a;
    else if(code == 1)
      v = e;
    else if(four)
      v = code == 2 ? (2 * a + e) / 3 : (a + 2 * e) / 3;
    else
      v = code == 2 ? (a + e) / 2 : 0u;
    rgb |= v << (8 * ch);
  }
  u32 alpha;
  if(fmt == VGX_TEX_BC2)
  {
    const u32 row = i < 8 ? b.x : b.y;
    alpha = ((row >> (4 * (i & 7))) & 15u) * 17u;
  }
  else
  {
    const u32 a0 = b.x & 0xffu, a1 = (b.x >> 8) & 0xffu;
    /* 3-bit indices: bytes 2..4 for texels 0..7, bytes 5..7 for texels 8..15 */
    const u32 bits = i < 8 ? (b.x >> 16) | ((b.y & 0xffu) << 16) : (b.y >> 8);
    const u32 ac = (bits >> (3 * (i & 7))) & 7u;
    if(ac == 0)
      alpha = a0;
    else if(ac == 1)
      alpha = a1;
    else if(a0 > a1)
      alpha = ((8 - ac) * a0 + (ac - 1) * a1) / 7;
    else if(ac == 6)
      alpha = 0;
    else if(ac == 7)
      alpha = 255;
    else
      alpha = ((6 - ac) * a0 + (ac - 1) * a1) / 5;
  }
  return rgb | (alpha << 24);
}
#endif

#ifndef VGX_TEX_BLOCKS
#define VGX_TEX_BLOCKS 0
#endif

__device__ __forceinline__ float4 vgx_texel(const u8 *base, u32 width, u32 fmt, int x, int y)
{
#if VGX_TEX_BLOCKS
  const u32 t = fmt == VGX_TEX_RGBA8 ? __ldg((const u32 *)(base + ((u64)y * width + (u32)x) * 4u))
                                     : vgx_bc_texel(base, width, fmt, x, y);
#else
  (void)fmt;
  const u32 t = __ldg((const u32 *)(base + ((u64)y * width + (u32)x) * 4u));
#endif
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
__device__ __forceinline__ float4 vgx_bilinear(const u8 *base, u32 W, u32 H, u32 fmt, float u, float v)
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
  float4 TL = vgx_texel(base, W, fmt, iu0, iv0);
  float4 TR = vgx_texel(base, W, fmt, iu1, iv0);
  float4 BL = vgx_texel(base, W, fmt, iu0, iv1);
  float4 BR = vgx_texel(base, W, fmt, iu1, iv1);
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
    float4 c0 = vgx_bilinear(base + t.mip_offset[l0], w0, h0, t.format, u, v);
    if(f > 0.0f)
    {
      u32 w1 = max(t.width >> l1, 1u), h1 = max(t.height >> l1, 1u);
      float4 c1 = vgx_bilinear(base + t.mip_offset[l1], w1, h1, t.format, u, v);
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
    return vgx_texel(base, t.width, t.format, iu, iv);
  }
  return vgx_bilinear(base, t.width, t.height, t.format, u, v);
}

/*
 * sample_cube_wrapped (texture_sampling.cpp:186-250): the major axis picks the
 * face, tested in this order so that a later match replaces an earlier one on
 * ties; then the reference's bilinear sample of that face's mip 0 at
 * 0.5 * (u / axis + 1).  The sampler object is ignored, as in the reference.
 */
__device__ __forceinline__ float4 vgx_sample_cube(const VgxDraw &D, u32 slot, float x, float y,
                                                  float z)
{
  if(slot >= VGX_MAX_TEX || D.tex[slot].base == 0)
    return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const VgxTex &t = D.tex[slot];
  const float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  const bool px = x > 0.0f, py = y > 0.0f, pz = z > 0.0f;
  float axis = 0.0f, u = 0.0f, v = 0.0f;
  u32 face = 0;
  if(px && ax >= ay && ax >= az) { axis = ax; u = -z; v = -y; face = 0; }
  if(!px && ax >= ay && ax >= az) { axis = ax; u = z; v = -y; face = 1; }
  if(py && ay >= ax && ay >= az) { axis = ay; u = x; v = z; face = 2; }
  if(!py && ay >= ax && ay >= az) { axis = ay; u = x; v = -z; face = 3; }
  if(pz && az >= ax && az >= ay) { axis = az; u = x; v = -y; face = 4; }
  if(!pz && az >= ax && az >= ay) { axis = az; u = -x; v = -y; face = 5; }
  if(face >= t.layers)
    face = 0;
  const u8 *base = (const u8 *)t.base + t.layer_bytes * face;
  return vgx_bilinear(base, t.width, t.height, t.format, 0.5f * (u / axis + 1.0f),
                      0.5f * (v / axis + 1.0f));
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
