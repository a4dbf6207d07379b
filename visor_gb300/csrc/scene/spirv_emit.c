/*
 * SPIR-V 1.0 emitter for the scenes' shader pairs (see include/visor_spirv.h).
 *
 * Opcode, decoration and enum numbers are those of the published SPIR-V 1.0
 * and GLSL.std.450 specifications.  Modules are laid out in the section order
 * the specification requires (capabilities, imports, memory model, entry
 * points, execution modes, debug, annotations, types/globals, functions).
 */
#include "visor_spirv.h"

#include <stdlib.h>
#include <string.h>

#include "visor_scene.h"

enum {
  OpSource = 3, OpSourceExtension = 4, OpName = 5, OpExtInstImport = 11, OpExtInst = 12,
  OpMemoryModel = 14, OpEntryPoint = 15, OpExecutionMode = 16, OpCapability = 17,
  OpTypeVoid = 19, OpTypeInt = 21, OpTypeFloat = 22, OpTypeVector = 23, OpTypeMatrix = 24,
  OpTypeImage = 25, OpTypeSampledImage = 27, OpTypeStruct = 30, OpTypePointer = 32,
  OpTypeFunction = 33, OpConstant = 43, OpFunction = 54, OpFunctionEnd = 56, OpVariable = 59,
  OpLoad = 61, OpStore = 62, OpAccessChain = 65, OpDecorate = 71, OpMemberDecorate = 72,
  OpVectorShuffle = 79, OpCompositeConstruct = 80, OpCompositeExtract = 81, OpCompositeInsert = 82,
  OpConvertSToF = 111, OpFAdd = 129, OpFMul = 133,
  OpImageSampleImplicitLod = 87, OpVectorTimesScalar = 142, OpMatrixTimesVector = 145,
  OpDot = 148, OpLabel = 248, OpReturn = 253,
};
enum { DecBlock = 2, DecColMajor = 5, DecMatrixStride = 7, DecBuiltIn = 11, DecLocation = 30,
       DecBinding = 33, DecDescriptorSet = 34, DecOffset = 35 };
enum { BuiltInPosition = 0, BuiltInPointSize = 1, BuiltInInstanceIndex = 43 };
enum { SCUniformConstant = 0, SCInput = 1, SCOutput = 3, SCFunction = 7, SCPushConstant = 9 };
enum { GLSLFMax = 40, GLSLNormalize = 69 };

typedef struct buf {
  uint32_t *w;
  size_t n, cap;
} buf;

typedef struct mod {
  buf head, debug, annot, types, code;
  uint32_t next;
} mod;

static void put(buf *b, uint32_t v)
{
  if(b->n == b->cap)
  {
    b->cap = b->cap ? b->cap * 2 : 64;
    b->w = (uint32_t *)realloc(b->w, b->cap * 4);
  }
  b->w[b->n++] = v;
}

static void inst(buf *b, uint32_t opcode, uint32_t nops, const uint32_t *ops)
{
  put(b, ((nops + 1) << 16) | opcode);
  for(uint32_t i = 0; i < nops; i++)
    put(b, ops[i]);
}

#define I(b, opc, ...)                                              \
  do                                                                \
  {                                                                 \
    const uint32_t ops_[] = {__VA_ARGS__};                          \
    inst((b), (opc), (uint32_t)(sizeof(ops_) / sizeof(ops_[0])), ops_); \
  } while(0)

/* Instruction whose operands end with a literal string (packed little-endian, NUL-terminated). */
static void inst_str(buf *b, uint32_t opcode, uint32_t npre, const uint32_t *pre, const char *s,
                     uint32_t npost, const uint32_t *post)
{
  size_t len = strlen(s) + 1, sw = (len + 3) / 4;
  put(b, (uint32_t)((1 + npre + sw + npost) << 16) | opcode);
  for(uint32_t i = 0; i < npre; i++)
    put(b, pre[i]);
  for(size_t i = 0; i < sw; i++)
  {
    uint32_t word = 0;
    for(size_t k = 0; k < 4; k++)
    {
      size_t idx = i * 4 + k;
      uint32_t ch = idx < len ? (uint8_t)s[idx] : 0;
      word |= ch << (8 * k);
    }
    put(b, word);
  }
  for(uint32_t i = 0; i < npost; i++)
    put(b, post[i]);
}

static uint32_t fbits(float f)
{
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

typedef struct common {
  uint32_t glsl, main, tvoid, tfn, tfloat, tint, vec2, vec3, vec4, mat4;
  uint32_t int0, int1, f0, f1;
} common;

static void common_types(mod *m, common *c)
{
  c->tvoid = m->next++;
  I(&m->types, OpTypeVoid, c->tvoid);
  c->tfn = m->next++;
  I(&m->types, OpTypeFunction, c->tfn, c->tvoid);
  c->tfloat = m->next++;
  I(&m->types, OpTypeFloat, c->tfloat, 32);
  c->tint = m->next++;
  I(&m->types, OpTypeInt, c->tint, 32, 1);
  c->vec2 = m->next++;
  I(&m->types, OpTypeVector, c->vec2, c->tfloat, 2);
  c->vec3 = m->next++;
  I(&m->types, OpTypeVector, c->vec3, c->tfloat, 3);
  c->vec4 = m->next++;
  I(&m->types, OpTypeVector, c->vec4, c->tfloat, 4);
  c->mat4 = m->next++;
  I(&m->types, OpTypeMatrix, c->mat4, c->vec4, 4);
  c->int0 = m->next++;
  I(&m->types, OpConstant, c->tint, c->int0, 0);
  c->int1 = m->next++;
  I(&m->types, OpConstant, c->tint, c->int1, 1);
  c->f0 = m->next++;
  I(&m->types, OpConstant, c->tfloat, c->f0, fbits(0.0f));
  c->f1 = m->next++;
  I(&m->types, OpConstant, c->tfloat, c->f1, fbits(1.0f));
}

static uint32_t var(mod *m, uint32_t ptrtype, uint32_t sc)
{
  uint32_t id = m->next++;
  I(&m->types, OpVariable, ptrtype, id, sc);
  return id;
}

static uint32_t ptr(mod *m, uint32_t sc, uint32_t type)
{
  uint32_t id = m->next++;
  I(&m->types, OpTypePointer, id, sc, type);
  return id;
}

static void decorate_loc(mod *m, uint32_t id, uint32_t loc) { I(&m->annot, OpDecorate, id, DecLocation, loc); }

/* push-constant block { mat4 mvp; vec4 light; } */
static uint32_t push_block(mod *m, common *c, uint32_t *pc_var)
{
  uint32_t pcs = m->next++;
  I(&m->types, OpTypeStruct, pcs, c->mat4, c->vec4);
  I(&m->annot, OpDecorate, pcs, DecBlock);
  I(&m->annot, OpMemberDecorate, pcs, 0, DecColMajor);
  I(&m->annot, OpMemberDecorate, pcs, 0, DecOffset, 0);
  I(&m->annot, OpMemberDecorate, pcs, 0, DecMatrixStride, 16);
  I(&m->annot, OpMemberDecorate, pcs, 1, DecOffset, 64);
  uint32_t pptr = ptr(m, SCPushConstant, pcs);
  *pc_var = var(m, pptr, SCPushConstant);
  return pcs;
}

static size_t finish(mod *m, common *c, uint32_t model, const char *marker, const uint32_t *iface,
                     uint32_t niface, int fragment, uint32_t *words, size_t capacity)
{
  buf out;
  memset(&out, 0, sizeof(out));
  put(&out, 0x07230203u); /* magic */
  put(&out, 0x00010000u); /* version 1.0 */
  put(&out, 0x00000000u); /* generator */
  put(&out, m->next);     /* id bound */
  put(&out, 0);
  I(&out, OpCapability, 1 /* Shader */);
  {
    uint32_t pre[1] = {c->glsl};
    inst_str(&out, OpExtInstImport, 1, pre, "GLSL.std.450", 0, NULL);
  }
  I(&out, OpMemoryModel, 0 /* Logical */, 1 /* GLSL450 */);
  {
    uint32_t pre[2] = {model, c->main};
    inst_str(&out, OpEntryPoint, 2, pre, "main", niface, iface);
  }
  if(fragment)
    I(&out, OpExecutionMode, c->main, 7 /* OriginUpperLeft */);
  I(&out, OpSource, 2 /* GLSL */, 450);
  inst_str(&out, OpSourceExtension, 0, NULL, marker, 0, NULL);
  {
    uint32_t pre[1] = {c->main};
    inst_str(&out, OpName, 1, pre, "main", 0, NULL);
  }
  for(size_t i = 0; i < m->debug.n; i++) put(&out, m->debug.w[i]);
  for(size_t i = 0; i < m->annot.n; i++) put(&out, m->annot.w[i]);
  for(size_t i = 0; i < m->types.n; i++) put(&out, m->types.w[i]);
  for(size_t i = 0; i < m->code.n; i++) put(&out, m->code.w[i]);
  out.w[3] = m->next;
  size_t n = out.n;
  if(words && capacity >= n)
    memcpy(words, out.w, n * 4);
  free(out.w);
  free(m->head.w);
  free(m->debug.w);
  free(m->annot.w);
  free(m->types.w);
  free(m->code.w);
  return n;
}

static void begin(mod *m, common *c)
{
  memset(m, 0, sizeof(*m));
  m->next = 1;
  c->glsl = m->next++;
  c->main = m->next++;
  common_types(m, c);
}

/* gl_PerVertex { vec4 gl_Position; float gl_PointSize; } output block */
static uint32_t per_vertex(mod *m, common *c, uint32_t *ptr_out_vec4)
{
  uint32_t pvs = m->next++;
  I(&m->types, OpTypeStruct, pvs, c->vec4, c->tfloat);
  I(&m->annot, OpMemberDecorate, pvs, 0, DecBuiltIn, BuiltInPosition);
  I(&m->annot, OpMemberDecorate, pvs, 1, DecBuiltIn, BuiltInPointSize);
  I(&m->annot, OpDecorate, pvs, DecBlock);
  uint32_t pptr = ptr(m, SCOutput, pvs);
  uint32_t pv = var(m, pptr, SCOutput);
  *ptr_out_vec4 = ptr(m, SCOutput, c->vec4);
  return pv;
}

static size_t emit_lambert_vs(int alpha, uint32_t *words, size_t cap)
{
  mod m;
  common c;
  begin(&m, &c);
  uint32_t pvo4;
  uint32_t pv = per_vertex(&m, &c, &pvo4);
  uint32_t pc;
  push_block(&m, &c, &pc);
  uint32_t ppc_mat4 = ptr(&m, SCPushConstant, c.mat4);
  uint32_t pin3 = ptr(&m, SCInput, c.vec3), pin2 = ptr(&m, SCInput, c.vec2);
  uint32_t pout3 = ptr(&m, SCOutput, c.vec3), pout2 = ptr(&m, SCOutput, c.vec2);
  uint32_t pinf = 0, poutf = 0;
  if(alpha)
  {
    pinf = ptr(&m, SCInput, c.tfloat);
    poutf = ptr(&m, SCOutput, c.tfloat);
  }
  uint32_t inPos = var(&m, pin3, SCInput), inNrm = var(&m, pin3, SCInput),
           inUV = var(&m, pin2, SCInput);
  uint32_t outNrm = var(&m, pout3, SCOutput), outUV = var(&m, pout2, SCOutput);
  uint32_t inA = 0, outA = 0;
  decorate_loc(&m, inPos, 0);
  decorate_loc(&m, inNrm, 1);
  decorate_loc(&m, inUV, 2);
  decorate_loc(&m, outNrm, 0);
  decorate_loc(&m, outUV, 1);
  if(alpha)
  {
    inA = var(&m, pinf, SCInput);
    outA = var(&m, poutf, SCOutput);
    decorate_loc(&m, inA, 3);
    decorate_loc(&m, outA, 2);
  }

  buf *f = &m.code;
  I(f, OpFunction, c.tvoid, c.main, 0, c.tfn);
  I(f, OpLabel, m.next++);
  uint32_t pos = m.next++;
  I(f, OpLoad, c.vec3, pos, inPos);
  uint32_t px = m.next++, py = m.next++, pz = m.next++;
  I(f, OpCompositeExtract, c.tfloat, px, pos, 0);
  I(f, OpCompositeExtract, c.tfloat, py, pos, 1);
  I(f, OpCompositeExtract, c.tfloat, pz, pos, 2);
  uint32_t p4 = m.next++;
  I(f, OpCompositeConstruct, c.vec4, p4, px, py, pz, c.f1);
  uint32_t mp = m.next++, mv = m.next++, clip = m.next++, gp = m.next++;
  I(f, OpAccessChain, ppc_mat4, mp, pc, c.int0);
  I(f, OpLoad, c.mat4, mv, mp);
  I(f, OpMatrixTimesVector, c.vec4, clip, mv, p4);
  I(f, OpAccessChain, pvo4, gp, pv, c.int0);
  I(f, OpStore, gp, clip);
  uint32_t n = m.next++, uv = m.next++;
  I(f, OpLoad, c.vec3, n, inNrm);
  I(f, OpStore, outNrm, n);
  I(f, OpLoad, c.vec2, uv, inUV);
  I(f, OpStore, outUV, uv);
  if(alpha)
  {
    uint32_t a = m.next++;
    I(f, OpLoad, c.tfloat, a, inA);
    I(f, OpStore, outA, a);
  }
  inst(f, OpReturn, 0, NULL);
  inst(f, OpFunctionEnd, 0, NULL);

  uint32_t iface[8];
  uint32_t ni = 0;
  iface[ni++] = pv;
  iface[ni++] = inPos;
  iface[ni++] = inNrm;
  iface[ni++] = inUV;
  if(alpha) iface[ni++] = inA;
  iface[ni++] = outNrm;
  iface[ni++] = outUV;
  if(alpha) iface[ni++] = outA;
  return finish(&m, &c, 0, alpha ? "visor_shader:lambert_tex_alpha.vert" : "visor_shader:lambert_tex.vert",
                iface, ni, 0, words, cap);
}

static size_t emit_lambert_fs(int alpha, uint32_t *words, size_t cap)
{
  mod m;
  common c;
  begin(&m, &c);
  uint32_t pc;
  push_block(&m, &c, &pc);
  uint32_t ppc_vec4 = ptr(&m, SCPushConstant, c.vec4);
  uint32_t img = m.next++;
  I(&m.types, OpTypeImage, img, c.tfloat, 1 /* 2D */, 0, 0, 0, 1, 0 /* Unknown */);
  uint32_t simg = m.next++;
  I(&m.types, OpTypeSampledImage, simg, img);
  uint32_t puc = ptr(&m, SCUniformConstant, simg);
  uint32_t tex = var(&m, puc, SCUniformConstant);
  I(&m.annot, OpDecorate, tex, DecDescriptorSet, 0);
  I(&m.annot, OpDecorate, tex, DecBinding, 0);
  uint32_t pin3 = ptr(&m, SCInput, c.vec3), pin2 = ptr(&m, SCInput, c.vec2);
  uint32_t pout4 = ptr(&m, SCOutput, c.vec4);
  uint32_t pinf = alpha ? ptr(&m, SCInput, c.tfloat) : 0;
  uint32_t inNrm = var(&m, pin3, SCInput), inUV = var(&m, pin2, SCInput);
  uint32_t outCol = var(&m, pout4, SCOutput);
  uint32_t inA = alpha ? var(&m, pinf, SCInput) : 0;
  decorate_loc(&m, inNrm, 0);
  decorate_loc(&m, inUV, 1);
  if(alpha)
    decorate_loc(&m, inA, 2);
  decorate_loc(&m, outCol, 0);

  buf *f = &m.code;
  I(f, OpFunction, c.tvoid, c.main, 0, c.tfn);
  I(f, OpLabel, m.next++);
  uint32_t n = m.next++, nn = m.next++;
  I(f, OpLoad, c.vec3, n, inNrm);
  I(f, OpExtInst, c.vec3, nn, c.glsl, GLSLNormalize, n);
  uint32_t lp = m.next++, l4 = m.next++, l3 = m.next++, d = m.next++, lam = m.next++;
  I(f, OpAccessChain, ppc_vec4, lp, pc, c.int1);
  I(f, OpLoad, c.vec4, l4, lp);
  I(f, OpVectorShuffle, c.vec3, l3, l4, l4, 0, 1, 2);
  I(f, OpDot, c.tfloat, d, nn, l3);
  I(f, OpExtInst, c.tfloat, lam, c.glsl, GLSLFMax, d, c.f0);
  uint32_t s = m.next++, uv = m.next++, t = m.next++;
  I(f, OpLoad, simg, s, tex);
  I(f, OpLoad, c.vec2, uv, inUV);
  I(f, OpImageSampleImplicitLod, c.vec4, t, s, uv);
  if(!alpha)
  {
    uint32_t col = m.next++;
    I(f, OpVectorTimesScalar, c.vec4, col, t, lam);
    I(f, OpStore, outCol, col);
  }
  else
  {
    uint32_t rgb = m.next++, lit = m.next++, a = m.next++;
    I(f, OpVectorShuffle, c.vec3, rgb, t, t, 0, 1, 2);
    I(f, OpVectorTimesScalar, c.vec3, lit, rgb, lam);
    I(f, OpLoad, c.tfloat, a, inA);
    uint32_t x = m.next++, y = m.next++, z = m.next++, col = m.next++;
    I(f, OpCompositeExtract, c.tfloat, x, lit, 0);
    I(f, OpCompositeExtract, c.tfloat, y, lit, 1);
    I(f, OpCompositeExtract, c.tfloat, z, lit, 2);
    I(f, OpCompositeConstruct, c.vec4, col, x, y, z, a);
    I(f, OpStore, outCol, col);
  }
  inst(f, OpReturn, 0, NULL);
  inst(f, OpFunctionEnd, 0, NULL);

  uint32_t iface[4];
  uint32_t ni = 0;
  iface[ni++] = inNrm;
  iface[ni++] = inUV;
  if(alpha) iface[ni++] = inA;
  iface[ni++] = outCol;
  return finish(&m, &c, 4, alpha ? "visor_shader:lambert_tex_alpha.frag" : "visor_shader:lambert_tex.frag",
                iface, ni, 1, words, cap);
}

/* gl_Position = inPos (instanced: inPos.x += float(gl_InstanceIndex) * 0.25); colour passed on */
static size_t emit_color_vs(int instanced, uint32_t *words, size_t cap)
{
  mod m;
  common c;
  begin(&m, &c);
  uint32_t pvo4;
  uint32_t pv = per_vertex(&m, &c, &pvo4);
  uint32_t pin4 = ptr(&m, SCInput, c.vec4);
  uint32_t inPos = var(&m, pin4, SCInput), inCol = var(&m, pin4, SCInput);
  uint32_t outCol = var(&m, pvo4, SCOutput);
  decorate_loc(&m, inPos, 0);
  decorate_loc(&m, inCol, 1);
  decorate_loc(&m, outCol, 0);
  uint32_t inInst = 0, quarter = 0;
  if(instanced)
  {
    inInst = var(&m, ptr(&m, SCInput, c.tint), SCInput);
    I(&m.annot, OpDecorate, inInst, DecBuiltIn, BuiltInInstanceIndex);
    quarter = m.next++;
    I(&m.types, OpConstant, c.tfloat, quarter, fbits(0.25f));
  }
  buf *f = &m.code;
  I(f, OpFunction, c.tvoid, c.main, 0, c.tfn);
  I(f, OpLabel, m.next++);
  uint32_t p = m.next++, gp = m.next++, col = m.next++;
  I(f, OpLoad, c.vec4, p, inPos);
  if(instanced)
  {
    uint32_t ii = m.next++, fi = m.next++, dx = m.next++, x = m.next++, x2 = m.next++, p2 = m.next++;
    I(f, OpLoad, c.tint, ii, inInst);
    I(f, OpConvertSToF, c.tfloat, fi, ii);
    I(f, OpFMul, c.tfloat, dx, fi, quarter);
    I(f, OpCompositeExtract, c.tfloat, x, p, 0);
    I(f, OpFAdd, c.tfloat, x2, x, dx);
    I(f, OpCompositeInsert, c.vec4, p2, x2, p, 0);
    p = p2;
  }
  I(f, OpAccessChain, pvo4, gp, pv, c.int0);
  I(f, OpStore, gp, p);
  I(f, OpLoad, c.vec4, col, inCol);
  I(f, OpStore, outCol, col);
  inst(f, OpReturn, 0, NULL);
  inst(f, OpFunctionEnd, 0, NULL);
  uint32_t iface[5] = {pv, inPos, inCol, outCol, inInst};
  return finish(&m, &c, 0, instanced ? "visor_shader:color_instanced.vert" : "visor_shader:color.vert", iface,
                instanced ? 5 : 4, 0, words, cap);
}

static size_t emit_color_fs(uint32_t *words, size_t cap)
{
  mod m;
  common c;
  begin(&m, &c);
  uint32_t pin4 = ptr(&m, SCInput, c.vec4), pout4 = ptr(&m, SCOutput, c.vec4);
  uint32_t inCol = var(&m, pin4, SCInput), outCol = var(&m, pout4, SCOutput);
  decorate_loc(&m, inCol, 0);
  decorate_loc(&m, outCol, 0);
  buf *f = &m.code;
  I(f, OpFunction, c.tvoid, c.main, 0, c.tfn);
  I(f, OpLabel, m.next++);
  uint32_t col = m.next++;
  I(f, OpLoad, c.vec4, col, inCol);
  I(f, OpStore, outCol, col);
  inst(f, OpReturn, 0, NULL);
  inst(f, OpFunctionEnd, 0, NULL);
  uint32_t iface[2] = {inCol, outCol};
  return finish(&m, &c, 4, "visor_shader:color.frag", iface, 2, 1, words, cap);
}

/* samplerCube at binding 0, read at the interpolated (unnormalised) normal */
static size_t emit_cube_fs(uint32_t *words, size_t cap)
{
  mod m;
  common c;
  begin(&m, &c);
  uint32_t img = m.next++;
  I(&m.types, OpTypeImage, img, c.tfloat, 3 /* Cube */, 0, 0, 0, 1, 0 /* Unknown */);
  uint32_t simg = m.next++;
  I(&m.types, OpTypeSampledImage, simg, img);
  uint32_t puc = ptr(&m, SCUniformConstant, simg);
  uint32_t tex = var(&m, puc, SCUniformConstant);
  I(&m.annot, OpDecorate, tex, DecDescriptorSet, 0);
  I(&m.annot, OpDecorate, tex, DecBinding, 0);
  uint32_t pin3 = ptr(&m, SCInput, c.vec3), pout4 = ptr(&m, SCOutput, c.vec4);
  uint32_t inNrm = var(&m, pin3, SCInput), outCol = var(&m, pout4, SCOutput);
  decorate_loc(&m, inNrm, 0);
  decorate_loc(&m, outCol, 0);
  buf *f = &m.code;
  I(f, OpFunction, c.tvoid, c.main, 0, c.tfn);
  I(f, OpLabel, m.next++);
  uint32_t n = m.next++, smp = m.next++, t = m.next++;
  I(f, OpLoad, c.vec3, n, inNrm);
  I(f, OpLoad, simg, smp, tex);
  I(f, OpImageSampleImplicitLod, c.vec4, t, smp, n);
  I(f, OpStore, outCol, t);
  inst(f, OpReturn, 0, NULL);
  inst(f, OpFunctionEnd, 0, NULL);
  uint32_t iface[2] = {inNrm, outCol};
  return finish(&m, &c, 4, "visor_shader:cube.frag", iface, 2, 1, words, cap);
}

size_t vspv_emit(uint32_t shader, uint32_t stage, uint32_t *words, size_t capacity)
{
  switch(shader)
  {
    case VSC_SHADER_LAMBERT_TEX:
      return stage == VSPV_STAGE_VERTEX ? emit_lambert_vs(0, words, capacity)
                                        : emit_lambert_fs(0, words, capacity);
    case VSC_SHADER_LAMBERT_TEX_ALPHA:
      return stage == VSPV_STAGE_VERTEX ? emit_lambert_vs(1, words, capacity)
                                        : emit_lambert_fs(1, words, capacity);
    case VSC_SHADER_COLOR:
      return stage == VSPV_STAGE_VERTEX ? emit_color_vs(0, words, capacity)
                                        : emit_color_fs(words, capacity);
    case VSC_SHADER_COLOR_INSTANCED:
      return stage == VSPV_STAGE_VERTEX ? emit_color_vs(1, words, capacity)
                                        : emit_color_fs(words, capacity);
    case VSC_SHADER_CUBE:
      return stage == VSPV_STAGE_VERTEX ? emit_lambert_vs(0, words, capacity)
                                        : emit_cube_fs(words, capacity);
    default: return 0;
  }
}
