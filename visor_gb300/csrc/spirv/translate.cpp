/*
 * SPIR-V -> CUDA C++ translator (see translate.h).
 *
 * The module is parsed into types, constants, decorations, global variables
 * and functions (the three passes of spirv_compile.cpp:750-1892 become one
 * parse plus code generation).  Every SPIR-V function becomes a __device__
 * function over a per-invocation context holding the module's interface and
 * private variables; every result id becomes a local declared at the top of
 * its function (so structured control flow can be lowered to labels and
 * gotos).  Interface handling follows the reference's entry wrappers:
 *   vertex inputs   GetVertexAttributeData then truncation (:1957-1992)
 *   vertex outputs  Position; Location n padded with component 0 (:2057-2097)
 *   fragment inputs CreateDot of the perspective-corrected barycentrics with
 *                   the three vertices' values (:2159-2279)
 *   fragment output Location 0 (:2350-2355)
 *   resources       push constants, uniform blocks, combined image samplers
 */
#include "translate.h"

#include <string.h>

#include <algorithm>
#include <functional>
#include <map>
#include <set>
#include <sstream>

#define VGX_MAX_TEX_TRANSLATE 4
#define VGX_MAX_UBO_TRANSLATE 4

namespace vst
{
namespace
{
enum Op : uint32_t
{
  OpNop = 0, OpSource = 3, OpSourceExtension = 4, OpName = 5, OpMemberName = 6, OpString = 7,
  OpLine = 8, OpExtension = 10, OpExtInstImport = 11, OpExtInst = 12, OpMemoryModel = 14,
  OpEntryPoint = 15, OpExecutionMode = 16, OpCapability = 17, OpTypeVoid = 19, OpTypeBool = 20,
  OpTypeInt = 21, OpTypeFloat = 22, OpTypeVector = 23, OpTypeMatrix = 24, OpTypeImage = 25,
  OpTypeSampler = 26, OpTypeSampledImage = 27, OpTypeArray = 28, OpTypeRuntimeArray = 29,
  OpTypeStruct = 30, OpTypePointer = 32, OpTypeFunction = 33, OpConstantTrue = 41,
  OpConstantFalse = 42, OpConstant = 43, OpConstantComposite = 44, OpConstantNull = 46,
  OpFunction = 54, OpFunctionParameter = 55, OpFunctionEnd = 56, OpFunctionCall = 57,
  OpVariable = 59, OpLoad = 61, OpStore = 62, OpAccessChain = 65, OpInBoundsAccessChain = 66,
  OpDecorate = 71, OpMemberDecorate = 72, OpVectorExtractDynamic = 77, OpVectorShuffle = 79,
  OpCompositeConstruct = 80, OpCompositeExtract = 81, OpCompositeInsert = 82, OpCopyObject = 83,
  OpTranspose = 84, OpSampledImage = 86, OpImageSampleImplicitLod = 87,
  OpImageSampleExplicitLod = 88, OpConvertFToU = 109, OpConvertFToS = 110, OpConvertSToF = 111,
  OpConvertUToF = 112, OpBitcast = 124, OpSNegate = 126, OpFNegate = 127, OpIAdd = 128,
  OpFAdd = 129, OpISub = 130, OpFSub = 131, OpIMul = 132, OpFMul = 133, OpUDiv = 134,
  OpSDiv = 135, OpFDiv = 136, OpUMod = 137, OpSRem = 138, OpSMod = 139, OpFRem = 140,
  OpFMod = 141, OpVectorTimesScalar = 142, OpMatrixTimesScalar = 143, OpVectorTimesMatrix = 144,
  OpMatrixTimesVector = 145, OpMatrixTimesMatrix = 146, OpDot = 148, OpAny = 154, OpAll = 155,
  OpLogicalEqual = 164, OpLogicalNotEqual = 165, OpLogicalOr = 166, OpLogicalAnd = 167,
  OpLogicalNot = 168, OpSelect = 169, OpIEqual = 170, OpINotEqual = 171, OpUGreaterThan = 172,
  OpSGreaterThan = 173, OpUGreaterThanEqual = 174, OpSGreaterThanEqual = 175, OpULessThan = 176,
  OpSLessThan = 177, OpULessThanEqual = 178, OpSLessThanEqual = 179, OpFOrdEqual = 180,
  OpFUnordEqual = 181, OpFOrdNotEqual = 182, OpFUnordNotEqual = 183, OpFOrdLessThan = 184,
  OpFUnordLessThan = 185, OpFOrdGreaterThan = 186, OpFUnordGreaterThan = 187,
  OpFOrdLessThanEqual = 188, OpFUnordLessThanEqual = 189, OpFOrdGreaterThanEqual = 190,
  OpFUnordGreaterThanEqual = 191, OpShiftRightLogical = 194, OpShiftRightArithmetic = 195,
  OpShiftLeftLogical = 196, OpBitwiseOr = 197, OpBitwiseXor = 198, OpBitwiseAnd = 199, OpNot = 200,
  OpDPdx = 207, OpDPdy = 208, OpPhi = 245, OpLoopMerge = 246, OpSelectionMerge = 247,
  OpLabel = 248, OpBranch = 249, OpBranchConditional = 250, OpSwitch = 251, OpKill = 252,
  OpReturn = 253, OpReturnValue = 254, OpUnreachable = 255,
};

enum Kind
{
  K_VOID, K_BOOL, K_INT, K_FLOAT, K_VEC, K_MAT, K_ARR, K_RARR, K_STRUCT, K_PTR, K_FN, K_IMAGE,
  K_SIMAGE, K_SAMPLER
};

enum Storage : uint32_t
{
  SC_UniformConstant = 0, SC_Input = 1, SC_Uniform = 2, SC_Output = 3, SC_Workgroup = 4,
  SC_CrossWorkgroup = 5, SC_Private = 6, SC_Function = 7, SC_PushConstant = 9,
  SC_StorageBuffer = 12
};

enum Dec : uint32_t
{
  D_Block = 2, D_BufferBlock = 3, D_RowMajor = 4, D_ColMajor = 5, D_ArrayStride = 6,
  D_MatrixStride = 7, D_BuiltIn = 11, D_Flat = 14, D_Location = 30, D_Binding = 33,
  D_DescriptorSet = 34, D_Offset = 35
};

enum BuiltIn : uint32_t
{
  BI_Position = 0, BI_PointSize = 1, BI_ClipDistance = 3, BI_CullDistance = 4, BI_VertexId = 5,
  BI_InstanceId = 6, BI_VertexIndex = 42, BI_InstanceIndex = 43
};

struct Type
{
  Kind k = K_VOID;
  uint32_t width = 32, sign = 0, elem = 0, count = 0, storage = 0, dim = 0;
  std::vector<uint32_t> members;
};

struct Inst
{
  uint32_t op;
  std::vector<uint32_t> w;
};

struct Decor
{
  uint32_t dec;
  std::vector<uint32_t> p;
};

struct Var
{
  uint32_t type = 0; /* pointer type */
  uint32_t storage = 0;
  uint32_t init = 0;
};

struct Func
{
  uint32_t id = 0, ret = 0;
  std::vector<uint32_t> params;
  std::vector<Inst> body;
};

struct Entry
{
  uint32_t model = 0, fn = 0;
  std::string name;
  std::vector<uint32_t> iface;
};
}    // namespace

struct Module
{
  uint32_t bound = 0;
  uint32_t glsl = 0;
  std::map<uint32_t, Type> types;
  std::map<uint32_t, std::pair<uint32_t, std::vector<uint32_t>>> consts; /* id -> (type, words|ids) */
  std::set<uint32_t> composite_consts;
  std::map<uint32_t, Var> vars;
  std::map<uint32_t, std::vector<Decor>> decs;
  std::map<std::pair<uint32_t, uint32_t>, std::vector<Decor>> mdecs;
  std::map<uint32_t, Func> funcs;
  std::vector<uint32_t> func_order;
  std::vector<Entry> entries;
  std::map<uint32_t, uint32_t> rtype;    /* result id -> type id */
  std::map<uint32_t, const Inst *> defs; /* result id -> defining instruction */
};

namespace
{
bool has_result_type(uint32_t op)
{
  switch(op)
  {
    case OpExtInst: case OpFunctionParameter: case OpFunctionCall: case OpVariable: case OpLoad:
    case OpAccessChain: case OpInBoundsAccessChain: case OpVectorExtractDynamic:
    case OpVectorShuffle: case OpCompositeConstruct: case OpCompositeExtract:
    case OpCompositeInsert: case OpCopyObject: case OpTranspose: case OpSampledImage:
    case OpImageSampleImplicitLod: case OpImageSampleExplicitLod: case OpPhi:
      return true;
    default: return op >= 109 && op <= 208;
  }
}

bool get_dec(const Module &m, uint32_t id, uint32_t dec, uint32_t *val)
{
  auto it = m.decs.find(id);
  if(it == m.decs.end())
    return false;
  for(const Decor &d : it->second)
    if(d.dec == dec)
    {
      if(val)
        *val = d.p.empty() ? 0 : d.p[0];
      return true;
    }
  return false;
}

bool get_mdec(const Module &m, uint32_t id, uint32_t member, uint32_t dec, uint32_t *val)
{
  auto it = m.mdecs.find({id, member});
  if(it == m.mdecs.end())
    return false;
  for(const Decor &d : it->second)
    if(d.dec == dec)
    {
      if(val)
        *val = d.p.empty() ? 0 : d.p[0];
      return true;
    }
  return false;
}

std::string fbits(uint32_t u)
{
  char b[48];
  snprintf(b, sizeof(b), "__int_as_float(0x%08x)", u);
  return b;
}
}    // namespace

Module *parse(const uint32_t *words, size_t count, std::string &err)
{
  if(count < 5 || words[0] != 0x07230203u)
  {
    err = "not a SPIR-V module (bad magic)";
    return nullptr;
  }
  Module *m = new Module();
  m->bound = words[3];
  size_t i = 5;
  Func *cur = nullptr;
  while(i < count)
  {
    uint32_t op = words[i] & 0xffff, wc = words[i] >> 16;
    if(wc == 0 || i + wc > count)
    {
      err = "truncated instruction";
      delete m;
      return nullptr;
    }
    Inst in;
    in.op = op;
    in.w.assign(words + i + 1, words + i + wc);
    const std::vector<uint32_t> &w = in.w;
    i += wc;
    switch(op)
    {
      case OpExtInstImport:
        if(strcmp((const char *)&w[1], "GLSL.std.450") == 0)
          m->glsl = w[0];
        break;
      case OpEntryPoint:
      {
        Entry e;
        e.model = w[0];
        e.fn = w[1];
        e.name = (const char *)&w[2];
        size_t sw = (e.name.size() + 1 + 3) / 4;
        for(size_t k = 2 + sw; k < w.size(); k++)
          e.iface.push_back(w[k]);
        m->entries.push_back(e);
        break;
      }
      case OpDecorate:
      {
        Decor d;
        d.dec = w[1];
        d.p.assign(w.begin() + 2, w.end());
        m->decs[w[0]].push_back(d);
        break;
      }
      case OpMemberDecorate:
      {
        Decor d;
        d.dec = w[2];
        d.p.assign(w.begin() + 3, w.end());
        m->mdecs[{w[0], w[1]}].push_back(d);
        break;
      }
      case OpTypeVoid: m->types[w[0]].k = K_VOID; break;
      case OpTypeBool: m->types[w[0]].k = K_BOOL; break;
      case OpTypeInt:
      {
        Type &t = m->types[w[0]];
        t.k = K_INT;
        t.width = w[1];
        t.sign = w[2];
        break;
      }
      case OpTypeFloat:
      {
        Type &t = m->types[w[0]];
        t.k = K_FLOAT;
        t.width = w[1];
        break;
      }
      case OpTypeVector:
      case OpTypeMatrix:
      {
        Type &t = m->types[w[0]];
        t.k = op == OpTypeVector ? K_VEC : K_MAT;
        t.elem = w[1];
        t.count = w[2];
        break;
      }
      case OpTypeImage:
      {
        Type &t = m->types[w[0]];
        t.k = K_IMAGE;
        t.elem = w[1];
        t.dim = w[2];
        break;
      }
      case OpTypeSampler: m->types[w[0]].k = K_SAMPLER; break;
      case OpTypeSampledImage:
      {
        Type &t = m->types[w[0]];
        t.k = K_SIMAGE;
        t.elem = w[1];
        t.dim = m->types[w[1]].dim;
        break;
      }
      case OpTypeArray:
      {
        Type &t = m->types[w[0]];
        t.k = K_ARR;
        t.elem = w[1];
        auto c = m->consts.find(w[2]);
        t.count = c != m->consts.end() && !c->second.second.empty() ? c->second.second[0] : 0;
        break;
      }
      case OpTypeRuntimeArray:
      {
        Type &t = m->types[w[0]];
        t.k = K_RARR;
        t.elem = w[1];
        break;
      }
      case OpTypeStruct:
      {
        Type &t = m->types[w[0]];
        t.k = K_STRUCT;
        t.members.assign(w.begin() + 1, w.end());
        break;
      }
      case OpTypePointer:
      {
        Type &t = m->types[w[0]];
        t.k = K_PTR;
        t.storage = w[1];
        t.elem = w[2];
        break;
      }
      case OpTypeFunction:
      {
        Type &t = m->types[w[0]];
        t.k = K_FN;
        t.elem = w[1];
        t.members.assign(w.begin() + 2, w.end());
        break;
      }
      case OpConstantTrue:
      case OpConstantFalse:
        m->consts[w[1]] = {w[0], {op == OpConstantTrue ? 1u : 0u}};
        m->rtype[w[1]] = w[0];
        break;
      case OpConstant:
        m->consts[w[1]] = {w[0], std::vector<uint32_t>(w.begin() + 2, w.end())};
        m->rtype[w[1]] = w[0];
        break;
      case OpConstantComposite:
        m->consts[w[1]] = {w[0], std::vector<uint32_t>(w.begin() + 2, w.end())};
        m->composite_consts.insert(w[1]);
        m->rtype[w[1]] = w[0];
        break;
      case OpConstantNull:
        m->consts[w[1]] = {w[0], {}};
        m->rtype[w[1]] = w[0];
        break;
      case OpVariable:
        if(!cur)
        {
          Var v;
          v.type = w[0];
          v.storage = w[2];
          v.init = w.size() > 3 ? w[3] : 0;
          m->vars[w[1]] = v;
          m->rtype[w[1]] = w[0];
        }
        else
        {
          cur->body.push_back(in);
        }
        break;
      case OpFunction:
      {
        Func &f = m->funcs[w[1]];
        f.id = w[1];
        f.ret = w[0];
        m->func_order.push_back(w[1]);
        m->rtype[w[1]] = w[0];
        cur = &f;
        break;
      }
      case OpFunctionParameter:
        if(cur)
        {
          cur->params.push_back(w[1]);
          m->rtype[w[1]] = w[0];
        }
        break;
      case OpFunctionEnd: cur = nullptr; break;
      case OpSource: case OpSourceExtension: case OpName: case OpMemberName: case OpString:
      case OpLine: case OpExtension: case OpMemoryModel: case OpExecutionMode: case OpCapability:
      case OpNop:
        break;
      default:
        if(cur)
          cur->body.push_back(in);
        else
        {
          err = "unsupported module-scope opcode " + std::to_string(op);
          delete m;
          return nullptr;
        }
        break;
    }
  }
  for(auto &kv : m->funcs)
    for(const Inst &in : kv.second.body)
      if(has_result_type(in.op) && in.w.size() >= 2)
      {
        m->rtype[in.w[1]] = in.w[0];
        m->defs[in.w[1]] = &in;
      }
  if(m->entries.empty())
  {
    err = "module has no entry point";
    delete m;
    return nullptr;
  }
  return m;
}

void destroy(Module *m) { delete m; }

int entry_model(const Module *m, const char *name)
{
  for(const Entry &e : m->entries)
    if(e.name == name)
      return (int)e.model;
  return -1;
}

namespace
{
struct FsInput
{
  uint32_t var, loc, ncomp, slot, elems;
  bool is_int;
};

/* Per-module code generator. */
struct Gen
{
  const Module &m;
  std::string ns;      /* namespace of this stage */
  std::ostringstream out;
  std::string err;
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> *tex_slots; /* (set,binding) -> slot */
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> *ubo_slots;
  std::vector<Binding> *tex_list, *ubo_list;
  bool fragment = false;
  /* block pointers: id -> (pointee type, matrix stride, row major) */
  struct BlockPtr
  {
    uint32_t type, mstride, rowmajor;
  };
  std::map<uint32_t, BlockPtr> bptr;
  std::map<uint32_t, uint32_t> fs_slot_of_var; /* FS input var -> first slot */
  int lod_slot = -1, lod_tex = -1;
  int samples = 0; /* image sample instructions emitted */
  std::set<uint32_t> emitted_structs;

  Gen(const Module &mm) : m(mm) {}

  const Type &T(uint32_t id) const
  {
    static Type dummy;
    auto it = m.types.find(id);
    return it == m.types.end() ? dummy : it->second;
  }

  uint32_t ncomp(uint32_t tid) const
  {
    const Type &t = T(tid);
    return t.k == K_VEC ? t.count : 1;
  }

  uint32_t scalar_of(uint32_t tid) const
  {
    const Type &t = T(tid);
    return t.k == K_VEC ? t.elem : tid;
  }

  bool is_block_storage(uint32_t sc) const
  {
    return sc == SC_PushConstant || sc == SC_Uniform || sc == SC_StorageBuffer;
  }

  std::string ctype(uint32_t tid)
  {
    const Type &t = T(tid);
    switch(t.k)
    {
      case K_VOID: return "void";
      case K_BOOL: return "bool";
      case K_INT: return t.sign ? "int" : "unsigned";
      case K_FLOAT: return t.width == 64 ? "double" : "float";
      case K_VEC: return "vgx_v<" + ctype(t.elem) + ", " + std::to_string(t.count) + ">";
      case K_MAT: return "vgx_m<" + std::to_string(t.count) + ", " + std::to_string(T(t.elem).count) + ">";
      case K_ARR: return "vgx_a<" + ctype(t.elem) + ", " + std::to_string(t.count ? t.count : 1) + ">";
      case K_RARR: return ctype(t.elem);
      case K_STRUCT: return ns + "S" + std::to_string(tid);
      case K_PTR:
        if(is_block_storage(t.storage))
          return "const unsigned char *";
        if(t.storage == SC_UniformConstant)
          return "int";
        return ctype(t.elem) + " *";
      case K_IMAGE: case K_SIMAGE: case K_SAMPLER: return "int";
      default: return "int";
    }
  }

  void emit_struct(uint32_t tid, std::ostringstream &o)
  {
    if(emitted_structs.count(tid))
      return;
    const Type &t = T(tid);
    for(uint32_t mt : t.members)
      if(T(mt).k == K_STRUCT)
        emit_struct(mt, o);
      else if(T(mt).k == K_ARR && T(T(mt).elem).k == K_STRUCT)
        emit_struct(T(mt).elem, o);
    emitted_structs.insert(tid);
    o << "struct " << ns << "S" << tid << " {";
    for(size_t i = 0; i < t.members.size(); i++)
      o << " " << ctype(t.members[i]) << " m" << i << ";";
    o << " };\n";
  }

  /* expression of a value id */
  std::string val(uint32_t id)
  {
    auto c = m.consts.find(id);
    if(c != m.consts.end())
      return const_expr(id);
    auto v = m.vars.find(id);
    if(v != m.vars.end())
    {
      const Var &var = v->second;
      if(var.storage == SC_PushConstant)
        return "(ctx.D->push)";
      if(var.storage == SC_Uniform || var.storage == SC_StorageBuffer)
      {
        uint32_t set = 0, bind = 0;
        get_dec(m, id, D_DescriptorSet, &set);
        get_dec(m, id, D_Binding, &bind);
        return "((const unsigned char *)ctx.D->ubo[" + std::to_string(ubo_slot(set, bind)) + "])";
      }
      if(var.storage == SC_UniformConstant)
      {
        uint32_t set = 0, bind = 0;
        get_dec(m, id, D_DescriptorSet, &set);
        get_dec(m, id, D_Binding, &bind);
        return std::to_string(tex_slot(set, bind));
      }
      return "(&ctx.g" + std::to_string(id) + ")";
    }
    return "v" + std::to_string(id);
  }

  uint32_t tex_slot(uint32_t set, uint32_t bind)
  {
    auto it = tex_slots->find({set, bind});
    if(it != tex_slots->end())
      return it->second;
    uint32_t s = (uint32_t)tex_slots->size();
    (*tex_slots)[{set, bind}] = s;
    tex_list->push_back({set, bind});
    return s;
  }

  uint32_t ubo_slot(uint32_t set, uint32_t bind)
  {
    auto it = ubo_slots->find({set, bind});
    if(it != ubo_slots->end())
      return it->second;
    uint32_t s = (uint32_t)ubo_slots->size();
    (*ubo_slots)[{set, bind}] = s;
    ubo_list->push_back({set, bind});
    return s;
  }

  std::string scalar_const(uint32_t tid, uint32_t word)
  {
    const Type &t = T(tid);
    if(t.k == K_FLOAT)
      return fbits(word);
    if(t.k == K_BOOL)
      return word ? "true" : "false";
    if(t.k == K_INT)
      return t.sign ? "(int)" + std::to_string((int32_t)word) : std::to_string(word) + "u";
    return std::to_string(word);
  }

  std::string const_expr(uint32_t id)
  {
    const auto &c = m.consts.at(id);
    const Type &t = T(c.first);
    if(!m.composite_consts.count(id))
    {
      if(c.second.empty())
        return ctype(c.first) + "{}";
      return scalar_const(c.first, c.second[0]);
    }
    std::string s = ctype(c.first) + "{{";
    for(size_t i = 0; i < c.second.size(); i++)
      s += (i ? ", " : "") + val(c.second[i]);
    s += "}}";
    (void)t;
    return s;
  }

  /* component i of value id (scalars ignore i) */
  std::string comp(uint32_t id, uint32_t i)
  {
    uint32_t tid = m.rtype.count(id) ? m.rtype.at(id) : 0;
    if(T(tid).k == K_VEC)
      return val(id) + "[" + std::to_string(i) + "]";
    return val(id);
  }

  std::string lhs(uint32_t id, uint32_t i, uint32_t tid)
  {
    if(T(tid).k == K_VEC)
      return "v" + std::to_string(id) + "[" + std::to_string(i) + "]";
    return "v" + std::to_string(id);
  }

  /* statements loading a value of type tid from a block byte pointer */
  void block_load(std::ostringstream &o, const std::string &dst, uint32_t tid, const std::string &p,
                  uint32_t mstride, uint32_t rowmajor, int depth = 0)
  {
    const Type &t = T(tid);
    switch(t.k)
    {
      case K_FLOAT: o << "  " << dst << " = *(const float *)(" << p << ");\n"; break;
      case K_INT: o << "  " << dst << " = *(const " << ctype(tid) << " *)(" << p << ");\n"; break;
      case K_BOOL: o << "  " << dst << " = *(const unsigned *)(" << p << ") != 0u;\n"; break;
      case K_VEC:
        for(uint32_t i = 0; i < t.count; i++)
          block_load(o, dst + "[" + std::to_string(i) + "]", t.elem,
                     "(" + p + ") + " + std::to_string(i * 4), 0, 0, depth + 1);
        break;
      case K_MAT:
      {
        uint32_t rows = T(t.elem).count, stride = mstride ? mstride : 16;
        for(uint32_t c = 0; c < t.count; c++)
          for(uint32_t r = 0; r < rows; r++)
          {
            uint32_t off = rowmajor ? r * stride + c * 4 : c * stride + r * 4;
            o << "  " << dst << "[" << c << "][" << r << "] = *(const float *)((" << p << ") + "
              << off << ");\n";
          }
        break;
      }
      case K_STRUCT:
        for(size_t i = 0; i < t.members.size(); i++)
        {
          uint32_t off = 0, ms = 0;
          get_mdec(m, tid, (uint32_t)i, D_Offset, &off);
          get_mdec(m, tid, (uint32_t)i, D_MatrixStride, &ms);
          uint32_t rm = get_mdec(m, tid, (uint32_t)i, D_RowMajor, nullptr) ? 1 : 0;
          block_load(o, dst + ".m" + std::to_string(i), t.members[i],
                     "(" + p + ") + " + std::to_string(off), ms, rm, depth + 1);
        }
        break;
      case K_ARR:
      {
        uint32_t as = 0;
        get_dec(m, tid, D_ArrayStride, &as);
        for(uint32_t i = 0; i < t.count; i++)
          block_load(o, dst + "[" + std::to_string(i) + "]", t.elem,
                     "(" + p + ") + " + std::to_string(i * as), mstride, rowmajor, depth + 1);
        break;
      }
      default: err = "unsupported block member type"; break;
    }
  }

  BlockPtr block_root(uint32_t var_id)
  {
    const Var &v = m.vars.at(var_id);
    BlockPtr b;
    b.type = T(v.type).elem;
    b.mstride = 0;
    b.rowmajor = 0;
    return b;
  }

  bool is_block_ptr(uint32_t id)
  {
    auto v = m.vars.find(id);
    if(v != m.vars.end())
      return is_block_storage(v->second.storage);
    return bptr.count(id) != 0;
  }

  BlockPtr block_info(uint32_t id)
  {
    auto v = m.vars.find(id);
    if(v != m.vars.end())
      return block_root(id);
    return bptr.at(id);
  }

  bool is_uniform_constant(uint32_t id)
  {
    auto v = m.vars.find(id);
    return v != m.vars.end() && v->second.storage == SC_UniformConstant;
  }

  /* trace a sample coordinate back to a fragment input slot (for the per-triangle LOD) */
  int trace_slot(uint32_t id)
  {
    auto d = m.defs.find(id);
    if(d == m.defs.end())
      return -1;
    const Inst &in = *d->second;
    if(in.op == OpLoad)
    {
      auto s = fs_slot_of_var.find(in.w[2]);
      return s == fs_slot_of_var.end() ? -1 : (int)s->second;
    }
    if(in.op == OpVectorShuffle && in.w.size() >= 6)
    {
      int base = trace_slot(in.w[2]);
      uint32_t n0 = ncomp(m.rtype.at(in.w[2]));
      if(base >= 0 && in.w[4] < n0 && in.w[5] == in.w[4] + 1)
        return base + (int)in.w[4];
    }
    if(in.op == OpCopyObject)
      return trace_slot(in.w[2]);
    return -1;
  }

  void emit_function(const Func &f, bool is_entry);
  bool emit_inst(std::ostringstream &o, const Inst &in, const Func &f,
                 std::map<uint32_t, std::vector<std::pair<uint32_t, uint32_t>>> &phis);
};

const char *kPrelude = R"VGX(
#ifndef VGX_TRANSLATED_PRELUDE
#define VGX_TRANSLATED_PRELUDE
template <typename T, int N> struct vgx_v {
  T v[N];
  __device__ __forceinline__ T &operator[](int i) { return v[i]; }
  __device__ __forceinline__ const T &operator[](int i) const { return v[i]; }
};
template <int C, int R> struct vgx_m {
  vgx_v<float, R> c[C];
  __device__ __forceinline__ vgx_v<float, R> &operator[](int i) { return c[i]; }
  __device__ __forceinline__ const vgx_v<float, R> &operator[](int i) const { return c[i]; }
};
template <typename T, int N> struct vgx_a {
  T v[N];
  __device__ __forceinline__ T &operator[](int i) { return v[i]; }
  __device__ __forceinline__ const T &operator[](int i) const { return v[i]; }
};
#endif
)VGX";

void Gen::emit_function(const Func &f, bool is_entry)
{
  /* declarations of every result id and every function-scope variable */
  std::ostringstream decl, body;
  std::set<uint32_t> declared;
  std::map<uint32_t, std::vector<std::pair<uint32_t, uint32_t>>> phis; /* label -> (phi id, value from pred) */
  std::map<uint32_t, std::vector<std::pair<uint32_t, uint32_t>>> phi_sources; /* (label) */
  uint32_t cur_label = 0;
  for(const Inst &in : f.body)
  {
    if(in.op == OpLabel)
      cur_label = in.w[0];
    if(in.op == OpPhi)
    {
      for(size_t k = 2; k + 1 < in.w.size(); k += 2)
        phis[in.w[k + 1]].push_back({in.w[1], in.w[k]}); /* pred label -> (phi, value) */
      decl << "  " << ctype(in.w[0]) << " phi_tmp" << in.w[1] << ";\n";
    }
    if(in.op == OpVariable)
    {
      const Type &pt = T(in.w[0]);
      decl << "  " << ctype(pt.elem) << " var" << in.w[1] << ";\n";
      decl << "  " << ctype(in.w[0]) << " v" << in.w[1] << " = &var" << in.w[1] << ";\n";
      declared.insert(in.w[1]);
      continue;
    }
    if(has_result_type(in.op) && in.w.size() >= 2 && !declared.count(in.w[1]))
    {
      const Type &rt = T(in.w[0]);
      if(rt.k != K_VOID)
        decl << "  " << ctype(in.w[0]) << " v" << in.w[1] << ";\n";
      declared.insert(in.w[1]);
    }
  }
  (void)cur_label;
  for(const Inst &in : f.body)
  {
    if(!emit_inst(body, in, f, phis))
      return;
  }
  std::ostringstream sig;
  sig << "__device__ static " << ctype(f.ret) << " " << ns << "f" << f.id << "(" << ns << "Ctx &ctx";
  for(uint32_t p : f.params)
    sig << ", " << ctype(m.rtype.at(p)) << " v" << p;
  sig << ")";
  out << sig.str() << "\n{\n" << decl.str() << body.str() << "}\n";
  (void)is_entry;
}

bool Gen::emit_inst(std::ostringstream &o, const Inst &in, const Func &f,
                    std::map<uint32_t, std::vector<std::pair<uint32_t, uint32_t>>> &phis)
{
  const std::vector<uint32_t> &w = in.w;
  static uint32_t cur_block = 0;
  auto rt = [&]() { return w[0]; };
  auto id = [&]() { return w[1]; };
  auto n_of = [&](uint32_t tid) { return ncomp(tid); };
  auto branch_to = [&](uint32_t target) {
    std::ostringstream s;
    auto it = phis.find(cur_block);
    if(it != phis.end())
    {
      /* parallel copy into the target's phis */
      std::vector<std::pair<uint32_t, uint32_t>> mine;
      for(auto &pv : it->second)
      {
        auto d = m.defs.find(pv.first);
        if(d == m.defs.end())
          continue;
        /* only phis that live in `target` */
        mine.push_back(pv);
      }
      for(auto &pv : mine)
        s << "phi_tmp" << pv.first << " = " << val(pv.second) << "; ";
      for(auto &pv : mine)
        s << "v" << pv.first << " = phi_tmp" << pv.first << "; ";
    }
    s << "goto L" << target << ";";
    return s.str();
  };
  std::string ind = "  ";
  switch(in.op)
  {
    case OpLabel:
      cur_block = w[0];
      o << "L" << w[0] << ":;\n";
      return true;
    case OpBranch: o << ind << "{ " << branch_to(w[0]) << " }\n"; return true;
    case OpBranchConditional:
      o << ind << "if(" << val(w[0]) << ") { " << branch_to(w[1]) << " } else { " << branch_to(w[2])
        << " }\n";
      return true;
    case OpSwitch:
    {
      o << ind << "switch(" << val(w[0]) << ") {";
      for(size_t k = 2; k + 1 < w.size(); k += 2)
        o << " case " << (int32_t)w[k] << ": { " << branch_to(w[k + 1]) << " }";
      o << " default: { " << branch_to(w[1]) << " } }\n";
      return true;
    }
    case OpSelectionMerge: case OpLoopMerge: case OpNop: case OpLine: return true;
    case OpReturn: o << ind << "return;\n"; return true;
    case OpReturnValue: o << ind << "return " << val(w[0]) << ";\n"; return true;
    case OpKill: o << ind << "return;\n"; return true;
    case OpUnreachable: o << ind << "return" << (T(f.ret).k == K_VOID ? "" : " {}") << ";\n"; return true;
    case OpPhi:
      /* assigned on the incoming edges; declare the parallel-copy temporary */
      o << ind << "/* phi v" << id() << " */\n";
      return true;
    case OpVariable:
      if(w.size() > 3)
        o << ind << "var" << id() << " = " << val(w[3]) << ";\n";
      return true;
    case OpLoad:
    {
      uint32_t p = w[2];
      if(is_uniform_constant(p))
      {
        o << ind << "v" << id() << " = " << val(p) << ";\n";
        return true;
      }
      if(is_block_ptr(p))
      {
        BlockPtr b = block_info(p);
        block_load(o, "v" + std::to_string(id()), rt(), val(p), b.mstride, b.rowmajor);
        return true;
      }
      o << ind << "v" << id() << " = *" << val(p) << ";\n";
      return true;
    }
    case OpStore:
      if(is_block_ptr(w[0]))
      {
        err = "stores to uniform blocks are not supported";
        return false;
      }
      o << ind << "*" << val(w[0]) << " = " << val(w[1]) << ";\n";
      return true;
    case OpAccessChain:
    case OpInBoundsAccessChain:
    {
      uint32_t base = w[2];
      if(is_block_ptr(base))
      {
        BlockPtr b = block_info(base);
        std::string off = "0";
        uint32_t ty = b.type, ms = b.mstride, rm = b.rowmajor;
        for(size_t k = 3; k < w.size(); k++)
        {
          const Type &t = T(ty);
          if(t.k == K_STRUCT)
          {
            uint32_t mi = m.consts.at(w[k]).second[0], moff = 0;
            get_mdec(m, ty, mi, D_Offset, &moff);
            ms = 0;
            get_mdec(m, ty, mi, D_MatrixStride, &ms);
            rm = get_mdec(m, ty, mi, D_RowMajor, nullptr) ? 1 : 0;
            off += " + " + std::to_string(moff);
            ty = t.members[mi];
          }
          else if(t.k == K_ARR || t.k == K_RARR)
          {
            uint32_t as = 0;
            get_dec(m, ty, D_ArrayStride, &as);
            off += " + (" + val(w[k]) + ") * " + std::to_string(as);
            ty = t.elem;
          }
          else if(t.k == K_MAT)
          {
            uint32_t stride = ms ? ms : 16;
            off += " + (" + val(w[k]) + ") * " + std::to_string(rm ? 4 : stride);
            ty = t.elem;
            if(rm)
            {
              err = "row-major column access is not supported";
              return false;
            }
          }
          else if(t.k == K_VEC)
          {
            off += " + (" + val(w[k]) + ") * 4";
            ty = t.elem;
          }
        }
        BlockPtr nb;
        nb.type = ty;
        nb.mstride = ms;
        nb.rowmajor = rm;
        bptr[id()] = nb;
        o << ind << "v" << id() << " = " << val(base) << " + (" << off << ");\n";
        return true;
      }
      std::string e = "(*" + val(base) + ")";
      uint32_t ty = T(m.rtype.at(base)).elem;
      for(size_t k = 3; k < w.size(); k++)
      {
        const Type &t = T(ty);
        if(t.k == K_STRUCT)
        {
          uint32_t mi = m.consts.at(w[k]).second[0];
          e += ".m" + std::to_string(mi);
          ty = t.members[mi];
        }
        else
        {
          e += "[" + val(w[k]) + "]";
          ty = t.elem;
        }
      }
      o << ind << "v" << id() << " = &" << e << ";\n";
      return true;
    }
    case OpFunctionCall:
    {
      o << ind;
      if(T(rt()).k != K_VOID)
        o << "v" << id() << " = ";
      o << ns << "f" << w[2] << "(ctx";
      for(size_t k = 3; k < w.size(); k++)
        o << ", " << val(w[k]);
      o << ");\n";
      return true;
    }
    case OpCopyObject: o << ind << "v" << id() << " = " << val(w[2]) << ";\n"; return true;
    case OpCompositeExtract:
    {
      std::string e = val(w[2]);
      uint32_t ty = m.rtype.at(w[2]);
      for(size_t k = 3; k < w.size(); k++)
      {
        const Type &t = T(ty);
        if(t.k == K_STRUCT)
        {
          e += ".m" + std::to_string(w[k]);
          ty = t.members[w[k]];
        }
        else
        {
          e += "[" + std::to_string(w[k]) + "]";
          ty = t.elem;
        }
      }
      o << ind << "v" << id() << " = " << e << ";\n";
      return true;
    }
    case OpCompositeInsert:
    {
      o << ind << "v" << id() << " = " << val(w[3]) << ";\n";
      std::string e = "v" + std::to_string(id());
      uint32_t ty = rt();
      for(size_t k = 4; k < w.size(); k++)
      {
        const Type &t = T(ty);
        if(t.k == K_STRUCT)
        {
          e += ".m" + std::to_string(w[k]);
          ty = t.members[w[k]];
        }
        else
        {
          e += "[" + std::to_string(w[k]) + "]";
          ty = t.elem;
        }
      }
      o << ind << e << " = " << val(w[2]) << ";\n";
      return true;
    }
    case OpCompositeConstruct:
    {
      const Type &t = T(rt());
      if(t.k == K_VEC)
      {
        /* constituents may be scalars or vectors (flattened in order) */
        uint32_t c = 0;
        for(size_t k = 2; k < w.size(); k++)
        {
          uint32_t ct = m.rtype.at(w[k]);
          uint32_t n = n_of(ct);
          for(uint32_t i = 0; i < n && c < t.count; i++, c++)
            o << ind << "v" << id() << "[" << c << "] = " << comp(w[k], i) << ";\n";
        }
      }
      else if(t.k == K_STRUCT)
      {
        for(size_t k = 2; k < w.size(); k++)
          o << ind << "v" << id() << ".m" << (k - 2) << " = " << val(w[k]) << ";\n";
      }
      else
      {
        for(size_t k = 2; k < w.size(); k++)
          o << ind << "v" << id() << "[" << (k - 2) << "] = " << val(w[k]) << ";\n";
      }
      return true;
    }
    case OpVectorShuffle:
    {
      uint32_t na = n_of(m.rtype.at(w[2]));
      for(size_t k = 4; k < w.size(); k++)
      {
        uint32_t s = w[k];
        std::string src = s == 0xffffffffu ? "0" : (s < na ? comp(w[2], s) : comp(w[3], s - na));
        o << ind << "v" << id() << "[" << (k - 4) << "] = " << src << ";\n";
      }
      return true;
    }
    case OpVectorExtractDynamic:
      o << ind << "v" << id() << " = " << val(w[2]) << "[" << val(w[3]) << "];\n";
      return true;
    case OpTranspose:
    {
      const Type &t = T(rt());
      uint32_t rows = T(t.elem).count;
      for(uint32_t c = 0; c < t.count; c++)
        for(uint32_t r = 0; r < rows; r++)
          o << ind << "v" << id() << "[" << c << "][" << r << "] = " << val(w[2]) << "[" << r << "]["
            << c << "];\n";
      return true;
    }
    case OpSampledImage: o << ind << "v" << id() << " = " << val(w[2]) << ";\n"; return true;
    case OpImageSampleImplicitLod:
    case OpImageSampleExplicitLod:
    {
      uint32_t img = w[2], coord = w[3];
      samples++;
      std::string lod = "ctx.lod";
      if(in.op == OpImageSampleExplicitLod && w.size() > 5 && (w[4] & 0x2))
        lod = val(w[5]);
      if(fragment && in.op == OpImageSampleImplicitLod && lod_slot < 0)
      {
        int s = trace_slot(coord);
        /* the texture slot of this sample, when it is a direct descriptor load */
        auto d = m.defs.find(img);
        if(s >= 0 && d != m.defs.end() && d->second->op == OpLoad && is_uniform_constant(d->second->w[2]))
        {
          uint32_t set = 0, bind = 0;
          get_dec(m, d->second->w[2], D_DescriptorSet, &set);
          get_dec(m, d->second->w[2], D_Binding, &bind);
          lod_slot = s;
          lod_tex = (int)tex_slot(set, bind);
        }
      }
      const Type &it = T(m.rtype.at(img));
      if(it.dim == 3)
      {
        /* sample_cube_wrapped (texture_sampling.cpp:186-250): face from the major axis */
        o << ind << "{ float4 t_ = vgx_sample_cube(*ctx.D, (u32)(" << val(img) << "), "
          << comp(coord, 0) << ", " << comp(coord, 1) << ", " << comp(coord, 2) << "); v" << id()
          << "[0] = t_.x; v" << id() << "[1] = t_.y; v" << id() << "[2] = t_.z; v" << id()
          << "[3] = t_.w; }\n";
        return true;
      }
      o << ind << "{ float4 t_ = vgx_sample(*ctx.D, (u32)(" << val(img) << "), " << comp(coord, 0)
        << ", " << comp(coord, 1) << ", " << lod << "); v" << id() << "[0] = t_.x; v" << id()
        << "[1] = t_.y; v" << id() << "[2] = t_.z; v" << id() << "[3] = t_.w; }\n";
      return true;
    }
    case OpDot:
    {
      uint32_t n = n_of(m.rtype.at(w[2]));
      o << ind << "v" << id() << " = " << comp(w[2], 0) << " * " << comp(w[3], 0) << ";\n";
      for(uint32_t i = 1; i < n; i++)
        o << ind << "v" << id() << " = v" << id() << " + " << comp(w[2], i) << " * " << comp(w[3], i)
          << ";\n";
      return true;
    }
    case OpVectorTimesScalar:
    {
      uint32_t n = n_of(rt());
      for(uint32_t i = 0; i < n; i++)
        o << ind << lhs(id(), i, rt()) << " = " << comp(w[2], i) << " * " << val(w[3]) << ";\n";
      return true;
    }
    case OpMatrixTimesScalar:
    {
      const Type &t = T(rt());
      uint32_t rows = T(t.elem).count;
      for(uint32_t c = 0; c < t.count; c++)
        for(uint32_t r = 0; r < rows; r++)
          o << ind << "v" << id() << "[" << c << "][" << r << "] = " << val(w[2]) << "[" << c << "]["
            << r << "] * " << val(w[3]) << ";\n";
      return true;
    }
    case OpMatrixTimesVector:
    {
      /* Float4x4TimesVec4 / Float3x3TimesVec3 (spirv_compile.cpp:423-441): out[r] starts at 0.0f */
      const Type &mt = T(m.rtype.at(w[2]));
      uint32_t rows = n_of(rt());
      for(uint32_t r = 0; r < rows; r++)
      {
        o << ind << lhs(id(), r, rt()) << " = 0.0f;\n";
        for(uint32_t c = 0; c < mt.count; c++)
          o << ind << lhs(id(), r, rt()) << " = " << lhs(id(), r, rt()) << " + " << val(w[2]) << "["
            << c << "][" << r << "] * " << comp(w[3], c) << ";\n";
      }
      return true;
    }
    case OpVectorTimesMatrix:
    {
      /* Vec4TimesFloat4x4 (:443-461): out[j] = 0.0f + sum_i m[j][i] * v[i] */
      const Type &mt = T(m.rtype.at(w[3]));
      uint32_t rows = T(mt.elem).count;
      for(uint32_t j = 0; j < mt.count; j++)
      {
        o << ind << lhs(id(), j, rt()) << " = 0.0f;\n";
        for(uint32_t i = 0; i < rows; i++)
          o << ind << lhs(id(), j, rt()) << " = " << lhs(id(), j, rt()) << " + " << val(w[3]) << "["
            << j << "][" << i << "] * " << comp(w[2], i) << ";\n";
      }
      return true;
    }
    case OpMatrixTimesMatrix:
    {
      /* Float4x4TimesFloat4x4 (:463-473): out[x][y] = b[x][0]*a[0][y] + b[x][1]*a[1][y] + ... */
      const Type &t = T(rt());
      const Type &at = T(m.rtype.at(w[2]));
      uint32_t rows = T(t.elem).count;
      for(uint32_t x = 0; x < t.count; x++)
        for(uint32_t y = 0; y < rows; y++)
        {
          o << ind << "v" << id() << "[" << x << "][" << y << "] = ";
          for(uint32_t k = 0; k < at.count; k++)
          {
            if(k)
              o << " + ";
            o << val(w[3]) << "[" << x << "][" << k << "] * " << val(w[2]) << "[" << k << "][" << y << "]";
          }
          o << ";\n";
        }
      /* left-to-right evaluation of the sum above is the reference's order */
      return true;
    }
    case OpSelect:
    {
      uint32_t n = n_of(rt());
      uint32_t ct = m.rtype.at(w[2]);
      for(uint32_t i = 0; i < n; i++)
        o << ind << lhs(id(), i, rt()) << " = " << (T(ct).k == K_VEC ? comp(w[2], i) : val(w[2]))
          << " ? " << comp(w[3], i) << " : " << comp(w[4], i) << ";\n";
      return true;
    }
    case OpExtInst:
    {
      if(w[2] != m.glsl)
      {
        err = "unknown extended instruction set";
        return false;
      }
      uint32_t inst = w[3];
      uint32_t n = n_of(rt());
      auto A = [&](int k) { return w[4 + k]; };
      switch(inst)
      {
        case 40: /* FMax: select(a > b, a, b) */
        case 37: /* FMin: select(a < b, a, b) */
          for(uint32_t i = 0; i < n; i++)
            o << ind << lhs(id(), i, rt()) << " = (" << comp(A(0), i) << (inst == 40 ? " > " : " < ")
              << comp(A(1), i) << ") ? " << comp(A(0), i) << " : " << comp(A(1), i) << ";\n";
          return true;
        case 43: /* FClamp (:1546-1559) */
          for(uint32_t i = 0; i < n; i++)
          {
            std::string x = comp(A(0), i), lo = comp(A(1), i), hi = comp(A(2), i);
            o << ind << "{ float u_ = (" << x << " < " << hi << ") ? " << x << " : " << hi << "; "
              << lhs(id(), i, rt()) << " = (u_ > " << lo << ") ? u_ : " << lo << "; }\n";
          }
          return true;
        case 46: /* FMix: (1 - a) * x + a * y (:1561-1578) */
          for(uint32_t i = 0; i < n; i++)
            o << ind << lhs(id(), i, rt()) << " = (1.0f - " << comp(A(2), i) << ") * " << comp(A(0), i)
              << " + " << comp(A(2), i) << " * " << comp(A(1), i) << ";\n";
          return true;
        case 13: case 14: case 31: case 32: case 4: case 8: case 9: case 10: case 27: case 28:
        case 29: case 30: case 15: case 6:
        {
          for(uint32_t i = 0; i < n; i++)
          {
            std::string x = comp(A(0), i), e;
            switch(inst)
            {
              case 13: e = "sinf(" + x + ")"; break;
              case 14: e = "cosf(" + x + ")"; break;
              case 31: e = "sqrtf(" + x + ")"; break;
              case 32: e = "1.0f / sqrtf(" + x + ")"; break;
              case 4: e = "fabsf(" + x + ")"; break;
              case 8: e = "floorf(" + x + ")"; break;
              case 9: e = "ceilf(" + x + ")"; break;
              case 10: e = x + " - floorf(" + x + ")"; break;
              case 27: e = "expf(" + x + ")"; break;
              case 28: e = "logf(" + x + ")"; break;
              case 29: e = "exp2f(" + x + ")"; break;
              case 30: e = "log2f(" + x + ")"; break;
              case 15: e = "tanf(" + x + ")"; break;
              case 6: e = "(" + x + " > 0.0f ? 1.0f : (" + x + " < 0.0f ? -1.0f : 0.0f))"; break;
            }
            o << ind << lhs(id(), i, rt()) << " = " << e << ";\n";
          }
          return true;
        }
        case 26: /* Pow */
          for(uint32_t i = 0; i < n; i++)
            o << ind << lhs(id(), i, rt()) << " = powf(" << comp(A(0), i) << ", " << comp(A(1), i)
              << ");\n";
          return true;
        case 69: /* Normalize: a * (1 / sqrt(dot(a, a))) (:1632-1647) */
        case 66: /* Length: sqrt(dot(a, a)) */
        {
          uint32_t na = n_of(m.rtype.at(A(0)));
          o << ind << "{ float s_ = " << comp(A(0), 0) << " * " << comp(A(0), 0) << ";";
          for(uint32_t i = 1; i < na; i++)
            o << " s_ = s_ + " << comp(A(0), i) << " * " << comp(A(0), i) << ";";
          if(inst == 66)
          {
            o << " v" << id() << " = sqrtf(s_); }\n";
          }
          else
          {
            o << " float l_ = sqrtf(s_); float i_ = 1.0f / l_;";
            for(uint32_t i = 0; i < na; i++)
              o << " " << lhs(id(), i, rt()) << " = " << comp(A(0), i) << " * i_;";
            o << " }\n";
          }
          return true;
        }
        case 67: /* Distance */
        {
          uint32_t na = n_of(m.rtype.at(A(0)));
          o << ind << "{ float s_ = 0.0f;";
          for(uint32_t i = 0; i < na; i++)
            o << " { float d_ = " << comp(A(0), i) << " - " << comp(A(1), i) << "; s_ = " << (i ? "s_ + " : "")
              << "d_ * d_; }";
          o << " v" << id() << " = sqrtf(s_); }\n";
          return true;
        }
        case 68: /* Cross (correct semantics; the reference returns its first argument) */
          o << ind << "v" << id() << "[0] = " << comp(A(0), 1) << " * " << comp(A(1), 2) << " - "
            << comp(A(1), 1) << " * " << comp(A(0), 2) << ";\n";
          o << ind << "v" << id() << "[1] = " << comp(A(0), 2) << " * " << comp(A(1), 0) << " - "
            << comp(A(1), 2) << " * " << comp(A(0), 0) << ";\n";
          o << ind << "v" << id() << "[2] = " << comp(A(0), 0) << " * " << comp(A(1), 1) << " - "
            << comp(A(1), 0) << " * " << comp(A(0), 1) << ";\n";
          return true;
        case 71: /* Reflect: I - (dot(I, N) * 2) * N (:1674-1686) */
        {
          uint32_t na = n_of(m.rtype.at(A(0)));
          o << ind << "{ float d_ = " << comp(A(0), 0) << " * " << comp(A(1), 0) << ";";
          for(uint32_t i = 1; i < na; i++)
            o << " d_ = d_ + " << comp(A(0), i) << " * " << comp(A(1), i) << ";";
          o << " float d2_ = d_ * 2.0f;";
          for(uint32_t i = 0; i < na; i++)
            o << " " << lhs(id(), i, rt()) << " = " << comp(A(0), i) << " - d2_ * " << comp(A(1), i) << ";";
          o << " }\n";
          return true;
        }
        case 34: /* MatrixInverse (correct inverse; the reference transposes) */
        {
          const Type &t = T(rt());
          if(t.count != 4)
          {
            err = "MatrixInverse supports 4x4 only";
            return false;
          }
          std::string a = val(A(0));
          o << ind << "{ float m_[16], r_[16];";
          for(int c = 0; c < 4; c++)
            for(int r = 0; r < 4; r++)
              o << " m_[" << c * 4 + r << "] = " << a << "[" << c << "][" << r << "];";
          o << " vgx_inverse4(m_, r_);";
          for(int c = 0; c < 4; c++)
            for(int r = 0; r < 4; r++)
              o << " v" << id() << "[" << c << "][" << r << "] = r_[" << c * 4 + r << "];";
          o << " }\n";
          return true;
        }
        default:
          err = "unsupported GLSL.std.450 instruction " + std::to_string(inst);
          return false;
      }
    }
    default: break;
  }

  /* component-wise arithmetic, comparisons, conversions */
  if(!has_result_type(in.op) || w.size() < 3)
  {
    err = "unsupported opcode " + std::to_string(in.op);
    return false;
  }
  uint32_t n = n_of(rt());
  const char *bin = nullptr;
  const char *un = nullptr;
  std::string cast;
  switch(in.op)
  {
    case OpFAdd: case OpIAdd: bin = "+"; break;
    case OpFSub: case OpISub: bin = "-"; break;
    case OpFMul: case OpIMul: bin = "*"; break;
    case OpFDiv: case OpSDiv: case OpUDiv: bin = "/"; break;
    case OpSRem: case OpUMod: bin = "%"; break;
    case OpBitwiseAnd: case OpLogicalAnd: bin = in.op == OpLogicalAnd ? "&&" : "&"; break;
    case OpBitwiseOr: case OpLogicalOr: bin = in.op == OpLogicalOr ? "||" : "|"; break;
    case OpBitwiseXor: bin = "^"; break;
    case OpShiftLeftLogical: bin = "<<"; break;
    case OpShiftRightArithmetic: bin = ">>"; break;
    case OpFOrdLessThan: case OpSLessThan: case OpULessThan: case OpFUnordLessThan: bin = "<"; break;
    case OpFOrdGreaterThan: case OpSGreaterThan: case OpUGreaterThan: case OpFUnordGreaterThan: bin = ">"; break;
    case OpFOrdLessThanEqual: case OpSLessThanEqual: case OpULessThanEqual: case OpFUnordLessThanEqual: bin = "<="; break;
    case OpFOrdGreaterThanEqual: case OpSGreaterThanEqual: case OpUGreaterThanEqual: case OpFUnordGreaterThanEqual: bin = ">="; break;
    case OpFOrdEqual: case OpIEqual: case OpLogicalEqual: case OpFUnordEqual: bin = "=="; break;
    case OpFOrdNotEqual: case OpINotEqual: case OpLogicalNotEqual: case OpFUnordNotEqual: bin = "!="; break;
    case OpFNegate: case OpSNegate: un = "-"; break;
    case OpNot: un = "~"; break;
    case OpLogicalNot: un = "!"; break;
    case OpConvertSToF: cast = "(float)(int)"; break;
    case OpConvertUToF: cast = "(float)(unsigned)"; break;
    case OpConvertFToS: cast = "(int)"; break;
    case OpConvertFToU: cast = "(unsigned)"; break;
    case OpDPdx: case OpDPdy:
      /* no helper invocations on this path: derivatives are zero */
      for(uint32_t i = 0; i < n; i++)
        o << ind << lhs(id(), i, rt()) << " = 0.0f;\n";
      return true;
    case OpFMod:
      for(uint32_t i = 0; i < n; i++)
        o << ind << lhs(id(), i, rt()) << " = " << comp(w[2], i) << " - " << comp(w[3], i)
          << " * floorf(" << comp(w[2], i) << " / " << comp(w[3], i) << ");\n";
      return true;
    case OpFRem:
      for(uint32_t i = 0; i < n; i++)
        o << ind << lhs(id(), i, rt()) << " = fmodf(" << comp(w[2], i) << ", " << comp(w[3], i) << ");\n";
      return true;
    case OpShiftRightLogical:
      for(uint32_t i = 0; i < n; i++)
        o << ind << lhs(id(), i, rt()) << " = (" << ctype(scalar_of(rt())) << ")((unsigned)" << comp(w[2], i)
          << " >> " << comp(w[3], i) << ");\n";
      return true;
    case OpBitcast:
    {
      uint32_t dst = scalar_of(rt()), src = scalar_of(m.rtype.at(w[2]));
      for(uint32_t i = 0; i < n; i++)
      {
        std::string x = comp(w[2], i), e;
        if(T(dst).k == K_FLOAT && T(src).k == K_INT)
          e = "__int_as_float((int)" + x + ")";
        else if(T(dst).k == K_INT && T(src).k == K_FLOAT)
          e = "(" + ctype(dst) + ")__float_as_int(" + x + ")";
        else
          e = "(" + ctype(dst) + ")" + x;
        o << ind << lhs(id(), i, rt()) << " = " << e << ";\n";
      }
      return true;
    }
    case OpAny:
    case OpAll:
    {
      uint32_t na = n_of(m.rtype.at(w[2]));
      o << ind << "v" << id() << " = ";
      for(uint32_t i = 0; i < na; i++)
        o << (i ? (in.op == OpAny ? " || " : " && ") : "") << comp(w[2], i);
      o << ";\n";
      return true;
    }
    default:
      err = "unsupported opcode " + std::to_string(in.op);
      return false;
  }
  for(uint32_t i = 0; i < n; i++)
  {
    if(bin)
    {
      std::string a = comp(w[2], i), b = comp(w[3], i);
      if(in.op == OpUDiv || in.op == OpUMod || in.op == OpULessThan || in.op == OpUGreaterThan ||
         in.op == OpULessThanEqual || in.op == OpUGreaterThanEqual)
      {
        a = "(unsigned)" + a;
        b = "(unsigned)" + b;
      }
      o << ind << lhs(id(), i, rt()) << " = " << a << " " << bin << " " << b << ";\n";
    }
    else if(un)
      o << ind << lhs(id(), i, rt()) << " = " << un << comp(w[2], i) << ";\n";
    else
      o << ind << lhs(id(), i, rt()) << " = " << cast << comp(w[2], i) << ";\n";
  }
  return true;
}

const Entry *find_entry(const Module *m, const char *name, uint32_t model)
{
  for(const Entry &e : m->entries)
    if(e.name == name && e.model == model)
      return &e;
  return nullptr;
}

/* Emit the namespace (structs, context, functions) of one stage. */
bool emit_stage(Gen &g, const Entry &e)
{
  std::ostringstream structs;
  for(auto &kv : g.m.types)
    if(kv.second.k == K_STRUCT)
      g.emit_struct(kv.first, structs);
  std::ostringstream ctx;
  ctx << "struct " << g.ns << "Ctx { const VgxDraw *D; float lod;";
  for(auto &kv : g.m.vars)
  {
    const Var &v = kv.second;
    if(v.storage == SC_Input || v.storage == SC_Output || v.storage == SC_Private ||
       v.storage == SC_Workgroup)
      ctx << " " << g.ctype(g.T(v.type).elem) << " g" << kv.first << ";";
  }
  ctx << " };\n";
  g.out << structs.str() << ctx.str();
  /* prototypes, then bodies */
  for(uint32_t fid : g.m.func_order)
  {
    const Func &f = g.m.funcs.at(fid);
    g.out << "__device__ static " << g.ctype(f.ret) << " " << g.ns << "f" << f.id << "(" << g.ns << "Ctx &ctx";
    for(uint32_t p : f.params)
      g.out << ", " << g.ctype(g.m.rtype.at(p)) << " v" << p;
    g.out << ");\n";
  }
  for(uint32_t fid : g.m.func_order)
  {
    g.emit_function(g.m.funcs.at(fid), fid == e.fn);
    if(!g.err.empty())
      return false;
  }
  return true;
}
}    // namespace

bool translate(const Module *vs, const char *vs_entry, const Module *fs, const char *fs_entry,
               Result &res, std::string &err)
{
  const Entry *ve = find_entry(vs, vs_entry, 0);
  const Entry *fe = find_entry(fs, fs_entry, 4);
  if(!ve || !fe)
  {
    err = "entry point not found for the vertex or fragment stage";
    return false;
  }
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> tex_slots, ubo_slots;
  res.textures.clear();
  res.ubos.clear();

  /* fragment inputs -> interpolation slots, in location order */
  std::vector<FsInput> fin;
  for(uint32_t vid : fe->iface)
  {
    auto it = fs->vars.find(vid);
    if(it == fs->vars.end() || it->second.storage != SC_Input)
      continue;
    uint32_t loc = 0;
    if(!get_dec(*fs, vid, D_Location, &loc))
    {
      err = "fragment built-in inputs are not supported (the reference has none)";
      return false;
    }
    const Type &pt = fs->types.at(it->second.type);
    uint32_t ty = pt.elem, elems = 1;
    if(fs->types.at(ty).k == K_ARR)
    {
      elems = fs->types.at(ty).count;
      ty = fs->types.at(ty).elem;
    }
    const Type &t = fs->types.at(ty);
    FsInput f;
    f.var = vid;
    f.loc = loc;
    f.elems = elems;
    f.is_int = (t.k == K_INT) || (t.k == K_VEC && fs->types.at(t.elem).k == K_INT);
    f.ncomp = t.k == K_VEC ? t.count : 1;
    f.slot = 0;
    fin.push_back(f);
  }
  std::sort(fin.begin(), fin.end(), [](const FsInput &a, const FsInput &b) { return a.loc < b.loc; });
  uint32_t k = 0;
  for(FsInput &f : fin)
  {
    f.slot = k;
    k += f.ncomp * f.elems;
  }
  res.k = k;

  std::ostringstream src;
  src << kPrelude;
  src << "__device__ __forceinline__ void vgx_inverse4(const float *m, float *o) {\n"
         "  float c[16];\n"
         "  for(int i = 0; i < 16; i++) c[i] = 0.0f;\n"
         "  c[0] = m[5]*m[10]*m[15] - m[5]*m[11]*m[14] - m[9]*m[6]*m[15] + m[9]*m[7]*m[14] + m[13]*m[6]*m[11] - m[13]*m[7]*m[10];\n"
         "  c[4] = -m[4]*m[10]*m[15] + m[4]*m[11]*m[14] + m[8]*m[6]*m[15] - m[8]*m[7]*m[14] - m[12]*m[6]*m[11] + m[12]*m[7]*m[10];\n"
         "  c[8] = m[4]*m[9]*m[15] - m[4]*m[11]*m[13] - m[8]*m[5]*m[15] + m[8]*m[7]*m[13] + m[12]*m[5]*m[11] - m[12]*m[7]*m[9];\n"
         "  c[12] = -m[4]*m[9]*m[14] + m[4]*m[10]*m[13] + m[8]*m[5]*m[14] - m[8]*m[6]*m[13] - m[12]*m[5]*m[10] + m[12]*m[6]*m[9];\n"
         "  c[1] = -m[1]*m[10]*m[15] + m[1]*m[11]*m[14] + m[9]*m[2]*m[15] - m[9]*m[3]*m[14] - m[13]*m[2]*m[11] + m[13]*m[3]*m[10];\n"
         "  c[5] = m[0]*m[10]*m[15] - m[0]*m[11]*m[14] - m[8]*m[2]*m[15] + m[8]*m[3]*m[14] + m[12]*m[2]*m[11] - m[12]*m[3]*m[10];\n"
         "  c[9] = -m[0]*m[9]*m[15] + m[0]*m[11]*m[13] + m[8]*m[1]*m[15] - m[8]*m[3]*m[13] - m[12]*m[1]*m[11] + m[12]*m[3]*m[9];\n"
         "  c[13] = m[0]*m[9]*m[14] - m[0]*m[10]*m[13] - m[8]*m[1]*m[14] + m[8]*m[2]*m[13] + m[12]*m[1]*m[10] - m[12]*m[2]*m[9];\n"
         "  c[2] = m[1]*m[6]*m[15] - m[1]*m[7]*m[14] - m[5]*m[2]*m[15] + m[5]*m[3]*m[14] + m[13]*m[2]*m[7] - m[13]*m[3]*m[6];\n"
         "  c[6] = -m[0]*m[6]*m[15] + m[0]*m[7]*m[14] + m[4]*m[2]*m[15] - m[4]*m[3]*m[14] - m[12]*m[2]*m[7] + m[12]*m[3]*m[6];\n"
         "  c[10] = m[0]*m[5]*m[15] - m[0]*m[7]*m[13] - m[4]*m[1]*m[15] + m[4]*m[3]*m[13] + m[12]*m[1]*m[7] - m[12]*m[3]*m[5];\n"
         "  c[14] = -m[0]*m[5]*m[14] + m[0]*m[6]*m[13] + m[4]*m[1]*m[14] - m[4]*m[2]*m[13] - m[12]*m[1]*m[6] + m[12]*m[2]*m[5];\n"
         "  c[3] = -m[1]*m[6]*m[11] + m[1]*m[7]*m[10] + m[5]*m[2]*m[11] - m[5]*m[3]*m[10] - m[9]*m[2]*m[7] + m[9]*m[3]*m[6];\n"
         "  c[7] = m[0]*m[6]*m[11] - m[0]*m[7]*m[10] - m[4]*m[2]*m[11] + m[4]*m[3]*m[10] + m[8]*m[2]*m[7] - m[8]*m[3]*m[6];\n"
         "  c[11] = -m[0]*m[5]*m[11] + m[0]*m[7]*m[9] + m[4]*m[1]*m[11] - m[4]*m[3]*m[9] - m[8]*m[1]*m[7] + m[8]*m[3]*m[5];\n"
         "  c[15] = m[0]*m[5]*m[10] - m[0]*m[6]*m[9] - m[4]*m[1]*m[10] + m[4]*m[2]*m[9] + m[8]*m[1]*m[6] - m[8]*m[2]*m[5];\n"
         "  float det = m[0]*c[0] + m[1]*c[4] + m[2]*c[8] + m[3]*c[12];\n"
         "  float inv = det != 0.0f ? 1.0f / det : 0.0f;\n"
         "  for(int i = 0; i < 16; i++) o[i] = c[i] * inv;\n"
         "}\n";

  /* fragment stage first: it fixes the slot layout and the LOD source */
  Gen gf(*fs);
  gf.ns = "fs_";
  gf.fragment = true;
  gf.tex_slots = &tex_slots;
  gf.ubo_slots = &ubo_slots;
  gf.tex_list = &res.textures;
  gf.ubo_list = &res.ubos;
  for(const FsInput &f : fin)
    if(!f.is_int && f.elems == 1)
      gf.fs_slot_of_var[f.var] = f.slot;
  if(!emit_stage(gf, *fe))
  {
    err = "fragment stage: " + gf.err;
    return false;
  }
  Gen gv(*vs);
  gv.ns = "vs_";
  gv.tex_slots = &tex_slots;
  gv.ubo_slots = &ubo_slots;
  gv.tex_list = &res.textures;
  gv.ubo_list = &res.ubos;
  if(!emit_stage(gv, *ve))
  {
    err = "vertex stage: " + gv.err;
    return false;
  }
  if(res.textures.size() > VGX_MAX_TEX_TRANSLATE || res.ubos.size() > VGX_MAX_UBO_TRANSLATE)
  {
    err = "too many descriptor bindings";
    return false;
  }
  res.lod_slot = gf.lod_slot;
  src << "#define VGX_K " << k << "\n";
  src << "#define VGX_LOD_SLOT " << gf.lod_slot << "\n";
  src << "#define VGX_LOD_TEX " << (gf.lod_tex < 0 ? 0 : gf.lod_tex) << "\n";
  /* fragment shaders without texture fetches are cheap enough to run inline */
  src << "#define VGX_FS_SAMPLES " << gf.samples << "\n";
  src << gv.out.str() << gf.out.str();

  /* vertex wrapper */
  src << "__device__ __forceinline__ void vgx_vs(const VgxDraw &D, u32 vertex_index, u32 instance_index, "
         "float4 &pos, float *out)\n{\n";
  src << "  vs_Ctx ctx;\n  ctx.D = &D;\n  ctx.lod = 0.0f;\n";
  std::map<uint32_t, uint32_t> vs_out_loc; /* location -> var */
  std::string pos_expr;
  for(uint32_t vid : ve->iface)
  {
    auto it = vs->vars.find(vid);
    if(it == vs->vars.end())
      continue;
    const Var &v = it->second;
    uint32_t ty = vs->types.at(v.type).elem;
    const Type &t = vs->types.at(ty);
    uint32_t loc = 0, bi = 0;
    if(v.storage == SC_Input)
    {
      if(get_dec(*vs, vid, D_BuiltIn, &bi))
      {
        if(bi == BI_VertexIndex || bi == BI_VertexId)
          src << "  ctx.g" << vid << " = (" << gv.ctype(ty) << ")vertex_index;\n";
        else if(bi == BI_InstanceIndex || bi == BI_InstanceId)
          /* the reference stores 0 (spirv_compile.cpp:1946-1949); the draw's
             first_instance is 0 there too, unless Vulkan draw parameters are on */
          src << "  ctx.g" << vid << " = (" << gv.ctype(ty) << ")instance_index;\n";
        else
        {
          err = "unsupported vertex built-in input";
          return false;
        }
        continue;
      }
      if(!get_dec(*vs, vid, D_Location, &loc))
        continue;
      src << "  { float4 a_ = vgx_fetch(D, " << loc << "u, vertex_index, instance_index); float f_[4] = {a_.x, a_.y, a_.z, a_.w};";
      bool isint = t.k == K_INT || (t.k == K_VEC && vs->types.at(t.elem).k == K_INT);
      uint32_t n = t.k == K_VEC ? t.count : 1;
      for(uint32_t i = 0; i < n; i++)
      {
        std::string dst = "ctx.g" + std::to_string(vid) + (t.k == K_VEC ? "[" + std::to_string(i) + "]" : "");
        src << " " << dst << " = " << (isint ? "__float_as_int(f_[" + std::to_string(i) + "])" : "f_[" + std::to_string(i) + "]") << ";";
      }
      src << " }\n";
    }
    else if(v.storage == SC_Output)
    {
      if(get_dec(*vs, vid, D_BuiltIn, &bi))
      {
        if(bi == BI_Position)
          pos_expr = "ctx.g" + std::to_string(vid);
        continue;
      }
      if(t.k == K_STRUCT)
      {
        for(size_t mi = 0; mi < t.members.size(); mi++)
          if(get_mdec(*vs, ty, (uint32_t)mi, D_BuiltIn, &bi) && bi == BI_Position)
            pos_expr = "ctx.g" + std::to_string(vid) + ".m" + std::to_string(mi);
        continue;
      }
      if(get_dec(*vs, vid, D_Location, &loc))
        vs_out_loc[loc] = vid;
    }
  }
  if(pos_expr.empty())
  {
    err = "vertex shader writes no Position";
    return false;
  }
  src << "  vs_f" << ve->fn << "(ctx);\n";
  src << "  pos = make_float4(" << pos_expr << "[0], " << pos_expr << "[1], " << pos_expr << "[2], "
      << pos_expr << "[3]);\n";
  for(const FsInput &f : fin)
  {
    for(uint32_t a = 0; a < f.elems; a++)
    {
      auto it = vs_out_loc.find(f.loc + a);
      for(uint32_t i = 0; i < f.ncomp; i++)
      {
        uint32_t slot = f.slot + a * f.ncomp + i;
        if(it == vs_out_loc.end())
        {
          src << "  out[" << slot << "] = 0.0f;\n";
          continue;
        }
        uint32_t vty = vs->types.at(vs->vars.at(it->second).type).elem;
        const Type &vt = vs->types.at(vty);
        std::string g = "ctx.g" + std::to_string(it->second);
        bool vint = vt.k == K_INT || (vt.k == K_VEC && vs->types.at(vt.elem).k == K_INT);
        std::string e;
        if(vt.k == K_VEC)
          e = g + "[" + std::to_string(i < vt.count ? i : 0) + "]"; /* pad with component 0 */
        else
          e = g; /* scalars are splatted */
        if(vint)
          e = "__int_as_float(" + e + ")";
        src << "  out[" << slot << "] = " << e << ";\n";
      }
    }
  }
  src << "}\n";

  /* fragment wrapper */
  src << "__device__ __forceinline__ float4 vgx_fs(const VgxDraw &D, const float *b, const float *i0, "
         "const float *i1, const float *i2, float lod)\n{\n";
  src << "  fs_Ctx ctx;\n  ctx.D = &D;\n  ctx.lod = lod;\n";
  for(const FsInput &f : fin)
  {
    const Type &pt = fs->types.at(fs->vars.at(f.var).type);
    uint32_t ty = pt.elem;
    bool arr = fs->types.at(ty).k == K_ARR;
    uint32_t ety = arr ? fs->types.at(ty).elem : ty;
    const Type &et = fs->types.at(ety);
    for(uint32_t a = 0; a < f.elems; a++)
      for(uint32_t i = 0; i < f.ncomp; i++)
      {
        uint32_t slot = f.slot + a * f.ncomp + i;
        std::string dst = "ctx.g" + std::to_string(f.var) + (arr ? "[" + std::to_string(a) + "]" : "") +
                          (et.k == K_VEC ? "[" + std::to_string(i) + "]" : "");
        if(f.is_int)
          src << "  " << dst << " = __float_as_int(i0[" << slot << "]);\n"; /* flat: vertex 0 (:2229-2247) */
        else
          src << "  " << dst << " = vgx_interp(b, i0[" << slot << "], i1[" << slot << "], i2[" << slot << "]);\n";
      }
  }
  src << "  fs_f" << fe->fn << "(ctx);\n";
  std::string col;
  for(uint32_t vid : fe->iface)
  {
    auto it = fs->vars.find(vid);
    if(it == fs->vars.end() || it->second.storage != SC_Output)
      continue;
    uint32_t loc = 0;
    if(get_dec(*fs, vid, D_Location, &loc) && loc == 0)
    {
      const Type &t = fs->types.at(fs->types.at(it->second.type).elem);
      std::string g = "ctx.g" + std::to_string(vid);
      uint32_t n = t.k == K_VEC ? t.count : 1;
      std::string c[4];
      for(uint32_t i = 0; i < 4; i++)
        c[i] = i < n ? (t.k == K_VEC ? g + "[" + std::to_string(i) + "]" : g) : (i == 3 ? "1.0f" : "0.0f");
      col = "make_float4(" + c[0] + ", " + c[1] + ", " + c[2] + ", " + c[3] + ")";
    }
  }
  if(col.empty())
    col = "make_float4(0.0f, 0.0f, 0.0f, 1.0f)";
  src << "  return " << col << ";\n}\n";
  res.source = src.str();
  return true;
}
}    // namespace vst
