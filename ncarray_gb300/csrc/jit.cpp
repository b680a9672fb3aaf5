// Expression/reduction engine of libncgb300 (see jit.hpp).
//
// Replaces ncarray's device::RuntimeCompiler (src/lib/ncarray/jit/device/
// rtcompiler.cc:49-510) and the dispatch in GPUEngine::execute_binary_expression,
// execute_reduce_axes and execute_full_reduce (src/lib/ncarray/engines/
// gpuengine.hh:90-333). The reference builds one kernel string per tape and
// launches one thread per element with a div/mod decode per dimension; here a
// tape is compiled into one of five sm_103a kernel classes chosen from the
// canonical iteration space (size-1 dims dropped, dims ordered by the output's
// strides, mergeable dims fused), with 128-bit vector access where the layout
// allows and reductions fused into the same HBM pass.
#include "jit.hpp"
#include "tune.hpp"

#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <unordered_map>

namespace nca {

static const char* kPrelude =
#include "jit_prelude.inc"
    ;
static const char* kKernels =
#include "jit_kernels.inc"
    ;

// ============================================================================
// tape validation
// ============================================================================
enum Arity { A_NONE = -1, A_LOAD = 0, A_UNARY = 1, A_BINARY = 2 };

static int op_arity(int op) {
  switch (op) {
    case NCA_OP_NOOP: return A_NONE;
    case NCA_OP_IDX: case NCA_OP_LOAD_NCARR: case NCA_OP_LOAD_SOARR: case NCA_OP_LOAD_CONST:
      return A_LOAD;
    case NCA_OP_NEG: case NCA_OP_INC: case NCA_OP_DEC: case NCA_OP_LNOT: case NCA_OP_BNOT:
    case NCA_OP_ABS: case NCA_OP_SQRT:
      return A_UNARY;
    case NCA_OP_ADD: case NCA_OP_SUB: case NCA_OP_MUL: case NCA_OP_DIV: case NCA_OP_MOD:
    case NCA_OP_EQ: case NCA_OP_NE: case NCA_OP_LT: case NCA_OP_LE: case NCA_OP_GT:
    case NCA_OP_GE: case NCA_OP_LAND: case NCA_OP_LOR: case NCA_OP_BAND: case NCA_OP_BOR:
    case NCA_OP_XOR:
      return A_BINARY;
    default:
      return -2;  // SZOF, ADDR, INDR, CAST, FDIV, shifts: not evaluated by the reference VM
  }
}

Tape make_tape(const nca_tape* t, int n_operands) {
  if (!t || !t->instrs) fail(NCA_ERR_INVALID, "null tape");
  if (t->n_instrs <= 0 || t->n_instrs > NCA_MAX_INSTRS)
    fail(NCA_ERR_LIMIT, "tape has %d instructions (1..%d)", t->n_instrs, NCA_MAX_INSTRS);
  if (t->n_scalars < 0 || t->n_scalars > NCA_MAX_SCALARS)
    fail(NCA_ERR_LIMIT, "tape has %d scalars (0..%d)", t->n_scalars, NCA_MAX_SCALARS);
  if (t->n_scalars > 0 && (!t->scalar_dtypes || !t->scalar_slots))
    fail(NCA_ERR_INVALID, "tape scalars missing");
  Tape r;
  r.compute_dtype = t->compute_dtype;
  r.result_dtype = t->result_dtype;
  if (!dtype_valid(r.compute_dtype) || arith_dtype(r.compute_dtype) != r.compute_dtype)
    fail(NCA_ERR_DTYPE, "compute dtype %d is not an arithmetic device dtype", r.compute_dtype);
  if (!dtype_valid(r.result_dtype)) fail(NCA_ERR_DTYPE, "result dtype %d unsupported", r.result_dtype);
  const bool w_int = !dtinfo(r.compute_dtype).is_float;
  for (int i = 0; i < t->n_scalars; ++i) {
    if (!dtype_valid(t->scalar_dtypes[i])) fail(NCA_ERR_DTYPE, "scalar %d dtype %d unsupported", i, t->scalar_dtypes[i]);
    r.scalar_dtypes.push_back(t->scalar_dtypes[i]);
    r.scalar_slots.push_back(t->scalar_slots[i]);
  }
  int depth = 0;
  for (int i = 0; i < t->n_instrs; ++i) {
    const uint32_t ins = t->instrs[i];
    const int op = (int)(ins >> 24), idx = (int)(ins & 0xffffff);
    const int ar = op_arity(op);
    if (ar == -2) fail(NCA_ERR_UNSUPPORTED, "opcode %d is not supported on the device path", op);
    if ((op == NCA_OP_BNOT || op == NCA_OP_BAND || op == NCA_OP_BOR || op == NCA_OP_XOR) && !w_int)
      fail(NCA_ERR_DTYPE, "bitwise opcode %d on a floating compute dtype", op);
    if (op == NCA_OP_LOAD_NCARR || op == NCA_OP_LOAD_SOARR) {
      if (idx >= n_operands) fail(NCA_ERR_INVALID, "instruction %d loads operand %d of %d", i, idx, n_operands);
      r.n_arrays = std::max(r.n_arrays, idx + 1);
    }
    if (op == NCA_OP_LOAD_CONST && idx >= t->n_scalars)
      fail(NCA_ERR_INVALID, "instruction %d loads scalar %d of %d", i, idx, t->n_scalars);
    if (op == NCA_OP_IDX) r.uses_idx = true;
    if (ar == A_LOAD) ++depth;
    else if (ar == A_UNARY) { if (depth < 1) fail(NCA_ERR_INVALID, "stack underflow at %d", i); }
    else if (ar == A_BINARY) { if (depth < 2) fail(NCA_ERR_INVALID, "stack underflow at %d", i); --depth; }
    if (depth > 64) fail(NCA_ERR_LIMIT, "tape stack deeper than 64");
    r.instrs.push_back(ins);
  }
  if (depth != 1) fail(NCA_ERR_INVALID, "tape leaves %d values on the stack (expected 1)", depth);
  return r;
}

// ============================================================================
// host-side scalar conversion (static_cast<W>(scalar), op_traits::cast)
// ============================================================================
template <class To, class From>
static To hcast(From v) { return static_cast<To>(v); }

static float bf16_to_f32_host(uint16_t h) { uint32_t u = (uint32_t)h << 16; float f; memcpy(&f, &u, 4); return f; }
static float f16_to_f32_host(uint16_t h) {
  const uint32_t s = (h >> 15) & 1u, e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  float f;
  if (e == 0) f = (float)m * (1.0f / 16777216.0f);  // m * 2^-24
  else if (e == 31) { uint32_t u = (s << 31) | 0x7f800000u | (m << 13); memcpy(&f, &u, 4); return f; }
  else { uint32_t u = (s << 31) | ((e + 112u) << 23) | (m << 13); memcpy(&f, &u, 4); return f; }
  return s ? -f : f;
}

template <class W>
static W scalar_as(int sd, uint64_t slot) {
  switch (sd) {
    case NCA_BOOL: return hcast<W>((uint8_t)(slot & 0xff) != 0);
    case NCA_CHAR: case NCA_INT8: return hcast<W>((int8_t)(slot & 0xff));
    case NCA_UINT8: return hcast<W>((uint8_t)(slot & 0xff));
    case NCA_UINT16: return hcast<W>((uint16_t)(slot & 0xffff));
    case NCA_INT16: return hcast<W>((int16_t)(slot & 0xffff));
    case NCA_UINT32: return hcast<W>((uint32_t)slot);
    case NCA_INT32: return hcast<W>((int32_t)(uint32_t)slot);
    case NCA_UINT64: return hcast<W>((uint64_t)slot);
    case NCA_INT64: return hcast<W>((int64_t)slot);
    case NCA_FLOAT32: { uint32_t u = (uint32_t)slot; float f; memcpy(&f, &u, 4); return hcast<W>(f); }
    case NCA_FLOAT64: { double d; memcpy(&d, &slot, 8); return hcast<W>(d); }
    case NCA_BFLOAT16: return hcast<W>(bf16_to_f32_host((uint16_t)slot));
    case NCA_FLOAT16: return hcast<W>(f16_to_f32_host((uint16_t)slot));
  }
  fail(NCA_ERR_DTYPE, "bad scalar dtype %d", sd);
}

template <class W>
static uint64_t bits_of(W v) { uint64_t r = 0; memcpy(&r, &v, sizeof(W)); return r; }

static uint64_t scalar_word(int wdt, int sd, uint64_t slot) {
  switch (wdt) {
    case NCA_BOOL: return bits_of<bool>(scalar_as<bool>(sd, slot));
    case NCA_CHAR: case NCA_INT8: return bits_of<int8_t>(scalar_as<int8_t>(sd, slot));
    case NCA_UINT8: return bits_of<uint8_t>(scalar_as<uint8_t>(sd, slot));
    case NCA_UINT16: return bits_of<uint16_t>(scalar_as<uint16_t>(sd, slot));
    case NCA_INT16: return bits_of<int16_t>(scalar_as<int16_t>(sd, slot));
    case NCA_UINT32: return bits_of<uint32_t>(scalar_as<uint32_t>(sd, slot));
    case NCA_INT32: return bits_of<int32_t>(scalar_as<int32_t>(sd, slot));
    case NCA_UINT64: return bits_of<uint64_t>(scalar_as<uint64_t>(sd, slot));
    case NCA_INT64: return bits_of<int64_t>(scalar_as<int64_t>(sd, slot));
    case NCA_FLOAT32: return bits_of<float>(scalar_as<float>(sd, slot));
    case NCA_FLOAT64: return bits_of<double>(scalar_as<double>(sd, slot));
  }
  fail(NCA_ERR_DTYPE, "bad compute dtype %d", wdt);
}

// ============================================================================
// canonical iteration space
// ============================================================================
struct CArr {
  const char* base = nullptr;
  int dtype = 0;
  int64_t st[NCA_MAX_NDIM] = {0};
  // operands on a pointer axis: element address = *(table + sum_d c_d pts[d])
  // + ptc + sum_d c_d st[d] (st holds the panel strides, base is null)
  bool ptr = false;
  const char* table = nullptr;
  int64_t pts[NCA_MAX_NDIM] = {0};
  int64_t ptc = 0;
};

struct Space {
  int nd = 0;
  int64_t shape[NCA_MAX_NDIM] = {0};
  bool red[NCA_MAX_NDIM] = {false};
  std::vector<CArr> ops;
  bool has_out = false;
  CArr out;
  std::vector<CArr> reds;
  std::vector<CArr> xouts;   // extra outputs (other tapes over the same operands, out's shape)
  int64_t total() const { int64_t t = 1; for (int d = 0; d < nd; ++d) t *= shape[d]; return t; }
};

static void check_view(const nca_view& v, const char* what, bool pointer_ok = false) {
  if (v.ndim < 0 || v.ndim > NCA_MAX_NDIM) fail(NCA_ERR_LIMIT, "%s: ndim %d (0..%d)", what, v.ndim, NCA_MAX_NDIM);
  if (!dtype_valid(v.dtype)) fail(NCA_ERR_DTYPE, "%s: dtype %d not supported on the device", what, v.dtype);
  if (v.pointer_axis >= 0 && !pointer_ok)
    fail(NCA_ERR_UNSUPPORTED, "%s: pointer axes are supported on operands, not on results", what);
  if (v.pointer_axis >= v.ndim) fail(NCA_ERR_INVALID, "%s: pointer axis %d of %d", what, v.pointer_axis, v.ndim);
  if ((v.flags & ~NCA_VIEW_SUBOFFSETS) != 0 || ((v.flags & NCA_VIEW_SUBOFFSETS) && v.pointer_axis < 0))
    fail(NCA_ERR_INVALID, "%s: flags %d", what, v.flags);
  int64_t n = 1;
  for (int d = 0; d < v.ndim; ++d) {
    if (v.shape[d] < 0) fail(NCA_ERR_SHAPE, "%s: negative extent", what);
    n *= v.shape[d];
  }
  if (n > 0 && !v.data) fail(NCA_ERR_INVALID, "%s: null data pointer", what);
}

static const char* view_base(const nca_view& v) {
  int64_t off = 0;
  for (int d = 0; d < v.ndim; ++d) off += v.offsets[d];
  return static_cast<const char*>(v.data) + off;
}

// Builds the logical-order space (size-1 dims dropped). `lshape` has n dims.
static Space make_space(const int64_t* lshape, int n, const nca_view* ops, int nops,
                        const nca_view* out, uint32_t red_mask, const nca_reduction* reds, int nred,
                        const nca_view* xouts = nullptr, int nx = 0) {
  Space s;
  for (int k = 0; k < nops; ++k) {
    CArr a; a.dtype = ops[k].dtype;
    const nca_view& v = ops[k];
    if (v.pointer_axis < 0) {
      a.base = view_base(v);
    } else {
      // NC (layout.hh:468-535): axes before the pointer axis move the table
      // pointer, the pointer axis indexes it (index offset offsets[pa]), later
      // axes move the panel pointer. SO (suboffsets, layout.hh:677-778): the
      // pointer axis strides the table and offsets[pa] is added after reading.
      const int pa = v.pointer_axis;
      const bool so = (v.flags & NCA_VIEW_SUBOFFSETS) != 0;
      a.ptr = true;
      int64_t t = 0, c = 0;
      for (int d = 0; d < v.ndim; ++d) {
        if (d < pa) t += v.offsets[d];
        else if (d == pa) { if (so) c += v.offsets[d]; else t += v.offsets[d] * (int64_t)sizeof(void*); }
        else c += v.offsets[d];
      }
      a.table = static_cast<const char*>(v.data) + t;
      a.ptc = c;
    }
    s.ops.push_back(a);
  }
  if (out) { s.has_out = true; s.out.base = view_base(*out); s.out.dtype = out->dtype; }
  for (int k = 0; k < nred; ++k) {
    CArr a; a.base = view_base(reds[k].out); a.dtype = reds[k].out.dtype; s.reds.push_back(a);
  }
  for (int k = 0; k < nx; ++k) {
    CArr a; a.base = view_base(xouts[k]); a.dtype = xouts[k].dtype; s.xouts.push_back(a);
  }
  int kept_pos = 0;
  for (int d = 0; d < n; ++d) {
    const bool is_red = (red_mask >> d) & 1u;
    const int kd = kept_pos;
    if (!is_red) ++kept_pos;
    if (lshape[d] == 1) continue;
    const int c = s.nd++;
    s.shape[c] = lshape[d];
    s.red[c] = is_red;
    for (int k = 0; k < nops; ++k) {
      const nca_view& v = ops[k];
      const int vd = d - (n - v.ndim);
      const bool live = vd >= 0 && v.shape[vd] != 1;
      if (v.pointer_axis < 0 || vd > v.pointer_axis) {
        s.ops[k].st[c] = live ? v.strides[vd] : 0;
      } else {
        // a table axis: stride of the table (a pointer per index on NC's pointer axis)
        const bool nc_pa = vd == v.pointer_axis && !(v.flags & NCA_VIEW_SUBOFFSETS);
        s.ops[k].pts[c] = live ? (nc_pa ? (int64_t)sizeof(void*) : v.strides[vd]) : 0;
      }
    }
    if (out) s.out.st[c] = out->strides[d];
    for (int k = 0; k < nred; ++k) s.reds[k].st[c] = is_red ? 0 : reds[k].out.strides[kd];
    for (int k = 0; k < nx; ++k) s.xouts[k].st[c] = xouts[k].strides[d];
  }
  return s;
}

static bool mergeable(const Space& s, int i) {  // dims i (outer) and i+1 (inner)
  if (s.red[i] != s.red[i + 1]) return false;
  auto ok = [&](const CArr& a) {
    return a.st[i] == a.st[i + 1] * s.shape[i + 1] && a.pts[i] == a.pts[i + 1] * s.shape[i + 1];
  };
  for (auto& a : s.ops) if (!ok(a)) return false;
  if (s.has_out && !ok(s.out)) return false;
  for (auto& a : s.reds) if (!ok(a)) return false;
  for (auto& a : s.xouts) if (!ok(a)) return false;
  return true;
}

static void merge_dims(Space& s) {
  for (int i = s.nd - 2; i >= 0; --i) {
    if (!mergeable(s, i)) continue;
    s.shape[i] *= s.shape[i + 1];
    auto fold = [&](CArr& a) {
      a.st[i] = a.st[i + 1];
      a.pts[i] = a.pts[i + 1];
      for (int d = i + 1; d + 1 < s.nd; ++d) { a.st[d] = a.st[d + 1]; a.pts[d] = a.pts[d + 1]; }
    };
    for (auto& a : s.ops) fold(a);
    if (s.has_out) fold(s.out);
    for (auto& a : s.reds) fold(a);
    for (auto& a : s.xouts) fold(a);
    for (int d = i + 1; d + 1 < s.nd; ++d) { s.shape[d] = s.shape[d + 1]; s.red[d] = s.red[d + 1]; }
    --s.nd;
  }
}

static void permute_dims(Space& s, const std::vector<int>& perm) {
  Space t = s;
  for (int c = 0; c < s.nd; ++c) {
    t.shape[c] = s.shape[perm[c]];
    t.red[c] = s.red[perm[c]];
    for (size_t k = 0; k < s.ops.size(); ++k) {
      t.ops[k].st[c] = s.ops[k].st[perm[c]];
      t.ops[k].pts[c] = s.ops[k].pts[perm[c]];
    }
    if (s.has_out) t.out.st[c] = s.out.st[perm[c]];
    for (size_t k = 0; k < s.reds.size(); ++k) t.reds[k].st[c] = s.reds[k].st[perm[c]];
    for (size_t k = 0; k < s.xouts.size(); ++k) t.xouts[k].st[c] = s.xouts[k].st[perm[c]];
  }
  s = t;
}

static void ensure_nd1(Space& s) {
  if (s.nd > 0) return;
  s.nd = 1;
  s.shape[0] = 1;
  s.red[0] = false;
}

// ============================================================================
// source generation
// ============================================================================
// M_PAIR0 / M_PAIR1: strided by two elements along the vector axis; a group's
// elements sit at lanes 0, 2, 4, ... (or 1, 3, 5, ...) of a window of two
// aligned vectors (kind 2)
enum { M_CONTIG = 0, M_CONST = 1, M_STRIDED = 2, M_STAGED = 3, M_PAIR0 = 4, M_PAIR1 = 5 };

struct Spec {
  int kind = 1, nops = 0, nd = 1, vec = 1, idx32 = 0, nkept = 0, team = 256;
  uint32_t kept_mask = 0;
  bool has_out = false;
  int out_dtype = NCA_FLOAT64, w = NCA_FLOAT64, r = NCA_FLOAT64;
  int nred = 0;
  uint32_t red_ops = 0;
  bool has_sum = false, has_max = false, has_min = false;
  std::vector<int> op_dtypes, op_modes;
  std::vector<int> op_alias;   // M_PAIR*: earlier operand whose window loads this one shares (-1: none)
  std::vector<int> op_salias;  // kind 2: earlier operand with the same strides (same offsets; -1: none)
  int nscal = 0;
  // kind 6 (staged transposed operands)
  int qd = 0, qx = 1, qxp = 1, tp = 64, rb = 1;
  int unroll = 1;  // kind 1: vector groups per thread per trip
  int minb = 1;    // kind 6: minimum resident CTAs per SM requested from ptxas
  int grp = 4;     // kind 6: loop indices whose loads are issued together
  uint32_t tmask = 0;
  int tile_bytes = 0;
  // kind 7 (bulk-copy staged): stages, p-row / uniform operand masks, fastest
  // loop dim, number of p-row operands, log2(tp / 8)
  int ns = 0, ld = 0, npc = 0, ltp8 = 3, nmaps = 1;
  int nob = 2;     // kind 7: output tiles (TMA-store double buffering when 2)
  uint32_t pmask = 0, umask = 0, uumask = 0;
  uint32_t ptrmask = 0;   // operands on a pointer axis (kinds 2, 3, 4)
  int lastcta = 0;   // kinds 3 (block teams) and 4: the last CTA over a set of kept positions merges their partials
  int block = 256;   // kinds 1, 2: threads per block (NCA_LB)
  int k4r = 0;       // kind 4: row lanes per warp (row-lane form, one reduced dim rd); 0: thread per column group
  int rd = 0;
  int k4p = 0;       // kind 4 row-lane form on a persistent grid (equal contiguous ranges of units)
  int k4b = 0;       // kind 4 row-lane form with rows bulk-copied into a shared-memory ring
  int k4b_rb = 16, k4b_ns = 4, k4b_cb = 1;   // its rows per stage, stages, column blocks per CTA
  int k3rv = 0, k3tu = 1;   // kind 3 one-thread teams: reduced vectors per unit (compile time; 0: runtime
                            // loop) and units whose operands a thread gathers before reducing them
  int k3u = 8;       // kind 3 teams: loads of a thread in flight together (8 against 4: global sum
                     // 0.79 -> 0.83, argmax over rows of 16,384 0.79 -> 0.90 of measured)
  // kind 7: extra outputs, each a tape over the same operands stored elementwise
  std::vector<Tape> xtapes;
  std::vector<int> xout_dtypes;
  int xvec = 0;   // the extra tapes read only p-row and uniform operands: 16 bytes of a tile at a time
};

struct WordLayout {
  int opb, ops, outb, outs, shape, scal, redb, reds, total, psum, pmax, pmin, nsplit, chunk,
      keptn, redn, status, aux, magic, ptb, pts, ptc, nwords;
};

// symbol of each kernel class (distinct names keep profiler launch lists readable)
static const char* kernel_name(int kind) {
  switch (kind) {
    case 1: return "nca_flat";
    case 2: return "nca_nd";
    case 3: return "nca_red_inner";
    case 4: return "nca_red_outer";
    case 5: return "nca_finalize";
    case 6: return "nca_staged";
    case 7: return "nca_staged_async";
  }
  return "nca_kernel";
}

static WordLayout word_layout(int nops, int nd, int nscal, int nred, bool ptr) {
  WordLayout L;
  int p = 0;
  L.opb = p; p += nops;
  L.ops = p; p += nops * nd;
  L.outb = p; p += 1;
  L.outs = p; p += nd;
  L.shape = p; p += nd;
  L.scal = p; p += nscal;
  L.redb = p; p += nred;
  L.reds = p; p += nred * nd;
  L.total = p++; L.psum = p++; L.pmax = p++; L.pmin = p++; L.nsplit = p++; L.chunk = p++;
  L.keptn = p++; L.redn = p++; L.status = p++; L.aux = p++;
  L.magic = p; p += nd;
  // pointer-axis tables (a slot per operand when a launch has pointer operands)
  L.ptb = p; p += ptr ? nops : 0;
  L.pts = p; p += ptr ? nops * nd : 0;
  L.ptc = p; p += ptr ? nops : 0;
  L.nwords = p;
  return L;
}

static std::string cty(int dt) {  // arithmetic C type of a dtype (16-bit floats -> float)
  return arith_dtype(dt) == NCA_FLOAT32 && dt != NCA_FLOAT32 ? "float" : dtinfo(dt).ctype;
}

// value of a dtype from raw bits held in an integer expression
static std::string from_bits(int dt, const std::string& b) {
  switch (dt) {
    case NCA_BOOL: return "((((u32)(" + b + ")) & 0xffu) != 0u)";
    case NCA_CHAR: case NCA_INT8: return "((signed char)(unsigned char)(" + b + "))";
    case NCA_UINT8: return "((unsigned char)(" + b + "))";
    case NCA_INT16: return "((short)(unsigned short)(" + b + "))";
    case NCA_UINT16: return "((unsigned short)(" + b + "))";
    case NCA_INT32: return "((int)(u32)(" + b + "))";
    case NCA_UINT32: return "((u32)(" + b + "))";
    case NCA_INT64: return "((i64)(" + b + "))";
    case NCA_UINT64: return "((u64)(" + b + "))";
    case NCA_FLOAT32: return "__uint_as_float((u32)(" + b + "))";
    case NCA_FLOAT64: return "__longlong_as_double((i64)(" + b + "))";
    case NCA_BFLOAT16: return "nca_bf16_to_f32((unsigned short)(" + b + "))";
    case NCA_FLOAT16: return "nca_f16_to_f32((unsigned short)(" + b + "))";
  }
  fail(NCA_ERR_DTYPE, "from_bits dtype %d", dt);
}

// raw bits (u32 for <=4 bytes, u64 for 8) of value expression v stored as dtype dt
static std::string to_bits(int dt, const std::string& v) {
  switch (dt) {
    case NCA_BOOL: return "((u32)((" + v + ") != 0))";
    case NCA_CHAR: case NCA_INT8: return "((u32)(unsigned char)(signed char)(" + v + "))";
    case NCA_UINT8: return "((u32)(unsigned char)(" + v + "))";
    case NCA_INT16: return "((u32)(unsigned short)(short)(" + v + "))";
    case NCA_UINT16: return "((u32)(unsigned short)(" + v + "))";
    case NCA_INT32: return "((u32)(int)(" + v + "))";
    case NCA_UINT32: return "((u32)(" + v + "))";
    case NCA_INT64: return "((u64)(i64)(" + v + "))";
    case NCA_UINT64: return "((u64)(" + v + "))";
    case NCA_FLOAT32: return "((u32)__float_as_uint((float)(" + v + ")))";
    case NCA_FLOAT64: return "((u64)__double_as_longlong((double)(" + v + ")))";
    case NCA_BFLOAT16: return "((u32)nca_f32_to_bf16((float)(" + v + ")))";
    case NCA_FLOAT16: return "((u32)nca_f32_to_f16((float)(" + v + ")))";
  }
  fail(NCA_ERR_DTYPE, "to_bits dtype %d", dt);
}

static std::string storage_uint(int size) {
  switch (size) { case 1: return "unsigned char"; case 2: return "unsigned short"; case 4: return "u32"; default: return "u64"; }
}

static const char* kWordNames[4] = {"x", "y", "z", "w"};

// expression of lane q's bits in a vector of `bytes` loaded into variable u
static std::string lane_bits(int bytes, int es, int q, const std::string& u) {
  auto word = [&](int i) -> std::string {
    if (bytes == 16 || bytes == 8) return u + "." + kWordNames[i];
    return u;
  };
  if (es == 8) return "((((u64)" + word(2 * q + 1) + ") << 32) | (u64)" + word(2 * q) + ")";
  if (es == 4) return word(q);
  if (bytes <= 4 && es * 1 == bytes) return "(u32)" + u;
  const int bo = q * es;
  const int wi = bytes >= 8 ? bo / 4 : 0;
  const int sh = (bytes >= 8 ? bo % 4 : bo) * 8;
  return "((((u32)" + word(wi) + ") >> " + std::to_string(sh) + ") & " + (es == 1 ? "0xffu" : "0xffffu") + ")";
}

static std::string vec_type(int bytes) {
  switch (bytes) { case 16: return "uint4"; case 8: return "uint2"; case 4: return "u32"; case 2: return "unsigned short"; default: return "unsigned char"; }
}

// The tape as statements over the compute type nca_w ending in `return`;
// operand k is loaded as load_prefix + k + load_suffix.
// The tape as a C++ function body over the loaded operands (`load_prefix` k
// `load_suffix`), computing in the type named `W` (nca_w, or nca_wx<i> for an
// extra output's tape) with its scalars from s[sbase + i].
// An integer division or remainder by a tape constant takes the constant as a
// literal (the compiler then divides by multiplication); the kernel cache key
// holds the constants of integer tapes (literal_key).
static std::string int_literal(const Tape& t, int idx) {
  const int wdt = arith_dtype(t.compute_dtype);
  const uint64_t w = scalar_word(wdt, t.scalar_dtypes[(size_t)idx], t.scalar_slots[(size_t)idx]);
  const int sz = dtinfo(wdt).size;
  const uint64_t m = sz >= 8 ? ~0ull : ((1ull << (8 * sz)) - 1);
  const uint64_t u = w & m;
  if (dtinfo(wdt).is_signed) {
    const int64_t v = sz >= 8 ? (int64_t)u : (int64_t)(u ^ (1ull << (8 * sz - 1))) - (int64_t)(1ull << (8 * sz - 1));
    return "(" + std::to_string(v) + "ll)";
  }
  return "(" + std::to_string(u) + "ull)";
}
static bool literal_divisors(const Tape& t) {
  const int wdt = arith_dtype(t.compute_dtype);
  return !dtinfo(wdt).is_float && wdt != NCA_BOOL;
}
static std::string literal_key(const Tape& t) {
  std::string k;
  if (!literal_divisors(t)) return k;
  for (size_t i = 0; i < t.scalar_slots.size(); ++i) k += std::to_string(t.scalar_slots[i]) + ",";
  return k;
}

static std::string gen_eval(const Tape& t, const std::string& load_prefix = "v[",
                            const std::string& load_suffix = "][q]", const std::string& W = "nca_w",
                            int sbase = 0) {
  std::ostringstream os;
  const bool lit = literal_divisors(t);
  struct Ent { std::string e, lit; };   // an expression and, for an integer constant, its literal
  std::vector<Ent> st;
  int tmp = 0;
  auto pop = [&]() { Ent x = st.back(); st.pop_back(); return x; };
  for (uint32_t ins : t.instrs) {
    const int op = (int)(ins >> 24), idx = (int)(ins & 0xffffff);
    auto push_tmp = [&](const std::string& e) {
      const std::string n = "t" + std::to_string(tmp++);
      os << "  const " << W << " " << n << " = " << e << ";\n";
      st.push_back({n, ""});
    };
    switch (op) {
      case NCA_OP_NOOP: break;
      case NCA_OP_LOAD_NCARR: case NCA_OP_LOAD_SOARR:
        st.push_back({load_prefix + std::to_string(idx) + load_suffix, ""});
        break;
      case NCA_OP_LOAD_CONST:
        st.push_back({"nca_word<" + W + ">(s[" + std::to_string(idx + sbase) + "])", lit ? int_literal(t, idx) : ""});
        break;
      case NCA_OP_IDX: push_tmp("(" + W + ")lin"); break;
      default: {
        const int ar = op_arity(op);
        if (ar == A_UNARY) {
          const std::string a = pop().e;
          const char* f = op == NCA_OP_NEG ? "nca_neg" : op == NCA_OP_INC ? "nca_inc" : op == NCA_OP_DEC ? "nca_dec"
                        : op == NCA_OP_LNOT ? "nca_lnot" : op == NCA_OP_BNOT ? "nca_bnot" : op == NCA_OP_ABS ? "nca_abs" : "nca_sqrt";
          push_tmp(std::string(f) + "<" + W + ">(" + a + ")");
        } else {
          const Ent eb = pop(), ea = pop();
          const std::string& a = ea.e;
          const std::string& b = eb.e;
          const char* f = nullptr;
          switch (op) {
            case NCA_OP_ADD: f = "nca_add"; break; case NCA_OP_SUB: f = "nca_sub"; break;
            case NCA_OP_MUL: f = "nca_mul"; break; case NCA_OP_DIV: f = "nca_div"; break;
            case NCA_OP_MOD: f = "nca_mod"; break; case NCA_OP_EQ: f = "nca_eq"; break;
            case NCA_OP_NE: f = "nca_ne"; break; case NCA_OP_LT: f = "nca_lt"; break;
            case NCA_OP_LE: f = "nca_le"; break; case NCA_OP_GT: f = "nca_gt"; break;
            case NCA_OP_GE: f = "nca_ge"; break; case NCA_OP_LAND: f = "nca_land"; break;
            case NCA_OP_LOR: f = "nca_lor"; break; case NCA_OP_BAND: f = "nca_band"; break;
            case NCA_OP_BOR: f = "nca_bor"; break; case NCA_OP_XOR: f = "nca_xor"; break;
            default: fail(NCA_ERR_UNSUPPORTED, "opcode %d", op);
          }
          const bool ca = a.rfind("nca_word<", 0) == 0, cb = b.rfind("nca_word<", 0) == 0;
          if (!eb.lit.empty() && (op == NCA_OP_DIV || op == NCA_OP_MOD))
            // an integer divisor known when the kernel is compiled
            push_tmp(std::string(f) + "<" + W + ">(" + a + ", (" + W + ")" + eb.lit + ")");
          else if (op == NCA_OP_MUL && (ca != cb))
            // a multiplication by a tape constant (power-of-two constants
            // scale exactly on the integer pipe for float64)
            push_tmp("nca_mulc<" + W + ">(" + (cb ? a : b) + ", " + (cb ? b : a) + ")");
          else
            push_tmp(std::string(f) + "<" + W + ">(" + a + ", " + b + ")");
        }
      }
    }
  }
  return os.str() + "  return " + st.back().e + ";\n";
}

const char* jit_ctype(int dtype) { return dtinfo(arith_dtype(dtype)).ctype; }

uint64_t jit_scalar_word(int compute_dtype, int scalar_dtype, uint64_t slot) {
  return scalar_word(compute_dtype, scalar_dtype, slot);
}

std::string jit_gen_eval(const Tape& t, const std::string& load_prefix, const std::string& load_suffix) {
  return gen_eval(t, load_prefix, load_suffix);
}

std::string jit_gen_eval_w(const Tape& t, const std::string& load_prefix, const std::string& load_suffix,
                           const std::string& W) {
  return gen_eval(t, load_prefix, load_suffix, W);
}

std::string jit_from_bits(int dtype, const std::string& bits) { return from_bits(dtype, bits); }
std::string jit_to_bits(int dtype, const std::string& value) { return to_bits(dtype, value); }
std::string jit_storage_uint(int size) { return storage_uint(size); }

const char* jit_prelude() { return kPrelude; }

static std::string lim_expr(int dt, bool lowest) {
  switch (arith_dtype(dt)) {
    case NCA_BOOL: return lowest ? "false" : "true";
    case NCA_CHAR: case NCA_INT8: return lowest ? "((signed char)-128)" : "((signed char)127)";
    case NCA_UINT8: return lowest ? "((unsigned char)0)" : "((unsigned char)255)";
    case NCA_INT16: return lowest ? "((short)-32768)" : "((short)32767)";
    case NCA_UINT16: return lowest ? "((unsigned short)0)" : "((unsigned short)65535)";
    case NCA_INT32: return lowest ? "((int)0x80000000)" : "((int)0x7fffffff)";
    case NCA_UINT32: return lowest ? "0u" : "0xffffffffu";
    case NCA_INT64: return lowest ? "((i64)0x8000000000000000ull)" : "((i64)0x7fffffffffffffffll)";
    case NCA_UINT64: return lowest ? "0ull" : "0xffffffffffffffffull";
    case NCA_FLOAT32: return lowest ? "__uint_as_float(0xff7fffffu)" : "__uint_as_float(0x7f7fffffu)";
    case NCA_FLOAT64: return lowest ? "__longlong_as_double((i64)0xffefffffffffffffull)" : "__longlong_as_double(0x7fefffffffffffffll)";
  }
  fail(NCA_ERR_DTYPE, "limits of dtype %d", dt);
}

static std::string gen_source(const Spec& sp, const Tape& t) {
  const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
  std::ostringstream os;
  // NCA_F64_INTPIPE=0: float64 sqrt, constant products and comparisons as
  // float64 instructions instead of their integer-pipe forms (measurements)
  static const bool f64_fp = [] { const char* e = getenv("NCA_F64_INTPIPE"); return e && e[0] == '0'; }();
  if (f64_fp) os << "#define NCA_F64_FP 1\n";
  os << kPrelude;
  os << "#define NCA_NOPS " << sp.nops << "\n#define NCA_ND " << sp.nd << "\n#define NCA_NRED " << sp.nred
     << "\n#define NCA_KIND " << sp.kind << "\n#define NCA_VEC " << sp.vec << "\n#define NCA_IDX32 " << sp.idx32
     << "\n#define NCA_NKEPT " << sp.nkept << "\n#define NCA_KEPT_MASK " << sp.kept_mask << "u"
     << "\n#define NCA_RED_OPS " << sp.red_ops << "u\n#define NCA_TEAM " << sp.team
     << "\n#define NCA_HAS_OUT " << (sp.has_out ? 1 : 0) << "\n#define NCA_NWORDS " << L.nwords
     << "\n#define NCA_HAS_SUM " << (sp.has_sum ? 1 : 0) << "\n#define NCA_HAS_MAX " << (sp.has_max ? 1 : 0)
     << "\n#define NCA_HAS_MIN " << (sp.has_min ? 1 : 0) << "\n#define NCA_LASTCTA " << sp.lastcta
     << "\n#define NCA_K4R " << sp.k4r << "\n#define NCA_RD " << sp.rd << "\n#define NCA_K4P " << sp.k4p
     << "\n#define NCA_K4B " << sp.k4b << "\n#define NCA_K3RV " << sp.k3rv << "\n#define NCA_K3TU " << sp.k3tu << "\n";
  int sum_mode = 1;
  if (sp.nred > 0) {
    const int ra = arith_dtype(sp.r);
    sum_mode = ra == NCA_FLOAT32 ? 0 : ra == NCA_FLOAT64 ? 1 : 2;
  }
  os << "#define NCA_SUM_MODE " << sum_mode << "\n";
  // extremes keep an index only when an argmax (op 4) / argmin (op 5) is asked for
  {
    bool mxi = false, mni = false;
    for (int k = 0; k < sp.nred; ++k) {
      const int op = (int)((sp.red_ops >> (4 * k)) & 15u);
      if (op == 4) mxi = true;
      if (op == 5) mni = true;
    }
    os << "#define NCA_MX_IDX " << (mxi ? 1 : 0) << "\n#define NCA_MN_IDX " << (mni ? 1 : 0) << "\n";
  }
  os << "#define NCA_UNROLL " << sp.unroll << "\n#define NCA_KNAME " << kernel_name(sp.kind) << "\n";
  os << "#define NCA_K3U " << sp.k3u << "\n";
  // the staged class asks for sp.minb resident CTAs per SM (register cap)
  if (sp.kind == 6 && sp.minb > 1) os << "#define NCA_LB 256, " << sp.minb << "\n";
  else if (sp.kind == 1 || sp.kind == 2) os << "#define NCA_LB " << sp.block << "\n";
  else os << "#define NCA_LB 256\n";
  // kind 7: CTAs per SM its shared memory allows (the register cap follows)
  if (sp.kind == 7) os << "#define NCA_K7_MINB " << std::max(1, sp.minb) << "\n#define NCA_NOB " << sp.nob << "\n";
  os << "#define NCA_GRP " << sp.grp << "\n";
  os << "#define NCA_QD " << sp.qd << "\n#define NCA_QXP " << sp.qxp << "\n#define NCA_QX " << sp.qx << "\n#define NCA_TP " << sp.tp
     << "\n#define NCA_RB " << sp.rb << "\n#define NCA_TMASK " << sp.tmask << "u\n#define NCA_TILE_BYTES "
     << sp.tile_bytes << "\n#define NCA_NT " << __builtin_popcount(sp.tmask) << "\n";
  os << "#define NCA_W_OPB " << L.opb << "\n#define NCA_W_OPS " << L.ops << "\n#define NCA_W_OUTB " << L.outb
     << "\n#define NCA_W_OUTS " << L.outs << "\n#define NCA_W_SHAPE " << L.shape << "\n#define NCA_W_SCAL " << L.scal
     << "\n#define NCA_W_REDB " << L.redb << "\n#define NCA_W_REDS " << L.reds << "\n#define NCA_W_TOTAL " << L.total
     << "\n#define NCA_W_PSUM " << L.psum << "\n#define NCA_W_PMAX " << L.pmax << "\n#define NCA_W_PMIN " << L.pmin
     << "\n#define NCA_W_NSPLIT " << L.nsplit << "\n#define NCA_W_CHUNK " << L.chunk << "\n#define NCA_W_KEPTN " << L.keptn
     << "\n#define NCA_W_REDN " << L.redn << "\n#define NCA_W_STATUS " << L.status << "\n#define NCA_W_AUX " << L.aux
     << "\n#define NCA_W_MAGIC " << L.magic << "\n#define NCA_W_PTB " << L.ptb << "\n#define NCA_W_PTS " << L.pts
     << "\n#define NCA_W_PTC " << L.ptc << "\n#define NCA_PTRMASK " << sp.ptrmask << "u"
     << "\n";
  os << "#define NCA_NS " << sp.ns << "\n#define NCA_LD " << sp.ld << "\n#define NCA_NPC " << sp.npc << "\n#define NCA_LTP8 "
     << sp.ltp8 << "\n#define NCA_PMASK " << sp.pmask << "u\n#define NCA_UMASK " << sp.umask << "u\n#define NCA_UUMASK " << sp.uumask << "u\n#define NCA_NMAPS "
     << sp.nmaps << "\n";
  os << "typedef " << dtinfo(sp.w).ctype << " nca_w;\n";
  const std::string rty = sp.nred > 0 ? cty(sp.r) : std::string("nca_w");
  os << "typedef " << rty << " nca_r;\n";
  os << "#define NCA_R_LOWEST " << (sp.nred > 0 ? lim_expr(sp.r, true) : "0") << "\n";
  os << "#define NCA_R_HIGHEST " << (sp.nred > 0 ? lim_expr(sp.r, false) : "0") << "\n";
  os << "struct NcaArgs;\n";

  // ---- loads: nca_gather (NCA_VEC lanes) and nca_gather1 (lane 0, scalar) ----
  os << "#define OPB_(k) ((const char*)A.w[" << L.opb << " + (k)])\n";
  os << "#define OPS_(k, d) ((i64)A.w[" << L.ops << " + (k) * " << sp.nd << " + (d)])\n";
  auto scalar_load = [&](int k, const std::string& ptr) {
    const int dt = sp.op_dtypes[k];
    const int sz = dtinfo(dt).size;
    return "(nca_w)(" + from_bits(dt, "*(const " + storage_uint(sz) + "*)(" + ptr + ")") + ")";
  };
  std::ostringstream g, g1;
  for (int k = 0; k < sp.nops; ++k) {
    const int dt = sp.op_dtypes[k];
    const int es = dtinfo(dt).size;
    const std::string base = "OPB_(" + std::to_string(k) + ") + off[" + std::to_string(k) + "]";
    g1 << "  v[" << k << "][0] = " << scalar_load(k, base) << ";\n";
    const int mode = sp.op_modes[k];
    if (mode == M_STAGED) continue;   // filled from shared memory by the staged kernel
    if (mode == M_CONST || sp.vec == 1) {
      g << "  { const nca_w x = " << scalar_load(k, base) << ";";
      for (int q = 0; q < sp.vec; ++q) g << " v[" << k << "][" << q << "] = x;";
      g << " }\n";
    } else if (mode == M_CONTIG) {
      const int bytes = es * sp.vec;
      g << "  { const " << vec_type(bytes) << " u = *(const " << vec_type(bytes) << "*)(" << base << ");";
      for (int q = 0; q < sp.vec; ++q)
        g << " v[" << k << "][" << q << "] = (nca_w)(" << from_bits(dt, lane_bits(bytes, es, q, "u")) << ");";
      g << " }\n";
    } else if (mode == M_PAIR0 || mode == M_PAIR1) {
      // the window: two aligned vectors from the group's first element (minus
      // one element for M_PAIR1); every vector holds an element of the group
      const int ph = mode == M_PAIR1 ? 1 : 0;
      const int vb = es * sp.vec;
      const int lead = (k < (int)sp.op_alias.size() && sp.op_alias[k] >= 0) ? sp.op_alias[k] : k;
      const std::string wn = "pw" + std::to_string(lead);
      // a pointer operand's panels may sit anywhere: its window is used only when
      // the panel address is on the vector grid, else scalar loads
      const bool guarded = ((sp.ptrmask >> lead) & 1u) != 0;
      const std::string vt = vec_type(vb);
      if (lead == k && !guarded) {
        g << "  const " << vt << " " << wn << "_0 = *(const " << vt << "*)(" << base << " - " << ph * es << ");\n";
        g << "  const " << vt << " " << wn << "_1 = *(const " << vt << "*)(" << base << " + " << vb - ph * es << ");\n";
      } else if (lead == k) {
        g << "  const bool " << wn << "_ok = ((((u64)(" << base << ")) - " << ph * es << ") & " << vb - 1 << ") == 0;\n";
        g << "  " << vt << " " << wn << "_0 = {}, " << wn << "_1 = {};\n";
        g << "  if (" << wn << "_ok) { " << wn << "_0 = *(const " << vt << "*)(" << base << " - " << ph * es << "); "
          << wn << "_1 = *(const " << vt << "*)(" << base << " + " << vb - ph * es << "); }\n";
      }
      for (int q = 0; q < sp.vec; ++q) {
        const int j = ph + 2 * q;
        const std::string lanev = "(nca_w)(" + from_bits(dt, lane_bits(vb, es, j % sp.vec, wn + "_" + std::to_string(j / sp.vec))) + ")";
        if (!guarded) {
          g << "  v[" << k << "][" << q << "] = " << lanev << ";\n";
        } else {
          g << "  v[" << k << "][" << q << "] = " << wn << "_ok ? " << lanev << " : "
            << scalar_load(k, base + " + " + std::to_string(q) + " * OPS_(" + std::to_string(k) + ", " + std::to_string(sp.nd - 1) + ")")
            << ";\n";
        }
      }
    } else {
      for (int q = 0; q < sp.vec; ++q)
        g << "  v[" << k << "][" << q << "] = "
          << scalar_load(k, base + " + " + std::to_string(q) + " * OPS_(" + std::to_string(k) + ", " + std::to_string(sp.nd - 1) + ")")
          << ";\n";
    }
  }
  // the kernels take `const NcaArgs A`; the helpers take it by reference
  os << "struct NcaArgs { u64 w[" << L.nwords << "]; };\n";
  os << "__device__ __forceinline__ void nca_gather(const NcaArgs& A, const i64* off, nca_w (*v)[NCA_VEC]) {\n"
     << g.str() << "}\n";
  os << "__device__ __forceinline__ void nca_gather1(const NcaArgs& A, const i64* off, nca_w (*v)[NCA_VEC]) {\n"
     << g1.str() << "}\n";
  os << "#define nca_gather_ns nca_gather\n";
  if (sp.kind == 4 && sp.k4b) {
    // bulk-staged row-lane form: per operand its element size, its row
    // segment in a stage (64 kept groups) and its offset in the stage; the
    // lane's NCA_VEC elements of each operand read from shared memory
    int esum = 0, off = 0;
    std::ostringstream es_f, rb_f, of_f, sg;
    for (int k = 0; k < sp.nops; ++k) {
      const int dt = sp.op_dtypes[k], es = dtinfo(dt).size, rowb = 64 * sp.k4b_cb * sp.vec * es;
      es_f << "  if (k == " << k << ") return " << es << ";\n";
      rb_f << "  if (k == " << k << ") return " << rowb << ";\n";
      of_f << "  if (k == " << k << ") return " << off << ";\n";
      off += sp.k4b_rb * rowb;
      esum += es;
      const int bytes = es * sp.vec;
      sg << "  { const " << vec_type(bytes) << " u = *(const " << vec_type(bytes) << "*)(p[" << k << "]);";
      for (int q = 0; q < sp.vec; ++q)
        sg << " v[" << k << "][" << q << "] = (nca_w)(" << from_bits(dt, lane_bits(bytes, es, q, "u")) << ");";
      sg << " }\n";
    }
    os << "#define NCA_K4B_RB " << sp.k4b_rb << "\n#define NCA_K4B_NS " << sp.k4b_ns << "\n#define NCA_K4B_CB " << sp.k4b_cb
       << "\n#define NCA_K4B_STAGE " << off
       << "\n#define NCA_K4B_ESUM " << esum << "\n";
    os << "__device__ __forceinline__ constexpr int nca_k4b_es(int k) {\n" << es_f.str() << "  return 0;\n}\n";
    os << "__device__ __forceinline__ constexpr int nca_k4b_rowb(int k) {\n" << rb_f.str() << "  return 0;\n}\n";
    os << "__device__ __forceinline__ constexpr int nca_k4b_opoff(int k) {\n" << of_f.str() << "  return 0;\n}\n";
    os << "__device__ __forceinline__ void nca_sgather(const unsigned char* const* p, nca_w (*v)[NCA_VEC]) {\n"
       << sg.str() << "}\n";
  }
  // operands whose byte offsets equal an earlier operand's (same strides)
  os << "__device__ __forceinline__ constexpr int nca_sal(int k) {\n  return ";
  for (int k = 0; k < (int)sp.op_salias.size(); ++k)
    if (sp.op_salias[k] >= 0) os << "k == " << k << " ? " << sp.op_salias[k] << " : ";
  os << "(k < 0 ? 0 : -1);\n}\n";
  os << "__device__ __forceinline__ nca_w nca_ld_op(int k, const char* p) {\n  switch (k) {\n";
  for (int k = 0; k < sp.nops; ++k) os << "    case " << k << ": return " << scalar_load(k, "p") << ";\n";
  os << "  }\n  return (nca_w)0;\n}\n";
  os << "__device__ __forceinline__ nca_w nca_eval(const nca_w (*v)[NCA_VEC], int q, const u64* s, i64 lin) {\n"
     << "  (void)v; (void)q; (void)s; (void)lin;\n"
     << gen_eval(t) << "}\n";
  // extra outputs (kind 7): per tape its compute type, operand loads, value
  // and store; nca_xouts evaluates every extra tape at one element from the
  // operands' addresses and stores it to its output slot
  os << "#define NCA_NX " << sp.xtapes.size() << "\n";
  if (!sp.xtapes.empty()) {
    int sbase = (int)t.scalar_dtypes.size();
    std::ostringstream xo, xv;
    xo << "__device__ __forceinline__ void nca_xouts(const char* const* ap, const u64* s, char* const* op) {\n"
       << "  (void)ap; (void)s;\n";
    for (size_t x = 0; x < sp.xtapes.size(); ++x) {
      const Tape& xt = sp.xtapes[x];
      const std::string W = "nca_wx" + std::to_string(x);
      os << "typedef " << dtinfo(xt.compute_dtype).ctype << " " << W << ";\n";
      os << "__device__ __forceinline__ " << W << " nca_evalx" << x << "(const " << W << " (*v)[1], const u64* s) {\n"
         << "  (void)v; (void)s; const i64 lin = 0; (void)lin;\n"
         << gen_eval(xt, "v[", "][0]", W, sbase) << "}\n";
      const int dt = sp.xout_dtypes[x];
      const int es = dtinfo(dt).size;
      os << "__device__ __forceinline__ void nca_putx" << x << "(char* p, " << W << " e) { *(" << storage_uint(es)
         << "*)p = (" << storage_uint(es) << ")" << to_bits(dt, "e") << "; }\n";
      // loads of the operands this tape reads, converted to its compute type
      std::vector<bool> used(sp.nops, false);
      for (uint32_t ins : xt.instrs) {
        const int op = (int)(ins >> 24), idx = (int)(ins & 0xffffff);
        if ((op == NCA_OP_LOAD_NCARR || op == NCA_OP_LOAD_SOARR) && idx < sp.nops) used[idx] = true;
      }
      xo << "  {\n    " << W << " v[" << std::max(sp.nops, 1) << "][1];\n";
      for (int k = 0; k < sp.nops; ++k) {
        if (!used[k]) continue;
        const int odt = sp.op_dtypes[k];
        xo << "    v[" << k << "][0] = (" << W << ")(" << from_bits(odt, "*(const " + storage_uint(dtinfo(odt).size) +
              "*)(ap[" + std::to_string(k) + "])") << ");\n";
      }
      xo << "    nca_putx" << x << "(op[" << x << "], nca_evalx" << x << "(v, s));\n  }\n";
      // four consecutive elements: p-row operands 16 bytes at ap[k], uniform
      // operands one value at ap[k] (kind 7 operands and outputs are 4 bytes)
      xv << "  {\n    " << W << " v[" << std::max(sp.nops, 1) << "][1];\n    uint4 o;\n";
      for (int j = 0; j < 4; ++j) {
        for (int k = 0; k < sp.nops; ++k) {
          if (!used[k]) continue;
          const int odt = sp.op_dtypes[k];
          const bool prow = ((sp.pmask >> k) & 1u) != 0;
          const std::string src = prow ? "u" + std::to_string(k) + "." + kWordNames[j] : "*(const u32*)(ap[" + std::to_string(k) + "])";
          xv << "    v[" << k << "][0] = (" << W << ")(" << from_bits(odt, "(" + storage_uint(4) + ")(" + src + ")") << ");\n";
        }
        xv << "    o." << kWordNames[j] << " = (u32)" << to_bits(dt, "nca_evalx" + std::to_string(x) + "(v, s)") << ";\n";
      }
      xv << "    *(uint4*)op[" << x << "] = o;\n  }\n";
      sbase += (int)xt.scalar_dtypes.size();
    }
    xo << "}\n";
    os << xo.str();
    if (sp.xvec) {
      os << "__device__ __forceinline__ void nca_xouts4(const char* const* ap, const u64* s, char* const* op) {\n"
         << "  (void)ap; (void)s;\n";
      for (int k = 0; k < sp.nops; ++k)
        if ((sp.pmask >> k) & 1u) os << "  const uint4 u" << k << " = *(const uint4*)(ap[" << k << "]);\n";
      os << xv.str() << "}\n";
    }
  }
  os << "#define NCA_XVEC " << sp.xvec << "\n";

  // ---- stores ----
  if (sp.has_out) {
    const int dt = sp.out_dtype;
    const int es = dtinfo(dt).size;
    os << "__device__ __forceinline__ void nca_put1(char* p, nca_w e) { *(" << storage_uint(es) << "*)p = ("
       << storage_uint(es) << ")" << to_bits(dt, "e") << "; }\n";
    os << "__device__ __forceinline__ void nca_put(char* p, const nca_w* e) {\n";
    const int bytes = es * sp.vec;
    if (sp.vec == 1) {
      os << "  nca_put1(p, e[0]);\n";
    } else if (es == 8) {
      os << "  " << vec_type(bytes) << " u;\n";
      for (int q = 0; q < sp.vec; ++q) {
        os << "  { const u64 b = " << to_bits(dt, "e[" + std::to_string(q) + "]") << "; u." << kWordNames[2 * q]
           << " = (u32)b; u." << kWordNames[2 * q + 1] << " = (u32)(b >> 32); }\n";
      }
      os << "  *(" << vec_type(bytes) << "*)p = u;\n";
    } else if (es == 4) {
      os << "  " << vec_type(bytes) << " u;\n";
      for (int q = 0; q < sp.vec; ++q) {
        if (bytes == 4) os << "  u = " << to_bits(dt, "e[0]") << ";\n";
        else os << "  u." << kWordNames[q] << " = " << to_bits(dt, "e[" + std::to_string(q) + "]") << ";\n";
      }
      os << "  *(" << vec_type(bytes) << "*)p = u;\n";
    } else {
      const int nwords = bytes >= 4 ? bytes / 4 : 1;
      const int per = bytes >= 4 ? 4 / es : sp.vec;
      for (int wi = 0; wi < nwords; ++wi) {
        os << "  u32 w" << wi << " = 0u;\n";
        for (int j = 0; j < per; ++j) {
          const int q = wi * per + j;
          os << "  w" << wi << " |= (" << to_bits(dt, "e[" + std::to_string(q) + "]") << ") << " << (j * es * 8) << ";\n";
        }
      }
      if (bytes >= 8) {
        os << "  " << vec_type(bytes) << " u;";
        for (int wi = 0; wi < nwords; ++wi) os << " u." << kWordNames[wi] << " = w" << wi << ";";
        os << "\n  *(" << vec_type(bytes) << "*)p = u;\n";
      } else {
        os << "  *(" << vec_type(bytes) << "*)p = (" << vec_type(bytes) << ")w0;\n";
      }
    }
    os << "}\n";
  }
  // ---- reductions ----
  if (sp.nred > 0) {
    if (sp.r == NCA_BFLOAT16) os << "__device__ __forceinline__ nca_r nca_to_r(nca_w e) { return nca_bf16_to_f32(nca_f32_to_bf16((float)e)); }\n";
    else if (sp.r == NCA_FLOAT16) os << "__device__ __forceinline__ nca_r nca_to_r(nca_w e) { return nca_f16_to_f32(nca_f32_to_f16((float)e)); }\n";
    else if (sp.r == NCA_BOOL) os << "__device__ __forceinline__ nca_r nca_to_r(nca_w e) { return e != 0; }\n";
    else os << "__device__ __forceinline__ nca_r nca_to_r(nca_w e) { return (nca_r)e; }\n";
    const int sdt = sum_dtype(sp.r);
    const bool sgn = dtinfo(arith_dtype(sp.r)).is_signed;
    if (sum_mode == 2) {
      os << "__device__ __forceinline__ void nca_store_sum(char* p, u64 s) { *(" << storage_uint(dtinfo(sdt).size)
         << "*)p = (" << storage_uint(dtinfo(sdt).size) << ")s; }\n";
      os << "__device__ __forceinline__ double nca_sum_as_double(u64 s) { return (double)(" << (sgn ? "(i64)s" : "s") << "); }\n";
    } else {
      // a float32 sum of a float-float accumulator rounds hi + lo once, in float32
      if (sdt == NCA_FLOAT32 && sum_mode == 0) os << "#define NCA_SUM_FF32 1\n";
      if (sum_mode == 0) {
        os << "struct NcaFF { float hi, lo; };   // float-float partial sum\n";
        if (sdt == NCA_FLOAT32)
          os << "__device__ __forceinline__ void nca_store_sum(char* p, NcaFF s) { *(float*)p = __fadd_rn(s.hi, s.lo); }\n";
        else
          os << "__device__ __forceinline__ void nca_store_sum(char* p, NcaFF s) { *(double*)p = __dadd_rn((double)s.hi, (double)s.lo); }\n";
        os << "__device__ __forceinline__ double nca_sum_as_double(NcaFF s) { return __dadd_rn((double)s.hi, (double)s.lo); }\n";
      } else {
        if (sdt == NCA_FLOAT32) os << "__device__ __forceinline__ void nca_store_sum(char* p, double s) { *(float*)p = __double2float_rn(s); }\n";
        else os << "__device__ __forceinline__ void nca_store_sum(char* p, double s) { *(double*)p = s; }\n";
        os << "__device__ __forceinline__ double nca_sum_as_double(double s) { return s; }\n";
      }
    }
  }
  os << "#undef OPB_\n#undef OPS_\n";
  // the template redefines NcaArgs; skip that line by guarding
  std::string body = kKernels;
  const std::string decl = "struct NcaArgs { u64 w[NCA_NWORDS]; };";
  const size_t pos = body.find(decl);
  if (pos != std::string::npos) body.erase(pos, decl.size());
  os << body;
  return os.str();
}

// ============================================================================
// NVRTC + cache
// ============================================================================
static uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
  for (unsigned char c : s) { h ^= c; h *= 1099511628211ull; }
  return h;
}

struct JitState {
  std::mutex m;
  std::unordered_map<std::string, std::vector<char>> cubins;                 // key -> cubin
  std::map<std::pair<std::string, int>, CUfunction> funcs;                   // (key, device) -> fn
  std::string cache_dir;
  bool cache_dir_set = false;
  std::atomic<int64_t> compiled{0}, disk_hits{0}, mem_hits{0};
};

static JitState& js() { static JitState s; return s; }

static std::string default_cache_dir() {
  if (const char* e = getenv("NCA_GB300_CACHE_DIR")) if (*e) return e;
  if (const char* x = getenv("XDG_CACHE_HOME")) if (*x) return std::string(x) + "/ncarray_gb300";
  if (const char* h = getenv("HOME")) if (*h) return std::string(h) + "/.cache/ncarray_gb300";
  return "/tmp/ncarray_gb300";
}

std::string jit_cache_dir() {
  auto& s = js();
  std::lock_guard<std::mutex> lk(s.m);
  if (!s.cache_dir_set) { s.cache_dir = default_cache_dir(); s.cache_dir_set = true; }
  return s.cache_dir;
}

void jit_set_cache_dir(const char* dir) {
  auto& s = js();
  std::lock_guard<std::mutex> lk(s.m);
  s.cache_dir = dir ? std::string(dir) : default_cache_dir();
  s.cache_dir_set = true;
}

void jit_stats(int64_t* c, int64_t* d, int64_t* m) {
  auto& s = js();
  if (c) *c = s.compiled.load();
  if (d) *d = s.disk_hits.load();
  if (m) *m = s.mem_hits.load();
}

static void mkdirs(const std::string& path) {
  std::string cur;
  for (size_t i = 0; i < path.size(); ++i) {
    cur += path[i];
    if (path[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(path.c_str(), 0755);
}

static const char kMagic[8] = {'N', 'C', 'A', 'J', 'I', 'T', '1', 0};

static bool disk_load(const std::string& file, std::vector<char>& out) {
  std::ifstream f(file, std::ios::binary);
  if (!f) return false;
  char magic[8];
  uint64_t len = 0, h = 0;
  if (!f.read(magic, 8) || memcmp(magic, kMagic, 8) != 0) return false;
  if (!f.read(reinterpret_cast<char*>(&len), 8) || len == 0 || len > (64ull << 20)) return false;
  out.resize(len);
  if (!f.read(out.data(), (std::streamsize)len)) return false;
  if (!f.read(reinterpret_cast<char*>(&h), 8)) return false;
  return h == fnv1a(std::string(out.data(), out.size()));
}

static void disk_store(const std::string& dir, const std::string& file, const std::vector<char>& cubin) {
  mkdirs(dir);
  const std::string tmp = file + ".tmp." + std::to_string((long)getpid());
  {
    std::ofstream f(tmp, std::ios::binary);
    if (!f) return;
    const uint64_t len = cubin.size(), h = fnv1a(std::string(cubin.data(), cubin.size()));
    f.write(kMagic, 8);
    f.write(reinterpret_cast<const char*>(&len), 8);
    f.write(cubin.data(), (std::streamsize)len);
    f.write(reinterpret_cast<const char*>(&h), 8);
    if (!f) { std::remove(tmp.c_str()); return; }
  }
  std::rename(tmp.c_str(), file.c_str());
}

static std::string arch_for(int dev) {
  int major = 0, minor = 0;
  check_cuda(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev), "cc major");
  check_cuda(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev), "cc minor");
  std::string a = "sm_" + std::to_string(major) + std::to_string(minor);
  if (major >= 9) a += "a";
  return a;
}

static std::vector<char> nvrtc_compile(const std::string& src_in, const std::string& arch) {
  // NCA_JIT_EXTRA_SOURCE=<text> is appended to every generated source (a
  // diagnostic hook: extra definitions, or an #error to exercise the compile
  // failure path)
  std::string src = src_in;
  if (const char* extra = getenv("NCA_JIT_EXTRA_SOURCE")) src += std::string("\n") + extra + "\n";
  // NCA_JIT_DUMP=<dir> writes every generated source there (offline inspection)
  if (const char* dump = getenv("NCA_JIT_DUMP")) {
    if (*dump) {
      mkdirs(dump);
      char fn[48];
      snprintf(fn, sizeof(fn), "/%016llx.cu", (unsigned long long)fnv1a(src));
      std::ofstream f(std::string(dump) + fn);
      f << src;
    }
  }
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, src.c_str(), "nca_jit.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
    fail(NCA_ERR_COMPILE, "nvrtcCreateProgram failed");
  const std::string archopt = "--gpu-architecture=" + arch;
  const char* opts[] = {archopt.c_str(), "--fmad=false", "--std=c++17", "-DNDEBUG", "-lineinfo", "--device-int128"};
  nvrtcResult r = nvrtcCompileProgram(prog, 6, opts);
  if (r != NVRTC_SUCCESS) {
    size_t n = 0;
    nvrtcGetProgramLogSize(prog, &n);
    std::string log(n, '\0');
    if (n) nvrtcGetProgramLog(prog, &log[0]);
    nvrtcDestroyProgram(&prog);
    if (log.size() > 3000) log = log.substr(0, 3000);
    fail(NCA_ERR_COMPILE, "NVRTC: %s\n%s", nvrtcGetErrorString(r), log.c_str());
  }
  size_t n = 0;
  nvrtcGetCUBINSize(prog, &n);
  std::vector<char> cubin(n);
  nvrtcGetCUBIN(prog, cubin.data());
  nvrtcDestroyProgram(&prog);
  return cubin;
}

void jit_compile_only(const std::string& source, const std::string& arch) { (void)nvrtc_compile(source, arch); }

static std::string nvrtc_version_tag() {
  int a = 0, b = 0;
  nvrtcVersion(&a, &b);
  return std::to_string(a) + "." + std::to_string(b);
}

CUfunction jit_get(const std::string& source, const char* name) {
  const int dev = current_device();
  const std::string arch = arch_for(dev);
  const std::string key = [&] {
    char buf[32];
    snprintf(buf, sizeof(buf), "%016llx", (unsigned long long)fnv1a(source + "|" + arch + "|" + nvrtc_version_tag() + "|" + name + "|fmad=false"));
    return std::string(buf) + "_" + arch;
  }();
  auto& s = js();
  {
    std::lock_guard<std::mutex> lk(s.m);
    auto it = s.funcs.find({key, dev});
    if (it != s.funcs.end()) { s.mem_hits++; return it->second; }
  }
  std::vector<char> cubin;
  bool have = false;
  {
    std::lock_guard<std::mutex> lk(s.m);
    auto it = s.cubins.find(key);
    if (it != s.cubins.end()) { cubin = it->second; have = true; }
  }
  const std::string dir = jit_cache_dir();
  const std::string file = dir + "/" + key + ".cubin";
  if (!have && disk_load(file, cubin)) { have = true; s.disk_hits++; }
  if (!have) {
    cubin = nvrtc_compile(source, arch);
    s.compiled++;
    disk_store(dir, file, cubin);
  }
  CUmodule mod;
  check_cu(drv().cuModuleLoadData(&mod, cubin.data()), "cuModuleLoadData");
  CUfunction fn;
  check_cu(drv().cuModuleGetFunction(&fn, mod, name), "cuModuleGetFunction");
  std::lock_guard<std::mutex> lk(s.m);
  s.cubins[key] = cubin;
  s.funcs[{key, dev}] = fn;
  return fn;
}

// ============================================================================
// plan cache: a compact key of everything the generated source depends on,
// so that a launch whose kernel is known does no source generation or hashing
// of the full text
// ============================================================================
static std::string plan_key(const Spec& sp, const Tape& t) {
  std::string k;
  k.reserve(256);
  auto add = [&](long long v) { k += std::to_string(v); k += ','; };
  add(sp.kind); add(sp.nops); add(sp.nd); add(sp.vec); add(sp.idx32); add(sp.nkept); add(sp.team);
  add(sp.kept_mask); add(sp.has_out); add(sp.out_dtype); add(sp.w); add(sp.r); add(sp.nred); add(sp.red_ops);
  add(sp.has_sum); add(sp.has_max); add(sp.has_min); add(sp.nscal); add(sp.qd); add(sp.qx); add(sp.tp);
  add(sp.rb); add(sp.tmask); add(sp.tile_bytes); add(sp.unroll); add(sp.qxp); add(sp.minb); add(sp.grp);
  add(sp.ns); add(sp.ld); add(sp.npc); add(sp.ltp8); add(sp.pmask); add(sp.umask); add(sp.nmaps); add(sp.uumask); add(sp.ptrmask);
  add(sp.nob); add(sp.lastcta); add(sp.block); add(sp.k4r); add(sp.rd); add(sp.k4p); add(sp.k3u);
  add(sp.k4b); add(sp.k4b_rb); add(sp.k4b_ns); add(sp.k4b_cb); add(sp.k3rv); add(sp.k3tu);
  k += literal_key(t) + '|';
  add(sp.xvec);
  for (size_t x = 0; x < sp.xtapes.size(); ++x) {
    k += 'X';
    add(sp.xtapes[x].compute_dtype); add(sp.xout_dtypes[x]);
    for (uint32_t i : sp.xtapes[x].instrs) add(i);
    for (int d : sp.xtapes[x].scalar_dtypes) add(d);
    k += literal_key(sp.xtapes[x]);
  }
  for (int d : sp.op_dtypes) add(d);
  k += '|';
  for (int m : sp.op_modes) add(m);
  k += '|';
  for (int a : sp.op_alias) add(a);
  k += '|';
  for (int a : sp.op_salias) add(a);
  k += '|';
  for (uint32_t i : t.instrs) add(i);
  return k;
}

static CUfunction kernel_for(const Spec& sp, const Tape& t) {
  static std::mutex m;
  static std::unordered_map<std::string, CUfunction> cache;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::string key = plan_key(sp, t);
  key += "#" + std::to_string(dev);
  {
    std::lock_guard<std::mutex> lk(m);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  CUfunction fn = jit_get(gen_source(sp, t), kernel_name(sp.kind));
  if (sp.kind == 6 || sp.kind == 7 || sp.k4b) {
    // the staged class lives on shared memory: ask for the largest carveout
    check_cu(drv().cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT, 100), "carveout");
  }
  std::lock_guard<std::mutex> lk(m);
  cache[key] = fn;
  return fn;
}

// ============================================================================
// planning and launch
// ============================================================================
static void compute_magic(int64_t d, uint64_t& word) {
  // s = ceil(log2 d); m = 2^32 (2^s - d) / d + 1 (valid for d, x < 2^31)
  uint32_t sh = 0;
  while ((1ull << sh) < (uint64_t)d) ++sh;
  const uint64_t m = ((1ull << 32) * ((1ull << sh) - (uint64_t)d)) / (uint64_t)d + 1ull;
  word = (uint64_t)(uint32_t)m | ((uint64_t)sh << 32);
}

static bool aligned(const void* p, int64_t a) { return a <= 1 || ((uintptr_t)p % (uintptr_t)a) == 0; }

// chooses NCA_VEC and operand modes for a vector axis (the innermost canonical dim)
static void plan_vec(const Space& s, Spec& sp, int max_vec_elems, bool with_out) {
  const int ax = s.nd - 1;
  int maxsz = 1;
  if (with_out) maxsz = std::max(maxsz, dtinfo(s.out.dtype).size);
  for (int k = 0; k < sp.nops; ++k)
    if (s.ops[k].st[ax] == dtinfo(s.ops[k].dtype).size) maxsz = std::max(maxsz, dtinfo(s.ops[k].dtype).size);
  int vec = std::max(1, std::min(max_vec_elems, 16 / maxsz));
  auto out_ok = [&](int v) {
    if (!with_out) return true;
    const int64_t isz = dtinfo(s.out.dtype).size;
    if (s.out.st[ax] != isz) return false;
    if (!aligned(s.out.base, v * isz)) return false;
    for (int d = 0; d < ax; ++d) if (s.out.st[d] % (v * isz) != 0) return false;
    return true;
  };
  while (vec > 1 && (s.shape[ax] % vec != 0 || !out_ok(vec))) vec >>= 1;
  // a table axis innermost: every lane reads its own panel pointer
  for (int k = 0; k < sp.nops; ++k) if (s.ops[k].ptr && s.ops[k].pts[ax] != 0) vec = 1;
  sp.vec = vec;
  sp.op_modes.assign(sp.nops, M_STRIDED);
  for (int k = 0; k < sp.nops; ++k) {
    const CArr& a = s.ops[k];
    const int64_t isz = dtinfo(a.dtype).size;
    if (a.ptr) { sp.op_modes[k] = a.st[ax] == 0 && a.pts[ax] == 0 ? M_CONST : M_STRIDED; continue; }
    if (a.st[ax] == 0) { sp.op_modes[k] = M_CONST; continue; }
    if (vec == 1) { sp.op_modes[k] = M_STRIDED; continue; }
    bool ok = a.st[ax] == isz && aligned(a.base, vec * isz);
    for (int d = 0; d < ax && ok; ++d) if (a.st[d] % (vec * isz) != 0) ok = false;
    sp.op_modes[k] = ok ? M_CONTIG : M_STRIDED;
  }
}

// kind 2: strided operands whose elements along the vector axis are two apart
// read whole aligned windows of two vectors and keep every other lane
// (M_PAIR0: from lane 0, M_PAIR1: from lane 1). A window never reaches a
// 16-byte block without an element of the operand, so it stays inside the
// operand's memory. Operands whose windows coincide (the even and odd
// phases of one array, e.g. pixel-binning views) share the loads.
static void plan_pairs(const Space& s, Spec& sp) {
  sp.op_alias.assign(sp.nops, -1);
  const int ax = s.nd - 1;
  if (sp.vec < 2) return;
  // the window start of operand k in its own terms: the base (or, on a pointer
  // axis, the panel offset) minus the phase
  auto wstart = [&](int k) {
    const CArr& a = s.ops[k];
    const int64_t es = dtinfo(a.dtype).size, ph = sp.op_modes[k] == M_PAIR1 ? es : 0;
    return a.ptr ? (int64_t)a.ptc - ph : (int64_t)((uintptr_t)a.base - (uintptr_t)ph);
  };
  for (int k = 0; k < sp.nops; ++k) {
    if (sp.op_modes[k] != M_STRIDED) continue;
    const CArr& a = s.ops[k];
    const int64_t es = dtinfo(a.dtype).size, vb = es * sp.vec;
    if ((vb != 8 && vb != 16) || a.st[ax] != 2 * es) continue;
    // pointer operands: the table must not move along the vector axis; the
    // panels' own alignment is checked by the kernel (scalar loads otherwise)
    if (a.ptr && a.pts[ax] != 0) continue;
    const uintptr_t start = a.ptr ? (uintptr_t)a.ptc : (uintptr_t)a.base;
    const int64_t ph = (int64_t)(start % (uintptr_t)vb);
    if (ph != 0 && ph != es) continue;
    bool ok = true;
    for (int d = 0; d < ax && ok; ++d) if (a.st[d] % vb != 0) ok = false;
    if (!ok) continue;
    sp.op_modes[k] = ph == 0 ? M_PAIR0 : M_PAIR1;
    for (int j = 0; j < k; ++j) {
      if ((sp.op_modes[j] != M_PAIR0 && sp.op_modes[j] != M_PAIR1) || sp.op_alias[j] >= 0) continue;
      const CArr& o = s.ops[j];
      if (dtinfo(o.dtype).size != es || o.ptr != a.ptr || wstart(j) != wstart(k)) continue;
      bool same = true;
      for (int d = 0; d <= ax; ++d) if (o.st[d] != a.st[d]) same = false;
      if (a.ptr) {
        if (o.table != a.table) same = false;
        for (int d = 0; d <= ax; ++d) if (o.pts[d] != a.pts[d]) same = false;
      }
      if (same) { sp.op_alias[k] = j; break; }
    }
  }
}

// The device int that JIT kernels set when a bounded wait gives up (a
// __device__ variable of this library, so no allocation is ever needed).
int* jit_status_word();

// reads and clears the JIT status word of the current device (synchronises s)
int jit_read_status(cudaStream_t s) {
  int* p = jit_status_word();
  int v = 0;
  check_cuda(cudaMemcpyAsync(&v, p, sizeof(int), cudaMemcpyDeviceToHost, s), "status read");
  check_cuda(cudaMemsetAsync(p, 0, sizeof(int), s), "status clear");
  check_cuda(cudaStreamSynchronize(s), "status sync");
  return v ? NCA_ERR_TIMEOUT : 0;
}

static void fill_common_words(const Space& s, const Spec& sp, const Tape& t, const WordLayout& L,
                              std::vector<uint64_t>& w) {
  w.assign(L.nwords, 0);
  for (int k = 0; k < sp.nops; ++k) {
    w[L.opb + k] = (uint64_t)(uintptr_t)s.ops[k].base;
    for (int d = 0; d < sp.nd; ++d) w[L.ops + k * sp.nd + d] = (uint64_t)s.ops[k].st[d];
  }
  if (s.has_out) {
    w[L.outb] = (uint64_t)(uintptr_t)s.out.base;
    for (int d = 0; d < sp.nd; ++d) w[L.outs + d] = (uint64_t)s.out.st[d];
  }
  for (int d = 0; d < sp.nd; ++d) w[L.shape + d] = (uint64_t)s.shape[d];
  // the tape's scalars, then each extra output tape's (in its compute dtype)
  int si = 0;
  for (size_t i = 0; i < t.scalar_dtypes.size() && si < sp.nscal; ++i, ++si)
    w[L.scal + si] = scalar_word(sp.w, t.scalar_dtypes[i], t.scalar_slots[i]);
  for (const Tape& xt : sp.xtapes)
    for (size_t i = 0; i < xt.scalar_dtypes.size() && si < sp.nscal; ++i, ++si)
      w[L.scal + si] = scalar_word(xt.compute_dtype, xt.scalar_dtypes[i], xt.scalar_slots[i]);
  for (int k = 0; k < sp.nred; ++k) {
    w[L.redb + k] = (uint64_t)(uintptr_t)s.reds[k].base;
    for (int d = 0; d < sp.nd; ++d) w[L.reds + k * sp.nd + d] = (uint64_t)s.reds[k].st[d];
  }
  w[L.total] = (uint64_t)s.total();
  w[L.status] = (uint64_t)(uintptr_t)jit_status_word();
  for (int k = 0; k < sp.nops; ++k) {
    if (!s.ops[k].ptr) continue;
    w[L.opb + k] = 0;   // the kernel adds the panel address itself
    w[L.ptb + k] = (uint64_t)(uintptr_t)s.ops[k].table;
    for (int d = 0; d < sp.nd; ++d) w[L.pts + k * sp.nd + d] = (uint64_t)s.ops[k].pts[d];
    w[L.ptc + k] = (uint64_t)s.ops[k].ptc;
  }
}

static void launch(CUfunction fn, int64_t grid, std::vector<uint64_t>& words, cudaStream_t stream,
                   unsigned smem = 0, unsigned block = 256) {
  if (grid <= 0) return;
  count_launch();
  if (grid > 0x7fffffffLL) fail(NCA_ERR_LIMIT, "grid too large");
  if (smem > 48 * 1024)
    check_cu(drv().cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem), "smem attribute");
  void* params[] = {words.data()};
  check_cu(drv().cuLaunchKernel(fn, (unsigned)grid, 1, 1, block, 1, 1, smem, (CUstream)stream, params, nullptr),
           "cuLaunchKernel");
}

// byte range [lo, hi) a view can touch (false for pointer-axis views: unknown)
static bool view_range(const nca_view& v, uintptr_t& lo, uintptr_t& hi) {
  if (v.pointer_axis >= 0) return false;
  int64_t a = 0, b = 0;
  for (int d = 0; d < v.ndim; ++d) {
    a += v.offsets[d];
    b += v.offsets[d];
    if (v.shape[d] == 0) { lo = hi = (uintptr_t)v.data; return true; }
    const int64_t e = (v.shape[d] - 1) * v.strides[d];
    if (e < 0) a += e; else b += e;
  }
  lo = (uintptr_t)v.data + a;
  hi = (uintptr_t)v.data + b + dtinfo(v.dtype).size;
  return true;
}

// true when running the launch again cannot change what it reads (the
// outputs overlap no operand): the autotuner may time it several times
static bool rerun_safe(const nca_view* ops, int nops, const nca_view* outs, int nouts) {
  for (int j = 0; j < nouts; ++j) {
    uintptr_t ol, oh;
    if (!view_range(outs[j], ol, oh)) return false;
    for (int k = 0; k < nops; ++k) {
      uintptr_t l, h;
      if (!view_range(ops[k], l, h)) return false;
      if (l < oh && ol < h) return false;
    }
  }
  return true;
}

static int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

static void check_broadcast(const int64_t* lshape, int n, const nca_view& v, const char* what) {
  if (v.ndim > n) fail(NCA_ERR_SHAPE, "%s has %d dims, more than the result's %d", what, v.ndim, n);
  for (int d = 0; d < v.ndim; ++d) {
    const int ld = d + (n - v.ndim);
    if (v.shape[d] != 1 && v.shape[d] != lshape[ld])
      fail(NCA_ERR_SHAPE, "%s axis %d has extent %lld, result has %lld", what, d, (long long)v.shape[d], (long long)lshape[ld]);
  }
}

static int broadcast_shape(const nca_view* ops, int nops, int64_t* out) {
  int n = 0;
  for (int k = 0; k < nops; ++k) n = std::max(n, (int)ops[k].ndim);
  for (int d = 0; d < n; ++d) out[d] = 1;
  for (int k = 0; k < nops; ++k) {
    for (int d = 0; d < ops[k].ndim; ++d) {
      const int ld = d + (n - ops[k].ndim);
      const int64_t e = ops[k].shape[d];
      if (e == 1) continue;
      if (out[ld] == 1) out[ld] = e;
      else if (out[ld] != e) fail(NCA_ERR_SHAPE, "operands do not broadcast on axis %d", ld);
    }
  }
  return n;
}


// A kept dim q (extent <= 32) along which some operands are contiguous while
// they are strided along p, the innermost dim: those operands are staged
// through shared memory by kind 6. Returns q or -1.
static int find_staged(const Space& s, uint32_t& tmask, int& nt) {
  const int pd = s.nd - 1;
  if (s.nd < 2 || s.red[pd]) return -1;
  int qd = -1;
  for (size_t k = 0; k < s.ops.size() && qd < 0; ++k) {
    const int64_t isz = dtinfo(s.ops[k].dtype).size;
    if (s.ops[k].st[pd] == 0 || s.ops[k].st[pd] == isz) continue;
    for (int d = 0; d < pd; ++d)
      if (!s.red[d] && s.ops[k].st[d] == isz && s.shape[d] <= 32) { qd = d; break; }
  }
  if (qd < 0) return -1;
  tmask = 0;
  nt = 0;
  for (size_t k = 0; k < s.ops.size(); ++k) {
    const int64_t isz = dtinfo(s.ops[k].dtype).size;
    if (s.ops[k].st[qd] == isz && s.ops[k].st[pd] != isz && s.ops[k].st[pd] != 0) { tmask |= 1u << k; ++nt; }
  }
  return qd;
}

// Kind 7: the staged shape with 4-byte elements whose tiles TMA can move (see
// the template). Returns false, launching nothing, when the views do not
// allow it.
// the finalize pass: a block per kept position when there are very few (global
// reductions), a warp per kept position when there are few, a thread per kept
// position when there are many
static void launch_finalize(const Spec& sp, const Tape& tape, int64_t KN, int64_t S, int sms,
                            std::vector<uint64_t>& w, cudaStream_t stream) {
  Spec fs = sp;
  fs.kind = 5;
  // few splits: a thread walks them in order (no shuffle tree, whose adds are
  // float64 instructions for float64 sums and GB300 runs those slowly)
  fs.team = (KN >= 32768 || (S <= 32 && KN > 64)) ? 1 : (KN <= 64 ? 256 : 32);
  fs.lastcta = 0;
  CUfunction ff = kernel_for(fs, tape);
  const int64_t per_block = fs.team == 1 ? 256 : (fs.team == 32 ? 8 : 1);   // kept positions per block
  launch(ff, std::min<int64_t>(cdiv(KN, per_block), (int64_t)sms * 8), w, stream);
}

static bool launch_staged_async(const Space& s, Spec sp, const Tape& tape, int qd, uint32_t tmask, int nt, int64_t KN,
                                int64_t RN, cudaStream_t stream) {
  // NCA_STAGED_ASYNC=0 keeps these views on kind 6 (read on every call)
  if (const char* e = getenv("NCA_STAGED_ASYNC")) if (e[0] == '0') return false;
  if (!drv().cuTensorMapEncodeTiled) return false;
  const int pd = s.nd - 1;
  const int64_t P = s.shape[pd], QX = s.shape[qd];
  if (s.nd < 3 || s.nd > 5) return false;
  if (!(QX == 4 || QX == 8 || QX == 16 || QX == 32) || P % 32 != 0 || RN <= 0) return false;
  if (KN >= (1ll << 31) || RN >= (1ll << 31)) return false;
  if (sp.has_out && (dtinfo(s.out.dtype).size != 4 || s.out.st[pd] != 4)) return false;
  for (int k = 0; k < sp.nops; ++k) if (dtinfo(s.ops[k].dtype).size != 4) return false;
  int ld = -1;   // the fastest loop dim
  for (int d = pd - 1; d >= 0; --d) if (s.red[d]) { ld = d; break; }
  if (ld < 0 || ld == qd) return false;
  const int64_t LX = s.shape[ld];
  if (QX * LX >= (1ll << 31)) return false;
  auto al16 = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
  auto st_ok = [](int64_t st) { return st > 0 && st % 16 == 0 && st < (1ll << 40); };
  // every dim but p (and q, ld when listed) has a positive 16-byte multiple stride
  auto tma_ok = [&](const CArr& a, bool staged) {
    if (!al16(a.base)) return false;
    for (int d = 0; d <= pd; ++d) {
      if (d == pd) { if (staged ? !st_ok(a.st[d]) : a.st[d] != 4) return false; continue; }
      if (staged && d == qd) { if (a.st[d] != 4) return false; continue; }
      if (staged && d == ld) { if (a.st[d] != QX * 4) return false; continue; }
      if (!st_ok(a.st[d])) return false;
    }
    return true;
  };
  uint32_t pmask = 0, umask = 0, uumask = 0;
  int npc = 0;
  for (int k = 0; k < sp.nops; ++k) {
    const CArr& a = s.ops[k];
    if ((tmask >> k) & 1u) {
      if (!tma_ok(a, true)) return false;
    } else if (a.st[pd] == 4) {
      if (!tma_ok(a, false)) return false;
      pmask |= 1u << k;
      ++npc;
    } else if (a.st[pd] == 0) {
      if (a.st[qd] == 0 && a.st[ld] == 0) {
        umask |= 1u << k;
        bool unit_const = true;   // constant along every loop dim too
        for (int d = 0; d < pd; ++d) if (s.red[d] && a.st[d] != 0) unit_const = false;
        if (unit_const) uumask |= 1u << k;
      }
    } else {
      return false;
    }
  }
  if (sp.has_out && !tma_ok(s.out, false)) return false;
  const int nx = (int)sp.xtapes.size();
  if (nx > 0 && !sp.has_out) return false;
  for (const CArr& a : s.xouts)
    if (dtinfo(a.dtype).size != 4 || !tma_ok(a, false)) return false;
  // block of rb loop indices: a divisor of the fastest loop extent whose
  // (loop index, q) rows fill whole 128-byte boxes, at most 128 of them, the
  // largest whose stages fit in the 227 KiB a CTA may use. 128 rows per block
  // and 2 stages measured best on the permuted (8,256,256,64) float32 views (about 97 KiB per CTA, two
  // CTAs per SM: 5.6 TB/s against 5.4 TB/s for 64 rows and 3 stages, three
  // CTAs per SM)
  // with extra outputs (one more output tile each) the block shrinks so that
  // two CTAs still fit on an SM: (8, 256, 256, 64) with one extra output ran
  // 4.96 TB/s at 64 rows, 3.66 TB/s at 128 rows (one CTA per SM), before the
  // extra tape ran on whole tile chunks
  const int64_t budget = sp.xtapes.empty() ? 227 * 1024 : 113 * 1024;
  const int tp = 32;
  int rb_max = (int)std::max<int64_t>(1, 128 / QX);
  if (const char* e = getenv("NCA_STAGED_RB")) { const int v = atoi(e); if (v >= 1 && v <= 16) rb_max = v; }
  // 2 stages; 3 with extra outputs (the one-pass C2 step: 64 rows, 3 stages,
  // 2 CTAs per SM 5.68 TB/s against 5.51 for 2 stages and 3 CTAs per SM)
  int ns_want = sp.xtapes.empty() ? 2 : 3;
  if (const char* e = getenv("NCA_STAGED_STAGES")) { const int v = atoi(e); if (v >= 2 && v <= 6) ns_want = v; }
  int nob = 2;
  if (const char* e = getenv("NCA_STAGED_OUTBUFS")) { const int v = atoi(e); if (v == 1 || v == 2) nob = v; }
  // stages, output tiles, full/empty mbarriers per stage and per output tile
  auto smem_for = [&](int c, int n) {
    const int64_t rq = (int64_t)c * QX;
    const int64_t stage = nt * ((rq / 32) * tp * 128) + npc * (rq * 128);
    return n * stage + nob * (1 + nx) * (rq * 128) + 16 * n + 16 * nob + 1024;
  };
  int rb = 0, ns = 2;
  for (int c = 16; c >= 1 && rb == 0; c /= 2) {
    if (c > rb_max || LX % c != 0 || c * QX > 128 || (c * QX) % 32 != 0) continue;
    for (int n = ns_want; n >= 2; --n)
      if (smem_for(c, n) <= budget) { rb = c; ns = n; break; }
  }
  if (rb == 0) return false;
  auto smem_of = [&](int n) { return smem_for(rb, n); };
  const unsigned smem = (unsigned)smem_of(ns);
  sp.kind = 7;
  sp.nd = s.nd;
  sp.vec = 1;
  sp.op_modes.assign(sp.nops, M_CONST);
  for (int k = 0; k < sp.nops; ++k) {
    if ((tmask >> k) & 1u) sp.op_modes[k] = M_STAGED;
    else if ((pmask >> k) & 1u) sp.op_modes[k] = M_CONTIG;
  }
  sp.kept_mask = 0;
  for (int d = 0; d < s.nd; ++d) if (!s.red[d]) sp.kept_mask |= 1u << d;
  int qxp = 1;
  while (qxp < QX) qxp *= 2;
  sp.qd = qd; sp.qx = (int)QX; sp.qxp = qxp; sp.tp = tp; sp.rb = rb; sp.tmask = tmask; sp.tile_bytes = 0;
  sp.ns = ns; sp.ld = ld; sp.npc = npc; sp.pmask = pmask; sp.umask = umask; sp.uumask = uumask; sp.ltp8 = 2;
  sp.nob = nob;
  sp.nmaps = nt + npc + (sp.has_out ? 1 + nx : 0);
  // extra tapes over p-row and uniform operands only run on whole 16-byte
  // chunks of the tiles (the p-row and output tiles share one layout)
  sp.xvec = 0;
  if (nx > 0) {
    bool ok = true;
    for (const Tape& xt : sp.xtapes)
      for (uint32_t ins : xt.instrs) {
        const int op = (int)(ins >> 24), idx = (int)(ins & 0xffffff);
        if ((op == NCA_OP_LOAD_NCARR || op == NCA_OP_LOAD_SOARR) && !(((pmask | umask) >> idx) & 1u)) ok = false;
      }
    sp.xvec = ok ? 1 : 0;
  }
  // as many CTAs per SM as their shared memory allows (228 KiB per SM, 1 KiB
  // reserved per CTA), at most three: ptxas caps the registers to match
  sp.minb = (int)std::max<int64_t>(1, std::min<int64_t>(3, (228 * 1024) / ((int64_t)smem + 1024)));
  sp.grp = 1;
  // tensor maps: staged operands, p operands, the stored value
  struct Maps { CUtensorMap m[NCA_MAX_OPERANDS + 1 + NCA_MAX_EXTRA_OUTS]; };
  Maps maps;
  memset(&maps, 0, sizeof(maps));
  std::vector<int> other;
  for (int d = 0; d < pd; ++d) if (d != qd && d != ld) other.push_back(d);
  auto encode = [&](CUtensorMap* m, const CArr& a, bool staged) {
    cuuint64_t dims[5], strides[4];
    cuuint32_t box[5], estr[5] = {1u, 1u, 1u, 1u, 1u};
    int r = 0;
    if (staged) {
      dims[0] = (cuuint64_t)(QX * LX); box[0] = 32;
      dims[1] = (cuuint64_t)P; strides[0] = (cuuint64_t)a.st[pd]; box[1] = (cuuint32_t)tp;
      r = 2;
    } else {
      dims[0] = (cuuint64_t)P; box[0] = (cuuint32_t)tp;
      dims[1] = (cuuint64_t)QX; strides[0] = (cuuint64_t)a.st[qd]; box[1] = (cuuint32_t)QX;
      dims[2] = (cuuint64_t)LX; strides[1] = (cuuint64_t)a.st[ld]; box[2] = (cuuint32_t)rb;
      r = 3;
    }
    for (int d : other) { dims[r] = (cuuint64_t)s.shape[d]; strides[r - 1] = (cuuint64_t)a.st[d]; box[r] = 1; ++r; }
    check_cu(drv().cuTensorMapEncodeTiled(m, CU_TENSOR_MAP_DATA_TYPE_UINT32, (cuuint32_t)r, const_cast<char*>(a.base),
                                          dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                          CU_TENSOR_MAP_SWIZZLE_128B,
                                          // staged rows are read 4 boxes (512 bytes) at a time; p rows
                                          // are 128-byte boxes whose neighbour belongs to another unit
                                          staged ? CU_TENSOR_MAP_L2_PROMOTION_L2_256B : CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE),
             "cuTensorMapEncodeTiled");
  };
  int mi = 0;
  for (int k = 0; k < sp.nops; ++k) if ((tmask >> k) & 1u) encode(&maps.m[mi++], s.ops[k], true);
  for (int k = 0; k < sp.nops; ++k) if ((pmask >> k) & 1u) encode(&maps.m[mi++], s.ops[k], false);
  if (sp.has_out) encode(&maps.m[mi++], s.out, false);
  for (const CArr& a : s.xouts) encode(&maps.m[mi++], a, false);
  CUfunction fn = kernel_for(sp, tape);
  const int sms = sm_count(current_device());
  int per_sm = 0;
  check_cu(drv().cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem), "smem attribute");
  // 8 consumer warps, a load warp and (when a value is stored) a store warp
  const int threads = 256 + 32 + (sp.has_out ? 32 : 0);
  check_cu(drv().cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem), "occupancy");
  if (per_sm < 1) return false;
  const int64_t U = KN / ((int64_t)tp * QX), NB = RN / rb, W = U * NB;
  const int64_t G = std::min<int64_t>((int64_t)sms * per_sm, W);
  const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
  std::vector<uint64_t> w;
  fill_common_words(s, sp, tape, L, w);
  w[L.nsplit] = (uint64_t)G; w[L.chunk] = 0; w[L.keptn] = (uint64_t)KN; w[L.redn] = (uint64_t)RN;
  // partial pieces of split units, and one arrival counter per unit (zeroed
  // here; the merging CTA resets its unit's counter)
  const int64_t slots = (G + U) * (int64_t)tp * QX;
  const size_t pbytes = sp.nred > 0 ? (size_t)slots * 8 * ((sp.has_sum ? 1 : 0) + (sp.has_max ? 2 : 0) + (sp.has_min ? 2 : 0)) : 0;
  const size_t cbytes = sp.nred > 0 ? ((size_t)U * 4 + 255) / 256 * 256 : 0;
  StreamScratch part(pbytes + cbytes, stream);
  if (sp.nred > 0) {
    uint64_t* p = (uint64_t*)part.ptr;
    if (sp.has_sum) { w[L.psum] = (uint64_t)(uintptr_t)p; p += slots; }
    if (sp.has_max) { w[L.pmax] = (uint64_t)(uintptr_t)p; p += 2 * slots; }
    if (sp.has_min) { w[L.pmin] = (uint64_t)(uintptr_t)p; p += 2 * slots; }
    w[L.aux] = (uint64_t)(uintptr_t)p;
    check_cuda(cudaMemsetAsync(p, 0, cbytes, stream), "unit counters");
  }
  // the kernel takes the words and the first nmaps tensor maps
  std::vector<unsigned char> mp(sizeof(CUtensorMap) * sp.nmaps + 64);
  unsigned char* mpa = (unsigned char*)(((uintptr_t)mp.data() + 63) & ~(uintptr_t)63);
  memcpy(mpa, &maps, sizeof(CUtensorMap) * sp.nmaps);
  void* params[] = {w.data(), mpa};
  count_launch();
  check_cu(drv().cuLaunchKernel(fn, (unsigned)G, 1, 1, (unsigned)threads, 1, 1, smem, (CUstream)stream, params, nullptr),
           "cuLaunchKernel");
  return true;
}

// Launches kind 6 (and its finalize when the loop dims are split). Kept dims
// are those with s.red false; KN / RN are the kept / loop element counts.
static void launch_staged(const Space& s, Spec sp, const Tape& tape, int qd, uint32_t tmask, int nt, int64_t KN,
                          int64_t RN, cudaStream_t stream) {
  if (launch_staged_async(s, sp, tape, qd, tmask, nt, KN, RN, stream)) return;
  const int sms = sm_count(current_device());
  const int pd = s.nd - 1;
  const int64_t P = s.shape[pd], QX = s.shape[qd];
  const int wsz = dtinfo(sp.w).size;
  sp.nd = s.nd;
  sp.kind = 6;
  {
    // resident CTAs per SM asked of ptxas (NCA_STAGED_MINB overrides; 2 caps
    // registers at 128 and measured fastest with groups of 4 loop indices)
    static const int minb = [] {
      const char* e = getenv("NCA_STAGED_MINB");
      const int v = e ? atoi(e) : 0;
      return v >= 1 && v <= 8 ? v : 2;
    }();
    sp.minb = minb;
    static const int grp = [] {
      const char* e = getenv("NCA_STAGED_GRP");
      const int v = e ? atoi(e) : 0;
      return v == 1 || v == 2 || v == 4 || v == 8 ? v : 4;
    }();
    sp.grp = grp;
  }
  // 4-wide vectors along p for the other operands and the stored value when
  // they are contiguous and aligned there (plan_vec), else scalars
  plan_vec(s, sp, 4, sp.has_out);
  for (int k = 0; k < sp.nops; ++k) if ((tmask >> k) & 1u) sp.op_modes[k] = M_STAGED;
  sp.kept_mask = 0;
  for (int d = 0; d < s.nd; ++d) if (!s.red[d]) sp.kept_mask |= 1u << d;
  sp.qd = qd;
  sp.qx = (int)QX;
  sp.qxp = 1;
  while (sp.qxp < QX) sp.qxp *= 2;
  sp.tmask = tmask;
  // rb: power of two with qxp * rb <= 256; tp a multiple of 256 / (qxp * rb)
  // with at most 32 staged registers per thread and operand
  // tile of tp p values (a multiple of vec); rb: power of two with qxp * rb
  // <= 256 and at most 16 staged registers per thread over all staged operands
  sp.tp = P > 32 ? 64 : 32;
  sp.rb = std::max(1, std::min(16, 256 / sp.qxp));
  while (sp.rb > 1 && (int64_t)sp.tp * sp.qxp * sp.rb / 256 * nt > 16) sp.rb /= 2;
  const int64_t budget = 40 * 1024 / (int64_t)(nt * sp.tp * wsz);
  while (sp.rb > 1 && (int64_t)sp.rb * QX + 1 > budget) sp.rb /= 2;
  const int pstep = 256 / (sp.qxp * sp.rb);
  if (sp.tp < pstep) sp.tp = pstep;
  sp.tile_bytes = (int)(((int64_t)nt * sp.tp * (sp.rb * QX + 1) * wsz + 15) / 16 * 16);
  const int64_t ptiles = cdiv(P, sp.tp);
  const int64_t units = (KN / (P * QX)) * ptiles;
  const unsigned smem = (unsigned)(sp.tile_bytes + 2 * (sp.nops + 1) * sp.rb * 8);
  CUfunction fn = kernel_for(sp, tape);
  // split the loop dims so the grid fills whole waves of resident CTAs
  int per_sm = 1;
  if (drv().cuOccupancyMaxActiveBlocksPerMultiprocessor)
    check_cu(drv().cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, smem), "occupancy");
  const int64_t wave = (int64_t)sms * std::max(per_sm, 1);
  int64_t S = 1;
  if (RN > 0) {
    const int64_t smax = cdiv(RN, sp.rb);
    if (units < wave) S = std::min<int64_t>(cdiv(wave, units), smax);
    // round the CTA count up to whole waves when the loop dims allow it
    const int64_t ctas = units * S;
    if (ctas > wave && ctas % wave != 0) {
      const int64_t want = cdiv(ctas, wave) * wave;
      if (want % units == 0 && want / units <= smax) S = want / units;
    }
  }
  int64_t C = RN > 0 ? cdiv(cdiv(RN, S), sp.rb) * sp.rb : 0;
  if (C > 0) S = cdiv(RN, C);
  if (S < 1) S = 1;
  const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
  std::vector<uint64_t> w;
  fill_common_words(s, sp, tape, L, w);
  w[L.nsplit] = (uint64_t)S; w[L.chunk] = (uint64_t)C; w[L.keptn] = (uint64_t)KN; w[L.redn] = (uint64_t)RN;
  const bool split = S > 1 && sp.nred > 0;
  StreamScratch part(split ? (size_t)(S * KN) * 8 * ((sp.has_sum ? 1 : 0) + (sp.has_max ? 2 : 0) + (sp.has_min ? 2 : 0)) : 0,
                     stream);
  if (split) {
    uint64_t* p = (uint64_t*)part.ptr;
    if (sp.has_sum) { w[L.psum] = (uint64_t)(uintptr_t)p; p += S * KN; }
    if (sp.has_max) { w[L.pmax] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
    if (sp.has_min) { w[L.pmin] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
  }
  launch(fn, units * S, w, stream, smem);
  if (split) {
    launch_finalize(sp, tape, KN, S, sms, w, stream);
  }
}

void expr_eval(const Tape& tape, const nca_view* ops, int nops, const nca_view& out, cudaStream_t stream) {
  check_view(out, "out");
  if (nops < 0 || nops > NCA_MAX_OPERANDS) fail(NCA_ERR_LIMIT, "%d operands (0..%d)", nops, NCA_MAX_OPERANDS);
  if (tape.n_arrays > nops) fail(NCA_ERR_INVALID, "tape loads more operands than given");
  for (int k = 0; k < nops; ++k) { check_view(ops[k], "operand", true); check_broadcast(out.shape, out.ndim, ops[k], "operand"); }
  int64_t n = 1;
  for (int d = 0; d < out.ndim; ++d) n *= out.shape[d];
  if (n == 0) return;
  Space s = make_space(out.shape, out.ndim, ops, nops, &out, 0, nullptr, 0);
  if (!tape.uses_idx && s.nd > 1) {
    std::vector<int> perm(s.nd);
    for (int d = 0; d < s.nd; ++d) perm[d] = d;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) {
      return std::llabs(s.out.st[a]) > std::llabs(s.out.st[b]);
    });
    permute_dims(s, perm);
  }
  merge_dims(s);
  ensure_nd1(s);
  Spec sp;
  sp.nops = nops; sp.nd = s.nd; sp.has_out = true; sp.out_dtype = out.dtype; sp.w = tape.compute_dtype;
  sp.r = tape.result_dtype; sp.nscal = (int)tape.scalar_dtypes.size();
  for (int k = 0; k < nops; ++k) sp.op_dtypes.push_back(ops[k].dtype);
  for (int k = 0; k < nops; ++k) if (s.ops[k].ptr) sp.ptrmask |= 1u << k;
  // transposed operands: stage them (kind 6) with p and q kept and every other
  // dim walked as a loop dim; the output must be contiguous along p
  if (!tape.uses_idx && sp.ptrmask == 0 && s.nd >= 2 && s.out.st[s.nd - 1] == dtinfo(out.dtype).size) {
    uint32_t tmask = 0;
    int nt = 0;
    const int qd = find_staged(s, tmask, nt);
    if (qd >= 0) {
      Space t = s;
      int64_t KN = 1, RN = 1;
      for (int d = 0; d < t.nd; ++d) {
        t.red[d] = !(d == qd || d == t.nd - 1);
        if (t.red[d]) RN *= t.shape[d]; else KN *= t.shape[d];
      }
      launch_staged(t, sp, tape, qd, tmask, nt, KN, RN, stream);
      return;
    }
  }
  bool flat = s.nd == 1 && s.out.st[0] == dtinfo(out.dtype).size && sp.ptrmask == 0;
  for (int k = 0; k < nops && flat; ++k)
    if (s.ops[k].st[0] != 0 && s.ops[k].st[0] != dtinfo(ops[k].dtype).size) flat = false;
  plan_vec(s, sp, 16, true);
  if (flat) {
    for (int k = 0; k < nops; ++k) if (sp.op_modes[k] == M_STRIDED && sp.vec > 1) flat = false;
  }
  sp.kind = flat ? 1 : 2;
  if (sp.kind == 2) {
    plan_pairs(s, sp);
    sp.op_salias.assign(nops, -1);
    for (int k = 0; k < nops; ++k) {
      if (s.ops[k].ptr) continue;
      for (int j = 0; j < k; ++j) {
        if (s.ops[j].ptr || sp.op_salias[j] >= 0) continue;
        bool same = true;
        for (int d = 0; d < s.nd; ++d) if (s.ops[j].st[d] != s.ops[k].st[d]) same = false;
        if (same) { sp.op_salias[k] = j; break; }
      }
    }
  }
  sp.unroll = flat ? (nops <= 2 ? 4 : nops <= 4 ? 2 : 1) : 1;
  const int64_t total = s.total();
  bool small_dims = true;
  for (int d = 0; d < s.nd; ++d) if (s.shape[d] >= (1ll << 31)) small_dims = false;
  sp.idx32 = (total / sp.vec < (1ll << 31) && small_dims) ? 1 : 0;
  const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, 0, sp.ptrmask != 0);
  std::vector<uint64_t> w;
  fill_common_words(s, sp, tape, L, w);
  for (int d = 0; d < s.nd; ++d) {
    int64_t dv = s.shape[d];
    if (d == s.nd - 1) dv /= sp.vec;
    compute_magic(dv, w[L.magic + d]);
  }
  const int dev = current_device();
  const int64_t groups = total / sp.vec;
  // schedule: threads per block, vector groups per thread per trip (kind 1)
  // and resident threads per SM the grid is capped at; the autotuner's
  // cached choice for this (kind, dtypes, operand count, vector width, size
  // class), else the heuristic (candidate 0)
  std::vector<std::vector<int>> cands = {{256, sp.unroll, 2048}};
  if (sp.kind == 1) {
    for (std::vector<int> c : std::vector<std::vector<int>>{{256, 1, 2048}, {256, 2, 2048}, {256, 4, 2048},
                                                             {512, 2, 2048}, {128, 4, 1024}, {256, 4, 4096}})
      if (c != cands[0]) cands.push_back(c);
  } else {
    cands.push_back({512, 1, 2048});
    cands.push_back({128, 1, 2048});
    cands.push_back({256, 1, 1024});
    cands.push_back({256, 1, 4096});
  }
  std::string key = "ew|k" + std::to_string(sp.kind) + "|" + std::to_string(out.dtype) + "|" +
                    std::to_string(tape.compute_dtype) + "|";
  for (int k = 0; k < nops; ++k) key += std::to_string(ops[k].dtype) + ".";
  key += "|v" + std::to_string(sp.vec) + "|n" + size_class(total) + "|d" + std::to_string(s.nd);
  auto run = [&](const std::vector<int>& c) {
    Spec sc = sp;
    sc.block = c[0];
    sc.unroll = sp.kind == 1 ? c[1] : 1;
    CUfunction fn = kernel_for(sc, tape);
    const int64_t grid = std::min<int64_t>(cdiv(std::max<int64_t>(groups, 1), (int64_t)sc.block * sc.unroll),
                                           (int64_t)sm_count(dev) * std::max(1, c[2] / sc.block));
    launch(fn, grid, w, stream, 0, (unsigned)sc.block);
  };
  std::vector<int> choice;
  if (tune_get(key, choice) && choice.size() == 3 && (choice[0] == 128 || choice[0] == 256 || choice[0] == 512) &&
      choice[1] >= 1 && choice[1] <= 4 && choice[2] >= 256) {
    run(choice);
    return;
  }
  if (tune_should_search(stream) && groups >= (1 << 16) && rerun_safe(ops, nops, &out, 1)) {
    const int best = tune_pick(stream, (int)cands.size(), [&](int i) { run(cands[(size_t)i]); });
    tune_put(key, cands[(size_t)best]);
    run(cands[(size_t)best]);
    return;
  }
  run(cands[0]);
}

int reduce_out_dtype(int op, int in_dt) {
  switch (op) {
    case NCA_RED_SUM: return sum_dtype(in_dt);
    case NCA_RED_MEAN: return NCA_FLOAT64;
    case NCA_RED_MAX: case NCA_RED_MIN: return arith_dtype(in_dt);
    case NCA_RED_ARGMAX: case NCA_RED_ARGMIN: return NCA_INT64;
  }
  fail(NCA_ERR_INVALID, "unknown reduction op %d", op);
}

// NCA_K4_BULK=1 puts eligible outer reductions on the bulk-staged row-lane
// form (measured, GB300, CUDA-graph replays: sum over axis 0 of (4096, 16384)
// float32 0.72 of measured HBM at best over 1-4 column blocks, 2-8 stages and
// 4-32 rows per stage, against 0.73 for the plain row-lane form; max over axis
// 1 of (256, 256, 1024) 0.79 against 0.81: the loads in flight are not what
// bounds these shapes); any NCA_K4_ROWS setting names another form
static bool k4b_on() {
  const char* e = getenv("NCA_K4_BULK");
  const char* r = getenv("NCA_K4_ROWS");
  return e && e[0] == '1' && !(r && r[0]);
}

// NCA_K4_ROWS=0 keeps outer reductions on the thread-per-column-group form
// unless a tuned choice names the row-lane form; NCA_K4_ROWS=2 has the
// row-lane form merge its splits in a finalize launch instead of the last CTA
// (tests and measurements)
static bool k4r_off() {
  const char* e = getenv("NCA_K4_ROWS");
  return e && e[0] == '0';
}
static int k4r_lastcta() {
  const char* e = getenv("NCA_K4_ROWS");
  return (e && e[0] == '2') ? 0 : 1;
}
// NCA_K4_ROWS=3: the row-lane form on a persistent grid of equal unit ranges
// (a tuner candidate; measured slower than the splits on (4096, 16384) axis 0,
// 0.66 against 0.73, and (256, 256, 1024) axis 1, 0.74 against 0.77)
static bool k4r_persistent() {
  const char* e = getenv("NCA_K4_ROWS");
  return e && e[0] == '3';
}

bool expr_reduce(const Tape& tape, const nca_view* ops, int nops, const nca_view* out,
                 const nca_reduction* reds, int nred, cudaStream_t stream, const Tape* xtapes,
                 const nca_view* xouts, int nx) {
  if (nred < 1 || nred > NCA_MAX_REDUCTIONS) fail(NCA_ERR_LIMIT, "%d reductions (1..%d)", nred, NCA_MAX_REDUCTIONS);
  if (nops < 0 || nops > NCA_MAX_OPERANDS) fail(NCA_ERR_LIMIT, "%d operands (0..%d)", nops, NCA_MAX_OPERANDS);
  if (tape.n_arrays > nops) fail(NCA_ERR_INVALID, "tape loads more operands than given");
  for (int k = 0; k < nops; ++k) check_view(ops[k], "operand", true);
  int64_t lshape[NCA_MAX_NDIM];
  int n;
  if (out) {
    check_view(*out, "expr_out");
    n = out->ndim;
    for (int d = 0; d < n; ++d) lshape[d] = out->shape[d];
  } else {
    n = broadcast_shape(ops, nops, lshape);
  }
  for (int k = 0; k < nops; ++k) check_broadcast(lshape, n, ops[k], "operand");
  const uint32_t all = n >= 32 ? 0xffffffffu : ((1u << n) - 1u);
  const uint32_t mask = reds[0].axes_mask & all;
  int kept_count = 0;
  for (int d = 0; d < n; ++d) if (!((mask >> d) & 1u)) ++kept_count;
  bool has_sum = false, has_max = false, has_min = false;
  uint32_t red_ops = 0;
  for (int k = 0; k < nred; ++k) {
    if ((reds[k].axes_mask & all) != mask) fail(NCA_ERR_INVALID, "all reductions of one call must share axes_mask");
    const int op = reds[k].op;
    const int want = reduce_out_dtype(op, tape.result_dtype);
    const nca_view& ov = reds[k].out;
    check_view(ov, "reduction out");
    if (ov.dtype != want)
      fail(NCA_ERR_DTYPE, "reduction %d writes dtype %d, expected %s", k, ov.dtype, dtinfo(want).name);
    if (ov.ndim != kept_count && !(kept_count == 0 && ov.ndim == 1 && ov.shape[0] == 1))
      fail(NCA_ERR_SHAPE, "reduction %d output has %d dims, expected %d", k, ov.ndim, kept_count);
    int kd = 0;
    for (int d = 0; d < n && kept_count > 0; ++d) {
      if ((mask >> d) & 1u) continue;
      if (ov.shape[kd] != lshape[d]) fail(NCA_ERR_SHAPE, "reduction %d output extent mismatch on axis %d", k, d);
      ++kd;
    }
    if (op == NCA_RED_SUM || op == NCA_RED_MEAN) has_sum = true;
    if (op == NCA_RED_MAX || op == NCA_RED_ARGMAX) has_max = true;
    if (op == NCA_RED_MIN || op == NCA_RED_ARGMIN) has_min = true;
    red_ops |= (uint32_t)op << (4 * k);
  }
  // reduction views with kept_count==0 but ndim 1: treat their stride as unused
  std::vector<nca_reduction> rv(reds, reds + nred);
  for (auto& r : rv) if (kept_count == 0) { r.out.ndim = 0; }
  int64_t KN = 1, RN = 1;
  for (int d = 0; d < n; ++d) { if ((mask >> d) & 1u) RN *= lshape[d]; else KN *= lshape[d]; }
  if (nx > 0) {
    // extra outputs: fused into the staged pass only (the caller runs them
    // separately when this returns false); each has out's shape
    if (!out || KN * RN == 0) return false;
    for (int x = 0; x < nx; ++x) {
      check_view(xouts[x], "extra out");
      if (xouts[x].ndim != n) return false;
      for (int d = 0; d < n; ++d) if (xouts[x].shape[d] != lshape[d]) return false;
      if (xtapes[x].n_arrays > nops || xtapes[x].uses_idx) return false;
    }
  }
  if (KN == 0) return true;
  Space s = make_space(lshape, n, ops, nops, out, mask, rv.data(), nred, xouts, nx);
  const int dev = current_device();
  const int sms = sm_count(dev);
  Spec sp;
  sp.nops = nops; sp.has_out = out != nullptr; sp.out_dtype = out ? out->dtype : 0; sp.w = tape.compute_dtype;
  sp.r = tape.result_dtype; sp.nscal = (int)tape.scalar_dtypes.size(); sp.nred = nred; sp.red_ops = red_ops;
  sp.has_sum = has_sum; sp.has_max = has_max; sp.has_min = has_min;
  for (int k = 0; k < nops; ++k) sp.op_dtypes.push_back(ops[k].dtype);
  for (int k = 0; k < nops; ++k) if (s.ops[k].ptr) sp.ptrmask |= 1u << k;
  for (int x = 0; x < nx; ++x) {
    sp.xtapes.push_back(xtapes[x]);
    sp.xout_dtypes.push_back(xouts[x].dtype);
    sp.nscal += (int)xtapes[x].scalar_dtypes.size();
  }
  merge_dims(s);
  ensure_nd1(s);
  const bool inner_reduced = (RN == 0) || s.red[s.nd - 1];
  if (nx > 0 && (inner_reduced || sp.ptrmask != 0 || tape.uses_idx)) return false;
  if (inner_reduced && out) fail(NCA_ERR_UNSUPPORTED, "storing the expression while reducing its innermost axis is not supported; reduce without expr_out");
  if (inner_reduced) {
    // order [kept..., reduced...]
    std::vector<int> perm;
    for (int d = 0; d < s.nd; ++d) if (!s.red[d]) perm.push_back(d);
    for (int d = 0; d < s.nd; ++d) if (s.red[d]) perm.push_back(d);
    bool identity = true;
    for (int d = 0; d < s.nd; ++d) if (perm[d] != d) identity = false;
    if (!identity) {
      if (tape.uses_idx) fail(NCA_ERR_UNSUPPORTED, "IDX in a reduction whose kept axes follow reduced axes");
      permute_dims(s, perm);
      merge_dims(s);
    }
    sp.nd = s.nd;
    sp.kind = 3;
    int nkept = 0;
    for (int d = 0; d < s.nd; ++d) if (!s.red[d]) ++nkept;
    sp.nkept = nkept;
    for (int d = 0; d < s.nd; ++d) if (!s.red[d]) sp.kept_mask |= 1u << d;
    if (RN > 0) plan_vec(s, sp, 16, false); else { sp.vec = 1; sp.op_modes.assign(nops, M_STRIDED); }
    if (sp.vec > 1 && s.shape[s.nd - 1] % sp.vec != 0) { sp.vec = 1; sp.op_modes.assign(nops, M_STRIDED); }
    // team of threads per kept position: a block for long reductions, a warp
    // for medium ones; along one reduced dim, two threads below 1024 elements
    // (whole sectors per load, where one thread per row uses half of each, and
    // no warp-wide tree) and one thread up to 8; over several reduced dims, one
    // thread below 64 elements (its offsets from a per-block table)
    const int heur_team = s.nd - sp.nkept == 1 ? (RN >= 4096 ? 256 : (RN >= 1024 ? 32 : (RN > 8 ? 2 : 1)))
                                               : (RN >= 4096 ? 256 : (RN >= 64 ? 32 : 1));
    // one launch (plus its finalize) with teams of `team` threads
    auto run_team = [&](int team) {
      sp.team = team;
      sp.lastcta = 0;
      if (const char* e = getenv("NCA_K3_UNROLL")) sp.k3u = std::max(1, std::min(16, atoi(e)));   // measurements
      const int64_t tpb = 256 / sp.team;
      const int64_t target = (int64_t)sms * tpb * 8;
      int64_t S = 1;
      if (KN < target && RN > 0) {
        S = cdiv(target, KN);
        S = std::min<int64_t>(S, std::max<int64_t>(1, RN / ((int64_t)sp.team * sp.vec * 8)));
      }
      int64_t C = RN > 0 ? cdiv(RN, S) : 0;
      C = cdiv(C, sp.vec) * sp.vec;
      if (C > 0) S = cdiv(RN, C);
      if (S < 1) S = 1;
      // one-thread teams over at most 8 vectors, no splits, no pointer
      // operands: a thread gathers the operands of 2 units before reducing
      // either (NCA_K3_UNITS: 1 keeps one unit at a time; the binning
      // reshape-sum of (32, 512, 1024) float32 at 1 / 2 / 3 / 4 / 8 units:
      // 0.56 / 0.66-0.68 / 0.60 / 0.60 / 0.49 of measured HBM)
      sp.k3rv = 0;
      sp.k3tu = 1;
      if (sp.team == 1 && S == 1 && sp.ptrmask == 0 && RN > 0 && RN % sp.vec == 0 && RN / sp.vec <= 8) {
        int tu = 2;
        if (const char* e = getenv("NCA_K3_UNITS")) tu = std::max(1, std::min(8, atoi(e)));
        if (tu > 1) { sp.k3rv = (int)(RN / sp.vec); sp.k3tu = tu; }
      }
      const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
      std::vector<uint64_t> w;
      fill_common_words(s, sp, tape, L, w);
      w[L.nsplit] = (uint64_t)S; w[L.chunk] = (uint64_t)C; w[L.keptn] = (uint64_t)KN; w[L.redn] = (uint64_t)RN;
      // 32-bit coordinate decoding (magic-number division) when every index fits
      {
        bool small = KN * S < (1ll << 31) && RN < (1ll << 31);
        for (int d = 0; d < s.nd; ++d) if (s.shape[d] >= (1ll << 31)) small = false;
        if (small) for (int d = 0; d < s.nd; ++d) compute_magic(std::max<int64_t>(s.shape[d], 1), w[L.magic + d]);
        sp.idx32 = small ? 1 : 0;
      }
      // block teams over few kept positions (global reductions): the CTA that
      // stores the last partial of a kept position merges them in the order the
      // finalize pass uses (one arrival counter per kept position, zeroed here),
      // so there is no second launch and the result is the same
      sp.lastcta = (S > 1 && sp.team == 256 && KN <= 64) ? 1 : 0;
      const size_t pbytes = S > 1 ? (size_t)(S * KN) * 8 * ((has_sum ? 1 : 0) + (has_max ? 2 : 0) + (has_min ? 2 : 0)) : 0;
      const size_t cbytes = sp.lastcta ? ((size_t)KN * 4 + 255) / 256 * 256 : 0;
      StreamScratch part(pbytes + cbytes, stream);
      if (S > 1) {
        uint64_t* p = (uint64_t*)part.ptr;
        if (has_sum) { w[L.psum] = (uint64_t)(uintptr_t)p; p += S * KN; }
        if (has_max) { w[L.pmax] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
        if (has_min) { w[L.pmin] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
        if (sp.lastcta) {
          w[L.aux] = (uint64_t)(uintptr_t)p;
          check_cuda(cudaMemsetAsync(p, 0, cbytes, stream), "arrival counters");
        }
      }
      CUfunction fn = kernel_for(sp, tape);
      // warp and smaller teams stride over their units from a few blocks per SM
      // (one-thread teams build their reduced-offset table once per block); a
      // block team takes one unit per block, so one block's tree and store
      // overlap the other blocks' loads
      const int64_t groups = cdiv(KN * S, tpb);
      launch(fn, sp.team == 256 ? groups : std::min<int64_t>(groups, (int64_t)sms * 8), w, stream);
      if (S > 1 && !sp.lastcta) {
        launch_finalize(sp, tape, KN, S, sms, w, stream);
      }
    };
    // team size: the autotuner's cached choice for this (dtypes, ops, reduced
    // and kept size class, dims), else the heuristic; rows of 64 to 64 Ki
    // elements are searched in search mode
    std::string key = "red|k3|" + std::to_string(tape.compute_dtype) + "|" + std::to_string(red_ops) + "|";
    for (int k = 0; k < nops; ++k) key += std::to_string(ops[k].dtype) + ".";
    key += "|r" + size_class(RN) + "|k" + size_class(KN) + "|d" + std::to_string(s.nd) + "." + std::to_string(sp.nkept) +
           "|v" + std::to_string(sp.vec);
    const bool one_dim = s.nd - sp.nkept == 1;
    auto team_ok = [&](int t) { return t == 2 || t == 32 || t == 256 || (t == 1 && (one_dim || RN < 64)); };
    std::vector<int> choice;
    if (tune_get(key, choice) && choice.size() == 1 && team_ok(choice[0])) {
      run_team(choice[0]);
      return true;
    }
    std::vector<nca_view> routs;
    for (int k = 0; k < nred; ++k) routs.push_back(rv[(size_t)k].out);
    if (RN >= 64 && RN <= 65536 && KN * RN >= (1 << 16) && tune_should_search(stream) &&
        rerun_safe(ops, nops, routs.data(), nred)) {
      std::vector<int> cands = {heur_team};
      for (int t : {1, 2, 32, 256})
        if (t != heur_team && team_ok(t) && (t != 1 || RN <= 1024)) cands.push_back(t);
      const int best = tune_pick(stream, (int)cands.size(), [&](int i) { run_team(cands[(size_t)i]); });
      tune_put(key, {cands[(size_t)best]});
      run_team(cands[(size_t)best]);
      return true;
    }
    run_team(heur_team);
    return true;
  }
  // innermost dim kept. Operands strided along it but contiguous along another
  // kept dim q are staged through shared memory (kind 6); otherwise RED_OUTER.
  sp.nd = s.nd;
  {
    uint32_t tmask = 0;
    int nt = 0;
    const int qd = (tape.uses_idx || sp.ptrmask != 0) ? -1 : find_staged(s, tmask, nt);
    if (qd >= 0) {
      if (nx > 0) return launch_staged_async(s, sp, tape, qd, tmask, nt, KN, RN, stream);
      launch_staged(s, sp, tape, qd, tmask, nt, KN, RN, stream);
      return true;
    }
  }
  if (nx > 0) return false;
  sp.kind = 4;
  sp.kept_mask = 0;
  for (int d = 0; d < s.nd; ++d) if (!s.red[d]) sp.kept_mask |= 1u << d;
  plan_vec(s, sp, 4, out != nullptr);
  const int64_t KG = KN / sp.vec;
  // one launch (plus its finalize) with `unroll` rows per thread in flight and
  // splits chosen for `tps` threads per SM
  // the row-lane form applies with one reduced dim, no pointer axes and no IDX
  int nrd = 0, rdim = -1;
  for (int d = 0; d < s.nd; ++d) if (s.red[d]) { ++nrd; rdim = d; }
  const bool rows_ok = nrd == 1 && sp.ptrmask == 0 && !tape.uses_idx && RN > 0;
  // row-lane form: 4 row lanes per warp, 64 kept groups per CTA; splits for
  // `tps` threads per SM with at least 8 rows per row lane
  auto run_k4r = [&](int unroll, int tps, int lastcta) {
    const int R = 4, GPC = (32 / R) * 8;
    sp.unroll = unroll;
    sp.k4r = R;
    sp.rd = rdim;
    const int64_t nset = cdiv(KG, GPC);
    if (tps == 0) {
      // persistent grid: every resident CTA, units of 4R rows split evenly
      sp.k4p = 1;
      sp.lastcta = 0;
      CUfunction fn = kernel_for(sp, tape);
      int per_sm = 0;
      check_cu(drv().cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0), "occupancy");
      const int64_t W = nset * cdiv(RN, 4 * R);
      const int64_t G = std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * std::max(per_sm, 1), W));
      const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
      std::vector<uint64_t> w;
      fill_common_words(s, sp, tape, L, w);
      w[L.nsplit] = (uint64_t)G; w[L.chunk] = 0; w[L.keptn] = (uint64_t)KN; w[L.redn] = (uint64_t)RN;
      const int64_t slots = (G + nset) * GPC * sp.vec;
      const size_t pbytes = (size_t)slots * 8 * ((has_sum ? 1 : 0) + (has_max ? 2 : 0) + (has_min ? 2 : 0));
      const size_t cbytes = ((size_t)nset * 4 + 255) / 256 * 256;
      StreamScratch part(pbytes + cbytes, stream);
      uint64_t* p = (uint64_t*)part.ptr;
      if (has_sum) { w[L.psum] = (uint64_t)(uintptr_t)p; p += slots; }
      if (has_max) { w[L.pmax] = (uint64_t)(uintptr_t)p; p += 2 * slots; }
      if (has_min) { w[L.pmin] = (uint64_t)(uintptr_t)p; p += 2 * slots; }
      w[L.aux] = (uint64_t)(uintptr_t)p;
      check_cuda(cudaMemsetAsync(p, 0, cbytes, stream), "arrival counters");
      launch(fn, G, w, stream);
      sp.k4r = 0;
      sp.rd = 0;
      sp.k4p = 0;
      return;
    }
    const int64_t target = (int64_t)sms * tps;
    int64_t S = std::max<int64_t>(1, std::min<int64_t>(cdiv(target, nset * 256), RN / (8 * R)));
    int64_t C = cdiv(RN, S);
    S = cdiv(RN, C);
    const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
    std::vector<uint64_t> w;
    fill_common_words(s, sp, tape, L, w);
    w[L.nsplit] = (uint64_t)S; w[L.chunk] = (uint64_t)C; w[L.keptn] = (uint64_t)KN; w[L.redn] = (uint64_t)RN;
    sp.lastcta = (lastcta && S > 1) ? 1 : 0;
    const size_t pbytes = S > 1 ? (size_t)(S * KN) * 8 * ((has_sum ? 1 : 0) + (has_max ? 2 : 0) + (has_min ? 2 : 0)) : 0;
    const size_t cbytes = sp.lastcta ? ((size_t)nset * 4 + 255) / 256 * 256 : 0;
    StreamScratch part(pbytes + cbytes, stream);
    if (S > 1) {
      uint64_t* p = (uint64_t*)part.ptr;
      if (has_sum) { w[L.psum] = (uint64_t)(uintptr_t)p; p += S * KN; }
      if (has_max) { w[L.pmax] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
      if (has_min) { w[L.pmin] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
      if (sp.lastcta) {
        w[L.aux] = (uint64_t)(uintptr_t)p;
        check_cuda(cudaMemsetAsync(p, 0, cbytes, stream), "arrival counters");
      }
    }
    CUfunction fn = kernel_for(sp, tape);
    launch(fn, nset * S, w, stream);
    if (S > 1 && !sp.lastcta) launch_finalize(sp, tape, KN, S, sms, w, stream);
    sp.k4r = 0;
    sp.rd = 0;
  };
  auto run_k4 = [&](int unroll, int tps, int lastcta) {
    if (unroll >= 100) {   // the row-lane form: unroll - 100 rows in flight
      run_k4r(unroll - 100, tps, lastcta);
      return;
    }
    sp.unroll = unroll;
    const int64_t target = (int64_t)sms * tps;
    int64_t S = 1;
    if (KG < target) S = std::min<int64_t>(cdiv(target, KG), std::max<int64_t>(1, RN / 8));
    int64_t C = cdiv(RN, S);
    S = cdiv(RN, C);
    const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
    std::vector<uint64_t> w;
    fill_common_words(s, sp, tape, L, w);
    w[L.nsplit] = (uint64_t)S; w[L.chunk] = (uint64_t)C; w[L.keptn] = (uint64_t)KN; w[L.redn] = (uint64_t)RN;
    // lastcta: when the kept groups fill whole 256-thread blocks, the last of
    // the S blocks over a set of kept groups merges their partials (one arrival
    // counter per set, zeroed here) instead of a finalize launch; a tuned choice
    sp.lastcta = (lastcta && S > 1 && KG % 256 == 0) ? 1 : 0;
    const size_t pbytes = S > 1 ? (size_t)(S * KN) * 8 * ((has_sum ? 1 : 0) + (has_max ? 2 : 0) + (has_min ? 2 : 0)) : 0;
    const size_t cbytes = sp.lastcta ? ((size_t)(KG / 256) * 4 + 255) / 256 * 256 : 0;
    StreamScratch part(pbytes + cbytes, stream);
    if (S > 1) {
      uint64_t* p = (uint64_t*)part.ptr;
      if (has_sum) { w[L.psum] = (uint64_t)(uintptr_t)p; p += S * KN; }
      if (has_max) { w[L.pmax] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
      if (has_min) { w[L.pmin] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
      if (sp.lastcta) {
        w[L.aux] = (uint64_t)(uintptr_t)p;
        check_cuda(cudaMemsetAsync(p, 0, cbytes, stream), "arrival counters");
      }
    }
    CUfunction fn = kernel_for(sp, tape);
    launch(fn, cdiv(KG * S, 256), w, stream);
    if (S > 1 && !sp.lastcta) {
      launch_finalize(sp, tape, KN, S, sms, w, stream);
    }
  };
  // bulk-staged row-lane form (NCA_K4_BULK=1): every operand contiguous along
  // the kept innermost dim with 16-byte aligned rows, one reduced dim
  // (outermost of two, or the middle of three), not float64 work (bound by
  // its pipe, not by loads). Rows per stage for about 16 KB, 4 stages; splits
  // so that every CTA is resident at once (a CTA per set and split)
  bool bulk_ok = rows_ok && k4b_on() && arith_dtype(tape.compute_dtype) != NCA_FLOAT64 &&
                 ((s.nd == 2 && rdim == 0) || (s.nd == 3 && rdim == 1));
  for (int k = 0; k < nops && bulk_ok; ++k) {
    const CArr& a = s.ops[k];
    const int es = dtinfo(a.dtype).size, vb = es * sp.vec;
    if (sp.op_modes[k] != M_CONTIG || a.st[s.nd - 1] != es || (vb != 4 && vb != 8 && vb != 16)) bulk_ok = false;
    else if ((uintptr_t)a.base % 16 || a.st[rdim] % 16 || (s.nd == 3 && a.st[0] % 16) || (s.shape[s.nd - 1] * es) % 16)
      bulk_ok = false;
  }
  if (bulk_ok && s.shape[s.nd - 1] % sp.vec) bulk_ok = false;
  if (bulk_ok) {
    const int R = 4, GPC = 64;
    const int64_t inner = s.shape[s.nd - 1];
    sp.unroll = 1;
    sp.k4r = R;
    sp.rd = rdim;
    sp.k4b = 1;
    // column blocks: up to 4 KB of each row per CTA while the sets still
    // give every SM a CTA
    sp.k4b_cb = 1;
    for (int cb : {4, 2}) {
      const int64_t sets = cdiv(inner / sp.vec, (int64_t)GPC * cb) * (s.nd == 3 ? s.shape[0] : 1);
      if (inner / sp.vec >= (int64_t)GPC * cb && (sets * std::max<int64_t>(1, RN / 64) >= sms)) { sp.k4b_cb = cb; break; }
    }
    if (const char* e = getenv("NCA_K4B_CB")) { const int v = atoi(e); if (v == 1 || v == 2 || v == 4) sp.k4b_cb = v; }
    int rowsum = 0;
    for (int k = 0; k < nops; ++k) rowsum += GPC * sp.k4b_cb * sp.vec * dtinfo(s.ops[k].dtype).size;
    sp.k4b_rb = std::max(R, std::min(64, 16384 / rowsum / R * R));
    sp.k4b_ns = 4;
    if (const char* e = getenv("NCA_K4B_RB")) { const int v = atoi(e); if (v >= R && v <= 256 && v % R == 0) sp.k4b_rb = v; }
    if (const char* e = getenv("NCA_K4B_NS")) { const int v = atoi(e); if (v >= 2 && v <= 8) sp.k4b_ns = v; }
    const int64_t smem = (int64_t)sp.k4b_ns * sp.k4b_rb * rowsum + 16 * sp.k4b_ns;
    if (smem <= 200 * 1024) {
      const int64_t nset = cdiv(inner / sp.vec, (int64_t)GPC * sp.k4b_cb) * (s.nd == 3 ? s.shape[0] : 1);
      // resident CTAs per SM of the form (the merging variant; the other has the same footprint)
      sp.lastcta = 1;
      CUfunction fn = kernel_for(sp, tape);
      check_cu(drv().cuFuncSetAttribute(fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)smem), "smem attribute");
      int per_sm = 0;
      check_cu(drv().cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 288, (size_t)smem), "occupancy");
      int64_t S = std::max<int64_t>(1, std::min<int64_t>((int64_t)sms * std::max(per_sm, 1) / nset, RN / sp.k4b_rb));
      const int64_t C = cdiv(RN, S);
      S = cdiv(RN, C);
      if (S == 1) { sp.lastcta = 0; fn = kernel_for(sp, tape); }
      const WordLayout L = word_layout(sp.nops, sp.nd, sp.nscal, sp.nred, sp.ptrmask != 0);
      std::vector<uint64_t> w;
      fill_common_words(s, sp, tape, L, w);
      w[L.nsplit] = (uint64_t)S; w[L.chunk] = (uint64_t)C; w[L.keptn] = (uint64_t)KN; w[L.redn] = (uint64_t)RN;
      const size_t pbytes = S > 1 ? (size_t)(S * KN) * 8 * ((has_sum ? 1 : 0) + (has_max ? 2 : 0) + (has_min ? 2 : 0)) : 0;
      const size_t cbytes = sp.lastcta ? ((size_t)nset * 4 + 255) / 256 * 256 : 0;
      StreamScratch part(pbytes + cbytes, stream);
      if (S > 1) {
        uint64_t* p = (uint64_t*)part.ptr;
        if (has_sum) { w[L.psum] = (uint64_t)(uintptr_t)p; p += S * KN; }
        if (has_max) { w[L.pmax] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
        if (has_min) { w[L.pmin] = (uint64_t)(uintptr_t)p; p += 2 * S * KN; }
        w[L.aux] = (uint64_t)(uintptr_t)p;
        check_cuda(cudaMemsetAsync(p, 0, cbytes, stream), "arrival counters");
      }
      launch(fn, nset * S, w, stream, (unsigned)smem, 288);
      return true;
    }
    sp.k4r = 0;
    sp.rd = 0;
    sp.k4b = 0;
  }
  // schedule: the autotuner's cached choice for this (dtypes, ops, stored
  // value, kept and reduced size class, dims), else 4 rows in flight and 1024
  // threads per SM; searched (rows 4 / 8, 512 / 1024 / 2048 threads per SM)
  // when the kernel writes nothing it reads
  std::string key = "red|k4|" + std::to_string(tape.compute_dtype) + "|" + std::to_string(red_ops) + "|o" +
                    std::to_string(out ? out->dtype : -1) + "|";
  for (int k = 0; k < nops; ++k) key += std::to_string(ops[k].dtype) + ".";
  key += "|r" + size_class(RN) + "|k" + size_class(KN) + "|d" + std::to_string(s.nd) + "|v" + std::to_string(sp.vec);
  std::vector<int> choice;
  if (tune_get(key, choice) && choice.size() == 3 &&
      (choice[0] == 4 || choice[0] == 8 || (rows_ok && (choice[0] == 102 || choice[0] == 104 || choice[0] == 108))) &&
      (choice[1] == 512 || choice[1] == 1024 || choice[1] == 2048 || (choice[0] >= 100 && choice[1] == 0)) &&
      (choice[2] == 0 || choice[2] == 1)) {
    run_k4(choice[0], choice[1], choice[2]);
    return true;
  }
  std::vector<nca_view> routs;
  for (int k = 0; k < nred; ++k) routs.push_back(rv[(size_t)k].out);
  if (out) routs.push_back(*out);
  if (KN * RN >= (1 << 16) && tune_should_search(stream) && rerun_safe(ops, nops, routs.data(), (int)routs.size())) {
    std::vector<std::vector<int>> cands = {{4, 1024, 0}, {8, 1024, 0}, {4, 2048, 0}, {8, 2048, 0}, {8, 512, 0},
                                           {4, 1024, 1}, {8, 512, 1}};
    if (rows_ok)
      for (auto c : std::vector<std::vector<int>>{{104, 0, 0}, {104, 2048, 1}, {104, 2048, 0}, {102, 2048, 1}, {104, 1024, 1},
                                                  {108, 1024, 1}, {108, 512, 1}, {104, 512, 1}})
        cands.push_back(c);
    const int best = tune_pick(stream, (int)cands.size(), [&](int i) {
      run_k4(cands[(size_t)i][0], cands[(size_t)i][1], cands[(size_t)i][2]);
    });
    tune_put(key, cands[(size_t)best]);
    run_k4(cands[(size_t)best][0], cands[(size_t)best][1], cands[(size_t)best][2]);
    return true;
  }
  // row-lane form: 8 rows in flight per row lane (the tuner's choice on the
  // outer-axis benchmarks and C1: max over axis 1 0.77 -> 0.81 of measured);
  // splits for 1024 threads per SM, 512 for short reduced axes (the tuner's
  // choices: (4096, 16384) over axis 0 and C1's 128 rows)
  if (rows_ok && !k4r_off()) run_k4(108, k4r_persistent() ? 0 : (RN <= 256 ? 512 : 1024), k4r_lastcta());
  else run_k4(4, 1024, 0);
  return true;
}


// tapes[0] stored to outs[0] and reduced, tapes[1..] stored to outs[1..]:
// one staged pass when the outputs overlap neither the operands nor each
// other and the views fit it, else the calls one after another
void expr_multi(const std::vector<Tape>& tapes, const nca_view* ops, int nops, const nca_view* outs,
                const nca_reduction* reds, int nred, cudaStream_t stream) {
  const int nx = (int)tapes.size() - 1;
  if (nx < 0) fail(NCA_ERR_INVALID, "at least one tape");
  if (nx > NCA_MAX_EXTRA_OUTS) fail(NCA_ERR_LIMIT, "%d extra outputs (at most %d)", nx, NCA_MAX_EXTRA_OUTS);
  bool fuse = nx > 0 && nred > 0;
  if (fuse) {
    std::vector<nca_view> all(outs, outs + nx + 1);
    for (int k = 0; k < nred; ++k) all.push_back(reds[k].out);
    fuse = rerun_safe(ops, nops, all.data(), (int)all.size());
    for (size_t i = 0; fuse && i < all.size(); ++i)
      for (size_t j = i + 1; fuse && j < all.size(); ++j) {
        uintptr_t l1, h1, l2, h2;
        if (!view_range(all[i], l1, h1) || !view_range(all[j], l2, h2) || (l1 < h2 && l2 < h1)) fuse = false;
      }
  }
  if (fuse && expr_reduce(tapes[0], ops, nops, &outs[0], reds, nred, stream, tapes.data() + 1, outs + 1, nx)) return;
  if (nred > 0) expr_reduce(tapes[0], ops, nops, &outs[0], reds, nred, stream);
  else expr_eval(tapes[0], ops, nops, outs[0], stream);
  for (int x = 1; x <= nx; ++x) expr_eval(tapes[(size_t)x], ops, nops, outs[x], stream);
}

}  // namespace nca

namespace nca {

// Generates and NVRTC-compiles one kernel of every class for `arch` without a
// device (the compile-only check of the template). Returns the number compiled.
int jit_selftest(const char* arch) {
  const std::string a = arch ? arch : "sm_103a";
  int n = 0;
  // tape: a*b + sqrt(abs(c)) - 0.5*a
  Tape t;
  auto I = [](int op, int idx) { return (uint32_t)(op << 24) | (uint32_t)idx; };
  t.instrs = {I(NCA_OP_LOAD_NCARR, 0), I(NCA_OP_LOAD_NCARR, 1), I(NCA_OP_MUL, 0),
              I(NCA_OP_LOAD_NCARR, 2), I(NCA_OP_ABS, 0), I(NCA_OP_SQRT, 0), I(NCA_OP_ADD, 0),
              I(NCA_OP_LOAD_CONST, 0), I(NCA_OP_LOAD_NCARR, 0), I(NCA_OP_MUL, 0), I(NCA_OP_SUB, 0)};
  t.scalar_dtypes = {NCA_FLOAT64};
  double half = 0.5; uint64_t hb; memcpy(&hb, &half, 8);
  t.scalar_slots = {hb};
  t.n_arrays = 3;
  const int dts[][4] = {  // w, out/r, op dtype, vec
      {NCA_FLOAT64, NCA_FLOAT64, NCA_FLOAT64, 2}, {NCA_FLOAT32, NCA_FLOAT32, NCA_INT32, 4},
      {NCA_INT32, NCA_INT32, NCA_INT32, 4},       {NCA_FLOAT32, NCA_BFLOAT16, NCA_BFLOAT16, 4},
      {NCA_UINT8, NCA_BOOL, NCA_UINT8, 16},       {NCA_INT64, NCA_INT64, NCA_INT16, 2}};
  for (auto& d : dts) {
    t.compute_dtype = d[0];
    t.result_dtype = d[1];
    for (int kind = 1; kind <= 5; ++kind) {
      Spec sp;
      sp.kind = kind; sp.nops = 3; sp.nd = kind == 1 ? 1 : 3; sp.vec = kind == 4 ? std::min(d[3], 4) : d[3];
      sp.idx32 = 1; sp.w = d[0]; sp.r = d[1]; sp.out_dtype = d[1]; sp.nscal = 1;
      sp.op_dtypes = {d[2], d[2], d[2]};
      sp.op_modes = {M_CONTIG, M_CONST, M_STRIDED};
      if (kind == 1) sp.op_modes = {M_CONTIG, M_CONST, M_CONTIG};
      sp.has_out = kind <= 2 || kind == 4;
      if (kind >= 3) {
        sp.nred = 4; sp.red_ops = 0 | (2u << 4) | (4u << 8) | (1u << 12);
        sp.has_sum = sp.has_max = true;
        if (kind == 3) { sp.nkept = 1; sp.kept_mask = 1u; sp.red_ops = 3u | (5u << 4) | (0u << 8) | (1u << 12); sp.has_min = true; sp.has_max = false; }
        else sp.kept_mask = 1u | 4u;
      }
      const std::string src = gen_source(sp, t);
      nvrtc_compile(src, a);
      ++n;
      if (kind == 3 || kind == 5) {   // one thread per kept position (offset table; thread-per-position finalize)
        Spec s1 = sp;
        s1.team = 1;
        nvrtc_compile(gen_source(s1, t), a);
        ++n;
        if (kind == 3) {               // and its form that gathers 4 units of 2 vectors at once
          s1.k3rv = 2; s1.k3tu = 4;
          nvrtc_compile(gen_source(s1, t), a);
          ++n;
        }
      }
      if (kind == 3 || kind == 5) {   // two-thread teams; the warp-per-position finalize
        Spec s2 = sp;
        s2.team = kind == 3 ? 2 : 32;
        nvrtc_compile(gen_source(s2, t), a);
        ++n;
      }
      if (kind == 3 || kind == 4) {   // last CTA over a set of kept positions merges the partials
        Spec s3 = sp;
        s3.lastcta = 1;
        nvrtc_compile(gen_source(s3, t), a);
        ++n;
      }
      if (kind == 4) {                 // row-lane form over the one reduced dim 1
        Spec s4 = sp;
        s4.k4r = 4; s4.rd = 1; s4.lastcta = 1; s4.unroll = 4;
        nvrtc_compile(gen_source(s4, t), a);
        ++n;
        s4.lastcta = 0; s4.k4p = 1;    // on a persistent grid
        nvrtc_compile(gen_source(s4, t), a);
        ++n;
        Spec s5 = sp;                  // rows bulk-copied into a shared-memory ring
        s5.k4r = 4; s5.rd = 1; s5.k4b = 1; s5.lastcta = 1; s5.k4b_cb = 2;
        nvrtc_compile(gen_source(s5, t), a);
        ++n;
      }
    }
    // kinds 2, 3, 4 with operand 0 on a pointer axis (first two dtype rows)
    if (&d - &dts[0] < 2) {
      for (int kind = 2; kind <= 4; ++kind) {
        Spec sp;
        sp.kind = kind; sp.nops = 3; sp.nd = 3; sp.vec = 1; sp.idx32 = 1; sp.w = d[0]; sp.r = d[1]; sp.out_dtype = d[1];
        sp.nscal = 1; sp.op_dtypes = {d[2], d[2], d[2]}; sp.op_modes = {M_STRIDED, M_CONST, M_STRIDED};
        sp.ptrmask = 1u;
        sp.has_out = kind != 3;
        if (kind == 3) sp.team = 1;   // one thread per kept position
        if (kind >= 3) {
          sp.nred = 2; sp.red_ops = 0u | (4u << 4); sp.has_sum = sp.has_max = true;
          if (kind == 3) { sp.nkept = 1; sp.kept_mask = 1u; } else sp.kept_mask = 1u | 4u;
        }
        nvrtc_compile(gen_source(sp, t), a);
        ++n;
      }
    }
    // kind 6: operand 0 staged through shared memory, dims (q, b, r, p)
    Spec sp;
    sp.kind = 6; sp.nops = 3; sp.nd = 4; sp.vec = 1; sp.w = d[0]; sp.r = d[1]; sp.out_dtype = d[1]; sp.nscal = 1;
    sp.op_dtypes = {d[2], d[2], d[2]};
    sp.op_modes = {M_STAGED, M_CONTIG, M_CONST};
    sp.vec = std::min(d[3], 4);
    sp.has_out = true; sp.nred = 2; sp.red_ops = 2u | (4u << 4); sp.has_max = true;
    sp.kept_mask = 1u | 2u | 8u; sp.qd = 0; sp.qx = 8; sp.qxp = 8; sp.tmask = 1u; sp.tp = 64; sp.rb = 8; sp.minb = 3;
    sp.tile_bytes = 64 * (8 * 8 + 1) * dtinfo(d[0]).size;
    nvrtc_compile(gen_source(sp, t), a);
    ++n;
    // kind 6 without reductions (a transposed elementwise expression)
    sp.nred = 0; sp.red_ops = 0; sp.has_max = false; sp.kept_mask = 1u | 8u;
    nvrtc_compile(gen_source(sp, t), a);
    ++n;
    // kind 7 (4-byte operands and result): operand 0 staged, 1 in p rows, 2 uniform
    if (dtinfo(d[2]).size == 4 && dtinfo(d[1]).size == 4) {
      Spec a7;
      a7.kind = 7; a7.nops = 3; a7.nd = 4; a7.vec = 1; a7.w = d[0]; a7.r = d[1]; a7.out_dtype = d[1]; a7.nscal = 1;
      a7.op_dtypes = {d[2], d[2], d[2]};
      a7.op_modes = {M_STAGED, M_CONTIG, M_CONST};
      a7.has_out = true; a7.nred = 2; a7.red_ops = 2u | (4u << 4); a7.has_max = true;
      a7.kept_mask = 1u | 2u | 8u; a7.qd = 0; a7.qx = 8; a7.qxp = 8; a7.tp = 32; a7.ltp8 = 2; a7.rb = 8;
      a7.tmask = 1u; a7.pmask = 2u; a7.umask = 4u; a7.npc = 1; a7.ns = 3; a7.ld = 2; a7.nmaps = 3; a7.minb = 3;
      nvrtc_compile(gen_source(a7, t), a);
      ++n;
      a7.nred = 0; a7.red_ops = 0; a7.has_max = false; a7.kept_mask = 1u | 8u;
      nvrtc_compile(gen_source(a7, t), a);
      // five dims: two other dims besides p, q and the fastest loop dim
      a7.nd = 5; a7.kept_mask = 1u | 2u | 16u; a7.ld = 3; a7.nred = 2; a7.red_ops = 2u | (4u << 4); a7.has_max = true;
      nvrtc_compile(gen_source(a7, t), a);
      ++n;
      ++n;
      // one output tile (three stages fit beside it)
      a7.nob = 1; a7.ns = 3;
      nvrtc_compile(gen_source(a7, t), a);
      ++n;
      // an extra output: (x1 * 3 + 7) % 11 in int32 over the p-row operand
      Tape xt;
      xt.instrs = {I(NCA_OP_LOAD_NCARR, 1), I(NCA_OP_LOAD_CONST, 0), I(NCA_OP_MUL, 0), I(NCA_OP_LOAD_CONST, 1),
                   I(NCA_OP_ADD, 0), I(NCA_OP_LOAD_CONST, 2), I(NCA_OP_MOD, 0)};
      xt.scalar_dtypes = {NCA_INT32, NCA_INT32, NCA_INT32};
      xt.scalar_slots = {3, 7, 11};
      xt.compute_dtype = NCA_INT32; xt.result_dtype = NCA_INT32; xt.n_arrays = 2;
      a7.nob = 2; a7.ns = 2; a7.nd = 4; a7.kept_mask = 1u | 2u | 8u; a7.ld = 2;
      a7.xtapes = {xt}; a7.xout_dtypes = {NCA_INT32}; a7.nscal = 4; a7.nmaps = 4;
      nvrtc_compile(gen_source(a7, t), a);
      ++n;
      a7.xvec = 1;   // the same on whole 16-byte tile chunks (operand 1 is a p-row operand)
      nvrtc_compile(gen_source(a7, t), a);
      ++n;
    }
  }
  // kind 2 with window-pair operands (phases 0 and 1, one sharing the other's
  // loads): the pixel-binning shape, 4-byte and 2-byte elements
  for (int dt : {NCA_FLOAT32, NCA_BFLOAT16}) {
    Spec sp;
    sp.kind = 2; sp.nops = 3; sp.nd = 3; sp.vec = 16 / dtinfo(dt).size; sp.idx32 = 1; sp.nscal = 1;
    sp.w = NCA_FLOAT32; sp.r = NCA_FLOAT32; sp.out_dtype = dt; sp.has_out = true;
    sp.op_dtypes = {dt, dt, dt};
    sp.op_modes = {M_PAIR0, M_PAIR1, M_PAIR1};
    sp.op_alias = {-1, 0, -1};
    sp.op_salias = {-1, 0, 0};
    nvrtc_compile(gen_source(sp, t), a);
    ++n;
    // the same with operands 0 and 1 on a pointer axis (windows guarded per panel)
    sp.ptrmask = 3u;
    sp.op_salias = {-1, -1, -1};
    nvrtc_compile(gen_source(sp, t), a);
    ++n;
  }
  n += batch_expr_selftest(a.c_str());
  n += stencil_tile_selftest(a.c_str());
  return n;
}

}  // namespace nca
