/*
 * oracle.c -- CPU restatement of the reference algorithms on the hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle the GPU kernels are
 * compared against; it is never part of the product path. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 *
 * Restated from ncarray v0.7.8:
 *  - expression VM: DynamicExprMVNode::eval (src/lib/ncarray/expression/
 *    dynamicmvnode.hh:146-251) with apply_op (expression/interface.hh:103-181):
 *    every tape value in one compute type W, loads cast to W
 *    (op_traits::cast, op_traits.hh:88-110), result cast to the output dtype.
 *    Division by zero: NaN if the dividend is finite, else the dividend
 *    (interface.hh:134-140). Cases the reference leaves undefined are defined
 *    as in the device prelude: integer x/0 -> 0, x%0 -> 0, x%-1 -> 0,
 *    INT_MIN/-1 -> INT_MIN, signed add/sub/mul/neg wrap.
 *  - reductions: host scans of src/lib/ncarray/host/reductions.hh:35-251
 *    (max/argmax: strict '>' against lowest(), first index kept; min/argmin
 *    mirrored), with sums accumulated in float64 (Neumaier compensation) for
 *    floating inputs and as 64-bit wrapping integers for integer inputs; mean
 *    = sum / count. Axis reductions index the reduced axes in C order.
 *  - 3-D stencil, 2-D histogram and batched reductions: float64 restatements
 *    of the operations the reference expresses through Stencil<3>
 *    (expression/stencil.hh:58-255) and scatter_add (device/kernels.cuh:660-680).
 *
 * Compiled with -ffp-contract=off so float arithmetic rounds after every
 * operation, as the device kernels do (NVRTC --fmad=false).
 */
#include <math.h>
#include <stdbool.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_MAXD 10

enum {
  D_BOOL = 0, D_CHAR = 1, D_U8 = 2, D_U16 = 3, D_U32 = 4, D_U64 = 5, D_I8 = 6, D_I16 = 7,
  D_I32 = 8, D_I64 = 9, D_F32 = 10, D_F64 = 11, D_BF16 = 22, D_F16 = 23
};

enum {
  OP_NOOP = 0, OP_IDX = 1, OP_LOAD_NCARR = 2, OP_LOAD_SOARR = 3, OP_LOAD_CONST = 4, OP_NEG = 5,
  OP_INC = 6, OP_DEC = 7, OP_LNOT = 12, OP_BNOT = 13, OP_ADD = 14, OP_SUB = 15, OP_MUL = 16,
  OP_DIV = 17, OP_MOD = 18, OP_EQ = 20, OP_NE = 21, OP_LT = 22, OP_LE = 23, OP_GT = 24,
  OP_GE = 25, OP_LAND = 26, OP_LOR = 27, OP_BAND = 28, OP_BOR = 29, OP_XOR = 30, OP_ABS = 34,
  OP_SQRT = 35
};

/* same memory layout as nca_view of include/ncgb300.h */
typedef struct orc_view {
  void* data;
  int32_t dtype;
  int32_t ndim;
  int64_t shape[ORC_MAXD];
  int64_t strides[ORC_MAXD];
  int64_t offsets[ORC_MAXD];
  int32_t pointer_axis;
  int32_t flags;
} orc_view;

static int dsize(int dt) {
  switch (dt) {
    case D_BOOL: case D_CHAR: case D_U8: case D_I8: return 1;
    case D_U16: case D_I16: case D_BF16: case D_F16: return 2;
    case D_U32: case D_I32: case D_F32: return 4;
    case D_U64: case D_I64: case D_F64: return 8;
  }
  return 0;
}

static char* vbase(const orc_view* v) {
  int64_t off = 0;
  for (int d = 0; d < v->ndim; ++d) off += v->offsets[d];
  return (char*)v->data + off;
}

/* ---- 16-bit floats ---------------------------------------------------------- */
static float bf16_to_f32(uint16_t h) { uint32_t u = (uint32_t)h << 16; float f; memcpy(&f, &u, 4); return f; }
static uint16_t f32_to_bf16(float f) {
  uint32_t u; memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40u);
  return (uint16_t)((u + 0x7fffu + ((u >> 16) & 1u)) >> 16);
}
static float f16_to_f32(uint16_t h) { _Float16 x; memcpy(&x, &h, 2); return (float)x; }
static uint16_t f32_to_f16(float f) { _Float16 x = (_Float16)f; uint16_t h; memcpy(&h, &x, 2); return h; }

static const uint32_t kNanF = 0x7fc00000u;
static const uint64_t kNanD = 0x7ff8000000000000ull;
static float nanf_() { float f; memcpy(&f, &kNanF, 4); return f; }
static double nand_() { double d; memcpy(&d, &kNanD, 8); return d; }

/* ---- typed VM ------------------------------------------------------------------
 * VM_TYPE(T, SUF, U, KIND): KIND 0 bool, 1 signed, 2 unsigned, 3 float, 4 double.
 * U is the same-width unsigned type used for wrapping arithmetic. */
#define LOAD_AS(T)                                                                         \
  static T ld_##T(int dt, const void* p) {                                                 \
    switch (dt) {                                                                          \
      case D_BOOL: return (T)(*(const uint8_t*)p != 0);                                    \
      case D_CHAR: case D_I8: return (T)(*(const int8_t*)p);                               \
      case D_U8: return (T)(*(const uint8_t*)p);                                           \
      case D_U16: return (T)(*(const uint16_t*)p);                                         \
      case D_I16: return (T)(*(const int16_t*)p);                                          \
      case D_U32: return (T)(*(const uint32_t*)p);                                         \
      case D_I32: return (T)(*(const int32_t*)p);                                          \
      case D_U64: return (T)(*(const uint64_t*)p);                                         \
      case D_I64: return (T)(*(const int64_t*)p);                                          \
      case D_F32: return (T)(*(const float*)p);                                            \
      case D_F64: return (T)(*(const double*)p);                                           \
      case D_BF16: return (T)bf16_to_f32(*(const uint16_t*)p);                             \
      case D_F16: return (T)f16_to_f32(*(const uint16_t*)p);                               \
    }                                                                                      \
    return (T)0;                                                                           \
  }                                                                                        \
  static void st_##T(int dt, void* p, T v) {                                               \
    switch (dt) {                                                                          \
      case D_BOOL: *(uint8_t*)p = (uint8_t)(v != 0); break;                                \
      case D_CHAR: case D_I8: *(int8_t*)p = (int8_t)v; break;                              \
      case D_U8: *(uint8_t*)p = (uint8_t)v; break;                                         \
      case D_U16: *(uint16_t*)p = (uint16_t)v; break;                                      \
      case D_I16: *(int16_t*)p = (int16_t)v; break;                                        \
      case D_U32: *(uint32_t*)p = (uint32_t)v; break;                                      \
      case D_I32: *(int32_t*)p = (int32_t)v; break;                                        \
      case D_U64: *(uint64_t*)p = (uint64_t)v; break;                                      \
      case D_I64: *(int64_t*)p = (int64_t)v; break;                                        \
      case D_F32: *(float*)p = (float)v; break;                                            \
      case D_F64: *(double*)p = (double)v; break;                                          \
      case D_BF16: *(uint16_t*)p = f32_to_bf16((float)v); break;                           \
      case D_F16: *(uint16_t*)p = f32_to_f16((float)v); break;                             \
    }                                                                                      \
  }

typedef bool b8;
typedef int8_t i8;
typedef uint8_t u8;
typedef int16_t i16;
typedef uint16_t u16;
typedef int32_t i32;
typedef uint32_t u32;
typedef int64_t i64;
typedef uint64_t u64;
typedef float f32;
typedef double f64;

LOAD_AS(b8) LOAD_AS(i8) LOAD_AS(u8) LOAD_AS(i16) LOAD_AS(u16) LOAD_AS(i32) LOAD_AS(u32)
LOAD_AS(i64) LOAD_AS(u64) LOAD_AS(f32) LOAD_AS(f64)

#define VM_TYPE(T, U, KIND)                                                                  \
  static T neg_##T(T a) { return (KIND == 1) ? (T)(U)((U)0 - (U)a) : (T)(-a); }             \
  static T add_##T(T a, T b) { return (KIND == 1 || KIND == 2) ? (T)(U)((U)a + (U)b) : (T)(a + b); } \
  static T sub_##T(T a, T b) { return (KIND == 1 || KIND == 2) ? (T)(U)((U)a - (U)b) : (T)(a - b); } \
  static T mul_##T(T a, T b) {                                                              \
    if (KIND == 0) return (T)(a && b);                                                      \
    return (KIND == 1 || KIND == 2) ? (T)(U)((U)a * (U)b) : (T)(a * b);                     \
  }                                                                                         \
  static int fin_##T(T a) { return KIND == 3 ? isfinite((float)a) : KIND == 4 ? isfinite((double)a) : 1; } \
  static T nan_##T(void) { return KIND == 0 ? (T)1 : KIND == 3 ? (T)nanf_() : KIND == 4 ? (T)nand_() : (T)0; } \
  static T div_##T(T a, T b) {                                                              \
    if (b == (T)0) return fin_##T(a) ? nan_##T() : a;                                       \
    if (KIND == 1 && b == (T)(-1)) return neg_##T(a);                                       \
    return (T)(a / b);                                                                      \
  }                                                                                         \
  static T mod_##T(T a, T b);                                                               \
  static T bnot_##T(T a);                                                                   \
  static T band_##T(T a, T b);                                                              \
  static T bor_##T(T a, T b);                                                               \
  static T xor_##T(T a, T b);                                                               \
  static T abs_##T(T a) {                                                                   \
    if (KIND == 3) return (T)fabsf((float)a);                                               \
    if (KIND == 4) return (T)fabs((double)a);                                               \
    if (KIND == 1 && a < (T)0) return neg_##T(a);                                           \
    return a;                                                                               \
  }                                                                                         \
  static T sqrt_##T(T a) {                                                                  \
    if (KIND == 3) return (T)sqrtf((float)a);                                               \
    if (KIND == 4) return (T)sqrt((double)a);                                               \
    if (KIND == 0) return a;                                                                \
    return a < (T)0 ? (T)0 : (T)sqrt((double)a);                                            \
  }                                                                                         \
  static int vm_##T(const uint32_t* ins, int n, char* const* ptrs, const int* dts,          \
                    const T* sc, int64_t lin, T* out) {                                     \
    T st[80];                                                                               \
    int top = -1;                                                                           \
    for (int i = 0; i < n; ++i) {                                                           \
      const int op = (int)(ins[i] >> 24), ix = (int)(ins[i] & 0xffffff);                    \
      T a, b;                                                                               \
      switch (op) {                                                                         \
        case OP_NOOP: break;                                                                \
        case OP_IDX: st[++top] = (T)lin; break;                                             \
        case OP_LOAD_NCARR: case OP_LOAD_SOARR: st[++top] = ld_##T(dts[ix], ptrs[ix]); break; \
        case OP_LOAD_CONST: st[++top] = sc[ix]; break;                                      \
        case OP_NEG: st[top] = neg_##T(st[top]); break;                                     \
        case OP_INC: st[top] = add_##T(st[top], (T)1); break;                               \
        case OP_DEC: st[top] = sub_##T(st[top], (T)1); break;                               \
        case OP_LNOT: st[top] = (T)(!st[top]); break;                                       \
        case OP_BNOT: st[top] = bnot_##T(st[top]); break;                                   \
        case OP_ABS: st[top] = abs_##T(st[top]); break;                                     \
        case OP_SQRT: st[top] = sqrt_##T(st[top]); break;                                   \
        default:                                                                            \
          b = st[top--]; a = st[top--];                                                     \
          switch (op) {                                                                     \
            case OP_ADD: st[++top] = add_##T(a, b); break;                                  \
            case OP_SUB: st[++top] = sub_##T(a, b); break;                                  \
            case OP_MUL: st[++top] = mul_##T(a, b); break;                                  \
            case OP_DIV: st[++top] = div_##T(a, b); break;                                  \
            case OP_MOD: st[++top] = mod_##T(a, b); break;                                  \
            case OP_EQ: st[++top] = (T)(a == b); break;                                     \
            case OP_NE: st[++top] = (T)(a != b); break;                                     \
            case OP_LT: st[++top] = (T)(a < b); break;                                      \
            case OP_LE: st[++top] = (T)(a <= b); break;                                     \
            case OP_GT: st[++top] = (T)(a > b); break;                                      \
            case OP_GE: st[++top] = (T)(a >= b); break;                                     \
            case OP_LAND: st[++top] = (T)(a && b); break;                                   \
            case OP_LOR: st[++top] = (T)(a || b); break;                                    \
            case OP_BAND: st[++top] = band_##T(a, b); break;                                \
            case OP_BOR: st[++top] = bor_##T(a, b); break;                                  \
            case OP_XOR: st[++top] = xor_##T(a, b); break;                                  \
            default: return -1;                                                             \
          }                                                                                 \
      }                                                                                     \
    }                                                                                       \
    *out = st[0];                                                                           \
    return 0;                                                                               \
  }

/* bitwise ops: the reference VM skips them (dynamicmvnode.hh:238); defined
 * here as two's complement operations in the compute type, bool NOT as !a
 * (the device prelude's nca_bnot/band/bor/xor). Floating compute types are
 * rejected before evaluation. */
#define BIT_INT(T, U)                                                                         \
  static T bnot_##T(T a) { return (T)(U)(~(U)a); }                                          \
  static T band_##T(T a, T b) { return (T)(U)((U)a & (U)b); }                               \
  static T bor_##T(T a, T b) { return (T)(U)((U)a | (U)b); }                                \
  static T xor_##T(T a, T b) { return (T)(U)((U)a ^ (U)b); }
BIT_INT(i8, u8) BIT_INT(u8, u8) BIT_INT(i16, u16) BIT_INT(u16, u16) BIT_INT(i32, u32) BIT_INT(u32, u32)
BIT_INT(i64, u64) BIT_INT(u64, u64)
static b8 bnot_b8(b8 a) { return !a; }
static b8 band_b8(b8 a, b8 b) { return a && b; }
static b8 bor_b8(b8 a, b8 b) { return a || b; }
static b8 xor_b8(b8 a, b8 b) { return a != b; }
#define BIT_FLT(T)                                                                            \
  static T bnot_##T(T a) { (void)a; return (T)0; }                                          \
  static T band_##T(T a, T b) { (void)a; (void)b; return (T)0; }                            \
  static T bor_##T(T a, T b) { (void)a; (void)b; return (T)0; }                             \
  static T xor_##T(T a, T b) { (void)a; (void)b; return (T)0; }
BIT_FLT(f32) BIT_FLT(f64)

static b8 mod_b8(b8 a, b8 b) { (void)a; (void)b; return false; }
#define INT_MOD(T, SIGNED)                                                                  \
  static T mod_##T(T a, T b) {                                                              \
    if (b == 0) return 0;                                                                   \
    if (SIGNED && b == (T)(-1)) return 0;                                                   \
    return (T)(a % b);                                                                      \
  }
INT_MOD(i8, 1) INT_MOD(u8, 0) INT_MOD(i16, 1) INT_MOD(u16, 0) INT_MOD(i32, 1) INT_MOD(u32, 0)
INT_MOD(i64, 1) INT_MOD(u64, 0)
static f32 mod_f32(f32 a, f32 b) { return fmodf(a, b); }
static f64 mod_f64(f64 a, f64 b) { return fmod(a, b); }

VM_TYPE(b8, u8, 0)
VM_TYPE(i8, u8, 1) VM_TYPE(i16, u16, 1) VM_TYPE(i32, u32, 1) VM_TYPE(i64, u64, 1)
VM_TYPE(u8, u8, 2) VM_TYPE(u16, u16, 2) VM_TYPE(u32, u32, 2) VM_TYPE(u64, u64, 2)
VM_TYPE(f32, f32, 3) VM_TYPE(f64, f64, 4)

/* bitwise ops are defined for integer and bool compute types only */
static int bitwise_ok(const uint32_t* ins, int n, int compute_dtype) {
  if (compute_dtype != D_F32 && compute_dtype != D_F64) return 1;
  for (int i = 0; i < n; ++i) {
    const int op = (int)(ins[i] >> 24);
    if (op == OP_BNOT || op == OP_BAND || op == OP_BOR || op == OP_XOR) return 0;
  }
  return 1;
}

/* element pointers of every operand at C-order coords of out shape */
static void op_ptrs(const orc_view* ops, int nops, int n, const int64_t* c, char** ptrs) {
  for (int k = 0; k < nops; ++k) {
    const orc_view* v = &ops[k];
    char* p = vbase(v);
    for (int d = 0; d < v->ndim; ++d) {
      const int ld = d + (n - v->ndim);
      if (v->shape[d] != 1) p += c[ld] * v->strides[d];
    }
    ptrs[k] = p;
  }
}

#define RUN_EVAL(T)                                                                          \
  {                                                                                          \
    T sc[64];                                                                                \
    for (int i = 0; i < n_scalars; ++i) sc[i] = ld_##T(scalar_dtypes[i], &slots[i]);         \
    int bad = 0;                                                                             \
    _Pragma("omp parallel for schedule(static) reduction(|:bad)")                            \
    for (int64_t e = 0; e < total; ++e) {                                                    \
      int64_t c[ORC_MAXD];                                                                   \
      char* ptrs[32];                                                                        \
      int64_t rem = e;                                                                       \
      for (int d = n - 1; d >= 0; --d) { c[d] = rem % out->shape[d]; rem /= out->shape[d]; }  \
      op_ptrs(ops, nops, n, c, ptrs);                                                        \
      char* po = ob;                                                                         \
      for (int d = 0; d < n; ++d) po += c[d] * out->strides[d];                              \
      T v;                                                                                   \
      if (vm_##T(instrs, n_instrs, ptrs, dts, sc, e, &v)) { bad = 1; continue; }             \
      st_##T(out->dtype, po, v);                                                             \
    }                                                                                        \
    if (bad) return 2;                                                                       \
  }                                                                                          \
  break;

/* out = tape(ops) evaluated in compute dtype W; returns 0 on success. Elements
 * are independent, so the loop runs on all OpenMP threads. */
int orc_expr_eval(const uint32_t* instrs, int n_instrs, const int* scalar_dtypes,
                  const uint64_t* slots, int n_scalars, int compute_dtype, const orc_view* ops,
                  int nops, const orc_view* out) {
  if (n_scalars > 64 || nops > 32 || n_instrs > 128) return 3;
  const int n = out->ndim;
  int64_t total = 1;
  for (int d = 0; d < n; ++d) total *= out->shape[d];
  int dts[32];
  for (int k = 0; k < nops; ++k) dts[k] = ops[k].dtype;
  char* ob = vbase(out);
  if (!bitwise_ok(instrs, n_instrs, compute_dtype)) return 4;
  for (int i = 0; i < n_instrs; ++i) {
    const int op = (int)(instrs[i] >> 24), ix = (int)(instrs[i] & 0xffffff);
    if ((op == OP_LOAD_NCARR || op == OP_LOAD_SOARR) && ix >= nops) return 5;
    if (op == OP_LOAD_CONST && ix >= n_scalars) return 5;
  }
  switch (compute_dtype) {
    case D_BOOL: RUN_EVAL(b8)
    case D_CHAR: case D_I8: RUN_EVAL(i8)
    case D_U8: RUN_EVAL(u8)
    case D_I16: RUN_EVAL(i16)
    case D_U16: RUN_EVAL(u16)
    case D_I32: RUN_EVAL(i32)
    case D_U32: RUN_EVAL(u32)
    case D_I64: RUN_EVAL(i64)
    case D_U64: RUN_EVAL(u64)
    case D_F32: RUN_EVAL(f32)
    case D_F64: RUN_EVAL(f64)
    default: return 1;
  }
  return 0;
}

/* ---- reductions -----------------------------------------------------------------
 * op: 0 sum, 1 mean, 2 max, 3 min, 4 argmax, 5 argmin. `out` has the kept axes
 * (ndim 0 for a full reduction). Sum output dtype: sum_type of the input
 * (op_traits.hh:72-76,380-410; 16-bit floats -> float32); mean -> float64;
 * max/min -> input dtype (16-bit floats -> float32); arg* -> int64. */
/* Neumaier-compensated float64 sum. Once the running sum is infinite or NaN
 * its compensation is meaningless (inf - inf would make it NaN), so it is no
 * longer updated and neum_get returns the sum alone: an all -inf input sums to
 * -inf, as the reference's plain accumulation gives. */
typedef struct { double s, c; } neum;
static void neum_add(neum* a, double x) {
  const double t = a->s + x;
  if (isfinite(t)) {
    if (fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x; else a->c += (x - t) + a->s;
  }
  a->s = t;
}
static double neum_get(const neum* a) { return isfinite(a->s) ? a->s + a->c : a->s; }

static int is_float_dt(int dt) { return dt == D_F32 || dt == D_F64 || dt == D_BF16 || dt == D_F16; }
static int is_signed_dt(int dt) {
  return dt == D_CHAR || dt == D_I8 || dt == D_I16 || dt == D_I32 || dt == D_I64 || is_float_dt(dt);
}

static double as_double(int dt, const void* p) { return ld_f64(dt, p); }
static uint64_t as_u64bits(int dt, const void* p) {  /* integer value as 64-bit two's complement */
  switch (dt) {
    case D_BOOL: return *(const uint8_t*)p != 0;
    case D_CHAR: case D_I8: return (uint64_t)(int64_t)*(const int8_t*)p;
    case D_U8: return *(const uint8_t*)p;
    case D_U16: return *(const uint16_t*)p;
    case D_I16: return (uint64_t)(int64_t)*(const int16_t*)p;
    case D_U32: return *(const uint32_t*)p;
    case D_I32: return (uint64_t)(int64_t)*(const int32_t*)p;
    case D_U64: return *(const uint64_t*)p;
    case D_I64: return (uint64_t)*(const int64_t*)p;
  }
  return 0;
}

/* compares element values in their own type: returns 1 if a > b */
static int gt_vals(int dt, const void* a, const void* b) {
  switch (dt) {
    case D_BOOL: return (*(const uint8_t*)a != 0) > (*(const uint8_t*)b != 0);
    case D_CHAR: case D_I8: return *(const int8_t*)a > *(const int8_t*)b;
    case D_U8: return *(const uint8_t*)a > *(const uint8_t*)b;
    case D_U16: return *(const uint16_t*)a > *(const uint16_t*)b;
    case D_I16: return *(const int16_t*)a > *(const int16_t*)b;
    case D_U32: return *(const uint32_t*)a > *(const uint32_t*)b;
    case D_I32: return *(const int32_t*)a > *(const int32_t*)b;
    case D_U64: return *(const uint64_t*)a > *(const uint64_t*)b;
    case D_I64: return *(const int64_t*)a > *(const int64_t*)b;
    case D_F32: return *(const float*)a > *(const float*)b;
    case D_F64: return *(const double*)a > *(const double*)b;
  }
  return 0;
}

/* max/min identity in the arithmetic dtype, written to an 8-byte buffer */
static void ident(int adt, int is_max, void* out) {
  memset(out, 0, 8);
  switch (adt) {
    case D_BOOL: *(uint8_t*)out = is_max ? 0 : 1; break;
    case D_CHAR: case D_I8: *(int8_t*)out = is_max ? INT8_MIN : INT8_MAX; break;
    case D_U8: *(uint8_t*)out = is_max ? 0 : UINT8_MAX; break;
    case D_U16: *(uint16_t*)out = is_max ? 0 : UINT16_MAX; break;
    case D_I16: *(int16_t*)out = is_max ? INT16_MIN : INT16_MAX; break;
    case D_U32: *(uint32_t*)out = is_max ? 0 : UINT32_MAX; break;
    case D_I32: *(int32_t*)out = is_max ? INT32_MIN : INT32_MAX; break;
    case D_U64: *(uint64_t*)out = is_max ? 0 : UINT64_MAX; break;
    case D_I64: *(int64_t*)out = is_max ? INT64_MIN : INT64_MAX; break;
    case D_F32: *(float*)out = is_max ? -3.4028234663852886e38f : 3.4028234663852886e38f; break;
    case D_F64: *(double*)out = is_max ? -1.7976931348623157e308 : 1.7976931348623157e308; break;
  }
}

static int arith(int dt) { return (dt == D_BF16 || dt == D_F16) ? D_F32 : dt; }
static int sum_dt(int dt) {
  switch (dt) {
    case D_BOOL: case D_U8: case D_U16: return D_U64;
    case D_I8: case D_I16: return D_I64;
    case D_BF16: case D_F16: return D_F32;
  }
  return dt;
}

int orc_reduce(const orc_view* src, int op, uint32_t axes_mask, const orc_view* out) {
  const int n = src->ndim;
  int64_t KN = 1, RN = 1;
  for (int d = 0; d < n; ++d) { if ((axes_mask >> d) & 1u) RN *= src->shape[d]; else KN *= src->shape[d]; }
  if (KN == 0) return 0;
  const int dt = src->dtype, adt = arith(dt);
  neum* fs = NULL; uint64_t* is = NULL; unsigned char* ext = NULL; int64_t* idx = NULL;
  const int isf = is_float_dt(dt);
  if (op <= 1) { if (isf) fs = calloc((size_t)KN, sizeof(neum)); else is = calloc((size_t)KN, 8); }
  else {
    ext = malloc((size_t)KN * 8); idx = malloc((size_t)KN * 8);
    for (int64_t j = 0; j < KN; ++j) { ident(adt, op == 2 || op == 4, ext + 8 * j); idx[j] = 0; }
  }
  int64_t c[ORC_MAXD] = {0};
  int64_t total = KN * RN;
  char* sb = vbase(src);
  for (int64_t e = 0; e < total; ++e) {
    int64_t rem = e;
    for (int d = n - 1; d >= 0; --d) { c[d] = rem % src->shape[d]; rem /= src->shape[d]; }
    int64_t j = 0, r = 0;
    for (int d = 0; d < n; ++d) {
      if ((axes_mask >> d) & 1u) r = r * src->shape[d] + c[d]; else j = j * src->shape[d] + c[d];
    }
    char* p = sb;
    for (int d = 0; d < n; ++d) p += c[d] * src->strides[d];
    if (op <= 1) {
      if (isf) neum_add(&fs[j], as_double(dt, p)); else is[j] += as_u64bits(dt, p);
    } else {
      unsigned char v[8] = {0};
      if (adt != dt) { const float f = ld_f32(dt, p); memcpy(v, &f, 4); } else memcpy(v, p, dsize(dt));
      const int better = (op == 2 || op == 4) ? gt_vals(adt, v, ext + 8 * j) : gt_vals(adt, ext + 8 * j, v);
      if (better) { memcpy(ext + 8 * j, v, 8); idx[j] = r; }
    }
  }
  /* write outputs in kept C order */
  const int kept = out->ndim;
  int64_t kshape[ORC_MAXD];
  int kd = 0;
  for (int d = 0; d < n; ++d) if (!((axes_mask >> d) & 1u)) kshape[kd++] = src->shape[d];
  char* obase = vbase(out);
  for (int64_t j = 0; j < KN; ++j) {
    int64_t rem = j;
    char* po = obase;
    for (int d = kept - 1; d >= 0; --d) { po += (rem % kshape[d]) * out->strides[d]; rem /= kshape[d]; }
    if (op == 0) {
      const int sdt = sum_dt(dt);
      if (isf) { const double s = neum_get(&fs[j]); st_f64(sdt, po, s); }
      else memcpy(po, &is[j], dsize(sdt));
    } else if (op == 1) {
      double s;
      if (isf) s = neum_get(&fs[j]);
      else s = is_signed_dt(dt) ? (double)(int64_t)is[j] : (double)is[j];
      *(double*)po = s / (double)RN;
    } else if (op == 2 || op == 3) {
      memcpy(po, ext + 8 * j, dsize(adt));
    } else {
      *(int64_t*)po = idx[j];
    }
  }
  free(fs); free(is); free(ext); free(idx);
  return 0;
}

/* ---- 3-D stencil ------------------------------------------------------------------
 * u_{t+1}[z,y,x] = u_t[z,y,x] + dt * sum_{o} w[o] u_t[z+oz, y+oy, x+ox], zero outside
 * the grid; w indexed (oz+1)*9 + (oy+1)*3 + (ox+1). In-place over `iters` steps in
 * float64 (u is float64, C-contiguous nz*ny*nx). */
int orc_stencil3d_f64(double* u, int64_t nz, int64_t ny, int64_t nx, const double* w, double dt,
                      int iters) {
  const int64_t n = nz * ny * nx;
  double* t = malloc((size_t)n * sizeof(double));
  if (!t) return 1;
  for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < nz; ++z) {
      for (int64_t y = 0; y < ny; ++y) {
        for (int64_t x = 0; x < nx; ++x) {
          double acc = 0.0;
          for (int oz = -1; oz <= 1; ++oz) {
            const int64_t zz = z + oz;
            if (zz < 0 || zz >= nz) continue;
            for (int oy = -1; oy <= 1; ++oy) {
              const int64_t yy = y + oy;
              if (yy < 0 || yy >= ny) continue;
              for (int ox = -1; ox <= 1; ++ox) {
                const int64_t xx = x + ox;
                const double wv = w[(oz + 1) * 9 + (oy + 1) * 3 + (ox + 1)];
                if (xx < 0 || xx >= nx || wv == 0.0) continue;
                acc += wv * u[(zz * ny + yy) * nx + xx];
              }
            }
          }
          const int64_t i = (z * ny + y) * nx + x;
          t[i] = u[i] + dt * acc;
        }
      }
    }
    memcpy(u, t, (size_t)n * sizeof(double));
  }
  free(t);
  return 0;
}

/* ---- scatter-add ------------------------------------------------------------------
 * host::scatter_add_recursive (src/lib/ncarray/host/elementwise.hh:482-505, walking
 * impl::scatter_reduce_recursive, :33-68): idx and src (equal shapes) are walked in C
 * index order; an index i with 0 <= i < dest->shape[0] adds the src value, cast to the
 * dest dtype (op_traits::cast), to dest[i] in the dest dtype (integers wrap, floats
 * round after every addition). dest is 1-D. Index dtypes are read as int64 (uint64
 * values >= 2^63 are out of range either way). */
int orc_scatter_add(const orc_view* dest, const orc_view* idx, const orc_view* src) {
  if (dest->ndim != 1 || idx->ndim != src->ndim) return 1;
  const int n = src->ndim;
  int64_t total = 1;
  for (int d = 0; d < n; ++d) {
    if (idx->shape[d] != src->shape[d]) return 2;
    total *= src->shape[d];
  }
  char* db = vbase(dest);
  const char* ib = vbase(idx);
  const char* sb = vbase(src);
  const int64_t dn = dest->shape[0];
  int64_t c[ORC_MAXD] = {0};
  for (int64_t e = 0; e < total; ++e) {
    int64_t rem = e;
    for (int d = n - 1; d >= 0; --d) { c[d] = rem % src->shape[d]; rem /= src->shape[d]; }
    const char* pi = ib;
    const char* ps = sb;
    for (int d = 0; d < n; ++d) { pi += c[d] * idx->strides[d]; ps += c[d] * src->strides[d]; }
    const int64_t t = ld_i64(idx->dtype, pi);
    if (t < 0 || t >= dn) continue;
    char* pd = db + t * dest->strides[0];
    switch (dest->dtype) {
      case D_I32: case D_U32: *(u32*)pd = (u32)(*(u32*)pd + (u32)ld_i64(src->dtype, ps)); break;
      case D_I64: case D_U64: *(u64*)pd = *(u64*)pd + (u64)ld_i64(src->dtype, ps); break;
      case D_F32: *(f32*)pd = *(f32*)pd + ld_f32(src->dtype, ps); break;
      case D_F64: *(f64*)pd = *(f64*)pd + ld_f64(src->dtype, ps); break;
      default: return 3;
    }
  }
  return 0;
}

/* ---- 2-D histogram ----------------------------------------------------------------
 * Binning rule of nca_hist2d: ix = floor((x - x_lo) * sx) in float32 with
 * sx = (float)(nbx / (x_hi - x_lo)); dropped unless 0 <= ix < nbx (NaN dropped).
 * counts accumulate (uint64); wsum (float64 here) accumulates w when w != NULL. */
int orc_hist2d(const float* x, const float* y, const float* w, int64_t n, int nbx, int nby,
               double x_lo, double x_hi, double y_lo, double y_hi, uint64_t* counts, double* wsum) {
  const float sx = (float)((double)nbx / (x_hi - x_lo));
  const float sy = (float)((double)nby / (y_hi - y_lo));
  const float xl = (float)x_lo, yl = (float)y_lo;
  for (int64_t i = 0; i < n; ++i) {
    const float fx = floorf((x[i] - xl) * sx);
    const float fy = floorf((y[i] - yl) * sy);
    if (!(fx >= 0.0f && fx < (float)nbx && fy >= 0.0f && fy < (float)nby)) continue;
    const int64_t b = (int64_t)fy * nbx + (int64_t)fx;
    counts[b] += 1;
    if (w && wsum) wsum[b] += (double)w[i];
  }
  return 0;
}

/* ---- batched reductions -----------------------------------------------------------
 * Per array: sum(x), sum(x)/len, max(x) (host rule), sum(x*x - x), all in float64. */
typedef struct { const void* data; int64_t length; int32_t dtype; int32_t reserved; } orc_item;
typedef struct { double sum, mean, max, sum_sq_m; } orc_result;

int orc_batch_reduce(const orc_item* items, int n, orc_result* res, int nthreads) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
  for (int i = 0; i < n; ++i) {
    neum s = {0, 0}, q = {0, 0};
    float mx = -3.4028234663852886e38f;
    const int64_t L = items[i].length;
    for (int64_t k = 0; k < L; ++k) {
      float x;
      if (items[i].dtype == D_F32) x = ((const float*)items[i].data)[k];
      else if (items[i].dtype == D_BF16) x = bf16_to_f32(((const uint16_t*)items[i].data)[k]);
      else x = f16_to_f32(((const uint16_t*)items[i].data)[k]);
      const double xd = (double)x;
      neum_add(&s, xd);
      neum_add(&q, xd * xd - xd);
      if (x > mx) mx = x;
    }
    res[i].sum = neum_get(&s);
    res[i].mean = neum_get(&s) / (double)L;
    res[i].max = (double)mx;
    res[i].sum_sq_m = neum_get(&q);
  }
  return 0;
}
