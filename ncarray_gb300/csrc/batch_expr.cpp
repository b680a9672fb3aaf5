// General batched reductions: many 1-D arrays of uneven length, each with up
// to NCA_BATCH_MAX_OUTS (tape, reduction) outputs -- any expression of the
// element (an ncarray tape over one operand) reduced by sum, mean, max, min,
// argmax or argmin -- in one persistent launch.
//
// ncarray has no batched form: a list of arrays must share one shape
// (src/lib/pyncarray/utilities.hh:271-314), and each reduction of each array
// is one synchronous GPUEngine launch (src/lib/ncarray/engines/gpuengine.hh:
// 222-333). Here:
//   - nca_batch_expr_create groups the items into programs (input dtype plus
//     the list of (tape, op) outputs), splits every array into chunks of about
//     `chunk_bytes` and uploads the item and chunk tables once; it generates one
//     kernel for the batch with NVRTC: every tape becomes an inlined device
//     function, every program an inlined chunk walker that evaluates each
//     distinct tape once per element and feeds one accumulator per distinct
//     (tape, sum / max / min) -- sum and mean share one, max and argmax one;
//   - the persistent kernel's CTAs walk the chunk table with a static stride;
//     a CTA reads its chunk with 16-byte streaming loads (scalar loads for the
//     unaligned head and tail), float32 sums are float-float pairs updated by
//     packed f32x2 TwoSum steps on two elements at once, max/min keep the first
//     index of the extreme (the host scan rule of host/reductions.hh:118-169:
//     strict comparison against lowest()/max(), NaN never wins);
//   - a block tree merges the threads; an item with one chunk is finished by
//     that CTA; otherwise each CTA stores a partial per output and the CTA that
//     stores an item's last partial (per-item arrival counter) merges the
//     item's partials in chunk order (deterministic) and resets the counter,
//     so the launch can be replayed from a CUDA graph with no memset.
// Results: per item NCA_BATCH_MAX_OUTS rows of {value (float64), index}.
// Tapes must have a float32 or float64 result; sums are accumulated as
// float-float pairs (float32 results) or in float64 (float64 results).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "common.hpp"
#include "jit.hpp"

namespace {

struct ItemDev {            // NcaBItem in the generated source
  const void* data;
  long long length;
  int prog;
  int first_chunk;
  int nchunks;
  int pad;
};

struct ChunkDev {           // NcaBChunk
  int item;
  int pad;
  long long begin;
  long long count;
};

struct PartDev {            // NcaBPart
  double s;
  double v;
  long long i;
  long long pad;
};

// (input dtype, outputs) shared by the items of one program
struct Program {
  int dtype = NCA_FLOAT32;
  int n_outs = 0;
  int tape[NCA_BATCH_MAX_OUTS] = {0};
  int op[NCA_BATCH_MAX_OUTS] = {0};
  bool operator<(const Program& o) const {
    if (dtype != o.dtype) return dtype < o.dtype;
    if (n_outs != o.n_outs) return n_outs < o.n_outs;
    for (int k = 0; k < n_outs; ++k) {
      if (tape[k] != o.tape[k]) return tape[k] < o.tape[k];
      if (op[k] != o.op[k]) return op[k] < o.op[k];
    }
    return false;
  }
};

int op_kind(int op) {   // 0 sum (sum, mean), 1 max (max, argmax), 2 min (min, argmin)
  switch (op) {
    case NCA_RED_SUM: case NCA_RED_MEAN: return 0;
    case NCA_RED_MAX: case NCA_RED_ARGMAX: return 1;
    default: return 2;
  }
}

// Static part of the generated source: tables, loads, accumulators, block merge.
const char* kBatchCommon = R"NCB(
struct NcaBItem { const void* data; long long length; int prog; int first_chunk; int nchunks; int pad; };
struct NcaBChunk { int item; int pad; long long begin; long long count; };
struct NcaBPart { double s; double v; long long i; long long pad; };
struct NcaBRes { double value; long long index; };
struct NcaBArgs {
  const NcaBItem* items; const NcaBChunk* chunks; NcaBPart* parts; unsigned* cnt; NcaBRes* res;
  const u64* scal; long long nchunks; int* status;
};
// threads of the consumer block (the pipelined form adds a producer warp) and
// the barrier over them
#if NCA_BPIPE
#define NCA_BT 256
__device__ __forceinline__ void nca_bsync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }
#else
#define NCA_BT 256
__device__ __forceinline__ void nca_bsync() { __syncthreads(); }
#endif

// a partial of a float32 result inside a block: float-float sum (h, l),
// extreme v and its index i
struct NcaBPartF { float h, l, v; long long i; };
// (h, l) += (h2, l2) in float32 (TwoSum of the high parts); an infinite or
// NaN sum keeps no error term
__device__ __forceinline__ void nca_ffadd(float& h, float& l, float h2, float l2) {
  const float s = __fadd_rn(h, h2);
  if (!(fabsf(s) < __int_as_float(0x7f800000))) { h = s; l = 0.f; return; }
  const float bb = __fsub_rn(s, h);
  const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
  h = s;
  l = __fadd_rn(__fadd_rn(l, l2), e);
}

template <class R> __device__ __forceinline__ R nca_blo();
template <> __device__ __forceinline__ float nca_blo<float>() { return __uint_as_float(0xff7fffffu); }
template <> __device__ __forceinline__ double nca_blo<double>() { return __longlong_as_double((i64)0xffefffffffffffffull); }
template <class R> __device__ __forceinline__ R nca_bhi();
template <> __device__ __forceinline__ float nca_bhi<float>() { return __uint_as_float(0x7f7fffffu); }
template <> __device__ __forceinline__ double nca_bhi<double>() { return __longlong_as_double(0x7fefffffffffffffll); }

// packed f32x2 arithmetic (two float32 lanes per instruction)
__device__ __forceinline__ u64 nca_pk(float2 v) { u64 r; asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y)); return r; }
__device__ __forceinline__ float2 nca_upk(u64 r) { float2 v; asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r)); return v; }
__device__ __forceinline__ float2 nca_fadd2(float2 a, float2 b) {
  u64 d; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(nca_pk(a)), "l"(nca_pk(b))); return nca_upk(d);
}
__device__ __forceinline__ float2 nca_ffma2(float2 a, float2 b, float2 c) {
  u64 d; asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(nca_pk(a)), "l"(nca_pk(b)), "l"(nca_pk(c))); return nca_upk(d);
}

// Accumulators. K: 0 sum, 1 max, 2 min; IDX: keep the first index of the extreme.
template <class R, int K, bool IDX> struct NcaBAcc;

// float32 sums: two float-float pairs (even / odd elements of a pair), every
// TwoSum step one packed f32x2 instruction (a - b as ffma2(b, -1, a)). Once a
// running sum is infinite or NaN it stays so; its error term is then ignored.
template <bool IDX> struct NcaBAcc<float, 0, IDX> {
  float2 hi, lo;
  __device__ __forceinline__ void init() { hi = make_float2(0.f, 0.f); lo = hi; }
  __device__ __forceinline__ void see2(float a, float b, i64) {
    const float2 x = make_float2(a, b), m1 = make_float2(-1.f, -1.f);
    const float2 s = nca_fadd2(hi, x);
    const float2 bb = nca_ffma2(hi, m1, s);
    const float2 e1 = nca_ffma2(nca_ffma2(bb, m1, s), m1, hi);
    const float2 e2 = nca_ffma2(bb, m1, x);
    lo = nca_fadd2(lo, nca_fadd2(e1, e2));
    hi = s;
  }
  __device__ __forceinline__ void see(float a, i64 i) { see2(a, 0.f, i); }
  __device__ __forceinline__ NcaBPart part() const {
    NcaBPart p;
    const double x = nca_isfinite(hi.x) ? (double)hi.x + (double)lo.x : (double)hi.x;
    const double y = nca_isfinite(hi.y) ? (double)hi.y + (double)lo.y : (double)hi.y;
    p.s = x + y; p.v = 0.0; p.i = -1; p.pad = 0;
    return p;
  }
  __device__ __forceinline__ NcaBPartF partf() const;
};
template <bool IDX> __device__ __forceinline__ NcaBPartF NcaBAcc<float, 0, IDX>::partf() const {
  NcaBPartF p;
  p.h = hi.x;
  p.l = nca_isfinite(hi.x) ? lo.x : 0.f;
  nca_ffadd(p.h, p.l, hi.y, nca_isfinite(hi.y) ? lo.y : 0.f);
  p.v = 0.f; p.i = -1;
  return p;
}
template <bool IDX> struct NcaBAcc<double, 0, IDX> {
  double d;
  __device__ __forceinline__ void init() { d = 0.0; }
  __device__ __forceinline__ void see(double a, i64) { d = __dadd_rn(d, a); }
  __device__ __forceinline__ void see2(double a, double b, i64) { d = __dadd_rn(__dadd_rn(d, a), b); }
  __device__ __forceinline__ NcaBPart part() const { NcaBPart p; p.s = d; p.v = 0.0; p.i = -1; p.pad = 0; return p; }
};
template <class R, int K, bool IDX> struct NcaBAcc {
  R v; i64 i;
  __device__ __forceinline__ NcaBPartF partf() const { NcaBPartF p; p.h = 0.f; p.l = 0.f; p.v = (float)v; p.i = i; return p; }
  __device__ __forceinline__ void init() { v = K == 1 ? nca_blo<R>() : nca_bhi<R>(); i = -1; }
  __device__ __forceinline__ void see(R a, i64 idx) {
    const bool better = K == 1 ? a > v : a < v;
    if (IDX) { if (better) { v = a; i = idx; } } else { v = better ? a : v; }
  }
  __device__ __forceinline__ void see2(R a, R b, i64 idx) { see(a, idx); see(b, idx + 1); }
  __device__ __forceinline__ NcaBPart part() const { NcaBPart p; p.s = 0.0; p.v = (double)v; p.i = i; p.pad = 0; return p; }
};

// merge of two partials of accumulator kind K (ties of extremes to the smaller index)
template <int K, bool IDX>
__device__ __forceinline__ void nca_bmerge(NcaBPart& a, const NcaBPart& b) {
  if (K == 0) { a.s = __dadd_rn(a.s, b.s); return; }
  const bool better = K == 1 ? b.v > a.v : b.v < a.v;
  if (!IDX) { a.v = better ? b.v : a.v; return; }
  if (b.i < 0) return;
  if (a.i < 0 || better || (b.v == a.v && b.i < a.i)) { a.v = b.v; a.i = b.i; }
}

template <int K, bool IDX>
__device__ __forceinline__ NcaBPart nca_bshfl_merge(NcaBPart p) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    NcaBPart o;
    o.s = __shfl_down_sync(0xffffffffu, p.s, off);
    o.v = __shfl_down_sync(0xffffffffu, p.v, off);
    o.i = __shfl_down_sync(0xffffffffu, p.i, off);
    nca_bmerge<K, IDX>(p, o);
  }
  return p;
}

// block tree of one partial per consumer thread; valid in thread 0 (NCA_BT == 256)
template <int K, bool IDX>
__device__ __forceinline__ NcaBPart nca_bblock(NcaBPart p, NcaBPart* sh) {
  p = nca_bshfl_merge<K, IDX>(p);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = p;
  nca_bsync();
  if (wid == 0) {
    if (lane < 8) p = sh[lane];
    else { p.s = 0.0; p.v = K == 1 ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll); p.i = -1; }
    p = nca_bshfl_merge<K, IDX>(p);
  }
  nca_bsync();
  return p;
}

// the same in float32 for float32 results; thread 0 widens the result once
template <int K, bool IDX>
__device__ __forceinline__ void nca_bmergef(NcaBPartF& a, const NcaBPartF& b) {
  if (K == 0) { nca_ffadd(a.h, a.l, b.h, b.l); return; }
  const bool better = K == 1 ? b.v > a.v : b.v < a.v;
  if (!IDX) { a.v = better ? b.v : a.v; return; }
  if (b.i < 0) return;
  if (a.i < 0 || better || (b.v == a.v && b.i < a.i)) { a.v = b.v; a.i = b.i; }
}
template <int K, bool IDX>
__device__ __forceinline__ NcaBPartF nca_bshflf(NcaBPartF p) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    NcaBPartF o;
    o.h = __shfl_down_sync(0xffffffffu, p.h, off);
    o.l = __shfl_down_sync(0xffffffffu, p.l, off);
    o.v = __shfl_down_sync(0xffffffffu, p.v, off);
    o.i = __shfl_down_sync(0xffffffffu, p.i, off);
    nca_bmergef<K, IDX>(p, o);
  }
  return p;
}
template <int K, bool IDX>
__device__ __forceinline__ NcaBPart nca_bblockf(NcaBPartF p, NcaBPart* shd) {
  NcaBPartF* sh = reinterpret_cast<NcaBPartF*>(shd);
  p = nca_bshflf<K, IDX>(p);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = p;
  nca_bsync();
  if (wid == 0) {
    if (lane < 8) p = sh[lane];
    else { p.h = 0.f; p.l = 0.f; p.v = K == 1 ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000); p.i = -1; }
    p = nca_bshflf<K, IDX>(p);
  }
  nca_bsync();
  NcaBPart r;
  r.s = nca_isfinite(p.h) ? (double)p.h + (double)p.l : (double)p.h;
  r.v = (double)p.v; r.i = p.i; r.pad = 0;
  return r;
}

// final value of one output from its merged partial
__device__ __forceinline__ void nca_bstore(NcaBRes* r, int op, const NcaBPart& p, long long length, double ext_none) {
  if (op == 0) { r->value = p.s; r->index = 0; }
  else if (op == 1) { r->value = __ddiv_rn(p.s, (double)length); r->index = 0; }
  else if (op == 2 || op == 3) { r->value = p.v; r->index = 0; }
  else { r->value = p.i < 0 ? ext_none : p.v; r->index = p.i < 0 ? 0 : p.i; }
}

// Walkers over elements [b, b + n) of a typed array: every thread takes its
// elements in increasing index order; 16-byte loads on the aligned body.
template <class F> __device__ __forceinline__ void nca_bwalk_f32(const void* base, i64 b, i64 n, F& f) {
  const float* p = (const float*)base + b;
  i64 head = (i64)(((16u - ((unsigned)(unsigned long long)p & 15u)) & 15u) >> 2);
  if (((unsigned long long)p & 3u) != 0) head = n;
  if (head > n) head = n;
  for (i64 i = threadIdx.x; i < head; i += blockDim.x) f.one(__ldcs(p + i), b + i);
  const i64 nv = (n - head) >> 2;
  const float4* pv = (const float4*)(p + head);
#pragma unroll NCA_BUNROLL
  for (i64 k = threadIdx.x; k < nv; k += blockDim.x) {
    const float4 v = __ldcs(pv + k);
    const i64 i = b + head + 4 * k;
    f.two(v.x, v.y, i);
    f.two(v.z, v.w, i + 2);
  }
  for (i64 i = head + 4 * nv + threadIdx.x; i < n; i += blockDim.x) f.one(__ldcs(p + i), b + i);
}
template <int HALF, class F> __device__ __forceinline__ void nca_bwalk_h16(const void* base, i64 b, i64 n, F& f) {
  const unsigned short* p = (const unsigned short*)base + b;
  auto cv = [](unsigned short h) { return HALF ? nca_f16_to_f32(h) : nca_bf16_to_f32(h); };
  i64 head = (i64)(((16u - ((unsigned)(unsigned long long)p & 15u)) & 15u) >> 1);
  if (((unsigned long long)p & 1u) != 0) head = n;
  if (head > n) head = n;
  for (i64 i = threadIdx.x; i < head; i += blockDim.x) f.one(cv(__ldcs(p + i)), b + i);
  const i64 nv = (n - head) >> 3;
  const uint4* pv = (const uint4*)(p + head);
#pragma unroll NCA_BUNROLL
  for (i64 k = threadIdx.x; k < nv; k += blockDim.x) {
    const uint4 v = __ldcs(pv + k);
    const i64 i = b + head + 8 * k;
    const u32 w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int j = 0; j < 4; ++j)
      f.two(cv((unsigned short)(w[j] & 0xffffu)), cv((unsigned short)(w[j] >> 16)), i + 2 * j);
  }
  for (i64 i = head + 8 * nv + threadIdx.x; i < n; i += blockDim.x) f.one(cv(__ldcs(p + i)), b + i);
}
template <class F> __device__ __forceinline__ void nca_bwalk_f64(const void* base, i64 b, i64 n, F& f) {
  const double* p = (const double*)base + b;
  i64 head = (i64)(((16u - ((unsigned)(unsigned long long)p & 15u)) & 15u) >> 3);
  if (((unsigned long long)p & 7u) != 0) head = n;
  if (head > n) head = n;
  for (i64 i = threadIdx.x; i < head; i += blockDim.x) f.one(__ldcs(p + i), b + i);
  const i64 nv = (n - head) >> 1;
  const double2* pv = (const double2*)(p + head);
#pragma unroll NCA_BUNROLL
  for (i64 k = threadIdx.x; k < nv; k += blockDim.x) {
    const double2 v = __ldcs(pv + k);
    f.two(v.x, v.y, b + head + 2 * k);
  }
  for (i64 i = head + 2 * nv + threadIdx.x; i < n; i += blockDim.x) f.one(__ldcs(p + i), b + i);
}
template <class T, class F> __device__ __forceinline__ void nca_bwalk_int(const void* base, i64 b, i64 n, F& f) {
  const T* p = (const T*)base + b;
  for (i64 i = threadIdx.x; i < n; i += blockDim.x) f.one(__ldcs(p + i), b + i);
}

#if NCA_BPIPE
// ---- pipelined form: a producer warp streams each chunk's 16-byte aligned
// body through NCA_BNS shared-memory slabs of NCA_BSLAB bytes by bulk copies
// (full / empty mbarriers); the consumer threads take the unaligned head and
// tail elements with plain loads and the body from the slabs. Every wait is
// bounded (2 s): one that runs out records NCA_ERR_TIMEOUT in the status word,
// stops the producer, and the consumers finish without waiting (void results).
__device__ __forceinline__ u64 nca_bgt() { u64 t; asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t)); return t; }
__device__ __forceinline__ bool nca_btry(u32 bar, u32 par) {
  u32 ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
               : "=r"(ok) : "r"(bar), "r"(par) : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool nca_bwait(u32 bar, u32 par) {
  if (nca_btry(bar, par)) return true;
  const u64 t0 = nca_bgt();
  while (true) {
    if (nca_btry(bar, par)) return true;
    if (nca_bgt() - t0 > 2000000000ull) return false;
  }
}
struct NcaBPipe {
  u32 slabs, full0, empty0;   // shared addresses
  const unsigned char* sm;    // generic pointer of slab 0
  long long k;                // slabs consumed by this CTA so far
  bool dead;                  // a wait ran out: no more waits, results void
  volatile int* stop;
};
// the 16-byte aligned body [a, e) of a chunk (a == e: none, every element scalar)
__device__ __forceinline__ void nca_bbody(const NcaBItem& it, const NcaBChunk& c, unsigned long long& p0,
                                          unsigned long long& a, unsigned long long& e) {
  const unsigned long long es = (unsigned long long)it.pad;
  p0 = (unsigned long long)it.data + (unsigned long long)c.begin * es;
  const unsigned long long p1 = p0 + (unsigned long long)c.count * es;
  a = (p0 + 15ull) & ~15ull;
  e = p1 & ~15ull;
  if (e <= a || (p0 % es) != 0ull) { a = p1; e = p1; }
}
// one chunk: head and tail elements by plain loads (LOAD(i) gives element i of
// the chunk), the body slab by slab (VEC(v, i) takes the 16-byte vector v
// whose first element has chunk index i)
template <int ES, class F, class LOAD, class VEC>
__device__ __forceinline__ void nca_bpipe_chunk(const NcaBArgs& A, const NcaBItem& it, const NcaBChunk& c, F& f,
                                                NcaBPipe& P, LOAD ld, VEC vec) {
  unsigned long long p0, a, e;
  nca_bbody(it, c, p0, a, e);
  const i64 nh = (i64)((a - p0) / ES), ne = (i64)((e - a) / ES);
  for (i64 i = threadIdx.x; i < nh; i += NCA_BT) ld(i, c.begin + i);
  for (i64 i = nh + ne + threadIdx.x; i < c.count; i += NCA_BT) ld(i, c.begin + i);
  const int lane = threadIdx.x & 31;
  for (unsigned long long src = a; src < e; src += NCA_BSLAB, ++P.k) {
    const int k = (int)(P.k % NCA_BNS);
    if (!P.dead && *P.stop) P.dead = true;
    if (!P.dead && !nca_bwait(P.full0 + 8u * (u32)k, (u32)((P.k / NCA_BNS) & 1))) {
      P.dead = true;
      if (lane == 0) { atomicExch(A.status, 1); *P.stop = 1; }
    }
    if (!P.dead) {
      const unsigned long long left = e - src;
      const int nv = (int)((left < (unsigned long long)NCA_BSLAB ? left : (unsigned long long)NCA_BSLAB) / 16ull);
      const uint4* v = (const uint4*)(P.sm + (size_t)k * NCA_BSLAB);
      const i64 i0 = c.begin + nh + (i64)((src - a) / ES);
      for (int j = threadIdx.x; j < nv; j += NCA_BT) vec(v[j], i0 + (i64)j * (16 / ES));
    }
    __syncwarp();
    if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(P.empty0 + 8u * (u32)k) : "memory");
  }
}
#endif
)NCB";

const char* kBatchKernel = R"NCB(
extern "C" __global__ void __launch_bounds__(256) nca_batch_expr(const NcaBArgs A) {
  __shared__ NcaBPart sh[8];
  __shared__ int last;
  for (long long cid = blockIdx.x; cid < A.nchunks; cid += gridDim.x) {
    const NcaBChunk c = A.chunks[cid];
    const NcaBItem it = A.items[c.item];
    nca_bdispatch(A, it, c, cid, sh);
    if (it.nchunks == 1) continue;
    // the CTA that stores the item's last partial merges them in chunk order
    if (threadIdx.x == 0) {
      __threadfence();
      last = atomicAdd(A.cnt + c.item, 1u) + 1u == (unsigned)it.nchunks;
    }
    __syncthreads();
    if (last) {
      __threadfence();
      nca_bfinish(A, it, c.item, sh);
      if (threadIdx.x == 0) A.cnt[c.item] = 0u;
    }
    __syncthreads();
  }
}
)NCB";

const char* kBatchKernelPipe = R"NCB(
extern "C" __global__ void __launch_bounds__(288) nca_batch_expr(const NcaBArgs A) {
  extern __shared__ __align__(128) unsigned char nca_bsm[];
  __shared__ NcaBPart sh[8];
  __shared__ int last;
  __shared__ volatile int stop;
  const u32 sbase = (u32)__cvta_generic_to_shared(nca_bsm);
  const u32 full0 = sbase + NCA_BNS * NCA_BSLAB, empty0 = full0 + 8 * NCA_BNS;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    stop = 0;
    for (int k = 0; k < NCA_BNS; ++k) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8 * k) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;" ::"r"(empty0 + 8 * k) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (wid == 8) {
    // producer: lane 0 copies the bodies of this CTA's chunks slab by slab
    if (lane != 0) return;
    long long issued = 0;
    bool bad = false;
    for (long long cid = blockIdx.x; cid < A.nchunks && !bad; cid += gridDim.x) {
      const NcaBChunk c = A.chunks[cid];
      const NcaBItem it = A.items[c.item];
      unsigned long long p0, a, e;
      nca_bbody(it, c, p0, a, e);
      for (unsigned long long src = a; src < e; src += NCA_BSLAB, ++issued) {
        const int k = (int)(issued % NCA_BNS);
        if (issued >= NCA_BNS && !nca_bwait(empty0 + 8 * k, (u32)((issued / NCA_BNS - 1) & 1))) { bad = true; break; }
        if (stop) { bad = true; break; }
        const unsigned long long left = e - src;
        const u32 bytes = (u32)(left < (unsigned long long)NCA_BSLAB ? left : (unsigned long long)NCA_BSLAB);
        const u32 bar = full0 + 8 * k;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(sbase + (u32)(k * NCA_BSLAB)), "l"(src), "r"(bytes), "r"(bar) : "memory");
      }
    }
    if (bad) {
      atomicExch(A.status, 1);
      stop = 1;
      // the copies still in flight land before the CTA's shared memory goes away
      for (long long j = issued > NCA_BNS ? issued - NCA_BNS : 0; j < issued; ++j)
        nca_bwait(full0 + 8 * (int)(j % NCA_BNS), (u32)((j / NCA_BNS) & 1));
    }
    return;
  }
  NcaBPipe P;
  P.slabs = sbase; P.full0 = full0; P.empty0 = empty0; P.sm = nca_bsm; P.k = 0; P.dead = false; P.stop = &stop;
  for (long long cid = blockIdx.x; cid < A.nchunks; cid += gridDim.x) {
    const NcaBChunk c = A.chunks[cid];
    const NcaBItem it = A.items[c.item];
    nca_bdispatch(A, it, c, cid, sh, P);
    if (it.nchunks == 1) continue;
    // the CTA that stores the item's last partial merges them in chunk order
    if (threadIdx.x == 0) {
      __threadfence();
      last = atomicAdd(A.cnt + c.item, 1u) + 1u == (unsigned)it.nchunks;
    }
    nca_bsync();
    if (last) {
      __threadfence();
      nca_bfinish(A, it, c.item, sh);
      if (threadIdx.x == 0) A.cnt[c.item] = 0u;
    }
    nca_bsync();
  }
}
)NCB";

std::string dtype_walker(int dt) {
  switch (dt) {
    case NCA_FLOAT32: return "nca_bwalk_f32";
    case NCA_BFLOAT16: return "nca_bwalk_h16<0>";
    case NCA_FLOAT16: return "nca_bwalk_h16<1>";
    case NCA_FLOAT64: return "nca_bwalk_f64";
    case NCA_INT32: return "nca_bwalk_int<int>";
    case NCA_INT64: return "nca_bwalk_int<i64>";
  }
  nca::fail(NCA_ERR_DTYPE, "batched input dtype %d: float32, float64, bfloat16, float16, int32 or int64", dt);
}

int dtinfo_size(int dt) { return nca::dtinfo(dt).size; }

// element gi of the item in the pipelined walker (plain load), as the program's load type
std::string pipe_load(int dt, const std::string& gi) {
  switch (dt) {
    case NCA_FLOAT32: return "__ldcs((const float*)it.data + " + gi + ")";
    case NCA_BFLOAT16: return "nca_bf16_to_f32(__ldcs((const unsigned short*)it.data + " + gi + "))";
    case NCA_FLOAT16: return "nca_f16_to_f32(__ldcs((const unsigned short*)it.data + " + gi + "))";
    case NCA_FLOAT64: return "__ldcs((const double*)it.data + " + gi + ")";
    case NCA_INT32: return "__ldcs((const int*)it.data + " + gi + ")";
    default: return "__ldcs((const i64*)it.data + " + gi + ")";
  }
}

// the elements of one 16-byte vector v whose first element is gi
std::string pipe_vec(int dt) {
  switch (dt) {
    case NCA_FLOAT32:
      return "      f.two(__uint_as_float(v.x), __uint_as_float(v.y), gi);\n"
             "      f.two(__uint_as_float(v.z), __uint_as_float(v.w), gi + 2);\n";
    case NCA_BFLOAT16: case NCA_FLOAT16: {
      const std::string cv = dt == NCA_FLOAT16 ? "nca_f16_to_f32" : "nca_bf16_to_f32";
      std::string r;
      const char* w[4] = {"v.x", "v.y", "v.z", "v.w"};
      for (int j = 0; j < 4; ++j)
        r += std::string("      f.two(") + cv + "((unsigned short)(" + w[j] + " & 0xffffu)), " + cv + "((unsigned short)(" +
             w[j] + " >> 16)), gi + " + std::to_string(2 * j) + ");\n";
      return r;
    }
    case NCA_FLOAT64:
      return "      f.two(__longlong_as_double((i64)(((u64)v.y << 32) | v.x)), "
             "__longlong_as_double((i64)(((u64)v.w << 32) | v.z)), gi);\n";
    case NCA_INT32:
      return "      f.two((int)v.x, (int)v.y, gi);\n      f.two((int)v.z, (int)v.w, gi + 2);\n";
    default:
      return "      f.two((i64)(((u64)v.y << 32) | v.x), (i64)(((u64)v.w << 32) | v.z), gi);\n";
  }
}

const char* load_type(int dt) {
  switch (dt) {
    case NCA_FLOAT64: return "double";
    case NCA_INT32: return "int";
    case NCA_INT64: return "i64";
    default: return "float";
  }
}

struct Acc {   // one accumulator of a program
  int tape, kind;
  bool idx;
};

}  // namespace

struct nca_batch_expr {
  int dev = 0;
  int n = 0;
  std::vector<nca::Tape> tapes;
  std::vector<nca_batch_expr_item> items;
  std::vector<Program> progs;
  std::vector<uint64_t> scal;         // compute-type words of every tape's scalars
  std::vector<int> scal_off;          // first word of tape t
  CUfunction fn = nullptr;
  void* d_items = nullptr;
  void* d_chunks = nullptr;
  void* d_parts = nullptr;
  void* d_cnt = nullptr;
  void* d_scal = nullptr;
  long long nchunks = 0;
  long long chunk_bytes = 512 * 1024;   // fastest with 4 loads in flight and 4 CTAs per SM on 20,000 uneven arrays
  int unroll = 4;          // 16-byte loads per thread issued together in the walkers
  int ctas_per_sm = 4;
  bool pipe = true;        // a producer warp streams the chunks through shared-memory slabs
  int nslab = 4, slab = 16384;
  int ctas = 0;
  cudaGraphExec_t graph = nullptr;
  void* graph_results = nullptr;
  void* graph_stream = nullptr;
};

namespace {

std::string tape_fn(const nca::Tape& t, int k) {
  std::ostringstream os;
  const char* W = nca::jit_ctype(t.compute_dtype);
  const char* R = nca::jit_ctype(t.result_dtype);
  os << "__device__ __forceinline__ " << R << " nca_bt" << k << "(" << W << " x0, const u64* s) {\n"
     << "  typedef " << W << " nca_w;\n  (void)s;\n" << nca::jit_gen_eval(t, "x", "") << "}\n";
  return os.str();
}

// the accumulators of program p: one per distinct (tape, kind)
std::vector<Acc> prog_accs(const Program& p, int* acc_of_out) {
  std::vector<Acc> accs;
  for (int o = 0; o < p.n_outs; ++o) {
    const int kind = op_kind(p.op[o]);
    const bool idx = p.op[o] == NCA_RED_ARGMAX || p.op[o] == NCA_RED_ARGMIN;
    int found = -1;
    for (size_t a = 0; a < accs.size(); ++a)
      if (accs[a].tape == p.tape[o] && accs[a].kind == kind) found = (int)a;
    if (found < 0) { accs.push_back({p.tape[o], kind, idx}); found = (int)accs.size() - 1; }
    if (idx) accs[(size_t)found].idx = true;
    acc_of_out[o] = found;
  }
  return accs;
}

std::string gen_batch_source(const nca_batch_expr& b) {
  std::ostringstream os;
  os << nca::jit_prelude() << "#define NCA_BUNROLL " << b.unroll << "\n#define NCA_BPIPE " << (b.pipe ? 1 : 0)
     << "\n#define NCA_BNS " << b.nslab << "\n#define NCA_BSLAB " << b.slab << "\n" << kBatchCommon;
  for (size_t k = 0; k < b.tapes.size(); ++k) os << tape_fn(b.tapes[k], (int)k);
  for (size_t p = 0; p < b.progs.size(); ++p) {
    const Program& pg = b.progs[p];
    int acc_of_out[NCA_BATCH_MAX_OUTS];
    const std::vector<Acc> accs = prog_accs(pg, acc_of_out);
    const std::string LT = load_type(pg.dtype);
    // element functor: every distinct tape once per element, fed to its accumulators
    os << "struct NcaBF" << p << " {\n";
    for (size_t a = 0; a < accs.size(); ++a)
      os << "  NcaBAcc<" << nca::jit_ctype(b.tapes[(size_t)accs[a].tape].result_dtype) << ", " << accs[a].kind << ", "
         << (accs[a].idx ? "true" : "false") << "> a" << a << ";\n";
    os << "  const u64* s;\n";
    os << "  __device__ __forceinline__ void init(const u64* sc) { s = sc;";
    for (size_t a = 0; a < accs.size(); ++a) os << " a" << a << ".init();";
    os << " }\n";
    std::vector<int> used;
    for (const Acc& a : accs) if (std::find(used.begin(), used.end(), a.tape) == used.end()) used.push_back(a.tape);
    os << "  __device__ __forceinline__ void one(" << LT << " x, i64 i) {\n";
    for (int t : used)
      os << "    const auto r" << t << " = nca_bt" << t << "((" << nca::jit_ctype(b.tapes[(size_t)t].compute_dtype)
         << ")x, s + " << b.scal_off[(size_t)t] << ");\n";
    for (size_t a = 0; a < accs.size(); ++a) os << "    a" << a << ".see(r" << accs[a].tape << ", i);\n";
    os << "  }\n  __device__ __forceinline__ void two(" << LT << " x, " << LT << " y, i64 i) {\n";
    for (int t : used) {
      const char* W = nca::jit_ctype(b.tapes[(size_t)t].compute_dtype);
      os << "    const auto r" << t << " = nca_bt" << t << "((" << W << ")x, s + " << b.scal_off[(size_t)t] << ");\n"
         << "    const auto q" << t << " = nca_bt" << t << "((" << W << ")y, s + " << b.scal_off[(size_t)t] << ");\n";
    }
    for (size_t a = 0; a < accs.size(); ++a) os << "    a" << a << ".see2(r" << accs[a].tape << ", q" << accs[a].tape << ", i);\n";
    os << "  }\n};\n";
    // chunk of an item of program p: walk, block trees, partials or final values
    if (b.pipe) {
      os << "__device__ __forceinline__ void nca_bprog" << p
         << "(const NcaBArgs& A, const NcaBItem& it, const NcaBChunk& c, long long cid, NcaBPart* sh, NcaBPipe& P) {\n"
         << "  NcaBF" << p << " f; f.init(A.scal);\n"
         << "  nca_bpipe_chunk<" << dtinfo_size(pg.dtype) << ">(A, it, c, f, P,\n"
         << "    [&](i64 i, i64 gi) { (void)i; f.one(" << pipe_load(pg.dtype, "gi") << ", gi); },\n"
         << "    [&](const uint4 v, i64 gi) {\n" << pipe_vec(pg.dtype) << "    });\n";
    } else {
      os << "__device__ __forceinline__ void nca_bprog" << p
         << "(const NcaBArgs& A, const NcaBItem& it, const NcaBChunk& c, long long cid, NcaBPart* sh) {\n"
         << "  NcaBF" << p << " f; f.init(A.scal);\n"
         << "  " << dtype_walker(pg.dtype) << "(it.data, c.begin, c.count, f);\n";
    }
    for (size_t a = 0; a < accs.size(); ++a) {
      const bool f32 = b.tapes[(size_t)accs[a].tape].result_dtype == NCA_FLOAT32;
      os << "  {\n    const NcaBPart m = " << (f32 ? "nca_bblockf<" : "nca_bblock<") << accs[a].kind << ", "
         << (accs[a].idx ? "true" : "false") << ">(f.a" << a << (f32 ? ".partf(), sh);" : ".part(), sh);")
         << "\n    if (threadIdx.x == 0) {\n";
      for (int o = 0; o < pg.n_outs; ++o) {
        if (acc_of_out[o] != (int)a) continue;
        const std::string none = pg.op[o] == NCA_RED_ARGMAX ? "(double)nca_blo<" + std::string(nca::jit_ctype(b.tapes[(size_t)pg.tape[o]].result_dtype)) + ">()"
                                                           : "(double)nca_bhi<" + std::string(nca::jit_ctype(b.tapes[(size_t)pg.tape[o]].result_dtype)) + ">()";
        os << "      if (it.nchunks == 1) nca_bstore(A.res + (long long)c.item * " << NCA_BATCH_MAX_OUTS << " + " << o
           << ", " << pg.op[o] << ", m, it.length, " << none << ");\n";
      }
      os << "      if (it.nchunks > 1) A.parts[cid * " << NCA_BATCH_MAX_OUTS << " + " << a << "] = m;\n    }\n  }\n";
    }
    os << "}\n";
    // the merge of an item's partials (chunk order), then its final values
    os << "__device__ __forceinline__ void nca_bfin" << p << "(const NcaBArgs& A, const NcaBItem& it, int item, NcaBPart* sh) {\n";
    for (size_t a = 0; a < accs.size(); ++a) {
      const int K = accs[a].kind;
      const char* IDX = accs[a].idx ? "true" : "false";
      // identity: lowest() / max() of the result type, the value an output
      // reports when no element beats it (partials without a candidate are
      // skipped by the indexed merge)
      const std::string R = nca::jit_ctype(b.tapes[(size_t)accs[a].tape].result_dtype);
      os << "  {\n    NcaBPart m; m.s = 0.0; m.i = -1; m.pad = 0;\n"
         << "    m.v = (double)" << (K == 1 ? "nca_blo<" : "nca_bhi<") << R << ">();\n"
         << "    for (int k = threadIdx.x; k < it.nchunks; k += NCA_BT) {\n"
         << "      NcaBPart o = A.parts[(long long)(it.first_chunk + k) * " << NCA_BATCH_MAX_OUTS << " + " << a << "];\n"
         << "      nca_bmerge<" << K << ", " << IDX << ">(m, o);\n    }\n"
         << "    m = nca_bblock<" << K << ", " << IDX << ">(m, sh);\n    if (threadIdx.x == 0) {\n";
      for (int o = 0; o < pg.n_outs; ++o) {
        if (acc_of_out[o] != (int)a) continue;
        const std::string none = pg.op[o] == NCA_RED_ARGMAX ? "(double)nca_blo<" + std::string(nca::jit_ctype(b.tapes[(size_t)pg.tape[o]].result_dtype)) + ">()"
                                                           : "(double)nca_bhi<" + std::string(nca::jit_ctype(b.tapes[(size_t)pg.tape[o]].result_dtype)) + ">()";
        os << "      nca_bstore(A.res + (long long)item * " << NCA_BATCH_MAX_OUTS << " + " << o << ", " << pg.op[o]
           << ", m, it.length, " << none << ");\n";
      }
      os << "    }\n  }\n";
    }
    os << "}\n";
  }
  const std::string PX = b.pipe ? ", NcaBPipe& P" : "";
  const std::string PA = b.pipe ? ", P" : "";
  os << "__device__ __forceinline__ void nca_bdispatch(const NcaBArgs& A, const NcaBItem& it, const NcaBChunk& c, long long cid, NcaBPart* sh"
     << PX << ") {\n  switch (it.prog) {\n";
  for (size_t p = 0; p < b.progs.size(); ++p) os << "    case " << p << ": nca_bprog" << p << "(A, it, c, cid, sh" << PA << "); break;\n";
  os << "  }\n}\n__device__ __forceinline__ void nca_bfinish(const NcaBArgs& A, const NcaBItem& it, int item, NcaBPart* sh) {\n  switch (it.prog) {\n";
  for (size_t p = 0; p < b.progs.size(); ++p) os << "    case " << p << ": nca_bfin" << p << "(A, it, item, sh); break;\n";
  os << "  }\n}\n" << (b.pipe ? kBatchKernelPipe : kBatchKernel);
  return os.str();
}

struct Args {
  const void* items;
  const void* chunks;
  void* parts;
  void* cnt;
  void* res;
  const void* scal;
  long long nchunks;
  int* status;
};

// dynamic shared memory of the pipelined form: the slabs and two mbarriers per slab
size_t pipe_smem(const nca_batch_expr& b) { return b.pipe ? (size_t)b.nslab * (size_t)b.slab + 16 * (size_t)b.nslab : 0; }

void launch(nca_batch_expr* b, void* results, cudaStream_t s) {
  if (b->nchunks == 0) return;
  Args a{b->d_items, b->d_chunks, b->d_parts, b->d_cnt, results, b->d_scal, b->nchunks, nca::jit_status_word()};
  void* params[] = {&a};
  nca::count_launch();
  nca::check_cu(nca::drv().cuLaunchKernel(b->fn, (unsigned)std::min<long long>(b->ctas, b->nchunks), 1, 1,
                                          b->pipe ? 288 : 256, 1, 1, (unsigned)pipe_smem(*b), (CUstream)s, params,
                                          nullptr),
                "cuLaunchKernel(batched expressions)");
}

void free_batch(nca_batch_expr* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (void* p : {b->d_items, b->d_chunks, b->d_parts, b->d_cnt, b->d_scal})
    if (p) cudaFree(p);
  delete b;
}

}  // namespace

extern "C" int32_t nca_batch_expr_create(const nca_batch_expr_item* items, int32_t n_items, const nca_tape* tapes,
                                         int32_t n_tapes, nca_batch_expr** out, void* stream) {
  nca_batch_expr* b = nullptr;
  const int32_t st = nca::guarded([&] {
    using namespace nca;
    if (!out) fail(NCA_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (n_items < 0 || (n_items > 0 && !items)) fail(NCA_ERR_INVALID, "bad item list");
    if (n_tapes < 1 || n_tapes > 64 || !tapes) fail(NCA_ERR_LIMIT, "%d tapes (1..64)", n_tapes);
    b = new nca_batch_expr();
    b->dev = current_device();
    b->n = n_items;
    for (int t = 0; t < n_tapes; ++t) {
      Tape tp = make_tape(&tapes[t], 1);
      const int r = tp.result_dtype;
      if (r != NCA_FLOAT32 && r != NCA_FLOAT64)
        fail(NCA_ERR_DTYPE, "tape %d: batched outputs need a float32 or float64 result (got dtype %d)", t, r);
      if (tp.uses_idx) fail(NCA_ERR_UNSUPPORTED, "tape %d: IDX is not available in batched tapes", t);
      b->scal_off.push_back((int)b->scal.size());
      for (size_t k = 0; k < tp.scalar_dtypes.size(); ++k)
        b->scal.push_back(jit_scalar_word(tp.compute_dtype, tp.scalar_dtypes[k], tp.scalar_slots[k]));
      b->tapes.push_back(tp);
    }
    if (b->scal.empty()) b->scal.push_back(0);
    b->items.assign(items, items + n_items);
    std::map<Program, int> prog_id;
    std::vector<ItemDev> hi((size_t)n_items);
    std::vector<ChunkDev> hc;
    // schedule knobs: chunk bytes, 16-byte loads per thread in flight, CTAs per SM
    if (const char* e = getenv("NCA_BATCH_EXPR_CHUNK")) b->chunk_bytes = std::max(4096ll, atoll(e));
    if (const char* e = getenv("NCA_BATCH_EXPR_UNROLL")) b->unroll = std::max(1, std::min(16, atoi(e)));
    if (const char* e = getenv("NCA_BATCH_EXPR_CTAS")) b->ctas_per_sm = std::max(1, std::min(8, atoi(e)));
    if (const char* e = getenv("NCA_BATCH_EXPR_PIPE")) b->pipe = e[0] != '0';
    if (const char* e = getenv("NCA_BATCH_EXPR_SLAB")) b->slab = std::max(1024, std::min(65536, atoi(e) / 16 * 16));
    if (const char* e = getenv("NCA_BATCH_EXPR_NSLAB")) b->nslab = std::max(2, std::min(8, atoi(e)));
    if (b->pipe && !getenv("NCA_BATCH_EXPR_CTAS")) b->ctas_per_sm = 3;
    for (int i = 0; i < n_items; ++i) {
      const nca_batch_expr_item& it = items[i];
      if (it.length < 0) fail(NCA_ERR_SHAPE, "item %d: negative length", i);
      if (it.length > 0 && !it.data) fail(NCA_ERR_INVALID, "item %d: null data", i);
      (void)dtype_walker(it.dtype);
      if (it.n_outs < 1 || it.n_outs > NCA_BATCH_MAX_OUTS)
        fail(NCA_ERR_LIMIT, "item %d: %d outputs (1..%d)", i, it.n_outs, NCA_BATCH_MAX_OUTS);
      Program pg;
      pg.dtype = it.dtype;
      pg.n_outs = it.n_outs;
      for (int o = 0; o < it.n_outs; ++o) {
        if (it.tape[o] < 0 || it.tape[o] >= n_tapes) fail(NCA_ERR_INVALID, "item %d output %d: tape %d", i, o, it.tape[o]);
        if (it.op[o] < NCA_RED_SUM || it.op[o] > NCA_RED_ARGMIN) fail(NCA_ERR_INVALID, "item %d output %d: op %d", i, o, it.op[o]);
        pg.tape[o] = it.tape[o];
        pg.op[o] = it.op[o];
      }
      auto f = prog_id.find(pg);
      int pid;
      if (f == prog_id.end()) {
        pid = (int)b->progs.size();
        if (pid >= 64) fail(NCA_ERR_LIMIT, "more than 64 distinct (dtype, outputs) programs in one batch");
        prog_id[pg] = pid;
        b->progs.push_back(pg);
      } else {
        pid = f->second;
      }
      const long long isz = dtinfo(it.dtype).size;
      const long long per = std::max(256ll, b->chunk_bytes / isz);
      const long long nc = it.length == 0 ? 1 : (it.length + per - 1) / per;
      hi[(size_t)i] = ItemDev{it.data, it.length, pid, (int)hc.size(), (int)nc, (int)isz};
      for (long long c = 0; c < nc; ++c) {
        const long long beg = c * per;
        hc.push_back(ChunkDev{i, 0, beg, std::min(per, it.length - beg)});
      }
      if (hc.size() > (size_t)0x7fffffff) fail(NCA_ERR_LIMIT, "too many chunks");
    }
    b->nchunks = (long long)hc.size();
    cudaStream_t s = (cudaStream_t)stream;
    auto upload = [&](void** dst, const void* src, size_t bytes) {
      check_cuda(cudaMalloc(dst, std::max<size_t>(bytes, 16)), "cudaMalloc(batch tables)");
      if (bytes) check_cuda(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s), "batch table upload");
    };
    upload(&b->d_items, hi.data(), hi.size() * sizeof(ItemDev));
    upload(&b->d_chunks, hc.data(), hc.size() * sizeof(ChunkDev));
    upload(&b->d_scal, b->scal.data(), b->scal.size() * sizeof(uint64_t));
    check_cuda(cudaMalloc(&b->d_parts, std::max<size_t>((size_t)b->nchunks * NCA_BATCH_MAX_OUTS * sizeof(PartDev), 16)),
               "cudaMalloc(batch partials)");
    check_cuda(cudaMalloc(&b->d_cnt, std::max<size_t>((size_t)n_items * 4, 16)), "cudaMalloc(batch counters)");
    check_cuda(cudaMemsetAsync(b->d_cnt, 0, std::max<size_t>((size_t)n_items * 4, 16), s), "batch counters");
    b->fn = jit_get(gen_batch_source(*b), "nca_batch_expr");
    int per_sm = 0;
    if (b->pipe)
      check_cu(drv().cuFuncSetAttribute(b->fn, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, (int)pipe_smem(*b)),
               "smem attribute");
    check_cu(drv().cuOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->fn, b->pipe ? 288 : 256, pipe_smem(*b)),
             "occupancy");
    b->ctas = sm_count(b->dev) * std::max(1, std::min(per_sm, b->ctas_per_sm));
    check_cuda(cudaStreamSynchronize(s), "batch table upload");
    *out = b;
  });
  if (st != NCA_OK) free_batch(b);
  return st;
}

extern "C" int32_t nca_batch_expr_run(nca_batch_expr* b, nca_batch_value* results, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!b || (!results && b->n > 0)) fail(NCA_ERR_INVALID, "null argument");
    launch(b, results, (cudaStream_t)stream);
    check_cuda(cudaGetLastError(), "batched expressions launch");
  });
}

extern "C" int32_t nca_batch_expr_run_graph(nca_batch_expr* b, nca_batch_value* results, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!b || (!results && b->n > 0)) fail(NCA_ERR_INVALID, "null argument");
    if (b->graph && (b->graph_results != results || b->graph_stream != stream)) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    if (!b->graph) {
      cudaStream_t cs;
      check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        launch(b, results, cs);
        e = cudaStreamEndCapture(cs, &g);
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
      if (g) cudaGraphDestroy(g);
      cudaStreamDestroy(cs);
      check_cuda(e, "batched expressions graph");
      b->graph_results = results;
      b->graph_stream = stream;
    }
    count_launch(b->nchunks > 0 ? 1 : 0);
    check_cuda(cudaGraphLaunch(b->graph, (cudaStream_t)stream), "cudaGraphLaunch");
  });
}

// The plain form: per item and output, one nca_expr_reduce launch of the tape
// in float64 over the array (float64 accumulation), written into the result row.
extern "C" int32_t nca_batch_expr_run_plain(nca_batch_expr* b, nca_batch_value* results, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!b || (!results && b->n > 0)) fail(NCA_ERR_INVALID, "null argument");
    for (int i = 0; i < b->n; ++i) {
      const nca_batch_expr_item& it = b->items[(size_t)i];
      nca_view src;
      std::memset(&src, 0, sizeof(src));
      src.data = const_cast<void*>(it.data);
      src.dtype = it.dtype;
      src.ndim = 1;
      src.shape[0] = it.length;
      src.strides[0] = dtinfo(it.dtype).size;
      src.pointer_axis = -1;
      for (int o = 0; o < it.n_outs; ++o) {
        const Tape& tp = b->tapes[(size_t)it.tape[o]];
        nca_tape t;
        std::memset(&t, 0, sizeof(t));
        t.instrs = tp.instrs.data();
        t.n_instrs = (int32_t)tp.instrs.size();
        t.n_scalars = (int32_t)tp.scalar_slots.size();
        t.scalar_dtypes = tp.scalar_dtypes.data();
        t.scalar_slots = tp.scalar_slots.data();
        t.compute_dtype = NCA_FLOAT64;
        t.result_dtype = NCA_FLOAT64;
        Tape t64 = make_tape(&t, 1);
        nca_batch_value* row = results + (long long)i * NCA_BATCH_MAX_OUTS + o;
        nca_reduction r[2];
        std::memset(r, 0, sizeof(r));
        int nr = 1;
        const int op = it.op[o];
        auto scalar_out = [&](nca_reduction& red, int rop, void* p, int dt) {
          red.op = rop;
          red.axes_mask = 1u;
          red.out.data = p;
          red.out.dtype = dt;
          red.out.ndim = 0;
          red.out.pointer_axis = -1;
        };
        if (op == NCA_RED_ARGMAX || op == NCA_RED_ARGMIN) {
          scalar_out(r[0], op == NCA_RED_ARGMAX ? NCA_RED_MAX : NCA_RED_MIN, &row->value, NCA_FLOAT64);
          scalar_out(r[1], op, &row->index, NCA_INT64);
          nr = 2;
        } else {
          scalar_out(r[0], op, &row->value, NCA_FLOAT64);
        }
        if (it.length == 0) fail(NCA_ERR_SHAPE, "the plain form needs non-empty arrays");
        expr_reduce(t64, &src, 1, nullptr, r, nr, (cudaStream_t)stream);
      }
    }
  });
}

extern "C" int32_t nca_batch_expr_info(const nca_batch_expr* b, int64_t* n_chunks, int32_t* n_programs, int32_t* ctas) {
  return nca::guarded([&] {
    if (!b) nca::fail(NCA_ERR_INVALID, "null batch");
    if (n_chunks) *n_chunks = b->nchunks;
    if (n_programs) *n_programs = (int32_t)b->progs.size();
    if (ctas) *ctas = b->ctas;
  });
}

extern "C" void nca_batch_expr_destroy(nca_batch_expr* b) { free_batch(b); }

namespace nca {
// Compile-only check of the batched kernel class for `arch` (no device): four
// tapes (identity, x*x - x in float32 and float64, a float32 comparison) and
// programs over float32, bfloat16, float64 and int32 inputs with every op.
int batch_expr_selftest(const char* arch) {
  nca_batch_expr b;
  b.unroll = 4;
  auto mk = [](std::vector<uint32_t> ins, int w) {
    Tape t;
    t.instrs = std::move(ins);
    t.compute_dtype = w;
    t.result_dtype = w;
    t.n_arrays = 1;
    return t;
  };
  const uint32_t L0 = (uint32_t)NCA_OP_LOAD_NCARR << 24, MUL = (uint32_t)NCA_OP_MUL << 24;
  const uint32_t SUB = (uint32_t)NCA_OP_SUB << 24, GT = (uint32_t)NCA_OP_GT << 24, C0 = (uint32_t)NCA_OP_LOAD_CONST << 24;
  b.tapes.push_back(mk({L0}, NCA_FLOAT32));
  b.tapes.push_back(mk({L0, L0, MUL, L0, SUB}, NCA_FLOAT32));
  b.tapes.push_back(mk({L0, L0, MUL, L0, SUB}, NCA_FLOAT64));
  Tape g = mk({L0, C0, GT}, NCA_FLOAT32);
  g.scalar_dtypes = {NCA_FLOAT32};
  g.scalar_slots = {0};
  b.tapes.push_back(g);
  b.scal_off = {0, 0, 0, 0};
  b.scal = {0};
  Program p1;
  p1.dtype = NCA_FLOAT32; p1.n_outs = 4;
  p1.tape[0] = 0; p1.op[0] = NCA_RED_SUM; p1.tape[1] = 0; p1.op[1] = NCA_RED_MEAN;
  p1.tape[2] = 0; p1.op[2] = NCA_RED_MAX; p1.tape[3] = 1; p1.op[3] = NCA_RED_SUM;
  Program p2 = p1;
  p2.dtype = NCA_BFLOAT16;
  Program p3;
  p3.dtype = NCA_FLOAT64; p3.n_outs = 3;
  p3.tape[0] = 2; p3.op[0] = NCA_RED_ARGMIN; p3.tape[1] = 2; p3.op[1] = NCA_RED_MIN; p3.tape[2] = 2; p3.op[2] = NCA_RED_SUM;
  Program p4;
  p4.dtype = NCA_INT32; p4.n_outs = 2;
  p4.tape[0] = 3; p4.op[0] = NCA_RED_ARGMAX; p4.tape[1] = 0; p4.op[1] = NCA_RED_MEAN;
  b.progs = {p1, p2, p3, p4};
  b.pipe = false;
  jit_compile_only(gen_batch_source(b), arch);
  b.pipe = true;   // the pipelined form (producer warp, shared-memory slabs)
  Program p5 = p4;
  p5.dtype = NCA_INT64;
  Program p6 = p2;
  p6.dtype = NCA_FLOAT16;
  b.progs = {p1, p2, p3, p4, p5, p6};
  jit_compile_only(gen_batch_source(b), arch);
  return 2;
}
}  // namespace nca
