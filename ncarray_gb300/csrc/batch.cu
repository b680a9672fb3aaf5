// Batched reductions over many arrays of uneven length (float32 / bfloat16 /
// float16): per array sum, mean, max and sum(x*x - x).
//
// ncarray has no batched API (a list of arrays must share one shape:
// src/lib/pyncarray/utilities.hh:271-314); issued through its GPUEngine, each
// reduction of each array is one synchronous launch (gpuengine.hh:301-333).
// Here the whole batch is one persistent launch:
//   - nca_batch_create splits every array into chunks of `chunk_bytes` and
//     uploads a descriptor table (array, first element, element count) once;
//   - the persistent kernel's CTAs walk the chunk table with a static stride
//     (chunks carry equal bytes, so the walk is balanced); a producer warp
//     streams each chunk through shared-memory slabs by bulk copies and the
//     consumer warps reduce it with per-thread float-float sums (Knuth TwoSum,
//     packed float32x2) of x and of fma(x, x, -x) and a float max, then a
//     float-float warp tree; each warp writes one partial record per chunk;
//   - the warp writing an array's last partial (a per-array counter
//     incremented after a release fence) combines that array's partials in a
//     fixed order (deterministic) and resets the counter for the next launch.
// The only waits are the bounded mbarrier waits of the bulk-copy pipeline
// (below). The schedule (chunk bytes, slab bytes, CTAs per SM) comes from an
// autotuner whose choices are cached per shape class in a text file next to
// the JIT cache.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "common.hpp"
#include "mbar.cuh"
#include "jit.hpp"

struct nca_batch {
  int n = 0;
  int dev = 0;
  std::vector<nca_batch_item> items;
  // device tables
  void* d_items = nullptr;    // ItemDev[n]
  void* d_chunks = nullptr;   // ChunkDev[nchunks]
  void* d_parts = nullptr;    // PartDev[nchunks * consumer warps]
  void* d_done = nullptr;     // unsigned[n]
  void* d_status = nullptr;   // int: NCA_ERR_TIMEOUT after a wait that ran out
  long long nchunks = 0;
  // schedule
  long long chunk_bytes = 256 * 1024;
  int threads = 256, slab = 16384, ctas_per_sm = 3;
  std::string shape_class;
  // graph
  cudaGraphExec_t graph = nullptr;
  cudaStream_t capture_stream = nullptr;
  void* graph_results = nullptr;
};

namespace {

struct ItemDev {
  const void* data;
  long long length;
  int dtype;
  int first_chunk;
  int nchunks;
  int pad;
};

struct ChunkDev {
  int item;
  int index;        // chunk number within the item
  long long begin;  // first element
  long long count;  // elements
  unsigned long long a, e;   // byte range of the 16-byte aligned body (a == e: none)
  long long slabs;           // bulk-copy slabs of the body
};

struct PartDev {
  double s, q;   // sum(x), sum(x*x - x)
  float mx;      // max (lowest() if none above it)
  int pad;
};

__device__ __forceinline__ float ld_elem(const void* p, long long i, int dt) {
  if (dt == NCA_FLOAT32) return __ldcs(static_cast<const float*>(p) + i);
  const unsigned short h = __ldcs(static_cast<const unsigned short*>(p) + i);
  if (dt == NCA_BFLOAT16) return __uint_as_float(((unsigned)h) << 16);
  float f;
  asm("{.reg .b16 t; mov.b16 t, %1; cvt.f32.f16 %0, t;}" : "=f"(f) : "h"(h));
  return f;
}

__device__ __forceinline__ float lowest_f() { return __uint_as_float(0xff7fffffu); }

// Two float-float accumulators held as float2 pairs (even / odd elements), so
// every step of Knuth's TwoSum is one packed f32x2 instruction; a - b is
// ffma2(b, -1, a), exact up to its single rounding.
struct FF2 {
  float2 hi = make_float2(0.f, 0.f), lo = make_float2(0.f, 0.f);
  __device__ __forceinline__ void add(float2 x) {
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 s = __fadd2_rn(hi, x);
    const float2 bb = __ffma2_rn(hi, m1, s);
    const float2 e1 = __ffma2_rn(__ffma2_rn(bb, m1, s), m1, hi);
    const float2 e2 = __ffma2_rn(bb, m1, x);
    lo = __fadd2_rn(lo, __fadd2_rn(e1, e2));
    hi = s;
  }
  __device__ __forceinline__ double get() const {
    return ((double)hi.x + (double)lo.x) + ((double)hi.y + (double)lo.y);
  }
};

__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

struct Acc2 {
  FF2 s, q;
  float mx = -3.40282347e+38f;   // lowest float (bit pattern 0xff7fffff)
  // a pair of elements
  __device__ __forceinline__ void see(float2 x) {
    s.add(x);
    const float2 nx = make_float2(-x.x, -x.y);
    q.add(__ffma2_rn(x, x, nx));
    mx = max3f(mx, x.x, x.y);
  }
  // one element (the other lane adds zero)
  __device__ __forceinline__ void see1(float x) {
    s.add(make_float2(x, 0.f));
    q.add(make_float2(__fmaf_rn(x, x, -x), 0.f));
    mx = fmaxf(mx, x);
  }
};

// 16 bytes -> float2 pairs: float32 gives 2 pairs, 16-bit types 4
template <int DT> struct Vec;
template <> struct Vec<NCA_FLOAT32> {
  static constexpr int kElems = 4;
  static __device__ __forceinline__ void unpack(const uint4& u, float2* o) {
    o[0] = make_float2(__uint_as_float(u.x), __uint_as_float(u.y));
    o[1] = make_float2(__uint_as_float(u.z), __uint_as_float(u.w));
  }
  static __device__ __forceinline__ float one(const void* p, long long i) { return __ldcs(static_cast<const float*>(p) + i); }
};
template <> struct Vec<NCA_BFLOAT16> {
  static constexpr int kElems = 8;
  static __device__ __forceinline__ float2 w2(unsigned w) {
    return make_float2(__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u));
  }
  static __device__ __forceinline__ void unpack(const uint4& u, float2* o) {
    o[0] = w2(u.x); o[1] = w2(u.y); o[2] = w2(u.z); o[3] = w2(u.w);
  }
  static __device__ __forceinline__ float one(const void* p, long long i) {
    return __uint_as_float(((unsigned)__ldcs(static_cast<const unsigned short*>(p) + i)) << 16);
  }
};
template <> struct Vec<NCA_FLOAT16> {
  static constexpr int kElems = 8;
  static __device__ __forceinline__ float2 w2(unsigned w) {
    float a, b;
    asm("{.reg .b16 l, h; mov.b32 {l, h}, %2; cvt.f32.f16 %0, l; cvt.f32.f16 %1, h;}" : "=f"(a), "=f"(b) : "r"(w));
    return make_float2(a, b);
  }
  static __device__ __forceinline__ void unpack(const uint4& u, float2* o) {
    o[0] = w2(u.x); o[1] = w2(u.y); o[2] = w2(u.z); o[3] = w2(u.w);
  }
  static __device__ __forceinline__ float one(const void* p, long long i) {
    const unsigned short h = __ldcs(static_cast<const unsigned short*>(p) + i);
    float f;
    asm("{.reg .b16 t; mov.b16 t, %1; cvt.f32.f16 %0, t;}" : "=f"(f) : "h"(h));
    return f;
  }
};

// bulk-copy slabs per CTA and the limit of every wait on one of their mbarriers
constexpr int NSLAB = 4;
constexpr unsigned long long kWaitNs = 2000000000ull;


using nca_dev::mbar_wait;

// the 16-byte aligned body of a chunk (computed on the host)
struct Body {
  uintptr_t a, e;
  long long slabs;
};
__device__ __forceinline__ Body chunk_body(const ChunkDev& c) { return Body{(uintptr_t)c.a, (uintptr_t)c.e, c.slabs}; }

// elements of 16 bytes: float32 gives 2 pairs, 16-bit types 4
template <int DT>
__device__ __forceinline__ void see_vec(Acc2& acc, const uint4& u) {
  float2 f[Vec<DT>::kElems / 2];
  Vec<DT>::unpack(u, f);
#pragma unroll
  for (int j = 0; j < Vec<DT>::kElems / 2; ++j) acc.see(f[j]);
}

// two accumulator sets take alternate vectors: two independent TwoSum chains.
// t: this thread's index among the T consumer threads
template <int DT>
__device__ __forceinline__ void see_slab(Acc2& a0, Acc2& a1, const uint4* v, int nv, int t, int T) {
  int i = t;
  for (; i + T < nv; i += 2 * T) {
    const uint4 u0 = v[i], u1 = v[i + T];
    see_vec<DT>(a0, u0);
    see_vec<DT>(a1, u1);
  }
  if (i < nv) see_vec<DT>(a0, v[i]);
}

// head and tail elements of chunk c outside its aligned body (one warp: < 16 elements)
__device__ __forceinline__ void see_edges(Acc2& acc, const ItemDev& it, const ChunkDev& c, const Body& b, int lane) {
  const int isz = it.dtype == NCA_FLOAT32 ? 4 : 2;
  const uintptr_t lo = (uintptr_t)it.data + (uintptr_t)(c.begin * isz);
  const long long nh = (long long)((b.a - lo) / isz);               // elements before the body
  const long long nt = c.count - nh - (long long)((b.e - b.a) / isz);  // elements after it
  for (long long t = lane; t < nh + nt; t += 32) {
    const long long i = t < nh ? c.begin + t : c.begin + c.count - nt + (t - nh);
    acc.see1(ld_elem(it.data, i, it.dtype));
  }
}

// float-float addition of two (hi, lo) pairs, both lanes at once (Knuth TwoSum
// of the highs, the lows added to its error, Fast2Sum renormalisation)
__device__ __forceinline__ void ff2_add(float2& h, float2& l, float2 h2, float2 l2) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 s = __fadd2_rn(h, h2);
  const float2 bb = __ffma2_rn(h, m1, s);
  const float2 e1 = __ffma2_rn(__ffma2_rn(bb, m1, s), m1, h);
  const float2 e2 = __ffma2_rn(bb, m1, h2);
  const float2 e = __fadd2_rn(__fadd2_rn(e1, e2), __fadd2_rn(l, l2));
  const float2 hi = __fadd2_rn(s, e);
  l = __ffma2_rn(__ffma2_rn(s, m1, hi), m1, e);
  h = hi;
}

__device__ __forceinline__ float2 shfl_down2(float2 v, int off) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, off), __shfl_down_sync(0xffffffffu, v.y, off));
}

// a warp's accumulators -> one partial (valid in lane 0). float32 float-float
// all the way down the warp tree; float64 only for lane 0's final conversion.
__device__ PartDev warp_part(const Acc2& a0, const Acc2& a1) {
  float2 sh = a0.s.hi, sl = a0.s.lo, qh = a0.q.hi, ql = a0.q.lo;
  ff2_add(sh, sl, a1.s.hi, a1.s.lo);
  ff2_add(qh, ql, a1.q.hi, a1.q.lo);
  // lanes now (even, odd) elements; regroup as (sum, sum_sq_m) and add the halves
  float2 h = make_float2(sh.x, qh.x), l = make_float2(sl.x, ql.x);
  ff2_add(h, l, make_float2(sh.y, qh.y), make_float2(sl.y, ql.y));
  float mx = fmaxf(a0.mx, a1.mx);
  for (int off = 16; off > 0; off >>= 1) {
    const float2 h2 = shfl_down2(h, off), l2 = shfl_down2(l, off);
    ff2_add(h, l, h2, l2);
    mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, off));
  }
  PartDev p;
  p.s = (double)h.x + (double)l.x;
  p.q = (double)h.y + (double)l.y;
  p.mx = mx;
  p.pad = 0;
  return p;
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// ---- the persistent kernel --------------------------------------------------------
// blockDim = consumer threads + one producer warp (the last warp). The
// producer's lane 0 walks this CTA's chunk sequence issuing one bulk copy per
// slab into NSLAB shared-memory slabs; slab k completes on full[k] (transaction
// bytes) and is released on empty[k] once every consumer warp has read it
// (one arrival per warp), so consumer warps run without block barriers. Each
// consumer warp reduces its share of every slab, writes one partial per chunk
// (parts[chunk * NW + warp]) and counts it on the array's counter; the warp
// that brings the count to nchunks * NW merges the array's partials in a fixed
// order (float64; deterministic) and resets the counter for the next launch.
// Waits are bounded (2 s of %globaltimer); a wait that runs out records
// NCA_ERR_TIMEOUT, raises the CTA's stop flag, and the producer then waits
// (bounded) for its copies in flight before the CTA exits.
__global__ void batch_persistent_kernel(const ItemDev* __restrict__ items, const ChunkDev* __restrict__ chunks,
                                        long long nchunks, PartDev* __restrict__ parts, unsigned* __restrict__ done,
                                        nca_batch_result* __restrict__ results, int slab, int* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char sm[];
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
  const uint32_t full0 = sbase + NSLAB * slab;   // full[k] at full0 + 8k, empty[k] at full0 + 8(NSLAB + k)
  const uint32_t empty0 = full0 + 8 * NSLAB;
  __shared__ volatile int s_stop;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int T = (int)blockDim.x - 32, NW = T >> 5;   // consumer threads and warps
  if (threadIdx.x == 0) {
    s_stop = 0;
    for (int k = 0; k < NSLAB; ++k) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8 * k) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(empty0 + 8 * k), "r"(NW) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (wid == NW) {   // producer warp
    if (lane != 0) return;
    long long issued = 0;
    bool failed = false;
    for (long long c = blockIdx.x; c < nchunks && !failed; c += gridDim.x) {
      const Body bd = chunk_body(chunks[c]);
      for (long long i = 0; i < bd.slabs; ++i, ++issued) {
        const int k = (int)(issued % NSLAB);
        if (issued >= NSLAB &&
            !mbar_wait(empty0 + 8 * k, (uint32_t)((issued / NSLAB - 1) & 1), kWaitNs)) {
          failed = true;
          break;
        }
        if (s_stop) { failed = true; break; }
        const uintptr_t src = bd.a + (uintptr_t)i * slab;
        const uintptr_t left = bd.e - src;
        const uint32_t bytes = (uint32_t)(left < (uintptr_t)slab ? left : (uintptr_t)slab);
        const uint32_t bar = full0 + 8 * k;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(sbase + (uint32_t)(k * slab)), "l"(src), "r"(bytes), "r"(bar) : "memory");
      }
    }
    if (failed) {
      atomicExch(status, (int)NCA_ERR_TIMEOUT);
      s_stop = 1;
      // the copies still in flight land before the CTA (and its shared memory) goes away
      for (long long j = issued > NSLAB ? issued - NSLAB : 0; j < issued; ++j)
        mbar_wait(full0 + 8 * (int)(j % NSLAB), (uint32_t)((j / NSLAB) & 1), kWaitNs / 2);
    }
    return;
  }

  // consumer warps
  long long consumed = 0;
  for (long long c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const ChunkDev ch = chunks[c];
    const ItemDev it = items[ch.item];
    const Body bd = chunk_body(ch);
    Acc2 acc, acc1;
    if (wid == 0) see_edges(acc, it, ch, bd, lane);
    for (long long i = 0; i < bd.slabs; ++i, ++consumed) {
      const int k = (int)(consumed % NSLAB);
      if (!mbar_wait(full0 + 8 * k, (uint32_t)((consumed / NSLAB) & 1), kWaitNs) || s_stop) {
        if (lane == 0) { atomicExch(status, (int)NCA_ERR_TIMEOUT); s_stop = 1; }
        return;
      }
      const uintptr_t src = bd.a + (uintptr_t)i * slab;
      const uintptr_t left = bd.e - src;
      const int nv = (int)((left < (uintptr_t)slab ? left : (uintptr_t)slab) / 16);
      const uint4* v = reinterpret_cast<const uint4*>(sm + k * slab);
      if (it.dtype == NCA_FLOAT32) see_slab<NCA_FLOAT32>(acc, acc1, v, nv, threadIdx.x, T);
      else if (it.dtype == NCA_BFLOAT16) see_slab<NCA_BFLOAT16>(acc, acc1, v, nv, threadIdx.x, T);
      else see_slab<NCA_FLOAT16>(acc, acc1, v, nv, threadIdx.x, T);
      __syncwarp();
      if (lane == 0) mbar_arrive(empty0 + 8 * k);   // this warp is done with slab k
    }
    const PartDev p = warp_part(acc, acc1);
    const unsigned want = (unsigned)it.nchunks * (unsigned)NW;
    unsigned prev = 0;
    if (lane == 0) {
      parts[c * NW + wid] = p;
      __threadfence();
      prev = atomicAdd(done + ch.item, 1u);
    }
    prev = __shfl_sync(0xffffffffu, prev, 0);
    if (prev + 1 == want) {   // this warp merges the array: lanes take partials in a fixed order
      __threadfence();
      double s = 0.0, q = 0.0;
      float mx = lowest_f();
      const PartDev* pk = parts + (long long)it.first_chunk * NW;
      for (unsigned j = lane; j < want; j += 32) {
        s += __ldcg(&pk[j].s);
        q += __ldcg(&pk[j].q);
        const float m = __ldcg(&pk[j].mx);
        mx = m > mx ? m : mx;
      }
      for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        q += __shfl_down_sync(0xffffffffu, q, off);
        const float m = __shfl_down_sync(0xffffffffu, mx, off);
        mx = m > mx ? m : mx;
      }
      if (lane == 0) {
        nca_batch_result r;
        r.sum = s;
        r.mean = s / (double)it.length;
        r.max = (double)mx;
        r.sum_sq_m = q;
        results[ch.item] = r;
        done[ch.item] = 0u;   // ready for the next launch
      }
    }
  }
}

// ---- plain form: one launch per op per array, float64 accumulation ----------------
// OP 0: sum, 1: max, 2: sum(x*x - x); mean is sum / length (a fourth launch).
template <int OP>
__global__ void plain_kernel(const void* data, long long n, int dt, double* out) {
  double acc = OP == 1 ? -1.0e300 : 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = (double)ld_elem(data, i, dt);
    if (OP == 0) acc += v;
    if (OP == 1) acc = v > acc ? v : acc;
    if (OP == 2) acc += v * v - v;
  }
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_down_sync(0xffffffffu, acc, off);
    if (OP == 1) acc = o > acc ? o : acc; else acc += o;
  }
  __shared__ double sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = OP == 1 ? -1.0e300 : 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r = OP == 1 ? (sh[k] > r ? sh[k] : r) : r + sh[k];
    if (OP == 1) {
      // ordered max on the bit pattern of a double
      unsigned long long b = (unsigned long long)__double_as_longlong(r);
      b = (b >> 63) ? ~b : (b | 0x8000000000000000ull);
      atomicMax(reinterpret_cast<unsigned long long*>(out), b);
    } else {
      atomicAdd(out, r);
    }
  }
}

__global__ void plain_init_kernel(nca_batch_result* r, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { r[i].sum = 0.0; r[i].mean = 0.0; r[i].max = 0.0; r[i].sum_sq_m = 0.0; }
}

__global__ void plain_mean_kernel(nca_batch_result* r, const ItemDev* items, int i) {
  r[i].mean = r[i].sum / (double)items[i].length;
  unsigned long long b = (unsigned long long)__double_as_longlong(r[i].max);
  // the max slot holds the ordered bit pattern; 0 means no element
  if (b == 0ull) { r[i].max = (double)lowest_f(); return; }
  b = (b >> 63) ? (b & 0x7fffffffffffffffull) : ~b;
  r[i].max = __longlong_as_double((long long)b);
}

void launch_persistent(nca_batch* B, nca_batch_result* results, cudaStream_t s) {
  const int grid = (int)std::min<long long>(B->nchunks, (long long)nca::sm_count(B->dev) * B->ctas_per_sm);
  if (grid <= 0) return;
  const ItemDev* it = (const ItemDev*)B->d_items;
  const ChunkDev* ch = (const ChunkDev*)B->d_chunks;
  PartDev* pa = (PartDev*)B->d_parts;
  unsigned* dn = (unsigned*)B->d_done;
  const int smem = NSLAB * B->slab + 16 * NSLAB;
  nca::check_cuda(cudaFuncSetAttribute(batch_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                  "batch smem");
  batch_persistent_kernel<<<grid, B->threads + 32, smem, s>>>(it, ch, B->nchunks, pa, dn, results, B->slab,
                                                         (int*)B->d_status);
  nca::check_cuda(cudaGetLastError(), "batched kernel launch");
  nca::count_launch();
}

void free_tables(nca_batch* B) {
  if (B->d_chunks) cudaFree(B->d_chunks);
  if (B->d_parts) cudaFree(B->d_parts);
  B->d_chunks = B->d_parts = nullptr;
  if (B->graph) { cudaGraphExecDestroy(B->graph); B->graph = nullptr; }
}

// (re)builds the chunk table for the current chunk_bytes
void build_chunks(nca_batch* B, cudaStream_t s) {
  free_tables(B);
  std::vector<ItemDev> items(B->n);
  std::vector<ChunkDev> chunks;
  for (int i = 0; i < B->n; ++i) {
    const nca_batch_item& src = B->items[i];
    const int isz = src.dtype == NCA_FLOAT32 ? 4 : 2;
    const long long per = std::max<long long>(B->chunk_bytes / isz, 256);
    items[i].data = src.data;
    items[i].length = src.length;
    items[i].dtype = src.dtype;
    items[i].first_chunk = (int)chunks.size();
    long long k = 0;
    for (long long b = 0; b < src.length || (b == 0 && src.length == 0); b += per, ++k) {
      ChunkDev c{i, (int)k, b, std::min(per, src.length - b), 0, 0, 0};
      // the 16-byte aligned part of the chunk's bytes, moved by bulk copies
      const uintptr_t lo = (uintptr_t)src.data + (uintptr_t)(c.begin * isz), hi = lo + (uintptr_t)(c.count * isz);
      const uintptr_t a = (lo + 15) & ~(uintptr_t)15, e = hi & ~(uintptr_t)15;
      if (e > a) {
        c.a = a;
        c.e = e;
        c.slabs = (long long)((e - a + B->slab - 1) / B->slab);
      } else {
        c.a = c.e = lo;
      }
      chunks.push_back(c);
      if (src.length == 0) break;
    }
    items[i].nchunks = (int)k + (src.length == 0 ? 1 : 0);
    items[i].pad = 0;
  }
  B->nchunks = (long long)chunks.size();
  using nca::check_cuda;
  if (!B->d_items) check_cuda(cudaMalloc(&B->d_items, sizeof(ItemDev) * std::max(B->n, 1)), "batch items");
  if (!B->d_done) {
    check_cuda(cudaMalloc(&B->d_done, sizeof(unsigned) * std::max(B->n, 1)), "batch counters");
    check_cuda(cudaMemsetAsync(B->d_done, 0, sizeof(unsigned) * std::max(B->n, 1), s), "batch counters");
  }
  if (!B->d_status) {
    check_cuda(cudaMalloc(&B->d_status, sizeof(int)), "batch status");
    check_cuda(cudaMemsetAsync(B->d_status, 0, sizeof(int), s), "batch status");
  }
  check_cuda(cudaMalloc(&B->d_chunks, sizeof(ChunkDev) * std::max<long long>(B->nchunks, 1)), "batch chunks");
  check_cuda(cudaMalloc(&B->d_parts, sizeof(PartDev) * std::max<long long>(B->nchunks, 1) * (B->threads / 32)),
             "batch partials");
  check_cuda(cudaMemcpyAsync(B->d_items, items.data(), sizeof(ItemDev) * B->n, cudaMemcpyHostToDevice, s), "items");
  check_cuda(cudaMemcpyAsync(B->d_chunks, chunks.data(), sizeof(ChunkDev) * B->nchunks, cudaMemcpyHostToDevice, s),
             "chunks");
  check_cuda(cudaStreamSynchronize(s), "batch tables");
}

std::string shape_class(const nca_batch* B) {
  long long bytes = 0, n16 = 0;
  for (auto& it : B->items) {
    bytes += it.length * (it.dtype == NCA_FLOAT32 ? 4 : 2);
    if (it.dtype != NCA_FLOAT32) ++n16;
  }
  const int lb = bytes > 0 ? (int)std::log2((double)bytes) : 0;
  const int ln = B->n > 0 ? (int)std::log2((double)B->n) : 0;
  const int mix = B->n > 0 ? (int)(4.0 * n16 / B->n + 0.5) : 0;
  std::ostringstream os;
  os << "batch_b" << lb << "_n" << ln << "_m" << mix;
  return os.str();
}

// lines "<shape class> <chunk bytes> <threads> <slab bytes> <ctas per sm>"
std::string tune_file() { return nca::jit_cache_dir() + "/batch_tune_ws.txt"; }

bool schedule_ok(long long cb, int th, int slab, int cps) {
  return cb >= (64ll << 10) && (th == 256 || th == 512) && (slab == 8192 || slab == 16384 || slab == 32768) &&
         cps >= 1 && cps <= 8 && (long long)cps * NSLAB * slab <= 200ll * 1024 && (th + 32) * cps <= 2048;
}

bool load_tuned(nca_batch* B) {
  std::ifstream f(tune_file());
  std::string key;
  long long cb;
  int th, sl, cps;
  bool found = false;
  while (f >> key >> cb >> th >> sl >> cps) {
    if (key == B->shape_class && schedule_ok(cb, th, sl, cps)) {
      B->chunk_bytes = cb; B->threads = th; B->slab = sl; B->ctas_per_sm = cps;
      found = true;
    }
  }
  return found;
}

void store_tuned(const nca_batch* B) {
  std::ofstream f(tune_file(), std::ios::app);
  if (f) f << B->shape_class << " " << B->chunk_bytes << " " << B->threads << " " << B->slab << " "
           << B->ctas_per_sm << "\n";
}

}  // namespace

extern "C" {

int32_t nca_batch_create(const nca_batch_item* items, int32_t n_items, nca_batch** out, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!out) fail(NCA_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (n_items < 0 || (n_items > 0 && !items)) fail(NCA_ERR_INVALID, "bad item list");
    if (n_items > (1 << 30)) fail(NCA_ERR_LIMIT, "too many items");
    for (int i = 0; i < n_items; ++i) {
      const auto& it = items[i];
      if (it.dtype != NCA_FLOAT32 && it.dtype != NCA_BFLOAT16 && it.dtype != NCA_FLOAT16)
        fail(NCA_ERR_DTYPE, "item %d: batched reductions take float32, bfloat16 or float16", i);
      if (it.length < 0) fail(NCA_ERR_INVALID, "item %d: negative length", i);
      if (it.length > 0 && !it.data) fail(NCA_ERR_INVALID, "item %d: null data", i);
    }
    auto* B = new nca_batch();
    try {
      B->n = n_items;
      B->dev = current_device();
      B->items.assign(items, items + n_items);
      B->shape_class = shape_class(B);
      load_tuned(B);
      // NCA_BATCH_SCHEDULE="<chunk bytes>,<threads>,<slab bytes>,<CTAs per SM>" overrides the tuned schedule
      if (const char* e = getenv("NCA_BATCH_SCHEDULE")) {
        long long cb = 0;
        int th = 0, sl = 0, cps = 0;
        if (sscanf(e, "%lld,%d,%d,%d", &cb, &th, &sl, &cps) == 4 && schedule_ok(cb, th, sl, cps)) {
          B->chunk_bytes = cb; B->threads = th; B->slab = sl; B->ctas_per_sm = cps;
        }
      }
      build_chunks(B, (cudaStream_t)stream);
    } catch (...) {
      nca_batch_destroy(B);
      throw;
    }
    *out = B;
  });
}

int32_t nca_batch_reduce(nca_batch* B, nca_batch_result* results, void* stream) {
  return nca::guarded([&] {
    if (!B || !results) nca::fail(NCA_ERR_INVALID, "null argument");
    launch_persistent(B, results, (cudaStream_t)stream);
  });
}

int32_t nca_batch_reduce_graph(nca_batch* B, nca_batch_result* results, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!B || !results) fail(NCA_ERR_INVALID, "null argument");
    if (!B->graph || B->graph_results != results) {
      if (B->graph) { cudaGraphExecDestroy(B->graph); B->graph = nullptr; }
      if (!B->capture_stream) check_cuda(cudaStreamCreateWithFlags(&B->capture_stream, cudaStreamNonBlocking), "stream");
      check_cuda(cudaStreamBeginCapture(B->capture_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
      try {
        launch_persistent(B, results, B->capture_stream);
      } catch (...) {
        cudaGraph_t g;
        cudaStreamEndCapture(B->capture_stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      cudaGraph_t g = nullptr;
      check_cuda(cudaStreamEndCapture(B->capture_stream, &g), "end capture");
      cudaError_t e = cudaGraphInstantiate(&B->graph, g, 0);
      cudaGraphDestroy(g);
      check_cuda(e, "graph instantiate");
      B->graph_results = results;
    }
    check_cuda(cudaGraphLaunch(B->graph, (cudaStream_t)stream), "graph launch");
    count_launch();
  });
}

int32_t nca_batch_reduce_plain(nca_batch* B, nca_batch_result* results, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!B || !results) fail(NCA_ERR_INVALID, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    if (B->n == 0) return;
    plain_init_kernel<<<(B->n + 255) / 256, 256, 0, s>>>(results, B->n);
    count_launch();
    const int sms = sm_count(B->dev);
    for (int i = 0; i < B->n; ++i) {
      const auto& it = B->items[i];
      const int grid = (int)std::max<long long>(1, std::min<long long>((it.length + 2047) / 2048, 2ll * sms));
      double* r = &results[i].sum;
      plain_kernel<0><<<grid, 256, 0, s>>>(it.data, it.length, it.dtype, r);
      plain_kernel<1><<<grid, 256, 0, s>>>(it.data, it.length, it.dtype, &results[i].max);
      plain_kernel<2><<<grid, 256, 0, s>>>(it.data, it.length, it.dtype, &results[i].sum_sq_m);
      plain_mean_kernel<<<1, 1, 0, s>>>(results, (const ItemDev*)B->d_items, i);
      count_launch(4);
    }
    check_cuda(cudaGetLastError(), "plain launches");
  });
}

int32_t nca_batch_autotune(nca_batch* B, nca_batch_result* results, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!B || !results) fail(NCA_ERR_INVALID, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    struct Cand { long long cb; int th, sl, cps; };
    std::vector<Cand> cands;
    check_cuda(cudaFuncSetAttribute(batch_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    NSLAB * 32768 + 16 * NSLAB),
               "batch smem");
    for (long long cb : {256ll << 10, 512ll << 10, 1024ll << 10})
      for (int sl : {8192, 16384, 32768})
        for (int cps : {2, 3, 4}) {
          int resident = 0;   // CTAs of this shape that fit on an SM at once
          check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, batch_persistent_kernel, 256 + 32,
                                                                   NSLAB * sl + 16 * NSLAB),
                     "occupancy");
          if (schedule_ok(cb, 256, sl, cps) && resident >= cps) cands.push_back({cb, 256, sl, cps});
        }
    if (cands.empty()) cands.push_back({256ll << 10, 256, 16384, 3});
    cudaEvent_t e0, e1;
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    Cand bestc = cands[0];
    for (const auto& c : cands) {
      B->chunk_bytes = c.cb; B->threads = c.th; B->slab = c.sl; B->ctas_per_sm = c.cps;
      build_chunks(B, s);
      launch_persistent(B, results, s);   // warm-up
      check_cuda(cudaEventRecord(e0, s), "record");
      for (int r = 0; r < 3; ++r) launch_persistent(B, results, s);
      check_cuda(cudaEventRecord(e1, s), "record");
      check_cuda(cudaEventSynchronize(e1), "sync");
      float ms = 0.f;
      check_cuda(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
      if (ms < best) { best = ms; bestc = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->chunk_bytes = bestc.cb; B->threads = bestc.th; B->slab = bestc.sl; B->ctas_per_sm = bestc.cps;
    build_chunks(B, s);
    store_tuned(B);
  });
}

int32_t nca_batch_schedule(const nca_batch* B, int64_t* chunk, int32_t* threads, int32_t* items_per_thread,
                           int32_t* ctas) {
  return nca::guarded([&] {
    if (!B) nca::fail(NCA_ERR_INVALID, "null batch");
    if (chunk) *chunk = B->chunk_bytes;
    if (threads) *threads = B->threads;
    if (items_per_thread) *items_per_thread = B->slab / (16 * B->threads);   // 16-byte vectors per thread per slab
    if (ctas) *ctas = (int32_t)std::min<long long>(B->nchunks, (long long)nca::sm_count(B->dev) * B->ctas_per_sm);
  });
}

int32_t nca_batch_status(nca_batch* B, int32_t* status, void* stream) {
  return nca::guarded([&] {
    if (!B || !status) nca::fail(NCA_ERR_INVALID, "null argument");
    // NCA_ERR_TIMEOUT if a bounded wait of the pipeline gave up (read and cleared)
    cudaStream_t s = (cudaStream_t)stream;
    int v = 0;
    nca::check_cuda(cudaMemcpyAsync(&v, B->d_status, sizeof(int), cudaMemcpyDeviceToHost, s), "batch status");
    nca::check_cuda(cudaMemsetAsync(B->d_status, 0, sizeof(int), s), "batch status");
    nca::check_cuda(cudaStreamSynchronize(s), "batch stream");
    *status = v;
  });
}

void nca_batch_destroy(nca_batch* B) {
  if (!B) return;
  free_tables(B);
  if (B->d_items) cudaFree(B->d_items);
  if (B->d_done) cudaFree(B->d_done);
  if (B->d_status) cudaFree(B->d_status);
  if (B->capture_stream) cudaStreamDestroy(B->capture_stream);
  delete B;
}

}  // extern "C"
