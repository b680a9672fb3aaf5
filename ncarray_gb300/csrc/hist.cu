// 2-D histogram binning of float32 (x, y) points with optional float32 weights.
//
// The reference has only an internal scatter-add (`dest[idx[i]] += src[i]`,
// src/lib/ncarray/device/kernels.cuh:660-680, host/elementwise.hh:482-505) and
// no public histogram API; this file adds one.
// Binning rule (the oracle restates it bit for bit): in float32,
//   fx = floor((x - x_lo) * sx),  sx = (float)(nbx / (x_hi - x_lo))   (same for y)
// and the point is kept only if 0 <= fx < nbx and 0 <= fy < nby (NaN dropped).
// counts (uint64) are exact; weights are summed per bin with float32 partial
// sums whose rounding errors are collected exactly (compensated), combined in
// float64, and added to the float32 output once at the end.
//
// A bin grid of more than a few thousand bins does not fit in shared memory
// and global atomics on it run at the L2 atomic rate, far below HBM speed.
// The partitioned path therefore reads the points once and the much smaller
// per-tile records once:
//   1. sample: one block of 1024 points in 32 estimates how many points fall
//      in each tile of TB consecutive bins; each tile gets a bucket with 25 %
//      slack (the total is bounded, so the scratch is sized on the host);
//   2. scatter: every CTA bins a chunk of points, ranks them per tile with
//      shared-memory atomics, orders the chunk's (bin within tile: uint16,
//      weight: float32) records by tile in shared memory and appends each
//      tile's run to its bucket with coalesced stores (one global atomic per
//      tile and CTA reserves the space); records that do not fit in their
//      bucket are added with global atomics directly;
//   3. accumulate: a persistent grid splits the concatenated buckets into
//      equal record ranges; a CTA counts each tile piece of its range into a
//      shared-memory copy of the tile (uint32 counts, float32 sums and
//      compensation terms: the value returned by the float atomic gives the
//      exact rounding error of each addition via TwoSum) and stores the piece;
//   4. combine: every bin adds its tile's pieces in a fixed order (uint64
//      counts, float64 weights) to the outputs.
// Small inputs and grids with too many tiles use direct global atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <string>

#include "common.hpp"
#include "mbar.cuh"

namespace {

constexpr int THREADS = 256;
constexpr int TB_LOG2 = 14;
constexpr int TB = 1 << TB_LOG2;        // bins per tile (local index fits in uint16)
constexpr int MAX_TILES = 256;          // partitioned path limit (4 Mi bins; tile index fits in uint8)
constexpr int SAMPLE = 32;              // 1 block of 1024 points in SAMPLE is counted in pass 1
constexpr int CHUNK = 2048;             // points per chunk in the scatter pass
constexpr int PER_THREAD = CHUNK / THREADS;
static_assert(MAX_TILES == THREADS, "the scatter pass scans one tile count per thread");
constexpr int ACC_THREADS = 1024;
constexpr int NSUB = 1;                 // sub-buckets per tile (by scatter CTA index)
constexpr int SCAN_THREADS = 1024;      // one-block scans over <= 4 * SCAN_THREADS buckets
constexpr int SLACK = 2048;             // records of slack per bucket
constexpr int FPAD = 16;                // fill counters 128 bytes apart (uint64)
constexpr int EPAD = 32;                // estimate counters 128 bytes apart (uint32)
static_assert(MAX_TILES * NSUB <= 4 * SCAN_THREADS, "bucket scan size");

constexpr unsigned long long kWaitNs = 2000000000ull;   // bound of every mbarrier wait

static __device__ int g_hist_status;   // NCA_ERR_TIMEOUT after a wait that ran out

struct Bins {
  float xl, yl, sx, sy, fnx, fny;
  int nbx, nby;
};

__device__ __forceinline__ int bin_of(const Bins& B, float x, float y) {
  const float fx = floorf(__fmul_rn(__fsub_rn(x, B.xl), B.sx));
  const float fy = floorf(__fmul_rn(__fsub_rn(y, B.yl), B.sy));
  if (!(fx >= 0.0f && fx < B.fnx && fy >= 0.0f && fy < B.fny)) return -1;
  return (int)fy * B.nbx + (int)fx;
}

// The same bin for grids of at most 2^22 bins (the partitioned path), without
// float-to-int conversions: the floor of v in [0, 2^23) is the low mantissa
// bits of v + 2^23 rounded toward zero, and v >= 0 / v < n (integer n) accept
// exactly the values whose floor floorf(v) does.
constexpr unsigned NO_BIN = 0xffffffffu;
__device__ __forceinline__ unsigned tile_bin_of(const Bins& B, float x, float y) {
  const float fx = __fmul_rn(__fsub_rn(x, B.xl), B.sx);
  const float fy = __fmul_rn(__fsub_rn(y, B.yl), B.sy);
  if (!(fx >= 0.0f && fx < B.fnx && fy >= 0.0f && fy < B.fny)) return NO_BIN;
  const unsigned ix = (unsigned)__float_as_int(__fadd_rz(fx, 8388608.0f)) & 0x7fffffu;
  const unsigned iy = (unsigned)__float_as_int(__fadd_rz(fy, 8388608.0f)) & 0x7fffffu;
  return iy * (unsigned)B.nbx + ix;
}

// ---- direct path: global atomics per point -------------------------------------
template <bool WEIGHTED>
__global__ void __launch_bounds__(THREADS)
hist2d_direct_kernel(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ w,
                     long long n, Bins B, unsigned long long* __restrict__ counts, double* __restrict__ wacc) {
  const long long stride = (long long)gridDim.x * THREADS;
  for (long long i = (long long)blockIdx.x * THREADS + threadIdx.x; i < n; i += stride) {
    const int b = bin_of(B, __ldcs(x + i), __ldcs(y + i));
    if (b >= 0) {
      atomicAdd(counts + b, 1ull);
      if (WEIGHTED) atomicAdd(wacc + b, (double)__ldcs(w + i));
    }
  }
}

__global__ void __launch_bounds__(THREADS) wsum_finish_kernel(const double* __restrict__ wacc, float* __restrict__ wsum,
                                                               long long nb) {
  for (long long i = (long long)blockIdx.x * THREADS + threadIdx.x; i < nb; i += (long long)gridDim.x * THREADS)
    wsum[i] = __double2float_rn((double)wsum[i] + wacc[i]);
}

// Exclusive prefix sums of n <= SCAN_THREADS * 4 values v(i) by one block of
// SCAN_THREADS threads: out[i] for i < n and out[n] = total.
template <class F>
__device__ __forceinline__ void block_scan(int n, F v, long long* __restrict__ out) {
  __shared__ long long sc[SCAN_THREADS];
  const int t = threadIdx.x;
  long long a[4];
  long long sum = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = t * 4 + j;
    a[j] = i < n ? v(i) : 0;
    sum += a[j];
  }
  sc[t] = sum;
  __syncthreads();
  for (int d = 1; d < SCAN_THREADS; d <<= 1) {
    const long long u = t >= d ? sc[t - d] : 0;
    __syncthreads();
    sc[t] += u;
    __syncthreads();
  }
  long long run = sc[t] - sum;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = t * 4 + j;
    if (i < n) out[i] = run;
    run += a[j];
  }
  if (t == SCAN_THREADS - 1) out[n] = sc[t];
}

// ---- pass 1: sampled tile counts -------------------------------------------------
__global__ void __launch_bounds__(THREADS)
tile_sample_kernel(const float* __restrict__ x, const float* __restrict__ y, long long n, Bins B, int ntiles,
                   unsigned* __restrict__ est) {
  __shared__ unsigned cnt[MAX_TILES];
  for (int t = threadIdx.x; t < ntiles; t += THREADS) cnt[t] = 0;
  __syncthreads();
  // the sample: every SAMPLE-th block of 1024 consecutive points
  const long long nblk = (n + 1023) / 1024;
  const long long ns = ((nblk + SAMPLE - 1) / SAMPLE) * 1024;
  for (long long s = (long long)blockIdx.x * THREADS + threadIdx.x; s < ns; s += (long long)gridDim.x * THREADS) {
    const long long i = (s / 1024) * SAMPLE * 1024 + (s % 1024);
    if (i >= n) continue;
    const int b = bin_of(B, __ldg(x + i), __ldg(y + i));
    if (b >= 0) atomicAdd(&cnt[b / TB], 1u);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < ntiles; t += THREADS)
    if (cnt[t]) atomicAdd(est + (long long)t * EPAD, cnt[t]);
}

__device__ __forceinline__ long long bucket_cap(const unsigned* __restrict__ est, int v) {
  const long long e = est[(long long)(v / NSUB) * EPAD];
  return ((e * (SAMPLE * 5 / 4) / NSUB + 7) & ~7ll) + SLACK;
}

// capacity and offset of every bucket (tile t, sub-bucket u) = t * NSUB + u;
// capacities are multiples of 8 records so every bucket starts 16-byte aligned
__global__ void __launch_bounds__(SCAN_THREADS)
tile_plan_kernel(const unsigned* __restrict__ est, int nv, long long* __restrict__ off,
                 long long* __restrict__ cap, unsigned long long* __restrict__ fill) {
  block_scan(nv, [&](int v) { return bucket_cap(est, v); }, off);
  for (int v = threadIdx.x; v < nv; v += SCAN_THREADS) {
    cap[v] = bucket_cap(est, v);
    fill[(long long)v * FPAD] = 0;
  }
}

// ---- pass 2: scatter points into buckets ------------------------------------------
// A persistent grid walks the chunks of CHUNK points; the next chunk of x, y
// (and w) is fetched by bulk copies into the other half of a double buffer
// while the current one is binned. Waits are bounded (2 s of %globaltimer):
// on a timeout the CTA records NCA_ERR_TIMEOUT, waits for its copies in
// flight and stops. CTA c appends to sub-bucket c % NSUB of every tile.

using nca_dev::mbar_wait;

__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
}

template <bool WEIGHTED>
__host__ __device__ constexpr int scatter_smem() {
  return 2 * (WEIGHTED ? 3 : 2) * CHUNK * 4 + 16;
}

template <bool WEIGHTED>
__global__ void __launch_bounds__(THREADS, 3)
tile_scatter_kernel(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ w,
                    long long n, Bins B, int ntiles, const long long* __restrict__ off,
                    const long long* __restrict__ cap, unsigned long long* __restrict__ fill,
                    unsigned short* __restrict__ rec_bin, float* __restrict__ rec_w,
                    unsigned long long* __restrict__ counts, double* __restrict__ wacc) {
  constexpr int NA = WEIGHTED ? 3 : 2;              // arrays fetched per chunk
  constexpr uint32_t ABYTES = CHUNK * 4;
  extern __shared__ __align__(128) unsigned char sm[];
  const float* buf = reinterpret_cast<const float*>(sm);   // [2][NA][CHUNK]
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sm);
  const uint32_t bbase = sbase + 2 * NA * ABYTES;          // two mbarriers
  __shared__ unsigned cnt[MAX_TILES];
  __shared__ unsigned loff[MAX_TILES];      // start of each tile's run in the staged chunk
  __shared__ unsigned wpre[THREADS / 32];
  __shared__ uint2 tinfo[MAX_TILES];        // (record index - staged position, end of the stored part)
  __shared__ unsigned srec[CHUNK];          // the chunk's bins ordered by tile
  __shared__ float sw[WEIGHTED ? CHUNK : 1];
  const long long nfull = n / CHUNK, nchunks = (n + CHUNK - 1) / CHUNK;
  const int sub = (int)(blockIdx.x % NSUB);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bbase) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bbase + 8) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](long long ch, int b) {
    const uint32_t bar = bbase + 8 * b, dst = sbase + (uint32_t)(b * NA) * ABYTES;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(NA * ABYTES) : "memory");
    bulk_load(dst, x + ch * CHUNK, ABYTES, bar);
    bulk_load(dst + ABYTES, y + ch * CHUNK, ABYTES, bar);
    if (WEIGHTED) bulk_load(dst + 2 * ABYTES, w + ch * CHUNK, ABYTES, bar);
  };
  long long ch = blockIdx.x;
  if (threadIdx.x == 0 && ch < nfull) issue(ch, 0);
  int it = 0;
  bool failed = false;
  for (; ch < nchunks; ch += gridDim.x, ++it) {
    const int b = it & 1;
    const long long nxt = ch + gridDim.x;
    // buffer b ^ 1 was released by the barrier that ended the previous iteration
    if (threadIdx.x == 0 && nxt < nfull) issue(nxt, b ^ 1);
    for (int t = threadIdx.x; t < ntiles; t += THREADS) cnt[t] = 0;
    const bool full = ch < nfull;
    const bool ok = !full || mbar_wait(bbase + 8 * b, (uint32_t)((it >> 1) & 1), kWaitNs);
    if (__syncthreads_or(ok ? 0 : 1)) { failed = true; break; }
    const long long c0 = ch * CHUNK;
    const float* bx = buf + (size_t)(b * NA) * CHUNK;
    unsigned bins[PER_THREAD];
    float ws[PER_THREAD];
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
      const int li = threadIdx.x + k * THREADS;
      ws[k] = 0.f;
      if (full) {
        bins[k] = tile_bin_of(B, bx[li], bx[CHUNK + li]);
        if (WEIGHTED) ws[k] = bx[2 * CHUNK + li];
      } else if (c0 + li < n) {
        bins[k] = tile_bin_of(B, __ldcs(x + c0 + li), __ldcs(y + c0 + li));
        if (WEIGHTED) ws[k] = __ldcs(w + c0 + li);
      } else {
        bins[k] = NO_BIN;
      }
    }
    // rank within the CTA's run of the tile (lanes of a warp on the same
    // counter are serialised by the shared-memory unit, one issue slot each)
    unsigned rank[PER_THREAD];
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) rank[k] = bins[k] != NO_BIN ? atomicAdd(&cnt[bins[k] >> TB_LOG2], 1u) : 0u;
    __syncthreads();
    // exclusive scan of the tile counts (ntiles <= MAX_TILES == THREADS); the
    // thread of tile t then reserves the tile's run in its bucket
    {
      const int t = threadIdx.x, lane = t & 31, wp = t >> 5;
      const unsigned v0 = t < ntiles ? cnt[t] : 0u;
      unsigned v = v0;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned u = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += u;
      }
      if (lane == 31) wpre[wp] = v;
      __syncthreads();
      if (wp == 0) {
        unsigned q = lane < THREADS / 32 ? wpre[lane] : 0u;
        const unsigned q0 = q;
#pragma unroll
        for (int d = 1; d < THREADS / 32; d <<= 1) {
          const unsigned u = __shfl_up_sync(0xffffffffu, q, d);
          if (lane >= d) q += u;
        }
        if (lane < THREADS / 32) wpre[lane] = q - q0;
      }
      __syncthreads();
      const unsigned lo = v - v0 + wpre[wp];
      loff[t] = lo;
      if (v0) {
        // positions [p, p + cnt) are this CTA's; the part below the capacity is
        // always written, so every position below min(fill, cap) holds a record
        const int vb = t * NSUB + sub;
        const unsigned long long p = atomicAdd(fill + (long long)vb * FPAD, (unsigned long long)v0);
        const long long room = cap[vb] - (long long)p;
        const unsigned avail = room <= 0 ? 0u : (room >= (long long)v0 ? v0 : (unsigned)room);
        tinfo[t] = make_uint2((unsigned)(off[vb] + (long long)p) - lo, lo + avail);
      }
    }
    __syncthreads();
    // stage the bins in tile order
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
      if (bins[k] == NO_BIN) continue;
      const unsigned j = loff[bins[k] >> TB_LOG2] + rank[k];
      srec[j] = bins[k];
      if (WEIGHTED) sw[j] = ws[k];
    }
    __syncthreads();
    // consecutive threads write consecutive records of a tile's run; a record
    // past its bucket's capacity is added with global atomics instead
    const unsigned total = loff[ntiles - 1] + cnt[ntiles - 1];
#pragma unroll
    for (int k = 0; k < PER_THREAD; ++k) {
      const unsigned j = threadIdx.x + k * THREADS;
      if (j >= total) break;
      const unsigned bn = srec[j];
      const uint2 ti = tinfo[bn >> TB_LOG2];
      if (j < ti.y) {
        rec_bin[ti.x + j] = (unsigned short)(bn & (TB - 1));
        if (WEIGHTED) rec_w[ti.x + j] = sw[j];
      } else {
        atomicAdd(counts + bn, 1ull);
        if (WEIGHTED) atomicAdd(wacc + bn, (double)sw[j]);
      }
    }
    __syncthreads();
  }
  if (failed && threadIdx.x == 0) {
    atomicExch(&g_hist_status, (int)NCA_ERR_TIMEOUT);
    // copies in flight: buffer it & 1 (this chunk) and the prefetch of the next
    const int b = it & 1;
    if (ch < nfull) mbar_wait(bbase + 8 * b, (uint32_t)((it >> 1) & 1), kWaitNs / 2);
    if (ch + gridDim.x < nfull) mbar_wait(bbase + 8 * (b ^ 1), (uint32_t)(((it + 1) >> 1) & 1), kWaitNs / 2);
  }
}

// stored records per bucket and their exclusive prefix sum PV (PV[nv] = total)
__global__ void __launch_bounds__(SCAN_THREADS)
tile_prefix_kernel(int nv, const long long* __restrict__ cap, const unsigned long long* __restrict__ fill,
                   long long* __restrict__ PV) {
  block_scan(nv, [&](int v) {
    const long long ft = (long long)fill[(long long)v * FPAD];
    return ft < cap[v] ? ft : cap[v];
  }, PV);
}

// ---- pass 3: per-tile shared-memory histograms of record ranges -------------------
// CTA g takes records [R g / G, R (g + 1) / G) of the concatenated buckets
// (bucket v holds positions [PV[v], PV[v+1]), tile t the buckets t * NSUB ..
// t * NSUB + NSUB - 1); its piece of tile t is stored in partial slot g + t,
// which is unique because both g and t grow along the concatenation.
__device__ __forceinline__ long long range_start(long long R, int g, int G) { return R * g / G; }

template <bool WEIGHTED>
__device__ __forceinline__ void acc_record(unsigned* c, float* s, float* e, unsigned l, float wv) {
  atomicAdd(&c[l], 1u);
  if (WEIGHTED) {
    const float old = atomicAdd(&s[l], wv);       // s[l] became fl(old + wv)
    const float sum = __fadd_rn(old, wv);
    const float bb = __fsub_rn(sum, old);
    const float err = __fadd_rn(__fsub_rn(old, __fsub_rn(sum, bb)), __fsub_rn(wv, bb));
    if (err != 0.f) atomicAdd(&e[l], err);
  }
}

template <bool WEIGHTED>
__device__ __forceinline__ void acc_vec(unsigned* c, float* s, float* e, uint4 q, float4 w0, float4 w1) {
  acc_record<WEIGHTED>(c, s, e, q.x & 0xffffu, w0.x);
  acc_record<WEIGHTED>(c, s, e, q.x >> 16, w0.y);
  acc_record<WEIGHTED>(c, s, e, q.y & 0xffffu, w0.z);
  acc_record<WEIGHTED>(c, s, e, q.y >> 16, w0.w);
  acc_record<WEIGHTED>(c, s, e, q.z & 0xffffu, w1.x);
  acc_record<WEIGHTED>(c, s, e, q.z >> 16, w1.y);
  acc_record<WEIGHTED>(c, s, e, q.w & 0xffffu, w1.z);
  acc_record<WEIGHTED>(c, s, e, q.w >> 16, w1.w);
}

template <bool WEIGHTED>
__device__ __forceinline__ void acc_range(unsigned* c, float* s, float* e, const unsigned short* __restrict__ rec_bin,
                                          const float* __restrict__ rec_w, long long a, long long b) {
  // records [a, b) of the record arrays; bucket starts are multiples of 8
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  long long a8 = (a + 7) & ~7ll;
  if (a8 > b) a8 = b;
  const long long nv = (b - a8) >> 3, b8 = a8 + (nv << 3);
  for (long long r = a + threadIdx.x; r < a8; r += ACC_THREADS)
    acc_record<WEIGHTED>(c, s, e, rec_bin[r], WEIGHTED ? rec_w[r] : 0.f);
  for (long long r = b8 + threadIdx.x; r < b; r += ACC_THREADS)
    acc_record<WEIGHTED>(c, s, e, rec_bin[r], WEIGHTED ? rec_w[r] : 0.f);
  const uint4* vb = reinterpret_cast<const uint4*>(rec_bin + a8);
  const float4* vw = reinterpret_cast<const float4*>(WEIGHTED ? rec_w + a8 : nullptr);
  long long v = threadIdx.x;
  for (; v + ACC_THREADS < nv; v += 2 * ACC_THREADS) {
    const uint4 q0 = __ldcs(vb + v), q1 = __ldcs(vb + v + ACC_THREADS);
    float4 w0 = z4, w1 = z4, w2 = z4, w3 = z4;
    if (WEIGHTED) {
      w0 = __ldcs(vw + 2 * v);
      w1 = __ldcs(vw + 2 * v + 1);
      w2 = __ldcs(vw + 2 * (v + ACC_THREADS));
      w3 = __ldcs(vw + 2 * (v + ACC_THREADS) + 1);
    }
    acc_vec<WEIGHTED>(c, s, e, q0, w0, w1);
    acc_vec<WEIGHTED>(c, s, e, q1, w2, w3);
  }
  if (v < nv) {
    const uint4 q0 = __ldcs(vb + v);
    float4 w0 = z4, w1 = z4;
    if (WEIGHTED) {
      w0 = __ldcs(vw + 2 * v);
      w1 = __ldcs(vw + 2 * v + 1);
    }
    acc_vec<WEIGHTED>(c, s, e, q0, w0, w1);
  }
}

template <bool WEIGHTED>
__global__ void __launch_bounds__(ACC_THREADS)
tile_accumulate_kernel(int nv, const long long* __restrict__ off, const long long* __restrict__ PV,
                       const unsigned short* __restrict__ rec_bin, const float* __restrict__ rec_w,
                       unsigned* __restrict__ pc, float* __restrict__ ps, float* __restrict__ pe) {
  extern __shared__ __align__(128) unsigned char sm[];
  unsigned* c = reinterpret_cast<unsigned*>(sm);
  float* s = reinterpret_cast<float*>(sm + TB * 4);
  float* e = reinterpret_cast<float*>(sm + TB * 8);
  const int G = gridDim.x, g = blockIdx.x;
  const long long R = PV[nv];
  const long long S1 = range_start(R, g + 1, G);
  long long pos = range_start(R, g, G);
  int v = 0;
  while (pos < S1) {
    while (PV[v + 1] <= pos) ++v;                // pos < R = PV[nv], so v < nv
    const int t = v / NSUB;
    const long long tend = PV[(t + 1) * NSUB] < S1 ? PV[(t + 1) * NSUB] : S1;
    for (int i = threadIdx.x; i < TB; i += ACC_THREADS) {
      c[i] = 0u;
      if (WEIGHTED) { s[i] = 0.f; e[i] = 0.f; }
    }
    __syncthreads();
    // the sub-buckets of tile t inside [pos, tend)
    while (pos < tend) {
      while (PV[v + 1] <= pos) ++v;
      const long long end = PV[v + 1] < tend ? PV[v + 1] : tend;
      acc_range<WEIGHTED>(c, s, e, rec_bin, rec_w, off[v] + (pos - PV[v]), off[v] + (end - PV[v]));
      pos = end;
    }
    __syncthreads();
    const long long slot = (long long)(g + t) * TB;
    for (int i = threadIdx.x; i < TB; i += ACC_THREADS) {
      pc[slot + i] = c[i];
      if (WEIGHTED) {
        ps[slot + i] = s[i];
        pe[slot + i] = e[i];
      }
    }
    __syncthreads();
  }
}

// ---- pass 4: add the pieces of every bin's tile to the outputs ----------------------
template <bool WEIGHTED>
__global__ void __launch_bounds__(THREADS)
tile_combine_kernel(long long nbins, int nv, int G, const long long* __restrict__ PV,
                    const unsigned* __restrict__ pc, const float* __restrict__ ps, const float* __restrict__ pe,
                    const double* __restrict__ wacc, unsigned long long* __restrict__ counts,
                    float* __restrict__ wsum) {
  const long long R = PV[nv];
  for (long long bin = (long long)blockIdx.x * THREADS + threadIdx.x; bin < nbins;
       bin += (long long)gridDim.x * THREADS) {
    const int t = (int)(bin / TB);
    const long long i = bin - (long long)t * TB;
    const long long lo = PV[t * NSUB], hi = PV[(t + 1) * NSUB];
    unsigned long long cn = 0;
    double wv = 0.0;
    if (hi > lo) {
      // the CTAs whose ranges meet [lo, hi), in order: from the one holding lo
      // to the one holding hi - 1 (every CTA range is non-empty when R >= G)
      int g = (int)(lo * G / R);
      while (g > 0 && range_start(R, g, G) > lo) --g;
      while (g + 1 < G && range_start(R, g + 1, G) <= lo) ++g;
      int gl = (int)((hi - 1) * G / R);
      while (gl + 1 < G && range_start(R, gl + 1, G) <= hi - 1) ++gl;
      for (; g <= gl; ++g) {
        if (R < G && range_start(R, g, G) == range_start(R, g + 1, G)) continue;
        const long long slot = (long long)(g + t) * TB + i;
        cn += pc[slot];
        if (WEIGHTED) wv += (double)ps[slot] + (double)pe[slot];
      }
    }
    counts[bin] += cn;
    if (WEIGHTED) wsum[bin] = __double2float_rn((double)wsum[bin] + (wacc[bin] + wv));
  }
}

template <typename T>
T* carve(char*& p, long long count) {
  T* r = reinterpret_cast<T*>(p);
  p += ((size_t)count * sizeof(T) + 255) & ~(size_t)255;
  return r;
}

}  // namespace

namespace nca {
// NCA_OK or the error a histogram kernel recorded since the last read (cleared)
int hist_read_status(cudaStream_t s) {
  int v = 0, zero = 0;
  check_cuda(cudaMemcpyFromSymbolAsync(&v, g_hist_status, sizeof(int), 0, cudaMemcpyDeviceToHost, s), "status read");
  check_cuda(cudaMemcpyToSymbolAsync(g_hist_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s), "status clear");
  check_cuda(cudaStreamSynchronize(s), "status sync");
  return v;
}
}  // namespace nca

extern "C" int32_t nca_hist2d(const float* x, const float* y, const float* w, int64_t n, int32_t nbx, int32_t nby,
                              double x_lo, double x_hi, double y_lo, double y_hi, uint64_t* counts, float* wsum,
                              void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (n < 0) fail(NCA_ERR_INVALID, "negative point count");
    if (nbx <= 0 || nby <= 0 || (int64_t)nbx * nby > (1ll << 30)) fail(NCA_ERR_SHAPE, "bin grid %d x %d out of range", nbx, nby);
    if (!(x_hi > x_lo) || !(y_hi > y_lo)) fail(NCA_ERR_INVALID, "empty bin range");
    if (!counts) fail(NCA_ERR_INVALID, "null counts");
    if (n > 0 && (!x || !y)) fail(NCA_ERR_INVALID, "null coordinates");
    if ((w == nullptr) != (wsum == nullptr)) fail(NCA_ERR_INVALID, "weights and wsum go together");
    if (n == 0) return;
    Bins B;
    B.xl = (float)x_lo;
    B.yl = (float)y_lo;
    B.sx = (float)((double)nbx / (x_hi - x_lo));
    B.sy = (float)((double)nby / (y_hi - y_lo));
    B.fnx = (float)nbx;
    B.fny = (float)nby;
    B.nbx = nbx;
    B.nby = nby;
    cudaStream_t s = (cudaStream_t)stream;
    const int dev = current_device();
    const int sms = sm_count(dev);
    const long long nbins = (long long)nbx * nby;
    const long long ntiles = (nbins + TB - 1) / TB;
    const bool weighted = w != nullptr;
    unsigned long long* cnt = (unsigned long long*)counts;
    // the bulk copies of the partitioned path need 16-byte aligned point arrays
    const bool aligned = ((uintptr_t)x % 16 == 0) && ((uintptr_t)y % 16 == 0) && (!weighted || (uintptr_t)w % 16 == 0);
    // NCA_HIST_PATH=direct forces the direct path (tests and measurements)
    const char* hp = getenv("NCA_HIST_PATH");
    const std::string path = hp ? hp : "";
    if (ntiles > MAX_TILES || n < (1 << 20) || !aligned || path == "direct") {
      StreamScratch acc(weighted ? (size_t)nbins * sizeof(double) : 0, s);
      double* wacc = (double*)acc.ptr;
      if (weighted) check_cuda(cudaMemsetAsync(wacc, 0, (size_t)nbins * sizeof(double), s), "memset weights");
      const long long grid = std::min<long long>((n + THREADS - 1) / THREADS, (long long)sms * 8);
      if (weighted) hist2d_direct_kernel<true><<<(unsigned)grid, THREADS, 0, s>>>(x, y, w, n, B, cnt, wacc);
      else hist2d_direct_kernel<false><<<(unsigned)grid, THREADS, 0, s>>>(x, y, nullptr, n, B, cnt, nullptr);
      check_cuda(cudaGetLastError(), "hist2d launch");
      count_launch();
      if (weighted) {
        wsum_finish_kernel<<<(unsigned)std::min<long long>((nbins + THREADS - 1) / THREADS, (long long)sms * 8),
                             THREADS, 0, s>>>(wacc, wsum, nbins);
        check_cuda(cudaGetLastError(), "wsum finish launch");
        count_launch();
      }
      return;
    }
    // partitioned path, at most 2^30 points per pass so that record indices
    // fit in 31 bits; longer inputs add up pass by pass
    auto pass = [&](const float* x, const float* y, const float* w, long long n) {
      // persistent accumulate grid: as many CTAs as fit with the tile in shared memory
      const size_t smem = weighted ? (size_t)TB * 12 : (size_t)TB * 4;
      const void* acc_fn = weighted ? (const void*)tile_accumulate_kernel<true> : (const void*)tile_accumulate_kernel<false>;
      check_cuda(cudaFuncSetAttribute(acc_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attribute");
      int per_sm = 0;
      check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, acc_fn, ACC_THREADS, smem), "occupancy");
      if (per_sm < 1) per_sm = 1;
      const int G = sms * per_sm;
      // bucket storage bound: the sample has at most nsamp points, so the
      // capacities add up to at most 1.25 * SAMPLE * nsamp + (SLACK + 8) per bucket
      const long long nv = ntiles * NSUB;
      const long long nsamp = (((n + 1023) / 1024 + SAMPLE - 1) / SAMPLE) * 1024;
      const long long maxrec = (long long)(SAMPLE * 5 / 4) * nsamp + (long long)(SLACK + 8) * nv;
      const long long nslots = (long long)(G + ntiles) * TB;
      const size_t bytes = 16 * 256 + (size_t)(nv + 1) * 8 * 3 + (size_t)nv * FPAD * 8 + (size_t)ntiles * EPAD * 4 +
                           (size_t)maxrec * 2 + (weighted ? (size_t)maxrec * 4 : 0) + (size_t)nslots * (weighted ? 12 : 4);
      StreamScratch scratch(bytes, s);
      StreamScratch acc(weighted ? (size_t)nbins * sizeof(double) : 0, s);
      double* wacc = (double*)acc.ptr;
      if (weighted) check_cuda(cudaMemsetAsync(wacc, 0, (size_t)nbins * sizeof(double), s), "memset weights");
      char* p = (char*)(((uintptr_t)scratch.ptr + 255) & ~(uintptr_t)255);
      long long* off = carve<long long>(p, nv + 1);
      long long* cap = carve<long long>(p, nv + 1);
      long long* PV = carve<long long>(p, nv + 1);
      unsigned long long* fill = carve<unsigned long long>(p, nv * FPAD);
      unsigned* est = carve<unsigned>(p, ntiles * EPAD);
      float* rec_w = weighted ? carve<float>(p, maxrec) : nullptr;
      unsigned short* rec_bin = carve<unsigned short>(p, maxrec);
      unsigned* pc = carve<unsigned>(p, nslots);
      float* ps = weighted ? carve<float>(p, nslots) : nullptr;
      float* pe = weighted ? carve<float>(p, nslots) : nullptr;
      check_cuda(cudaMemsetAsync(est, 0, (size_t)ntiles * EPAD * 4, s), "memset estimates");
      tile_sample_kernel<<<(unsigned)std::min<long long>((nsamp + THREADS - 1) / THREADS, (long long)sms * 4), THREADS, 0,
                           s>>>(x, y, n, B, (int)ntiles, est);
      tile_plan_kernel<<<1, SCAN_THREADS, 0, s>>>(est, (int)nv, off, cap, fill);
      // persistent scatter grid: every resident CTA, at most one per chunk
      {
        const long long chunks = (n + CHUNK - 1) / CHUNK;
        const int ssm = weighted ? scatter_smem<true>() : scatter_smem<false>();
        const void* sc_fn = weighted ? (const void*)tile_scatter_kernel<true> : (const void*)tile_scatter_kernel<false>;
        check_cuda(cudaFuncSetAttribute(sc_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, ssm), "smem attribute");
        int sper = 0;
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sper, sc_fn, THREADS, ssm), "occupancy");
        const unsigned sgrid = (unsigned)std::min<long long>(chunks, (long long)sms * std::max(sper, 1));
        if (weighted)
          tile_scatter_kernel<true><<<sgrid, THREADS, ssm, s>>>(x, y, w, n, B, (int)ntiles, off, cap, fill, rec_bin, rec_w,
                                                                cnt, wacc);
        else
          tile_scatter_kernel<false><<<sgrid, THREADS, ssm, s>>>(x, y, nullptr, n, B, (int)ntiles, off, cap, fill,
                                                                 rec_bin, nullptr, cnt, nullptr);
      }
      tile_prefix_kernel<<<1, SCAN_THREADS, 0, s>>>((int)nv, cap, fill, PV);
      if (weighted)
        tile_accumulate_kernel<true><<<G, ACC_THREADS, smem, s>>>((int)nv, off, PV, rec_bin, rec_w, pc, ps, pe);
      else
        tile_accumulate_kernel<false><<<G, ACC_THREADS, smem, s>>>((int)nv, off, PV, rec_bin, nullptr, pc, nullptr,
                                                                   nullptr);
      const unsigned cgrid = (unsigned)std::min<long long>((nbins + THREADS - 1) / THREADS, (long long)sms * 8);
      if (weighted)
        tile_combine_kernel<true><<<cgrid, THREADS, 0, s>>>(nbins, (int)nv, G, PV, pc, ps, pe, wacc, cnt, wsum);
      else
        tile_combine_kernel<false><<<cgrid, THREADS, 0, s>>>(nbins, (int)nv, G, PV, pc, nullptr, nullptr, nullptr,
                                                             cnt, nullptr);
      check_cuda(cudaGetLastError(), "hist2d launches");
      count_launch(6);
    };
    for (long long s0 = 0; s0 < n; s0 += (1ll << 30)) {
      const long long len = std::min<long long>(n - s0, 1ll << 30);
      pass(x + s0, y + s0, weighted ? w + s0 : nullptr, len);
    }
  });
}
