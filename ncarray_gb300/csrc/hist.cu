// 2-D histogram binning of float32 (x, y) points with optional float32 weights.
//
// The reference has only an internal scatter-add (`dest[idx[i]] += src[i]`,
// src/lib/ncarray/device/kernels.cuh:660-680, host/elementwise.hh:482-505) and
// no public histogram API; this is the histogram the benchmark spec asks for.
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
//      warp-aggregated shared-memory atomics and appends (bin within tile:
//      uint16, weight: float32) records to the tile buckets (one global atomic
//      per tile and CTA); records that do not fit in their bucket are added
//      with global atomics directly;
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

#include "common.hpp"

namespace {

constexpr int THREADS = 256;
constexpr int TB = 16384;               // bins per tile (local index fits in uint16)
constexpr int MAX_TILES = 256;          // partitioned path limit (4 Mi bins)
constexpr int SAMPLE = 32;              // 1 block of 1024 points in SAMPLE is counted in pass 1
constexpr int CHUNK = 4096;             // points per CTA in the scatter pass
constexpr int PER_THREAD = CHUNK / THREADS;
constexpr int ACC_THREADS = 1024;

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

// inclusive prefix sum of MAX_TILES values held one per thread
__device__ __forceinline__ long long block_scan(long long v, long long* sc) {
  const int t = threadIdx.x;
  sc[t] = v;
  __syncthreads();
  for (int d = 1; d < MAX_TILES; d <<= 1) {
    const long long u = t >= d ? sc[t - d] : 0;
    __syncthreads();
    sc[t] += u;
    __syncthreads();
  }
  return sc[t];
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
    if (cnt[t]) atomicAdd(est + t, cnt[t]);
}

// bucket capacity and offset of every tile; capacities are multiples of 8
// records so that every bucket starts 16-byte aligned
__global__ void __launch_bounds__(MAX_TILES)
tile_plan_kernel(const unsigned* __restrict__ est, int ntiles, long long* __restrict__ off,
                 long long* __restrict__ cap, unsigned long long* __restrict__ fill) {
  __shared__ long long sc[MAX_TILES];
  const int t = threadIdx.x;
  const long long c = t < ntiles ? (long long)est[t] * (SAMPLE * 5 / 4) + 4096 : 0;
  const long long inc = block_scan(c, sc);
  if (t < ntiles) {
    off[t] = inc - c;
    cap[t] = c;
    fill[t] = 0;
  }
  if (t == ntiles - 1) off[ntiles] = inc;
}

// ---- pass 2: scatter points into tile buckets -------------------------------------
template <bool WEIGHTED>
__global__ void __launch_bounds__(THREADS)
tile_scatter_kernel(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ w,
                    long long n, Bins B, int ntiles, const long long* __restrict__ off,
                    const long long* __restrict__ cap, unsigned long long* __restrict__ fill,
                    unsigned short* __restrict__ rec_bin, float* __restrict__ rec_w,
                    unsigned long long* __restrict__ counts, double* __restrict__ wacc) {
  __shared__ unsigned cnt[MAX_TILES];
  __shared__ long long base[MAX_TILES];   // start of this CTA's run in the bucket
  __shared__ unsigned avail[MAX_TILES];   // how many of the run fit in the bucket
  const long long c0 = (long long)blockIdx.x * CHUNK;
  if (c0 >= n) return;
  for (int t = threadIdx.x; t < ntiles; t += THREADS) cnt[t] = 0;
  __syncthreads();
  int bins[PER_THREAD];
  float ws[PER_THREAD];
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const long long i = c0 + threadIdx.x + (long long)k * THREADS;
    bins[k] = -1;
    ws[k] = 0.f;
    if (i < n) {
      bins[k] = bin_of(B, __ldcs(x + i), __ldcs(y + i));
      if (WEIGHTED) ws[k] = __ldcs(w + i);
    }
  }
  // rank within the CTA's run of the tile: one shared atomic per distinct tile in the warp
  const unsigned lane = threadIdx.x & 31u;
  unsigned rank[PER_THREAD];
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int t = bins[k] >= 0 ? bins[k] / TB : -1;
    const unsigned m = __match_any_sync(0xffffffffu, t);
    const int leader = __ffs(m) - 1;
    unsigned r0 = 0;
    if ((int)lane == leader && t >= 0) r0 = atomicAdd(&cnt[t], (unsigned)__popc(m));
    r0 = __shfl_sync(0xffffffffu, r0, leader);
    rank[k] = r0 + (unsigned)__popc(m & ((1u << lane) - 1u));
  }
  __syncthreads();
  for (int t = threadIdx.x; t < ntiles; t += THREADS) {
    base[t] = 0;
    avail[t] = 0;
    if (cnt[t]) {
      // positions [p, p + cnt) are this CTA's; the part below the capacity is
      // always written, so every position below min(fill, cap) holds a record
      const unsigned long long p = atomicAdd(fill + t, (unsigned long long)cnt[t]);
      const long long room = cap[t] - (long long)p;
      base[t] = off[t] + (long long)p;
      avail[t] = room <= 0 ? 0u : (room >= (long long)cnt[t] ? cnt[t] : (unsigned)room);
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < PER_THREAD; ++k) {
    const int b = bins[k];
    if (b < 0) continue;
    const int t = b / TB;
    if (rank[k] < avail[t]) {
      const long long bs = base[t];
      rec_bin[bs + rank[k]] = (unsigned short)(b - t * TB);
      if (WEIGHTED) rec_w[bs + rank[k]] = ws[k];
    } else {
      atomicAdd(counts + b, 1ull);
      if (WEIGHTED) atomicAdd(wacc + b, (double)ws[k]);
    }
  }
}

// stored records per tile and their exclusive prefix sum P (P[ntiles] = total)
__global__ void __launch_bounds__(MAX_TILES)
tile_prefix_kernel(int ntiles, const long long* __restrict__ cap, const unsigned long long* __restrict__ fill,
                   long long* __restrict__ P) {
  __shared__ long long sc[MAX_TILES];
  const int t = threadIdx.x;
  long long f = 0;
  if (t < ntiles) {
    const long long ft = (long long)fill[t];
    f = ft < cap[t] ? ft : cap[t];
  }
  const long long inc = block_scan(f, sc);
  if (t < ntiles) P[t] = inc - f;
  if (t == ntiles - 1) P[ntiles] = inc;
}

// ---- pass 3: per-tile shared-memory histograms of record ranges -------------------
// CTA g takes records [R g / G, R (g + 1) / G) of the concatenated buckets
// (tile t holds positions [P[t], P[t+1])); its piece of tile t is stored in
// partial slot g + t, which is unique because both g and t grow along the
// concatenation.
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
__global__ void __launch_bounds__(ACC_THREADS)
tile_accumulate_kernel(int ntiles, const long long* __restrict__ off, const long long* __restrict__ P,
                       const unsigned short* __restrict__ rec_bin, const float* __restrict__ rec_w,
                       unsigned* __restrict__ pc, float* __restrict__ ps, float* __restrict__ pe) {
  extern __shared__ __align__(16) unsigned char sm[];
  unsigned* c = reinterpret_cast<unsigned*>(sm);
  float* s = reinterpret_cast<float*>(sm + TB * 4);
  float* e = reinterpret_cast<float*>(sm + TB * 8);
  const int G = gridDim.x, g = blockIdx.x;
  const long long R = P[ntiles];
  const long long S1 = range_start(R, g + 1, G);
  long long pos = range_start(R, g, G);
  int t = 0;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  while (pos < S1) {
    while (P[t + 1] <= pos) ++t;                 // pos < R = P[ntiles], so t < ntiles
    const long long end = P[t + 1] < S1 ? P[t + 1] : S1;
    for (int i = threadIdx.x; i < TB; i += ACC_THREADS) {
      c[i] = 0u;
      if (WEIGHTED) { s[i] = 0.f; e[i] = 0.f; }
    }
    __syncthreads();
    // records [a, b) of the record arrays; bucket starts are multiples of 8
    const long long a = off[t] + (pos - P[t]), b = off[t] + (end - P[t]);
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
    pos = end;
  }
}

// ---- pass 4: add the pieces of every bin's tile to the outputs ----------------------
template <bool WEIGHTED>
__global__ void __launch_bounds__(THREADS)
tile_combine_kernel(long long nbins, int ntiles, int G, const long long* __restrict__ P,
                    const unsigned* __restrict__ pc, const float* __restrict__ ps, const float* __restrict__ pe,
                    const double* __restrict__ wacc, unsigned long long* __restrict__ counts,
                    float* __restrict__ wsum) {
  const long long R = P[ntiles];
  for (long long bin = (long long)blockIdx.x * THREADS + threadIdx.x; bin < nbins;
       bin += (long long)gridDim.x * THREADS) {
    const int t = (int)(bin / TB);
    const long long i = bin - (long long)t * TB;
    const long long lo = P[t], hi = P[t + 1];
    unsigned long long cn = 0;
    double wv = 0.0;
    if (hi > lo) {
      // the CTAs whose ranges meet [lo, hi), in order
      int g = (int)(lo * G / R);
      if (g > 0) --g;
      for (; g < G; ++g) {
        const long long s0 = range_start(R, g, G), s1 = range_start(R, g + 1, G);
        if (s0 >= hi) break;
        if ((s0 > lo ? s0 : lo) < (s1 < hi ? s1 : hi)) {
          const long long slot = (long long)(g + t) * TB + i;
          cn += pc[slot];
          if (WEIGHTED) wv += (double)ps[slot] + (double)pe[slot];
        }
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
    if (ntiles > MAX_TILES || n < (1 << 20)) {
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
    // persistent accumulate grid: as many CTAs as fit with the tile in shared memory
    const size_t smem = weighted ? (size_t)TB * 12 : (size_t)TB * 4;
    const void* acc_fn = weighted ? (const void*)tile_accumulate_kernel<true> : (const void*)tile_accumulate_kernel<false>;
    check_cuda(cudaFuncSetAttribute(acc_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "smem attribute");
    int per_sm = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, acc_fn, ACC_THREADS, smem), "occupancy");
    if (per_sm < 1) per_sm = 1;
    const int G = sms * per_sm;
    // bucket storage bound: the sample has at most nsamp points, and the
    // capacities add up to at most 1.25 * SAMPLE * nsamp + 4096 per tile
    const long long nsamp = (((n + 1023) / 1024 + SAMPLE - 1) / SAMPLE) * 1024;
    const long long maxrec = (long long)(SAMPLE * 5 / 4) * nsamp + 4096 * ntiles;
    const long long nslots = (long long)(G + ntiles) * TB;
    const size_t bytes = 5 * 256 + (size_t)(ntiles + 1) * 8 * 4 + (size_t)ntiles * 4 + (size_t)maxrec * 2 +
                         (weighted ? (size_t)maxrec * 4 : 0) + (size_t)nslots * (weighted ? 12 : 4) + 8 * 256;
    StreamScratch scratch(bytes, s);
    StreamScratch acc(weighted ? (size_t)nbins * sizeof(double) : 0, s);
    double* wacc = (double*)acc.ptr;
    if (weighted) check_cuda(cudaMemsetAsync(wacc, 0, (size_t)nbins * sizeof(double), s), "memset weights");
    char* p = (char*)(((uintptr_t)scratch.ptr + 255) & ~(uintptr_t)255);
    long long* off = carve<long long>(p, ntiles + 1);
    long long* cap = carve<long long>(p, ntiles + 1);
    unsigned long long* fill = carve<unsigned long long>(p, ntiles + 1);
    long long* P = carve<long long>(p, ntiles + 1);
    unsigned* est = carve<unsigned>(p, ntiles);
    float* rec_w = weighted ? carve<float>(p, maxrec) : nullptr;
    unsigned short* rec_bin = carve<unsigned short>(p, maxrec);
    unsigned* pc = carve<unsigned>(p, nslots);
    float* ps = weighted ? carve<float>(p, nslots) : nullptr;
    float* pe = weighted ? carve<float>(p, nslots) : nullptr;
    check_cuda(cudaMemsetAsync(est, 0, ntiles * 4, s), "memset estimates");
    tile_sample_kernel<<<(unsigned)std::min<long long>((nsamp + THREADS - 1) / THREADS, (long long)sms * 4), THREADS, 0,
                         s>>>(x, y, n, B, (int)ntiles, est);
    tile_plan_kernel<<<1, MAX_TILES, 0, s>>>(est, (int)ntiles, off, cap, fill);
    const long long chunks = (n + CHUNK - 1) / CHUNK;
    if (weighted)
      tile_scatter_kernel<true><<<(unsigned)chunks, THREADS, 0, s>>>(x, y, w, n, B, (int)ntiles, off, cap, fill, rec_bin,
                                                                     rec_w, cnt, wacc);
    else
      tile_scatter_kernel<false><<<(unsigned)chunks, THREADS, 0, s>>>(x, y, nullptr, n, B, (int)ntiles, off, cap, fill,
                                                                      rec_bin, nullptr, cnt, nullptr);
    tile_prefix_kernel<<<1, MAX_TILES, 0, s>>>((int)ntiles, cap, fill, P);
    if (weighted)
      tile_accumulate_kernel<true><<<G, ACC_THREADS, smem, s>>>((int)ntiles, off, P, rec_bin, rec_w, pc, ps, pe);
    else
      tile_accumulate_kernel<false><<<G, ACC_THREADS, smem, s>>>((int)ntiles, off, P, rec_bin, nullptr, pc, nullptr,
                                                                 nullptr);
    const unsigned cgrid = (unsigned)std::min<long long>((nbins + THREADS - 1) / THREADS, (long long)sms * 8);
    if (weighted)
      tile_combine_kernel<true><<<cgrid, THREADS, 0, s>>>(nbins, (int)ntiles, G, P, pc, ps, pe, wacc, cnt, wsum);
    else
      tile_combine_kernel<false><<<cgrid, THREADS, 0, s>>>(nbins, (int)ntiles, G, P, pc, nullptr, nullptr, nullptr,
                                                           cnt, nullptr);
    check_cuda(cudaGetLastError(), "hist2d launches");
    count_launch(6);
  });
}
