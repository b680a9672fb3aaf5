// nca_scatter_add: dest[idx[i]] += cast<Dest>(src[i]) for every element i of
// src (idx has src's shape), dropping indices outside [0, dest length).
//
// The reference's scatter primitive: host::scatter_add_recursive
// (src/lib/ncarray/host/elementwise.hh:482-505) and device scatter_add_kernel
// (src/lib/ncarray/device/kernels.cuh:660-680), one thread and one global
// atomic per element. This version:
//   - walks idx and src as N-d strided views (dims merged on the host; 1-D
//     contiguous views skip the coordinate decode);
//   - groups the lanes of a warp that hit the same destination
//     (__match_any_sync), sums each group by pointer jumping over the group's
//     lanes and lets one lane per group issue the atomic (warp-aggregated
//     atomics: the hot bins of skewed index distributions cost one atomic per
//     warp instead of one per element);
//   - privatises the destination in shared memory when it is small next to the
//     input (each CTA accumulates its grid-stride share there and adds the
//     non-zero entries to the destination once);
//   - in the common case (1-D views, source of the destination's type) keeps
//     four index and four source loads in flight per thread.
// Integer destinations wrap (two's complement) exactly as the reference's
// `+=` does. Floating destinations add in the order the atomics land, so the
// result equals the reference's sequential sum up to rounding (the order of a
// float atomicAdd sum is not fixed; the reference's device kernel has the same
// property).
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "common.hpp"

namespace {

constexpr int THREADS = 256;
constexpr int SMEM_MAX_BYTES = 48 * 1024;   // privatised destination limit per CTA

struct ScatterArgs {
  const char* idx;
  const char* src;
  char* dest;
  long long n;            // elements of idx / src
  long long dest_n;       // destination length
  long long dest_stride;  // bytes
  int nd;                 // canonical dims (1..NCA_MAX_NDIM)
  int idx_dt, src_dt;
  long long shape[NCA_MAX_NDIM];
  long long istr[NCA_MAX_NDIM];
  long long sstr[NCA_MAX_NDIM];
};

__device__ __forceinline__ long long load_index(int dt, const char* p) {
  switch (dt) {
    case NCA_INT32: return (long long)*(const int*)p;
    case NCA_UINT32: return (long long)*(const unsigned*)p;
    case NCA_INT64: return *(const long long*)p;
    default: return (long long)*(const unsigned long long*)p;   // >= 2^63 reads negative: dropped
  }
}

template <class D>
__device__ __forceinline__ D load_as(int dt, const char* p) {
  switch (dt) {
    case NCA_BOOL: return (D)(*(const unsigned char*)p != 0);
    case NCA_CHAR: case NCA_INT8: return (D)*(const signed char*)p;
    case NCA_UINT8: return (D)*(const unsigned char*)p;
    case NCA_INT16: return (D)*(const short*)p;
    case NCA_UINT16: return (D)*(const unsigned short*)p;
    case NCA_INT32: return (D)*(const int*)p;
    case NCA_UINT32: return (D)*(const unsigned*)p;
    case NCA_INT64: return (D)*(const long long*)p;
    case NCA_UINT64: return (D)*(const unsigned long long*)p;
    case NCA_FLOAT32: return (D)*(const float*)p;
    case NCA_FLOAT64: return (D)*(const double*)p;
    case NCA_BFLOAT16: return (D)__uint_as_float((unsigned)*(const unsigned short*)p << 16);
    default: return (D)__half2float(*(const __half*)p);
  }
}

// the storage type the atomics work on
template <class D> struct AtomicT { typedef D type; };
template <> struct AtomicT<int> { typedef unsigned type; };
template <> struct AtomicT<long long> { typedef unsigned long long type; };

template <class D>
__device__ __forceinline__ void atomic_add(D* p, D v) {
  typedef typename AtomicT<D>::type A;
  atomicAdd(reinterpret_cast<A*>(p), (A)v);
}

template <class D>
__device__ __forceinline__ D shfl(D v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// Sum of v over the lanes whose key equals this lane's key; valid in the
// lowest lane of each group (returned true there). All 32 lanes take part.
// Pointer jumping along each group's lanes in lane order: after round r a lane
// holds the sum of itself and the next 2^(r+1) - 1 members of its group.
template <class D>
__device__ __forceinline__ bool warp_group_sum(long long key, D& v) {
  const int lane = threadIdx.x & 31;
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  const unsigned above = peers & ~((2u << lane) - 1u);          // members after this lane
  int next = above ? __ffs(above) - 1 : lane;
  bool has = above != 0;
  if (__any_sync(0xffffffffu, has)) {
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      const D ov = shfl(v, next);
      const int onext = __shfl_sync(0xffffffffu, next, next);
      const bool ohas = __shfl_sync(0xffffffffu, has, next);
      if (has) { v += ov; next = onext; has = ohas; }
    }
  }
  return (peers & ((1u << lane) - 1u)) == 0;
}

__device__ __forceinline__ void offsets_of(const ScatterArgs& a, long long i, long long& oi, long long& os) {
  if (a.nd == 1) {
    oi = i * a.istr[0];
    os = i * a.sstr[0];
    return;
  }
  oi = 0;
  os = 0;
  for (int d = a.nd - 1; d >= 0; --d) {
    const long long c = i % a.shape[d];
    i /= a.shape[d];
    oi += c * a.istr[d];
    os += c * a.sstr[d];
  }
}

// One grid-stride pass; SMEM: accumulate into the CTA's shared copy of dest.
template <class D, bool SMEM>
__global__ void __launch_bounds__(THREADS) scatter_add_kernel(ScatterArgs a) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  D* priv = reinterpret_cast<D*>(sm_raw);
  if (SMEM) {
    for (long long b = threadIdx.x; b < a.dest_n; b += THREADS) priv[b] = D(0);
    __syncthreads();
  }
  const long long stride = (long long)gridDim.x * THREADS;
  // every lane of a warp runs the same number of rounds (the group sum needs all 32)
  const long long warp0 = (long long)blockIdx.x * THREADS + (threadIdx.x & ~31);
  for (long long base = warp0; base < a.n; base += stride) {
    const long long i = base + (threadIdx.x & 31);
    long long t = -1;
    D v = D(0);
    if (i < a.n) {
      long long oi, os;
      offsets_of(a, i, oi, os);
      t = load_index(a.idx_dt, a.idx + oi);
      if (t >= 0 && t < a.dest_n) v = load_as<D>(a.src_dt, a.src + os);
      else t = -1;
    }
    const long long key = t >= 0 ? t : -1 - (long long)(threadIdx.x & 31);   // invalid lanes stay alone
    const bool leader = warp_group_sum<D>(key, v);
    if (leader && t >= 0) {
      if (SMEM) atomic_add<D>(priv + t, v);
      else atomic_add<D>(reinterpret_cast<D*>(a.dest + t * a.dest_stride), v);
    }
  }
  if (SMEM) {
    __syncthreads();
    for (long long b = threadIdx.x; b < a.dest_n; b += THREADS) {
      const D v = priv[b];
      if (v != D(0)) atomic_add<D>(reinterpret_cast<D*>(a.dest + b * a.dest_stride), v);
    }
  }
}

// The common case in one pass with more loads in flight: 1-D views, the
// source already of the destination's type, indices of 32 or 64 bits, a
// destination below 2^31 entries (32-bit match keys). A warp takes 32 * U
// consecutive elements per trip (U loads of each array in flight per thread,
// the source loaded without waiting for its index); grouping and atomics as
// in scatter_add_kernel.
constexpr int U = 4;

template <class D, class IW, bool SMEM>
__global__ void __launch_bounds__(THREADS) scatter_fast_kernel(ScatterArgs a, int idx_signed) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  D* priv = reinterpret_cast<D*>(sm_raw);
  if (SMEM) {
    for (long long b = threadIdx.x; b < a.dest_n; b += THREADS) priv[b] = D(0);
    __syncthreads();
  }
  const IW* idx = reinterpret_cast<const IW*>(a.idx);
  const D* src = reinterpret_cast<const D*>(a.src);
  const long long ist = a.istr[0] / (long long)sizeof(IW), sst = a.sstr[0] / (long long)sizeof(D);
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * THREADS * U;
  for (long long base = ((long long)blockIdx.x * THREADS + (threadIdx.x & ~31)) * U; base < a.n; base += stride) {
    IW raw[U];
    D v[U];
#pragma unroll
    for (int k = 0; k < U; ++k) {
      const long long i = base + k * 32 + lane;
      raw[k] = (IW)0;
      v[k] = D(0);
      if (i < a.n) {
        raw[k] = idx[i * ist];
        v[k] = src[i * sst];
      }
    }
#pragma unroll
    for (int k = 0; k < U; ++k) {
      long long t;
      if (sizeof(IW) == 4) t = idx_signed ? (long long)(int)(unsigned)raw[k] : (long long)(unsigned)raw[k];
      else t = (long long)(unsigned long long)raw[k];   // uint64 >= 2^63 reads negative: dropped
      if (base + k * 32 + lane >= a.n) t = -1;
      const bool ok = t >= 0 && t < a.dest_n;
      const unsigned key = ok ? (unsigned)t : 0x80000000u + (unsigned)lane;   // invalid lanes stay alone
      const unsigned peers = __match_any_sync(0xffffffffu, key);
      D s = ok ? v[k] : D(0);
      const unsigned above = peers & ~((2u << lane) - 1u);
      int next = above ? __ffs(above) - 1 : lane;
      bool has = above != 0;
      if (__any_sync(0xffffffffu, has)) {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          const D ov = shfl(s, next);
          const int onext = __shfl_sync(0xffffffffu, next, next);
          const bool ohas = __shfl_sync(0xffffffffu, has, next);
          if (has) { s += ov; next = onext; has = ohas; }
        }
      }
      if (ok && (peers & ((1u << lane) - 1u)) == 0) {
        if (SMEM) atomic_add<D>(priv + t, s);
        else atomic_add<D>(reinterpret_cast<D*>(a.dest + t * a.dest_stride), s);
      }
    }
  }
  if (SMEM) {
    __syncthreads();
    for (long long b = threadIdx.x; b < a.dest_n; b += THREADS) {
      const D v = priv[b];
      if (v != D(0)) atomic_add<D>(reinterpret_cast<D*>(a.dest + b * a.dest_stride), v);
    }
  }
}

// true when the source dtype loads as D directly (same size and kind)
template <class D> constexpr bool same_src(int dt) {
  return (sizeof(D) == 4 && (D)0.5 != 0 && dt == NCA_FLOAT32) || (sizeof(D) == 8 && (D)0.5 != 0 && dt == NCA_FLOAT64) ||
         (sizeof(D) == 4 && (D)0.5 == 0 && (dt == NCA_INT32 || dt == NCA_UINT32)) ||
         (sizeof(D) == 8 && (D)0.5 == 0 && (dt == NCA_INT64 || dt == NCA_UINT64));
}

bool index_dtype_ok(int dt) {
  return dt == NCA_INT32 || dt == NCA_UINT32 || dt == NCA_INT64 || dt == NCA_UINT64;
}

template <class D>
void launch(ScatterArgs& a, cudaStream_t s) {
  const int dev = nca::current_device();
  const int sms = nca::sm_count(dev);
  const long long bytes = a.dest_n * (long long)sizeof(D);
  long long blocks = (a.n + THREADS - 1) / THREADS;
  // privatise when the destination fits and every CTA has several times more
  // elements to add than destination entries to flush
  const long long priv_ctas = (long long)sms * 4;
  const bool smem = bytes <= SMEM_MAX_BYTES && a.n >= 4 * priv_ctas * a.dest_n;
  const int isz = (a.idx_dt == NCA_INT64 || a.idx_dt == NCA_UINT64) ? 8 : 4;
  const bool fast = a.nd == 1 && same_src<D>(a.src_dt) && a.dest_n < (1ll << 31) &&
                    a.istr[0] % isz == 0 && a.sstr[0] % (long long)sizeof(D) == 0 &&
                    (uintptr_t)a.idx % isz == 0 && (uintptr_t)a.src % sizeof(D) == 0;
  if (fast) {
    const int sgn = a.idx_dt == NCA_INT32 ? 1 : 0;
    long long fb = (a.n + (long long)THREADS * U - 1) / ((long long)THREADS * U);
    if (smem) {
      fb = std::min(fb, priv_ctas);
      if (isz == 4) scatter_fast_kernel<D, unsigned, true><<<(unsigned)fb, THREADS, (size_t)bytes, s>>>(a, sgn);
      else scatter_fast_kernel<D, unsigned long long, true><<<(unsigned)fb, THREADS, (size_t)bytes, s>>>(a, sgn);
    } else {
      fb = std::min(fb, (long long)sms * 8);
      if (isz == 4) scatter_fast_kernel<D, unsigned, false><<<(unsigned)fb, THREADS, 0, s>>>(a, sgn);
      else scatter_fast_kernel<D, unsigned long long, false><<<(unsigned)fb, THREADS, 0, s>>>(a, sgn);
    }
  } else if (smem) {
    blocks = std::min(blocks, priv_ctas);
    scatter_add_kernel<D, true><<<(unsigned)blocks, THREADS, (size_t)bytes, s>>>(a);
  } else {
    blocks = std::min(blocks, (long long)sms * 8);
    scatter_add_kernel<D, false><<<(unsigned)blocks, THREADS, 0, s>>>(a);
  }
  nca::check_cuda(cudaGetLastError(), "scatter-add kernel launch");
  nca::count_launch();
}

}  // namespace

extern "C" int32_t nca_scatter_add(const nca_view* dest, const nca_view* indices, const nca_view* src,
                                   void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!dest || !indices || !src) fail(NCA_ERR_INVALID, "null view");
    if (dest->ndim != 1) fail(NCA_ERR_SHAPE, "the destination must be 1-D (got %d dims)", dest->ndim);
    if (src->ndim < 0 || src->ndim > NCA_MAX_NDIM || indices->ndim != src->ndim)
      fail(NCA_ERR_SHAPE, "indices and src must have the same number of dims (<= %d)", NCA_MAX_NDIM);
    if (dest->pointer_axis >= 0 || indices->pointer_axis >= 0 || src->pointer_axis >= 0)
      fail(NCA_ERR_UNSUPPORTED, "pointer axes are not supported by nca_scatter_add");
    const int ddt = dest->dtype;
    if (ddt != NCA_INT32 && ddt != NCA_UINT32 && ddt != NCA_INT64 && ddt != NCA_UINT64 && ddt != NCA_FLOAT32 &&
        ddt != NCA_FLOAT64)
      fail(NCA_ERR_DTYPE, "destination dtype %d: int32, uint32, int64, uint64, float32 or float64", ddt);
    if (!index_dtype_ok(indices->dtype))
      fail(NCA_ERR_DTYPE, "index dtype %d: int32, uint32, int64 or uint64", indices->dtype);
    if (!dtype_valid(src->dtype) || !dtinfo(src->dtype).device_ok)
      fail(NCA_ERR_DTYPE, "source dtype %d not supported on the device", src->dtype);
    if (dest->shape[0] < 0) fail(NCA_ERR_SHAPE, "negative destination length");
    ScatterArgs a{};
    a.idx_dt = indices->dtype;
    a.src_dt = src->dtype;
    a.dest_n = dest->shape[0];
    a.dest_stride = dest->strides[0];
    a.dest = static_cast<char*>(dest->data) + dest->offsets[0];
    long long ioff = 0, soff = 0, n = 1;
    // canonical dims: size-1 dims dropped, neighbours merged when both views allow
    int nd = 0;
    for (int d = 0; d < src->ndim; ++d) {
      if (indices->shape[d] != src->shape[d]) fail(NCA_ERR_SHAPE, "indices and src shapes differ on dim %d", d);
      if (src->shape[d] < 0) fail(NCA_ERR_SHAPE, "negative extent");
      ioff += indices->offsets[d];
      soff += src->offsets[d];
      n *= src->shape[d];
      if (src->shape[d] == 1) continue;
      if (nd > 0 && a.istr[nd - 1] == indices->strides[d] * src->shape[d] &&
          a.sstr[nd - 1] == src->strides[d] * src->shape[d]) {
        a.shape[nd - 1] *= src->shape[d];
        a.istr[nd - 1] = indices->strides[d];
        a.sstr[nd - 1] = src->strides[d];
        continue;
      }
      a.shape[nd] = src->shape[d];
      a.istr[nd] = indices->strides[d];
      a.sstr[nd] = src->strides[d];
      ++nd;
    }
    if (nd == 0) { a.shape[0] = 1; a.istr[0] = 0; a.sstr[0] = 0; nd = 1; }
    a.nd = nd;
    a.n = n;
    if (n == 0 || a.dest_n == 0) return;
    if (!indices->data || !src->data || !dest->data) fail(NCA_ERR_INVALID, "null data pointer");
    a.idx = static_cast<const char*>(indices->data) + ioff;
    a.src = static_cast<const char*>(src->data) + soff;
    cudaStream_t s = (cudaStream_t)stream;
    switch (ddt) {
      case NCA_INT32: case NCA_UINT32: launch<int>(a, s); break;
      case NCA_INT64: case NCA_UINT64: launch<long long>(a, s); break;
      case NCA_FLOAT32: launch<float>(a, s); break;
      case NCA_FLOAT64: launch<double>(a, s); break;
    }
  });
}
