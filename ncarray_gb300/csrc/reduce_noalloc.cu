// nca_reduce_noalloc: a full reduction (sum, mean, max, min, argmax, argmin
// over every element) that allocates no device memory.
//
// Who needs it: callers that must not allocate at call time -- code running
// while a CUDA stream is being captured into a graph whose allocation policy
// forbids new memory nodes, real-time loops that pre-plan every byte, and
// hosts that hand the library a device but no allocator (cudaMalloc may be
// unavailable or forbidden there). nca_reduce's full reduction splits the
// input across CTAs and keeps the per-CTA partials in stream-ordered scratch
// from cudaMallocAsync; this variant keeps them in a fixed array compiled
// into the library instead.
//
// Limits and behaviour:
//   - inputs: C-contiguous float32, float64, int32 or int64 views of at most
//     NCA_NOALLOC_MAX_ELEMENTS elements (larger inputs are rejected with
//     NCA_ERR_LIMIT before anything runs);
//   - the scratch holds NCA_NOALLOC_MAX_BLOCKS partials of 32 bytes (64 KiB)
//     and stays resident on every device that loads this library until the
//     process exits;
//   - the first call on a device takes the array's device address with
//     cudaGetSymbolAddress (which may load this file's module); make that first
//     call before capturing any stream;
//   - every call writes each partial slot it reads before reading it, so
//     nothing has to start at zero; but all calls share the one array, so
//     calls whose kernels overlap on the GPU (different streams without
//     ordering between them) race on it and must be serialised by the caller.
// Results follow nca_reduce: float32 sums keep a per-thread float-float pair
// widened to float64 across threads; max/min keep the first index of the
// extreme value and ignore NaN (src/lib/ncarray/host/reductions.hh:118-169).
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "common.hpp"

#define NCA_NOALLOC_MAX_BLOCKS 2048
#define NCA_NOALLOC_MAX_ELEMENTS (1ll << 31)
#define NCA_NOALLOC_THREADS 256

namespace {

struct Partial {
  double s;              // sum (float inputs)
  unsigned long long u;  // sum (integer inputs, 64-bit wrap) or extreme value bits
  long long i;           // index of the extreme value, -1 = none
  long long pad;
};

// the scratch: one partial per CTA of the first kernel
static __device__ __align__(256) Partial g_noalloc_partials[NCA_NOALLOC_MAX_BLOCKS];

template <class T> struct Lim;
template <> struct Lim<float> {
  static __device__ float lo() { return __uint_as_float(0xff7fffffu); }
  static __device__ float hi() { return __uint_as_float(0x7f7fffffu); }
  static __device__ unsigned long long bits(float v) { return __float_as_uint(v); }
  static __device__ float from(unsigned long long b) { return __uint_as_float((unsigned)b); }
};
template <> struct Lim<double> {
  static __device__ double lo() { return __longlong_as_double((long long)0xffefffffffffffffull); }
  static __device__ double hi() { return __longlong_as_double(0x7fefffffffffffffll); }
  static __device__ unsigned long long bits(double v) { return (unsigned long long)__double_as_longlong(v); }
  static __device__ double from(unsigned long long b) { return __longlong_as_double((long long)b); }
};
template <> struct Lim<int> {
  static __device__ int lo() { return (int)0x80000000; }
  static __device__ int hi() { return 0x7fffffff; }
  static __device__ unsigned long long bits(int v) { return (unsigned)v; }
  static __device__ int from(unsigned long long b) { return (int)(unsigned)b; }
};
template <> struct Lim<long long> {
  static __device__ long long lo() { return (long long)0x8000000000000000ull; }
  static __device__ long long hi() { return 0x7fffffffffffffffll; }
  static __device__ unsigned long long bits(long long v) { return (unsigned long long)v; }
  static __device__ long long from(unsigned long long b) { return (long long)b; }
};

// OP: 0 sum, 1 mean, 2 max, 3 min, 4 argmax, 5 argmin
template <class T, int OP>
struct Acc {
  static constexpr bool kSum = OP <= 1;
  static constexpr bool kMax = OP == 2 || OP == 4;
  float hi = 0.f, lo = 0.f;   // float32 sum: float-float (Knuth TwoSum)
  double d = 0.0;             // float64 sum
  unsigned long long u = 0;   // integer sum
  T v;
  long long i = -1;
  __device__ void init() { v = kMax ? Lim<T>::lo() : Lim<T>::hi(); }
  __device__ void see(T x, long long idx) {
    if constexpr (kSum) {
      if constexpr (sizeof(T) == 4 && T(0.5) != T(0)) {
        const float s = __fadd_rn(hi, x);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
        hi = s;
        // an infinite or NaN running sum has no rounding error to keep
        // (inf - inf would turn lo, and with it the result, into NaN)
        lo = fabsf(s) < __int_as_float(0x7f800000) ? __fadd_rn(lo, err) : lo;
      } else if constexpr (T(0.5) != T(0)) {
        d = __dadd_rn(d, x);
      } else {
        u += (unsigned long long)(long long)x;
      }
    } else if constexpr (kMax) {
      if (x > v) { v = x; i = idx; }
    } else {
      if (x < v) { v = x; i = idx; }
    }
  }
};

template <class T, int OP>
__device__ Partial to_partial(const Acc<T, OP>& a) {
  Partial p;
  p.s = __dadd_rn((double)a.hi, (double)a.lo) + a.d;
  p.u = Acc<T, OP>::kSum ? a.u : Lim<T>::bits(a.v);
  p.i = a.i;
  p.pad = 0;
  return p;
}

template <class T, int OP>
__device__ void merge(Partial& a, const Partial& b) {
  if constexpr (OP <= 1) {
    a.s += b.s;
    a.u += b.u;
  } else {
    if (b.i < 0) return;
    const T av = Lim<T>::from(a.u), bv = Lim<T>::from(b.u);
    const bool better = (OP == 2 || OP == 4) ? (bv > av) : (bv < av);
    if (a.i < 0 || better || (bv == av && b.i < a.i)) { a.u = b.u; a.i = b.i; }
  }
}

template <class T, int OP>
__device__ Partial block_combine(Partial p) {
  __shared__ Partial sh[NCA_NOALLOC_THREADS / 32];
  for (int off = 16; off > 0; off >>= 1) {
    Partial o;
    o.s = __shfl_down_sync(0xffffffffu, p.s, off);
    o.u = __shfl_down_sync(0xffffffffu, p.u, off);
    o.i = __shfl_down_sync(0xffffffffu, p.i, off);
    merge<T, OP>(p, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = p;
  __syncthreads();
  if (wid == 0) {
    if (lane < NCA_NOALLOC_THREADS / 32) {
      p = sh[lane];
    } else {
      p.s = 0.0; p.u = 0; p.i = -1;
    }
    for (int off = 16; off > 0; off >>= 1) {
      Partial o;
      o.s = __shfl_down_sync(0xffffffffu, p.s, off);
      o.u = __shfl_down_sync(0xffffffffu, p.u, off);
      o.i = __shfl_down_sync(0xffffffffu, p.i, off);
      merge<T, OP>(p, o);
    }
  }
  return p;
}

// CTA b reduces the contiguous chunk [b*chunk, min(n, (b+1)*chunk)) into part[b].
template <class T, int OP>
__global__ void __launch_bounds__(NCA_NOALLOC_THREADS)
noalloc_partial_kernel(const T* __restrict__ x, long long n, long long chunk, Partial* part) {
  Acc<T, OP> acc;
  acc.init();
  const long long b0 = (long long)blockIdx.x * chunk;
  const long long b1 = b0 + chunk < n ? b0 + chunk : n;
  for (long long i = b0 + threadIdx.x; i < b1; i += NCA_NOALLOC_THREADS) acc.see(__ldg(x + i), i);
  Partial p = block_combine<T, OP>(to_partial(acc));
  if (threadIdx.x == 0) part[blockIdx.x] = p;
}

// One CTA combines the nb partials and writes the result.
template <class T, int OP>
__global__ void __launch_bounds__(NCA_NOALLOC_THREADS)
noalloc_final_kernel(const Partial* part, int nb, long long n, void* out) {
  Partial p;
  p.s = 0.0; p.u = 0; p.i = -1; p.pad = 0;
  if constexpr (OP >= 2) p.u = Lim<T>::bits((OP == 2 || OP == 4) ? Lim<T>::lo() : Lim<T>::hi());
  for (int b = threadIdx.x; b < nb; b += NCA_NOALLOC_THREADS) merge<T, OP>(p, part[b]);
  p = block_combine<T, OP>(p);
  if (threadIdx.x != 0) return;
  constexpr bool is_float = T(0.5) != T(0);
  if constexpr (OP == 0) {
    if constexpr (is_float) {
      if constexpr (sizeof(T) == 4) *(float*)out = __double2float_rn(p.s);
      else *(double*)out = p.s;
    } else {
      *(T*)out = (T)p.u;
    }
  } else if constexpr (OP == 1) {
    const double s = is_float ? p.s : (double)(long long)p.u;
    *(double*)out = __ddiv_rn(s, (double)n);
  } else if constexpr (OP == 2 || OP == 3) {
    *(T*)out = p.i < 0 ? ((OP == 2) ? Lim<T>::lo() : Lim<T>::hi()) : Lim<T>::from(p.u);
  } else {
    *(long long*)out = p.i < 0 ? 0 : p.i;
  }
}

struct DeviceScratch {
  std::mutex m;
  Partial* ptr[64] = {nullptr};
};

DeviceScratch& scratch_table() {
  static DeviceScratch s;
  return s;
}

// Device address of g_noalloc_partials on the current device (set up once per device).
Partial* scratch_for(int dev) {
  if (dev < 0 || dev >= 64) nca::fail(NCA_ERR_LIMIT, "device ordinal %d out of range", dev);
  auto& t = scratch_table();
  std::lock_guard<std::mutex> lk(t.m);
  if (!t.ptr[dev]) {
    Partial* p = nullptr;
    nca::check_cuda(cudaGetSymbolAddress((void**)&p, g_noalloc_partials),
                    "cudaGetSymbolAddress(no-allocation scratch)");
    t.ptr[dev] = p;
  }
  return t.ptr[dev];
}

template <class T, int OP>
void run(const T* x, long long n, void* out, Partial* part, cudaStream_t s) {
  int nb = 0;
  long long chunk = 0;
  if (n > 0) {
    const long long per_block = (long long)NCA_NOALLOC_THREADS * 16;
    long long want = (n + per_block - 1) / per_block;
    nb = (int)(want < NCA_NOALLOC_MAX_BLOCKS ? want : NCA_NOALLOC_MAX_BLOCKS);
    chunk = (n + nb - 1) / nb;
    noalloc_partial_kernel<T, OP><<<nb, NCA_NOALLOC_THREADS, 0, s>>>(x, n, chunk, part);
    nca::check_cuda(cudaGetLastError(), "no-allocation partial kernel launch");
    nca::count_launch();
  }
  noalloc_final_kernel<T, OP><<<1, NCA_NOALLOC_THREADS, 0, s>>>(part, nb, n, out);
  nca::check_cuda(cudaGetLastError(), "no-allocation final kernel launch");
  nca::count_launch();
}

template <class T>
void dispatch_op(int op, const T* x, long long n, void* out, Partial* part, cudaStream_t s) {
  switch (op) {
    case NCA_RED_SUM: run<T, 0>(x, n, out, part, s); break;
    case NCA_RED_MEAN: run<T, 1>(x, n, out, part, s); break;
    case NCA_RED_MAX: run<T, 2>(x, n, out, part, s); break;
    case NCA_RED_MIN: run<T, 3>(x, n, out, part, s); break;
    case NCA_RED_ARGMAX: run<T, 4>(x, n, out, part, s); break;
    case NCA_RED_ARGMIN: run<T, 5>(x, n, out, part, s); break;
    default: nca::fail(NCA_ERR_INVALID, "unknown reduction op %d", op);
  }
}

int out_dtype_for(int op, int dt) {
  switch (op) {
    case NCA_RED_SUM: case NCA_RED_MAX: case NCA_RED_MIN: return dt;
    case NCA_RED_MEAN: return NCA_FLOAT64;
    case NCA_RED_ARGMAX: case NCA_RED_ARGMIN: return NCA_INT64;
  }
  nca::fail(NCA_ERR_INVALID, "unknown reduction op %d", op);
}

}  // namespace

extern "C" int32_t nca_reduce_noalloc(const nca_view* src, int32_t op, const nca_view* out, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!src || !out) fail(NCA_ERR_INVALID, "null view");
    const int dt = src->dtype;
    if (dt != NCA_FLOAT32 && dt != NCA_FLOAT64 && dt != NCA_INT32 && dt != NCA_INT64)
      fail(NCA_ERR_DTYPE, "nca_reduce_noalloc takes float32, float64, int32 or int64 input (got dtype %d)", dt);
    if (src->ndim < 0 || src->ndim > NCA_MAX_NDIM) fail(NCA_ERR_LIMIT, "ndim %d", src->ndim);
    if (src->pointer_axis >= 0) fail(NCA_ERR_UNSUPPORTED, "pointer axes are not supported");
    long long n = 1, expect = dtinfo(dt).size, off = 0;
    for (int d = src->ndim - 1; d >= 0; --d) {
      if (src->shape[d] < 0) fail(NCA_ERR_SHAPE, "negative extent");
      if (src->shape[d] != 1 && src->strides[d] != expect)
        fail(NCA_ERR_UNSUPPORTED, "nca_reduce_noalloc needs a C-contiguous input");
      expect *= src->shape[d];
      n *= src->shape[d];
      off += src->offsets[d];
    }
    if (n > NCA_NOALLOC_MAX_ELEMENTS)
      fail(NCA_ERR_LIMIT, "nca_reduce_noalloc handles at most %lld elements (input has %lld); use nca_reduce",
           (long long)NCA_NOALLOC_MAX_ELEMENTS, n);
    if (n > 0 && !src->data) fail(NCA_ERR_INVALID, "null input data");
    const int odt = out_dtype_for(op, dt);
    if (out->dtype != odt) fail(NCA_ERR_DTYPE, "output dtype %d, expected %s", out->dtype, dtinfo(odt).name);
    if (out->ndim < 0 || out->ndim > NCA_MAX_NDIM) fail(NCA_ERR_LIMIT, "output ndim %d", out->ndim);
    long long on = 1;
    for (int d = 0; d < out->ndim; ++d) on *= out->shape[d];
    if (on != 1 || !out->data) fail(NCA_ERR_SHAPE, "output must be one element");
    long long ooff = 0;
    for (int d = 0; d < out->ndim; ++d) ooff += out->offsets[d];
    void* o = static_cast<char*>(out->data) + ooff;
    const void* x = static_cast<const char*>(src->data) + off;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    Partial* part = scratch_for(dev);
    cudaStream_t s = (cudaStream_t)stream;
    switch (dt) {
      case NCA_FLOAT32: dispatch_op<float>(op, (const float*)x, n, o, part, s); break;
      case NCA_FLOAT64: dispatch_op<double>(op, (const double*)x, n, o, part, s); break;
      case NCA_INT32: dispatch_op<int>(op, (const int*)x, n, o, part, s); break;
      case NCA_INT64: dispatch_op<long long>(op, (const long long*)x, n, o, part, s); break;
    }
  });
}
