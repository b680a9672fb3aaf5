// 3-D stencils: dst[c] = src[c] + dt * sum_o w[o] * src[c + o] over the 3x3x3
// neighbourhood with zero halo. Replaces ncarray's device-only Stencil<3>
// (src/lib/ncarray/expression/stencil.hh:58-255), whose NVRTC kernel reloads
// every neighbour from global memory per output (jit/device/rtcompiler.hh:187-385).
//
// GB300 design: each CTA owns a TX x TY column of outputs and marches along z.
// One elected thread streams z-planes (TX + 2*HX) x (TY + 2) x 1 into a ring of
// NST shared-memory stages with TMA (cp.async.bulk.tensor.3d) completing on
// mbarriers; the tensor map's out-of-bounds zero fill supplies the halo. The
// x origin of every box is x0 - HX with HX = 16 / sizeof(T), so it stays on a
// 16-byte boundary. Every thread owns 4 consecutive x outputs of one y row and
// keeps three rolling accumulators: plane p adds its dz = +1 / 0 / -1
// in-plane partial sums to outputs p-1, p, p+1, so each plane is read from
// shared memory once. Waits are bounded (2 s of %globaltimer); on timeout the
// CTA stops, records NCA_ERR_TIMEOUT in a status word, drains its copies in
// flight (bounded too) and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include <mutex>

#include "common.hpp"
#include "mbar.cuh"
#include "tune.hpp"

namespace {

// tile shapes (x, y) of the TMA kernel; each has (TX / 4) * TY = THREADS threads
constexpr int NST = 4, THREADS = 256;
constexpr int kTiles[3][2] = {{64, 16}, {128, 8}, {32, 32}};
constexpr unsigned long long kWaitNs = 2000000000ull;

static __device__ int g_stencil_status;
__device__ int g_jit_status;   // set by JIT kernels (kind 7) whose bounded waits give up

template <class T>
struct Weights {
  T w[27];
  T dt;
};

template <class T> __host__ __device__ constexpr int halo_x() { return 16 / (int)sizeof(T); }
template <class T, int TX> __host__ __device__ constexpr int box_w() { return TX + 2 * halo_x<T>(); }
template <class T, int TX, int TY> __host__ __device__ constexpr int stage_bytes() {
  return ((box_w<T, TX>() * (TY + 2) * (int)sizeof(T)) + 127) / 128 * 128;
}


using nca_dev::mbar_wait;

template <class T, int TX, int TY>
__device__ __forceinline__ void issue_plane(const CUtensorMap* tmap, uint32_t dst, uint32_t bar, int x, int y, int z) {
  constexpr uint32_t bytes = (uint32_t)(box_w<T, TX>() * (TY + 2) * sizeof(T));
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(dst), "l"(reinterpret_cast<unsigned long long>(tmap)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

// 6 consecutive row values starting at column c0 - 1 (c0 is 16-byte aligned)
template <class T>
__device__ __forceinline__ void load_row(const T* row, int c0, T* v) {
  v[0] = row[c0 - 1];
  if constexpr (sizeof(T) == 4) {
    const float4 m = *reinterpret_cast<const float4*>(row + c0);
    v[1] = m.x; v[2] = m.y; v[3] = m.z; v[4] = m.w;
  } else {
    const double2 m0 = *reinterpret_cast<const double2*>(row + c0);
    const double2 m1 = *reinterpret_cast<const double2*>(row + c0 + 2);
    v[1] = m0.x; v[2] = m0.y; v[3] = m1.x; v[4] = m1.y;
  }
  v[5] = row[c0 + 4];
}

template <class T>
__device__ __forceinline__ T fmaT(T a, T b, T c) {
  if constexpr (sizeof(T) == 4) return __fmaf_rn(a, b, c); else return __fma_rn(a, b, c);
}

// MODE 0: any 27 weights; 1: 7-point star (weights of offsets with two or
// three non-zero components are zero); 2: isotropic 27-point (the weight of an
// offset depends only on how many of its components are non-zero: w[13] for
// none, w[12] for one, w[9] for two, w[0] for three), evaluated per plane from
// the in-plane centre, face and corner sums (12 instead of 27 FMAs a point).
template <class T, int MODE, int TX, int TY>
__global__ void __launch_bounds__(THREADS)
stencil_tma_kernel(const __grid_constant__ CUtensorMap tmap, T* __restrict__ out, int nx, int ny, int nz,
                   int zt, const __grid_constant__ Weights<T> W) {
  extern __shared__ __align__(128) unsigned char smem[];
  static_assert((TX / 4) * TY == THREADS, "a tile has one thread per 4 outputs");
  constexpr int BW = box_w<T, TX>(), HX = halo_x<T>(), SB = stage_bytes<T, TX, TY>();
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NST * SB);
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY, z0 = blockIdx.z * zt;
  const int zend = min(z0 + zt, nz);
  const int nplanes = zend - z0 + 2;  // planes z0-1 .. zend
  const int ty = threadIdx.x / (TX / 4), tx4 = (threadIdx.x % (TX / 4)) * 4;
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t bbase = (uint32_t)__cvta_generic_to_shared(bars);
  if (threadIdx.x == 0) {
    for (int s = 0; s < NST; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bbase + 8 * s) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  int issued = 0;
  if (threadIdx.x == 0) {
    for (; issued < NST && issued < nplanes; ++issued)
      issue_plane<T, TX, TY>(&tmap, sbase + issued * SB, bbase + 8 * issued, x0 - HX, y0 - 1, z0 - 1 + issued);
  }
  // acc_a: output p-1 (missing only plane p's dz=+1 part), acc_b: output p
  // (has plane p-1's dz=-1 part), cen: centre value of output p-1
  T acc_a[4], acc_b[4], cen[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) { acc_a[j] = acc_b[j] = cen[j] = T(0); }
  const int x = x0 + tx4, y = y0 + ty;
  const bool active = x < nx && y < ny;
  bool timed_out = false;
  int i = 0;
  for (; i < nplanes; ++i) {
    const int st = i % NST;
    const bool ok = mbar_wait(bbase + 8 * st, (uint32_t)((i / NST) & 1), kWaitNs);
    if (ok) {
      const T* plane = reinterpret_cast<const T*>(smem + st * SB);
      const int c0 = HX + tx4;
      T v[3][6];
      load_row(plane + (ty + 1) * BW, c0, v[1]);
      if constexpr (MODE == 1) {
#pragma unroll
        for (int r = 0; r < 3; r += 2) {
          const T* row = plane + (ty + r) * BW;
          if constexpr (sizeof(T) == 4) {
            const float4 m = *reinterpret_cast<const float4*>(row + c0);
            v[r][1] = m.x; v[r][2] = m.y; v[r][3] = m.z; v[r][4] = m.w;
          } else {
            const double2 m0 = *reinterpret_cast<const double2*>(row + c0);
            const double2 m1 = *reinterpret_cast<const double2*>(row + c0 + 2);
            v[r][1] = m0.x; v[r][2] = m0.y; v[r][3] = m1.x; v[r][4] = m1.y;
          }
        }
      } else {
        load_row(plane + ty * BW, c0, v[0]);
        load_row(plane + (ty + 2) * BW, c0, v[2]);
      }
      // partial sums of this plane for dz = -1 (output p+1), 0 (output p), +1 (output p-1)
      T pm[4], p0[4], pp[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if constexpr (MODE == 2) {
          // in-plane centre C, faces F and corners K of output column j
          const T C = v[1][j + 1];
          const T F = ((v[1][j] + v[1][j + 2]) + v[0][j + 1]) + v[2][j + 1];
          const T K = (v[0][j] + v[0][j + 2]) + (v[2][j] + v[2][j + 2]);
          p0[j] = fmaT(W.w[9], K, fmaT(W.w[12], F, W.w[13] * C));
          const T q = fmaT(W.w[0], K, fmaT(W.w[9], F, W.w[12] * C));
          pm[j] = q;
          pp[j] = q;
        } else if constexpr (MODE == 1) {
          pm[j] = W.w[4] * v[1][j + 1];
          pp[j] = W.w[22] * v[1][j + 1];
          T s = W.w[13] * v[1][j + 1];
          s = fmaT(W.w[12], v[1][j], s);
          s = fmaT(W.w[14], v[1][j + 2], s);
          s = fmaT(W.w[10], v[0][j + 1], s);
          p0[j] = fmaT(W.w[16], v[2][j + 1], s);
        } else {
          T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
          for (int oy = 0; oy < 3; ++oy)
#pragma unroll
            for (int ox = 0; ox < 3; ++ox) {
              const T u = v[oy][j + ox];
              s0 = fmaT(W.w[0 * 9 + oy * 3 + ox], u, s0);
              s1 = fmaT(W.w[1 * 9 + oy * 3 + ox], u, s1);
              s2 = fmaT(W.w[2 * 9 + oy * 3 + ox], u, s2);
            }
          pm[j] = s0; p0[j] = s1; pp[j] = s2;
        }
      }
      const int p = z0 - 1 + i;
      // output p-1 is complete
      if (active && i >= 2) {
        T o[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) o[j] = fmaT(W.dt, acc_a[j] + pp[j], cen[j]);
        T* dst = out + ((size_t)(p - 1) * ny + y) * nx + x;
        if constexpr (sizeof(T) == 4) {
          *reinterpret_cast<float4*>(dst) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
          reinterpret_cast<double2*>(dst)[0] = make_double2(o[0], o[1]);
          reinterpret_cast<double2*>(dst)[1] = make_double2(o[2], o[3]);
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        acc_a[j] = acc_b[j] + p0[j];   // output p: now lacks only plane p+1
        acc_b[j] = pm[j];              // output p+1: plane p's dz=-1 part
        cen[j] = v[1][j + 1];          // centre of output p
      }
    }
    if (__syncthreads_or(ok ? 0 : 1)) { timed_out = true; break; }
    if (threadIdx.x == 0 && issued < nplanes) {
      issue_plane<T, TX, TY>(&tmap, sbase + st * SB, bbase + 8 * st, x0 - HX, y0 - 1, z0 - 1 + issued);
      ++issued;
    }
  }
  if (timed_out && threadIdx.x == 0) {
    atomicExch(&g_stencil_status, (int)NCA_ERR_TIMEOUT);
    for (int k = i; k < issued; ++k) mbar_wait(bbase + 8 * (k % NST), (uint32_t)((k / NST) & 1), kWaitNs / 2);
  }
}

// Any shape: one thread per output, neighbours read through L1/L2.
template <class T>
__global__ void __launch_bounds__(THREADS)
stencil_direct_kernel(const T* __restrict__ src, T* __restrict__ out, int nx, int ny, int nz,
                      const __grid_constant__ Weights<T> W) {
  const long long n = (long long)nx * ny * nz;
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(id % nx), y = (int)((id / nx) % ny), z = (int)(id / ((long long)nx * ny));
    T pz[3] = {T(0), T(0), T(0)};
#pragma unroll
    for (int dz = 0; dz < 3; ++dz) {
      const int zz = z + dz - 1;
      if (zz < 0 || zz >= nz) continue;
#pragma unroll
      for (int oy = 0; oy < 3; ++oy) {
        const int yy = y + oy - 1;
        if (yy < 0 || yy >= ny) continue;
#pragma unroll
        for (int ox = 0; ox < 3; ++ox) {
          const int xx = x + ox - 1;
          if (xx < 0 || xx >= nx) continue;
          pz[dz] = fmaT(W.w[dz * 9 + oy * 3 + ox], __ldg(src + ((long long)zz * ny + yy) * nx + xx), pz[dz]);
        }
      }
    }
    const T acc = (pz[2] + pz[0]) + pz[1];
    out[id] = fmaT(W.dt, acc, src[id]);
  }
}

struct Grid3 {
  int nz, ny, nx, dtype;
  const void* base;
  void* mut;
};

Grid3 check_grid(const nca_view* v, const char* what) {
  using namespace nca;
  if (!v) fail(NCA_ERR_INVALID, "%s: null view", what);
  if (v->ndim != 3) fail(NCA_ERR_SHAPE, "%s: stencil grids are 3-D (got %d dims)", what, v->ndim);
  if (v->dtype != NCA_FLOAT32 && v->dtype != NCA_FLOAT64)
    fail(NCA_ERR_DTYPE, "%s: stencil grids are float32 or float64", what);
  if (v->pointer_axis >= 0) fail(NCA_ERR_UNSUPPORTED, "%s: pointer axes are not supported", what);
  const int64_t isz = dtinfo(v->dtype).size;
  if (v->strides[2] != isz || v->strides[1] != isz * v->shape[2] || v->strides[0] != isz * v->shape[2] * v->shape[1])
    fail(NCA_ERR_UNSUPPORTED, "%s: stencil grids must be C-contiguous", what);
  for (int d = 0; d < 3; ++d)
    if (v->shape[d] <= 0 || v->shape[d] >= (1 << 30)) fail(NCA_ERR_SHAPE, "%s: extent out of range", what);
  int64_t off = v->offsets[0] + v->offsets[1] + v->offsets[2];
  if (!v->data) fail(NCA_ERR_INVALID, "%s: null data", what);
  Grid3 g{(int)v->shape[0], (int)v->shape[1], (int)v->shape[2], v->dtype, (const char*)v->data + off,
          (char*)v->data + off};
  return g;
}

template <class T>
Weights<T> make_weights(const double* w27, double dt) {
  Weights<T> W;
  for (int i = 0; i < 27; ++i) W.w[i] = (T)w27[i];
  W.dt = (T)dt;
  return W;
}

bool star7(const double* w) {
  for (int i = 0; i < 27; ++i) {
    const int dz = i / 9, oy = (i / 3) % 3, ox = i % 3;
    const int nz = (dz != 1) + (oy != 1) + (ox != 1);
    if (nz >= 2 && w[i] != 0.0) return false;
  }
  return true;
}

// the weight of every offset depends only on its number of non-zero components
bool isotropic27(const double* w) {
  const double cls[4] = {w[13], w[12], w[9], w[0]};
  for (int i = 0; i < 27; ++i) {
    const int dz = i / 9, oy = (i / 3) % 3, ox = i % 3;
    const int nz = (dz != 1) + (oy != 1) + (ox != 1);
    if (w[i] != cls[nz]) return false;
  }
  return true;
}

bool tma_ok(const Grid3& g) {
  // row pitch and plane pitch must be multiples of 16 bytes and the x extent a
  // multiple of 4 (each thread stores 4 aligned outputs)
  return g.nx % 4 == 0 && ((uintptr_t)g.base % 16) == 0 && nca::drv().cuTensorMapEncodeTiled != nullptr;
}

template <class T, int TX, int TY>
void encode_map(CUtensorMap* m, const Grid3& g) {
  const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.nz};
  const cuuint64_t strides[2] = {(cuuint64_t)g.nx * sizeof(T), (cuuint64_t)g.nx * g.ny * sizeof(T)};
  const cuuint32_t box[3] = {(cuuint32_t)box_w<T, TX>(), (cuuint32_t)(TY + 2), 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  nca::check_cu(nca::drv().cuTensorMapEncodeTiled(
                    m, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
                    const_cast<void*>(g.base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE),
                "cuTensorMapEncodeTiled");
}

template <class T, int TX, int TY>
void launch_tma(const Grid3& src, const Grid3& dst, const Weights<T>& W, int mode, int zt, cudaStream_t s) {
  CUtensorMap m;
  encode_map<T, TX, TY>(&m, src);
  dim3 grid((src.nx + TX - 1) / TX, (src.ny + TY - 1) / TY, (src.nz + zt - 1) / zt);
  const size_t smem = NST * stage_bytes<T, TX, TY>() + NST * 8;
  if (mode == 1)
    stencil_tma_kernel<T, 1, TX, TY><<<grid, THREADS, smem, s>>>(m, (T*)dst.mut, src.nx, src.ny, src.nz, zt, W);
  else if (mode == 2)
    stencil_tma_kernel<T, 2, TX, TY><<<grid, THREADS, smem, s>>>(m, (T*)dst.mut, src.nx, src.ny, src.nz, zt, W);
  else
    stencil_tma_kernel<T, 0, TX, TY><<<grid, THREADS, smem, s>>>(m, (T*)dst.mut, src.nx, src.ny, src.nz, zt, W);
  nca::check_cuda(cudaGetLastError(), "stencil launch");
  nca::count_launch();
}

template <class T>
void launch_tile(int tile, const Grid3& src, const Grid3& dst, const Weights<T>& W, int mode, int zt, cudaStream_t s) {
  switch (tile) {
    case 1: launch_tma<T, kTiles[1][0], kTiles[1][1]>(src, dst, W, mode, zt, s); break;
    case 2: launch_tma<T, kTiles[2][0], kTiles[2][1]>(src, dst, W, mode, zt, s); break;
    default: launch_tma<T, kTiles[0][0], kTiles[0][1]>(src, dst, W, mode, zt, s); break;
  }
}

// Tile shape and z-march depth: the autotuner's cached choice for this
// (dtype, stencil form, grid size class), else the built-in heuristic; in
// search mode a miss times every (tile, depth) candidate on this call first.
template <class T>
void tma_schedule(const Grid3& src, const Grid3& dst, const Weights<T>& W, int mode, cudaStream_t s, int& tile,
                  int& zt) {
  using namespace nca;
  tile = 0;
  zt = src.nz >= 256 ? 32 : (src.nz >= 64 ? 16 : 8);
  const std::string key = std::string("stencil3d|") + (sizeof(T) == 4 ? "f32" : "f64") + "|" + std::to_string(mode) +
                          "|" + size_class(src.nz) + "x" + size_class(src.ny) + "x" + size_class(src.nx);
  std::vector<int> v;
  if (tune_get(key, v) && v.size() == 2 && v[0] >= 0 && v[0] < 3 && v[1] >= 1) {
    tile = v[0];
    zt = v[1];
    return;
  }
  if (!tune_should_search(s)) return;
  std::vector<std::pair<int, int>> cands;
  for (int t = 0; t < 3; ++t)
    for (int z : {8, 16, 32, 64})
      if (z <= std::max(8, src.nz)) cands.push_back({t, z});
  const int best = tune_pick(s, (int)cands.size(), [&](int i) {
    launch_tile<T>(cands[(size_t)i].first, src, dst, W, mode, cands[(size_t)i].second, s);
  });
  tile = cands[(size_t)best].first;
  zt = cands[(size_t)best].second;
  tune_put(key, {tile, zt});
}

template <class T>
void launch_one(const Grid3& src, const Grid3& dst, const Weights<T>& W, int mode, cudaStream_t s) {
  using namespace nca;
  const int dev = current_device();
  if (tma_ok(src) && tma_ok(dst)) {
    int tile = 0, zt = 8;
    tma_schedule<T>(src, dst, W, mode, s, tile, zt);
    launch_tile<T>(tile, src, dst, W, mode, zt, s);
    return;
  } else {
    const long long n = (long long)src.nx * src.ny * src.nz;
    const long long blocks = std::min<long long>((n + THREADS - 1) / THREADS, (long long)sm_count(dev) * 32);
    stencil_direct_kernel<T><<<(unsigned)blocks, THREADS, 0, s>>>((const T*)src.base, (T*)dst.mut, src.nx, src.ny,
                                                                  src.nz, W);
  }
  check_cuda(cudaGetLastError(), "stencil launch");
  count_launch();
}

void run(const nca_view* a, const nca_view* b, const double* w27, double dt, int iters, cudaStream_t s) {
  using namespace nca;
  if (!w27) fail(NCA_ERR_INVALID, "null weights");
  if (iters < 0) fail(NCA_ERR_INVALID, "negative iteration count");
  Grid3 ga = check_grid(a, "a"), gb = check_grid(b, "b");
  if (ga.nx != gb.nx || ga.ny != gb.ny || ga.nz != gb.nz || ga.dtype != gb.dtype)
    fail(NCA_ERR_SHAPE, "stencil grids differ in shape or dtype");
  const size_t bytes = (size_t)ga.nx * ga.ny * ga.nz * dtinfo(ga.dtype).size;
  const char *pa = (const char*)ga.base, *pb = (const char*)gb.base;
  if (pa < pb + bytes && pb < pa + bytes) fail(NCA_ERR_INVALID, "stencil source and destination overlap");
  const int mode = star7(w27) ? 1 : isotropic27(w27) ? 2 : 0;
  for (int it = 0; it < iters; ++it) {
    const Grid3& src = (it % 2 == 0) ? ga : gb;
    const Grid3& dst = (it % 2 == 0) ? gb : ga;
    if (ga.dtype == NCA_FLOAT32) launch_one<float>(src, dst, make_weights<float>(w27, dt), mode, s);
    else launch_one<double>(src, dst, make_weights<double>(w27, dt), mode, s);
  }
}

}  // namespace

namespace nca {
// address of the status word of JIT kernels on the current device
int* jit_status_word() {
  static std::mutex mu;
  static int* addr[64] = {nullptr};
  const int dev = current_device();
  if (dev < 0 || dev >= 64) fail(NCA_ERR_LIMIT, "device %d", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    check_cuda(cudaGetSymbolAddress(&p, g_jit_status), "status word address");
    addr[dev] = static_cast<int*>(p);
  }
  return addr[dev];
}

// reads and clears the stencil status word (synchronises the stream)
int stencil_read_status(cudaStream_t s) {
  int v = 0, zero = 0;
  check_cuda(cudaMemcpyFromSymbolAsync(&v, g_stencil_status, sizeof(int), 0, cudaMemcpyDeviceToHost, s), "status read");
  check_cuda(cudaMemcpyToSymbolAsync(g_stencil_status, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s), "status clear");
  check_cuda(cudaStreamSynchronize(s), "status sync");
  return v;
}
}  // namespace nca

namespace {
// One thread waits, through the bounded-wait helper every pipeline kernel
// uses, on an mbarrier that expects one arrival which never comes (no copy is
// issued, so none is in flight); after limit_ns it records NCA_ERR_TIMEOUT in
// the stencil status word and returns.
__global__ void wait_probe_kernel(unsigned long long limit_ns) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x != 0) return;
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (!mbar_wait(b, 0u, limit_ns)) atomicExch(&g_stencil_status, (int)NCA_ERR_TIMEOUT);
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(b) : "memory");
}
}  // namespace

extern "C" int32_t nca_wait_probe(double limit_s, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!(limit_s >= 1e-3 && limit_s <= 2.0)) fail(NCA_ERR_INVALID, "limit %g s: 0.001 .. 2 s", limit_s);
    wait_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>((unsigned long long)(limit_s * 1e9));
    check_cuda(cudaGetLastError(), "wait probe launch");
    count_launch();
  });
}

extern "C" int32_t nca_stencil3d(const nca_view* src, const nca_view* dst, const double* weights27, double dt,
                                 void* stream) {
  return nca::guarded([&] { run(src, dst, weights27, dt, 1, (cudaStream_t)stream); });
}

extern "C" int32_t nca_stencil3d_iterate(const nca_view* a, const nca_view* b, const double* weights27, double dt,
                                         int32_t iters, void* stream) {
  return nca::guarded([&] { run(a, b, weights27, dt, iters, (cudaStream_t)stream); });
}
