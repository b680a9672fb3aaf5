// Host <-> device copies of strided views (nca_copy_host).
//
// The reference moves arrays between host and device through
// GPUEngine::execute_copy_into (src/lib/ncarray/engines/gpuengine.hh:378-510):
// one synchronous cudaMemcpy when the array is contiguous, otherwise a packing
// kernel into a contiguous buffer first. Here a pair of views of equal shape
// and dtype, each contiguous along its innermost axis, is copied on the
// caller's stream with no staging: axes that both views allow are merged, the
// innermost run becomes the width of a 2-D copy and the next axis its height;
// any further axes loop over 2-D copies. With pinned host memory the copies
// are asynchronous.
#include <cuda_runtime.h>

#include <cstdint>

#include "common.hpp"

extern "C" int32_t nca_copy_host(const nca_view* src, const nca_view* dst, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!dst || !src) fail(NCA_ERR_INVALID, "null view");
    if (dst->dtype != src->dtype) fail(NCA_ERR_DTYPE, "host-device copies keep the dtype (%d vs %d)", src->dtype, dst->dtype);
    if (!dtype_valid(src->dtype)) fail(NCA_ERR_DTYPE, "dtype %d", src->dtype);
    if (dst->ndim != src->ndim || dst->ndim < 0 || dst->ndim > NCA_MAX_NDIM) fail(NCA_ERR_SHAPE, "views differ in rank");
    if (dst->pointer_axis >= 0 || src->pointer_axis >= 0) fail(NCA_ERR_UNSUPPORTED, "pointer axes");
    const int64_t isz = dtinfo(src->dtype).size;
    // canonical dims: extent > 1, (dst stride, src stride), outer to inner
    int nd = 0;
    int64_t ext[NCA_MAX_NDIM], sd[NCA_MAX_NDIM], ss[NCA_MAX_NDIM];
    int64_t n = 1;
    for (int d = 0; d < src->ndim; ++d) {
      if (dst->shape[d] != src->shape[d] || src->shape[d] < 0) fail(NCA_ERR_SHAPE, "views differ in shape on axis %d", d);
      n *= src->shape[d];
      if (src->shape[d] == 1) continue;
      if (dst->strides[d] <= 0 || src->strides[d] <= 0)
        fail(NCA_ERR_UNSUPPORTED, "host-device copies take positive strides (axis %d)", d);
      ext[nd] = src->shape[d]; sd[nd] = dst->strides[d]; ss[nd] = src->strides[d]; ++nd;
    }
    if (n == 0) return;
    if (!dst->data || !src->data) fail(NCA_ERR_INVALID, "null data");
    char* dp = static_cast<char*>(dst->data);
    const char* sp = static_cast<const char*>(src->data);
    for (int d = 0; d < dst->ndim; ++d) { dp += dst->offsets[d]; sp += src->offsets[d]; }
    // merge an axis into the next inner one where both views allow it
    for (int i = nd - 2; i >= 0; --i) {
      if (sd[i] == sd[i + 1] * ext[i + 1] && ss[i] == ss[i + 1] * ext[i + 1]) {
        ext[i] *= ext[i + 1];
        sd[i] = sd[i + 1];
        ss[i] = ss[i + 1];
        for (int j = i + 1; j + 1 < nd; ++j) { ext[j] = ext[j + 1]; sd[j] = sd[j + 1]; ss[j] = ss[j + 1]; }
        --nd;
      }
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (nd == 0) {   // a single element
      check_cuda(cudaMemcpyAsync(dp, sp, (size_t)isz, cudaMemcpyDefault, s), "copy");
      return;
    }
    if (sd[nd - 1] != isz || ss[nd - 1] != isz)
      fail(NCA_ERR_UNSUPPORTED, "both views must be contiguous along the innermost axis; copy through a contiguous array");
    const size_t width = (size_t)(ext[nd - 1] * isz);
    if (nd == 1) {
      check_cuda(cudaMemcpyAsync(dp, sp, width, cudaMemcpyDefault, s), "copy");
      return;
    }
    const int h = nd - 2;   // rows axis
    if (sd[h] < (int64_t)width || ss[h] < (int64_t)width) fail(NCA_ERR_UNSUPPORTED, "overlapping rows");
    int64_t outer = 1;
    for (int d = 0; d < h; ++d) outer *= ext[d];
    if (outer > (1 << 20)) fail(NCA_ERR_LIMIT, "too many 2-D copies (%lld); merge the outer axes first", (long long)outer);
    for (int64_t o = 0; o < outer; ++o) {
      int64_t rem = o, od = 0, os = 0;
      for (int d = h - 1; d >= 0; --d) { const int64_t c = rem % ext[d]; rem /= ext[d]; od += c * sd[d]; os += c * ss[d]; }
      check_cuda(cudaMemcpy2DAsync(dp + od, (size_t)sd[h], sp + os, (size_t)ss[h], width, (size_t)ext[h],
                                   cudaMemcpyDefault, s),
                 "2-D copy");
    }
  });
}
