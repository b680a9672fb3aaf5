// Entry points whose kernels are not in this build yet: they report
// NCA_ERR_UNSUPPORTED so that callers fail loudly.
#include "common.hpp"

using namespace nca;

extern "C" {
int32_t nca_stencil3d(const nca_view*, const nca_view*, const double*, double, void*) {
  return guarded([] { fail(NCA_ERR_UNSUPPORTED, "nca_stencil3d is not built yet"); });
}
int32_t nca_stencil3d_iterate(const nca_view*, const nca_view*, const double*, double, int32_t, void*) {
  return guarded([] { fail(NCA_ERR_UNSUPPORTED, "nca_stencil3d_iterate is not built yet"); });
}
int32_t nca_hist2d(const float*, const float*, const float*, int64_t, int32_t, int32_t, double, double,
                   double, double, uint64_t*, float*, void*) {
  return guarded([] { fail(NCA_ERR_UNSUPPORTED, "nca_hist2d is not built yet"); });
}
int32_t nca_batch_create(const nca_batch_item*, int32_t, nca_batch**, void*) {
  return guarded([] { fail(NCA_ERR_UNSUPPORTED, "batched reductions are not built yet"); });
}
int32_t nca_batch_reduce(nca_batch*, nca_batch_result*, void*) { return NCA_ERR_UNSUPPORTED; }
int32_t nca_batch_reduce_graph(nca_batch*, nca_batch_result*, void*) { return NCA_ERR_UNSUPPORTED; }
int32_t nca_batch_reduce_plain(nca_batch*, nca_batch_result*, void*) { return NCA_ERR_UNSUPPORTED; }
int32_t nca_batch_autotune(nca_batch*, nca_batch_result*, void*) { return NCA_ERR_UNSUPPORTED; }
int32_t nca_batch_schedule(const nca_batch*, int64_t*, int32_t*, int32_t*, int32_t*) { return NCA_ERR_UNSUPPORTED; }
int32_t nca_batch_status(nca_batch*, int32_t*, void*) { return NCA_ERR_UNSUPPORTED; }
void nca_batch_destroy(nca_batch*) {}
}
