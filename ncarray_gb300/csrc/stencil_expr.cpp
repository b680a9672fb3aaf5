// nca_stencil: the general stencil of ncarray's Stencil<NDIM>
// (src/lib/ncarray/expression/stencil.hh:58-255, kernel source generated by
// device::RuntimeCompiler::get_stencil_expr_kernel_str,
// src/lib/ncarray/jit/device/rtcompiler.hh:187-385):
//
//   dest[c] = tape(src[c * step + o_0], ..., src[c * step + o_{k-1}], scalars)
//   step[d] = src.shape[d] / dest.shape[d]   (integer division)
//
// for every coordinate c of dest, with any number of offsets o_i (one per
// tape operand). Each offset becomes one strided view of src (strides scaled
// by step, the offset folded into the view's constant part), so the stencil
// runs through the fused-expression kernels: every operand shares one stride
// set, so the kernels compute one offset per element and add a constant per
// operand; 16-byte vector loads and the stride-2 window loads apply as for
// any expression.
//
// Pointer axes of src: an NC table (layout.hh:468-535) is rewritten as the
// equivalent suboffset view (the table stride becomes step * sizeof(void*),
// the index offset moves into the table base), so a stepped, shifted pointer
// axis needs no new kernel path; SO views (layout.hh:677-778) keep their form.
//
// Differences from the reference, each by design:
//   - every read is checked against src's extents on the host (the reference
//     reads out of bounds when an offset leaves the array); violations return
//     NCA_ERR_SHAPE before anything runs;
//   - the tape is evaluated with the expression engine's rules (the operator
//     set is the full opcode set, not only ADD/SUB/MUL/DIV/GT), in the
//     tape's compute dtype;
//   - the reference's pro/epilogue code strings (StencilJITExtensions,
//     jit/device/extensions.hh:68-72) inject arbitrary CUDA into its kernel;
//     there is no counterpart.
#include <cstring>
#include <vector>

#include "common.hpp"
#include "jit.hpp"

namespace nca {
namespace {

void check_stencil_view(const nca_view& v, const char* what) {
  if (v.ndim < 1 || v.ndim > NCA_MAX_NDIM) fail(NCA_ERR_LIMIT, "%s: ndim %d (1..%d)", what, v.ndim, NCA_MAX_NDIM);
  for (int d = 0; d < v.ndim; ++d)
    if (v.shape[d] < 0) fail(NCA_ERR_SHAPE, "%s: negative extent", what);
}

}  // namespace

// Builds the operand view of offset `o` (ndim values) of src for dest.
nca_view stencil_operand(const nca_view& src, const int64_t* step, const int64_t* o, const nca_view& dest) {
  nca_view v = src;
  const int pa = src.pointer_axis;
  const bool so = (src.flags & NCA_VIEW_SUBOFFSETS) != 0;
  char* data = static_cast<char*>(src.data);
  for (int d = 0; d < src.ndim; ++d) {
    v.shape[d] = dest.shape[d];
    if (d == pa) {
      // the pointer axis: strides the table before the read
      const int64_t tstride = so ? src.strides[d] : (int64_t)sizeof(void*);
      v.strides[d] = tstride * step[d];
      data += so ? o[d] * src.strides[d] : (src.offsets[d] + o[d]) * (int64_t)sizeof(void*);
      v.offsets[d] = so ? src.offsets[d] : 0;   // suboffset after the read
    } else {
      v.strides[d] = src.strides[d] * step[d];
      v.offsets[d] = src.offsets[d] + o[d] * src.strides[d];
    }
  }
  if (pa >= 0) v.flags = NCA_VIEW_SUBOFFSETS;
  v.data = data;
  return v;
}

}  // namespace nca

extern "C" int32_t nca_stencil(const nca_view* src, const nca_view* dest, const int64_t* offsets,
                               int32_t n_offsets, const nca_tape* tape, void* stream) {
  return nca::guarded([&] {
    using namespace nca;
    if (!src || !dest || !tape) fail(NCA_ERR_INVALID, "null argument");
    if (n_offsets < 1 || !offsets) fail(NCA_ERR_INVALID, "a stencil needs at least one offset");
    if (n_offsets > NCA_MAX_OPERANDS)
      fail(NCA_ERR_LIMIT, "%d offsets: at most %d (one operand each)", n_offsets, NCA_MAX_OPERANDS);
    check_stencil_view(*src, "stencil source");
    check_stencil_view(*dest, "stencil destination");
    if (dest->ndim != src->ndim)
      fail(NCA_ERR_SHAPE, "source has %d dims, destination %d", src->ndim, dest->ndim);
    if (dest->pointer_axis >= 0) fail(NCA_ERR_UNSUPPORTED, "the destination cannot have a pointer axis");
    const int nd = src->ndim;
    int64_t step[NCA_MAX_NDIM];
    int64_t dn = 1;
    for (int d = 0; d < nd; ++d) {
      dn *= dest->shape[d];
      if (dest->shape[d] == 0) { step[d] = 1; continue; }
      step[d] = src->shape[d] / dest->shape[d];
      if (step[d] < 1)
        fail(NCA_ERR_SHAPE, "dim %d: destination extent %lld exceeds the source's %lld", d,
             (long long)dest->shape[d], (long long)src->shape[d]);
    }
    // every read src[c * step + o] must be inside src
    for (int i = 0; i < n_offsets; ++i) {
      const int64_t* o = offsets + (int64_t)i * nd;
      for (int d = 0; d < nd && dn > 0; ++d) {
        const int64_t last = (dest->shape[d] - 1) * step[d] + o[d];
        if (o[d] < 0 || last >= src->shape[d])
          fail(NCA_ERR_SHAPE, "offset %d leaves the source on dim %d (reads %lld..%lld of %lld)", i, d,
               (long long)o[d], (long long)last, (long long)src->shape[d]);
      }
    }
    Tape t = make_tape(tape, n_offsets);
    if (dn == 0) return;
    std::vector<nca_view> ops((size_t)n_offsets);
    for (int i = 0; i < n_offsets; ++i) ops[(size_t)i] = stencil_operand(*src, step, offsets + (int64_t)i * nd, *dest);
    expr_eval(t, ops.data(), n_offsets, *dest, (cudaStream_t)stream);
  });
}
