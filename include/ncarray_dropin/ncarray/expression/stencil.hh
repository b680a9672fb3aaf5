/*
 * Drop-in Stencil<NDIM> for ncarray v0.7.8 backed by libncgb300's nca_stencil.
 *
 * Same interface and include guard as ncarray's expression/stencil.hh
 * (src/lib/ncarray/expression/stencil.hh:58-255): create() takes the offsets,
 * the pointer-axis flags and a lambda that builds an expression over one
 * placeholder view per offset; apply(src, dest, stream) evaluates
 *   dest[c] = expr(src[c*step + o_0], src[c*step + o_1], ...),  step = src.shape / dest.shape.
 * As in the reference's generated kernel (jit/device/rtcompiler.hh:187-385),
 * the k-th array load of the expression reads the view of offsets[k], and float
 * expressions are evaluated in their work dtype. apply() without a stream
 * synchronises the device; with a stream it does not, so it can be captured in
 * a CUDA graph (stencil.hh:166-173,236-242).
 * Differences, by design: every read is checked against the source's extents
 * (std::runtime_error instead of an out-of-bounds read), and StencilJITExtensions
 * code strings and extra kernel arguments are not supported (they throw).
 */
#ifndef NCARRAY_EXPRESSION_STENCIL_HH
#define NCARRAY_EXPRESSION_STENCIL_HH

#include "ncarray/array_impl.hh"
#include "ncarray/engines/gpuengine.hh"
#include "ncarray/expression/interface.hh"
#include "ncarray/expression/mvnode.hh"
#include "ncarray/indexing.hh"
#include "ncarray/jit/device/extensions.hh"

#include "ncgb300.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <optional>
#include <stdexcept>
#include <vector>

namespace ncarray {
  template <int NDIM>
  class Stencil {
  public:
    Stencil() = default;

    template <typename SrcT, typename Func>
    static Stencil<NDIM> create(const std::vector<StaticCoords<NDIM>>& offsets_in,
                                const std::vector<std::uint8_t>& is_pointer_axis,
                                Func&& op_func,
                                const device::StencilJITExtensions& ext = {},
                                bool is_soarr = false) {
      if (!ext.extra_params.empty() || !ext.prologue_code.empty() || !ext.epilogue_code.empty())
        throw std::runtime_error("StencilJITExtensions code is not supported by the GB300 stencil");
      Stencil s;
      s.m_pointer_axis = is_pointer_axis;
      s.m_soarr = is_soarr;
      for (const auto& o : offsets_in)
        for (int d = 0; d < NDIM; ++d) s.m_offsets.push_back(static_cast<int64_t>(o[d]));
      s.m_n = static_cast<int32_t>(offsets_in.size());

      ssize_t unit[NDIM];
      for (int i = 0; i < NDIM; ++i) unit[i] = 1;
      Metadata meta;
      meta.set(unit, NDIM);
      std::vector<NCViewFor<DevTag>> placeholders;
      for (std::size_t i = 0; i < offsets_in.size(); ++i)
        placeholders.push_back(NCViewFor<DevTag>(nullptr, meta, meta, meta, dtype_traits<SrcT>::value, -1, false));
      ExprMVNode<DevTag> expr = op_func(placeholders);

      const DType work = expr.work_dtype;
      const bool float_work = work == DType::float32 || work == DType::float64;
      s.m_tape = gb300::to_tape(expr, float_work ? static_cast<int>(work) : -1);
      // the k-th array load reads offsets[k]
      int k = 0;
      for (auto& ins : s.m_tape.instrs)
        if (get_op(ins) == OpCode::LOAD_NCARR || get_op(ins) == OpCode::LOAD_SOARR)
          ins = (static_cast<std::uint32_t>(get_op(ins)) << 24) | static_cast<std::uint32_t>(k++);
      s.m_expr_dtype = expr.dtype();
      return s;
    }

    template <ViewArrayLike Src, OwningArrayLike Dest, typename... Args>
    void apply(const Src& src, Dest& dest, std::optional<cudaStream_t> stream = std::nullopt,
               Args&&... extra_args) {
      static_assert(sizeof...(Args) == 0, "extra kernel arguments are not supported by the GB300 stencil");
      for (int d = 0; d < NDIM && d < static_cast<int>(m_pointer_axis.size()); ++d)
        if (static_cast<bool>(m_pointer_axis[d]) != src.is_pointer_axis(d))
          throw std::runtime_error("the source's pointer axes differ from those the stencil was created for");
      nca_view sv = gb300::to_view(src);
      nca_view dv = gb300::to_view(dest);
      cudaStream_t s = stream.has_value() ? *stream : nullptr;
      nca_tape t = m_tape.tape;   // storage pointers of this object (it may have been copied)
      t.instrs = m_tape.instrs.data();
      t.scalar_dtypes = m_tape.scalar_dtypes.data();
      t.scalar_slots = m_tape.scalar_slots.data();
      gb300::check(nca_stencil(&sv, &dv, m_offsets.data(), m_n, &t, s), "GB300 stencil");
      if (!stream.has_value()) gb300::check_cuda(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    }

    /// The tape this stencil evaluates (for inspection and tests).
    const gb300::TapeHolder& tape() const { return m_tape; }
    const std::vector<int64_t>& flat_offsets() const { return m_offsets; }

  private:
    std::vector<int64_t> m_offsets;
    std::vector<std::uint8_t> m_pointer_axis;
    gb300::TapeHolder m_tape;
    int32_t m_n = 0;
    bool m_soarr = false;
    DType m_expr_dtype = DType::float32;
  };
}  // namespace ncarray

#endif  // NCARRAY_EXPRESSION_STENCIL_HH
