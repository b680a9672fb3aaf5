// C entry points over ncarray's OWN host code (compiled from the reference's
// sources where they lie, by oracle/Makefile, into oracle/_ref/libncref.so).
// Test infrastructure only: the parity tests call these to pin the oracle
// restatement against the reference implementation on small inputs.
//
// Expressions run through the reference's stack VM exactly as HostEngine's
// non-linearizable branch does (src/lib/ncarray/engines/hostengine.hh:76-145):
// ExprMVNode -> get_dynamic_mv_node -> host::execute_expression_recursive.
// (The asmjit path is not built: asmjit is not vendored.) Reductions call the
// public ArrayImpl members (array_operations.hh:512-1092).
#include "ncarray/array_impl.hh"
#include "ncarray/array_operations.hh"

#include <cstdint>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <variant>
#include <vector>

using namespace ncarray;

// The reference's own aliases (src/lib/ncarray/ncarrays.hh:16-18), restated so
// that the templates instantiate here instead of through its extern-template
// translation units.
using NCArrayView = ArrayImpl<NCOffsetsPolicy, ViewPolicy>;
using NCArray = ArrayImpl<NCOffsetsPolicy, OwnerPolicy>;

// asmjit is absent: the linearizable host path must never be taken here.
namespace ncarray {
namespace host {
RuntimeCompiler& RuntimeCompiler::instance() {
  throw std::runtime_error("asmjit host JIT is not vendored with the reference sources");
}
ExprKernelFunc RuntimeCompiler::get_expr_kernel(DType, DType, DType, const SOArrayPolicy&,
                                                const std::vector<Instruction>&,
                                                const std::vector<SOArrayPolicy>&,
                                                const std::vector<Scalar>&, bool) {
  throw std::runtime_error("asmjit host JIT is not vendored with the reference sources");
}
}  // namespace host
}  // namespace ncarray

static thread_local std::string g_err;

static Scalar make_scalar(int dt, uint64_t slot) {
  auto rd = [&](auto tag) {
    using T = decltype(tag);
    T v;
    std::memcpy(&v, &slot, sizeof(T));
    return Scalar(v);
  };
  switch ((DType)dt) {
    case DType::bool_: return Scalar((slot & 0xff) != 0);
    case DType::char_: return rd(char{});
    case DType::uint8: return rd(std::uint8_t{});
    case DType::uint16: return rd(std::uint16_t{});
    case DType::uint32: return rd(std::uint32_t{});
    case DType::uint64: return rd(std::uint64_t{});
    case DType::int8: return rd(std::int8_t{});
    case DType::int16: return rd(std::int16_t{});
    case DType::int32: return rd(std::int32_t{});
    case DType::int64: return rd(std::int64_t{});
    case DType::float32: return rd(float{});
    case DType::float64: return rd(double{});
    default: throw std::runtime_error("scalar dtype not supported by the reference driver");
  }
}

static NCArrayView make_view(void* data, int dt, int ndim, const int64_t* shape, const int64_t* strides) {
  std::vector<ssize_t> sh(shape, shape + ndim), st(strides, strides + ndim);
  return NCArrayView(data, (ssize_t)ndim, sh.data(), st.data(), (DType)dt, -1, false);
}

// writes a Scalar's value into an 8-byte slot and returns its dtype
static int put_scalar(const Scalar& s, void* out) {
  return std::visit([&](auto&& v) -> int {
    using T = std::decay_t<decltype(v)>;
    if constexpr (sizeof(T) <= 8 && std::is_trivially_copyable_v<T>) {
      std::memset(out, 0, 8);
      std::memcpy(out, &v, sizeof(T));
      return (int)dtype_traits<T>::value;
    } else {
      throw std::runtime_error("result type does not fit the slot");
    }
  }, s);
}

template <int NDim, typename DestT>
static void run_vm(const ExprMVNode<HostTag>& expr, NCArrayView& result) {
  auto bytes = bytes_for_dynamic_vm(expr);
  std::vector<std::uint8_t, host::impl::AlignedAllocator<std::uint8_t>> buf(bytes);
  auto vm = get_dynamic_mv_node(expr, buf.data());
  using CoordsT = StaticCoords<NDim, ssize_t>;
  const ssize_t limit = result.shape(0);
  for (ssize_t i = 0; i < limit; ++i) {
    CoordsT coords;
    coords[0] = i;
    if constexpr (NDim > 1) {
      host::execute_expression_recursive<DestT, CoordsT>(vm, result, coords, 1);
    } else {
      result[coords] = vm.template eval<DestT>(coords);
    }
  }
}

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

// out (C-contiguous, dtype out_dtype, shape out_shape) = tape over the views.
int ref_expr_eval(const uint32_t* instrs, int n_instrs, int n_arrays, void* const* data,
                  const int* dtypes, const int* ndims, const int64_t* shapes,
                  const int64_t* strides, int n_scalars, const int* scalar_dtypes,
                  const uint64_t* scalar_slots, int work_dtype, int expr_dtype, void* out,
                  int out_ndim, const int64_t* out_shape) {
  try {
    std::vector<NCArrayView> views;
    ExprMVNode<HostTag> e;
    for (int k = 0; k < n_arrays; ++k) {
      views.push_back(make_view(data[k], dtypes[k], ndims[k], shapes + 10 * k, strides + 10 * k));
    }
    for (int k = 0; k < n_arrays; ++k) {
      e.layouts.push_back(reinterpret_cast<const SOArrayPolicy&>(views[k]));
      e.dtypes.push_back((DType)dtypes[k]);
      e.data.push_back(views[k].data());
    }
    e.soarray = false;
    for (int i = 0; i < n_instrs; ++i) e.instrs.push_back(instrs[i]);
    for (int i = 0; i < n_scalars; ++i) e.scalars.push_back(make_scalar(scalar_dtypes[i], scalar_slots[i]));
    e.work_dtype = (DType)work_dtype;
    e.expr_dtype = (DType)expr_dtype;
    e.has_expr_dtype = true;
    e.final_shape.set(out_shape, out_ndim);
    ssize_t n = 1;
    for (int d = 0; d < out_ndim; ++d) n *= out_shape[d];
    e.final_size = n;
    std::vector<int64_t> ost(out_ndim);
    int64_t acc = itemsize((DType)expr_dtype);
    for (int d = out_ndim - 1; d >= 0; --d) { ost[d] = acc; acc *= out_shape[d]; }
    NCArrayView result = make_view(out, expr_dtype, out_ndim, out_shape, ost.data());
    auto go = [&]<typename DestT>() {
      switch (out_ndim) {
        case 1: run_vm<1, DestT>(e, result); break;
        case 2: run_vm<2, DestT>(e, result); break;
        case 3: run_vm<3, DestT>(e, result); break;
        case 4: run_vm<4, DestT>(e, result); break;
        case 5: run_vm<5, DestT>(e, result); break;
        default: throw std::runtime_error("ndim 1..5 supported by ref_driver");
      }
    };
    switch ((DType)expr_dtype) {
      case DType::bool_: go.operator()<bool>(); break;
      case DType::char_: go.operator()<char>(); break;
      case DType::uint8: go.operator()<std::uint8_t>(); break;
      case DType::uint16: go.operator()<std::uint16_t>(); break;
      case DType::uint32: go.operator()<std::uint32_t>(); break;
      case DType::uint64: go.operator()<std::uint64_t>(); break;
      case DType::int8: go.operator()<std::int8_t>(); break;
      case DType::int16: go.operator()<std::int16_t>(); break;
      case DType::int32: go.operator()<std::int32_t>(); break;
      case DType::int64: go.operator()<std::int64_t>(); break;
      case DType::float32: go.operator()<float>(); break;
      case DType::float64: go.operator()<double>(); break;
      default: throw std::runtime_error("expr dtype not supported by ref_driver");
    }
    return 0;
  } catch (const std::exception& ex) {
    g_err = ex.what();
    return 1;
  }
}

// op: 0 sum, 1 mean, 2 max, 3 min, 4 argmax, 5 argmin. Writes the scalar into
// *out (8 bytes) and its dtype into *out_dtype.
int ref_reduce_full(void* data, int dtype, int ndim, const int64_t* shape, const int64_t* strides,
                    int op, void* out, int* out_dtype) {
  try {
    NCArrayView v = make_view(data, dtype, ndim, shape, strides);
    Scalar s;
    switch (op) {
      case 0: s = v.sum(); break;
      case 1: s = v.mean(); break;
      case 2: s = v.max(); break;
      case 3: s = v.min(); break;
      case 4: s = v.argmax(); break;
      case 5: s = v.argmin(); break;
      default: throw std::runtime_error("bad op");
    }
    *out_dtype = put_scalar(s, out);
    return 0;
  } catch (const std::exception& ex) {
    g_err = ex.what();
    return 1;
  }
}

// Axis reduction through ArrayImpl::sum/max/min(axes); the result (an owner,
// C-contiguous) is copied into out, its dtype into *out_dtype, its element
// count into *out_n. op: 0 sum, 2 max, 3 min.
int ref_reduce_axes(void* data, int dtype, int ndim, const int64_t* shape, const int64_t* strides,
                    uint32_t axes_mask, int op, void* out, int64_t out_cap_bytes, int* out_dtype,
                    int64_t* out_n) {
  try {
    NCArrayView v = make_view(data, dtype, ndim, shape, strides);
    std::vector<ssize_t> axes;
    for (int d = 0; d < ndim; ++d) if ((axes_mask >> d) & 1u) axes.push_back(d);
    NCArray r;
    switch (op) {
      case 0: r = v.sum(axes); break;
      case 2: r = v.max(axes); break;
      case 3: r = v.min(axes); break;
      default: throw std::runtime_error("axis op not pinned by ref_driver");
    }
    const int64_t bytes = (int64_t)r.size() * (int64_t)r.itemsize();
    if (bytes > out_cap_bytes) throw std::runtime_error("output buffer too small");
    std::memcpy(out, r.data(), (size_t)bytes);
    *out_dtype = (int)r.dtype();
    *out_n = (int64_t)r.size();
    return 0;
  } catch (const std::exception& ex) {
    g_err = ex.what();
    return 1;
  }
}

// dest (1-D view, dtype dest_dtype) += src scattered by indices through the
// reference's host::scatter_add_recursive (src/lib/ncarray/host/elementwise.hh:
// 482-505): for every element i of src in index order, when 0 <= idx[i] <
// dest.size(), dest[idx[i]] += cast<DestT>(src[i]). indices and src are views
// of equal shape (ndim, shape, byte strides).
int ref_scatter_add(void* dest, int dest_dtype, int64_t dest_n, int64_t dest_stride,
                    const void* idx, int idx_dtype, const void* src, int src_dtype, int ndim,
                    const int64_t* shape, const int64_t* idx_strides, const int64_t* src_strides) {
  try {
    NCArrayView d = make_view(dest, dest_dtype, 1, &dest_n, &dest_stride);
    NCArrayView ix = make_view(const_cast<void*>(idx), idx_dtype, ndim, shape, idx_strides);
    NCArrayView sv = make_view(const_cast<void*>(src), src_dtype, ndim, shape, src_strides);
    auto with_src = [&]<typename DestT, typename IndexT>() {
      switch ((DType)src_dtype) {
        case DType::bool_: host::scatter_add_recursive<DestT, IndexT, bool>(d, ix, sv); break;
        case DType::uint8: host::scatter_add_recursive<DestT, IndexT, std::uint8_t>(d, ix, sv); break;
        case DType::int16: host::scatter_add_recursive<DestT, IndexT, std::int16_t>(d, ix, sv); break;
        case DType::int32: host::scatter_add_recursive<DestT, IndexT, std::int32_t>(d, ix, sv); break;
        case DType::uint32: host::scatter_add_recursive<DestT, IndexT, std::uint32_t>(d, ix, sv); break;
        case DType::int64: host::scatter_add_recursive<DestT, IndexT, std::int64_t>(d, ix, sv); break;
        case DType::uint64: host::scatter_add_recursive<DestT, IndexT, std::uint64_t>(d, ix, sv); break;
        case DType::float32: host::scatter_add_recursive<DestT, IndexT, float>(d, ix, sv); break;
        case DType::float64: host::scatter_add_recursive<DestT, IndexT, double>(d, ix, sv); break;
        default: throw std::runtime_error("src dtype not supported by ref_scatter_add");
      }
    };
    auto with_idx = [&]<typename DestT>() {
      switch ((DType)idx_dtype) {
        case DType::int32: with_src.template operator()<DestT, std::int32_t>(); break;
        case DType::int64: with_src.template operator()<DestT, std::int64_t>(); break;
        case DType::uint32: with_src.template operator()<DestT, std::uint32_t>(); break;
        case DType::uint64: with_src.template operator()<DestT, std::uint64_t>(); break;
        default: throw std::runtime_error("index dtype not supported by ref_scatter_add");
      }
    };
    switch ((DType)dest_dtype) {
      case DType::int32: with_idx.operator()<std::int32_t>(); break;
      case DType::uint32: with_idx.operator()<std::uint32_t>(); break;
      case DType::int64: with_idx.operator()<std::int64_t>(); break;
      case DType::uint64: with_idx.operator()<std::uint64_t>(); break;
      case DType::float32: with_idx.operator()<float>(); break;
      case DType::float64: with_idx.operator()<double>(); break;
      default: throw std::runtime_error("dest dtype not supported by ref_scatter_add");
    }
    return 0;
  } catch (const std::exception& ex) {
    g_err = ex.what();
    return 1;
  }
}

}  // extern "C"
