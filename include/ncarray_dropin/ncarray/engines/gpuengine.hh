/*
 * Drop-in GPUEngine for ncarray v0.7.8 backed by libncgb300 (include/ncgb300.h).
 *
 * ncarray sends every device operation through the static templates of
 * ncarray::GPUEngine (src/lib/ncarray/engines/gpuengine.hh:64-638), called from
 * array_operations.hh (expression assignment :42-63, axis reductions :512-895,
 * full reductions :904-1090, copies :1105) and from the Python bindings built
 * on it (pyncarray/binding_builder.hh). This header defines the same struct
 * with the same signatures and include guard, so placing its directory before
 * ncarray's own on the include path (or copying it over
 * src/lib/ncarray/engines/gpuengine.hh) routes ncarray's C++ API and its
 * _pyncdevarray module through the GB300 kernels, with no change to ncarray's
 * sources. Link with -lncgb300.
 *
 * Behaviour kept from the reference: every call is synchronous on the legacy
 * default stream; failures throw std::runtime_error (here with the library's
 * message). Behaviour that differs, by design: mean() divides by the count
 * (the reference returns the sum: reductions.hh:343-381), axis argmax/argmin
 * give the index along the reduced axes, float32 sums are compensated, and
 * var/std/all/any are not provided on the device (they throw).
 */
#ifndef NCARRAY_ENGINES_GPUENGINE_HH
#define NCARRAY_ENGINES_GPUENGINE_HH

#include "ncarray/array_impl.hh"
#include "ncarray/array_traits.hh"
#include "ncarray/custom_types.hh"
#include "ncarray/device/mem_pool.cuh"
#include "ncarray/device/utilities.cuh"
#include "ncarray/engines/hostengine.hh"
#include "ncarray/expression/dynamicmvnode.hh"
#include "ncarray/expression/mvnode.hh"
#include "ncarray/expression/staticmvnode.hh"
#include "ncarray/indexing.hh"
#include "ncarray/layout.hh"
#include "ncarray/op_traits.hh"
#include "ncarray/reductions.hh"

#include "ncgb300.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <variant>
#include <vector>

namespace ncarray {
  namespace gb300 {
    /// Throws the library's message when a C-ABI call fails.
    inline void check(int32_t status, const char* what) {
      if (status != NCA_OK) {
        const char* msg = nca_last_error();
        throw std::runtime_error(std::string(what) + ": " + (msg ? msg : "unknown error"));
      }
    }

    inline void check_cuda(cudaError_t e, const char* what) {
      if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }

    /// A layout (NC offsets or PEP 3118 suboffsets) over `data` as an nca_view.
    template <class Layout>
    nca_view layout_view(const Layout& l, const void* data, DType dtype, bool soarray) {
      nca_view v;
      std::memset(&v, 0, sizeof(v));
      v.data = const_cast<void*>(data);
      v.dtype = static_cast<int32_t>(dtype);
      v.ndim = static_cast<int32_t>(l.ndim());
      v.pointer_axis = -1;
      if (v.ndim > NCA_MAX_NDIM) throw std::runtime_error("more dims than the GB300 engine supports");
      for (int d = 0; d < v.ndim; ++d) {
        v.shape[d] = l.shape(d);
        v.strides[d] = l.strides()[d];
        const bool ptr = l.is_pointer_axis(d);
        if (ptr) {
          if (v.pointer_axis >= 0) throw std::runtime_error("the GB300 engine takes one pointer axis per array");
          v.pointer_axis = d;
        }
        if (soarray) {
          // suboffsets: -1 on ordinary axes, the post-read offset on the pointer axis
          v.offsets[d] = ptr ? l.get_offset(d) : 0;
        } else {
          v.offsets[d] = l.get_offset(d);
        }
      }
      if (soarray && v.pointer_axis >= 0) v.flags = NCA_VIEW_SUBOFFSETS;
      return v;
    }

    /// An ncarray array (owner, view or ref; NC or SO layout) as an nca_view.
    template <class A>
    nca_view to_view(const A& arr) {
      using L = typename std::remove_cvref_t<A>::LayoutPolicy;
      return layout_view(arr, arr.data(), arr.dtype(), std::is_same_v<L, SOArrayPolicy>);
    }

    /// A C-contiguous view of `n` elements of dtype `dt` at `data` with `arr`'s shape.
    template <class A>
    nca_view contiguous_like(const A& arr, void* data, DType dt) {
      nca_view v;
      std::memset(&v, 0, sizeof(v));
      v.data = data;
      v.dtype = static_cast<int32_t>(dt);
      v.ndim = static_cast<int32_t>(arr.ndim());
      v.pointer_axis = -1;
      int64_t acc = static_cast<int64_t>(itemsize(dt));
      for (int d = v.ndim - 1; d >= 0; --d) {
        v.shape[d] = arr.shape(d);
        v.strides[d] = acc;
        acc *= arr.shape(d);
      }
      return v;
    }

    /// The value of an ncarray Scalar as (dtype, 8-byte slot).
    inline void scalar_slot(const Scalar& s, int32_t* dtype, uint64_t* slot) {
      std::visit([&](auto&& v) {
        using T = std::decay_t<decltype(v)>;
        if constexpr (std::is_arithmetic_v<T> && sizeof(T) <= 8 && !std::is_same_v<T, long double>) {
          *slot = 0;
          std::memcpy(slot, &v, sizeof(T));
          *dtype = static_cast<int32_t>(dtype_traits<T>::value);
        } else {
          throw std::runtime_error("scalar type not supported by the GB300 engine");
        }
      }, s);
    }

    /// An ExprMVNode's RPN tape with the storage its nca_tape points into.
    struct TapeHolder {
      std::vector<uint32_t> instrs;
      std::vector<int32_t> scalar_dtypes;
      std::vector<uint64_t> scalar_slots;
      nca_tape tape;
    };

    inline bool is_float(DType d) { return d == DType::float32 || d == DType::float64; }

    /// The tape of `expr`; every value is evaluated in the VM's compute type
    /// (the expression dtype, or the work dtype for bool results:
    /// dynamicmvnode.hh:146-251), or in `compute_override` when given.
    template <class Expr>
    TapeHolder to_tape(const Expr& expr, int compute_override = -1) {
      TapeHolder h;
      h.instrs.assign(expr.instrs.begin(), expr.instrs.end());
      for (const auto& s : expr.scalars) {
        int32_t dt;
        uint64_t slot;
        scalar_slot(s, &dt, &slot);
        h.scalar_dtypes.push_back(dt);
        h.scalar_slots.push_back(slot);
      }
      const DType ed = expr.dtype();
      const DType compute = ed == DType::bool_ ? expr.work_dtype : ed;
      std::memset(&h.tape, 0, sizeof(h.tape));
      h.tape.instrs = h.instrs.data();
      h.tape.n_instrs = static_cast<int32_t>(h.instrs.size());
      h.tape.n_scalars = static_cast<int32_t>(h.scalar_slots.size());
      h.tape.scalar_dtypes = h.scalar_dtypes.data();
      h.tape.scalar_slots = h.scalar_slots.data();
      h.tape.compute_dtype = compute_override >= 0 ? compute_override : static_cast<int32_t>(compute);
      h.tape.result_dtype = static_cast<int32_t>(ed);
      return h;
    }

    /// The operand views of an ExprMVNode (layouts reinterpreted as stored).
    template <class Expr>
    std::vector<nca_view> operand_views(const Expr& expr) {
      std::vector<nca_view> ops;
      for (std::size_t i = 0; i < expr.layouts.size(); ++i) {
        if (expr.soarray) {
          ops.push_back(layout_view(expr.layouts[i], expr.data[i], expr.dtypes[i], true));
        } else {
          const auto& nc = reinterpret_cast<const NCOffsetsPolicy&>(expr.layouts[i]);
          ops.push_back(layout_view(nc, expr.data[i], expr.dtypes[i], false));
        }
      }
      return ops;
    }

    /// nca_reduce_op of a reduction traits type, or -1 (not provided).
    template <class Traits>
    constexpr int reduce_op() {
      if constexpr (std::is_same_v<Traits, SumTraits>) return NCA_RED_SUM;
      else if constexpr (std::is_same_v<Traits, MeanTraits>) return NCA_RED_MEAN;
      else if constexpr (std::is_same_v<Traits, MaxTraits>) return NCA_RED_MAX;
      else if constexpr (std::is_same_v<Traits, MinTraits>) return NCA_RED_MIN;
      else if constexpr (std::is_same_v<Traits, ArgmaxTraits>) return NCA_RED_ARGMAX;
      else if constexpr (std::is_same_v<Traits, ArgminTraits>) return NCA_RED_ARGMIN;
      else return -1;
    }

    /// Reduced-axes mask of ReductionParams (an output stride of 0 marks a
    /// reduced axis: build_reduction_params, custom_types.hh:130-176).
    inline uint32_t axes_mask(const ReductionParams& p) {
      uint32_t m = 0;
      for (ssize_t d = 0; d < p.ndim; ++d)
        if (p.strides[d] == 0) m |= 1u << d;
      return m;
    }

    /// Eight bytes of device memory per device for scalar results.
    inline void* scalar_buffer() {
      static std::mutex mu;
      static void* bufs[64] = {nullptr};
      int dev = 0;
      check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
      if (dev < 0 || dev >= 64) throw std::runtime_error("device ordinal out of range");
      std::lock_guard<std::mutex> lk(mu);
      if (!bufs[dev]) check_cuda(cudaMalloc(&bufs[dev], 64), "cudaMalloc(scalar result)");
      return bufs[dev];
    }

    inline bool is_device_pointer(const void* p) {
      cudaPointerAttributes a;
      if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
      }
      return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
    }

    inline void sync() { check_cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize"); }
  }  // namespace gb300

  /**
   * GPUEngine with the reference's interface (engines/gpuengine.hh:64-638),
   * running on libncgb300.
   */
  struct GPUEngine {
    static constexpr bool is_gb300_engine = true;

    /// out = expression (gpuengine.hh:90-195).
    template <typename DestT, class Expr, OwningArrayLike Result>
    static void execute_binary_expression(const Expr& expr, Result& result) {
      if constexpr (is_exprmv_node_v<Expr>) {
        if (result.size() == 0) return;
        gb300::TapeHolder t = gb300::to_tape(expr);
        std::vector<nca_view> ops = gb300::operand_views(expr);
        nca_view out = gb300::to_view(result);
        gb300::check(nca_expr_eval(&t.tape, ops.data(), static_cast<int32_t>(ops.size()), &out, nullptr),
                     "GB300 expression");
        gb300::sync();
      }
    }

    /// Reduction over the axes `params` marks (gpuengine.hh:222-288).
    template <typename SrcT, ReductionTraits<SrcT> Traits, ViewArrayLike Array, ViewArrayLike Result>
    static void execute_reduce_axes(const Array& arr, const ReductionParams& params, Result& res) {
      constexpr int op = gb300::reduce_op<Traits>();
      if constexpr (op < 0) {
        throw std::runtime_error("this reduction is not provided by the GB300 engine");
      } else {
        nca_view src = gb300::to_view(arr);
        nca_view out = gb300::to_view(res);
        gb300::check(nca_reduce(&src, op, gb300::axes_mask(params), &out, nullptr), "GB300 axis reduction");
        gb300::sync();
      }
    }

    /// Reduction of every element to a Scalar (gpuengine.hh:301-333).
    template <typename SrcT, ReductionTraits<SrcT> Traits, class Array>
    static Scalar execute_full_reduce(const Array& arr, double ddof = 0.0) {
      (void)ddof;
      constexpr int op = gb300::reduce_op<Traits>();
      using OutT = typename Traits::template OutT<SrcT>;
      if constexpr (op < 0) {
        throw std::runtime_error("this reduction is not provided by the GB300 engine");
      } else {
        nca_view src = gb300::to_view(arr);
        // the library writes sum_type / float64 (mean) / T / int64 (arg*)
        using LibT = std::conditional_t<op == NCA_RED_MEAN, double, OutT>;
        void* buf = gb300::scalar_buffer();
        nca_view out;
        std::memset(&out, 0, sizeof(out));
        out.data = buf;
        out.dtype = static_cast<int32_t>(dtype_traits<LibT>::value);
        out.ndim = 0;
        out.pointer_axis = -1;
        gb300::check(nca_reduce(&src, op, 0xffffffffu, &out, nullptr), "GB300 reduction");
        LibT v{};
        gb300::check_cuda(cudaMemcpy(&v, buf, sizeof(LibT), cudaMemcpyDeviceToHost), "cudaMemcpy(result)");
        return Scalar{static_cast<OutT>(v)};
      }
    }

    /// arr[...] = val (gpuengine.hh:338-376).
    template <typename T, class ArrayT>
    static void execute_fill(const ArrayT& arr, Scalar val) {
      if constexpr (!std::is_arithmetic_v<T> || sizeof(T) > 8 || std::is_same_v<T, long double>) {
        (void)arr; (void)val;
        throw std::runtime_error("the GB300 engine has no device path for this dtype");
      } else {
        if (arr.size() == 0) return;
        T target = std::visit([](auto&& a) -> T {
          using FromT = std::decay_t<decltype(a)>;
          return op_traits<FromT>::template cast<T>(a);
        }, val);
        uint64_t slot = 0;
        std::memcpy(&slot, &target, sizeof(T));
        nca_view v = gb300::to_view(arr);
        gb300::check(nca_fill(&v, static_cast<int32_t>(dtype_traits<T>::value), &slot, nullptr), "GB300 fill");
        gb300::sync();
      }
    }

    /// Contiguous casting copy of arr into dest, which may be host or device
    /// memory (gpuengine.hh:378-510).
    template <typename SrcT, ArrayLike ArrayT, typename DestT>
    static void execute_copy_into(const ArrayT& arr, DestT* dest) {
      using SrcMemType = typename ArrayT::MemType;
      constexpr bool src_is_dev = std::is_same_v<SrcMemType, DevTag>;
      const bool dest_is_dev = gb300::is_device_pointer(dest);
      const DType ddt = dtype_traits<DestT>::value;
      const std::size_t nbytes = static_cast<std::size_t>(arr.size()) * sizeof(DestT);
      if (arr.size() == 0) return;
      if (src_is_dev) {
        nca_view src = gb300::to_view(arr);
        if (dest_is_dev) {
          nca_view dst = gb300::contiguous_like(arr, dest, ddt);
          gb300::check(nca_copy(&src, &dst, nullptr), "GB300 copy");
          gb300::sync();
        } else {
          void* tmp = nullptr;
          gb300::check_cuda(cudaMallocAsync(&tmp, nbytes, nullptr), "cudaMallocAsync(copy staging)");
          nca_view dst = gb300::contiguous_like(arr, tmp, ddt);
          const int32_t st = nca_copy(&src, &dst, nullptr);
          cudaError_t ce = st == NCA_OK ? cudaMemcpyAsync(dest, tmp, nbytes, cudaMemcpyDeviceToHost, nullptr)
                                        : cudaSuccess;
          cudaFreeAsync(tmp, nullptr);
          gb300::check(st, "GB300 copy");
          gb300::check_cuda(ce, "cudaMemcpyAsync(device to host)");
          gb300::sync();
        }
      } else {
        // host source: packed by ncarray's own host routine, then one copy
        if (dest_is_dev) {
          DestT* h_tmp = nullptr;
          gb300::check_cuda(cudaMallocHost(reinterpret_cast<void**>(&h_tmp), nbytes), "cudaMallocHost");
          DestT* h_ref = h_tmp;
          HostEngine::execute_copy_into<SrcT>(arr, h_ref);
          cudaError_t ce = cudaMemcpy(dest, h_tmp, nbytes, cudaMemcpyHostToDevice);
          cudaFreeHost(h_tmp);
          gb300::check_cuda(ce, "cudaMemcpy(host to device)");
        } else {
          HostEngine::execute_copy_into<SrcT>(arr, dest);
        }
      }
    }

    /// dest[...] = cast(src[...]) between any host/device pair (gpuengine.hh:512-636).
    template <typename DestT, ArrayLike Dest, ArrayLike Src>
    static void execute_assign(Dest& dest, const Src& src) {
      constexpr bool dest_is_dev = std::is_same_v<typename Dest::MemType, DevTag>;
      constexpr bool src_is_dev = std::is_same_v<typename Src::MemType, DevTag>;
      using NCDevArray = NCOwnerFor<DevTag>;
      if (dest.size() == 0) return;
      if constexpr (dest_is_dev && src_is_dev) {
        nca_view s = gb300::to_view(src);
        nca_view d = gb300::to_view(dest);
        gb300::check(nca_copy(&s, &d, nullptr), "GB300 assign");
        gb300::sync();
      } else if constexpr (dest_is_dev) {
        // host to device: a contiguous device copy in dest's dtype, then a strided copy
        NCDevArray tmp(dest.ndim(), dest.shape(), dtype_traits<DestT>::value);
        auto host_dev = [&]<typename SrcT>() {
          GPUEngine::execute_copy_into<SrcT>(src, reinterpret_cast<DestT*>(tmp.data()));
        };
        dispatch(src.dtype(), host_dev);
        nca_view s = gb300::to_view(tmp);
        nca_view d = gb300::to_view(dest);
        gb300::check(nca_copy(&s, &d, nullptr), "GB300 assign");
        gb300::sync();
      } else if constexpr (src_is_dev) {
        // device to host: a contiguous device copy in dest's dtype, then one transfer
        NCDevArray tmp(dest.ndim(), dest.shape(), dtype_traits<DestT>::value);
        nca_view s = gb300::to_view(src);
        nca_view d = gb300::to_view(tmp);
        gb300::check(nca_copy(&s, &d, nullptr), "GB300 assign");
        gb300::sync();
        GPUEngine::execute_copy_into<DestT>(tmp, reinterpret_cast<DestT*>(dest.data()));
      } else {
        HostEngine::execute_copy_into<DestT>(src, dest);
      }
    }
  };
}  // namespace ncarray

#endif  // NCARRAY_ENGINES_GPUENGINE_HH
