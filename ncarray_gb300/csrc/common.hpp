// Shared host-side plumbing of libncgb300: error state, dtype table, CUDA
// driver entry points (resolved through cudart, so the library loads on a
// machine without libcuda.so.1), and device properties.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/ncgb300.h"

namespace nca {

// Internal error: thrown inside the library, converted to a status code at the
// C ABI boundary (no exception crosses it).
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const char* fmt, ...);
void set_last_error(const std::string& msg);
void clear_last_error();
// message of the last failed call on this thread (valid until the next call)
const std::string& last_error();

// Runs f, mapping exceptions to status codes.
template <class F>
int32_t guarded(F&& f) {
  try {
    clear_last_error();
    f();
    return NCA_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return NCA_ERR_OOM;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return NCA_ERR_INVALID;
  } catch (...) {
    set_last_error("unknown error");
    return NCA_ERR_INVALID;
  }
}

void check_cuda(cudaError_t e, const char* what);
void check_cu(CUresult r, const char* what);

// ---- dtypes ----------------------------------------------------------------
struct DTypeInfo {
  const char* name;
  const char* ctype;   // C type in generated device code (storage type)
  int size;
  bool is_float;       // float32/float64/bfloat16/float16
  bool is_signed;
  bool device_ok;      // usable on the device path
};
const DTypeInfo& dtinfo(int dt);
bool dtype_valid(int dt);
// float32 stands in for the 16-bit float storage types in arithmetic
inline int arith_dtype(int dt) { return (dt == NCA_BFLOAT16 || dt == NCA_FLOAT16) ? NCA_FLOAT32 : dt; }
// op_traits<T>::sum_type (src/lib/ncarray/op_traits.hh:72-76,380-410); 16-bit floats -> float32
int sum_dtype(int dt);

// ---- driver API through cudart -----------------------------------------------
struct Driver {
  CUresult (*cuModuleLoadData)(CUmodule*, const void*);
  CUresult (*cuModuleGetFunction)(CUfunction*, CUmodule, const char*);
  CUresult (*cuLaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned,
                             unsigned, unsigned, CUstream, void**, void**);
  CUresult (*cuFuncSetAttribute)(CUfunction, CUfunction_attribute, int);
  CUresult (*cuOccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t);
  CUresult (*cuGetErrorString)(CUresult, const char**);
  CUresult (*cuTensorMapEncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                     const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                     const cuuint32_t*, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion,
                                     CUtensorMapFloatOOBfill);
};
const Driver& drv();

// Number of kernels this library has launched (all entry points).
void count_launch(int64_t n = 1);
int64_t launch_count();

// Current device (initialising its primary context) and its SM count.
int current_device();
int sm_count(int dev);

// Stream-ordered scratch (cudaMallocAsync) freed at scope exit on the same stream.
struct StreamScratch {
  void* ptr = nullptr;
  cudaStream_t stream = nullptr;
  StreamScratch() = default;
  StreamScratch(size_t bytes, cudaStream_t s);
  ~StreamScratch();
  StreamScratch(const StreamScratch&) = delete;
  StreamScratch& operator=(const StreamScratch&) = delete;
};

}  // namespace nca
