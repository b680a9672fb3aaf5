// Host-side plumbing of libncgb300 (see common.hpp).
#include "common.hpp"

#include <cstdarg>
#include <atomic>
#include <cstdio>
#include <mutex>
#include <vector>

namespace nca {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }
void clear_last_error() { g_last_error.clear(); }
const std::string& last_error() { return g_last_error; }

[[noreturn]] void fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw Error(code, buf);
}

void check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  if (e == cudaErrorMemoryAllocation) fail(NCA_ERR_OOM, "%s: %s", what, cudaGetErrorString(e));
  fail(NCA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void check_cu(CUresult r, const char* what) {
  if (r == CUDA_SUCCESS) return;
  const char* s = "unknown";
  if (drv().cuGetErrorString) drv().cuGetErrorString(r, &s);
  if (r == CUDA_ERROR_OUT_OF_MEMORY) fail(NCA_ERR_OOM, "%s: %s", what, s);
  fail(NCA_ERR_CUDA, "%s: %s (CUresult %d)", what, s, (int)r);
}

// name, ctype, size, is_float, is_signed, device_ok
static const DTypeInfo kDTypes[24] = {
    {"bool", "bool", 1, false, false, true},
    {"char", "signed char", 1, false, true, true},
    {"uint8", "unsigned char", 1, false, false, true},
    {"uint16", "unsigned short", 2, false, false, true},
    {"uint32", "u32", 4, false, false, true},
    {"uint64", "u64", 8, false, false, true},
    {"int8", "signed char", 1, false, true, true},
    {"int16", "short", 2, false, true, true},
    {"int32", "int", 4, false, true, true},
    {"int64", "i64", 8, false, true, true},
    {"float32", "float", 4, true, true, true},
    {"float64", "double", 8, true, true, true},
    {"float128", "", 16, true, true, false},
    {"complex64", "", 8, true, true, false},
    {"complex128", "", 16, true, true, false},
    {"complex256", "", 32, true, true, false},
    {"vfloat2", "", 8, true, true, false},
    {"vfloat3", "", 12, true, true, false},
    {"vfloat4", "", 16, true, true, false},
    {"vdouble2", "", 16, true, true, false},
    {"vdouble3", "", 24, true, true, false},
    {"vdouble4", "", 32, true, true, false},
    {"bfloat16", "unsigned short", 2, true, true, true},
    {"float16", "unsigned short", 2, true, true, true},
};

bool dtype_valid(int dt) { return dt >= 0 && dt < 24 && kDTypes[dt].device_ok; }

const DTypeInfo& dtinfo(int dt) {
  if (dt < 0 || dt >= 24) fail(NCA_ERR_DTYPE, "dtype %d out of range", dt);
  return kDTypes[dt];
}

int sum_dtype(int dt) {
  switch (dt) {
    case NCA_BOOL: case NCA_UINT8: case NCA_UINT16: return NCA_UINT64;
    case NCA_INT8: case NCA_INT16: return NCA_INT64;
    case NCA_BFLOAT16: case NCA_FLOAT16: return NCA_FLOAT32;
    default: return dt;
  }
}

template <class F>
static void resolve(const char* name, F*& fn) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
    fn = nullptr;
    return;
  }
  fn = reinterpret_cast<F*>(p);
}

const Driver& drv() {
  static Driver d = [] {
    Driver r{};
    resolve("cuModuleLoadData", r.cuModuleLoadData);
    resolve("cuModuleGetFunction", r.cuModuleGetFunction);
    resolve("cuLaunchKernel", r.cuLaunchKernel);
    resolve("cuFuncSetAttribute", r.cuFuncSetAttribute);
    resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", r.cuOccupancyMaxActiveBlocksPerMultiprocessor);
    resolve("cuGetErrorString", r.cuGetErrorString);
    resolve("cuTensorMapEncodeTiled", r.cuTensorMapEncodeTiled);
    return r;
  }();
  if (!d.cuModuleLoadData || !d.cuLaunchKernel || !d.cuModuleGetFunction)
    fail(NCA_ERR_CUDA, "CUDA driver entry points unavailable (no GPU driver?)");
  return d;
}

static std::atomic<int64_t> g_launches{0};
void count_launch(int64_t n) { g_launches += n; }
int64_t launch_count() { return g_launches.load(); }

int current_device() {
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  static std::mutex m;
  static std::vector<bool> inited;
  std::lock_guard<std::mutex> lk(m);
  if ((int)inited.size() <= dev) inited.resize(dev + 1, false);
  if (!inited[dev]) {
    check_cuda(cudaFree(nullptr), "cudaFree(0) context init");
    inited[dev] = true;
  }
  return dev;
}

int sm_count(int dev) {
  static std::mutex m;
  static std::vector<int> cache;
  std::lock_guard<std::mutex> lk(m);
  if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
  if (!cache[dev]) {
    int n = 0;
    check_cuda(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev), "SM count");
    cache[dev] = n;
  }
  return cache[dev];
}

// One stream-ordered memory pool per device owned by the library. Its
// release threshold is unbounded, so memory freed at the end of a call stays
// mapped for the next one instead of being returned to the driver at every
// synchronisation (remapping a gigabyte of scratch costs about a millisecond).
static cudaMemPool_t scratch_pool(int dev) {
  static std::mutex mu;
  static std::vector<cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lk(mu);
  if ((int)pools.size() <= dev) pools.resize(dev + 1, nullptr);
  if (!pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    check_cuda(cudaMemPoolCreate(&p, &props), "cudaMemPoolCreate");
    uint64_t threshold = ~0ull;
    check_cuda(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &threshold), "pool release threshold");
    pools[dev] = p;
  }
  return pools[dev];
}

StreamScratch::StreamScratch(size_t bytes, cudaStream_t s) : stream(s) {
  if (bytes == 0) return;
  cudaError_t e = cudaMallocFromPoolAsync(&ptr, bytes, scratch_pool(current_device()), s);
  if (e != cudaSuccess) {
    ptr = nullptr;
    check_cuda(e, "cudaMallocAsync(scratch)");
  }
}

StreamScratch::~StreamScratch() {
  if (ptr) cudaFreeAsync(ptr, stream);
}

}  // namespace nca
