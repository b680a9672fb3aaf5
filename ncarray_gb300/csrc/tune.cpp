// Launch-schedule autotuner shared by the stencil, the elementwise kernels and
// the row reductions: candidate schedules are timed on the caller's stream
// once per (op class, dtype, shape class) key and the fastest is cached in
// memory and in `tune.txt` next to the JIT cubin cache, one line per key:
//   <key> <value> <value> ...
// Modes (nca_tune_set_mode / NCA_TUNE): 0 = the built-in heuristics only;
// 1 = cached choices where present, else heuristics (default); 2 = as 1, and a
// call whose key has no entry times the candidates first (it synchronises its
// stream; skipped while the stream is being captured).
#include <cuda_runtime.h>

#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "common.hpp"
#include "jit.hpp"
#include "tune.hpp"

namespace nca {
namespace {

struct TuneState {
  std::mutex m;
  bool loaded = false;
  int mode = -1;
  std::map<std::string, std::vector<int>> table;
};

TuneState& ts() {
  static TuneState s;
  return s;
}

std::string tune_file() { return jit_cache_dir() + "/tune.txt"; }

void load_locked(TuneState& s) {
  if (s.loaded) return;
  s.loaded = true;
  std::ifstream f(tune_file());
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    std::string key;
    if (!(is >> key)) continue;
    std::vector<int> v;
    int x;
    while (is >> x) v.push_back(x);
    if (!v.empty()) s.table[key] = v;
  }
}

void save_locked(TuneState& s) {
  const std::string file = tune_file();
  const std::string tmp = file + ".tmp." + std::to_string((long)getpid());
  {
    std::ofstream f(tmp);
    if (!f) return;
    for (auto& kv : s.table) {
      f << kv.first;
      for (int v : kv.second) f << ' ' << v;
      f << '\n';
    }
    if (!f) { std::remove(tmp.c_str()); return; }
  }
  std::rename(tmp.c_str(), file.c_str());
}

}  // namespace

int tune_mode() {
  auto& s = ts();
  std::lock_guard<std::mutex> lk(s.m);
  if (s.mode < 0) {
    const char* e = getenv("NCA_TUNE");
    s.mode = (e && *e) ? std::max(0, std::min(2, atoi(e))) : 1;
  }
  return s.mode;
}

void tune_set_mode(int m) {
  if (m < 0 || m > 2) fail(NCA_ERR_INVALID, "tune mode %d (0, 1 or 2)", m);
  auto& s = ts();
  std::lock_guard<std::mutex> lk(s.m);
  s.mode = m;
}

bool tune_get(const std::string& key, std::vector<int>& out) {
  if (tune_mode() == 0) return false;
  auto& s = ts();
  std::lock_guard<std::mutex> lk(s.m);
  load_locked(s);
  auto it = s.table.find(key);
  if (it == s.table.end()) return false;
  out = it->second;
  return true;
}

void tune_put(const std::string& key, const std::vector<int>& v) {
  auto& s = ts();
  std::lock_guard<std::mutex> lk(s.m);
  load_locked(s);
  s.table[key] = v;
  save_locked(s);
}

void tune_clear() {
  auto& s = ts();
  std::lock_guard<std::mutex> lk(s.m);
  s.table.clear();
  s.loaded = true;
  std::remove(tune_file().c_str());
}

bool tune_should_search(cudaStream_t s) {
  if (tune_mode() != 2) return false;
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) { cudaGetLastError(); return false; }
  return st == cudaStreamCaptureStatusNone;
}

int tune_pick(cudaStream_t s, int n, const std::function<void(int)>& run, int reps) {
  cudaEvent_t a, b;
  check_cuda(cudaEventCreate(&a), "cudaEventCreate");
  check_cuda(cudaEventCreate(&b), "cudaEventCreate");
  int best = 0;
  float best_ms = 0.f;
  for (int i = 0; i < n; ++i) {
    run(i);   // first use: compiles and warms the candidate
    check_cuda(cudaEventRecord(a, s), "cudaEventRecord");
    for (int r = 0; r < reps; ++r) run(i);
    check_cuda(cudaEventRecord(b, s), "cudaEventRecord");
    check_cuda(cudaEventSynchronize(b), "cudaEventSynchronize");
    float ms = 0.f;
    check_cuda(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
    if (i == 0 || ms < best_ms) { best = i; best_ms = ms; }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

std::string size_class(long long n) {
  int l = 0;
  while (n > 1 && l < 62) { n >>= 1; ++l; }
  return std::to_string(l);
}

}  // namespace nca

extern "C" int32_t nca_tune_set_mode(int32_t mode) {
  return nca::guarded([&] { nca::tune_set_mode(mode); });
}

extern "C" int32_t nca_tune_get(const char* key, int32_t* values, int32_t cap, int32_t* n) {
  return nca::guarded([&] {
    if (!key || !n) nca::fail(NCA_ERR_INVALID, "null argument");
    std::vector<int> v;
    *n = 0;
    auto& s = nca::ts();
    std::lock_guard<std::mutex> lk(s.m);
    nca::load_locked(s);
    auto it = s.table.find(key);
    if (it == s.table.end()) return;
    v = it->second;
    *n = (int32_t)v.size();
    for (int i = 0; i < (int)v.size() && i < cap; ++i) values[i] = v[(size_t)i];
  });
}

extern "C" int32_t nca_tune_clear(void) {
  return nca::guarded([&] { nca::tune_clear(); });
}
