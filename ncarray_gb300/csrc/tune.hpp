// Launch-schedule autotuner (tune.cpp): cached per (op class, dtype, shape
// class) key, timed on the caller's stream on a miss in mode 2.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <string>
#include <vector>

namespace nca {

int tune_mode();                 // 0 heuristics, 1 cached choices (default), 2 search on a miss
void tune_set_mode(int mode);
bool tune_get(const std::string& key, std::vector<int>& values);
void tune_put(const std::string& key, const std::vector<int>& values);
void tune_clear();
// true when a miss should be searched now (mode 2 and the stream is not capturing)
bool tune_should_search(cudaStream_t s);
// runs each candidate once, then `reps` times between CUDA events; index of the fastest
int tune_pick(cudaStream_t s, int n, const std::function<void(int)>& run, int reps = 3);
// log2 bucket of a size ("20" for 1..2 Mi)
std::string size_class(long long n);

}  // namespace nca
