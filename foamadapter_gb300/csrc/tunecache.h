// The autotuner's cache of measured kernel variants (tunecache.cpp), for solver.cu.
#pragma once
#include <string>

constexpr int kTuneCacheKinds = 4;     // FP64 SpMV, FP64 update, FP32 SpMV, FP32 update
constexpr int kTuneCacheVariants = 4;  // launch-bound variants (at least 2, 4, 6, 8 blocks per SM)

// The cached variant of `kind` for systems of this shape; false when none is known.
bool tune_cache_get(const std::string& key, int kind, int* variant);
// Records a measured choice and its timings (ms[kTuneCacheVariants]).
void tune_cache_put(const std::string& key, int kind, int variant, const float* ms);
