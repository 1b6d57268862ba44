// Tile-shape overrides set by the autotuner (totri_gb300/autotune.py). A value
// of 0 (or an unknown key) leaves the launcher's own heuristic in charge.
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "common.cuh"
#include "tune.cuh"

namespace totri {
namespace tune {
namespace {
std::mutex g_mu;
std::map<std::string, int>& table() {
  static std::map<std::string, int> t;
  return t;
}
}  // namespace

int get(const char* key) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = table().find(key);
  return it == table().end() ? 0 : it->second;
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
    return 152;
  return n;
}

cudaError_t ensure_dynamic_smem(const void* func, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  size_t& have = done[std::make_pair(func, dev)];
  if (have >= bytes) return cudaSuccess;
  const cudaError_t r =
      cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (r == cudaSuccess) have = bytes;
  return r;
}

int grad_split(const char* key, int64_t ctas, int S, int max_slice) {
  const int least = (int)((S + (int64_t)max_slice - 1) / max_slice);
  int most = S >= 64 ? S / 64 : 1;
  if (most < least) most = least;
  int split = get(key);
  if (split <= 0) {
    // gradient CTAs run long (32 faces x a slice of every wall point): aim for
    // many waves so the last one is short
    const int64_t target = (int64_t)sm_count() * 32;
    split = ctas > 0 ? (int)((target + ctas - 1) / ctas) : 1;
  }
  if (split > most) split = most;
  return split < least ? least : split;
}

}  // namespace tune
}  // namespace totri

extern "C" {

int totri_tune_set(const char* key, int value) {
  if (!key) return totri::fail(TOTRI_ERR_INVALID_ARGUMENT, "tuning key is null");
  std::lock_guard<std::mutex> lk(totri::tune::g_mu);
  if (value == 0) totri::tune::table().erase(key);
  else totri::tune::table()[key] = value;
  return TOTRI_OK;
}

int totri_tune_get(const char* key) { return key ? totri::tune::get(key) : 0; }

}  // extern "C"
