// Launch counting and optional per-kernel event timing.
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "profile.cuh"

namespace totri {
namespace prof {
namespace {

struct Pending {
  std::string name;
  cudaEvent_t start, stop;
};

struct Totals {
  int64_t launches = 0;
  double ms = 0.0;
  int64_t timed = 0;
};

std::mutex g_mu;
std::atomic<bool> g_on{false};
std::vector<Pending> g_pending;
std::vector<cudaEvent_t> g_pool;
std::map<std::string, Totals> g_totals;

cudaEvent_t take_event() {
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

}  // namespace

bool enabled() { return g_on.load(std::memory_order_relaxed); }

bool nvtx_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("TOTRI_NVTX");
    return v && v[0] && std::strcmp(v, "0") != 0;
  }();
  return on;
}
void nvtx_push(const char* name) { nvtxRangePushA(name); }
void nvtx_pop() { nvtxRangePop(); }

void begin(const char* name, cudaStream_t stream, cudaEvent_t* start) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_totals[name].launches += 1;
  *start = nullptr;
  if (!enabled()) return;
  // launches recorded into a CUDA graph are not timed (the events would
  // become graph nodes)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return;
  cudaEvent_t e = take_event();
  if (e && cudaEventRecord(e, stream) == cudaSuccess) *start = e;
}

void end(const char* name, cudaStream_t stream, cudaEvent_t start) {
  if (!start) return;
  std::lock_guard<std::mutex> lk(g_mu);
  cudaEvent_t stop = take_event();
  if (!stop || cudaEventRecord(stop, stream) != cudaSuccess) {
    g_pool.push_back(start);
    return;
  }
  g_pending.push_back(Pending{name, start, stop});
}

}  // namespace prof
}  // namespace totri

using namespace totri;

extern "C" {

int totri_profile_enable(int on) {
  prof::g_on.store(on != 0);
  return TOTRI_OK;
}

void totri_profile_reset(void) {
  std::lock_guard<std::mutex> lk(prof::g_mu);
  for (auto& p : prof::g_pending) {
    prof::g_pool.push_back(p.start);
    prof::g_pool.push_back(p.stop);
  }
  prof::g_pending.clear();
  prof::g_totals.clear();
}

int totri_profile_read(int max_entries, char* names, int64_t* launches, int64_t* timed,
                       double* total_ms, int* n_entries) {
  std::lock_guard<std::mutex> lk(prof::g_mu);
  for (auto& p : prof::g_pending) {
    if (cudaEventSynchronize(p.stop) != cudaSuccess)
      return fail(TOTRI_ERR_CUDA, "profile: event synchronize failed");
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.start, p.stop) == cudaSuccess) {
      auto& t = prof::g_totals[p.name];
      t.ms += ms;
      t.timed += 1;
    }
    prof::g_pool.push_back(p.start);
    prof::g_pool.push_back(p.stop);
  }
  prof::g_pending.clear();
  int i = 0;
  for (auto& kv : prof::g_totals) {
    if (i >= max_entries) break;
    std::strncpy(names + 64 * i, kv.first.c_str(), 63);
    names[64 * i + 63] = 0;
    launches[i] = kv.second.launches;
    timed[i] = kv.second.timed;
    total_ms[i] = kv.second.ms;
    ++i;
  }
  *n_entries = i;
  return TOTRI_OK;
}

}  // extern "C"
