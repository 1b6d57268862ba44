// Launch accounting: every kernel launch of the library goes through a
// prof::Scope, which counts it and, while profiling is enabled, brackets it
// with CUDA events on the launching stream. With TOTRI_NVTX=1 in the
// environment each launch is also an NVTX range named after the kernel, for
// timeline tools.
#pragma once

#include <cuda_runtime.h>

namespace totri {
namespace prof {

bool enabled();
void begin(const char* name, cudaStream_t stream, cudaEvent_t* start);
void end(const char* name, cudaStream_t stream, cudaEvent_t start);

bool nvtx_enabled();
void nvtx_push(const char* name);
void nvtx_pop();

struct Scope {
  const char* name;
  cudaStream_t stream;
  cudaEvent_t start = nullptr;
  bool nvtx;
  Scope(const char* n, cudaStream_t s) : name(n), stream(s), nvtx(nvtx_enabled()) {
    if (nvtx) nvtx_push(name);
    begin(name, stream, &start);
  }
  ~Scope() {
    end(name, stream, start);
    if (nvtx) nvtx_pop();
  }
};

}  // namespace prof
}  // namespace totri
