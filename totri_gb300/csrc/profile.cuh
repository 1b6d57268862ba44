// Launch accounting: every kernel launch of the library goes through a
// prof::Scope, which counts it and, while profiling is enabled, brackets it
// with CUDA events on the launching stream.
#pragma once

#include <cuda_runtime.h>

namespace totri {
namespace prof {

bool enabled();
void begin(const char* name, cudaStream_t stream, cudaEvent_t* start);
void end(const char* name, cudaStream_t stream, cudaEvent_t start);

struct Scope {
  const char* name;
  cudaStream_t stream;
  cudaEvent_t start = nullptr;
  Scope(const char* n, cudaStream_t s) : name(n), stream(s) { begin(name, stream, &start); }
  ~Scope() { end(name, stream, start); }
};

}  // namespace prof
}  // namespace totri
