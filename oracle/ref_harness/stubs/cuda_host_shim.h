// Host emulation of the CUDA built-ins used by the reference kernel sources,
// so those sources compile and run as plain C++ on the CPU (test
// infrastructure: it produces golden vectors from the reference's own
// arithmetic). Kernels run one simulated thread at a time; blocks that use
// __syncthreads are run with one OS thread per simulated thread.
#pragma once

#include <cuda_runtime.h>  // float3/uint3/dim3 and make_* (host-usable)

#include <algorithm>
#include <atomic>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <functional>
#include <thread>
#include <vector>

#undef __shared__
#define __shared__ static
#undef __constant__
#define __constant__
#undef __global__
#define __global__
#undef __device__
#define __device__
#undef __host__
#define __host__
#undef __forceinline__
#define __forceinline__ inline

namespace refshim {
inline thread_local dim3 tIdx, bIdx, bDim, gDim;
inline thread_local std::barrier<>* block_barrier = nullptr;
}  // namespace refshim

#define threadIdx (::refshim::tIdx)
#define blockIdx (::refshim::bIdx)
#define blockDim (::refshim::bDim)
#define gridDim (::refshim::gDim)

inline void __syncthreads() {
  if (::refshim::block_barrier) ::refshim::block_barrier->arrive_and_wait();
}

inline float atomicAdd(float* p, float v) {
  std::atomic_ref<float> r(*p);
  float old = r.load();
  while (!r.compare_exchange_weak(old, old + v)) {
  }
  return old;
}
inline double atomicAdd(double* p, double v) {
  std::atomic_ref<double> r(*p);
  double old = r.load();
  while (!r.compare_exchange_weak(old, old + v)) {
  }
  return old;
}

// CUDA's norm3df: sqrt(x^2 + y^2 + z^2) without undue overflow; evaluated in
// double and rounded once.
inline float norm3df(float x, float y, float z) {
  return (float)std::sqrt((double)x * x + (double)y * y + (double)z * z);
}

using std::isnan;

// CUDA's global min/max overloads.
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline double max(double a, double b) { return std::fmax(a, b); }
inline double min(double a, double b) { return std::fmin(a, b); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }

namespace refshim {
// Runs kernel(...) over a grid; threads of a block run sequentially unless
// `sync_blocks` (then one OS thread per simulated thread with a barrier).
inline void launch(dim3 grid, dim3 block, bool sync_blocks, const std::function<void()>& body) {
  for (unsigned bz = 0; bz < grid.z; ++bz)
    for (unsigned by = 0; by < grid.y; ++by)
      for (unsigned bx = 0; bx < grid.x; ++bx) {
        const dim3 b(bx, by, bz);
        if (!sync_blocks) {
          for (unsigned tz = 0; tz < block.z; ++tz)
            for (unsigned ty = 0; ty < block.y; ++ty)
              for (unsigned tx = 0; tx < block.x; ++tx) {
                tIdx = dim3(tx, ty, tz);
                bIdx = b;
                bDim = block;
                gDim = grid;
                body();
              }
        } else {
          const unsigned n = block.x * block.y * block.z;
          std::barrier<> bar(n);
          std::vector<std::thread> th;
          for (unsigned i = 0; i < n; ++i) {
            th.emplace_back([&, i] {
              tIdx = dim3(i % block.x, (i / block.x) % block.y, i / (block.x * block.y));
              bIdx = b;
              bDim = block;
              gDim = grid;
              block_barrier = &bar;
              body();
              block_barrier = nullptr;
            });
          }
          for (auto& t : th) t.join();
        }
      }
}
}  // namespace refshim
