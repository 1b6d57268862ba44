// Seeded standard normal fill (a benchmark loss head: the batched mesh
// workload's d loss / d transient is an N(0, 1) field drawn from a seed).
//
// Element i of the output depends only on (seed, i): a counter-based draw, so
// the same values come out whatever the launch shape, inside or outside a
// CUDA graph, for the batched renderer and for plain per-mesh calls alike.
// Two 24-bit uniforms come from the splitmix64 finaliser (Steele, Lea and
// Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014) of
// seed + (i + 1) * 0x9E3779B97F4A7C15, and the Box-Muller transform (Box and
// Muller 1958) turns them into one normal value.
#include <algorithm>

#include "common.cuh"

namespace totri {
namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void __launch_bounds__(256) fill_normal_kernel(float* __restrict__ out, int64_t n,
                                                          uint64_t seed) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t h = splitmix64(seed + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull);
    // u1 in (0, 1] (never 0, so the logarithm is finite), u2 in [0, 1)
    const float u1 = ((float)(uint32_t)(h >> 40) + 1.f) * (1.f / 16777216.f);
    const float u2 = (float)((uint32_t)h >> 8) * (1.f / 16777216.f);
    float s, c;
    sincospif(2.f * u2, &s, &c);
    out[i] = sqrtf(-2.f * logf(u1)) * c;
  }
}

}  // namespace
}  // namespace totri

extern "C" {

int totri_fill_normal(float* out, int64_t n, uint64_t seed, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  if (n < 0) return totri::fail(TOTRI_ERR_INVALID_ARGUMENT, "fill_normal: negative count");
  if (n == 0) return TOTRI_OK;
  if (!out) return totri::fail(TOTRI_ERR_INVALID_ARGUMENT, "fill_normal: output is null");
  const int64_t blocks = std::min<int64_t>(totri::ceil_div(n, 256), 152 * 32);
  TOTRI_KERNEL("fill normal", stream,
               totri::fill_normal_kernel<<<(unsigned)blocks, 256, 0, stream>>>(out, n, seed));
  return TOTRI_OK;
}

}  // extern "C"
