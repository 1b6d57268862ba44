// Shared device/host helpers for the totri_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "profile.cuh"
#include "totri_gb300.h"

namespace totri {

// ---------------------------------------------------------------------------
// Host-side status plumbing.

void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_status(cudaError_t e, const char* what);

#define TOTRI_CUDA(call)                                         \
  do {                                                           \
    cudaError_t e__ = (call);                                    \
    if (e__ != cudaSuccess) return ::totri::cuda_status(e__, #call); \
  } while (0)

#define TOTRI_LAUNCHED(name)                                     \
  do {                                                           \
    cudaError_t e__ = cudaGetLastError();                        \
    if (e__ != cudaSuccess) return ::totri::cuda_status(e__, name); \
  } while (0)

// Launches a kernel through the launch accounting (profile.cuh) and checks the
// launch status: TOTRI_KERNEL("name", stream, kernel<<<g, b, smem, stream>>>(...)).
#define TOTRI_KERNEL(name, stream, ...)                               \
  do {                                                                \
    {                                                                 \
      ::totri::prof::Scope ps__(name, stream);                        \
      __VA_ARGS__;                                                    \
    }                                                                 \
    cudaError_t e__ = cudaGetLastError();                             \
    if (e__ != cudaSuccess) return ::totri::cuda_status(e__, name);   \
  } while (0)

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Device status bits written into a workspace header. kStatusFaceIndexRange
// reports an input (a face index >= V ends the face list); the other two are
// internal errors: a BVH search that hit its step or stack limit, and (in
// the bounds-checking build only) an index read from device data that was
// out of range.
enum : uint32_t {
  kStatusFaceIndexRange = 1u,
  kStatusTraversalCap = 2u,
  kStatusIndexRange = 4u,
};

// TOTRI_INDEX_OK(cond, status): in the bounds-checking build (TOTRI_BOUNDS_CHECK)
// evaluates cond and, when it fails, sets kStatusIndexRange in *status; the
// caller clamps or skips the access. Otherwise it is `true` and costs nothing.
#ifdef TOTRI_BOUNDS_CHECK
#define TOTRI_INDEX_OK(cond, status) \
  ((cond) ? true : (atomicOr((status), ::totri::kStatusIndexRange), false))
#else
#define TOTRI_INDEX_OK(cond, status) true
#endif

// ---------------------------------------------------------------------------
// Strided views of small input arrays (element strides).

struct View3f {  // [B, N, C] float
  const float* p;
  int64_t sb, sn, sc;
  __host__ __device__ float at(int64_t b, int64_t n, int64_t c) const {
    return p[b * sb + n * sn + c * sc];
  }
};

struct View3i {  // [B, N, 3] int32 or int64
  const void* p;
  int64_t sb, sn, sc;
  int is64;
  __device__ int64_t at(int64_t b, int64_t n, int64_t c) const {
    const int64_t off = b * sb + n * sn + c * sc;
    return is64 ? static_cast<const int64_t*>(p)[off]
                : (int64_t) static_cast<const int32_t*>(p)[off];
  }
};

// ---------------------------------------------------------------------------
// FP32 arithmetic with exactly one IEEE round-to-nearest per operation. Every
// quantity that drives a discrete decision (visibility, vertex order, bin
// index) is built from these so that the CPU oracle (compiled with
// -ffp-contract=off, fma only where written) reproduces it bit for bit.

// Three-input minimum / maximum (PTX min.f32 / max.f32 with three sources,
// sm_100 and later): one instruction where two nested fminf/fmaxf take two.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float xfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ float xrcp(float a) { return __frcp_rn(a); }

struct fv3 {
  float x, y, z;
};

__device__ __forceinline__ fv3 mkv(float x, float y, float z) { return fv3{x, y, z}; }
__device__ __forceinline__ fv3 xsub3(fv3 a, fv3 b) {
  return fv3{xsub(a.x, b.x), xsub(a.y, b.y), xsub(a.z, b.z)};
}
__device__ __forceinline__ float xlen2(fv3 a) {
  return xfma(a.x, a.x, xfma(a.y, a.y, xmul(a.z, a.z)));
}
__device__ __forceinline__ float xlen(fv3 a) { return xsqrt(xlen2(a)); }
__device__ __forceinline__ fv3 xcross(fv3 a, fv3 b) {
  return fv3{xfma(a.y, b.z, -xmul(a.z, b.y)), xfma(a.z, b.x, -xmul(a.x, b.z)),
             xfma(a.x, b.y, -xmul(a.y, b.x))};
}
__device__ __forceinline__ float xdot(fv3 a, fv3 b) {
  return xfma(a.x, b.x, xfma(a.y, b.y, xmul(a.z, b.z)));
}
// (1/3) * ((v0 + v1) + v2), the reference's centroid
// (mesh_confocal_forward_optix.cu:40).
__device__ __forceinline__ fv3 xcentroid(fv3 a, fv3 b, fv3 c) {
  const float third = 1.f / 3.f;
  return fv3{xmul(third, xadd(xadd(a.x, b.x), c.x)), xmul(third, xadd(xadd(a.y, b.y), c.y)),
             xmul(third, xadd(xadd(a.z, b.z), c.z))};
}

// C int() truncation of a bin coordinate with saturation (NaN -> never valid).
__device__ __forceinline__ int bin_of(float c) {
  if (!(c == c)) return -2147483647;
  if (c >= 1.0e9f) return 1000000000;
  if (c <= -1.0e9f) return -1000000000;
  return __float2int_rz(c);
}

// ---------------------------------------------------------------------------
// Value arithmetic (free to contract / reorder; compared with tolerances).

__device__ __forceinline__ fv3 operator+(fv3 a, fv3 b) { return fv3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ fv3 operator-(fv3 a, fv3 b) { return fv3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ fv3 operator*(float s, fv3 a) { return fv3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ fv3 operator-(fv3 a) { return fv3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(fv3 a, fv3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ fv3 cross(fv3 a, fv3 b) {
  return fv3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Two floats in one 64-bit register pair, for the paired FP32 FMA of sm_100
// and later (fma.rn.f32x2): each half is one correctly rounded fma, the same
// value fmaf gives.
__device__ __forceinline__ unsigned long long f2pack(float a, float b) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2unpack(unsigned long long v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2fma(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ unsigned long long f2add(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long f2sub(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ unsigned long long f2mul(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// Monotone float <-> int mapping for atomicMin/atomicMax on floats.
__device__ __forceinline__ int ford(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float iord(int i) {
  return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

}  // namespace totri
