// The reference's volume, backprojection and RBF kernels built for the GPU
// (test infrastructure: a same-device parity anchor and a same-device timing
// baseline for those operators). The kernel functions are cut from the
// reference tree at build time (oracle/ref_harness.py) and compiled here as
// device functions; each extern "C" __global__ entry below builds the packed
// accessors the reference kernel expects over contiguous device arrays and
// runs its body. The caller launches each entry with the launch geometry of
// the reference's host launcher (src/render/volume_cuda.cu:68-93, 161-186,
// 267-295, 379-412; src/reconstruct/backprojection_cuda.cu:117-150, 196-226,
// 289-322; src/util/rbf2volume_cuda.cu:95-117, 203-229), and zeroes the
// outputs that those launchers zero.
#include <cuda_runtime.h>
#include <cstdint>

namespace at {
struct DefaultPtrTraits {};
struct RestrictPtrTraits {};

template <typename T, int N>
struct DeviceView {
  T* data;
  const int32_t* sizes;
  const int32_t* strides;
  __device__ DeviceView<T, N - 1> operator[](int i) const {
    return DeviceView<T, N - 1>{data + (int64_t)i * strides[0], sizes + 1, strides + 1};
  }
};
template <typename T>
struct DeviceView<T, 1> {
  T* data;
  const int32_t* sizes;
  const int32_t* strides;
  __device__ T& operator[](int i) const { return data[(int64_t)i * strides[0]]; }
};

template <typename T, int N, typename Traits = DefaultPtrTraits>
struct PackedTensorAccessor32 {
  T* data_;
  int32_t sizes_[N];
  int32_t strides_[N];
  __device__ int32_t size(int d) const { return sizes_[d]; }
  __device__ DeviceView<T, N - 1> operator[](int i) const {
    return DeviceView<T, N - 1>{data_ + (int64_t)i * strides_[0], sizes_ + 1, strides_ + 1};
  }
};

template <typename T, int N>
__device__ PackedTensorAccessor32<T, N, RestrictPtrTraits> contiguous(T* p,
                                                                     const int (&sz)[N]) {
  PackedTensorAccessor32<T, N, RestrictPtrTraits> a;
  a.data_ = p;
  int32_t st = 1;
  for (int d = N - 1; d >= 0; --d) {
    a.sizes_[d] = sz[d];
    a.strides_[d] = st;
    st *= sz[d];
  }
  return a;
}
}  // namespace at

#include "common/const.h"
#include "common/math.h"

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include "volume_kernels.inc"
#include "backprojection_kernels.inc"
#include "rbf2volume_kernels.inc"
#pragma pop_macro("__global__")

using at::contiguous;

extern "C" {

// volume [X,Y,Z], mp [3,N], transient [N,T]; grid (ceil(N/8), ceil(T/8)), block (8,8)
__global__ void ref_volume_confocal_forward(float* volume, int X, int Y, int Z, float* mp,
                                            int N, float* transient, int T, float3 origin,
                                            float3 size, float bw, float bo) {
  totri::render::volume_confocal_forward_kernel<float>(
      contiguous<float, 3>(volume, {X, Y, Z}), contiguous<float, 2>(mp, {3, N}),
      contiguous<float, 2>(transient, {N, T}), origin, size, bw, bo);
}

// transposed operator transient [N,T] -> volume [X,Y,Z];
// grid (ceil(X/8), ceil(Y/8), ceil(Z/8)), block (8,8,8)
__global__ void ref_volume_confocal_grad_volume(float* volume, int X, int Y, int Z, float* mp,
                                                int N, float* transient, int T, float3 origin,
                                                float3 size, float bw, float bo) {
  totri::render::volume_confocal_grad_volume_kernel<float>(
      contiguous<float, 3>(volume, {X, Y, Z}), contiguous<float, 2>(mp, {3, N}),
      contiguous<float, 2>(transient, {N, T}), origin, size, bw, bo);
}

// mpg [3,N] (zeroed by the caller); grid (ceil(N/8), ceil(T/8)), block (8,8)
__global__ void ref_volume_confocal_grad_mp(float* mpg, float* volume, int X, int Y, int Z,
                                            float* mp, int N, float* tgrad, int T,
                                            float3 origin, float3 size, float bw, float bo) {
  totri::render::volume_confocal_grad_measurement_points_kernel<float>(
      contiguous<float, 2>(mpg, {3, N}), contiguous<float, 3>(volume, {X, Y, Z}),
      contiguous<float, 2>(mp, {3, N}), contiguous<float, 2>(tgrad, {N, T}), origin, size, bw,
      bo);
}

// volume [B,D,H,W]; sp [B,3,S]; lp [B,3,L]; so [B,3,So]; lo [B,3,Lo]; transient [B,T,S,L]
// (zeroed by the caller); grid (ceil(H*W/8), ceil(S/8), ceil(L/8)), block (8,8,8), per item b
__global__ void ref_volume_exhaustive_forward(float* volume, int B, int D, int H, int W,
                                              float* sp, int S, float* lp, int L, float* so,
                                              int So, float* lo, int Lo, float* transient, int T,
                                              float3 start, float3 end, float bw, float bo,
                                              int b) {
  totri::render::volume_render_exhaustive_forward_kernel<float>(
      contiguous<float, 4>(volume, {B, D, H, W}), contiguous<float, 3>(sp, {B, 3, S}),
      contiguous<float, 3>(lp, {B, 3, L}), contiguous<float, 3>(so, {B, 3, So}),
      contiguous<float, 3>(lo, {B, 3, Lo}), contiguous<float, 4>(transient, {B, T, S, L}),
      start, end, bw, bo, b);
}

// transient [B,T,S]; sp [B,S,3]; so [B,So,3]; volume [B,D,H,W];
// grid (ceil(W/8), ceil(H/8), ceil(D/8)), block (8,8,8), per item b
__global__ void ref_backprojection_confocal_velten(float* transient, int B, int T, float* sp,
                                                   int S, float* so, int So, float* volume,
                                                   int D, int H, int W, float3 start,
                                                   float3 end, float bw, float bo, int b) {
  totri::reconstruct::backprojection_confocal_velten_forward_kernel<float>(
      contiguous<float, 3>(transient, {B, T, S}), contiguous<float, 3>(sp, {B, S, 3}),
      contiguous<float, 3>(so, {B, So, 3}), contiguous<float, 4>(volume, {B, D, H, W}), start,
      end, bw, bo, b);
}

// transient [B,T,S,L]; sp [B,S,3]; lp [B,L,3]; so [B,So,3]; lo [B,Lo,3]; volume [B,D,H,W];
// grid (ceil(W/8), ceil(H/8), ceil(D/8)), block (8,8,8), per item b
__global__ void ref_backprojection_exhaustive_velten(float* transient, int B, int T, float* sp,
                                                     int S, float* lp, int L, float* so, int So,
                                                     float* lo, int Lo, float* volume, int D,
                                                     int H, int W, float3 start, float3 end,
                                                     float bw, float bo, int b) {
  totri::reconstruct::backprojection_exhaustive_velten_forward_kernel<float>(
      contiguous<float, 4>(transient, {B, T, S, L}), contiguous<float, 3>(sp, {B, S, 3}),
      contiguous<float, 3>(lp, {B, L, 3}), contiguous<float, 3>(so, {B, So, 3}),
      contiguous<float, 3>(lo, {B, Lo, 3}), contiguous<float, 4>(volume, {B, D, H, W}), start,
      end, bw, bo, b);
}

// transient [B,T,S,L]; sp [B,3,S]; lp [B,3,L]; so [B,3,So]; lo [B,3,Lo]; volume [B,D,H,W]
// (zeroed by the caller); grid (ceil(H*W/64), S, L), block (64), per item b
__global__ void ref_backprojection_exhaustive_arellano(float* transient, int B, int T, float* sp,
                                                       int S, float* lp, int L, float* so,
                                                       int So, float* lo, int Lo, float* volume,
                                                       int D, int H, int W, float3 start,
                                                       float3 end, float bw, float bo, int b) {
  totri::reconstruct::backprojection_exhaustive_arellano_forward_kernel<float>(
      contiguous<float, 4>(transient, {B, T, S, L}), contiguous<float, 3>(sp, {B, 3, S}),
      contiguous<float, 3>(lp, {B, 3, L}), contiguous<float, 3>(so, {B, 3, So}),
      contiguous<float, 3>(lo, {B, 3, Lo}), contiguous<float, 4>(volume, {B, D, H, W}), start,
      end, bw, bo, b);
}

// rbf [B,N,C]; volume [B,C-3,D,H,W]; grid (ceil(W/4), ceil(H/4), ceil(D/4)), block (4,4,4)
__global__ void ref_rbf2volume_forward(float* rbf, int B, int N, int C, float* volume, int D,
                                       int H, int W, float3 start, float3 end, int b) {
  totri::util::rbf2volume_gaussian_forward_kernel<float>(
      contiguous<float, 3>(rbf, {B, N, C}), contiguous<float, 5>(volume, {B, C - 3, D, H, W}),
      start, end, b);
}

// rbf_grad [B,N,C] (zeroed by the caller); grid (ceil(W*H/16), ceil(D/4), N), block (16,4,1)
__global__ void ref_rbf2volume_grad(float* rbf, int B, int N, int C, float* volume,
                                    float* volume_grad, int D, int H, int W, float* rbf_grad,
                                    float3 start, float3 end, int b) {
  totri::util::rbf2volume_gaussian_grad_kernel<float>(
      contiguous<float, 3>(rbf, {B, N, C}), contiguous<float, 5>(volume, {B, C - 3, D, H, W}),
      contiguous<float, 5>(volume_grad, {B, C - 3, D, H, W}),
      contiguous<float, 3>(rbf_grad, {B, N, C}), start, end, b);
}

}  // extern "C"
