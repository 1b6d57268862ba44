// Runs the reference's volume, backprojection and RBF kernels on the CPU with
// the launch geometry of their host launchers (src/render/volume_cuda.cu:68-93,
// 161-186, 267-295, 379-412; src/reconstruct/backprojection_cuda.cu:117-150,
// 196-226, 289-322; src/util/rbf2volume_cuda.cu:95-117, 203-229). The kernel
// functions themselves are cut from the reference tree at build time
// (oracle/ref_harness.py). Test infrastructure only.
#include "cuda_host_shim.h"

#include <array>
#include <cstring>
#include <torch/extension.h>

#include "common/const.h"
#include "common/math.h"

#include "volume_kernels.inc"
#include "backprojection_kernels.inc"
#include "rbf2volume_kernels.inc"

using at::make_accessor;

namespace {
inline unsigned cdiv(long a, long b) { return (unsigned)((a + b - 1) / b); }
}  // namespace

extern "C" {

// volume [X,Y,Z], mp [3,N], transient [N,T] (overwritten)
int ref_volume_confocal_forward(float* volume, int X, int Y, int Z, float* mp, int N,
                                float* transient, int T, const float* origin, const float* size,
                                float bw, float bo) {
  auto va = make_accessor<float, 3>(volume, {X, Y, Z});
  auto ma = make_accessor<float, 2>(mp, {3, N});
  auto ta = make_accessor<float, 2>(transient, {N, T});
  const float3 o = make_float3(origin[0], origin[1], origin[2]);
  const float3 s = make_float3(size[0], size[1], size[2]);
  refshim::launch(dim3(cdiv(N, 8), cdiv(T, 8), 1), dim3(8, 8, 1), false, [&] {
    totri::render::volume_confocal_forward_kernel<float>(va, ma, ta, o, s, bw, bo);
  });
  return 0;
}

// transposed operator: transient [N,T] -> volume [X,Y,Z] (overwritten)
int ref_volume_confocal_grad_volume(float* volume, int X, int Y, int Z, float* mp, int N,
                                    float* transient, int T, const float* origin,
                                    const float* size, float bw, float bo) {
  auto va = make_accessor<float, 3>(volume, {X, Y, Z});
  auto ma = make_accessor<float, 2>(mp, {3, N});
  auto ta = make_accessor<float, 2>(transient, {N, T});
  const float3 o = make_float3(origin[0], origin[1], origin[2]);
  const float3 s = make_float3(size[0], size[1], size[2]);
  refshim::launch(dim3(cdiv(X, 8), cdiv(Y, 8), cdiv(Z, 8)), dim3(8, 8, 8), false, [&] {
    totri::render::volume_confocal_grad_volume_kernel<float>(va, ma, ta, o, s, bw, bo);
  });
  return 0;
}

// mpg [3,N] (zeroed then accumulated, as the reference launcher does)
int ref_volume_confocal_grad_mp(float* mpg, float* volume, int X, int Y, int Z, float* mp, int N,
                                float* tgrad, int T, const float* origin, const float* size,
                                float bw, float bo) {
  std::memset(mpg, 0, sizeof(float) * 3 * N);
  auto ga = make_accessor<float, 2>(mpg, {3, N});
  auto va = make_accessor<float, 3>(volume, {X, Y, Z});
  auto ma = make_accessor<float, 2>(mp, {3, N});
  auto ta = make_accessor<float, 2>(tgrad, {N, T});
  const float3 o = make_float3(origin[0], origin[1], origin[2]);
  const float3 s = make_float3(size[0], size[1], size[2]);
  refshim::launch(dim3(cdiv(N, 8), cdiv(T, 8), 1), dim3(8, 8, 1), false, [&] {
    totri::render::volume_confocal_grad_measurement_points_kernel<float>(ga, va, ma, ta, o, s, bw,
                                                                         bo);
  });
  return 0;
}

// volume [B,D,H,W]; sp [B,3,S]; lp [B,3,L]; so [B,3,So]; lo [B,3,Lo];
// transient [B,T,S,L] (zeroed, then accumulated)
int ref_volume_exhaustive_forward(float* volume, int B, int D, int H, int W, float* sp, int S,
                                  float* lp, int L, float* so, int So, float* lo, int Lo,
                                  float* transient, int T, const float* start, const float* end,
                                  float bw, float bo) {
  std::memset(transient, 0, sizeof(float) * (size_t)B * T * S * L);
  auto va = make_accessor<float, 4>(volume, {B, D, H, W});
  auto sa = make_accessor<float, 3>(sp, {B, 3, S});
  auto la = make_accessor<float, 3>(lp, {B, 3, L});
  auto soa = make_accessor<float, 3>(so, {B, 3, So});
  auto loa = make_accessor<float, 3>(lo, {B, 3, Lo});
  auto ta = make_accessor<float, 4>(transient, {B, T, S, L});
  const float3 a = make_float3(start[0], start[1], start[2]);
  const float3 e = make_float3(end[0], end[1], end[2]);
  for (int b = 0; b < B; ++b)
    refshim::launch(dim3(cdiv((long)H * W, 8), cdiv(S, 8), cdiv(L, 8)), dim3(8, 8, 8), false,
                    [&] {
                      totri::render::volume_render_exhaustive_forward_kernel<float>(
                          va, sa, la, soa, loa, ta, a, e, bw, bo, b);
                    });
  return 0;
}

// transient [B,T,S]; sp [B,S,3]; so [B,So,3]; volume [B,D,H,W] (overwritten)
int ref_backprojection_confocal_velten(float* transient, int B, int T, float* sp, int S, float* so,
                                       int So, float* volume, int D, int H, int W,
                                       const float* start, const float* end, float bw,
                                       float bo) {
  auto ta = make_accessor<float, 3>(transient, {B, T, S});
  auto sa = make_accessor<float, 3>(sp, {B, S, 3});
  auto soa = make_accessor<float, 3>(so, {B, So, 3});
  auto va = make_accessor<float, 4>(volume, {B, D, H, W});
  const float3 a = make_float3(start[0], start[1], start[2]);
  const float3 e = make_float3(end[0], end[1], end[2]);
  for (int b = 0; b < B; ++b)
    refshim::launch(dim3(cdiv(W, 8), cdiv(H, 8), cdiv(D, 8)), dim3(8, 8, 8), false, [&] {
      totri::reconstruct::backprojection_confocal_velten_forward_kernel<float>(ta, sa, soa, va,
                                                                               a, e, bw, bo, b);
    });
  return 0;
}

// transient [B,T,S,L]; sp [B,S,3]; lp [B,L,3]; volume [B,D,H,W] (overwritten)
int ref_backprojection_exhaustive_velten(float* transient, int B, int T, float* sp, int S,
                                         float* lp, int L, float* so, int So, float* lo, int Lo,
                                         float* volume, int D, int H, int W, const float* start,
                                         const float* end, float bw, float bo) {
  auto ta = make_accessor<float, 4>(transient, {B, T, S, L});
  auto sa = make_accessor<float, 3>(sp, {B, S, 3});
  auto la = make_accessor<float, 3>(lp, {B, L, 3});
  auto soa = make_accessor<float, 3>(so, {B, So, 3});
  auto loa = make_accessor<float, 3>(lo, {B, Lo, 3});
  auto va = make_accessor<float, 4>(volume, {B, D, H, W});
  const float3 a = make_float3(start[0], start[1], start[2]);
  const float3 e = make_float3(end[0], end[1], end[2]);
  for (int b = 0; b < B; ++b)
    refshim::launch(dim3(cdiv(W, 8), cdiv(H, 8), cdiv(D, 8)), dim3(8, 8, 8), false, [&] {
      totri::reconstruct::backprojection_exhaustive_velten_forward_kernel<float>(
          ta, sa, la, soa, loa, va, a, e, bw, bo, b);
    });
  return 0;
}

// transient [B,T,S,L]; sp [B,3,S]; lp [B,3,L]; volume [B,D,H,W] (zeroed, accumulated)
int ref_backprojection_exhaustive_arellano(float* transient, int B, int T, float* sp, int S,
                                           float* lp, int L, float* so, int So, float* lo,
                                           int Lo, float* volume, int D, int H, int W,
                                           const float* start, const float* end, float bw,
                                           float bo) {
  std::memset(volume, 0, sizeof(float) * (size_t)B * D * H * W);
  auto ta = make_accessor<float, 4>(transient, {B, T, S, L});
  auto sa = make_accessor<float, 3>(sp, {B, 3, S});
  auto la = make_accessor<float, 3>(lp, {B, 3, L});
  auto soa = make_accessor<float, 3>(so, {B, 3, So});
  auto loa = make_accessor<float, 3>(lo, {B, 3, Lo});
  auto va = make_accessor<float, 4>(volume, {B, D, H, W});
  const float3 a = make_float3(start[0], start[1], start[2]);
  const float3 e = make_float3(end[0], end[1], end[2]);
  for (int b = 0; b < B; ++b)
    refshim::launch(dim3(cdiv((long)H * W, 64), S, L), dim3(64, 1, 1), false, [&] {
      totri::reconstruct::backprojection_exhaustive_arellano_forward_kernel<float>(
          ta, sa, la, soa, loa, va, a, e, bw, bo, b);
    });
  return 0;
}

// rbf [B,N,4+A]; volume [B,1+A,D,H,W] (overwritten)
int ref_rbf2volume_forward(float* rbf, int B, int N, int C, float* volume, int D, int H, int W,
                           const float* start, const float* end) {
  auto ra = make_accessor<float, 3>(rbf, {B, N, C});
  auto va = make_accessor<float, 5>(volume, {B, C - 3, D, H, W});
  const float3 a = make_float3(start[0], start[1], start[2]);
  const float3 e = make_float3(end[0], end[1], end[2]);
  for (int b = 0; b < B; ++b)
    refshim::launch(dim3(cdiv(W, 4), cdiv(H, 4), cdiv(D, 4)), dim3(4, 4, 4), false, [&] {
      totri::util::rbf2volume_gaussian_forward_kernel<float>(ra, va, a, e, b);
    });
  return 0;
}

// rbf_grad [B,N,4+A] (zeroed, accumulated)
int ref_rbf2volume_grad(float* rbf, int B, int N, int C, float* volume, float* volume_grad,
                        int D, int H, int W, float* rbf_grad, const float* start,
                        const float* end) {
  std::memset(rbf_grad, 0, sizeof(float) * (size_t)B * N * C);
  auto ra = make_accessor<float, 3>(rbf, {B, N, C});
  auto va = make_accessor<float, 5>(volume, {B, C - 3, D, H, W});
  auto ga = make_accessor<float, 5>(volume_grad, {B, C - 3, D, H, W});
  auto rg = make_accessor<float, 3>(rbf_grad, {B, N, C});
  const float3 a = make_float3(start[0], start[1], start[2]);
  const float3 e = make_float3(end[0], end[1], end[2]);
  for (int b = 0; b < B; ++b)
    refshim::launch(dim3(cdiv((long)W * H, 16), cdiv(D, 4), N), dim3(16, 4, 1), true, [&] {
      totri::util::rbf2volume_gaussian_grad_kernel<float>(ra, va, ga, rg, a, e, b);
    });
  return 0;
}

}  // extern "C"
