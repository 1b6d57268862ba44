// RBF-to-volume splatting and its gradient.
//
// Reference: src/util/rbf2volume_cuda.cu (:50-93 forward, one thread per voxel
// reading every Gaussian from global memory; :124-201 gradient, one block
// column per Gaussian with a shared-memory tree reduction and an atomic per
// (Gaussian, channel, 64 voxels)). Here the forward stages Gaussians in shared
// memory tiles; the gradient gives each thread one Gaussian and a chunk of
// voxels staged in shared memory, accumulates all 4+A channels in registers
// and issues 4+A atomics per (Gaussian, chunk).
#include <algorithm>
#include <string>

#include "capi_common.cuh"
#include "tune.cuh"

namespace totri {
namespace rbf {

constexpr int kMaxAttr = 8;
constexpr int kTile = 256;

struct Grid {
  int D, H, W;
  float sx, sy, sz, ex, ey, ez;
};

// Voxel coordinate (rbf2volume_cuda.cu:58-60): midpoint for a single-voxel
// axis, else start + ((end - start) * i) / (n - 1).
__device__ __forceinline__ float coord(float s, float e, int n, int i) {
  return n == 1 ? 0.5f * (s + e) : s + ((e - s) * (float)i) / (float)(n - 1);
}

// 2^x from the hardware approximation (ex2.approx, relative error about
// 2^-22; results below the normal range flush to zero): the Gaussians are
// values, compared with tolerances, and -d2 / (2 sigma^2) folds into one
// multiply by a per-Gaussian constant -log2(e) / (2 sigma^2).
__device__ __forceinline__ float exp2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

constexpr float kLog2e = 1.4426950408889634f;

struct Rbf {  // [B, N, C] with strides
  const float* p;
  int64_t sb, sn, sc;
  __device__ float at(int b, int i, int c) const { return p[b * sb + i * sn + c * sc]; }
};

__global__ void __launch_bounds__(256) forward_kernel(Grid g, int b, Rbf r, int N, int C,
                                                      float* __restrict__ vol) {
  __shared__ float tile[kTile][4 + kMaxAttr];
  const int A = C - 4;
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int xi = (int)(v % g.W), yi = (int)((v / g.W) % g.H), zi = (int)(v / ((int64_t)g.W * g.H));
  const float x = coord(g.sx, g.ex, g.W, xi), y = coord(g.sy, g.ey, g.H, yi);
  const float z = coord(g.sz, g.ez, g.D, zi);
  float sum = 0.f;
  float attr[kMaxAttr];
#pragma unroll
  for (int a = 0; a < kMaxAttr; ++a) attr[a] = 0.f;
  for (int i0 = 0; i0 < N; i0 += kTile) {
    __syncthreads();
    for (int j = threadIdx.x; j < kTile * C; j += blockDim.x) {
      const int i = j / C, c = j - i * C;
      if (i0 + i < N) {
        const float val = r.at(b, i0 + i, c);
        // slot 3 holds -log2(e) / (2 sigma^2) instead of sigma
        tile[i][c] = c == 3 ? -0.5f * kLog2e / (val * val) : val;
      }
    }
    __syncthreads();
    const int cnt = min(kTile, N - i0);
    for (int i = 0; i < cnt; ++i) {
      const float dx = tile[i][0] - x, dy = tile[i][1] - y, dz = tile[i][2] - z;
      const float w = exp2_approx(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * tile[i][3]);
      sum += w;
#pragma unroll
      for (int a = 0; a < kMaxAttr; ++a)
        if (a < A) attr[a] += w * tile[i][4 + a];
    }
  }
  if (v >= nv) return;
  float* out = vol + (size_t)b * (1 + A) * nv;
  out[v] = sum;
  const float norm = sum < 1e-8f ? 1.f : sum;
#pragma unroll
  for (int a = 0; a < kMaxAttr; ++a)
    if (a < A) out[(size_t)(1 + a) * nv + v] = attr[a] / norm;
}

constexpr int kChunk = 512;  // voxels staged per pass

// Gradient (rbf2volume_cuda.cu:124-201): thread = Gaussian, CTA = chunk of
// voxels (coordinates, volume and volume_grad channels staged in shared memory).
__global__ void __launch_bounds__(128) grad_kernel(Grid g, int b, Rbf r, int N, int C,
                                                   const float* __restrict__ vol,
                                                   const float* __restrict__ vgrad,
                                                   float* __restrict__ rgrad, int64_t gsb,
                                                   int64_t gsn, int64_t gsc, int64_t vox_per_cta) {
  extern __shared__ float sm[];  // [kChunk][4 + 2 * (1 + A)] : x y z pad | vol[1+A] | grad[1+A]
  const int A = C - 4;
  const int stride = 4 + 2 * (1 + A);
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < N;
  float xr = 0.f, yr = 0.f, zr = 0.f, sigma = 1.f;
  float ra[kMaxAttr];
#pragma unroll
  for (int a = 0; a < kMaxAttr; ++a) ra[a] = 0.f;
  if (active) {
    xr = r.at(b, i, 0);
    yr = r.at(b, i, 1);
    zr = r.at(b, i, 2);
    sigma = r.at(b, i, 3);
#pragma unroll
    for (int a = 0; a < kMaxAttr; ++a)
      if (a < A) ra[a] = r.at(b, i, 4 + a);
  }
  const float is2 = 1.f / (sigma * sigma);
  const float k2 = -0.5f * kLog2e * is2;  // w = 2^(d2 * k2)
  const float is3 = is2 / sigma;
  float gx = 0.f, gy = 0.f, gz = 0.f, gs = 0.f;
  float ga[kMaxAttr];
#pragma unroll
  for (int a = 0; a < kMaxAttr; ++a) ga[a] = 0.f;
  const float* vb = vol + (size_t)b * (1 + A) * nv;
  const float* gb = vgrad + (size_t)b * (1 + A) * nv;
  const int64_t v_begin = (int64_t)blockIdx.y * vox_per_cta;
  const int64_t v_end = min(nv, v_begin + vox_per_cta);
  for (int64_t c0 = v_begin; c0 < v_end; c0 += kChunk) {
    const int cnt = (int)min((int64_t)kChunk, v_end - c0);
    __syncthreads();
    for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
      const int64_t v = c0 + j;
      const int xi = (int)(v % g.W), yi = (int)((v / g.W) % g.H), zi = (int)(v / ((int64_t)g.W * g.H));
      float* e = sm + j * stride;
      e[0] = coord(g.sx, g.ex, g.W, xi);
      e[1] = coord(g.sy, g.ey, g.H, yi);
      e[2] = coord(g.sz, g.ez, g.D, zi);
      for (int q = 0; q <= A; ++q) {
        e[4 + q] = vb[(size_t)q * nv + v];
        e[4 + 1 + A + q] = gb[(size_t)q * nv + v];
      }
    }
    __syncthreads();
    if (!active) continue;
    for (int j = 0; j < cnt; ++j) {
      const float* e = sm + j * stride;
      const float x = e[0], y = e[1], z = e[2];
      const float ex = x - xr, ey = y - yr, ez = z - zr;
      const float d2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
      const float w = exp2_approx(d2 * k2);
      const float wi = is2 * w;
      const float dwx = ex * wi, dwy = ey * wi, dwz = ez * wi;
      const float dws = d2 * is3 * w;
      float dl = e[4 + 1 + A];
      if (A > 0) {
        float v0 = e[4];
        if (v0 < 1e-8f) v0 = 1.f;
        const float inv = 1.f / v0;
        float sum = 0.f;
#pragma unroll
        for (int a = 0; a < kMaxAttr; ++a) {
          if (a < A) {
            const float dla = e[4 + 1 + A + 1 + a];
            sum += dla * (ra[a] - e[4 + 1 + a]);
            ga[a] += dla * w * inv;
          }
        }
        dl += sum * inv;
      }
      gx += dwx * dl;
      gy += dwy * dl;
      gz += dwz * dl;
      gs += dws * dl;
    }
  }
  if (!active) return;
  float* out = rgrad + b * gsb + i * gsn;
  atomicAdd(out, gx);
  atomicAdd(out + gsc, gy);
  atomicAdd(out + 2 * gsc, gz);
  atomicAdd(out + 3 * gsc, gs);
#pragma unroll
  for (int a = 0; a < kMaxAttr; ++a)
    if (a < A) atomicAdd(out + (4 + a) * gsc, ga[a]);
}

}  // namespace rbf

namespace {

int check_rbf(const totri_array_t* r, const totri_array_t* vol, rbf::Grid& g, rbf::Rbf& rr,
              int64_t& B, int64_t& N, int& C, const float* start, const float* end) {
  TOTRI_TRY(check_array(r, "rbf", 3, -1));
  if (r->dtype != TOTRI_FLOAT32)
    return fail(TOTRI_ERR_UNSUPPORTED, "rbf2volume: only float32 tensors are supported");
  B = r->shape[0];
  N = r->shape[1];
  C = (int)r->shape[2];
  if (C < 4 || C > 4 + rbf::kMaxAttr)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "rbf must be [B, N, 4+A] with A <= 8");
  TOTRI_TRY(check_array(vol, "volume", 5, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(vol, "volume", 0, B));
  TOTRI_TRY(check_dim(vol, "volume", 1, C - 3));
  TOTRI_TRY(check_contiguous(vol, "volume"));
  g = rbf::Grid{(int)vol->shape[2], (int)vol->shape[3], (int)vol->shape[4], start[0], start[1],
                start[2], end[0], end[1], end[2]};
  rr = rbf::Rbf{static_cast<const float*>(r->data), r->strides[0], r->strides[1], r->strides[2]};
  return TOTRI_OK;
}

}  // namespace
}  // namespace totri

using namespace totri;

extern "C" {

int totri_rbf2volume_gaussian_forward(const totri_array_t* r, const totri_array_t* vol,
                                      const float start[3], const float end[3], void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  rbf::Grid g;
  rbf::Rbf rr;
  int64_t B, N;
  int C;
  TOTRI_TRY(check_rbf(r, vol, g, rr, B, N, C, start, end));
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  if (nv == 0 || B == 0) return TOTRI_OK;
  for (int b = 0; b < (int)B; ++b)
    TOTRI_KERNEL("rbf2volume forward", stream,
                 rbf::forward_kernel<<<(unsigned)ceil_div(nv, 256), 256, 0, stream>>>(
                     g, b, rr, (int)N, C, static_cast<float*>(vol->data)));
  return TOTRI_OK;
}

int totri_rbf2volume_gaussian_grad(const totri_array_t* r, const totri_array_t* vol,
                                   const totri_array_t* vgrad, const totri_array_t* rgrad,
                                   const float start[3], const float end[3], void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  rbf::Grid g;
  rbf::Rbf rr;
  int64_t B, N;
  int C;
  TOTRI_TRY(check_rbf(r, vol, g, rr, B, N, C, start, end));
  TOTRI_TRY(check_array(vgrad, "volume_grad", 5, TOTRI_FLOAT32));
  for (int d = 0; d < 5; ++d)
    if (vgrad->shape[d] != vol->shape[d])
      return fail(TOTRI_ERR_INVALID_ARGUMENT, "volume_grad must have the shape of volume");
  TOTRI_TRY(check_contiguous(vgrad, "volume_grad"));
  TOTRI_TRY(check_array(rgrad, "rbf_grad", 3, TOTRI_FLOAT32));
  for (int d = 0; d < 3; ++d)
    if (rgrad->shape[d] != r->shape[d])
      return fail(TOTRI_ERR_INVALID_ARGUMENT, "rbf_grad must have the shape of rbf");
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  if (nv == 0 || N == 0 || B == 0) return TOTRI_OK;
  const int A = C - 4;
  const size_t smem = sizeof(float) * rbf::kChunk * (4 + 2 * (1 + A));
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(rbf::grad_kernel), smem));
  // voxels per CTA: enough CTAs to fill the GPU several times over
  const int64_t rbf_blocks = ceil_div(N, 128);
  int64_t chunks = std::max<int64_t>(1, (152 * 8 + rbf_blocks - 1) / rbf_blocks);
  chunks = std::min<int64_t>(chunks, ceil_div(nv, rbf::kChunk));
  const int64_t per = ceil_div(ceil_div(nv, chunks), rbf::kChunk) * rbf::kChunk;
  chunks = ceil_div(nv, per);
  for (int b = 0; b < (int)B; ++b)
    TOTRI_KERNEL("rbf2volume grad", stream,
                 rbf::grad_kernel<<<dim3((unsigned)rbf_blocks, (unsigned)chunks), 128, smem,
                                    stream>>>(
                     g, b, rr, (int)N, C, static_cast<const float*>(vol->data),
                     static_cast<const float*>(vgrad->data), static_cast<float*>(rgrad->data),
                     rgrad->strides[0], rgrad->strides[1], rgrad->strides[2], per));
  return TOTRI_OK;
}

}  // extern "C"
