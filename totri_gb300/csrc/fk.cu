// f-k migration (reference totri/reconstruct/fk_migration.py:5-120): the
// transient is prepared (square root, linear time ramp, zero padding to 2D
// bins), transformed by a 3-D FFT (cuFFT through the caller), resampled in
// the frequency domain by the Stolt mapping, transformed back, and cropped
// to the magnitude of the first D bins.
//
// The reference centres the spectrum with fftshift before the resampling
// and un-centres it with ifftshift after; here both shifts are folded into
// the Stolt kernel's index arithmetic (fftshift(F)[q] = F[(q + ceil(n/2)) mod
// n], ifftshift(S)[j] = S[(j + floor(n/2)) mod n]), so the spectrum is read and
// written once. The resampling is grid_sample's trilinear interpolation
// without aligned corners and with zeros outside: the sample of output
// (z, y, x) on linspace(-1, 1) grids is taken at
// (x, y, sqrt(x^2 A + y^2 B + z^2)), A = (W depth / (2D width))^2,
// B = (H depth / (2D height))^2, and weighted by |z| / max(root, 1e-6) for
// z > 0 (fk_migration.py:40-86).
#include "capi_common.cuh"
#include "common.cuh"

namespace totri {
namespace fk {

// linspace(lo, hi, n)[i], evaluated from the nearer end as torch does.
__device__ __forceinline__ float lin(int i, int n, float lo, float hi) {
  if (n == 1) return lo;
  const float step = (hi - lo) / (float)(n - 1);
  return i < n / 2 ? lo + step * (float)i : hi - step * (float)(n - 1 - i);
}

__global__ void prepare_kernel(const float* __restrict__ t, float2* __restrict__ out, int N,
                               int D, int H, int W) {
  const int64_t plane = (int64_t)H * W;
  const int64_t total = (int64_t)N * 2 * D * plane;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int64_t p = i % plane;
  const int64_t nd = i / plane;
  const int d = (int)(nd % (2 * D));
  const int n = (int)(nd / (2 * D));
  float v = 0.f;
  if (d < D) v = sqrtf(t[((int64_t)n * D + d) * plane + p]) * lin(d, D, 0.f, 1.f);
  out[i] = make_float2(v, 0.f);
}

__global__ void stolt_kernel(const float2* __restrict__ in, float2* __restrict__ out, int M,
                             int D2, int H, int W, float A, float B, int in_centred,
                             int out_centred) {
  const int64_t plane = (int64_t)H * W;
  const int64_t total = (int64_t)M * D2 * plane;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int jw = (int)(i % W);
  const int jh = (int)((i / W) % H);
  const int jd = (int)((i / plane) % D2);
  const int64_t m = i / (plane * D2);
  // index in the centred spectrum the output element holds
  const int sd = out_centred ? jd : (jd + D2 / 2) % D2;
  const int sh = out_centred ? jh : (jh + H / 2) % H;
  const int sw = out_centred ? jw : (jw + W / 2) % W;
  const float z = lin(sd, D2, -1.f, 1.f);
  if (!(z > 0.f)) {
    out[i] = make_float2(0.f, 0.f);
    return;
  }
  const float x = lin(sw, W, -1.f, 1.f), y = lin(sh, H, -1.f, 1.f);
  const float zz = sqrtf(x * x * A + y * y * B + z * z);
  const float weight = fabsf(z) / fmaxf(zz, 1e-6f);
  const float pd = ((zz + 1.f) * D2 - 1.f) * 0.5f;
  const float ph = ((y + 1.f) * H - 1.f) * 0.5f;
  const float pw = ((x + 1.f) * W - 1.f) * 0.5f;
  const int d0 = (int)floorf(pd), h0 = (int)floorf(ph), w0 = (int)floorf(pw);
  const float fd = pd - d0, fh = ph - h0, fw = pw - w0;
  // centred index -> storage index of the input
  const int cd = in_centred ? 0 : (D2 + 1) / 2, ch = in_centred ? 0 : (H + 1) / 2,
            cw = in_centred ? 0 : (W + 1) / 2;
  const float2* base = in + m * D2 * plane;
  float re = 0.f, im = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int d = d0 + (k >> 2), h = h0 + ((k >> 1) & 1), w = w0 + (k & 1);
    if (d < 0 || d >= D2 || h < 0 || h >= H || w < 0 || w >= W) continue;
    const float wt = ((k >> 2) ? fd : 1.f - fd) * (((k >> 1) & 1) ? fh : 1.f - fh) *
                     ((k & 1) ? fw : 1.f - fw);
    const float2 v = base[((int64_t)((d + cd) % D2) * H + (h + ch) % H) * W + (w + cw) % W];
    re += wt * v.x;
    im += wt * v.y;
  }
  out[i] = make_float2(weight * re, weight * im);
}

__global__ void finish_kernel(const float2* __restrict__ v, float* __restrict__ out, int N,
                              int D, int H, int W) {
  const int64_t plane = (int64_t)H * W;
  const int64_t total = (int64_t)N * D * plane;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int64_t p = i % plane;
  const int64_t nd = i / plane;
  const int d = (int)(nd % D);
  const int n = (int)(nd / D);
  const float2 c = v[((int64_t)n * 2 * D + d) * plane + p];
  out[i] = hypotf(c.x, c.y);
}

int check_complex(const totri_array_t* a, const char* name) {
  TOTRI_TRY(check_array(a, name, 5, TOTRI_FLOAT32));
  TOTRI_TRY(check_contiguous(a, name));
  return check_dim(a, name, 4, 2);
}

}  // namespace fk
}  // namespace totri

using namespace totri;

extern "C" {

int totri_fk_prepare(const totri_array_t* transient, const totri_array_t* out, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  TOTRI_TRY(check_array(transient, "transient", 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  TOTRI_TRY(fk::check_complex(out, "out"));
  const int64_t N = transient->shape[0], D = transient->shape[1], H = transient->shape[2],
                W = transient->shape[3];
  TOTRI_TRY(check_dim(out, "out", 0, N));
  TOTRI_TRY(check_dim(out, "out", 1, 2 * D));
  TOTRI_TRY(check_dim(out, "out", 2, H));
  TOTRI_TRY(check_dim(out, "out", 3, W));
  const int64_t total = N * 2 * D * H * W;
  if (total == 0) return TOTRI_OK;
  TOTRI_KERNEL("fk prepare", stream,
               fk::prepare_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, stream>>>(
                   static_cast<const float*>(transient->data), static_cast<float2*>(out->data),
                   (int)N, (int)D, (int)H, (int)W));
  return TOTRI_OK;
}

int totri_fk_stolt(const totri_array_t* fourier, const totri_array_t* out, float depth,
                   float height, float width, int input_centred, int output_centred,
                   void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  TOTRI_TRY(fk::check_complex(fourier, "fourier"));
  TOTRI_TRY(fk::check_complex(out, "out"));
  for (int d = 0; d < 4; ++d) TOTRI_TRY(check_dim(out, "out", d, fourier->shape[d]));
  if (fourier->data == out->data)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "the Stolt resampling cannot run in place");
  const int64_t M = fourier->shape[0], D2 = fourier->shape[1], H = fourier->shape[2],
                W = fourier->shape[3];
  if (D2 % 2 != 0) return fail(TOTRI_ERR_INVALID_ARGUMENT, "the spectrum needs 2D time bins");
  const int64_t total = M * D2 * H * W;
  if (total == 0) return TOTRI_OK;
  const float D = (float)(D2 / 2);
  const float a = (float)W * depth / (2.f * D * width), b = (float)H * depth / (2.f * D * height);
  TOTRI_KERNEL("fk stolt", stream,
               fk::stolt_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, stream>>>(
                   static_cast<const float2*>(fourier->data), static_cast<float2*>(out->data),
                   (int)M, (int)D2, (int)H, (int)W, a * a, b * b, input_centred, output_centred));
  return TOTRI_OK;
}

int totri_fk_finish(const totri_array_t* volume, const totri_array_t* out, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  TOTRI_TRY(fk::check_complex(volume, "volume"));
  TOTRI_TRY(check_array(out, "out", 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_contiguous(out, "out"));
  const int64_t N = out->shape[0], D = out->shape[1], H = out->shape[2], W = out->shape[3];
  TOTRI_TRY(check_dim(volume, "volume", 0, N));
  TOTRI_TRY(check_dim(volume, "volume", 1, 2 * D));
  TOTRI_TRY(check_dim(volume, "volume", 2, H));
  TOTRI_TRY(check_dim(volume, "volume", 3, W));
  const int64_t total = N * D * H * W;
  if (total == 0) return TOTRI_OK;
  TOTRI_KERNEL("fk finish", stream,
               fk::finish_kernel<<<(unsigned)ceil_div(total, 256), 256, 0, stream>>>(
                   static_cast<const float2*>(volume->data), static_cast<float*>(out->data),
                   (int)N, (int)D, (int)H, (int)W));
  return TOTRI_OK;
}

}  // extern "C"
