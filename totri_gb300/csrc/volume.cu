// Voxel-volume transient renderer: confocal forward, its exact adjoint, the
// reference's transposed operator, the measurement-point gradient, and the
// exhaustive (laser/detector) forward with its adjoint.
//
// Reference: src/render/volume_cuda.cu. The reference forward gathers over
// every (point, bin, voxel column) (:12-66), O(N T X Y). The forward here
// scatters only occupied voxels: a voxel at slice k receives samples whose
// interpolation cell is k-1 or k, i.e. a contiguous run of ~4 bins per
// (voxel, point), found by inverting the sphere/column geometry and then
// re-deciding each bin with the reference's FP32 sample arithmetic. Each CTA
// owns a tile of points and keeps their transient rows in shared memory.
#include <cstring>
#include <string>

#include "capi_common.cuh"
#include "tune.cuh"

namespace totri {
namespace volume {

struct Geo {
  int X, Y, Z;
  float ox, oy, oz, sx, sy, sz;
  float scale;  // Z / sz
  float bw, bo;
  int T;
  int exact;  // 1: every sample takes the exact chain (tuning key "volume.exact")
};

// Column / slice centre: origin + ((i + 0.5) * size) / n (volume_cuda.cu:35,38).
__device__ __forceinline__ float centre(float o, float s, int n, int i) {
  return xadd(o, xdiv(xmul(xadd((float)i, 0.5f), s), (float)n));
}

struct Sample {
  bool ok;
  int zi;
  float alpha, f2;
};

// The reference's sample at (point w, bin t, column x/y) (volume_cuda.cu:23-57):
// FP32 decisions (depth^2 > 0, floor(z_hat), 0 <= zi, zi + 1 < Z) with one
// rounding per operation; alpha and f2 are values.
__device__ __forceinline__ Sample sample(const Geo& g, float wx, float wy, float wz, int t,
                                         float x, float y) {
  Sample s{false, 0, 0.f, 0.f};
  const float tc = xadd(xmul((float)t, g.bw), g.bo);
  const float dx = xsub(wx, x), dy = xsub(wy, y);
  const float d2 = xsub(xsub(xmul(tc, tc), xmul(dx, dx)), xmul(dy, dy));
  if (!(d2 > 0.f)) return s;
  const float depth = xsqrt(d2);
  const float z = xadd(wz, depth);
  const float zh = xsub(xmul(xsub(z, g.oz), g.scale), 0.5f);
  const float fl = floorf(zh);
  if (!(fl >= 0.f && fl + 1.f < (float)g.Z)) return s;
  s.ok = true;
  s.zi = (int)fl;
  s.alpha = zh - fl;
  const float q = __fdividef(depth, tc * tc);  // a value: the hardware reciprocal (2 ulp)
  s.f2 = (q * q) * (q * q);
  return s;
}

// sample() with a filtered fast path: the depth from the hardware reciprocal
// square root (within 6 u of the exact root, u = 2^-24) and z_hat from one
// fused multiply-add. Against the exact chain z_hat moves by at most
// scale 8 u (depth + |z| + |oz|) + 4 u |z_hat|, so where its fraction is
// farther than that (with |wz| added) from 0 and 1 the fast floor is the
// exact floor and the sample is kept; otherwise the exact sample() runs. The
// d2 > 0 test is taken on the exact d2 either way. alpha and f2 are values
// (few-ulp differences); every decision is the exact chain's. Used by the
// adjoint (247 -> 195 ms on 128^3 x 16384 points x 1024 bins); the forward,
// which only walks bins next to each occupied voxel's cell, ran 5% slower
// with it and keeps sample().
__device__ __forceinline__ Sample sample_filtered(const Geo& g, float wx, float wy, float wz,
                                                  int t, float x, float y) {
  if (g.exact) return sample(g, wx, wy, wz, t, x, y);
  Sample s{false, 0, 0.f, 0.f};
  const float tc = xadd(xmul((float)t, g.bw), g.bo);
  const float dx = xsub(wx, x), dy = xsub(wy, y);
  const float d2 = xsub(xsub(xmul(tc, tc), xmul(dx, dx)), xmul(dy, dy));
  if (!(d2 > 0.f)) return s;
  const float depth = d2 * rsqrtf(d2);
  const float z = wz + depth;
  const float zh = fmaf(z - g.oz, g.scale, -0.5f);
  const float fl = floorf(zh);
  const float fr = zh - fl;
  const float u = 5.9604645e-8f;
  const float m = 8.f * u * g.scale * (depth + fabsf(wz) + fabsf(z) + fabsf(g.oz)) +
                  4.f * u * fabsf(zh) + 1e-7f;
  if (!(fr > m && fr < 1.f - m)) return sample(g, wx, wy, wz, t, x, y);
  if (!(fl >= 0.f && fl + 1.f < (float)g.Z)) return s;
  s.ok = true;
  s.zi = (int)fl;
  s.alpha = fr;
  const float q = __fdividef(depth, tc * tc);
  s.f2 = (q * q) * (q * q);
  return s;
}

// Bins whose sample may fall in interpolation cells k-1 or k of a column
// (conservative: one extra bin each side).
__device__ __forceinline__ void bin_range(const Geo& g, float rho2, float wz, int k, int& t0,
                                          int& t1) {
  const float zlo = g.oz + ((float)k - 0.5f) / g.scale;
  const float zhi = g.oz + ((float)k + 1.5f) / g.scale;
  const float dhi = zhi - wz;
  if (!(dhi > 0.f)) {
    t0 = 1;
    t1 = 0;
    return;
  }
  const float dlo = fmaxf(zlo - wz, 0.f);
  const float tclo = sqrtf(dlo * dlo + rho2), tchi = sqrtf(dhi * dhi + rho2);
  t0 = max((int)floorf((tclo - g.bo) / g.bw) - 1, 0);
  t1 = min((int)ceilf((tchi - g.bo) / g.bw) + 1, g.T - 1);
}

struct Points {  // measurement points [3, N] with strides
  const float* p;
  int64_t sc, sn;
  __device__ float at(int c, int i) const { return p[c * sc + i * sn]; }
};

__global__ void compact_kernel(const float* __restrict__ vol, int64_t n, uint32_t* list,
                               uint32_t* count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool occ = i < n && vol[i] != 0.f;
  const uint32_t m = __ballot_sync(0xffffffffu, occ);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (occ) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)i;
}

constexpr int kPT = 8;  // points per CTA tile

// Confocal forward: tile of kPT points x all occupied voxels -> rows of the
// transient in shared memory -> coalesced row stores.
__global__ void __launch_bounds__(256) confocal_forward_kernel(
    Geo g, const float* __restrict__ vol, const uint32_t* __restrict__ list,
    const uint32_t* __restrict__ count, Points mp, int N, float* __restrict__ out) {
  extern __shared__ float hist[];  // [kPT][T]
  const int i0 = blockIdx.x * kPT;
  for (int j = threadIdx.x; j < kPT * g.T; j += blockDim.x) hist[j] = 0.f;
  __syncthreads();
  const uint32_t nnz = *count;
  const int pl = threadIdx.x % kPT;
  const int i = i0 + pl;
  if (i < N) {
    const float wx = mp.at(0, i), wy = mp.at(1, i), wz = mp.at(2, i);
    float* row = hist + pl * g.T;
    for (uint32_t v = threadIdx.x / kPT; v < nnz; v += blockDim.x / kPT) {
      const uint32_t lin = __ldg(list + v);
      const int k = (int)(lin % g.Z);
      const int yi = (int)((lin / g.Z) % g.Y), xi = (int)(lin / ((uint32_t)g.Z * g.Y));
      const float val = __ldg(vol + lin);
      const float x = centre(g.ox, g.sx, g.X, xi), y = centre(g.oy, g.sy, g.Y, yi);
      const float rho2 = (wx - x) * (wx - x) + (wy - y) * (wy - y);
      int t0, t1;
      bin_range(g, rho2, wz, k, t0, t1);
      for (int t = t0; t <= t1; ++t) {
        const Sample s = sample(g, wx, wy, wz, t, x, y);
        if (!s.ok) continue;
        float w;
        if (s.zi == k) w = 1.f - s.alpha;
        else if (s.zi == k - 1) w = s.alpha;
        else continue;
        atomicAdd(row + t, val * w * s.f2);
      }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < kPT * g.T; j += blockDim.x) {
    const int p = j / g.T, t = j - p * g.T;
    if (i0 + p < N) out[(size_t)(i0 + p) * g.T + t] = hist[j];
  }
}

// d transient / d measurement points (volume_cuda.cu:189-265) with the same
// occupied-voxel scatter; one thread accumulates one point's gradient over a
// share of the voxels, reduced across the kPT-strided threads in shared memory.
__global__ void __launch_bounds__(256) grad_mp_kernel(Geo g, const float* __restrict__ vol,
                                                      const uint32_t* __restrict__ list,
                                                      const uint32_t* __restrict__ count,
                                                      Points mp, int N,
                                                      const float* __restrict__ tg,
                                                      float* __restrict__ out, int64_t osc,
                                                      int64_t osn) {
  __shared__ float red[256][3];
  const int i0 = blockIdx.x * kPT;
  const uint32_t nnz = *count;
  const int pl = threadIdx.x % kPT;
  const int i = i0 + pl;
  float gx = 0.f, gy = 0.f, gz = 0.f;
  if (i < N) {
    const float wx = mp.at(0, i), wy = mp.at(1, i), wz = mp.at(2, i);
    const float* trow = tg + (size_t)i * g.T;
    for (uint32_t v = threadIdx.x / kPT; v < nnz; v += blockDim.x / kPT) {
      const uint32_t lin = __ldg(list + v);
      const int k = (int)(lin % g.Z);
      const int yi = (int)((lin / g.Z) % g.Y), xi = (int)(lin / ((uint32_t)g.Z * g.Y));
      const float val = __ldg(vol + lin);
      const float x = centre(g.ox, g.sx, g.X, xi), y = centre(g.oy, g.sy, g.Y, yi);
      const float rho2 = (wx - x) * (wx - x) + (wy - y) * (wy - y);
      int t0, t1;
      bin_range(g, rho2, wz, k, t0, t1);
      for (int t = t0; t <= t1; ++t) {
        const Sample s = sample(g, wx, wy, wz, t, x, y);
        if (!s.ok || (s.zi != k && s.zi != k - 1)) continue;
        const float tc = (float)t * g.bw + g.bo;
        const float depth = sqrtf(fmaxf(tc * tc - (wx - x) * (wx - x) - (wy - y) * (wy - y), 0.f));
        const float dzx = -(wx - x) / depth, dzy = -(wy - y) / depth;
        const float tc2 = tc * tc, tc4 = tc2 * tc2;
        const float df2 = 4.f * depth * depth * depth / (tc4 * tc4);
        // this voxel is the lower (zi == k) or upper (zi == k-1) interpolation node
        const bool lower = s.zi == k;
        const float wgt = lower ? 1.f - s.alpha : s.alpha;
        const float sgn = lower ? -1.f : 1.f;
        const float dl = __ldg(trow + t) * val;
        gx += dl * (wgt * df2 * dzx + sgn * g.scale * dzx * s.f2);
        gy += dl * (wgt * df2 * dzy + sgn * g.scale * dzy * s.f2);
        gz += dl * (sgn * g.scale * s.f2);
      }
    }
  }
  red[threadIdx.x][0] = gx;
  red[threadIdx.x][1] = gy;
  red[threadIdx.x][2] = gz;
  __syncthreads();
  if (threadIdx.x < kPT && i0 + threadIdx.x < N) {
    float a = 0.f, b = 0.f, c = 0.f;
    for (int j = threadIdx.x; j < blockDim.x; j += kPT) {
      a += red[j][0];
      b += red[j][1];
      c += red[j][2];
    }
    const int ii = i0 + threadIdx.x;
    out[ii * osn] = a;
    out[osc + ii * osn] = b;
    out[2 * osc + ii * osn] = c;
  }
}

// Bins whose samples can land in any interpolation cell of a column seen from
// a point at squared horizontal distance rho2 and height wz: cells 0 .. Z-2
// hold z in [oz + 0.5/scale, oz + (Z - 0.5)/scale), widened by one cell above
// and one bin each side (bin_range's span for cells 1 and Z - 1). Empty
// (t0 > t1) when the whole column lies below the point.
__device__ __forceinline__ void column_span(const Geo& g, float rho2, float wz, int& t0,
                                            int& t1) {
  const float zlo = g.oz + 0.5f / g.scale;
  const float zhi = g.oz + ((float)g.Z + 0.5f) / g.scale;
  const float dhi = zhi - wz;
  if (!(dhi > 0.f)) {
    t0 = 1;
    t1 = 0;
    return;
  }
  const float dlo = fmaxf(zlo - wz, 0.f);
  const float tclo = sqrtf(dlo * dlo + rho2), tchi = sqrtf(dhi * dhi + rho2);
  t0 = max((int)floorf((tclo - g.bo) / g.bw) - 1, 0);
  t1 = min((int)ceilf((tchi - g.bo) / g.bw) + 1, g.T - 1);
}

// Exact adjoint of the forward: one CTA per voxel column, a warp per point at a
// time, its lanes over the point's bins (neighbouring lanes' samples fall in
// neighbouring cells and the transient row is read 128 bytes at a time). Each
// warp accumulates into its own copy of the column in shared memory (eight
// copies), summed at the end. The per-point work (the column's bin span, the
// exact squared horizontal offsets of the sample chain, the filtered path's
// margin) is done once per point by one lane for 32 points at a time and
// handed to the warp with shuffles, instead of by all 32 lanes for every point
// (148 ms for that version on 128^3 voxels x 16,384 points x 1,024 bins).
// Samples are those of sample_filtered: the margin here bounds its
// per-sample margin over every bin of the span, so the kept samples and every
// decision are the exact chain's.
__global__ void __launch_bounds__(256) confocal_adjoint_kernel(Geo g, Points mp, int N,
                                                               const float* __restrict__ tr,
                                                               float* __restrict__ vol) {
  extern __shared__ float cols[];  // [8][Z]
  const int c = blockIdx.x;
  const int xi = c / g.Y, yi = c - xi * g.Y;
  for (int z = threadIdx.x; z < 8 * g.Z; z += blockDim.x) cols[z] = 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* col = cols + warp * g.Z;
  const float x = centre(g.ox, g.sx, g.X, xi), y = centre(g.oy, g.sy, g.Y, yi);
  const float u = 5.9604645e-8f;
  for (int base = warp * 32; base < N; base += 256) {
    // lane j prepares point base + j
    const int ip = base + lane;
    float wx = 0.f, wy = 0.f, wz = 0.f, ddx = 0.f, ddy = 0.f, marg = 0.f;
    int ta = 1, tb = 0;
    if (ip < N) {
      wx = mp.at(0, ip);
      wy = mp.at(1, ip);
      wz = mp.at(2, ip);
      const float dx = xsub(wx, x), dy = xsub(wy, y);
      ddx = xmul(dx, dx);
      ddy = xmul(dy, dy);
      column_span(g, dx * dx + dy * dy, wz, ta, tb);
      // sample_filtered's margin 8 u scale (depth + |wz| + |z| + |oz|) + 4 u |zh|
      // + 1e-7 with depth, |z| and |zh| at their largest over the span's bins
      const float tcm = fmaxf(fabsf((float)tb * g.bw + g.bo), fabsf((float)ta * g.bw + g.bo));
      const float dmax = 1.001f * tcm;
      const float zmax = fabsf(wz) + dmax;
      const float zhmax = (zmax + fabsf(g.oz)) * g.scale + 0.5f;
      marg = 8.f * u * g.scale * (dmax + fabsf(wz) + zmax + fabsf(g.oz)) + 4.f * u * zhmax +
             1e-7f;
    }
    const int np = min(32, N - base);
    for (int j = 0; j < np; ++j) {
      const int t0 = __shfl_sync(0xffffffffu, ta, j), t1 = __shfl_sync(0xffffffffu, tb, j);
      if (t0 > t1) continue;  // warp-uniform
      const float pwx = __shfl_sync(0xffffffffu, wx, j), pwy = __shfl_sync(0xffffffffu, wy, j);
      const float pwz = __shfl_sync(0xffffffffu, wz, j);
      const float pddx = __shfl_sync(0xffffffffu, ddx, j);
      const float pddy = __shfl_sync(0xffffffffu, ddy, j);
      const float pm = __shfl_sync(0xffffffffu, marg, j);
      const float* row = tr + (size_t)(base + j) * g.T;
      for (int t = t0 + lane; t <= t1; t += 32) {
        // sample_filtered with the point's constants
        const float tc = xadd(xmul((float)t, g.bw), g.bo);
        const float d2 = xsub(xsub(xmul(tc, tc), pddx), pddy);
        if (!(d2 > 0.f)) continue;
        Sample sm;
        const float depth = d2 * rsqrtf(d2);
        const float zh = fmaf((pwz + depth) - g.oz, g.scale, -0.5f);
        const float fl = floorf(zh);
        const float fr = zh - fl;
        if (!g.exact && fr > pm && fr < 1.f - pm) {
          if (!(fl >= 0.f && fl + 1.f < (float)g.Z)) continue;
          sm.zi = (int)fl;
          sm.alpha = fr;
          const float q = __fdividef(depth, tc * tc);
          sm.f2 = (q * q) * (q * q);
        } else {
          sm = sample(g, pwx, pwy, pwz, t, x, y);
          if (!sm.ok) continue;
        }
        const float v = __ldg(row + t) * sm.f2;
        atomicAdd(col + sm.zi, (1.f - sm.alpha) * v);
        atomicAdd(col + sm.zi + 1, sm.alpha * v);
      }
    }
  }
  __syncthreads();
  for (int z = threadIdx.x; z < g.Z; z += blockDim.x) {
    float sum = 0.f;
    for (int w = 0; w < 8; ++w) sum += cols[w * g.Z + z];
    vol[(size_t)c * g.Z + z] = sum;
  }
}

// The reference's transposed operator, per voxel (volume_cuda.cu:96-160).
__global__ void confocal_transposed_kernel(Geo g, Points mp, int N, const float* __restrict__ tr,
                                           float* __restrict__ vol) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (int64_t)g.X * g.Y * g.Z) return;
  const int zi = (int)(v % g.Z), yi = (int)((v / g.Z) % g.Y), xi = (int)(v / ((int64_t)g.Z * g.Y));
  const float x = centre(g.ox, g.sx, g.X, xi), y = centre(g.oy, g.sy, g.Y, yi);
  const float z = centre(g.oz, g.sz, g.Z, zi);
  const float dz = xdiv(g.sz, (float)g.Z);
  const float zz = zi > 0 ? dz : 0.f;
  float value = 0.f;
  for (int i = 0; i < N; ++i) {
    const float wx = mp.at(0, i), wy = mp.at(1, i), wz = mp.at(2, i);
    const float dp2 = xadd(xmul(xsub(x, wx), xsub(x, wx)), xmul(xsub(y, wy), xsub(y, wy)));
    const float a = xsub(xsub(z, zz), wz), m = xsub(z, wz), e = xsub(xadd(z, dz), wz);
    auto tbin = [&](float q) {
      const float d = xsqrt(xadd(dp2, xmul(q, q)));
      const float cb = ceilf(xdiv(xsub(d, g.bo), g.bw));
      return (int)fminf(fmaxf(cb, 0.f), (float)g.T);
    };
    const int ts = tbin(a), tm = tbin(m), te = tbin(e);
    const float* row = tr + (size_t)i * g.T;
    for (int t = ts; t < te; ++t) {
      const float tc = xadd(xmul((float)t, g.bw), g.bo);
      const float d2 = xsub(xmul(tc, tc), dp2);
      if (!(d2 > 0.f)) continue;
      const float depth = xsqrt(d2);
      const float zh = xsub(xmul(xsub(xadd(wz, depth), g.oz), g.scale), 0.5f);
      const float al = zh - floorf(zh);
      const float w = (t >= tm) ? 1.f - al : al;
      const float q = depth / (tc * tc);
      value += w * ((q * q) * (q * q)) * __ldg(row + t);
    }
  }
  vol[v] = value;
}

}  // namespace volume

namespace {

using volume::Geo;
using volume::Points;

int check_volume_args(const totri_array_t* vol, const totri_array_t* mp, int& X, int& Y, int& Z,
                      int& N, Points& pts) {
  TOTRI_TRY(check_array(vol, "volume", 3, -1));
  if (vol->dtype != TOTRI_FLOAT32)
    return fail(TOTRI_ERR_UNSUPPORTED, "volume renderer: only float32 tensors are supported");
  TOTRI_TRY(check_contiguous(vol, "volume"));
  TOTRI_TRY(check_array(mp, "measurement_points", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(mp, "measurement_points", 0, 3));
  X = (int)vol->shape[0];
  Y = (int)vol->shape[1];
  Z = (int)vol->shape[2];
  N = (int)mp->shape[1];
  pts = Points{static_cast<const float*>(mp->data), mp->strides[0], mp->strides[1]};
  return TOTRI_OK;
}

Geo make_geo(int X, int Y, int Z, const float* o, const float* s, float bw, float bo, int T) {
  Geo g;
  g.X = X;
  g.Y = Y;
  g.Z = Z;
  g.ox = o[0];
  g.oy = o[1];
  g.oz = o[2];
  g.sx = s[0];
  g.sy = s[1];
  g.sz = s[2];
  g.scale = (float)Z / s[2];
  g.bw = bw;
  g.bo = bo;
  g.T = T;
  g.exact = tune::get("volume.exact") == 1;
  return g;
}

size_t occupancy_bytes(int64_t nvox) { return align_up(sizeof(uint32_t) * (nvox + 64), 256); }

int compact(const float* vol, int64_t n, void* ws, size_t ws_bytes, uint32_t** list,
            uint32_t** count, cudaStream_t stream) {
  const size_t need = occupancy_bytes(n);
  if (!ws || ws_bytes < need)
    return fail(TOTRI_ERR_WORKSPACE,
                "workspace of " + std::to_string(need) + " bytes required, got " +
                    std::to_string(ws_bytes));
  *count = static_cast<uint32_t*>(ws);
  *list = *count + 64;
  TOTRI_CUDA(cudaMemsetAsync(*count, 0, sizeof(uint32_t), stream));
  TOTRI_KERNEL("volume compact", stream,
               volume::compact_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, stream>>>(
                   vol, n, *list, *count));
  return TOTRI_OK;
}

}  // namespace
}  // namespace totri

using namespace totri;

extern "C" {

size_t totri_volume_workspace(int64_t num_voxels) {
  return num_voxels > 0 ? occupancy_bytes(num_voxels) : 0;
}

int totri_volume_confocal_forward(const totri_array_t* vol, const totri_array_t* mp,
                                  const totri_array_t* tr, const float origin[3],
                                  const float size[3], float bw, float bo, void* ws,
                                  size_t ws_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  int X, Y, Z, N;
  Points pts;
  TOTRI_TRY(check_volume_args(vol, mp, X, Y, Z, N, pts));
  TOTRI_TRY(check_array(tr, "transient", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(tr, "transient", 0, N));
  TOTRI_TRY(check_contiguous(tr, "transient"));
  const int T = (int)tr->shape[1];
  if (N == 0 || T == 0) return TOTRI_OK;
  const size_t smem = sizeof(float) * volume::kPT * T;
  if (smem > 200 * 1024) return fail(TOTRI_ERR_UNSUPPORTED, "too many bins for one tile");
  uint32_t *list, *count;
  TOTRI_TRY(compact(static_cast<const float*>(vol->data), numel(vol), ws, ws_bytes, &list,
                    &count, stream));
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(volume::confocal_forward_kernel), smem));
  const Geo g = make_geo(X, Y, Z, origin, size, bw, bo, T);
  TOTRI_KERNEL("volume confocal forward", stream,
               volume::confocal_forward_kernel<<<(unsigned)ceil_div(N, volume::kPT), 256, smem,
                                                 stream>>>(
                   g, static_cast<const float*>(vol->data), list, count, pts, N,
                   static_cast<float*>(tr->data)));
  return TOTRI_OK;
}

int totri_volume_confocal_adjoint(const totri_array_t* vol, const totri_array_t* mp,
                                  const totri_array_t* tr, const float origin[3],
                                  const float size[3], float bw, float bo, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  int X, Y, Z, N;
  Points pts;
  TOTRI_TRY(check_volume_args(vol, mp, X, Y, Z, N, pts));
  TOTRI_TRY(check_array(tr, "transient", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(tr, "transient", 0, N));
  TOTRI_TRY(check_contiguous(tr, "transient"));
  const int T = (int)tr->shape[1];
  if (numel(vol) == 0) return TOTRI_OK;
  if (N == 0 || T == 0) {
    TOTRI_CUDA(cudaMemsetAsync(vol->data, 0, sizeof(float) * numel(vol), stream));
    return TOTRI_OK;
  }
  const Geo g = make_geo(X, Y, Z, origin, size, bw, bo, T);
  const size_t smem = sizeof(float) * 8 * (size_t)Z;
  if (smem > 200 * 1024) return fail(TOTRI_ERR_UNSUPPORTED, "volume too deep for one column tile");
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(volume::confocal_adjoint_kernel), smem));
  TOTRI_KERNEL("volume confocal adjoint", stream,
               volume::confocal_adjoint_kernel<<<(unsigned)(X * Y), 256, smem, stream>>>(
                   g, pts, N, static_cast<const float*>(tr->data), static_cast<float*>(vol->data)));
  return TOTRI_OK;
}

int totri_volume_confocal_grad_volume(const totri_array_t* vol, const totri_array_t* mp,
                                      const totri_array_t* tr, const float origin[3],
                                      const float size[3], float bw, float bo, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  int X, Y, Z, N;
  Points pts;
  TOTRI_TRY(check_volume_args(vol, mp, X, Y, Z, N, pts));
  TOTRI_TRY(check_array(tr, "transient", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(tr, "transient", 0, N));
  TOTRI_TRY(check_contiguous(tr, "transient"));
  const int T = (int)tr->shape[1];
  const int64_t nv = numel(vol);
  if (nv == 0) return TOTRI_OK;
  const Geo g = make_geo(X, Y, Z, origin, size, bw, bo, T);
  TOTRI_KERNEL("volume confocal transposed", stream,
               volume::confocal_transposed_kernel<<<(unsigned)ceil_div(nv, 128), 128, 0, stream>>>(
                   g, pts, N, static_cast<const float*>(tr->data), static_cast<float*>(vol->data)));
  return TOTRI_OK;
}

int totri_volume_confocal_grad_measurement_points(const totri_array_t* mpg,
                                                  const totri_array_t* vol,
                                                  const totri_array_t* mp,
                                                  const totri_array_t* tg, const float origin[3],
                                                  const float size[3], float bw, float bo,
                                                  void* ws, size_t ws_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  int X, Y, Z, N;
  Points pts;
  TOTRI_TRY(check_volume_args(vol, mp, X, Y, Z, N, pts));
  TOTRI_TRY(check_array(mpg, "measurement_points_grad", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(mpg, "measurement_points_grad", 0, 3));
  TOTRI_TRY(check_dim(mpg, "measurement_points_grad", 1, N));
  TOTRI_TRY(check_array(tg, "transient_grad", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(tg, "transient_grad", 0, N));
  TOTRI_TRY(check_contiguous(tg, "transient_grad"));
  const int T = (int)tg->shape[1];
  if (N == 0) return TOTRI_OK;
  uint32_t *list, *count;
  TOTRI_TRY(compact(static_cast<const float*>(vol->data), numel(vol), ws, ws_bytes, &list,
                    &count, stream));
  const Geo g = make_geo(X, Y, Z, origin, size, bw, bo, T);
  TOTRI_KERNEL("volume confocal grad points", stream,
               volume::grad_mp_kernel<<<(unsigned)ceil_div(N, volume::kPT), 256, 0, stream>>>(
                   g, static_cast<const float*>(vol->data), list, count, pts, N,
                   static_cast<const float*>(tg->data), static_cast<float*>(mpg->data),
                   mpg->strides[0], mpg->strides[1]));
  return TOTRI_OK;
}

}  // extern "C"
