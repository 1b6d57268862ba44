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
#include <algorithm>
#include <climits>
#include <cmath>
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
  float inv_bw;
  int T;
  int exact;     // 1: every sample takes the exact chain (tuning key "volume.exact")
  int all_bins;  // bin width not positive and finite (or offset not finite): walk every bin
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

// First bin whose centre t bw + bo (the sample chain's FP32 arithmetic) is not
// negative; 0 unless the bin offset is negative. Bins before it have negative
// centres, whose samples mirror those of the positive centres (the reference
// walks every bin and squares the centre).
__device__ __forceinline__ int first_nonneg_bin(const Geo& g) {
  if (g.all_bins || !(g.bo < 0.f)) return 0;
  const float tf = ceilf(-g.bo * g.inv_bw);
  if (!(tf < (float)g.T)) return g.T;
  int t = max((int)tf - 2, 0);
  while (t > 0 && xadd(xmul((float)(t - 1), g.bw), g.bo) >= 0.f) --t;
  while (t < g.T && xadd(xmul((float)t, g.bw), g.bo) < 0.f) ++t;
  return t;
}

// Bins whose centre's magnitude lies in [cl, ch] widened by eps bins: [p0, p1]
// with non-negative centres (t >= tz) and [n0, n1] with negative ones (t < tz).
// Every bin when the bin width is degenerate. A NaN bound gives empty spans.
struct Spans {
  int p0, p1, n0, n1;
};
__device__ __forceinline__ Spans tc_spans(const Geo& g, int tz, float cl, float ch, float eps) {
  Spans s{1, 0, 1, 0};
  if (g.all_bins) {
    s.p0 = 0;
    s.p1 = g.T - 1;
    return s;
  }
  if (!(cl <= ch)) return s;
  s.p0 = max(__float2int_ru((cl - g.bo) * g.inv_bw - eps), tz);
  s.p1 = min(__float2int_rd((ch - g.bo) * g.inv_bw + eps), g.T - 1);
  if (tz > 0) {
    s.n0 = max(__float2int_ru((-ch - g.bo) * g.inv_bw - eps), 0);
    s.n1 = min(__float2int_rd((-cl - g.bo) * g.inv_bw + eps), tz - 1);
  }
  return s;
}

// Centre magnitudes [cl, ch] of the bins whose samples from a point at squared
// horizontal distance rho2 and height wz can land in z in [zlo, zhi); false
// when the whole interval lies below the point.
__device__ __forceinline__ bool tc_bounds(float rho2, float wz, float zlo, float zhi, float& cl,
                                          float& ch) {
  const float dhi = zhi - wz;
  if (!(dhi > 0.f)) return false;
  const float dlo = fmaxf(zlo - wz, 0.f);
  cl = sqrtf(dlo * dlo + rho2);
  ch = sqrtf(dhi * dhi + rho2);
  return true;
}

// The widening, in bins, of a span from tc_bounds whose largest centre
// magnitude is ch: the bound of confocal_adjoint_cells_kernel on the FP32
// rounding of the sample chain against that inverse (64 u of the largest
// magnitudes over the bin width, plus 0.01, at most one bin), with the
// largest |tc| of the walked bins at most ch plus one bin.
__device__ __forceinline__ float span_eps(const Geo& g, float ch, float wz) {
  const float u = 5.9604645e-8f;
  const float dmax = 1.001f * (ch + fabsf(g.bw));
  const float zmax = fabsf(wz) + dmax;
  return fminf(64.f * u * (dmax + fabsf(g.bo) + fabsf(wz) + zmax + fabsf(g.oz) +
                           fabsf(1.f / g.scale)) * g.inv_bw + 0.01f,
               1.f);
}

// Bins whose sample may fall in interpolation cells k-1 or k of a column,
// widened by span_eps (a whole bin each side walked about two more bins per
// (voxel, point) pair of the forward).
__device__ __forceinline__ Spans bin_range(const Geo& g, int tz, float rho2, float wz, int k) {
  float cl, ch;
  if (!tc_bounds(rho2, wz, g.oz + ((float)k - 0.5f) / g.scale,
                 g.oz + ((float)k + 1.5f) / g.scale, cl, ch))
    return Spans{1, 0, 1, 0};
  return tc_spans(g, tz, cl, ch, span_eps(g, ch, wz));
}

struct Points {  // measurement points [3, N] with strides
  const float* p;
  int64_t sc, sn;
  __device__ float at(int c, int i) const { return p[c * sc + i * sn]; }
};

// The occupied voxels of a [X][Y][Z] volume as records (column centre x, y,
// value, cell k): the per-voxel decoding (two divisions of the index, two
// correctly rounded divisions for the centres) is done once here instead of
// once per (voxel, point) pair.
__global__ void compact_kernel(Geo g, const float* __restrict__ vol, int64_t n, float4* recs,
                               uint32_t* count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool occ = i < n && vol[i] != 0.f;
  const uint32_t m = __ballot_sync(0xffffffffu, occ);
  if (!m) return;
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  if (occ) {
    const uint32_t lin = (uint32_t)i;
    const int k = (int)(lin % g.Z);
    const int yi = (int)((lin / g.Z) % g.Y), xi = (int)(lin / ((uint32_t)g.Z * g.Y));
    recs[base + __popc(m & ((1u << lane) - 1u))] =
        make_float4(centre(g.ox, g.sx, g.X, xi), centre(g.oy, g.sy, g.Y, yi), vol[i],
                    __int_as_float(k));
  }
}

constexpr int kPT = 8;  // points per CTA tile

// Confocal forward: tile of kPT points x all occupied voxels -> rows of the
// transient in shared memory -> coalesced row stores.
__global__ void __launch_bounds__(256) confocal_forward_kernel(
    Geo g, const float4* __restrict__ recs, const uint32_t* __restrict__ count, Points mp, int N,
    float* __restrict__ out) {
  extern __shared__ float hist[];  // [kPT][T]
  const int i0 = blockIdx.x * kPT;
  for (int j = threadIdx.x; j < kPT * g.T; j += blockDim.x) hist[j] = 0.f;
  __syncthreads();
  const uint32_t nnz = *count;
  const int pl = threadIdx.x % kPT;
  const int i = i0 + pl;
  const int tz = first_nonneg_bin(g);
  if (i < N) {
    const float wx = mp.at(0, i), wy = mp.at(1, i), wz = mp.at(2, i);
    float* row = hist + pl * g.T;
    for (uint32_t v = threadIdx.x / kPT; v < nnz; v += blockDim.x / kPT) {
      const float4 rec = __ldg(recs + v);
      const float x = rec.x, y = rec.y, val = rec.z;
      const int k = __float_as_int(rec.w);
      const float rho2 = (wx - x) * (wx - x) + (wy - y) * (wy - y);
      const Spans sp = bin_range(g, tz, rho2, wz, k);
      for (int r = 0; r < 2; ++r) {
        const int t0 = r ? sp.n0 : sp.p0, t1 = r ? sp.n1 : sp.p1;
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
__global__ void __launch_bounds__(256) grad_mp_kernel(Geo g, const float4* __restrict__ recs,
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
  const int tz = first_nonneg_bin(g);
  if (i < N) {
    const float wx = mp.at(0, i), wy = mp.at(1, i), wz = mp.at(2, i);
    const float* trow = tg + (size_t)i * g.T;
    for (uint32_t v = threadIdx.x / kPT; v < nnz; v += blockDim.x / kPT) {
      const float4 rec = __ldg(recs + v);
      const float x = rec.x, y = rec.y, val = rec.z;
      const int k = __float_as_int(rec.w);
      const float rho2 = (wx - x) * (wx - x) + (wy - y) * (wy - y);
      const Spans sp = bin_range(g, tz, rho2, wz, k);
      for (int r = 0; r < 2; ++r) {
        const int t0 = r ? sp.n0 : sp.p0, t1 = r ? sp.n1 : sp.p1;
        for (int t = t0; t <= t1; ++t) {
          const Sample s = sample(g, wx, wy, wz, t, x, y);
          if (!s.ok || (s.zi != k && s.zi != k - 1)) continue;
          const float tc = (float)t * g.bw + g.bo;
          const float depth =
              sqrtf(fmaxf(tc * tc - (wx - x) * (wx - x) - (wy - y) * (wy - y), 0.f));
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
// and one bin each side (bin_range's spans for cells 1 and Z - 1).
__device__ __forceinline__ Spans column_span(const Geo& g, int tz, float rho2, float wz) {
  float cl, ch;
  if (!tc_bounds(rho2, wz, g.oz + 0.5f / g.scale, g.oz + ((float)g.Z + 0.5f) / g.scale, cl, ch))
    return Spans{1, 0, 1, 0};
  return tc_spans(g, tz, cl, ch, 1.f);
}

// Largest |t bw + bo| over the bins of two spans (0 when both are empty).
__device__ __forceinline__ float span_tc_max(const Geo& g, const Spans& s) {
  float m = 0.f;
  if (s.p0 <= s.p1)
    m = fmaxf(fabsf((float)s.p1 * g.bw + g.bo), fabsf((float)s.p0 * g.bw + g.bo));
  if (s.n0 <= s.n1)
    m = fmaxf(m, fmaxf(fabsf((float)s.n1 * g.bw + g.bo), fabsf((float)s.n0 * g.bw + g.bo)));
  return m;
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
  const int tz = first_nonneg_bin(g);
  for (int base = warp * 32; base < N; base += 256) {
    // lane j prepares point base + j
    const int ip = base + lane;
    float wx = 0.f, wy = 0.f, wz = 0.f, ddx = 0.f, ddy = 0.f, marg = 0.f;
    Spans sp{1, 0, 1, 0};
    if (ip < N) {
      wx = mp.at(0, ip);
      wy = mp.at(1, ip);
      wz = mp.at(2, ip);
      const float dx = xsub(wx, x), dy = xsub(wy, y);
      ddx = xmul(dx, dx);
      ddy = xmul(dy, dy);
      sp = column_span(g, tz, dx * dx + dy * dy, wz);
      // sample_filtered's margin 8 u scale (depth + |wz| + |z| + |oz|) + 4 u |zh|
      // + 1e-7 with depth, |z| and |zh| at their largest over the spans' bins
      const float dmax = 1.001f * span_tc_max(g, sp);
      const float zmax = fabsf(wz) + dmax;
      const float zhmax = (zmax + fabsf(g.oz)) * g.scale + 0.5f;
      marg = 8.f * u * g.scale * (dmax + fabsf(wz) + zmax + fabsf(g.oz)) + 4.f * u * zhmax +
             1e-7f;
    }
    const int np = min(32, N - base);
    for (int j = 0; j < np; ++j) {
      const int p0 = __shfl_sync(0xffffffffu, sp.p0, j), p1 = __shfl_sync(0xffffffffu, sp.p1, j);
      const int n0 = __shfl_sync(0xffffffffu, sp.n0, j), n1 = __shfl_sync(0xffffffffu, sp.n1, j);
      if (p0 > p1 && n0 > n1) continue;  // warp-uniform
      const float pwx = __shfl_sync(0xffffffffu, wx, j), pwy = __shfl_sync(0xffffffffu, wy, j);
      const float pwz = __shfl_sync(0xffffffffu, wz, j);
      const float pddx = __shfl_sync(0xffffffffu, ddx, j);
      const float pddy = __shfl_sync(0xffffffffu, ddy, j);
      const float pm = __shfl_sync(0xffffffffu, marg, j);
      const float* row = tr + (size_t)(base + j) * g.T;
      for (int r = 0; r < 2; ++r) {
        const int t0 = r ? n0 : p0, t1 = r ? n1 : p1;
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
  }
  __syncthreads();
  for (int z = threadIdx.x; z < g.Z; z += blockDim.x) {
    float sum = 0.f;
    for (int w = 0; w < 8; ++w) sum += cols[w * g.Z + z];
    vol[(size_t)c * g.Z + z] = sum;
  }
}

// Exact adjoint of the forward without atomics, for columns of at most 32 CPL
// cells: one CTA per voxel column, each warp over a share of the points (all
// 32 lanes on the same point), lane l owning the CPL cells z0 = l CPL ..
// z0 + CPL - 1. A sample whose lower interpolation cell zi is the lane's adds
// (1 - alpha) v to cell zi and alpha v to cell zi + 1; when zi + 1 is the next
// lane's first cell that share goes to a per-lane carry register, added in at
// the end. The samples a lane walks are those of the bins whose centres map to
// its cells: the bin coordinate of each cell boundary from one square root,
// widened by eps bins, a bound on the FP32 rounding of the sample chain
// against that inverse (64 u of the largest magnitudes, over the bin width,
// plus 0.01, at most the one bin of column_span, inside which the per-point
// margin holds). Each sample's decisions are the exact chain's (sample_filtered
// with the per-point margin, as in confocal_adjoint_kernel), so every kept
// sample is the forward's and each lands in exactly one lane.
template <int CPL>
__global__ void __launch_bounds__(256) confocal_adjoint_cells_kernel(Geo g, Points mp, int N,
                                                                     const float* __restrict__ tr,
                                                                     float* __restrict__ vol) {
  __shared__ float cells[8][CPL][32];  // [warp][cell of the lane][lane]
  __shared__ float carry_in[8][32];
  const int c = blockIdx.x;
  const int xi = c / g.Y, yi = c - xi * g.Y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < CPL; ++k) cells[warp][k][lane] = 0.f;
  const float x = centre(g.ox, g.sx, g.X, xi), y = centre(g.oy, g.sy, g.Y, yi);
  const float u = 5.9604645e-8f;
  const int tz = first_nonneg_bin(g);
  // this lane's lower cells zi in [za, zb): z in [zlo, zhi)
  const int za = lane * CPL, zb = min(za + CPL, g.Z - 1);
  const float zlo = g.oz + ((float)za + 0.5f) / g.scale;
  const float zhi = g.oz + ((float)zb + 0.5f) / g.scale;
  float carry = 0.f;
  for (int base = warp * 32; base < N; base += 256) {
    // lane j prepares point base + j
    const int ip = base + lane;
    float wx = 0.f, wy = 0.f, wz = 0.f, ddx = 0.f, ddy = 0.f, marg = 0.f, eps = 0.f;
    if (ip < N) {
      wx = mp.at(0, ip);
      wy = mp.at(1, ip);
      wz = mp.at(2, ip);
      const float dx = xsub(wx, x), dy = xsub(wy, y);
      ddx = xmul(dx, dx);
      ddy = xmul(dy, dy);
      const Spans sp = column_span(g, tz, dx * dx + dy * dy, wz);
      const float dmax = 1.001f * span_tc_max(g, sp);
      const float zmax = fabsf(wz) + dmax;
      const float zhmax = (zmax + fabsf(g.oz)) * g.scale + 0.5f;
      marg = 8.f * u * g.scale * (dmax + fabsf(wz) + zmax + fabsf(g.oz)) + 4.f * u * zhmax +
             1e-7f;
      eps = fminf(64.f * u * (dmax + fabsf(g.bo) + fabsf(wz) + zmax + fabsf(g.oz) +
                              1.f / g.scale) * g.inv_bw + 0.01f,
                  1.f);
    }
    const int np = min(32, N - base);
    for (int j = 0; j < np; ++j) {
      const float pwx = __shfl_sync(0xffffffffu, wx, j), pwy = __shfl_sync(0xffffffffu, wy, j);
      const float pwz = __shfl_sync(0xffffffffu, wz, j);
      const float pddx = __shfl_sync(0xffffffffu, ddx, j);
      const float pddy = __shfl_sync(0xffffffffu, ddy, j);
      const float pm = __shfl_sync(0xffffffffu, marg, j);
      const float pe = __shfl_sync(0xffffffffu, eps, j);
      Spans sp{1, 0, 1, 0};
      float cl, ch;
      if (za < zb && tc_bounds(pddx + pddy, pwz, zlo, zhi, cl, ch))
        sp = tc_spans(g, tz, cl, ch, pe);
      const float* row = tr + (size_t)(base + j) * g.T;
      for (int r = 0; r < 2; ++r) {
        const int t0 = r ? sp.n0 : sp.p0, t1 = r ? sp.n1 : sp.p1;
        for (int t = t0; t <= t1; ++t) {
          const float tc = xadd(xmul((float)t, g.bw), g.bo);
          const float d2 = xsub(xsub(xmul(tc, tc), pddx), pddy);
          if (!(d2 > 0.f)) continue;
          int zi;
          float alpha, f2;
          const float depth = d2 * rsqrtf(d2);
          const float zh = fmaf((pwz + depth) - g.oz, g.scale, -0.5f);
          const float fl = floorf(zh);
          const float fr = zh - fl;
          if (!g.exact && fr > pm && fr < 1.f - pm) {
            if (!(fl >= (float)za && fl < (float)zb)) continue;
            zi = (int)fl;
            alpha = fr;
            const float q = __fdividef(depth, tc * tc);
            f2 = (q * q) * (q * q);
          } else {
            const Sample sm = sample(g, pwx, pwy, pwz, t, x, y);
            if (!sm.ok || sm.zi < za || sm.zi >= zb) continue;
            zi = sm.zi;
            alpha = sm.alpha;
            f2 = sm.f2;
          }
          const float v = __ldg(row + t) * f2;
          const int k = zi - za;
          cells[warp][k][lane] += (1.f - alpha) * v;
          if (k + 1 < CPL) cells[warp][k + 1][lane] += alpha * v;
          else carry += alpha * v;
        }
      }
    }
  }
  carry_in[warp][lane] = carry;
  __syncthreads();
  for (int z = threadIdx.x; z < g.Z; z += blockDim.x) {
    const int l = z / CPL, k = z - l * CPL;
    float sum = 0.f;
    for (int w = 0; w < 8; ++w) {
      sum += cells[w][k][l];
      if (k == 0 && l > 0) sum += carry_in[w][l - 1];
    }
    vol[(size_t)c * g.Z + z] = sum;
  }
}

constexpr int kAdjUnroll = 4;  // bins per step of the lanes-over-columns adjoint
// (8 bins per step, at 80 registers, measured the same: 65.6 against 65.8 ms)
constexpr int kAdjTablePad = kAdjUnroll;  // table entries past the last bin

// The bins [t0, t1] of one point for the lanes' columns, kAdjUnroll at a time:
// the fast path without branches (a sample that is not taken adds zero to
// cell 0), then the few samples that sit within the rounding margin of a cell
// boundary through the exact chain. Without kCheck (the bins with
// non-negative centres, walked last) the step may run up to kAdjUnroll - 1
// bins past t1: those are real bins (walked with their values, and rejected
// unless they hold a sample) up to T - 1, and table padding (tc^2 = -inf)
// beyond it; with kCheck (the negative centres, whose later bins belong to
// the other walk) bins past t1 are skipped. z_hat = (depth + (wz - oz)) scale
// - 0.5: the rounding of either association is inside sample_filtered's
// margin.
template <bool kCheck, int U>
__device__ __forceinline__ void adj_walk(const Geo& g, const float2* __restrict__ tab,
                                         const float* __restrict__ row, float* col, int t0,
                                         int t1, int lane, float ddx, float ddy, float wz,
                                         float wzo, float pm, float wx, float wy, float x,
                                         float y, int za, int zn) {
  const int tend = kCheck ? t1 : g.T - 1;  // last bin whose value is read
  float wval = 0.f;                        // bin t0 + 32 k + lane
  for (int t = t0; t <= t1; t += U) {
    const int wo = (t - t0) & 31;
    if (wo == 0) wval = t + lane <= tend ? __ldg(row + t + lane) : 0.f;
    int zi[U];
    float w0[U], w1[U];
    bool slow[U];
    bool any_slow = false;
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const float val = __shfl_sync(0xffffffffu, wval, wo + q);
      const float2 tb = (!kCheck || t + q <= t1) ? tab[t + q] : make_float2(-INFINITY, 0.f);
      const float d2 = xsub(xsub(tb.x, ddx), ddy);
      const bool valid = d2 > 0.f;
      const float depth = d2 * rsqrtf(d2);  // NaN when d2 <= 0: never taken
      const float zh = fmaf(depth + wzo, g.scale, -0.5f);
      const float fl = floorf(zh);
      const float fr = zh - fl;
      const bool fast = !g.exact && fabsf(fr - 0.5f) < 0.5f - pm;
      const int z = __float2int_rz(fl);
      const bool ok = valid && fast && (unsigned)(z - za) < (unsigned)zn;
      const float v = val * ((d2 * d2) * tb.y);
      zi[q] = ok ? z - za : 0;
      w0[q] = ok ? (1.f - fr) * v : 0.f;
      w1[q] = ok ? fr * v : 0.f;
      slow[q] = valid && !fast;
      any_slow |= slow[q];
    }
    if (__any_sync(0xffffffffu, any_slow)) {
#pragma unroll
      for (int q = 0; q < U; ++q) {
        if (!slow[q]) continue;
        const Sample sm = sample(g, wx, wy, wz, t + q, x, y);
        if (sm.ok && (unsigned)(sm.zi - za) < (unsigned)zn) {
          const float vv = __ldg(row + t + q) * sm.f2;
          zi[q] = sm.zi - za;
          w0[q] = (1.f - sm.alpha) * vv;
          w1[q] = sm.alpha * vv;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < U; ++q) {
      col[zi[q] * 32] += w0[q];
      col[zi[q] * 32 + 32] += w1[q];
    }
  }
}

// Exact adjoint of the forward with the lanes of a warp over 32 neighbouring
// voxel columns (an 8 x 4 tile: y fastest) and all lanes on one point and one
// bin at a time. The point's transient row is then read once per warp (32 bins
// per coalesced load, handed out by shuffles), and the bin's tc^2 (the sample
// chain's FP32 value) and 1 / tc^8 come from a per-CTA table in shared memory
// (broadcast reads), so f2 = (depth / tc^2)^4 = d2^2 / tc^8 needs no second
// special-function op. A CTA takes one slab of the columns' cells (the
// samples whose cell pair starts there; the pair's second cell may be the next
// slab's first, one extra row), and each lane owns its column's cells of the
// slab in shared memory ([cell][lane]: no bank conflicts, no atomics), one
// copy per warp; the warps of a CTA take interleaved runs of 32 points of one
// point group, and the CTA adds its summed columns into the volume (which the
// launcher zeroes) with one atomic per cell when there is more than one group
// or slab. A point's bins are those whose samples can land in the slab. Four bins per step,
// evaluated without branches, give each lane four independent sample chains
// (a branchy two-bin version issued 52 warp instructions per sample at 46% of
// issue slots, latency-bound with 12 warps per SM). The bins walked for a point
// are the union of the lanes' column spans: every valid sample of a lane lies
// in its own span, and a sample outside it is decided (and rejected) like any
// other, so each (column, point, bin) is counted once. Decisions are the exact
// chain's (sample_filtered's margin, taken over the largest |tc| of the union).
template <int U>
__global__ void __launch_bounds__(256) confocal_adjoint_columns_kernel(
    Geo g, Points mp, int N, int points_per_group, const float* __restrict__ tr,
    float* __restrict__ vol, int accumulate, int slab) {
  // slab blockIdx.z: the samples in cells [za, za + zn) (cell pairs (z, z + 1)
  // with z < Z - 1), held in rows 0 .. slab of the column copies (row slab is
  // cell za + slab, the next slab's first)
  const int za = blockIdx.z * slab, zb = min(g.Z, za + slab), zn = min(zb, g.Z - 1) - za;
  const int rows = slab + 1;
  extern __shared__ float acc[];  // [warp][rows][32], then the bin table
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  float2* tab = reinterpret_cast<float2*>(acc + (size_t)nw * rows * 32);  // [T]: tc^2, 1/tc^8
  const int tiles_y = (g.Y + 7) >> 3;
  const int ty = (blockIdx.x % tiles_y) * 8, tx = (blockIdx.x / tiles_y) * 4;
  const int yi = ty + (lane & 7), xi = tx + (lane >> 3);
  const bool live = xi < g.X && yi < g.Y;
  for (int j = threadIdx.x; j < nw * rows * 32; j += blockDim.x) acc[j] = 0.f;
  for (int t = threadIdx.x; t < g.T + kAdjTablePad; t += blockDim.x) {
    if (t >= g.T) {  // padding: no sample
      tab[t] = make_float2(-INFINITY, 0.f);
      continue;
    }
    const float tc = xadd(xmul((float)t, g.bw), g.bo);
    const float tc2 = xmul(tc, tc);
    const float i2 = __fdividef(1.f, tc2);
    tab[t] = make_float2(tc2, (i2 * i2) * (i2 * i2));
  }
  __syncthreads();
  float* col = acc + (size_t)warp * rows * 32 + lane;
  const float x = centre(g.ox, g.sx, g.X, live ? xi : 0);
  const float y = centre(g.oy, g.sy, g.Y, live ? yi : 0);
  const float u = 5.9604645e-8f;
  const int tz = first_nonneg_bin(g);
  const int i0 = blockIdx.y * points_per_group;
  const int i1 = min(N, i0 + points_per_group);
  for (int base = i0 + warp * 32; base < i1; base += nw * 32) {
    // lane j loads point base + j
    const int ip = base + lane;
    float lwx = 0.f, lwy = 0.f, lwz = 0.f;
    if (ip < i1) {
      lwx = mp.at(0, ip);
      lwy = mp.at(1, ip);
      lwz = mp.at(2, ip);
    }
    const int np = min(32, i1 - base);
    for (int j = 0; j < np; ++j) {
      const float wx = __shfl_sync(0xffffffffu, lwx, j);
      const float wy = __shfl_sync(0xffffffffu, lwy, j);
      const float wz = __shfl_sync(0xffffffffu, lwz, j);
      const float dx = xsub(wx, x), dy = xsub(wy, y);
      const float ddx = live ? xmul(dx, dx) : INFINITY, ddy = live ? xmul(dy, dy) : 0.f;
      Spans sp{1, 0, 1, 0};
      float cl, ch;
      if (live && zn > 0 &&
          tc_bounds(dx * dx + dy * dy, wz, g.oz + ((float)za + 0.5f) / g.scale,
                    g.oz + ((float)zb + 0.5f) / g.scale, cl, ch))
        sp = tc_spans(g, tz, cl, ch, span_eps(g, ch, wz));
      // warp union of the lanes' spans
      const int p0 = __reduce_min_sync(0xffffffffu, sp.p0 <= sp.p1 ? sp.p0 : INT_MAX);
      const int p1 = __reduce_max_sync(0xffffffffu, sp.p0 <= sp.p1 ? sp.p1 : -1);
      int n0 = INT_MAX, n1 = -1;
      if (tz > 0) {  // warp-uniform
        n0 = __reduce_min_sync(0xffffffffu, sp.n0 <= sp.n1 ? sp.n0 : INT_MAX);
        n1 = __reduce_max_sync(0xffffffffu, sp.n0 <= sp.n1 ? sp.n1 : -1);
      }
      if (p0 > p1 && n0 > n1) continue;  // warp-uniform
      const Spans un{p0, p1, n0, n1};
      // sample_filtered's margin over the union's largest |tc| (warp-uniform)
      const float dmax = 1.001f * span_tc_max(g, un);
      const float zmax = fabsf(wz) + dmax;
      const float zhmax = (zmax + fabsf(g.oz)) * g.scale + 0.5f;
      const float pm = 8.f * u * g.scale * (dmax + fabsf(wz) + zmax + fabsf(g.oz)) +
                       4.f * u * zhmax + 1e-7f;
      const float* row = tr + (size_t)(base + j) * g.T;
      const float wzo = wz - g.oz;
      adj_walk<false, U>(g, tab, row, col, p0, p1, lane, ddx, ddy, wz, wzo, pm, wx, wy, x, y,
                         za, zn);
      if (n0 <= n1)  // warp-uniform: negative bin centres (a negative bin offset)
        adj_walk<true, U>(g, tab, row, col, n0, n1, lane, ddx, ddy, wz, wzo, pm, wx, wy, x, y,
                          za, zn);
    }
  }
  __syncthreads();
  // cell za + r of column l: the sum over the warps' copies (l fastest: no
  // bank conflicts in the reads)
  for (int jj = threadIdx.x; jj < rows * 32; jj += blockDim.x) {
    const int r = jj >> 5, l = jj & 31, z = za + r;
    const int cy = ty + (l & 7), cx = tx + (l >> 3);
    if (cx >= g.X || cy >= g.Y || z >= g.Z) continue;
    float sum = 0.f;
    for (int w = 0; w < nw; ++w) sum += acc[((size_t)w * rows + r) * 32 + l];
    float* dst = vol + ((size_t)cx * g.Y + cy) * g.Z + z;
    if (accumulate) atomicAdd(dst, sum);
    else *dst = sum;
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
  g.inv_bw = 1.f / bw;
  g.T = T;
  g.exact = tune::get("volume.exact") == 1;
  g.all_bins = !(bw > 0.f) || !std::isfinite(bw) || !std::isfinite(bo) ||
               !std::isfinite(g.inv_bw);
  return g;
}

// the count (in a 256-byte header), then one record per voxel
size_t occupancy_bytes(int64_t nvox) { return align_up(256 + sizeof(float4) * nvox, 256); }

int compact(const Geo& g, const float* vol, int64_t n, void* ws, size_t ws_bytes, float4** recs,
            uint32_t** count, cudaStream_t stream) {
  const size_t need = occupancy_bytes(n);
  if (!ws || ws_bytes < need)
    return fail(TOTRI_ERR_WORKSPACE,
                "workspace of " + std::to_string(need) + " bytes required, got " +
                    std::to_string(ws_bytes));
  *count = static_cast<uint32_t*>(ws);
  *recs = reinterpret_cast<float4*>(static_cast<char*>(ws) + 256);
  TOTRI_CUDA(cudaMemsetAsync(*count, 0, sizeof(uint32_t), stream));
  TOTRI_KERNEL("volume compact", stream,
               volume::compact_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, stream>>>(
                   g, vol, n, *recs, *count));
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
  const Geo g = make_geo(X, Y, Z, origin, size, bw, bo, T);
  float4* recs;
  uint32_t* count;
  TOTRI_TRY(compact(g, static_cast<const float*>(vol->data), numel(vol), ws, ws_bytes, &recs,
                    &count, stream));
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(volume::confocal_forward_kernel), smem));
  TOTRI_KERNEL("volume confocal forward", stream,
               volume::confocal_forward_kernel<<<(unsigned)ceil_div(N, volume::kPT), 256, smem,
                                                 stream>>>(g, recs, count, pts, N,
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
  const unsigned grid = (unsigned)(X * Y);
  const float* trd = static_cast<const float*>(tr->data);
  float* vd = static_cast<float*>(vol->data);
  // "volume.adjoint.mode": 0 (default) lanes over columns, 1 shared-memory
  // atomics, 2 lane-owned cells (columns of up to 256 cells)
  const int mode = tune::get("volume.adjoint.mode");
  // lanes over columns: warps per CTA such that two CTAs' copies of 32
  // columns and the bin table fit an SM's shared memory
  // ("volume.adjoint.warps" overrides); bins beyond 4,096 take the atomic kernel
  const size_t table = sizeof(float2) * ((size_t)T + volume::kAdjTablePad);
  // The columns split into slabs of at most 64 cells, a CTA per slab: each
  // warp's column copy is then 65 rows (8.3 KB), and 3 CTAs of 8 warps share
  // an SM (24 warps) instead of 2 of 6 with whole 128-cell columns. 128^3
  // voxels x 16,384 points: 65.8 ms with 2 slabs, 75.4 ms with 1 and 72.5 ms
  // with 4 (each slab walks the union of its lanes' bins, so thinner slabs
  // walk more bins in all). "volume.adjoint.slabs" sets the count.
  int slabs = (int)tune::get("volume.adjoint.slabs");
  if (slabs <= 0) slabs = (int)ceil_div(Z, 64);
  slabs = std::min(slabs, Z);
  const int slab = (int)ceil_div(Z, slabs);
  const size_t per_warp = (size_t)(slab + 1) * 32 * sizeof(float);
  int warps = T <= 4096 && table < 113 * 1024 ? (int)((113 * 1024 - table) / per_warp) : 0;
  if (tune::get("volume.adjoint.warps") > 0) warps = tune::get("volume.adjoint.warps");
  warps = std::min(warps, 8);
  if (Z < 2) {  // no interpolation pair: no samples
    TOTRI_CUDA(cudaMemsetAsync(vd, 0, sizeof(float) * numel(vol), stream));
    return TOTRI_OK;
  }
  if (mode == 0 && warps >= 1 && T <= 4096) {
    const size_t smem = (size_t)warps * per_warp + table;
    const int64_t tiles = ceil_div(Y, 8) * ceil_div(X, 4);
    // point groups: about 16 CTAs per SM in all, each group at least four
    // runs of 32 points per warp
    const int nslab = (int)ceil_div(Z, slab);
    const int64_t want = std::max<int64_t>(1, (16 * tune::sm_count()) / (tiles * nslab));
    const int groups =
        (int)std::max<int64_t>(1, std::min<int64_t>(want, N / (128 * warps)));
    const int per = (int)(ceil_div(ceil_div(N, groups), 32) * 32);
    const int used = (int)ceil_div(N, per);
    const int accumulate = used > 1 || nslab > 1;
    if (accumulate) TOTRI_CUDA(cudaMemsetAsync(vd, 0, sizeof(float) * numel(vol), stream));
    const dim3 grid3((unsigned)tiles, (unsigned)used, (unsigned)nslab);
    TOTRI_CUDA(tune::ensure_dynamic_smem(
        reinterpret_cast<const void*>(volume::confocal_adjoint_columns_kernel<volume::kAdjUnroll>),
        smem));
    TOTRI_KERNEL("volume confocal adjoint", stream,
                 volume::confocal_adjoint_columns_kernel<volume::kAdjUnroll>
                 <<<grid3, warps * 32, smem, stream>>>(g, pts, N, per, trd, vd, accumulate, slab));
    return TOTRI_OK;
  }
  if (Z <= 256 && mode == 2) {
    if (Z <= 32)
      TOTRI_KERNEL("volume confocal adjoint", stream,
                   volume::confocal_adjoint_cells_kernel<1><<<grid, 256, 0, stream>>>(
                       g, pts, N, trd, vd));
    else if (Z <= 64)
      TOTRI_KERNEL("volume confocal adjoint", stream,
                   volume::confocal_adjoint_cells_kernel<2><<<grid, 256, 0, stream>>>(
                       g, pts, N, trd, vd));
    else if (Z <= 128)
      TOTRI_KERNEL("volume confocal adjoint", stream,
                   volume::confocal_adjoint_cells_kernel<4><<<grid, 256, 0, stream>>>(
                       g, pts, N, trd, vd));
    else
      TOTRI_KERNEL("volume confocal adjoint", stream,
                   volume::confocal_adjoint_cells_kernel<8><<<grid, 256, 0, stream>>>(
                       g, pts, N, trd, vd));
    return TOTRI_OK;
  }
  const size_t smem = sizeof(float) * 8 * (size_t)Z;
  if (smem > 200 * 1024) return fail(TOTRI_ERR_UNSUPPORTED, "volume too deep for one column tile");
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(volume::confocal_adjoint_kernel), smem));
  TOTRI_KERNEL("volume confocal adjoint", stream,
               volume::confocal_adjoint_kernel<<<grid, 256, smem, stream>>>(g, pts, N, trd, vd));
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
  const Geo g = make_geo(X, Y, Z, origin, size, bw, bo, T);
  float4* recs;
  uint32_t* count;
  TOTRI_TRY(compact(g, static_cast<const float*>(vol->data), numel(vol), ws, ws_bytes, &recs,
                    &count, stream));
  TOTRI_KERNEL("volume confocal grad points", stream,
               volume::grad_mp_kernel<<<(unsigned)ceil_div(N, volume::kPT), 256, 0, stream>>>(
                   g, recs, count, pts, N,
                   static_cast<const float*>(tg->data), static_cast<float*>(mpg->data),
                   mpg->strides[0], mpg->strides[1]));
  return TOTRI_OK;
}

}  // extern "C"
