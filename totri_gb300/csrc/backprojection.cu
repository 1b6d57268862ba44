// Backprojection reconstructions: Velten confocal (and its adjoint), Velten
// exhaustive, Arellano exhaustive.
//
// Reference: src/reconstruct/backprojection_cuda.cu (:153-194 Velten
// confocal, :229-287 Velten exhaustive, :11-115 Arellano). The Velten kernels
// gather per voxel; here a CTA of 256 voxels stages scan points (and their
// wall-to-origin distances) in shared memory in tiles, so each scan point is
// read once per CTA rather than once per voxel. The adjoint owns a tile of
// scan points and keeps their transient columns in shared memory.
#include <cmath>
#include <string>

#include <climits>

#include "capi_common.cuh"
#include "tune.cuh"

namespace totri {
namespace bp {

struct Grid {
  int D, H, W;
  float sx, sy, sz, ex, ey, ez;
};

// start + (i / (n - 1)) * (end - start) (backprojection_cuda.cu:167-170).
__device__ __forceinline__ float grid_coord(float s, float e, int n, int i) {
  return xadd(s, xmul(xdiv((float)i, (float)(n - 1)), xsub(e, s)));
}

__device__ __forceinline__ fv3 voxel_point(const Grid& g, int x, int y, int z) {
  return mkv(grid_coord(g.sx, g.ex, g.W, x), grid_coord(g.sy, g.ey, g.H, y),
             grid_coord(g.sz, g.ez, g.D, z));
}

// floor((dist - offset) / width + 0.5) (backprojection_cuda.cu:187).
__device__ __forceinline__ int nearest_bin(float dist, float bw, float bo) {
  const float b = floorf(xadd(xdiv(xsub(dist, bo), bw), 0.5f));
  if (!(b == b)) return -1;
  if (b > 2.0e9f) return 2000000000;
  if (b < -2.0e9f) return -2000000000;
  return (int)b;
}

// Velten bins with a filtered fast path. The decision is nearest_bin(od2 + 2
// |q - p|) with one IEEE rounding per operation. The fast path evaluates the
// same expression with fused multiply-adds, the hardware reciprocal square
// root (2 ulp) and a precomputed 1/bw; against the exact chain its bin
// coordinate c = (dist - bo)/bw + 1/2 deviates by at most about
// 14 u (dist + |bo|)/bw + 5 u |c| (u = 2^-24: 3 u from the sum of squares,
// 6.5 u from the root, one rounding per remaining operation). Where c lies
// farther than twice that from an integer both floors are equal and the fast
// bin is returned; otherwise (and for NaN or infinite c) the exact chain runs,
// so the bins are those of the exact chain everywhere.
struct FastBin {
  float inv_bw, nbo, k1, k2;
};

inline FastBin make_fast_bin(float bw, float bo) {
  const float u = 5.9604645e-8f;  // 2^-24
  FastBin f;
  f.inv_bw = 1.f / bw;
  f.nbo = -bo * f.inv_bw;
  const bool ok = bw > 0.f && std::isfinite(f.inv_bw) && std::isfinite(f.nbo);
  f.k1 = ok ? 32.f * u * f.inv_bw : INFINITY;
  f.k2 = ok ? 32.f * u * std::fabs(bo) * f.inv_bw + 1e-6f : INFINITY;
  return f;
}

__device__ __forceinline__ int velten_bin(fv3 q, float od2, fv3 p, float bw, float bo,
                                          const FastBin& f) {
  const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
  const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float dist = fmaf(2.f, d2 * rsqrtf(d2), od2);
  const float c = fmaf(dist, f.inv_bw, f.nbo) + 0.5f;
  const float t = floorf(c);
  const float fr = c - t;
  const float m = fmaf(f.k1, dist, f.k2) + 1e-6f * fabsf(c);
  if (fr > m && fr < 1.f - m && fabsf(t) < 1.0e9f) return (int)t;
  return nearest_bin(xadd(od2, xmul(2.f, xlen(xsub3(q, p)))), bw, bo);
}

__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// velten_bin for the voxels of a column, with the margin m bounded once per
// tile (the tiled kernel derives it from the distance and bin bounds of its
// voxel block, 2% above velten_bin's per-pair margin there) and the +1/2 of
// the bin coordinate folded away. r2, the squared distance in x and y, is
// shared by the column's voxels (one fused multiply-add per voxel adds dz^2;
// the sum of squares keeps three roundings). The bin is rounded without the
// conversion units: v = dist / bw - bo / bw plus 1.5 2^23 holds rint(v) in
// its low mantissa bits for |v| < 2^22, and floor(v + 1/2) = rint(v) wherever
// v + 1/2 is farther than the margin from an integer, which is the test
// |v - rint(v)| < 1/2 - m (`half_m`; <= 0 sends every pair of a tile to the
// exact chain). The bins are those of the exact chain everywhere.
__device__ __forceinline__ int velten_bin_col(fv3 q, float od2, fv3 p, float r2, float bw,
                                              float bo, float inv_bw, float nbo, float half_m) {
  const float dz = q.z - p.z;
  const float d2 = fmaf(dz, dz, r2);
  const float dist = fmaf(2.f, d2 * rsqrt_approx(d2), od2);
  const float v = fmaf(dist, inv_bw, nbo);
  const float x = v + 12582912.f;  // 1.5 2^23
  const float rr = v - (x - 12582912.f);
  if (fabsf(rr) < half_m) return __float_as_int(x) - 0x4B400000;
  return nearest_bin(xadd(od2, xmul(2.f, xlen(xsub3(q, p)))), bw, bo);
}

// velten_bin_col for two voxels of the column at once: the same operations
// on (voxel a, voxel b) pairs with paired FP32 instructions (each rounds as
// its scalar form), the reciprocal square roots and the decisions per voxel.
__device__ __forceinline__ void velten_bin_col2(fv3 q, float od2, fv3 pa, fv3 pb, float r2,
                                                float bw, float bo, float inv_bw, float nbo,
                                                float half_m, int& ta, int& tb) {
  const unsigned long long dz = f2sub(f2pack(q.z, q.z), f2pack(pa.z, pb.z));
  const unsigned long long d2 = f2fma(dz, dz, f2pack(r2, r2));
  float d2a, d2b;
  f2unpack(d2, d2a, d2b);
  const unsigned long long prod = f2mul(d2, f2pack(rsqrt_approx(d2a), rsqrt_approx(d2b)));
  const unsigned long long dist = f2fma(f2pack(2.f, 2.f), prod, f2pack(od2, od2));
  const unsigned long long v = f2fma(dist, f2pack(inv_bw, inv_bw), f2pack(nbo, nbo));
  const unsigned long long big = f2pack(12582912.f, 12582912.f);  // 1.5 2^23
  const unsigned long long x = f2add(v, big);
  const unsigned long long rr = f2sub(v, f2sub(x, big));
  float xa, xb, ra, rb;
  f2unpack(x, xa, xb);
  f2unpack(rr, ra, rb);
  ta = fabsf(ra) < half_m ? __float_as_int(xa) - 0x4B400000
                          : nearest_bin(xadd(od2, xmul(2.f, xlen(xsub3(q, pa)))), bw, bo);
  tb = fabsf(rb) < half_m ? __float_as_int(xb) - 0x4B400000
                          : nearest_bin(xadd(od2, xmul(2.f, xlen(xsub3(q, pb)))), bw, bo);
}

struct Pts3 {  // [B, n, 3] with strides
  const float* p;
  int64_t sb, sn, sc;
  __device__ fv3 at(int b, int i) const {
    const float* q = p + b * sb + i * sn;
    return mkv(q[0], q[sc], q[2 * sc]);
  }
};

constexpr int kTile = 512;

__global__ void __launch_bounds__(256) velten_confocal_kernel(Grid g, int b, int T, int S,
                                                              Pts3 sp, Pts3 so, int has_origin,
                                                              float bw, float bo, FastBin fb,
                                                              const float* __restrict__ tr,
                                                              float* __restrict__ vol) {
  __shared__ float4 pts[kTile];  // scan point xyz, 2 * |scan - origin|
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int x = (int)(v % g.W), y = (int)((v / g.W) % g.H), z = (int)(v / ((int64_t)g.W * g.H));
  const fv3 p = voxel_point(g, x, y, z);
  const float* trb = tr + (size_t)b * T * S;
  float value = 0.f;
  for (int s0 = 0; s0 < S; s0 += kTile) {
    __syncthreads();
    for (int j = threadIdx.x; j < kTile && s0 + j < S; j += blockDim.x) {
      const fv3 q = sp.at(b, s0 + j);
      const float od = has_origin ? xlen(xsub3(q, so.at(b, s0 + j))) : 0.f;
      pts[j] = make_float4(q.x, q.y, q.z, xmul(2.f, od));
    }
    __syncthreads();
    if (v < nv) {
      const int cnt = min(kTile, S - s0);
      for (int j = 0; j < cnt; ++j) {
        const float4 q = pts[j];
        const int t = velten_bin(mkv(q.x, q.y, q.z), q.w, p, bw, bo, fb);
        if (t >= 0 && t < T) value += __ldg(trb + (size_t)t * S + s0 + j);
      }
    }
  }
  if (v < nv) vol[(size_t)b * nv + v] = value;
}

// Tiled Velten confocal: one CTA of 256 threads per 8x8x(4 VZ) block of
// voxels, each thread VZ voxels 4 apart in z (default VZ = 4: 42.7 ms against
// 51.1 ms for one voxel per thread and 46.3 ms for 8 on 128^3 voxels x 16,384
// points, as the staged window and each scan point's shared-memory load serve
// more voxels), scan points in tiles of 32. Per tile, warp 0 bounds the bins
// the block can reach from each point (distance from the point to the block's
// box, one bin of margin each side) and the CTA stages the union of those
// rows of the tile's 32 transient columns in shared memory with coalesced
// 128-byte row reads (row stride 33, so lanes reading different bins of one
// column hit different banks). Voxels then read their bin from shared memory;
// a bin outside the staged rows is read from global memory, so the window
// only affects speed. The sum runs over the scan points in the same order as
// velten_confocal_kernel, so the two give identical volumes.
//
// A tile whose union exceeds kWinRows (fine bins: the union of 32 points
// spans 2-4x the rows of 8 consecutive points) stages per group of
// consecutive points instead: 4 groups of 8, whose 8 columns of a row are one
// full 32-byte sector, when every group's union fits its part of the window;
// else 8 groups of 4; else one window per point, cut to its first rows. With
// one union per tile, 4,096 bins of 1.25 mm over 128^3 voxels from 128x128
// points took 4.6x the time of 1,024 bins. The group windows are compiled
// in only with kGrouped: their code alone, never taken, made the kernel 10%
// slower at 1,024 bins (38.3 -> 42.8 ms), so the host launches them when a
// point's bins over the voxel block alone span more than about 100 rows.
constexpr int kBX = 8, kBY = 8, kBZ = 4, kST = 32, kWinRows = 256;
constexpr int kWinFloats = kWinRows * (kST + 1);

// rows of a bin span [lo, hi]; an empty span (lo = INT_MAX, hi = INT_MIN)
// has none, and its difference is never formed (it overflows)
__device__ __forceinline__ int span_rows(int lo, int hi) { return hi >= lo ? hi - lo + 1 : 0; }

// Group windows: group g of COLS points holds rows [grp[g].x, grp[g].x +
// grp[g].y) of its columns at win + g REGION, row stride STRIDE (COLS + 1,
// odd, for COLS > 1). REGION = COLS mod 32, so one row of all groups, as
// staged, lands on 32 distinct banks; 4 x 2088, 8 x 1028 and 32 x 257 floats
// fit kWinFloats.
template <int COLS, int STRIDE, int REGION>
__device__ __forceinline__ void velten_group_stage(float* win, const int2* grp, int cnt, int rows_max,
                                                   const float* __restrict__ trb, int S, int s0) {
  const int k = threadIdx.x & 31;  // a warp stages one row of every group
  const int2 d = grp[k / COLS];
  const int rows = k < cnt ? d.y : 0;
  float* dst = win + (k / COLS) * REGION + k % COLS;
  for (int r = threadIdx.x >> 5; r < rows_max; r += blockDim.x >> 5)
    if (r < rows) dst[r * STRIDE] = __ldg(trb + (size_t)(d.x + r) * S + s0 + k);
}

// The samples of a tile with group windows. Points j >= cnt of a partial
// tile carry a NaN distance, whose bin (-1) is neither staged nor in [0, T):
// they add nothing.
template <int COLS, int STRIDE, int REGION, int VZ, bool kPair>
__device__ __forceinline__ void velten_group_samples(const float* win, const float4* pts,
                                                     const int2* grp, const fv3 (&p)[VZ],
                                                     float (&value)[VZ], int cnt, int T, int S,
                                                     int s0, float bw, float bo, float inv_bw,
                                                     float nbo, float half_m,
                                                     const float* __restrict__ trb) {
  for (int j0 = 0; j0 < cnt; j0 += COLS) {
    const int2 d = grp[j0 / COLS];
    const float* wg = win + (j0 / COLS) * REGION;
#pragma unroll 1
    for (int c = 0; c < COLS; ++c) {
      const float4 q = pts[j0 + c];
      const float dx = q.x - p[0].x, dy = q.y - p[0].y;
      const float r2 = fmaf(dx, dx, dy * dy);
      auto add = [&](int v, int t) {
        const unsigned r = (unsigned)t - (unsigned)d.x;
        if (r < (unsigned)d.y) value[v] += wg[r * STRIDE + c];
        else if ((unsigned)t < (unsigned)T)
          value[v] += __ldg(trb + (size_t)t * S + s0 + j0 + c);
      };
      if constexpr (kPair) {
#pragma unroll
        for (int v = 0; v < VZ; v += 2) {
          int ta, tb;
          velten_bin_col2(mkv(q.x, q.y, q.z), q.w, p[v], p[v + 1], r2, bw, bo, inv_bw, nbo,
                          half_m, ta, tb);
          add(v, ta);
          add(v + 1, tb);
        }
      } else {
#pragma unroll
        for (int v = 0; v < VZ; ++v)
          add(v, velten_bin_col(mkv(q.x, q.y, q.z), q.w, p[v], r2, bw, bo, inv_bw, nbo, half_m));
      }
    }
  }
}

template <int VZ, int kOcc = 1, bool kGrouped = false, bool kPair = false>
__global__ void __launch_bounds__(256, kOcc) velten_confocal_tiled_kernel(
    Grid g, int b, int T, int S, Pts3 sp, Pts3 so, int has_origin, float bw, float bo,
    FastBin fb, const float* __restrict__ tr, float* __restrict__ vol) {
  __shared__ float win[kWinFloats];
  __shared__ float4 pts[kST];
  __shared__ int2 grp[kST];  // group windows: first staged bin, staged rows
  __shared__ int span[2];
  __shared__ int tile_cols;  // 32: one window; 8, 4, 1: points per group window
  __shared__ int tile_rows;  // group windows: the most rows any group stages
  __shared__ float tile_margin;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x0 = blockIdx.x * kBX, y0 = blockIdx.y * kBY, z0 = blockIdx.z * kBZ * VZ;
  const int x = x0 + (threadIdx.x & 7), y = y0 + ((threadIdx.x >> 3) & 7);
  // voxels z0 + (threadIdx.x >> 6) + kBZ v, v < VZ: one bin window and one
  // scan-point load serve VZ voxels
  bool inside[VZ];
  fv3 p[VZ];
#pragma unroll
  for (int v = 0; v < VZ; ++v) {
    const int z = z0 + (threadIdx.x >> 6) + kBZ * v;
    inside[v] = x < g.W && y < g.H && z < g.D;
    p[v] = voxel_point(g, min(x, g.W - 1), min(y, g.H - 1), min(z, g.D - 1));
  }
  // the block's box: voxel coordinates are monotone in the index
  const fv3 ca = voxel_point(g, x0, y0, z0);
  const fv3 cb = voxel_point(g, min(x0 + kBX, g.W) - 1, min(y0 + kBY, g.H) - 1,
                             min(z0 + kBZ * VZ, g.D) - 1);
  const fv3 lo = mkv(fminf(ca.x, cb.x), fminf(ca.y, cb.y), fminf(ca.z, cb.z));
  const fv3 hi = mkv(fmaxf(ca.x, cb.x), fmaxf(ca.y, cb.y), fmaxf(ca.z, cb.z));
  const float* trb = tr + (size_t)b * T * S;
  float value[VZ];
#pragma unroll
  for (int v = 0; v < VZ; ++v) value[v] = 0.f;
  for (int s0 = 0; s0 < S; s0 += kST) {
    const int cnt = min(kST, S - s0);
    __syncthreads();  // the previous tile is consumed
    if (warp == 0) {
      int tlo = INT_MAX, thi = INT_MIN;
      float mrg = 0.f;  // margin bound of this lane's pairs (infinite: exact chain)
      float4 pt = make_float4(0.f, 0.f, 0.f, __int_as_float(0x7fc00000));  // NaN distance
      if (lane < cnt) {
        const fv3 q = sp.at(b, s0 + lane);
        const float od2 = xmul(2.f, has_origin ? xlen(xsub3(q, so.at(b, s0 + lane))) : 0.f);
        pt = make_float4(q.x, q.y, q.z, od2);
        const float ex = fmaxf(fmaxf(lo.x - q.x, q.x - hi.x), 0.f);
        const float ey = fmaxf(fmaxf(lo.y - q.y, q.y - hi.y), 0.f);
        const float ez = fmaxf(fmaxf(lo.z - q.z, q.z - hi.z), 0.f);
        const float fx = fmaxf(fabsf(lo.x - q.x), fabsf(hi.x - q.x));
        const float fy = fmaxf(fabsf(lo.y - q.y), fabsf(hi.y - q.y));
        const float fz = fmaxf(fabsf(lo.z - q.z), fabsf(hi.z - q.z));
        const float cmin = (od2 + 2.f * sqrtf(ex * ex + ey * ey + ez * ez) - bo) / bw + 0.5f;
        const float cmax = (od2 + 2.f * sqrtf(fx * fx + fy * fy + fz * fz) - bo) / bw + 0.5f;
        if (cmin == cmin && cmax == cmax && cmax >= -1.f && cmin <= (float)T + 1.f) {
          tlo = max((int)floorf(fmaxf(cmin, -2.f)) - 1, 0);
          thi = min((int)floorf(fminf(cmax, (float)T + 2.f)) + 1, T - 1);
        }
        // velten_bin's margin k1 dist + k2 + 1e-6 |c| at the largest distance
        // and |c| of the block (2% slack for the rounding of these bounds)
        const float dmax = fmaf(cmax - 0.5f, bw, bo);
        const float cabs = fmaxf(fabsf(cmin), fabsf(cmax));
        mrg = 1.02f * (fmaf(fb.k1, fabsf(dmax), fb.k2) + 1e-6f * cabs);
        if (!(mrg == mrg) || !(cabs < 2097152.f)) mrg = INFINITY;  // 2^21: rint range
      }
      if (kGrouped || lane < cnt) pts[lane] = pt;
      const int lo1 = tlo, hi1 = thi;
      int lo4 = 0, hi4 = 0, lo8 = 0, hi8 = 0;
      if constexpr (kGrouped) {
        // unions of aligned groups of 4, 8 and 32 lanes (each within [0, T) or empty)
        for (int o = 1; o < 32; o <<= 1) {
          tlo = min(tlo, __shfl_xor_sync(0xffffffffu, tlo, o));
          thi = max(thi, __shfl_xor_sync(0xffffffffu, thi, o));
          mrg = fmaxf(mrg, __shfl_xor_sync(0xffffffffu, mrg, o));
          if (o == 2) lo4 = tlo, hi4 = thi;
          if (o == 4) lo8 = tlo, hi8 = thi;
        }
      } else {
        for (int o = 16; o > 0; o >>= 1) {
          tlo = min(tlo, __shfl_xor_sync(0xffffffffu, tlo, o));
          thi = max(thi, __shfl_xor_sync(0xffffffffu, thi, o));
          mrg = fmaxf(mrg, __shfl_xor_sync(0xffffffffu, mrg, o));
        }
      }
      constexpr int kR8 = 232, kR4 = 205, kR1 = 257;  // rows of 2088 / 9, 1028 / 5, 257
      int cols = 32, grows = 0;
      if (kGrouped && span_rows(tlo, thi) > kWinRows) {
        int glo;
        if (__all_sync(0xffffffffu, span_rows(lo8, hi8) <= kR8))
          cols = 8, glo = lo8, grows = span_rows(lo8, hi8);
        else if (__all_sync(0xffffffffu, span_rows(lo4, hi4) <= kR4))
          cols = 4, glo = lo4, grows = span_rows(lo4, hi4);
        else
          cols = 1, glo = lo1, grows = min(span_rows(lo1, hi1), kR1);
        if ((lane & (cols - 1)) == 0) grp[lane / cols] = make_int2(glo, grows);
        for (int o = 16; o > 0; o >>= 1) grows = max(grows, __shfl_xor_sync(0xffffffffu, grows, o));
      }
      if (lane == 0) {
        span[0] = tlo;
        span[1] = thi;
        tile_cols = cols;
        tile_rows = grows;
        tile_margin = mrg;
      }
    }
    __syncthreads();
    // one unsigned compare accepts a staged row (the windows lie in [0, T));
    // anything else is read from global memory if it is a bin at all. Voxels
    // past the volume's edge compute on a clamped position and are never
    // written.
    const int cols = tile_cols;
    if (!kGrouped || cols == 32) {
      // (with kGrouped a tile takes this path only when its union fits)
      const int tlo = span[0], thi = span[1];
      const int rows = (tlo >= 0 && thi < T && thi >= tlo) ? thi - tlo + 1 : 0;
      const bool staged = rows > 0 && rows <= kWinRows;
      if (staged)
        for (int i = threadIdx.x; i < rows * kST; i += blockDim.x) {
          const int r = i >> 5, c = i & 31;
          win[r * (kST + 1) + c] = c < cnt ? __ldg(trb + (size_t)(tlo + r) * S + s0 + c) : 0.f;
        }
      __syncthreads();
      const unsigned srows = staged ? (unsigned)rows : 0u;
      const float half_m = 0.5f - tile_margin;
      for (int j = 0; j < cnt; ++j) {
        const float4 q = pts[j];
        const float dx = q.x - p[0].x, dy = q.y - p[0].y;
        const float r2 = fmaf(dx, dx, dy * dy);
        if constexpr (kPair) {
#pragma unroll
          for (int v = 0; v < VZ; v += 2) {
            int t[2];
            velten_bin_col2(mkv(q.x, q.y, q.z), q.w, p[v], p[v + 1], r2, bw, bo, fb.inv_bw,
                            fb.nbo, half_m, t[0], t[1]);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const unsigned r = (unsigned)t[h] - (unsigned)tlo;
              if (r < srows) value[v + h] += win[r * (kST + 1) + j];
              else if ((unsigned)t[h] < (unsigned)T)
                value[v + h] += __ldg(trb + (size_t)t[h] * S + s0 + j);
            }
          }
        } else {
#pragma unroll
          for (int v = 0; v < VZ; ++v) {
            const int t = velten_bin_col(mkv(q.x, q.y, q.z), q.w, p[v], r2, bw, bo, fb.inv_bw,
                                         fb.nbo, half_m);
            const unsigned r = (unsigned)t - (unsigned)tlo;
            if (r < srows) value[v] += win[r * (kST + 1) + j];
            else if ((unsigned)t < (unsigned)T) value[v] += __ldg(trb + (size_t)t * S + s0 + j);
          }
        }
      }
    } else if (cols == 8) {
      velten_group_stage<8, 9, 2088>(win, grp, cnt, tile_rows, trb, S, s0);
      __syncthreads();
      const float half_m = 0.5f - tile_margin;
      velten_group_samples<8, 9, 2088, VZ, kPair>(win, pts, grp, p, value, cnt, T, S, s0, bw, bo, fb.inv_bw,
                                       fb.nbo, half_m, trb);
    } else if (cols == 4) {
      velten_group_stage<4, 5, 1028>(win, grp, cnt, tile_rows, trb, S, s0);
      __syncthreads();
      const float half_m = 0.5f - tile_margin;
      velten_group_samples<4, 5, 1028, VZ, kPair>(win, pts, grp, p, value, cnt, T, S, s0, bw, bo, fb.inv_bw,
                                       fb.nbo, half_m, trb);
    } else {
      velten_group_stage<1, 1, 257>(win, grp, cnt, tile_rows, trb, S, s0);
      __syncthreads();
      const float half_m = 0.5f - tile_margin;
      velten_group_samples<1, 1, 257, VZ, kPair>(win, pts, grp, p, value, cnt, T, S, s0, bw, bo, fb.inv_bw,
                                      fb.nbo, half_m, trb);
    }
  }
#pragma unroll
  for (int v = 0; v < VZ; ++v) {
    const int z = z0 + (threadIdx.x >> 6) + kBZ * v;
    if (inside[v]) vol[(size_t)b * g.D * g.H * g.W + ((size_t)z * g.H + y) * g.W + x] = value[v];
  }
}

// Adjoint: transient [T, S] tile of TS scan points in shared memory, all voxels.
constexpr int kTS = 8;
__global__ void __launch_bounds__(256) velten_adjoint_kernel(Grid g, int b, int T, int S, Pts3 sp,
                                                             Pts3 so, int has_origin, float bw,
                                                             float bo, FastBin fb,
                                                             const float* __restrict__ vol,
                                                             float* __restrict__ tr) {
  extern __shared__ float hist[];  // [T][kTS]
  const int s0 = blockIdx.x * kTS;
  for (int j = threadIdx.x; j < T * kTS; j += blockDim.x) hist[j] = 0.f;
  __syncthreads();
  const int sl = threadIdx.x % kTS;
  const int s = s0 + sl;
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  if (s < S) {
    const fv3 q = sp.at(b, s);
    const float od2 = xmul(2.f, has_origin ? xlen(xsub3(q, so.at(b, s))) : 0.f);
    const float* vb = vol + (size_t)b * nv;
    for (int64_t v = threadIdx.x / kTS; v < nv; v += blockDim.x / kTS) {
      const float val = __ldg(vb + v);
      if (val == 0.f) continue;
      const int x = (int)(v % g.W), y = (int)((v / g.W) % g.H), z = (int)(v / ((int64_t)g.W * g.H));
      const int t = velten_bin(q, od2, voxel_point(g, x, y, z), bw, bo, fb);
      if (t >= 0 && t < T) atomicAdd(hist + t * kTS + sl, val);
    }
  }
  __syncthreads();
  float* out = tr + (size_t)b * T * S;
  for (int j = threadIdx.x; j < T * kTS; j += blockDim.x) {
    const int t = j / kTS, c = j - t * kTS;
    if (s0 + c < S) out[(size_t)t * S + s0 + c] = hist[j];
  }
}

__global__ void __launch_bounds__(128) velten_exhaustive_kernel(Grid g, int b, int T, int S, int L,
                                                                Pts3 sp, Pts3 lp, Pts3 so, Pts3 lo,
                                                                int has_so, int has_lo, float bw,
                                                                float bo,
                                                                const float* __restrict__ tr,
                                                                float* __restrict__ vol) {
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int x = (int)(v % g.W), y = (int)((v / g.W) % g.H), z = (int)(v / ((int64_t)g.W * g.H));
  const fv3 p = voxel_point(g, x, y, z);
  const float* trb = tr + (size_t)b * T * S * L;
  float value = 0.f;
  for (int s = 0; s < S; ++s) {
    const fv3 q = sp.at(b, s);
    const float sv = xlen(xsub3(q, p));
    const float sod = has_so ? xlen(xsub3(q, so.at(b, s))) : 0.f;
    const float a = xadd(sod, sv);
    for (int l = 0; l < L; ++l) {
      const fv3 r = lp.at(b, l);
      const float lv = xlen(xsub3(r, p));
      const float lod = has_lo ? xlen(xsub3(r, lo.at(b, l))) : 0.f;
      const int t = nearest_bin(xadd(xadd(a, lv), lod), bw, bo);
      if (t >= 0 && t < T) value += __ldg(trb + ((size_t)t * S + s) * L + l);
    }
  }
  vol[(size_t)b * nv + v] = value;
}

struct Pts3T {  // [B, 3, n] with strides
  const float* p;
  int64_t sb, sc, sn;
  __device__ fv3 at(int b, int i) const {
    const float* q = p + b * sb + i * sn;
    return mkv(q[0], q[sc], q[2 * sc]);
  }
};

// Arellano (backprojection_cuda.cu:11-115): per (column, scan, laser), scale
// the ellipsoid of constant path length to a sphere along the scan-laser axis
// and deposit each positive bin where the column's ray meets it. int()
// truncation makes the reference's interpolation weight always 0 (nearest).
__global__ void __launch_bounds__(64) arellano_kernel(Grid g, int b, int T, int S, int L, Pts3T sp,
                                                      Pts3T lp, Pts3T so, Pts3T lo, int has_so,
                                                      int has_lo, float bw, float bo,
                                                      const float* __restrict__ tr,
                                                      float* __restrict__ vol) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y, l = blockIdx.z;
  if (c >= g.H * g.W) return;
  const int xi = c % g.W, yi = c / g.W;
  const float xf = xadd(g.sx, xmul(xdiv((float)xi, (float)(g.W - 1)), xsub(g.ex, g.sx)));
  const float yf = xadd(g.sy, xmul(xdiv((float)yi, (float)(g.H - 1)), xsub(g.ey, g.sy)));
  const fv3 sc = sp.at(b, s), lc = lp.at(b, l);
  const float sd = has_so ? xlen(xsub3(sc, so.at(b, s))) : 0.f;
  const float ld = has_lo ? xlen(xsub3(lc, lo.at(b, l))) : 0.f;
  const fv3 center = mkv(xmul(0.5f, xadd(sc.x, lc.x)), xmul(0.5f, xadd(sc.y, lc.y)),
                         xmul(0.5f, xadd(sc.z, lc.z)));
  fv3 nrm = xsub3(sc, lc);
  const float length = xlen(nrm);
  if (length > 1e-6f) {
    const float inv = xdiv(1.f, length);
    nrm = mkv(xmul(inv, nrm.x), xmul(inv, nrm.y), xmul(inv, nrm.z));
  }
  const fv3 rs = xsub3(mkv(xf, yf, g.sz), center);
  const fv3 re = xsub3(mkv(xf, yf, g.ez), center);
  const float* col = tr + (((size_t)b * T) * S + s) * L + l;
  const size_t st = (size_t)S * L;
  float* vb = vol + (size_t)b * g.D * g.H * g.W + c;
  const size_t vs = (size_t)g.H * g.W;
  for (int t = 0; t < T; ++t) {
    const float value = __ldg(col + t * st);
    if (!(value > 0.f)) continue;
    const float tc = xsub(xsub(xadd(xmul((float)t, bw), bo), sd), ld);
    if (!(tc > length)) continue;
    const float r0 = xdiv(tc, 2.f);
    const float r1 = xsqrt(xsub(xmul(r0, r0), xdiv(xmul(length, length), 4.f)));
    const float scale = xdiv(r1, r0);
    const float ks = xmul(xsub(scale, 1.f), xdot(rs, nrm));
    const float ke = xmul(xsub(scale, 1.f), xdot(re, nrm));
    const fv3 st0 = mkv(xfma(ks, nrm.x, rs.x), xfma(ks, nrm.y, rs.y), xfma(ks, nrm.z, rs.z));
    const fv3 et = mkv(xfma(ke, nrm.x, re.x), xfma(ke, nrm.y, re.y), xfma(ke, nrm.z, re.z));
    fv3 dir = xsub3(et, st0);
    const float rl = xlen(dir);
    const float ir = xdiv(1.f, rl);
    dir = mkv(xmul(ir, dir.x), xmul(ir, dir.y), xmul(ir, dir.z));
    const float v0 = xdot(dir, st0);
    float v1 = xsub(xmul(v0, v0), xsub(xdot(st0, st0), xmul(r1, r1)));
    if (!(v1 > 0.f)) continue;
    v1 = xsqrt(v1);
    float d = xsub(-v0, v1);
    if (d < 0.f) d = xadd(-v0, v1);
    const float bf = xadd(xmul(xdiv(d, rl), (float)g.D), 0.5f);
    if (!(bf > -1.f && bf < (float)g.D)) continue;
    atomicAdd(vb + (size_t)(int)bf * vs, value);
  }
}

}  // namespace bp

namespace {

int check_volume_out(const totri_array_t* vol, bp::Grid& g, const float* start, const float* end,
                     int64_t& B) {
  TOTRI_TRY(check_array(vol, "volume", 4, -1));
  if (vol->dtype != TOTRI_FLOAT32)
    return fail(TOTRI_ERR_UNSUPPORTED, "backprojection: only float32 tensors are supported");
  TOTRI_TRY(check_contiguous(vol, "volume"));
  B = vol->shape[0];
  g = bp::Grid{(int)vol->shape[1], (int)vol->shape[2], (int)vol->shape[3], start[0], start[1],
               start[2], end[0], end[1], end[2]};
  return TOTRI_OK;
}

int check_pts3(const totri_array_t* a, const char* name, int64_t B, int64_t& n, bp::Pts3& p) {
  TOTRI_TRY(check_array(a, name, 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(a, name, 0, B));
  TOTRI_TRY(check_dim(a, name, 2, 3));
  n = a->shape[1];
  p = bp::Pts3{static_cast<const float*>(a->data), a->strides[0], a->strides[1], a->strides[2]};
  return TOTRI_OK;
}

int check_pts3t(const totri_array_t* a, const char* name, int64_t B, int64_t& n, bp::Pts3T& p) {
  TOTRI_TRY(check_array(a, name, 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(a, name, 0, B));
  TOTRI_TRY(check_dim(a, name, 1, 3));
  n = a->shape[2];
  p = bp::Pts3T{static_cast<const float*>(a->data), a->strides[0], a->strides[1], a->strides[2]};
  return TOTRI_OK;
}

int origin_of(const totri_array_t* o, int64_t n, int has) {
  (void)o;
  (void)n;
  return has;
}

}  // namespace
}  // namespace totri

using namespace totri;

extern "C" {

int totri_backprojection_confocal_velten_forward(const totri_array_t* transient,
                                                 const totri_array_t* scan_points,
                                                 const totri_array_t* scan_origin,
                                                 const totri_array_t* volume, const float start[3],
                                                 const float end[3], float bw, float bo,
                                                 void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  bp::Grid g;
  int64_t B, S, So;
  TOTRI_TRY(check_volume_out(volume, g, start, end, B));
  bp::Pts3 sp, so;
  TOTRI_TRY(check_pts3(scan_points, "scan_points", B, S, sp));
  TOTRI_TRY(check_pts3(scan_origin, "scan_origin", B, So, so));
  if (So != 0 && So != S) return fail(TOTRI_ERR_INVALID_ARGUMENT, "scan_origin size mismatch");
  TOTRI_TRY(check_array(transient, "transient", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient, "transient", 0, B));
  TOTRI_TRY(check_dim(transient, "transient", 2, S));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  const int T = (int)transient->shape[1];
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  if (nv == 0 || B == 0) return TOTRI_OK;
  const bool tiled = tune::get("backprojection.velten.mode") != 1;
  int vz = tune::get("backprojection.velten.vz");
  if (vz <= 0) vz = 4;
  if (vz != 1 && vz != 2 && vz != 4)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "backprojection.velten.vz must be 1, 2 or 4");
  const dim3 grid((unsigned)ceil_div(g.W, bp::kBX), (unsigned)ceil_div(g.H, bp::kBY),
                  (unsigned)ceil_div(g.D, bp::kBZ * vz));
  // Group windows when one point's bins over a voxel block alone, 2 |block
  // diagonal| / bw, span more than 100 rows (measured on 128^3 and 192^3
  // voxels from 128^2 and 256^2 points: whole-tile windows were faster up to
  // 82 rows, group windows from 122); "backprojection.velten.groups" = 1
  // forces whole-tile windows, 2 group windows.
  int groups = tune::get("backprojection.velten.groups");
  if (groups != 1 && groups != 2) {
    const auto pitch = [](float a, float e, int n) {
      return n > 1 ? std::fabs((double)e - (double)a) / (n - 1) : 0.0;
    };
    const double ex = bp::kBX * pitch(g.sx, g.ex, g.W), ey = bp::kBY * pitch(g.sy, g.ey, g.H);
    const double ez = bp::kBZ * vz * pitch(g.sz, g.ez, g.D);
    const double rows = 2.0 * std::sqrt(ex * ex + ey * ey + ez * ez) / std::fabs((double)bw);
    groups = rows > 100.0 ? 2 : 1;
  }
  const bool grouped = groups == 2;
  for (int b = 0; b < (int)B; ++b) {
    const bp::FastBin fb = bp::make_fast_bin(bw, bo);
    const float* trp = static_cast<const float*>(transient->data);
    float* volp = static_cast<float*>(volume->data);
    // 4 voxels per thread with registers capped for 6 CTAs per SM (38, no
    // spills; 34 KB of shared memory each): 38.2 ms against 40.4 ms uncapped
    // (47 registers, 5 CTAs; "backprojection.velten.occupancy" = 1), the same
    // volume bit for bit.
#define TOTRI_VELTEN_TILED(VZ, OCC, PAIR)                                                  \
  TOTRI_KERNEL("backprojection velten confocal", stream,                                  \
               grouped ? (bp::velten_confocal_tiled_kernel<VZ, OCC, true, PAIR>           \
                          <<<grid, 256, 0, stream>>>(g, b, T, (int)S, sp, so, So > 0, bw, \
                                                     bo, fb, trp, volp))                  \
                       : (bp::velten_confocal_tiled_kernel<VZ, OCC, false, PAIR>          \
                          <<<grid, 256, 0, stream>>>(g, b, T, (int)S, sp, so, So > 0, bw, \
                                                     bo, fb, trp, volp)))
    // Bins of two voxels at a time with paired FP32 instructions
    // (velten_bin_col2; "backprojection.velten.pair" = 2 takes them one at a
    // time): 33.3 ms against 39.0 ms, the same volume bit for bit.
    const bool pair = tune::get("backprojection.velten.pair") != 2;
    const int occ = (int)tune::get("backprojection.velten.occupancy");
    if (tiled && vz == 4 && pair && occ == 5)
      TOTRI_VELTEN_TILED(4, 5, true);
    else if (tiled && vz == 4 && pair && occ != 1)
      TOTRI_VELTEN_TILED(4, 6, true);
    else if (tiled && vz == 4 && occ != 1)
      TOTRI_VELTEN_TILED(4, 6, false);
    else if (tiled && vz == 4)
      TOTRI_VELTEN_TILED(4, 1, false);
    else if (tiled && vz == 2 && pair)
      TOTRI_VELTEN_TILED(2, 1, true);
    else if (tiled && vz == 2)
      TOTRI_VELTEN_TILED(2, 1, false);
    else if (tiled)
      TOTRI_VELTEN_TILED(1, 1, false);
#undef TOTRI_VELTEN_TILED
    else
      TOTRI_KERNEL("backprojection velten confocal", stream,
                   bp::velten_confocal_kernel<<<(unsigned)ceil_div(nv, 256), 256, 0, stream>>>(
                       g, b, T, (int)S, sp, so, So > 0, bw, bo, bp::make_fast_bin(bw, bo),
                       static_cast<const float*>(transient->data),
                       static_cast<float*>(volume->data)));
  }
  return TOTRI_OK;
}

int totri_backprojection_confocal_velten_adjoint(const totri_array_t* volume,
                                                 const totri_array_t* scan_points,
                                                 const totri_array_t* scan_origin,
                                                 const totri_array_t* transient,
                                                 const float start[3], const float end[3],
                                                 float bw, float bo, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  bp::Grid g;
  int64_t B, S, So;
  TOTRI_TRY(check_volume_out(volume, g, start, end, B));
  bp::Pts3 sp, so;
  TOTRI_TRY(check_pts3(scan_points, "scan_points", B, S, sp));
  TOTRI_TRY(check_pts3(scan_origin, "scan_origin", B, So, so));
  if (So != 0 && So != S) return fail(TOTRI_ERR_INVALID_ARGUMENT, "scan_origin size mismatch");
  TOTRI_TRY(check_array(transient, "transient", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient, "transient", 0, B));
  TOTRI_TRY(check_dim(transient, "transient", 2, S));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  const int T = (int)transient->shape[1];
  if (numel(transient) == 0) return TOTRI_OK;
  const size_t smem = sizeof(float) * (size_t)T * bp::kTS;
  if (smem > 200 * 1024) return fail(TOTRI_ERR_UNSUPPORTED, "too many bins for one tile");
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(bp::velten_adjoint_kernel), smem));
  for (int b = 0; b < (int)B; ++b)
    TOTRI_KERNEL("backprojection velten adjoint", stream,
                 bp::velten_adjoint_kernel<<<(unsigned)ceil_div(S, bp::kTS), 256, smem, stream>>>(
                     g, b, T, (int)S, sp, so, So > 0, bw, bo, bp::make_fast_bin(bw, bo),
                     static_cast<const float*>(volume->data),
                     static_cast<float*>(transient->data)));
  return TOTRI_OK;
}

int totri_backprojection_exhaustive_velten_forward(
    const totri_array_t* transient, const totri_array_t* scan_points,
    const totri_array_t* laser_points, const totri_array_t* scan_origin,
    const totri_array_t* laser_origin, const totri_array_t* volume, const float start[3],
    const float end[3], float bw, float bo, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  bp::Grid g;
  int64_t B, S, L, So, Lo;
  TOTRI_TRY(check_volume_out(volume, g, start, end, B));
  bp::Pts3 sp, lp, so, lo;
  TOTRI_TRY(check_pts3(scan_points, "scan_points", B, S, sp));
  TOTRI_TRY(check_pts3(laser_points, "laser_points", B, L, lp));
  TOTRI_TRY(check_pts3(scan_origin, "scan_origin", B, So, so));
  TOTRI_TRY(check_pts3(laser_origin, "laser_origin", B, Lo, lo));
  if ((So != 0 && So != S) || (Lo != 0 && Lo != L))
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "origin size mismatch");
  TOTRI_TRY(check_array(transient, "transient", 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient, "transient", 0, B));
  TOTRI_TRY(check_dim(transient, "transient", 2, S));
  TOTRI_TRY(check_dim(transient, "transient", 3, L));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  const int T = (int)transient->shape[1];
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  if (nv == 0) return TOTRI_OK;
  for (int b = 0; b < (int)B; ++b)
    TOTRI_KERNEL("backprojection velten exhaustive", stream,
                 bp::velten_exhaustive_kernel<<<(unsigned)ceil_div(nv, 128), 128, 0, stream>>>(
                     g, b, T, (int)S, (int)L, sp, lp, so, lo, So > 0, Lo > 0, bw, bo,
                     static_cast<const float*>(transient->data),
                     static_cast<float*>(volume->data)));
  return TOTRI_OK;
}

int totri_backprojection_exhaustive_arellano_forward(
    const totri_array_t* transient, const totri_array_t* scan_points,
    const totri_array_t* laser_points, const totri_array_t* scan_origin,
    const totri_array_t* laser_origin, const totri_array_t* volume, const float start[3],
    const float end[3], float bw, float bo, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  bp::Grid g;
  int64_t B, S, L, So, Lo;
  TOTRI_TRY(check_volume_out(volume, g, start, end, B));
  bp::Pts3T sp, lp, so, lo;
  TOTRI_TRY(check_pts3t(scan_points, "scan_points", B, S, sp));
  TOTRI_TRY(check_pts3t(laser_points, "laser_points", B, L, lp));
  TOTRI_TRY(check_pts3t(scan_origin, "scan_origin", B, So, so));
  TOTRI_TRY(check_pts3t(laser_origin, "laser_origin", B, Lo, lo));
  if ((So != 0 && So != S) || (Lo != 0 && Lo != L))
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "origin size mismatch");
  TOTRI_TRY(check_array(transient, "transient", 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient, "transient", 0, B));
  TOTRI_TRY(check_dim(transient, "transient", 2, S));
  TOTRI_TRY(check_dim(transient, "transient", 3, L));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  const int T = (int)transient->shape[1];
  if (g.H * g.W == 0 || S == 0 || L == 0) return TOTRI_OK;
  for (int b = 0; b < (int)B; ++b) {
    const dim3 grid((unsigned)ceil_div(g.H * g.W, 64), (unsigned)S, (unsigned)L);
    TOTRI_KERNEL("backprojection arellano", stream,
                 bp::arellano_kernel<<<grid, 64, 0, stream>>>(
                     g, b, T, (int)S, (int)L, sp, lp, so, lo, origin_of(scan_origin, S, So > 0),
                     origin_of(laser_origin, L, Lo > 0), bw, bo,
                     static_cast<const float*>(transient->data),
                     static_cast<float*>(volume->data)));
  }
  return TOTRI_OK;
}

}  // extern "C"
