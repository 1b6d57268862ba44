// RBF-to-volume splatting and its gradient.
//
// Reference: src/util/rbf2volume_cuda.cu (:50-93 forward, one thread per voxel
// reading every Gaussian from global memory; :124-201 gradient, one block
// column per Gaussian with a shared-memory tree reduction and an atomic per
// (Gaussian, channel, 64 voxels)). Here both kernels work on bricks of voxels
// and take the Gaussians in shared-memory tiles, skipping those that
// contribute exactly zero to the whole brick (the underflow cull below): the
// forward gives each thread one voxel; the gradient gives each surviving
// Gaussian a warp over the brick's voxels, accumulates all 4+A channels in
// registers and issues 4+A atomics per (Gaussian, brick).
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

__device__ __forceinline__ float warp_sum_f(float x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

struct Rbf {  // [B, N, C] with strides
  const float* p;
  int64_t sb, sn, sc;
  __device__ float at(int b, int i, int c) const { return p[b * sb + i * sn + c * sc]; }
};

// Tile-level cull at the underflow radius. ex2.approx.ftz flushes results
// below 2^-126 to zero, so a Gaussian whose exponent argument d2 * k2 lies
// below -126.5 at every voxel of a brick adds exactly +0 (or -0) there, and
// an accumulator that started at +0 is unchanged by it: skipping it leaves the
// sums bit for bit the same, in the same order. The test uses the squared
// distance from the centre to the brick's coordinate box (voxel coordinates
// are monotone in the index), computed in FP32, against 128 / |k2|, which
// leaves a margin far beyond the few ulps of the voxel-level arithmetic.
// Gaussians with a non-finite value are never culled (0 * inf would not be a
// zero term). The tuning key "rbf.cull" = 1 turns the cull off.
constexpr float kCullArg = 128.f;

// Squared distance from (cx, cy, cz) to the box [lo, hi].
__device__ __forceinline__ float box_dist2(float cx, float cy, float cz, const float lo[3],
                                           const float hi[3]) {
  const float dx = fmaxf(fmaxf(lo[0] - cx, cx - hi[0]), 0.f);
  const float dy = fmaxf(fmaxf(lo[1] - cy, cy - hi[1]), 0.f);
  const float dz = fmaxf(fmaxf(lo[2] - cz, cz - hi[2]), 0.f);
  return dx * dx + dy * dy + dz * dz;
}

// Coordinate box of the voxels [i0, i1] of one axis.
__device__ __forceinline__ void axis_box(float s, float e, int n, int i0, int i1, float& lo,
                                         float& hi) {
  const float a = coord(s, e, n, i0), b = coord(s, e, n, i1);
  lo = fminf(a, b);
  hi = fmaxf(a, b);
}

// Block-wide compaction: this thread's slot among the flagged threads (or -1);
// *total receives their count. All threads of the block call it.
__device__ __forceinline__ int block_slot(bool flag, int* warp_counts, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) warp_counts[warp] = __popc(bal);
  __syncthreads();
  int base = 0, sum = 0;
  for (int w = 0; w < nw; ++w) {
    const int c = warp_counts[w];
    base += w < warp ? c : 0;
    sum += c;
  }
  *total = sum;
  return flag ? base + __popc(bal & ((1u << lane) - 1u)) : -1;
}

// Forward: a CTA per brick of 8 x 8 x 4 voxels (x fastest), one thread per
// voxel; Gaussians come in tiles of 256, each culled against the brick's box,
// and the survivors are evaluated in their original order.
// VZ voxels of a column per thread, 4 apart in z (bricks of 8 x 8 x 4 VZ).
// With VZ = 2 the two voxels share the Gaussian's loads and dx, dy, and their
// exponents and sums run as paired FP32 instructions (each rounds as its
// scalar form, in the same order), so the volume is the same bit for bit.
template <int VZ>
__global__ void __launch_bounds__(256) forward_kernel(Grid g, int b, Rbf r, int N, int C, int cull,
                                                      float* __restrict__ vol) {
  __shared__ float tile[kTile][4 + kMaxAttr];
  __shared__ int counts[8];
  const int A = C - 4;
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const int tid = threadIdx.x;
  const int bx = blockIdx.x * 8, by = blockIdx.y * 8, bz = blockIdx.z * 4 * VZ;
  const int xi = bx + (tid & 7), yi = by + ((tid >> 3) & 7);
  int zi[VZ];
  bool inside[VZ];
  float z[VZ];
#pragma unroll
  for (int v = 0; v < VZ; ++v) {
    zi[v] = bz + (tid >> 6) + 4 * v;
    inside[v] = xi < g.W && yi < g.H && zi[v] < g.D;
    z[v] = coord(g.sz, g.ez, g.D, zi[v]);
  }
  const float x = coord(g.sx, g.ex, g.W, xi), y = coord(g.sy, g.ey, g.H, yi);
  float lo[3], hi[3];
  axis_box(g.sx, g.ex, g.W, bx, min(bx + 7, g.W - 1), lo[0], hi[0]);
  axis_box(g.sy, g.ey, g.H, by, min(by + 7, g.H - 1), lo[1], hi[1]);
  axis_box(g.sz, g.ez, g.D, bz, min(bz + 4 * VZ - 1, g.D - 1), lo[2], hi[2]);
  float sum[VZ];
  float attr[VZ][kMaxAttr];
#pragma unroll
  for (int v = 0; v < VZ; ++v) {
    sum[v] = 0.f;
#pragma unroll
    for (int a = 0; a < kMaxAttr; ++a) attr[v][a] = 0.f;
  }
  for (int i0 = 0; i0 < N; i0 += kTile) {
    __syncthreads();  // the previous tile has been read
    float val[4 + kMaxAttr];
    bool keep = false;
    if (i0 + tid < N) {
      bool finite = true;
      for (int c = 0; c < C; ++c) {
        val[c] = r.at(b, i0 + tid, c);
        finite = finite && isfinite(val[c]);
      }
      // slot 3 holds -log2(e) / (2 sigma^2) instead of sigma
      val[3] = -0.5f * kLog2e / (val[3] * val[3]);
      keep = !cull || !finite || !isfinite(val[3]) ||
             !(box_dist2(val[0], val[1], val[2], lo, hi) * -val[3] > kCullArg);
    }
    int cnt;
    const int at = block_slot(keep, counts, &cnt);
    if (keep)
      for (int c = 0; c < C; ++c) tile[at][c] = val[c];
    __syncthreads();
    for (int i = 0; i < cnt; ++i) {
      const float dx = tile[i][0] - x, dy = tile[i][1] - y;
      if constexpr (VZ == 2) {
        const unsigned long long dz = f2sub(f2pack(tile[i][2], tile[i][2]), f2pack(z[0], z[1]));
        const unsigned long long d2 =
            f2fma(f2pack(dx, dx), f2pack(dx, dx),
                  f2fma(f2pack(dy, dy), f2pack(dy, dy), f2mul(dz, dz)));
        float e0, e1;
        f2unpack(f2mul(d2, f2pack(tile[i][3], tile[i][3])), e0, e1);
        const unsigned long long w = f2pack(exp2_approx(e0), exp2_approx(e1));
        unsigned long long s2 = f2add(f2pack(sum[0], sum[1]), w);
        f2unpack(s2, sum[0], sum[1]);
#pragma unroll
        for (int a = 0; a < kMaxAttr; ++a)
          if (a < A) {
            const float t = tile[i][4 + a];
            f2unpack(f2fma(w, f2pack(t, t), f2pack(attr[0][a], attr[1][a])), attr[0][a],
                     attr[1][a]);
          }
      } else {
        const float dz = tile[i][2] - z[0];
        const float w = exp2_approx(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) * tile[i][3]);
        sum[0] += w;
#pragma unroll
        for (int a = 0; a < kMaxAttr; ++a)
          if (a < A) attr[0][a] = fmaf(w, tile[i][4 + a], attr[0][a]);
      }
    }
  }
  const int A1 = A;
  float* out = vol + (size_t)b * (1 + A1) * nv;
#pragma unroll
  for (int v = 0; v < VZ; ++v) {
    if (!inside[v]) continue;
    const int64_t o = ((int64_t)zi[v] * g.H + yi) * g.W + xi;
    out[o] = sum[v];
    const float norm = sum[v] < 1e-8f ? 1.f : sum[v];
#pragma unroll
    for (int a = 0; a < kMaxAttr; ++a)
      if (a < A1) out[(size_t)(1 + a) * nv + o] = attr[v][a] / norm;
  }
}

constexpr int kChunk = 512;  // voxels of a gradient brick (8 x 8 x 8)

// Floats per staged voxel of the gradient brick, rounded up to an odd count:
// lane j reads voxel j, so an even record (8 floats for one attribute) put
// 8 lanes on each of 4 banks (the gradient spent 9.7 short-scoreboard stalls
// per issue on it), an odd one spreads a warp's reads over all 32 banks.
__host__ __device__ constexpr int grad_stride(int A) { return (4 + 2 * (1 + A)) | 1; }

// Gradient (rbf2volume_cuda.cu:124-201): a CTA per brick of 8 x 8 x 8 voxels,
// whose coordinates, volume and volume_grad channels are staged in shared
// memory. Gaussians come in tiles of 256, culled against the brick's box as
// in the forward; each surviving Gaussian goes to one warp, whose lanes take
// the brick's voxels, accumulate all 4+A channels, reduce them across the
// warp and add them to rbf_grad with one atomic per channel.
__global__ void __launch_bounds__(256) grad_kernel(Grid g, int b, Rbf r, int N, int C, int cull,
                                                   const float* __restrict__ vol,
                                                   const float* __restrict__ vgrad,
                                                   float* __restrict__ rgrad, int64_t gsb,
                                                   int64_t gsn, int64_t gsc) {
  // [kChunk][grad_stride(A)]: x y z valid | vol[1+A] | grad[1+A] (| pad)
  extern __shared__ float sm[];
  __shared__ int list[kTile];
  __shared__ int counts[8];
  const int A = C - 4;
  const int stride = grad_stride(A);
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int bx = blockIdx.x * 8, by = blockIdx.y * 8, bz = blockIdx.z * 8;
  const float* vb = vol + (size_t)b * (1 + A) * nv;
  const float* gb = vgrad + (size_t)b * (1 + A) * nv;
  for (int j = tid; j < kChunk; j += blockDim.x) {
    const int xi = bx + (j & 7), yi = by + ((j >> 3) & 7), zi = bz + (j >> 6);
    float* e = sm + j * stride;
    const bool in = xi < g.W && yi < g.H && zi < g.D;
    e[0] = coord(g.sx, g.ex, g.W, xi);
    e[1] = coord(g.sy, g.ey, g.H, yi);
    e[2] = coord(g.sz, g.ez, g.D, zi);
    e[3] = in ? 1.f : 0.f;
    const int64_t v = in ? ((int64_t)zi * g.H + yi) * g.W + xi : 0;
    for (int q = 0; q <= A; ++q) {
      e[4 + q] = in ? vb[(size_t)q * nv + v] : 0.f;
      e[4 + 1 + A + q] = in ? gb[(size_t)q * nv + v] : 0.f;
    }
  }
  float lo[3], hi[3];
  axis_box(g.sx, g.ex, g.W, bx, min(bx + 7, g.W - 1), lo[0], hi[0]);
  axis_box(g.sy, g.ey, g.H, by, min(by + 7, g.H - 1), lo[1], hi[1]);
  axis_box(g.sz, g.ez, g.D, bz, min(bz + 7, g.D - 1), lo[2], hi[2]);
  for (int i0 = 0; i0 < N; i0 += kTile) {
    __syncthreads();  // the staged voxels are written / the previous list is read
    bool keep = false;
    if (i0 + tid < N) {
      const float cx = r.at(b, i0 + tid, 0), cy = r.at(b, i0 + tid, 1);
      const float cz = r.at(b, i0 + tid, 2), sg = r.at(b, i0 + tid, 3);
      const float k2 = -0.5f * kLog2e * (1.f / (sg * sg));
      keep = !cull || !(isfinite(cx) && isfinite(cy) && isfinite(cz) && isfinite(k2)) ||
             !(box_dist2(cx, cy, cz, lo, hi) * -k2 > kCullArg);
    }
    int cnt;
    const int at = block_slot(keep, counts, &cnt);
    if (keep) list[at] = i0 + tid;
    __syncthreads();
    for (int q = warp; q < cnt; q += 8) {
      const int i = list[q];
      const float xr = r.at(b, i, 0), yr = r.at(b, i, 1), zr = r.at(b, i, 2);
      const float sigma = r.at(b, i, 3);
      float ra[kMaxAttr];
#pragma unroll
      for (int a = 0; a < kMaxAttr; ++a) ra[a] = a < A ? r.at(b, i, 4 + a) : 0.f;
      const float is2 = 1.f / (sigma * sigma);
      const float k2 = -0.5f * kLog2e * is2;  // w = 2^(d2 * k2)
      const float is3 = is2 / sigma;
      float gx = 0.f, gy = 0.f, gz = 0.f, gs = 0.f;
      float ga[kMaxAttr];
#pragma unroll
      for (int a = 0; a < kMaxAttr; ++a) ga[a] = 0.f;
      for (int j = lane; j < kChunk; j += 32) {
        const float* e = sm + j * stride;
        if (e[3] == 0.f) continue;  // outside the grid
        const float ex = e[0] - xr, ey = e[1] - yr, ez = e[2] - zr;
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
          float s = 0.f;
#pragma unroll
          for (int a = 0; a < kMaxAttr; ++a) {
            if (a < A) {
              const float dla = e[4 + 1 + A + 1 + a];
              s += dla * (ra[a] - e[4 + 1 + a]);
              ga[a] += dla * w * inv;
            }
          }
          dl += s * inv;
        }
        gx += dwx * dl;
        gy += dwy * dl;
        gz += dwz * dl;
        gs += dws * dl;
      }
      gx = warp_sum_f(gx);
      gy = warp_sum_f(gy);
      gz = warp_sum_f(gz);
      gs = warp_sum_f(gs);
#pragma unroll
      for (int a = 0; a < kMaxAttr; ++a)
        if (a < A) ga[a] = warp_sum_f(ga[a]);
      if (lane == 0) {
        float* out = rgrad + b * gsb + i * gsn;
        atomicAdd(out, gx);
        atomicAdd(out + gsc, gy);
        atomicAdd(out + 2 * gsc, gz);
        atomicAdd(out + 3 * gsc, gs);
#pragma unroll
        for (int a = 0; a < kMaxAttr; ++a)
          if (a < A) atomicAdd(out + (4 + a) * gsc, ga[a]);
      }
    }
  }
}


// grad_kernel with two Gaussians per warp iteration: each staged voxel
// record is read once for both, the voxel's 1 / vol[0] is shared, and the
// two Gaussians' terms run as paired FP32 instructions (the ex2 per
// Gaussian). kA attributes at most (1 or kMaxAttr): fewer live registers for
// the common single weight.
template <int kA>
__global__ void __launch_bounds__(256) grad_pair_kernel(Grid g, int b, Rbf r, int N, int C,
                                                        int cull, const float* __restrict__ vol,
                                                        const float* __restrict__ vgrad,
                                                        float* __restrict__ rgrad, int64_t gsb,
                                                        int64_t gsn, int64_t gsc) {
  using u64 = unsigned long long;
  extern __shared__ float sm[];
  __shared__ int list[kTile];
  __shared__ int counts[8];
  const int A = C - 4;
  const int stride = grad_stride(A);
  const int64_t nv = (int64_t)g.D * g.H * g.W;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int bx = blockIdx.x * 8, by = blockIdx.y * 8, bz = blockIdx.z * 8;
  const float* vb = vol + (size_t)b * (1 + A) * nv;
  const float* gb = vgrad + (size_t)b * (1 + A) * nv;
  for (int j = tid; j < kChunk; j += blockDim.x) {
    const int xi = bx + (j & 7), yi = by + ((j >> 3) & 7), zi = bz + (j >> 6);
    float* e = sm + j * stride;
    const bool in = xi < g.W && yi < g.H && zi < g.D;
    e[0] = coord(g.sx, g.ex, g.W, xi);
    e[1] = coord(g.sy, g.ey, g.H, yi);
    e[2] = coord(g.sz, g.ez, g.D, zi);
    e[3] = in ? 1.f : 0.f;
    const int64_t v = in ? ((int64_t)zi * g.H + yi) * g.W + xi : 0;
    for (int q = 0; q <= A; ++q) {
      e[4 + q] = in ? vb[(size_t)q * nv + v] : 0.f;
      e[4 + 1 + A + q] = in ? gb[(size_t)q * nv + v] : 0.f;
    }
  }
  float lo[3], hi[3];
  axis_box(g.sx, g.ex, g.W, bx, min(bx + 7, g.W - 1), lo[0], hi[0]);
  axis_box(g.sy, g.ey, g.H, by, min(by + 7, g.H - 1), lo[1], hi[1]);
  axis_box(g.sz, g.ez, g.D, bz, min(bz + 7, g.D - 1), lo[2], hi[2]);
  for (int i0 = 0; i0 < N; i0 += kTile) {
    __syncthreads();  // the staged voxels are written / the previous list is read
    bool keep = false;
    if (i0 + tid < N) {
      const float cx = r.at(b, i0 + tid, 0), cy = r.at(b, i0 + tid, 1);
      const float cz = r.at(b, i0 + tid, 2), sg = r.at(b, i0 + tid, 3);
      const float k2 = -0.5f * kLog2e * (1.f / (sg * sg));
      keep = !cull || !(isfinite(cx) && isfinite(cy) && isfinite(cz) && isfinite(k2)) ||
             !(box_dist2(cx, cy, cz, lo, hi) * -k2 > kCullArg);
    }
    int cnt;
    const int at = block_slot(keep, counts, &cnt);
    if (keep) list[at] = i0 + tid;
    __syncthreads();
    for (int q = 2 * warp; q < cnt; q += 16) {
      const bool two = q + 1 < cnt;
      const int ia = list[q], ib = two ? list[q + 1] : ia;
      float sga = r.at(b, ia, 3), sgb = r.at(b, ib, 3);
      const float is2a = 1.f / (sga * sga), is2b = 1.f / (sgb * sgb);
      const u64 XR = f2pack(r.at(b, ia, 0), r.at(b, ib, 0));
      const u64 YR = f2pack(r.at(b, ia, 1), r.at(b, ib, 1));
      const u64 ZR = f2pack(r.at(b, ia, 2), r.at(b, ib, 2));
      const u64 IS2 = f2pack(is2a, is2b);
      const u64 K2 = f2pack(-0.5f * kLog2e * is2a, -0.5f * kLog2e * is2b);
      const u64 IS3 = f2pack(is2a / sga, is2b / sgb);
      u64 RA[kA];
#pragma unroll
      for (int a = 0; a < kA; ++a)
        RA[a] = a < A ? f2pack(r.at(b, ia, 4 + a), r.at(b, ib, 4 + a)) : 0ull;
      u64 GX = 0ull, GY = 0ull, GZ = 0ull, GS = 0ull;  // (+0, +0)
      u64 GA[kA];
#pragma unroll
      for (int a = 0; a < kA; ++a) GA[a] = 0ull;
      for (int j = lane; j < kChunk; j += 32) {
        const float* e = sm + j * stride;
        if (e[3] == 0.f) continue;  // outside the grid
        const u64 EX = f2sub(f2pack(e[0], e[0]), XR);
        const u64 EY = f2sub(f2pack(e[1], e[1]), YR);
        const u64 EZ = f2sub(f2pack(e[2], e[2]), ZR);
        const u64 D2 = f2fma(EX, EX, f2fma(EY, EY, f2mul(EZ, EZ)));
        float ta, tb;
        f2unpack(f2mul(D2, K2), ta, tb);
        const u64 W = f2pack(exp2_approx(ta), exp2_approx(tb));
        const u64 WI = f2mul(IS2, W);
        const u64 DWS = f2mul(f2mul(D2, IS3), W);
        const float dl0 = e[4 + 1 + A];
        u64 DL = f2pack(dl0, dl0);
        if (A > 0) {
          float v0 = e[4];
          if (v0 < 1e-8f) v0 = 1.f;
          const float inv = 1.f / v0;
          const u64 INV = f2pack(inv, inv);
          u64 S = 0ull;
#pragma unroll
          for (int a = 0; a < kA; ++a) {
            if (a < A) {
              const float dla = e[4 + 1 + A + 1 + a], ea = e[4 + 1 + a];
              const u64 DLA = f2pack(dla, dla);
              S = f2fma(DLA, f2sub(RA[a], f2pack(ea, ea)), S);
              GA[a] = f2fma(f2mul(DLA, W), INV, GA[a]);
            }
          }
          DL = f2fma(S, INV, DL);
        }
        GX = f2fma(f2mul(EX, WI), DL, GX);
        GY = f2fma(f2mul(EY, WI), DL, GY);
        GZ = f2fma(f2mul(EZ, WI), DL, GZ);
        GS = f2fma(DWS, DL, GS);
      }
      float out2[2][4 + kA];
      f2unpack(GX, out2[0][0], out2[1][0]);
      f2unpack(GY, out2[0][1], out2[1][1]);
      f2unpack(GZ, out2[0][2], out2[1][2]);
      f2unpack(GS, out2[0][3], out2[1][3]);
#pragma unroll
      for (int a = 0; a < kA; ++a) f2unpack(GA[a], out2[0][4 + a], out2[1][4 + a]);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int c = 0; c < 4 + kA; ++c)
          if (c < 4 + A) out2[h][c] = warp_sum_f(out2[h][c]);
        if (lane == 0 && (h == 0 || two)) {
          float* o = rgrad + b * gsb + (h ? ib : ia) * gsn;
#pragma unroll
          for (int c = 0; c < 4 + kA; ++c)
            if (c < 4 + A) atomicAdd(o + c * gsc, out2[h][c]);
        }
      }
    }
  }
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
  const int cull = tune::get("rbf.cull") != 1;
  // two voxels per thread ("rbf.forward.vz" = 1: one)
  const int vz = tune::get("rbf.forward.vz") == 1 ? 1 : 2;
  const dim3 grid((unsigned)ceil_div(g.W, 8), (unsigned)ceil_div(g.H, 8),
                  (unsigned)ceil_div(g.D, 4 * vz));
  for (int b = 0; b < (int)B; ++b) {
    if (vz == 2)
      TOTRI_KERNEL("rbf2volume forward", stream,
                   rbf::forward_kernel<2><<<grid, 256, 0, stream>>>(
                       g, b, rr, (int)N, C, cull, static_cast<float*>(vol->data)));
    else
      TOTRI_KERNEL("rbf2volume forward", stream,
                   rbf::forward_kernel<1><<<grid, 256, 0, stream>>>(
                       g, b, rr, (int)N, C, cull, static_cast<float*>(vol->data)));
  }
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
  const size_t smem = sizeof(float) * rbf::kChunk * rbf::grad_stride(A);
  const int cull = tune::get("rbf.cull") != 1;
  const dim3 grid((unsigned)ceil_div(g.W, 8), (unsigned)ceil_div(g.H, 8), (unsigned)ceil_div(g.D, 8));
  // two Gaussians per warp iteration ("rbf.grad.pair" = 2: one)
  const bool pair = tune::get("rbf.grad.pair") != 2;
  const void* fn = !pair ? reinterpret_cast<const void*>(rbf::grad_kernel)
                   : A <= 1 ? reinterpret_cast<const void*>(rbf::grad_pair_kernel<1>)
                            : reinterpret_cast<const void*>(rbf::grad_pair_kernel<rbf::kMaxAttr>);
  TOTRI_CUDA(tune::ensure_dynamic_smem(fn, smem));
  const float* vp = static_cast<const float*>(vol->data);
  const float* gp = static_cast<const float*>(vgrad->data);
  float* rp = static_cast<float*>(rgrad->data);
  for (int b = 0; b < (int)B; ++b) {
    if (!pair)
      TOTRI_KERNEL("rbf2volume grad", stream,
                   rbf::grad_kernel<<<grid, 256, smem, stream>>>(
                       g, b, rr, (int)N, C, cull, vp, gp, rp, rgrad->strides[0],
                       rgrad->strides[1], rgrad->strides[2]));
    else if (A <= 1)
      TOTRI_KERNEL("rbf2volume grad", stream,
                   rbf::grad_pair_kernel<1><<<grid, 256, smem, stream>>>(
                       g, b, rr, (int)N, C, cull, vp, gp, rp, rgrad->strides[0],
                       rgrad->strides[1], rgrad->strides[2]));
    else
      TOTRI_KERNEL("rbf2volume grad", stream,
                   rbf::grad_pair_kernel<rbf::kMaxAttr><<<grid, 256, smem, stream>>>(
                       g, b, rr, (int)N, C, cull, vp, gp, rp, rgrad->strides[0],
                       rgrad->strides[1], rgrad->strides[2]));
  }
  return TOTRI_OK;
}

}  // extern "C"
