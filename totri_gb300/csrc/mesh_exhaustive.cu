// Exhaustive (separate laser and detector points) mesh transient rendering:
// forward splat and vertex / albedo gradient.
//
// Reference: src/render/program/mesh_exhaustive_forward_optix.cu:18-169 and
// mesh_exhaustive_grad_verts_optix.cu:18-248: one OptiX thread per (face,
// scan, laser) triple tracing two visibility rays, global atomics into
// transient[b][bin][s][l]. Here visibility is separable: face f is visible
// from scan point s and from laser point l independently, so the two masks
// are computed once (S + L rows of the shared mask buffer) and each triple is
// their AND. The forward gives each CTA one scan point and a tile of laser
// points with a [T][tile] shared histogram flushed as rows of the [T][S][L]
// output; the gradient gives each CTA 32 faces and a slice of scan points and
// walks every (s, l) pair of the slice.
#include <cooperative_groups.h>

#include <algorithm>

#include "capi_common.cuh"
#include "mesh.cuh"
#include "mesh_kernels.cuh"
#include "tune.cuh"

namespace cg = cooperative_groups;

namespace totri {
namespace mesh {

struct ExhPair {
  fv3 v[3];
  int perm[3];
  float d[3];   // scan + laser path length (sort key)
  float ds[3];  // vertex - scan distance
  float dl[3];  // vertex - laser distance
  float c[3];
  int bin[3];
};

__device__ __forceinline__ void exh_sort(ExhPair& q) {
  auto sw = [&](int i, int j) {
    float t = q.d[i]; q.d[i] = q.d[j]; q.d[j] = t;
    t = q.ds[i]; q.ds[i] = q.ds[j]; q.ds[j] = t;
    t = q.dl[i]; q.dl[i] = q.dl[j]; q.dl[j] = t;
    fv3 tv = q.v[i]; q.v[i] = q.v[j]; q.v[j] = tv;
    int tp = q.perm[i]; q.perm[i] = q.perm[j]; q.perm[j] = tp;
  };
  if (q.d[0] > q.d[1]) sw(0, 1);
  if (q.d[1] > q.d[2]) sw(1, 2);
  if (q.d[0] > q.d[1]) sw(0, 1);
}

// FP32 decisions exactly as the oracle takes them (exhaustive_geom).
__device__ __forceinline__ void exh_pair(float4 s0, float4 s1, float4 s2, fv3 sp, fv3 lp, float od,
                                         float bw, float bo, ExhPair& q) {
  q.v[0] = mkv(s0.x, s0.y, s0.z);
  q.v[1] = mkv(s1.x, s1.y, s1.z);
  q.v[2] = mkv(s2.x, s2.y, s2.z);
  for (int k = 0; k < 3; ++k) {
    q.perm[k] = k;
    q.ds[k] = xlen(xsub3(q.v[k], sp));
    q.dl[k] = xlen(xsub3(q.v[k], lp));
    q.d[k] = xadd(q.ds[k], q.dl[k]);
  }
  exh_sort(q);
  for (int k = 0; k < 3; ++k) {
    q.c[k] = xdiv(xsub(xadd(q.d[k], od), bo), bw);
    q.bin[k] = bin_of(q.c[k]);
  }
}

// exh_pair with a filtered fast path (FastBins). The six lengths come from
// the hardware reciprocal square root and the bin coordinates from a fused
// multiply-add with a precomputed 1/bw. Against the exact chain each path
// length d = |v - s| + |v - l| deviates by at most 8 u d (u = 2^-24), so when
// the three fast lengths are separated by more than 16 u max(d) the exact
// sort gives the same order, and a bin coordinate farther than
// 32 u (d + od + |bo|)/bw + 8 u |c| from an integer truncates to the exact
// bin. Only then are the fast values kept (they differ from the exact ones
// by a few ulps, which the value tolerances absorb); otherwise, and for
// NaN or huge coordinates, the exact exh_pair runs. Bins and vertex order
// are therefore always those of the exact chain.
__device__ __forceinline__ void exh_pair_filtered(float4 s0, float4 s1, float4 s2, fv3 sp,
                                                  fv3 lp, float od, float bw, float bo,
                                                  const FastBins& fb, ExhPair& q) {
  q.v[0] = mkv(s0.x, s0.y, s0.z);
  q.v[1] = mkv(s1.x, s1.y, s1.z);
  q.v[2] = mkv(s2.x, s2.y, s2.z);
  for (int k = 0; k < 3; ++k) {
    q.perm[k] = k;
    q.ds[k] = len_fast(q.v[k] - sp);
    q.dl[k] = len_fast(q.v[k] - lp);
    q.d[k] = q.ds[k] + q.dl[k];
  }
  exh_sort(q);
  const float u = 5.9604645e-8f;
  bool ok = q.d[1] - q.d[0] > 16.f * u * q.d[2] && q.d[2] - q.d[1] > 16.f * u * q.d[2];
  for (int k = 0; k < 3; ++k) {
    const float c = fmaf(q.d[k] + od, fb.inv_bw, fb.nbo);
    const float m = fmaf(fb.kc, q.d[k] + od, fb.kb) + 8.f * u * fabsf(c);
    ok = ok && fabsf(c - rintf(c)) > m && fabsf(c) < 1.0e9f;
    q.c[k] = c;
    q.bin[k] = __float2int_rz(c);
  }
  if (!ok) exh_pair(s0, s1, s2, sp, lp, od, bw, bo, q);
}

// AlphaExhaustive (mesh_common.h:505-531), wall normals (0,0,1).
__device__ __forceinline__ float alpha_exhaustive(const ExhPair& q, fv3 c, fv3 sp, fv3 lp,
                                                  float rho) {
  const fv3 n = cross(q.v[1] - q.v[0], q.v[2] - q.v[0]);
  const fv3 rs = c - sp, rl = c - lp;
  if (!(rs.z > 0.f) || !(rl.z > 0.f)) return 0.f;
  const float rss = dot(rs, rs), rll = dot(rl, rl);
  return vdiv(100.f * rho * rs.z * rl.z * fabsf(dot(n, rs)) * fabsf(dot(n, rl)) *
                  rsqrtf(dot(n, n)),
              (rss * rss) * (rll * rll));
}

__device__ __forceinline__ float origin_term(const Origins& o, int b, int s, int l, fv3 sp,
                                             fv3 lp) {
  float od = 0.f;
  if (o.has_so) od = xlen(xsub3(sp, mkv(o.so.at(b, s, 0), o.so.at(b, s, 1), o.so.at(b, s, 2))));
  if (o.has_lo)
    od = xadd(od, xlen(xsub3(lp, mkv(o.lo.at(b, l, 0), o.lo.at(b, l, 1), o.lo.at(b, l, 2)))));
  return od;
}

// One CTA per (scan point, tile of LT lasers): the tile's [T][LT] histogram in
// shared memory, flushed once. With CL > 1 the CTAs of a cluster of CL
// neighbouring tiles (CL LT = 8 lasers) each flush every CL-th bin row for the
// whole cluster, reading the other tiles' histograms through distributed
// shared memory, so every row piece is one full 32-byte sector: a 4-laser
// tile's own 16-byte pieces make the memory read, merge and write back each
// sector (8.75 GB of DRAM traffic for a 2 GB transient).
template <int LT, int kOcc = 1, int CL = 1>
__global__ void __launch_bounds__(256, kOcc) exh_splat_kernel(Scene sc, View3f sp, View3f lp, Origins org,
                                                        int S, int L, float* __restrict__ out,
                                                        int T, float bw, float bo, FastBins fb) {
  extern __shared__ float hist[];  // [T][LT]
  const int b = blockIdx.z;
  const int s = blockIdx.x;
  const int l0 = blockIdx.y * LT;
  for (int i = threadIdx.x; i < T * LT; i += blockDim.x) hist[i] = 0.f;
  __syncthreads();
  const int n = sc.meta[b].n;
  const int ll = threadIdx.x % LT;
  const int l = l0 + ll;
  if (l < L) {
    const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
    const fv3 q = mkv(lp.at(b, l, 0), lp.at(b, l, 1), lp.at(b, l, 2));
    const float od = origin_term(org, b, s, l, p, q);
    const uint32_t* ms = sc.mask + ((size_t)b * sc.P + s) * sc.nch;
    const uint32_t* ml = sc.mask + ((size_t)b * sc.P + S + l) * sc.nch;
    const float4* shade = sc.shade + (size_t)b * sc.F * 4;
    Hist<LT> h{hist, ll, T};
    for (int k = threadIdx.x / LT; k < n; k += blockDim.x / LT) {
      const uint32_t bit = 1u << (k & 31);
      if (!(__ldg(ms + (k >> 5)) & bit) || !(__ldg(ml + (k >> 5)) & bit)) continue;
      const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
      const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
      ExhPair e;
      exh_pair_filtered(s0r, s1r, s2r, p, q, od, bw, bo, fb, e);
      const float alpha = alpha_exhaustive(e, mkv(s3r.x, s3r.y, s3r.z), p, q, s0r.w);
      if (!(alpha > 0.f)) continue;
      splat_tent(h, e.c, e.bin, alpha);
    }
  }
  __syncthreads();
  if (CL == 1) {
    // rows out[b][t][s][l0 .. l0+LT)
    float* ob = out + (((size_t)b * T) * S + s) * L + l0;
    for (int i = threadIdx.x; i < T * LT; i += blockDim.x) {
      const int t = i / LT, c = i - t * LT;
      if (l0 + c < L) ob[(size_t)t * S * L + c] = hist[i];
    }
  } else {
    cg::cluster_group cluster = cg::this_cluster();
    cluster.sync();  // every tile of the cluster has its histogram
    const int rank = (int)cluster.block_rank();
    const int L0 = l0 - rank * LT;  // the cluster's first laser
    float* ob = out + (((size_t)b * T) * S + s) * L + L0;
    const int rows = (T - rank + CL - 1) / CL;
    for (int i = threadIdx.x; i < rows * CL * LT; i += blockDim.x) {
      const int t = rank + CL * (i / (CL * LT)), j = i % (CL * LT);
      const int src = j / LT, c = j - src * LT;
      const float* rh = cluster.map_shared_rank(hist, src);
      if (L0 + j < L) ob[(size_t)t * S * L + j] = rh[t * LT + c];
    }
    cluster.sync();  // no tile leaves while another still reads its histogram
  }
}

// Forward with the visible triples compacted first (tuning option). Visibility is separable,
// so for the CTA's scan point s and each of its LT lasers the visible faces of
// a 32-face chunk are one AND of two mask words. Each warp walks its chunks,
// appends the visible (face, laser) pairs to a per-warp queue in shared memory
// and evaluates them 32 at a time, one per lane: every lane does useful work
// instead of most lanes waiting on mask tests that fail.
constexpr int kExhQueue = 64;

template <int LT>
__global__ void __launch_bounds__(256) exh_splat_compact_kernel(Scene sc, View3f sp, View3f lp,
                                                                Origins org, int S, int L,
                                                                float* __restrict__ out, int T,
                                                                float bw, float bo, FastBins fb) {
  extern __shared__ float hist[];  // [T][LT]
  __shared__ float lpt[LT][4];     // laser point, laser-origin term
  __shared__ int queue[8][kExhQueue];
  const int b = blockIdx.z;
  const int s = blockIdx.x;
  const int l0 = blockIdx.y * LT;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < T * LT; i += blockDim.x) hist[i] = 0.f;
  const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
  if (threadIdx.x < LT && l0 + (int)threadIdx.x < L) {
    const int l = l0 + threadIdx.x;
    const fv3 q = mkv(lp.at(b, l, 0), lp.at(b, l, 1), lp.at(b, l, 2));
    lpt[threadIdx.x][0] = q.x;
    lpt[threadIdx.x][1] = q.y;
    lpt[threadIdx.x][2] = q.z;
    lpt[threadIdx.x][3] = origin_term(org, b, s, l, p, q);
  }
  __syncthreads();
  const int n = sc.meta[b].n;
  const int nchu = (n + 31) >> 5;
  const uint32_t* ms = sc.mask + ((size_t)b * sc.P + s) * sc.nch;
  const uint32_t* ml = sc.mask + ((size_t)b * sc.P + S) * sc.nch;
  const float4* shade = sc.shade + (size_t)b * sc.F * 4;
  const int lts = min(LT, L - l0);
  const uint32_t below = (1u << lane) - 1u;
  int* qw = queue[warp];
  int cnt = 0;  // warp-uniform
  auto run = [&](int e) {
    const int k = e >> 5, l = e & 31;
    const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
    const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
    const fv3 q = mkv(lpt[l][0], lpt[l][1], lpt[l][2]);
    ExhPair ep;
    exh_pair_filtered(s0r, s1r, s2r, p, q, lpt[l][3], bw, bo, fb, ep);
    const float alpha = alpha_exhaustive(ep, mkv(s3r.x, s3r.y, s3r.z), p, q, s0r.w);
    if (!(alpha > 0.f)) return;
    const Hist<LT> h{hist, l, T};
    splat_tent(h, ep.c, ep.bin, alpha);
  };
  for (int ch = warp; ch < nchu; ch += 8) {
    const uint32_t msw = __ldg(ms + ch);
    if (msw == 0u) continue;
    const uint32_t lw =
        lane < lts ? (__ldg(ml + (size_t)(l0 + lane) * sc.nch + ch) & msw) : 0u;
    for (int l = 0; l < lts; ++l) {
      const uint32_t bits = __shfl_sync(0xffffffffu, lw, l);
      if (bits == 0u) continue;
      if ((bits >> lane) & 1u) qw[cnt + __popc(bits & below)] = ((ch * 32 + lane) << 5) | l;
      cnt += __popc(bits);
      if (cnt >= 32) {
        __syncwarp();
        const int e = qw[lane];
        __syncwarp();
        if (lane < cnt - 32) qw[lane] = qw[32 + lane];
        cnt -= 32;
        __syncwarp();
        run(e);
      }
    }
  }
  __syncwarp();
  if (lane < cnt) run(qw[lane]);
  __syncthreads();
  // rows out[b][t][s][l0 .. l0+LT)
  float* ob = out + (((size_t)b * T) * S + s) * L + l0;
  for (int i = threadIdx.x; i < T * LT; i += blockDim.x) {
    const int t = i / LT, c = i - t * LT;
    if (l0 + c < L) ob[(size_t)t * S * L + c] = hist[i];
  }
}

// The origin terms |s - o_s| + |l - o_l| as a double-float (zero without origins).
__device__ __forceinline__ DFloat origin_term_df(const Origins& o, int b, int s, int l, fv3 sp,
                                                 fv3 lp) {
  DFloat od{0.f, 0.f};
  if (o.has_so) od = len_df(sp, mkv(o.so.at(b, s, 0), o.so.at(b, s, 1), o.so.at(b, s, 2)));
  if (o.has_lo)
    od = df_add(od, len_df(lp, mkv(o.lo.at(b, l, 0), o.lo.at(b, l, 1), o.lo.at(b, l, 2))));
  return od;
}

// The tent corners of a triple relative to its first bin, from double-float
// path lengths |v_k - s| + |v_k - l| + od (bin_offset).
__device__ __forceinline__ void exh_corners(const ExhPair& q, fv3 sp, fv3 lp, DFloat od, float bw,
                                            float inv_bw, float bo, float x[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const DFloat d = df_add(df_add(len_df(q.v[k], sp), len_df(q.v[k], lp)), od);
    x[k] = bin_offset(d, bo, bw, inv_bw, q.bin[0]);
  }
}

// Gradient of one visible triple w.r.t. the sorted vertices and the albedo
// (mesh_exhaustive_grad_verts_optix.cu:336-412, AlphaExhaustiveGradVerts
// mesh_common.h:549-630), with the tent corners x taken relative to bin[0]
// (exh_corners).
__device__ __forceinline__ bool triple_grad(const ExhPair& q, const float x[3], fv3 c, fv3 sp,
                                            fv3 lp, float rho, float bw,
                                            const float* __restrict__ col, int64_t stride, int T,
                                            fv3 dv[3], float& dmat) {
  const float alpha = alpha_exhaustive(q, c, sp, lp, rho);
  if (!(alpha > 0.f)) return false;
  if (q.bin[0] >= T || q.bin[2] < 0) return false;
  const fv3 e1 = q.v[1] - q.v[0], e2 = q.v[2] - q.v[0];
  const fv3 n = cross(e1, e2);
  const fv3 rs = c - sp, rl = c - lp;
  const float kn = vdiv(-1.f, dot(n, n));
  const float krs = vdiv(-4.f, 3.f * dot(rs, rs)), krl = vdiv(-4.f, 3.f * dot(rl, rl));
  const float kw = vdiv(1.f, 3.f * rs.z) + vdiv(1.f, 3.f * rl.z);
  const float knrs = vdiv(1.f, dot(n, rs)), knrl = vdiv(1.f, dot(n, rl));
  const fv3 w = kn * n + knrs * rs + knrl * rl;
  const fv3 g1 = cross(e2, w), g2 = cross(w, e1);
  const fv3 common = krs * rs + krl * rl + ((knrs + knrl) * (1.f / 3.f)) * n + mkv(0.f, 0.f, kw);
  const fv3 da0 = alpha * (common - g1 - g2);
  const fv3 da1 = alpha * (common + g1);
  const fv3 da2 = alpha * (common + g2);
  const float dadm = vdiv(alpha, rho);
  if (q.bin[0] == q.bin[2]) {
    const float g = __ldg(col + (size_t)q.bin[0] * stride);
    dv[0] = g * da0;
    dv[1] = g * da1;
    dv[2] = g * da2;
    dmat = g * dadm;
    return true;
  }
  TentGrad tgr;
  tent_grad(col, stride, T, x, q.bin, tgr);
  const float span = x[2] - x[0];
  const float kk = vdiv(-2.f, bw * span * span);
  fv3 dc[3];
  for (int k = 0; k < 3; ++k)
    dc[k] = vdiv(1.f, bw * q.dl[k]) * (q.v[k] - lp) + vdiv(1.f, bw * q.ds[k]) * (q.v[k] - sp);
  const fv3 dyc0 = kk * (vdiv(-1.f, q.dl[0]) * (q.v[0] - lp) + vdiv(-1.f, q.ds[0]) * (q.v[0] - sp));
  const fv3 dyc2 = kk * (vdiv(1.f, q.dl[2]) * (q.v[2] - lp) + vdiv(1.f, q.ds[2]) * (q.v[2] - sp));
  dv[0] = tgr.part0 * da0 + alpha * (tgr.ayc * dyc0 + tgr.a0 * dc[0]);
  dv[1] = tgr.part0 * da1 + alpha * (tgr.a1 * dc[1]);
  dv[2] = tgr.part0 * da2 + alpha * (tgr.ayc * dyc2 + tgr.a2 * dc[2]);
  dmat = dadm * tgr.part0;
  return true;
}

__global__ void __launch_bounds__(256) exh_grad_kernel(Scene sc, View3f sp, View3f lp, Origins org,
                                                       int S, int L,
                                                       const float* __restrict__ tgrad, int T,
                                                       float bw, float bo, FastBins fb, GradOut out) {
  extern __shared__ uint32_t mcol[];  // [S + L] mask words of this 32-face chunk
  const int b = blockIdx.y;
  const int ch = blockIdx.x;
  const int n = sc.meta[b].n;
  if (ch * 32 >= n) return;
  // scan-point slice [s0, s1) of this CTA (gridDim.z slices); all laser rows
  const int s0 = (int)((int64_t)S * blockIdx.z / gridDim.z);
  const int s1 = (int)((int64_t)S * (blockIdx.z + 1) / gridDim.z);
  for (int i = threadIdx.x; i < S + L; i += blockDim.x)
    if (i >= S || (i >= s0 && i < s1)) mcol[i] = sc.mask[((size_t)b * sc.P + i) * sc.nch + ch];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const float* tgb = tgrad + (size_t)b * T * S * L;
  const int64_t stride = (int64_t)S * L;
  const float4* shade = sc.shade + (size_t)b * sc.F * 4;
  for (int j = warp; j < 32; j += nw) {
    const int k = ch * 32 + j;
    if (k >= n) break;
    const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
    const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
    const fv3 c = mkv(s3r.x, s3r.y, s3r.z);
    fv3 acc[3] = {mkv(0.f, 0.f, 0.f), mkv(0.f, 0.f, 0.f), mkv(0.f, 0.f, 0.f)};
    float accm = 0.f;
    for (int s = s0; s < s1; ++s) {
      if (!((mcol[s] >> j) & 1u)) continue;
      const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
      for (int l = lane; l < L; l += 32) {
        if (!((mcol[S + l] >> j) & 1u)) continue;
        const fv3 q = mkv(lp.at(b, l, 0), lp.at(b, l, 1), lp.at(b, l, 2));
        ExhPair e;
        exh_pair_filtered(s0r, s1r, s2r, p, q, origin_term(org, b, s, l, p, q), bw, bo, fb,
                          e);
        if (e.bin[0] >= T || e.bin[2] < 0) continue;
        float x[3];
        exh_corners(e, p, q, origin_term_df(org, b, s, l, p, q), bw, fb.inv_bw, bo, x);
        fv3 dv[3];
        float dm;
        if (!triple_grad(e, x, c, p, q, s0r.w, bw, tgb + (size_t)s * L + l, stride, T, dv, dm))
          continue;
        add_permuted(acc, dv, e.perm);
        accm += dm;
      }
    }
    scatter_face_grad(out, b, s1r, s2r, s3r, acc, accm, sc.status);
  }
}

// Gradient with the visible (scan point, laser) pairs of each face compacted:
// the CTA holds its 32 faces' scan-mask words for a slice of scan points and,
// per face, the set of lasers that see it (transposed from the laser rows by
// warp ballots). A warp walks one face at a time, queues its visible
// (s, l) pairs and evaluates them 32 at a time, one per lane; the face's
// gradient stays in registers and is reduced and scattered once per CTA.
__global__ void __launch_bounds__(256) exh_grad_compact_kernel(
    Scene sc, View3f sp, View3f lp, Origins org, int S, int L, const float* __restrict__ tgrad,
    int T, float bw, float bo, FastBins fb, GradOut out) {
  extern __shared__ uint32_t words[];  // [slice] scan words | [32][LW] laser sets
  __shared__ int qs[8][kExhQueue], ql[8][kExhQueue];
  const int b = blockIdx.y;
  const int ch = blockIdx.x;
  const int n = sc.meta[b].n;
  if (ch * 32 >= n) return;
  const int s0 = (int)((int64_t)S * blockIdx.z / gridDim.z);
  const int s1 = (int)((int64_t)S * (blockIdx.z + 1) / gridDim.z);
  const int ns = s1 - s0;
  const int LW = (L + 31) >> 5;
  uint32_t* mcs = words;
  uint32_t* lvis = words + ns;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t* mrow = sc.mask + (size_t)b * sc.P * sc.nch + ch;
  for (int i = threadIdx.x; i < ns; i += blockDim.x) mcs[i] = mrow[(size_t)(s0 + i) * sc.nch];
  for (int wl = warp; wl < LW; wl += 8) {
    const int l = wl * 32 + lane;
    const uint32_t m = l < L ? mrow[(size_t)(S + l) * sc.nch] : 0u;
    for (int j = 0; j < 32; ++j) {
      const uint32_t bal = __ballot_sync(0xffffffffu, (m >> j) & 1u);
      if (lane == 0) lvis[j * LW + wl] = bal;
    }
  }
  __syncthreads();
  const float* tgb = tgrad + (size_t)b * T * S * L;
  const int64_t stride = (int64_t)S * L;
  const float4* shade = sc.shade + (size_t)b * sc.F * 4;
  const uint32_t below = (1u << lane) - 1u;
  for (int j = warp; j < 32; j += 8) {
    const int k = ch * 32 + j;
    if (k >= n) break;
    const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
    const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
    const fv3 c = mkv(s3r.x, s3r.y, s3r.z);
    fv3 acc[3] = {mkv(0.f, 0.f, 0.f), mkv(0.f, 0.f, 0.f), mkv(0.f, 0.f, 0.f)};
    float accm = 0.f;
    auto run = [&](int s, int l) {
      const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
      const fv3 q = mkv(lp.at(b, l, 0), lp.at(b, l, 1), lp.at(b, l, 2));
      ExhPair e;
      exh_pair_filtered(s0r, s1r, s2r, p, q, origin_term(org, b, s, l, p, q), bw, bo, fb,
                          e);
      if (e.bin[0] >= T || e.bin[2] < 0) return;
      float x[3];
      exh_corners(e, p, q, origin_term_df(org, b, s, l, p, q), bw, fb.inv_bw, bo, x);
      fv3 dv[3];
      float dm;
      if (!triple_grad(e, x, c, p, q, s0r.w, bw, tgb + (size_t)s * L + l, stride, T, dv, dm))
        return;
      add_permuted(acc, dv, e.perm);
      accm += dm;
    };
    const uint32_t* lv = lvis + j * LW;
    int cnt = 0;  // warp-uniform
    for (int si = 0; si < ns; ++si) {
      if (!((mcs[si] >> j) & 1u)) continue;
      for (int wl = 0; wl < LW; ++wl) {
        const uint32_t bits = lv[wl];
        if (bits == 0u) continue;
        if ((bits >> lane) & 1u) {
          const int at = cnt + __popc(bits & below);
          qs[warp][at] = s0 + si;
          ql[warp][at] = wl * 32 + lane;
        }
        cnt += __popc(bits);
        if (cnt >= 32) {
          __syncwarp();
          const int es = qs[warp][lane], el = ql[warp][lane];
          __syncwarp();
          if (lane < cnt - 32) {
            qs[warp][lane] = qs[warp][32 + lane];
            ql[warp][lane] = ql[warp][32 + lane];
          }
          cnt -= 32;
          __syncwarp();
          run(es, el);
        }
      }
    }
    __syncwarp();
    if (lane < cnt) run(qs[warp][lane], ql[warp][lane]);
    __syncwarp();
    scatter_face_grad(out, b, s1r, s2r, s3r, acc, accm, sc.status);
  }
}

// Gradient that uses the separability of the triple terms. For one face,
// everything that depends on the scan point s alone or the laser point l alone
// is computed once per point into a shared-memory record:
//   - the exact FP32 lengths |v_m - p| that decide the vertex order and bins
//     (the same chain as exh_pair) and their double-float low parts;
//   - the origin term |p - o_p| (exact FP32 and low part);
//   - the point's alpha factor A_p = max(0, r.z) |n.r| / |r|^4 (r = c - p),
//     with alpha = 100 rho |n|^-1 A_s A_l (AlphaExhaustive, mesh_common.h:505-531);
//   - its parts of d log(alpha) / d v_m: cm = -4/3 r/|r|^2 + n/(3 n.r) +
//     (0, 0, 1/(3 r.z)), the same for every vertex, and wv = r/(n.r), which
//     enters through the normal's Jacobian (AlphaExhaustiveGradVerts,
//     mesh_common.h:549-630);
//   - the unit vectors u_m = (v_m - p)/|v_m - p| that make up d c_k / d v.
// A triple then only combines two records: the alpha gradient is taken in the
// face's own vertex order (the formula is the same in any order), and only
// the tent terms follow the sorted order. A CTA takes its faces one at a time
// over a slice of at most kFaceSlice scan points and the lasers in chunks of
// kFaceSlice; its 256 threads share each face's (s, l) pairs. The decisions
// (vertex order, bins) are those of exh_pair.
constexpr int kFaceSlice = 256;
constexpr int kFacesPerCta = 8;
// Most bytes of one bins-last copy of transient_grad (a range of scan points
// of one batch item; launch_exhaustive_grad).
constexpr size_t kGradChunkBytes = size_t(2) << 30;
constexpr int kRec = 24;  // floats per point record (fields below)
enum : int {
  kRecD = 0,     // [3] exact FP32 lengths
  kRecDlo = 3,   // [3] their low parts
  kRecOd = 6,    // origin term, FP32
  kRecOdlo = 7,  // its low part
  kRecA = 8,     // alpha factor
  kRecCm = 9,    // [3]
  kRecWv = 12,   // [3]
  kRecU = 15,    // [9] unit vectors u_m
};

// Fills the record of point p (origin o if has_o) for the face (v, c, n);
// rec[f * stride] is field f.
__device__ __forceinline__ void exh_point_record(const fv3 v[3], fv3 c, fv3 n, fv3 p, bool has_o,
                                                 fv3 o, float* rec, int stride) {
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const float d = xlen(xsub3(v[m], p));
    const DFloat df = len_df(v[m], p);
    rec[(kRecD + m) * stride] = d;
    rec[(kRecDlo + m) * stride] = (df.hi - d) + df.lo;
    const float inv = vdiv(1.f, d);
    const fv3 u = inv * (v[m] - p);
    rec[(kRecU + 3 * m) * stride] = u.x;
    rec[(kRecU + 3 * m + 1) * stride] = u.y;
    rec[(kRecU + 3 * m + 2) * stride] = u.z;
  }
  float od = 0.f, odlo = 0.f;
  if (has_o) {
    od = xlen(xsub3(p, o));
    const DFloat df = len_df(p, o);
    odlo = (df.hi - od) + df.lo;
  }
  rec[kRecOd * stride] = od;
  rec[kRecOdlo * stride] = odlo;
  const fv3 r = c - p;
  const float rr = dot(r, r), nr = dot(n, r);
  const bool front = r.z > 0.f;
  rec[kRecA * stride] = front ? vdiv(r.z * fabsf(nr), rr * rr) : 0.f;
  const float kr = vdiv(-4.f, 3.f * rr), knr = vdiv(1.f, nr), kw = vdiv(1.f, 3.f * r.z);
  const fv3 cm = kr * r + (knr * (1.f / 3.f)) * n + mkv(0.f, 0.f, front ? kw : 0.f);
  rec[kRecCm * stride] = cm.x;
  rec[(kRecCm + 1) * stride] = cm.y;
  rec[(kRecCm + 2) * stride] = cm.z;
  rec[kRecWv * stride] = knr * r.x;
  rec[(kRecWv + 1) * stride] = knr * r.y;
  rec[(kRecWv + 2) * stride] = knr * r.z;
}

// Block-wide compaction: returns this thread's slot among the threads whose
// flag is set (or -1) and leaves their count in *total. All 256 threads call it.
__device__ __forceinline__ int block_slot(bool flag, int* warp_counts, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  if (lane == 0) warp_counts[warp] = __popc(bal);
  __syncthreads();
  int base = 0, sum = 0;
  for (int w = 0; w < 8; ++w) {
    const int c = warp_counts[w];
    base += w < warp ? c : 0;
    sum += c;
  }
  *total = sum;
  return flag ? base + __popc(bal & ((1u << lane) - 1u)) : -1;
}

template <int kOcc>
__global__ void __launch_bounds__(256, kOcc) exh_grad_face_kernel(
    Scene sc, View3f sp, View3f lp, Origins org, int S, int L, const float* __restrict__ tgrad,
    int T, float bw, float bo, GradOut out, int faces_per_cta, int lchunk, int sslice, int b0,
    int s_base, int s_end, int64_t bstride, int64_t cstep, int64_t bstep) {
  // Batch item b0 + blockIdx.y, scan points [s_base, s_end); transient_grad
  // element (t, s, l) of item b is tgrad[(b - b0) bstride + ((s - s_base) L +
  // l) cstep + t bstep]: the caller's [B, T, S, L] tensor (b0 = s_base = 0,
  // bstride = T S L, cstep = 1, bstep = S L) or one item's bins-last copy of
  // a range of scan points (cstep = T, bstep = 1).
  extern __shared__ float recs[];        // scan-point then laser-point records, SoA
  float* srec = recs;
  float* lrec = recs + kRec * kFaceSlice;
  __shared__ short sidx[kFaceSlice], lidx[kFaceSlice];
  __shared__ int counts[2][8];
  __shared__ float red[8][10];
  const int b = b0 + blockIdx.y;
  const int n = sc.meta[b].n;
  const int nlc = (L + lchunk - 1) / lchunk;
  const int s0 = s_base + (blockIdx.z / nlc) * sslice;
  const int ns_all = min(sslice, s_end - s0);
  const int la = (blockIdx.z % nlc) * lchunk, lb = min(L, la + lchunk);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const float* tgb = tgrad + (int64_t)(b - b0) * bstride;
  const int64_t stride = bstep;
  const float4* shade = sc.shade + (size_t)b * sc.F * 4;
  const uint32_t* mrows = sc.mask + (size_t)b * sc.P * sc.nch;
  const float inv_bw = __frcp_rn(bw);
  for (int fi = 0; fi < faces_per_cta; ++fi) {
    const int k = blockIdx.x * faces_per_cta + fi;
    if (k >= n) break;  // CTA-uniform
    const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
    const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
    const fv3 v[3] = {mkv(s0r.x, s0r.y, s0r.z), mkv(s1r.x, s1r.y, s1r.z), mkv(s2r.x, s2r.y, s2r.z)};
    const fv3 c = mkv(s3r.x, s3r.y, s3r.z);
    const fv3 e1 = v[1] - v[0], e2 = v[2] - v[0];
    const fv3 nrm = cross(e1, e2);
    const float nn = dot(nrm, nrm);
    const float rho = s0r.w;
    const float kf = 100.f * rho * rsqrtf(nn);
    const fv3 wf = vdiv(-1.f, nn) * nrm;
    const int ch = k >> 5;
    const uint32_t bit = 1u << (k & 31);
    // the face's scan-point records over this slice
    int ns;
    {
      const int s = s0 + tid;
      const bool vis = tid < ns_all && (mrows[(size_t)s * sc.nch + ch] & bit);
      const int at = block_slot(vis, counts[0], &ns);
      if (vis) {
        const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
        const fv3 o = org.has_so ? mkv(org.so.at(b, s, 0), org.so.at(b, s, 1), org.so.at(b, s, 2))
                                 : mkv(0.f, 0.f, 0.f);
        exh_point_record(v, c, nrm, p, org.has_so, o, srec + at, kFaceSlice);
        sidx[at] = (short)tid;
      }
    }
    float acc[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) acc[q] = 0.f;
    for (int l0 = la; l0 < lb && ns > 0; l0 += kFaceSlice) {
      int nl;
      {
        const int l = l0 + tid;
        const bool vis = l < lb && tid < kFaceSlice &&
                         (mrows[(size_t)(S + l) * sc.nch + ch] & bit);
        const int at = block_slot(vis, counts[1], &nl);
        if (vis) {
          const fv3 p = mkv(lp.at(b, l, 0), lp.at(b, l, 1), lp.at(b, l, 2));
          const fv3 o = org.has_lo ? mkv(org.lo.at(b, l, 0), org.lo.at(b, l, 1), org.lo.at(b, l, 2))
                                   : mkv(0.f, 0.f, 0.f);
          exh_point_record(v, c, nrm, p, org.has_lo, o, lrec + at, kFaceSlice);
          lidx[at] = (short)tid;
        }
      }
      __syncthreads();
      const int pairs = ns * nl;
      // pair index tid + 256 t walks (si, li) with li fastest
      int si = nl > 0 ? tid / nl : 0, li = nl > 0 ? tid - si * nl : 0;
      const int dq = nl > 0 ? 256 / nl : 0, dr = nl > 0 ? 256 - dq * nl : 0;
      for (int pi = tid; pi < pairs; pi += 256) {
        const float* rs = srec + si;
        const float* rl = lrec + li;
        const int s = s0 + sidx[si], l = l0 + lidx[li];
        li += dr;
        si += dq;
        if (li >= nl) {
          li -= nl;
          ++si;
        }
        const float as = rs[kRecA * kFaceSlice], al = rl[kRecA * kFaceSlice];
        const float alpha = kf * as * al;
        if (!(alpha > 0.f)) continue;
        float d[3];
#pragma unroll
        for (int m = 0; m < 3; ++m)
          d[m] = xadd(rs[(kRecD + m) * kFaceSlice], rl[(kRecD + m) * kFaceSlice]);
        // the vertex order of exh_sort (stable compare-swaps on the path length)
        int p0 = 0, p1 = 1, p2 = 2;
        float d0 = d[0], d1 = d[1], d2 = d[2];
        if (d0 > d1) { float t = d0; d0 = d1; d1 = t; int u = p0; p0 = p1; p1 = u; }
        if (d1 > d2) { float t = d1; d1 = d2; d2 = t; int u = p1; p1 = p2; p2 = u; }
        if (d0 > d1) { float t = d0; d0 = d1; d1 = t; int u = p0; p0 = p1; p1 = u; }
        const float ods = rs[kRecOd * kFaceSlice], odl = rl[kRecOd * kFaceSlice];
        const float od = xadd(ods, odl);
        int bin[3];
        bin[0] = bin_of(xdiv(xsub(xadd(d0, od), bo), bw));
        bin[1] = bin_of(xdiv(xsub(xadd(d1, od), bo), bw));
        bin[2] = bin_of(xdiv(xsub(xadd(d2, od), bo), bw));
        if (bin[0] >= T || bin[2] < 0) continue;
        const float* col = tgb + ((int64_t)(s - s_base) * L + l) * cstep;
        fv3 da[3];
        {
          const fv3 w = wf + mkv(rs[kRecWv * kFaceSlice], rs[(kRecWv + 1) * kFaceSlice],
                                 rs[(kRecWv + 2) * kFaceSlice]) +
                        mkv(rl[kRecWv * kFaceSlice], rl[(kRecWv + 1) * kFaceSlice],
                            rl[(kRecWv + 2) * kFaceSlice]);
          const fv3 cm = mkv(rs[kRecCm * kFaceSlice] + rl[kRecCm * kFaceSlice],
                             rs[(kRecCm + 1) * kFaceSlice] + rl[(kRecCm + 1) * kFaceSlice],
                             rs[(kRecCm + 2) * kFaceSlice] + rl[(kRecCm + 2) * kFaceSlice]);
          const fv3 g1 = cross(e2, w), g2 = cross(w, e1);
          da[0] = alpha * (cm - g1 - g2);
          da[1] = alpha * (cm + g1);
          da[2] = alpha * (cm + g2);
        }
        const float dadm = vdiv(alpha, rho);
        if (bin[0] == bin[2]) {
          const float g = __ldg(col + (int64_t)bin[0] * stride);
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            acc[3 * m] += g * da[m].x;
            acc[3 * m + 1] += g * da[m].y;
            acc[3 * m + 2] += g * da[m].z;
          }
          acc[9] += g * dadm;
          continue;
        }
        // double-float path lengths of the three vertices, then the corners
        // of the sorted ones relative to bin[0]
        const DFloat odf = df_add(DFloat{ods, rs[kRecOdlo * kFaceSlice]},
                                  DFloat{odl, rl[kRecOdlo * kFaceSlice]});
        float xo[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const DFloat path =
              df_add(df_add(DFloat{rs[(kRecD + m) * kFaceSlice], rs[(kRecDlo + m) * kFaceSlice]},
                            DFloat{rl[(kRecD + m) * kFaceSlice], rl[(kRecDlo + m) * kFaceSlice]}),
                     odf);
          xo[m] = bin_offset(path, bo, bw, inv_bw, bin[0]);
        }
        auto pick = [](const float a[3], int i) { return i == 0 ? a[0] : (i == 1 ? a[1] : a[2]); };
        const float x[3] = {pick(xo, p0), pick(xo, p1), pick(xo, p2)};
        TentGrad tgr;
        tent_grad(col, stride, T, x, bin, tgr);
        const float span = x[2] - x[0];
        const float kk = vdiv(-2.f, bw * span * span);
        // tent terms per sorted position: gamma_k u_(perm k), u = u_s + u_l
        const float gs0 = vdiv(tgr.a0, bw) - tgr.ayc * kk, gs1 = vdiv(tgr.a1, bw);
        const float gs2 = vdiv(tgr.a2, bw) + tgr.ayc * kk;
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const float gm = m == p0 ? gs0 : (m == p1 ? gs1 : gs2);
          const float ag = alpha * gm;
          const fv3 u = mkv(rs[(kRecU + 3 * m) * kFaceSlice] + rl[(kRecU + 3 * m) * kFaceSlice],
                            rs[(kRecU + 3 * m + 1) * kFaceSlice] +
                                rl[(kRecU + 3 * m + 1) * kFaceSlice],
                            rs[(kRecU + 3 * m + 2) * kFaceSlice] +
                                rl[(kRecU + 3 * m + 2) * kFaceSlice]);
          acc[3 * m] += tgr.part0 * da[m].x + ag * u.x;
          acc[3 * m + 1] += tgr.part0 * da[m].y + ag * u.y;
          acc[3 * m + 2] += tgr.part0 * da[m].z + ag * u.z;
        }
        acc[9] += dadm * tgr.part0;
      }
      __syncthreads();  // records are rewritten for the next laser chunk / face
    }
    // the face's gradient: warp sums, then one thread per vertex component
#pragma unroll
    for (int q = 0; q < 10; ++q) {
      const float t = warp_sum(acc[q]);
      if (lane == 0) red[warp][q] = t;
    }
    __syncthreads();
    if (tid < 10 && ns > 0) {
      float t = 0.f;
      for (int w = 0; w < 8; ++w) t += red[w][tid];
      const int vi[3] = {__float_as_int(s1r.w), __float_as_int(s2r.w), __float_as_int(s3r.w)};
      if (tid < 9) {
        const int m = tid / 3, a = tid - 3 * m;
        if (vi[m] < 0 || vi[m] >= out.V) {
          atomicOr(sc.status, kStatusFaceIndexRange);
        } else if (out.vg) {
          atomicAdd(out.vg + b * out.vsb + vi[m] * out.vsv + a * out.vsc, t);
        }
      } else if (out.mg) {
        for (int m = 0; m < 3; ++m)
          if (vi[m] >= 0 && vi[m] < out.V)
            atomicAdd(out.mg + b * out.msb + vi[m] * out.msv, (1.f / 3.f) * t);
      }
    }
    __syncthreads();
  }
}

template <int LT>
static int launch_exh_splat(const Scene& sc, const View3f& sp, const View3f& lp,
                            const Origins& org, int S, int L, float* out, int T, float bw,
                            float bo, cudaStream_t stream) {
  const FastBins fast = make_fast_bins(bw, bo, tune::get("mesh.exhaustive.exact") != 1);
  const size_t smem = sizeof(float) * (size_t)T * LT;
  const dim3 grid((unsigned)S, (unsigned)ceil_div(L, LT), (unsigned)sc.B);
  // Per-thread mask tests by default: on the 32-mesh batch (2048 bins, 64x64
  // detector x 16x16 laser points) they took 4.4 s against 4.9 s for the
  // compacted variant, which "mesh.exhaustive.splat.mode" = 1 selects.
  if (tune::get("mesh.exhaustive.splat.mode") != 1) {
    // Tiles narrower than a 32-byte sector flush through a cluster of
    // 8 / LT tiles ("mesh.exhaustive.splat.cluster" = 1: each tile alone).
    constexpr int CL = LT < 8 ? 8 / LT : 1;
    if (CL > 1 && tune::get("mesh.exhaustive.splat.cluster") != 1) {
      const bool capped = tune::get("mesh.exhaustive.splat.occupancy") != 1;
      auto* kern = capped ? exh_splat_kernel<LT, 5, CL> : exh_splat_kernel<LT, 1, CL>;
      TOTRI_CUDA(tune::ensure_dynamic_smem(reinterpret_cast<const void*>(kern), smem));
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(grid.x, (unsigned)(ceil_div(grid.y, CL) * CL), grid.z);
      cfg.blockDim = dim3(256);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = stream;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = 1;
      attr[0].val.clusterDim.y = CL;
      attr[0].val.clusterDim.z = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      cudaError_t le = cudaSuccess;
      TOTRI_KERNEL("mesh exhaustive splat", stream,
                   le = cudaLaunchKernelEx(&cfg, kern, sc, sp, lp, org, S, L, out, T, bw, bo,
                                           fast));
      TOTRI_CUDA(le);
      return TOTRI_OK;
    }
    // Registers capped for 5 CTAs per SM (48, no spills): 36.5 ms against
    // 38.1 ms uncapped (58 registers; "mesh.exhaustive.splat.occupancy" = 1)
    // on one 20k-face mesh, 32x32 x 16x16 points, 2,048 bins.
    if (tune::get("mesh.exhaustive.splat.occupancy") != 1) {
      TOTRI_CUDA(tune::ensure_dynamic_smem(
          reinterpret_cast<const void*>(exh_splat_kernel<LT, 5>), smem));
      TOTRI_KERNEL("mesh exhaustive splat", stream,
                   (exh_splat_kernel<LT, 5><<<grid, 256, smem, stream>>>(
                       sc, sp, lp, org, S, L, out, T, bw, bo, fast)));
      return TOTRI_OK;
    }
    TOTRI_CUDA(tune::ensure_dynamic_smem(
        reinterpret_cast<const void*>(exh_splat_kernel<LT>), smem));
    TOTRI_KERNEL("mesh exhaustive splat", stream,
                 exh_splat_kernel<LT><<<grid, 256, smem, stream>>>(sc, sp, lp, org, S, L, out, T,
                                                                   bw, bo, fast));
    return TOTRI_OK;
  }
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(exh_splat_compact_kernel<LT>), smem));
  TOTRI_KERNEL("mesh exhaustive splat", stream,
               exh_splat_compact_kernel<LT><<<grid, 256, smem, stream>>>(
                   sc, sp, lp, org, S, L, out, T, bw, bo, fast));
  return TOTRI_OK;
}

int launch_exhaustive_splat(const Scene& sc, const View3f& sp, const View3f& lp,
                            const Origins& org, int S, int L, float* out, int T, float bw,
                            float bo, cudaStream_t stream) {
  const size_t budget = 200 * 1024;
  const int want = tune::get("mesh.exhaustive.splat.lt");
  if (want > 0) {
    if ((size_t)T * want * 4 > budget)
      return fail(TOTRI_ERR_INVALID_ARGUMENT, "tuned laser tile too large for the bin count");
    switch (want) {
      case 1: return launch_exh_splat<1>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
      case 4: return launch_exh_splat<4>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
      case 8: return launch_exh_splat<8>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
      case 16: return launch_exh_splat<16>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
      case 32: return launch_exh_splat<32>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
      default: return fail(TOTRI_ERR_INVALID_ARGUMENT, "laser tile must be 1, 4, 8, 16 or 32");
    }
  }
  // Built-in choice: the widest laser tile whose histogram stays within 40 KB,
  // so several CTAs share an SM (2048 bins x 64x64 x 16x16, 32 meshes: 4.4 s
  // with 4 lasers per tile, 12.7 s with 16, whose 128 KB tile leaves one CTA
  // per SM).
  const size_t kTileBytes = 40 * 1024;
  if ((size_t)T * 16 * 4 <= kTileBytes && L >= 16)
    return launch_exh_splat<16>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
  if ((size_t)T * 8 * 4 <= kTileBytes && L >= 8)
    return launch_exh_splat<8>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
  if ((size_t)T * 4 * 4 <= budget && L >= 4)
    return launch_exh_splat<4>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
  if ((size_t)T * 4 <= budget)
    return launch_exh_splat<1>(sc, sp, lp, org, S, L, out, T, bw, bo, stream);
  return fail(TOTRI_ERR_UNSUPPORTED, "number of bins too large for the shared-memory tile");
}

// out[c][t] = in[t row + c] for c < n, t < T: a [T][n] block of rows of
// length `row` into bins-last order, through 32 x 32 tiles in shared memory
// (coalesced reads and writes).
__global__ void __launch_bounds__(256) bins_last_kernel(const float* __restrict__ in,
                                                        float* __restrict__ out, int T,
                                                        int64_t row, int64_t n) {
  __shared__ float tile[32][33];
  const int64_t c0 = (int64_t)blockIdx.x * 32;
  const int t0 = blockIdx.y * 32;
  const float* src = in;
  float* dst = out;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int t = t0 + r;
    const int64_t c = c0 + threadIdx.x;
    tile[r][threadIdx.x] = (t < T && c < n) ? src[(int64_t)t * row + c] : 0.f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int64_t c = c0 + r;
    const int t = t0 + threadIdx.x;
    if (t < T && c < n) dst[c * T + t] = tile[threadIdx.x][r];
  }
}

int launch_bins_last(const float* in, float* out, int T, int64_t row, int64_t n,
                     cudaStream_t stream) {
  TOTRI_KERNEL("mesh grad layout", stream,
               bins_last_kernel<<<dim3((unsigned)ceil_div(n, 32), (unsigned)ceil_div(T, 32)),
                                  dim3(32, 8), 0, stream>>>(in, out, T, row, n));
  return TOTRI_OK;
}

int64_t exh_grad_chunk_points(int64_t S, int64_t L, int64_t T) {
  if (S <= 0 || L <= 0 || T <= 0) return 0;
  int64_t c = (int64_t)(kGradChunkBytes / ((size_t)L * (size_t)T * sizeof(float)));
  if (c <= 0) return 0;
  if (c >= S) return S;
  return c >= kFaceSlice ? c / kFaceSlice * kFaceSlice : c;
}

size_t exh_grad_scratch_bytes(int64_t S, int64_t L, int64_t T) {
  const int64_t c = exh_grad_chunk_points(S, L, T);
  return c > 0 ? align_up((size_t)c * (size_t)L * (size_t)T * sizeof(float), 256) : 0;
}

int launch_exhaustive_grad(const Scene& sc, const View3f& sp, const View3f& lp,
                           const Origins& org, int S, int L, const float* tgrad, int T, float bw,
                           float bo, const GradOut& out, void* scratch, size_t scratch_bytes,
                           cudaStream_t stream) {
  const FastBins fast = make_fast_bins(bw, bo, tune::get("mesh.exhaustive.exact") != 1);
  // At most 512 scan points per CTA: a warp walks one face over its slice and
  // then the next face over the same slice, re-reading the same transient_grad
  // rows (slice x L x the chunk's bins), which then stay in L2 (one 20k-face
  // mesh, 1024 x 256 wall points: 92 ms with 512-point slices, 139 ms with
  // 2048).
  constexpr int kMaxSlice = 512;
  const int split =
      tune::grad_split("mesh.exhaustive.grad.split", (int64_t)sc.nch * sc.B, S, kMaxSlice);
  const int64_t slice = ceil_div(S, split);
  // Separable point records (exh_grad_face_kernel) by default;
  // "mesh.exhaustive.grad.mode" = 1 selects per-lane mask tests and 2 the
  // compacted triples (14.7 s against 17.7 s for per-lane mask tests on the
  // 32-mesh batch).
  const int mode = tune::get("mesh.exhaustive.grad.mode");
  if (mode != 1 && mode != 2) {
    // "mesh.exhaustive.grad.faces": faces per CTA (default 8);
    // "mesh.exhaustive.grad.occupancy" = 4: registers capped for 4 CTAs per SM
    // (64, with spills) instead of 3 (80); "mesh.exhaustive.grad.sslice" /
    // ".lchunk": scan points / lasers per CTA.
    const int fpc = tune::get("mesh.exhaustive.grad.faces") > 0
                        ? (int)tune::get("mesh.exhaustive.grad.faces")
                        : kFacesPerCta;
    const bool occ4 = tune::get("mesh.exhaustive.grad.occupancy") == 4;
    const void* fn = occ4 ? reinterpret_cast<const void*>(exh_grad_face_kernel<4>)
                          : reinterpret_cast<const void*>(exh_grad_face_kernel<3>);
    const size_t smem = sizeof(float) * 2 * kRec * kFaceSlice;
    TOTRI_CUDA(tune::ensure_dynamic_smem(fn, smem));
    auto launch = [&](const float* tg, int lchunk, int sslice, int b0, int nb, int sa, int sb,
                      int64_t bstride, int64_t cstep, int64_t bstep) -> int {
      const dim3 grid((unsigned)ceil_div(sc.F, fpc), (unsigned)nb,
                      (unsigned)(ceil_div(sb - sa, sslice) * ceil_div(L, lchunk)));
      if (occ4)
        TOTRI_KERNEL("mesh exhaustive grad", stream,
                     exh_grad_face_kernel<4><<<grid, 256, smem, stream>>>(
                         sc, sp, lp, org, S, L, tg, T, bw, bo, out, fpc, lchunk, sslice, b0, sa,
                         sb, bstride, cstep, bstep));
      else
        TOTRI_KERNEL("mesh exhaustive grad", stream,
                     exh_grad_face_kernel<3><<<grid, 256, smem, stream>>>(
                         sc, sp, lp, org, S, L, tg, T, bw, bo, out, fpc, lchunk, sslice, b0, sa,
                         sb, bstride, cstep, bstep));
      return TOTRI_OK;
    };
    int lchunk = tune::get("mesh.exhaustive.grad.lchunk");
    int sslice = tune::get("mesh.exhaustive.grad.sslice");
    // Bins-last copies. A triple reads a few consecutive bins of its (s, l)
    // column; in the caller's [T, S, L] order they lie S L floats apart, one
    // L2 sector each, read one after another. When the workspace holds the
    // scratch (totri_mesh_exhaustive_grad_scratch), each item's transient_grad
    // is copied, one range of scan points at a time, into [s][l][t] order,
    // where those bins share one or two sectors: one 20k-face mesh, 2,048
    // bins, 16x16 laser points: 333 -> 189 ms at 64x64 scan points, 54.2 ->
    // 51.0 ms at 32x32 (copies included), with whole 256 x 256 tiles.
    // "mesh.exhaustive.grad.layout" = 2 reads transient_grad in place;
    // "mesh.exhaustive.grad.chunk" caps the scan points per copy.
    int64_t cpts = exh_grad_chunk_points(S, L, T);
    const int64_t cap = tune::get("mesh.exhaustive.grad.chunk");
    if (cap > 0) cpts = std::min(cpts, cap);
    if (tune::get("mesh.exhaustive.grad.layout") != 2 && cpts > 0 && scratch &&
        scratch_bytes >= (size_t)cpts * L * T * sizeof(float)) {
      if (lchunk <= 0 || lchunk > kFaceSlice) lchunk = kFaceSlice;
      if (sslice <= 0 || sslice > kFaceSlice) sslice = kFaceSlice;
      sslice = (int)std::min<int64_t>(sslice, cpts);
      float* copy = static_cast<float*>(scratch);
      const int64_t row = (int64_t)S * L;
      for (int b = 0; b < sc.B; ++b)
        for (int64_t sa = 0; sa < S; sa += cpts) {
          const int64_t sb = std::min<int64_t>(S, sa + cpts), n = (sb - sa) * L;
          TOTRI_TRY(launch_bins_last(tgrad + ((int64_t)b * T) * row + sa * L, copy, T, row, n,
                                     stream));
          TOTRI_TRY(launch(copy, lchunk, sslice, b, 1, (int)sa, (int)sb, 0, T, 1));
        }
      return TOTRI_OK;
    }
    // In place: each CTA takes `sslice` scan points and `lchunk` lasers,
    // faces varying fastest over the grid, so the CTAs that run together
    // read the transient_grad rows of one (scan slice, laser chunk). When a
    // bin row of transient_grad (S L floats) reaches 2 MB the per-pair cost
    // grows (one 20k-face mesh, 2,048 bins: 0.23 ms per thousand pairs at
    // 64x64 x 8x8 points, 0.36 at 64x64 x 16x16), and 128 scan points by 32
    // lasers per CTA recover part of it (378 -> 331 ms at 64x64 x 16x16; at
    // 32x32 x 16x16 whole 256 x 256 tiles stay faster, 54.8 against 58.5 ms).
    const bool wide_rows = (int64_t)S * L >= (int64_t)1 << 19;
    if (lchunk <= 0 || lchunk > kFaceSlice) lchunk = wide_rows ? 32 : kFaceSlice;
    if (sslice <= 0 || sslice > kFaceSlice) sslice = wide_rows ? 128 : kFaceSlice;
    return launch(tgrad, lchunk, sslice, 0, sc.B, 0, S, (int64_t)T * S * L, 1, (int64_t)S * L);
  }
  if (mode == 1) {
    const size_t smem = sizeof(uint32_t) * (size_t)(S + L);
    if (smem > 200 * 1024)
      return fail(TOTRI_ERR_UNSUPPORTED, "too many wall points for one tile");
    TOTRI_CUDA(tune::ensure_dynamic_smem(
        reinterpret_cast<const void*>(exh_grad_kernel), smem));
    const dim3 grid((unsigned)sc.nch, (unsigned)sc.B, (unsigned)split);
    TOTRI_KERNEL("mesh exhaustive grad", stream,
                 exh_grad_kernel<<<grid, 256, smem, stream>>>(sc, sp, lp, org, S, L, tgrad, T,
                                                              bw, bo, fast, out));
    return TOTRI_OK;
  }
  const size_t smem = sizeof(uint32_t) * (size_t)(slice + 32 * ceil_div(L, 32));
  if (smem > 180 * 1024) return fail(TOTRI_ERR_UNSUPPORTED, "too many laser points for one tile");
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(exh_grad_compact_kernel), smem));
  // (three CTAs per SM at 80 registers spills and runs 6% slower: 93.5 ms
  // against 87.8 ms on one 20k-face mesh; CTAs of 5 or 6 warps capped at 96
  // registers for 4 or 3 CTAs per SM spill and took 98 and 95 ms against
  // 69 ms for this kernel on that mesh)
  const dim3 grid((unsigned)sc.nch, (unsigned)sc.B, (unsigned)split);
  TOTRI_KERNEL("mesh exhaustive grad", stream,
               exh_grad_compact_kernel<<<grid, 256, smem, stream>>>(
                   sc, sp, lp, org, S, L, tgrad, T, bw, bo, fast, out));
  return TOTRI_OK;
}

}  // namespace mesh
}  // namespace totri
