// Device building blocks shared by the confocal and exhaustive mesh kernels:
// the vertex sort, the tent splat into a shared-memory tile, the tile flush,
// the tent gradient and the per-face gradient scatter.
#pragma once

#include <cmath>

#include "mesh.cuh"

namespace totri {
namespace mesh {

// Sorts the three vertices by FP32 path length with the reference's
// compare-swap sequence (mesh_confocal_forward_optix.cu:86-101). Ties keep the
// original order.
template <class Q>
__device__ __forceinline__ void sort3(Q& q) {
  auto sw = [&](int i, int j) {
    float td = q.d[i]; q.d[i] = q.d[j]; q.d[j] = td;
    fv3 tv = q.v[i]; q.v[i] = q.v[j]; q.v[j] = tv;
    int tp = q.perm[i]; q.perm[i] = q.perm[j]; q.perm[j] = tp;
  };
  if (q.d[0] > q.d[1]) sw(0, 1);
  if (q.d[1] > q.d[2]) sw(1, 2);
  if (q.d[0] > q.d[1]) sw(0, 1);
}

// One wall column of a shared-memory histogram [T][TS].
template <int TS>
struct Hist {
  float* h;
  int sl;
  int T;
  __device__ __forceinline__ bool in(int b) const { return b >= 0 && b < T; }
  __device__ __forceinline__ void add(int b, float v) const { atomicAdd(h + b * TS + sl, v); }
};

// Division for values that decide nothing (tent heights, gradient factors,
// alpha): the hardware reciprocal and one multiply, within 2 ulp, instead of
// the correctly rounded division sequence (alpha's 1/|n| is likewise the
// hardware reciprocal square root). Bins and vertex order never pass through
// it.
__device__ __forceinline__ float vdiv(float a, float b) { return __fdividef(a, b); }

// DrawTrapezoid (mesh_common.h:61-94): integrates the line through
// (ca, ya) - (cb, yb) over each bin it spans (midpoint rule, exact for a line).
template <class H>
__device__ __forceinline__ void splat_segment(const H& h, float ca, int ba, float ya, float cb,
                                              int bb, float yb) {
  if (ba == bb) {
    if (h.in(ba)) h.add(ba, 0.5f * (cb - ca) * (ya + yb));
    return;
  }
  const float slope = vdiv(yb - ya, cb - ca);
  if (h.in(ba)) {
    const float w = (float)(ba + 1) - ca;
    h.add(ba, w * (ya + 0.5f * w * slope));
  }
  const int lo = max(ba + 1, 0), hi = min(bb, h.T);
  for (int i = lo; i < hi; ++i) h.add(i, ya + (((float)i + 0.5f) - ca) * slope);
  if (h.in(bb)) {
    const float w = cb - (float)bb;
    h.add(bb, w * (ya + (0.5f * ((float)bb + cb) - ca) * slope));
  }
}

// The triangle's time profile: a tent of area alpha from c0 to c2 peaking at
// c1 (mesh_confocal_forward_optix.cu:114-129).
template <class H>
__device__ __forceinline__ void splat_tent(const H& h, const float c[3], const int bin[3],
                                           float alpha) {
  if (bin[0] >= h.T || bin[2] < 0) return;
  if (bin[0] == bin[2]) {
    h.add(bin[0], alpha);
    return;
  }
  const float yc = vdiv(2.f * alpha, c[2] - c[0]);
  splat_segment(h, c[0], bin[0], 0.f, c[1], bin[1], yc);
  splat_segment(h, c[1], bin[1], yc, c[2], bin[2], 0.f);
}

// Writes a [T][TS] shared tile to out[t * S + s0 + j] (coalesced; float4 when
// the rows are 16-byte aligned).
template <int TS>
__device__ __forceinline__ void flush_tile(const float* hist, float* __restrict__ out, int T,
                                           int S, int s0) {
  const bool vec = (TS % 4 == 0) && (S % 4 == 0) && (s0 + TS <= S) &&
                   ((reinterpret_cast<uintptr_t>(out) & 15) == 0);
  if (vec) {
    constexpr int Q = TS / 4 > 0 ? TS / 4 : 1;
    const float4* h4 = reinterpret_cast<const float4*>(hist);
    for (int idx = threadIdx.x; idx < T * Q; idx += blockDim.x) {
      const int row = idx / Q, q = idx - row * Q;
      *reinterpret_cast<float4*>(out + (size_t)row * S + s0 + 4 * q) = h4[idx];
    }
  } else {
    for (int idx = threadIdx.x; idx < T * TS; idx += blockDim.x) {
      const int row = idx / TS, j = idx - row * TS;
      if (s0 + j < S) out[(size_t)row * S + s0 + j] = hist[idx];
    }
  }
}

// Bin-relative tent corners for the gradients. A bin coordinate c is some
// hundreds of bins, so its FP32 value is off by up to ~3e-5 bin; the gradient
// weighs each bin's incoming gradient by where the tent's corners sit inside
// the bins, and that offset alone moved the FP32 vertex gradient 1.8e-4
// (rel-L2) from its FP64 value on the 20,480-face scene (the reference's FP32
// kernels carry the same error). The gradient kernels therefore take the
// corners as x = c - bin[0], from path lengths carried as unevaluated sums
// hi + lo of two floats (double-float arithmetic: Knuth's two-sum and the
// fused-multiply-add product error, Dekker 1971), which leaves ~1e-7 bin of
// error; the integer bins stay those of the FP32 decisions.
struct DFloat {
  float hi, lo;
};

// hi + lo == a + b exactly, hi = fl(a + b) (Knuth's branch-free two-sum).
__device__ __forceinline__ DFloat two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return DFloat{s, e};
}

// |v - p| as hi + lo, relative error near 2^-44: the coordinate differences
// and their squares are split exactly, the sum of squares keeps its rounding
// errors, and the square root takes one Newton correction.
__device__ __forceinline__ DFloat len_df(fv3 v, fv3 p) {
  const DFloat dx = two_sum(v.x, -p.x), dy = two_sum(v.y, -p.y), dz = two_sum(v.z, -p.z);
  const float hx = __fmul_rn(dx.hi, dx.hi), hy = __fmul_rn(dy.hi, dy.hi);
  const float hz = __fmul_rn(dz.hi, dz.hi);
  const float lx = __fmaf_rn(dx.hi, dx.hi, -hx), ly = __fmaf_rn(dy.hi, dy.hi, -hy);
  const float lz = __fmaf_rn(dz.hi, dz.hi, -hz);
  const DFloat s1 = two_sum(hx, hy);
  const DFloat s2 = two_sum(s1.hi, hz);
  const float lo = (s1.lo + s2.lo) + (lx + ly + lz) +
                   2.f * (dx.hi * dx.lo + dy.hi * dy.lo + dz.hi * dz.lo);
  if (!(s2.hi > 0.f)) return DFloat{0.f, 0.f};
  const float rs = rsqrtf(s2.hi);
  const float r = s2.hi * rs;
  const float res = __fmaf_rn(-r, r, s2.hi) + lo;
  return DFloat{r, res * 0.5f * rs};
}

// a + b for double-float operands (the low parts are added, not renormalised:
// the result feeds bin_offset only).
__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
  const DFloat s = two_sum(a.hi, b.hi);
  return DFloat{s.hi, s.lo + a.lo + b.lo};
}

// (path - bo) / bw - bin0 for a double-float path length: the quotient's
// remainder comes from one fused multiply-add, and q - bin0 is exact because
// bin0 is the truncated FP32 quotient of the same path.
__device__ __forceinline__ float bin_offset(DFloat path, float bo, float bw, float inv_bw,
                                            int bin0) {
  const DFloat a = two_sum(path.hi, -bo);
  const float q = a.hi * inv_bw;
  const float rem = __fmaf_rn(-q, bw, a.hi) + (a.lo + path.lo);
  return (q - (float)bin0) + rem * inv_bw;
}

// Gradient of the normalised tent (area 1, yc = 2 / (c2 - c0)) against the
// incoming transient gradient g(bin) = col[bin * stride]:
//   part0 = sum_bins g * area_bin
//   part1 = ayc * d(yc) + a0 * d(c0) + a1 * d(c1) + a2 * d(c2)
// which is DrawTrapezoidGrad (mesh_common.h:104-199) for both segments with the
// vector terms factored out of the bin sum.
struct TentGrad {
  float part0, ayc, a0, a1, a2;
};

struct SegSums {
  float ya, yb, ca, cb;
};

// Corners and bins are relative to bin boff (x = c - boff, b = bin - boff):
// bin b reads col[(b + boff) * stride] and exists for 0 <= b + boff < T.
__device__ __forceinline__ void grad_segment(const float* __restrict__ col, int64_t stride, int T,
                                             int boff, float& part0, SegSums& sm, float ca, int ba,
                                             float ya, float cb, int bb, float yb) {
  auto in = [&](int b) { return (unsigned)(b + boff) < (unsigned)T; };
  auto at = [&](int b) { return __ldg(col + (int64_t)(b + boff) * stride); };
  if (ba == bb) {
    if (in(ba)) {
      const float g = at(ba);
      const float half_span = 0.5f * (cb - ca), half_y = 0.5f * (ya + yb);
      part0 += g * half_span * (ya + yb);
      sm.ya += g * half_span;
      sm.yb += g * half_span;
      sm.ca -= g * half_y;
      sm.cb += g * half_y;
    }
    return;
  }
  const float inv = vdiv(1.f, cb - ca);
  const float slope = (yb - ya) * inv;
  const float q = slope * inv;
  if (in(ba)) {
    const float g = at(ba);
    const float base = (float)(ba + 1) - ca;
    const float hb2 = 0.5f * base * base;
    part0 += g * base * (ya + 0.5f * base * slope);
    sm.ya += g * (base - hb2 * inv);
    sm.yb += g * hb2 * inv;
    sm.ca += g * (-ya - base * slope + hb2 * q);
    sm.cb -= g * hb2 * q;
  }
  float sg = 0.f, sgm = 0.f;
  const int lo = max(ba + 1, -boff), hi = min(bb, T - boff);
  for (int i = lo; i < hi; ++i) {
    const float g = at(i);
    sg += g;
    sgm += g * (((float)i + 0.5f) - ca);
  }
  part0 += ya * sg + slope * sgm;
  sm.ya += sg - inv * sgm;
  sm.yb += inv * sgm;
  sm.ca += -slope * sg + q * sgm;
  sm.cb -= q * sgm;
  if (in(bb)) {
    const float g = at(bb);
    const float w = cb - (float)bb;
    const float mid = 0.5f * ((float)bb + cb) - ca;
    part0 += g * w * (ya + mid * slope);
    sm.ya += g * w * (1.f - mid * inv);
    sm.yb += g * w * mid * inv;
    sm.ca += g * w * (-slope + mid * q);
    sm.cb += g * ((ya + mid * slope) + w * (0.5f * slope - mid * q));
  }
}

// x: the corners relative to bin[0] (bin_offset); bins are absolute.
__device__ __forceinline__ void tent_grad(const float* __restrict__ col, int64_t stride, int T,
                                          const float x[3], const int bin[3], TentGrad& out) {
  const float yc = vdiv(2.f, x[2] - x[0]);
  const int b0 = bin[0];
  float part0 = 0.f;
  SegSums s1{0.f, 0.f, 0.f, 0.f}, s2{0.f, 0.f, 0.f, 0.f};
  grad_segment(col, stride, T, b0, part0, s1, x[0], 0, 0.f, x[1], bin[1] - b0, yc);
  grad_segment(col, stride, T, b0, part0, s2, x[1], bin[1] - b0, yc, x[2], bin[2] - b0, 0.f);
  out.part0 = part0;
  out.ayc = s1.yb + s2.ya;
  out.a0 = s1.ca;
  out.a1 = s1.cb + s2.ca;
  out.a2 = s2.cb;
}

// Gradient outputs (strided, may be absent).
struct GradOut {
  float* vg;           // [B, V, 3] or null
  int64_t vsb, vsv, vsc;
  float* mg;           // [B, V, Mg] (channel 0 receives the albedo gradient) or null
  int64_t msb, msv, msc;
  int64_t V;
};

__device__ __forceinline__ float warp_sum(float x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Reduces one face's gradient over the warp and adds it to its vertices
// (mesh_confocal_grad_verts_optix.cu:316-332; 1/3 of the albedo gradient
// goes to channel 0 of each vertex).
// Constants of the filtered fast paths of the pair/triple geometry: 1/bw,
// -bo/bw and the two terms of the bin-coordinate margin (32 u / bw and
// 32 u |bo| / bw + 1e-6, u = 2^-24). A disabled set has infinite margins, so
// every pair takes the exact chain. The tuning keys "mesh.exhaustive.exact"
// and "mesh.confocal.exact" = 1 disable them, for comparison.
struct FastBins {
  float inv_bw, nbo, kc, kb;
};

inline FastBins make_fast_bins(float bw, float bo, bool enabled) {
  const float u = 5.9604645e-8f;
  FastBins f;
  f.inv_bw = 1.f / bw;
  f.nbo = -bo * f.inv_bw;
  const bool ok = enabled && bw > 0.f && std::isfinite(f.inv_bw) && std::isfinite(f.nbo);
  f.kc = ok ? 32.f * u * f.inv_bw : INFINITY;
  f.kb = ok ? 32.f * u * std::fabs(bo) * f.inv_bw + 1e-6f : INFINITY;
  return f;
}

// |a| from the hardware reciprocal square root: within 6.5 u of the exact
// IEEE chain's value (2 ulp rsqrt, one rounding each for the sum and product).
__device__ __forceinline__ float len_fast(fv3 a) {
  const float d2 = fmaf(a.x, a.x, fmaf(a.y, a.y, a.z * a.z));
  return d2 * rsqrtf(d2);
}

// acc[perm[k]] += dv[k] for a permutation perm of {0, 1, 2}, with selects
// instead of a dynamically indexed array (which would live in local memory).
__device__ __forceinline__ void add_permuted(fv3 acc[3], const fv3 dv[3], const int perm[3]) {
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const fv3 v = perm[0] == m ? dv[0] : (perm[1] == m ? dv[1] : dv[2]);
    acc[m] = acc[m] + v;
  }
}

__device__ __forceinline__ void scatter_face_grad(const GradOut& out, int b, float4 s1r, float4 s2r,
                                                  float4 s3r, fv3 acc[3], float accm,
                                                  uint32_t* status) {
  float v[10] = {acc[0].x, acc[0].y, acc[0].z, acc[1].x, acc[1].y,
                 acc[1].z, acc[2].x, acc[2].y, acc[2].z, accm};
#pragma unroll
  for (int i = 0; i < 10; ++i) v[i] = warp_sum(v[i]);
  if ((threadIdx.x & 31) != 0) return;
  const int vi[3] = {__float_as_int(s1r.w), __float_as_int(s2r.w), __float_as_int(s3r.w)};
  for (int q = 0; q < 3; ++q) {
    if (vi[q] < 0 || vi[q] >= out.V) {
      atomicOr(status, kStatusFaceIndexRange);
      continue;
    }
    if (out.vg) {
      float* p = out.vg + b * out.vsb + vi[q] * out.vsv;
      atomicAdd(p, v[3 * q]);
      atomicAdd(p + out.vsc, v[3 * q + 1]);
      atomicAdd(p + 2 * out.vsc, v[3 * q + 2]);
    }
    if (out.mg) atomicAdd(out.mg + b * out.msb + vi[q] * out.msv, (1.f / 3.f) * v[9]);
  }
}

// Host launchers.
int launch_visibility(const Scene& sc, const View3f& pts, int P, int row0, bool brute,
                      cudaStream_t stream);
// Morton order of P wall points into sc.pscratch ([4][B][P]; order in the last quarter).
int launch_point_order(const Scene& sc, const View3f& pts, int P, cudaStream_t stream);
// Wall-to-origin terms of the exhaustive renderer (detector and laser).
struct Origins {
  View3f so, lo;
  int has_so, has_lo;
};

int launch_exhaustive_splat(const Scene& sc, const View3f& sp, const View3f& lp,
                            const Origins& org, int S, int L, float* out, int T, float bw,
                            float bo, cudaStream_t stream);
int launch_exhaustive_grad(const Scene& sc, const View3f& sp, const View3f& lp,
                           const Origins& org, int S, int L, const float* tgrad, int T, float bw,
                           float bo, const GradOut& out, void* scratch, size_t scratch_bytes,
                           cudaStream_t stream);
// out[c][t] = in[t row + c] for c < n, t < T (a block of transient rows into
// bins-last order).
int launch_bins_last(const float* in, float* out, int T, int64_t row, int64_t n,
                     cudaStream_t stream);
// Scan points per bins-last copy of transient_grad (0: none fits), and the
// scratch bytes those copies need.
int64_t exh_grad_chunk_points(int64_t S, int64_t L, int64_t T);
size_t exh_grad_scratch_bytes(int64_t S, int64_t L, int64_t T);

int launch_mask_unsort(const Scene& sc, int P, uint32_t* out, cudaStream_t stream);
int launch_confocal_splat(const Scene& sc, const View3f& sp, const View3f& so, int has_origin,
                          float* transient, int T, int S, float bw, float bo, cudaStream_t stream);
int launch_confocal_grad(const Scene& sc, const View3f& sp, const View3f& so, int has_origin,
                         const float* tgrad, int T, int S, float bw, float bo, const GradOut& out,
                         cudaStream_t stream);

int build_scene(const Scene& sc, const BuildInputs& in, cudaStream_t stream);

}  // namespace mesh
}  // namespace totri
