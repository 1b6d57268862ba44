// Confocal mesh transient rendering: visibility masks, forward splat and the
// vertex / albedo gradient.
//
// Reference: src/render/program/mesh_confocal_forward_optix.cu:18-129 and
// mesh_confocal_grad_verts_optix.cu:18-190 (one OptiX thread per
// (face, scan point) with global atomics into transient[b][bin][s] and into
// verts_grad). Here:
//  * visibility runs once per (scan point, face) into a bit mask
//    [B][P][ceil(F/32)] (one warp per 32 Morton-ordered faces of a point);
//  * the forward gives each CTA a tile of TS scan points and walks all faces,
//    splatting into a shared-memory histogram [T][TS] with shared atomics, and
//    flushes the tile with coalesced float4 stores (no global atomics, no
//    separate zero fill);
//  * the gradient gives each CTA one 32-face mask word and a slice of the scan
//    points (lanes over s, so transient_grad reads are row-coalesced; slices
//    keep every SM busy when there are few faces), keeps
//    the per-face gradient in registers, reduces it across the warp and issues
//    12 atomics per face instead of 9 + 3M per visible pair.
#include <algorithm>

#include "mesh.cuh"
#include "mesh_kernels.cuh"
#include "tune.cuh"

namespace totri {
namespace mesh {

namespace {

// One warp per (wall point, 32 Morton-consecutive faces): the 32 rays share
// their origin and end on a compact patch of the surface, so they walk
// largely the same BVH nodes. kVisRayPostponed lets each lane
// walk alone with its triangle tests postponed until the warp runs them
// together (target_visible_pp; 22.8 ms against 27.0 ms for kVisRay, the plain
// per-lane walk target_visible, on the 20,480-face sphere seen from a 64x64
// wall), kVisPacket walks the 32 rays as one warp packet (packet_visible;
// about twice the node visits there), kVisBrute tests every face; all four
// give the same bits. The patch kernels (one CTA per 32 Morton-consecutive
// wall points and up to 8 chunks of 32 faces) walk per lane after the
// seeded surface walk (kVisPatch, the default), as a packet, over the 4-wide
// tree, or (kVisPatchShaft) gather one candidate list per target with a
// warp-wide walk of the hull of the warp's wall points and the target's hit
// box and test it per lane: 9.7 ms against 8.5 ms for kVisPatch on the
// 20,480-face workload. The lanes of a warp already share the top of their
// walks in SIMT, and near the target a lane's own slab tests prune finer
// than one hull does.
constexpr int kVisBrute = 0;
constexpr int kVisRay = 1;
constexpr int kVisPacket = 2;
constexpr int kVisRayPostponed = 3;
constexpr int kVisPatch = 4;
constexpr int kVisPatchPacket = 5;
constexpr int kVisPatchWide = 6;
constexpr int kVisPatchShaft = 7;
constexpr int kShaftFrontier = 128;
constexpr int kShaftCand = 128;

template <int kMode>
__global__ void __launch_bounds__(256) visibility_kernel(Scene sc, View3f pts, int P, int row0) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t per_b = (int64_t)P * sc.nch;
  if (gw >= per_b * sc.B) return;  // whole warp
  const int b = (int)(gw / per_b);
  const int64_t rem = gw - (int64_t)b * per_b;
  const int p = (int)(rem / sc.nch);
  const int ch = (int)(rem - (int64_t)p * sc.nch);
  const int n = sc.meta[b].n;
  const int k = ch * 32 + lane;
  const fv3 o = mkv(pts.at(b, p, 0), pts.at(b, p, 1), pts.at(b, p, 2));
  bool vis = false;
  if (kMode == kVisPacket) {
    if (ch * 32 < n) {  // warp-uniform
      Target tg{};
      tg.k = k;
      if (k < n) tg = load_target(sc, b, k);
      vis = packet_visible(sc, b, n, k < n, tg, o, sc.status);
    }
  } else if (kMode == kVisRayPostponed) {
    int seed = -1;
    if (k < n) vis = target_visible_pp(sc, b, n, load_target(sc, b, k), o, sc.status, seed,
                                       kSeedOff, 0);
  } else if (k < n) {
    int cache = -1;
    vis = target_visible<kMode == kVisBrute>(sc, b, n, load_target(sc, b, k), o, cache,
                                             sc.status);
  }
  const uint32_t word = __ballot_sync(0xffffffffu, vis);
  if (lane == 0) sc.mask[((size_t)b * sc.P + row0 + p) * sc.nch + ch] = word;
}

// One CTA per (block of 32 wall points in Morton order, run of `chunks`
// 32-face chunks): each warp takes one face of the run at a time and its 32
// lanes cast the rays from the 32 points, which lie on a compact patch of
// the wall and end on the same centroid, so the lanes walk nearly the same BVH
// nodes (lockstep model on the 20,480-face sphere: 12% fewer warp iterations
// and 8.3 -> 5.7 distinct nodes per iteration against point-major warps;
// measured 15.3 ms against 22.6 ms for point-major warps with the same
// postponed-leaf walk). The eight warps of a CTA work on neighbouring faces
// from the same points, so they share their BVH nodes in L1 (a variant
// without the CTA, one warp per 32 x 32 block, took 23.2 ms).
//
// With the binary walk (kWalk 0) each point keeps a seed in shared memory: the
// last occluder any warp of the CTA found for it. Faces of neighbouring Morton
// positions are close on the surface, and so are the faces that hide them from
// one wall point, so a short surface walk from the seed (surface_walk) settles
// most hidden targets without a BVH walk. A CTA starts from the seeds that
// earlier CTAs of the same points left in global memory (the first quarter of
// the point scratch, -1 after the point sort) and leaves its own there. Seeds
// are read and written without synchronisation, as any face is a valid (if
// slower) start. The bits of every chunk are transposed in shared memory into
// one mask word per point and chunk. This is the default visibility kernel.
constexpr int kMaxPatchChunks = 16;

// kWalk 0: target_visible_pp, 1: packet_visible, 2: target_visible_pp4, 3: shaft
// search, 4: target_visible_pp's prefix and a 4-wide BVH search
// (bvh_occluded_wide); kOcc: CTAs per SM that the register allocation must allow.
template <int kWalk, int kOcc = 1>
__global__ void __launch_bounds__(256, kOcc) visibility_patch_kernel(Scene sc, View3f pts, int P,
                                                               int row0, int chunks,
                                                               int seed_mode, int seed_steps,
                                                               int shaft_cap) {
  __shared__ uint32_t bits[kMaxPatchChunks][32];  // [chunk][face j]: visible from point lane
  __shared__ int seeds[32];
  __shared__ int next_face;
  // per warp: two frontiers and the candidate list of the shaft search
  __shared__ int shaft_buf[kWalk == 3 ? 8 * (2 * kShaftFrontier + kShaftCand) : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = blockIdx.z;
  const int ch0 = blockIdx.y * chunks;
  const int i = blockIdx.x * 32 + lane;  // position in Morton order
  const int n = sc.meta[b].n;
  const bool okp = i < P;
  const uint32_t* order = sc.pscratch + 3 * (size_t)sc.B * P + (size_t)b * P;
  int p = okp ? (int)order[i] : 0;
  if (!TOTRI_INDEX_OK((unsigned)p < (unsigned)P, sc.status)) p = 0;
  const fv3 o = okp ? mkv(pts.at(b, p, 0), pts.at(b, p, 1), pts.at(b, p, 2)) : mkv(0.f, 0.f, 0.f);
  volatile int* vseeds = seeds;
  volatile int* gseeds = reinterpret_cast<int*>(sc.pscratch) + (size_t)b * P;
  if (threadIdx.x < 32) seeds[lane] = okp ? gseeds[i] : -1;
  if (threadIdx.x == 0) next_face = 0;
  __syncthreads();
  const int nc = min(chunks, sc.nch - ch0);
  // The warp's wall points bound every ray's start (shaft search only).
  float plo[3] = {0.f, 0.f, 0.f}, phi[3] = {0.f, 0.f, 0.f}, pad = 0.f;
  if (kWalk == 3) {
    const float oc[3] = {o.x, o.y, o.z};
    float mag = 0.f;
    for (int a = 0; a < 3; ++a) {
      float lo = okp ? oc[a] : INFINITY, hi = okp ? oc[a] : -INFINITY;
      for (int off = 16; off; off >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, off));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, off));
      }
      plo[a] = lo;
      phi[a] = hi;
      mag = fmaxf(mag, fmaxf(fabsf(lo), fabsf(hi)));
    }
    // the hit-point margin, plus room for the rounding of far wall points
    pad = sc.meta[b].delta + ldexpf(isfinite(mag) ? mag : 0.f, -14);
    for (int a = 0; a < 3; ++a) {
      plo[a] -= pad;
      phi[a] += pad;
    }
  }
  // Faces are handed out one at a time from a shared counter, in Morton
  // order: a hidden face settled by a short surface walk costs a fraction of a
  // visible one, so fixed shares would leave warps idle at the final barrier.
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&next_face, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= nc * 32) break;
    const int c = t >> 5, j = t & 31;
    const int k = (ch0 + c) * 32 + j;
    bool vis = false;
    if (k < n) {  // warp-uniform
      const Target tg = load_target(sc, b, k);
      if (kWalk == 1) {
        vis = packet_visible(sc, b, n, okp, tg, o, sc.status);
      } else if (kWalk == 2) {
        vis = okp && target_visible_pp4(sc, b, n, tg, o, sc.status);
      } else if (kWalk == 3) {
        int seed = okp ? vseeds[lane] : -1;
        const int s0 = seed;
        fv3 dir = mkv(0.f, 0.f, 0.f);
        float tmax = 0.f, tf = 0.f;
        int need = 0;
        if (okp)
          need = query_prefix(sc, b, n, tg, o, seed, seed_mode, seed_steps, dir, tmax, tf, vis);
        if (__any_sync(0xffffffffu, need)) {
          // every ray ends at its accepted hit on the target, which tri_hit
          // keeps inside the target's hit box (not near the centroid: for a
          // grazing target t is ill-conditioned along the ray)
          const float clo[3] = {tg.a2.y - pad, tg.a2.z - pad, tg.a2.w - pad};
          const float chi[3] = {tg.a3.x + pad, tg.a3.y + pad, tg.a3.z + pad};
          const Shaft h = make_shaft(plo, phi, clo, chi);
          int* wb = shaft_buf + warp * (2 * kShaftFrontier + kShaftCand);
          int* cand = wb + 2 * kShaftFrontier;
          const int ncand = shaft_candidates<kShaftFrontier, kShaftCand>(
              sc, b, n, tg.k, h, wb, wb + kShaftFrontier, cand, lane, shaft_cap);
          if (need) {
            bool occ = false;
            if (ncand >= 0) {
              for (int j = 0; j < ncand; ++j) {
                const int kk = cand[j];
                if ((unsigned)kk >= (unsigned)n) {
                  atomicOr(sc.status, kStatusTraversalCap);
                  continue;
                }
                const float4* q = tri_at(sc, b, kk);
                const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2),
                             q3 = __ldg(q + 3);
                float tq;
                if (tri_hit(q0, q1, q2, q3, o, dir, tmax, tq) &&
                    (tq < tf || (tq == tf && __float_as_int(q3.w) < tg.f))) {
                  occ = true;
                  seed = kk;
                  break;
                }
              }
            } else {
              occ = bvh_occluded(sc, b, n, tg.k, tg.f, o, dir, tmax, tf, sc.status, seed);
            }
            vis = !occ;
          }
        }
        if (okp && seed != s0) vseeds[lane] = seed;
      } else if (kWalk == 4) {
        if (okp) {
          const int s0 = vseeds[lane];
          int seed = s0;
          fv3 dir;
          float tmax, tf;
          if (query_prefix(sc, b, n, tg, o, seed, seed_mode, seed_steps, dir, tmax, tf, vis))
            vis = !bvh_occluded_wide(sc, b, n, tg.k, tg.f, o, dir, tmax, tf, sc.status, seed);
          if (seed != s0) vseeds[lane] = seed;
        }
      } else if (okp) {
        const int s0 = vseeds[lane];
        int seed = s0;
        vis = target_visible_pp(sc, b, n, tg, o, sc.status, seed, seed_mode, seed_steps);
        if (seed != s0) vseeds[lane] = seed;
      }
    }
    const uint32_t w = __ballot_sync(0xffffffffu, vis);
    if (lane == 0) bits[c][j] = w;
  }
  __syncthreads();
  if (threadIdx.x < 32 && okp && (kWalk == 0 || kWalk == 3 || kWalk == 4)) gseeds[i] = seeds[lane];
  for (int c = warp; c < nc; c += 8) {
    if (!okp) continue;
    uint32_t word = 0u;
#pragma unroll
    for (int j = 0; j < 32; ++j) word |= ((bits[c][j] >> lane) & 1u) << j;
    sc.mask[((size_t)b * sc.P + row0 + p) * sc.nch + ch0 + c] = word;
  }
}

// visibility_patch_kernel<0> with the BVH searches compacted. After a face's
// prefix (the target's own hit and, for faces seen from behind, the surface
// walk) only some lanes are still undecided: most hidden targets are settled
// by the walk, so a face seen from behind typically leaves a few rays, and
// the warp used to run their BVH walks with the other lanes idle. Here each
// undecided ray goes into its warp's queue in shared memory (its direction,
// limits and target), and the warp walks the BVH only for full batches of 32
// queued rays, one per lane, drawn from the faces it has taken so far (and the
// last partial batch at the end). A face's mask word is written when its
// prefix ends, with the queued rays counted visible, and a walk that finds an
// occluder clears its bit. The decisions per ray are those of
// target_visible_pp (same prefix, same search), so the masks are unchanged.
constexpr int kVisQueue = 64;  // entries per warp: < 32 left over + 32 added

template <int kOcc>
__global__ void __launch_bounds__(256, kOcc) visibility_queue_kernel(Scene sc, View3f pts, int P,
                                                                    int row0, int chunks,
                                                                    int seed_mode,
                                                                    int seed_steps) {
  __shared__ uint32_t bits[kMaxPatchChunks][32];
  __shared__ int seeds[32];
  __shared__ int next_face;
  __shared__ float opts[3][32];  // the block's wall points (ray origins)
  // per warp: (dir.xyz, tf) and (tmax, target k << 5 | point lane, face index, -)
  __shared__ float4 queue[8][kVisQueue][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = blockIdx.z;
  const int ch0 = blockIdx.y * chunks;
  const int i = blockIdx.x * 32 + lane;  // position in Morton order
  const int n = sc.meta[b].n;
  const bool okp = i < P;
  const uint32_t* order = sc.pscratch + 3 * (size_t)sc.B * P + (size_t)b * P;
  int p = okp ? (int)order[i] : 0;
  if (!TOTRI_INDEX_OK((unsigned)p < (unsigned)P, sc.status)) p = 0;
  const fv3 o = okp ? mkv(pts.at(b, p, 0), pts.at(b, p, 1), pts.at(b, p, 2)) : mkv(0.f, 0.f, 0.f);
  volatile int* vseeds = seeds;
  volatile int* gseeds = reinterpret_cast<int*>(sc.pscratch) + (size_t)b * P;
  if (threadIdx.x < 32) {
    seeds[lane] = okp ? gseeds[i] : -1;
    opts[0][lane] = o.x;
    opts[1][lane] = o.y;
    opts[2][lane] = o.z;
  }
  if (threadIdx.x == 0) next_face = 0;
  __syncthreads();
  const int nc = min(chunks, sc.nch - ch0);
  const uint32_t below = (1u << lane) - 1u;
  float4(*q)[2] = queue[warp];
  int cnt = 0;  // queued rays (warp-uniform)
  // Walks queue entries [0, m), entry `lane` on lane `lane`.
  auto walk = [&](int m) {
    if (lane < m) {
      const float4 a = q[lane][0], e = q[lane][1];
      const int code = __float_as_int(e.y);
      const int k = code >> 5, pl = code & 31;
      const fv3 oo = mkv(opts[0][pl], opts[1][pl], opts[2][pl]);
      int seed = -1;
      if (bvh_occluded(sc, b, n, k, __float_as_int(e.z), oo, mkv(a.x, a.y, a.z), e.x, a.w,
                       sc.status, seed)) {
        const int t = k - ch0 * 32;
        atomicAnd(&bits[t >> 5][t & 31], ~(1u << pl));
        vseeds[pl] = seed;
      }
    }
  };
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&next_face, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= nc * 32) break;
    const int c = t >> 5, j = t & 31;
    const int k = (ch0 + c) * 32 + j;
    if (k >= n) {  // warp-uniform
      if (lane == 0) bits[c][j] = 0u;
      continue;
    }
    bool vis = false;
    int need = 0;
    const Target tg = load_target(sc, b, k);
    fv3 dir = mkv(0.f, 0.f, 0.f);
    float tmax = 0.f, tf = 0.f;
    if (okp) {
      const int s0 = vseeds[lane];
      int seed = s0;
      need = query_prefix(sc, b, n, tg, o, seed, seed_mode, seed_steps, dir, tmax, tf, vis);
      if (seed != s0) vseeds[lane] = seed;
    }
    const uint32_t nm = __ballot_sync(0xffffffffu, need);
    const uint32_t w = __ballot_sync(0xffffffffu, vis || need);
    if (lane == 0) bits[c][j] = w;
    if (need) {
      const int at = cnt + __popc(nm & below);
      q[at][0] = make_float4(dir.x, dir.y, dir.z, tf);
      q[at][1] = make_float4(tmax, __int_as_float((k << 5) | lane), __int_as_float(tg.f), 0.f);
    }
    cnt += __popc(nm);
    if (cnt >= 32) {
      __syncwarp();
      walk(32);
      __syncwarp();
      if (lane < cnt - 32) {
        q[lane][0] = q[32 + lane][0];
        q[lane][1] = q[32 + lane][1];
      }
      cnt -= 32;
      __syncwarp();
    }
  }
  __syncwarp();
  walk(cnt);
  __syncthreads();
  if (threadIdx.x < 32 && okp) gseeds[i] = seeds[lane];
  for (int c = warp; c < nc; c += 8) {
    if (!okp) continue;
    uint32_t word = 0u;
#pragma unroll
    for (int j = 0; j < 32; ++j) word |= ((bits[c][j] >> lane) & 1u) << j;
    sc.mask[((size_t)b * sc.P + row0 + p) * sc.nch + ch0 + c] = word;
  }
}

// Per-pair confocal geometry: FP32 decisions exactly as the oracle takes them.
struct ConfocalPair {
  fv3 v[3];
  int perm[3];
  float d[3];
  float c[3];
  int bin[3];
};

__device__ __forceinline__ void confocal_pair(const float4 s0, const float4 s1, const float4 s2,
                                              fv3 sp, float od, float bw, float bo,
                                              ConfocalPair& q) {
  q.v[0] = mkv(s0.x, s0.y, s0.z);
  q.v[1] = mkv(s1.x, s1.y, s1.z);
  q.v[2] = mkv(s2.x, s2.y, s2.z);
  for (int k = 0; k < 3; ++k) {
    q.perm[k] = k;
    q.d[k] = xlen(xsub3(q.v[k], sp));
  }
  sort3(q);
  for (int k = 0; k < 3; ++k) {
    q.c[k] = xdiv(xsub(xadd(xmul(2.f, q.d[k]), od), bo), bw);
    q.bin[k] = bin_of(q.c[k]);
  }
}

// confocal_pair with a filtered fast path (FastBins): lengths from the
// hardware reciprocal square root, bin coordinates from one fused
// multiply-add. Each fast length is within 8 u d of the exact chain's
// (u = 2^-24), so three lengths separated by more than 16 u max(d) sort as the
// exact ones do, and a bin coordinate farther than
// 32 u (2d + od + |bo|)/bw + 8 u |c| + 1e-6 from an integer truncates to the
// exact bin. Only then are the fast values kept; otherwise (ties, NaN, huge
// coordinates) the exact confocal_pair runs. Bins and vertex order are always
// those of the exact chain; values differ from it by a few ulps. Used by the
// forward splat only: the gradient's FP32 cancellation amplifies those ulps
// (2.8e-4 rel-L2 on the 20,480-face vertex gradient), so the gradient keeps
// the exact chain.
__device__ __forceinline__ void confocal_pair_filtered(const float4 s0, const float4 s1,
                                                       const float4 s2, fv3 sp, float od,
                                                       float bw, float bo, const FastBins& fb,
                                                       ConfocalPair& q) {
  q.v[0] = mkv(s0.x, s0.y, s0.z);
  q.v[1] = mkv(s1.x, s1.y, s1.z);
  q.v[2] = mkv(s2.x, s2.y, s2.z);
  for (int k = 0; k < 3; ++k) {
    q.perm[k] = k;
    q.d[k] = len_fast(q.v[k] - sp);
  }
  sort3(q);
  const float u = 5.9604645e-8f;
  bool ok = q.d[1] - q.d[0] > 16.f * u * q.d[2] && q.d[2] - q.d[1] > 16.f * u * q.d[2];
  for (int k = 0; k < 3; ++k) {
    const float x = fmaf(2.f, q.d[k], od);
    const float c = fmaf(x, fb.inv_bw, fb.nbo);
    const float m = fmaf(fb.kc, x, fb.kb) + 8.f * u * fabsf(c);
    ok = ok && fabsf(c - rintf(c)) > m && fabsf(c) < 1.0e9f;
    q.c[k] = c;
    q.bin[k] = __float2int_rz(c);
  }
  if (!ok) confocal_pair(s0, s1, s2, sp, od, bw, bo, q);
}

// alpha of AlphaConfocal (mesh_common.h:394-413):
// 100 rho (n_w.r)^2 (n.r)^2 / (|n| |r|^8), n_w = (0,0,1), r = c - s.
__device__ __forceinline__ float alpha_confocal(const ConfocalPair& q, fv3 c, fv3 sp,
                                                float rho) {
  const fv3 n = cross(q.v[1] - q.v[0], q.v[2] - q.v[0]);
  const fv3 r = c - sp;
  if (!(r.z > 0.f)) return 0.f;
  const float nr = dot(n, r), rr = dot(r, r), nn = dot(n, n);
  const float rr2 = rr * rr;
  return vdiv(100.f * rho * (r.z * r.z) * (nr * nr) * rsqrtf(nn), rr2 * rr2);
}

template <int TS>
__global__ void __launch_bounds__(256) splat_kernel(Scene sc, View3f sp, View3f so, int has_origin,
                                                    float* __restrict__ transient, int T, int S,
                                                    float bw, float bo, FastBins fb) {
  extern __shared__ float hist[];  // [T][TS]
  const int b = blockIdx.y;
  const int s0 = blockIdx.x * TS;
  for (int i = threadIdx.x; i < T * TS; i += blockDim.x) hist[i] = 0.f;
  __syncthreads();
  const int n = sc.meta[b].n;
  const int sl = threadIdx.x % TS;
  const int s = s0 + sl;
  if (s < S) {
    const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
    float od = 0.f;
    if (has_origin) od = xmul(2.f, xlen(xsub3(p, mkv(so.at(b, s, 0), so.at(b, s, 1), so.at(b, s, 2)))));
    const uint32_t* mrow = sc.mask + ((size_t)b * sc.P + s) * sc.nch;
    const float4* shade = sc.shade + (size_t)b * sc.F * 4;
    Hist<TS> h{hist, sl, T};
    for (int k = threadIdx.x / TS; k < n; k += blockDim.x / TS) {
      if (!((__ldg(mrow + (k >> 5)) >> (k & 31)) & 1u)) continue;
      const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
      const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
      ConfocalPair q;
      confocal_pair_filtered(s0r, s1r, s2r, p, od, bw, bo, fb, q);
      const float alpha = alpha_confocal(q, mkv(s3r.x, s3r.y, s3r.z), p, s0r.w);
      if (!(alpha > 0.f)) continue;
      splat_tent(h, q.c, q.bin, alpha);
    }
  }
  __syncthreads();
  flush_tile<TS>(hist, transient + (size_t)b * T * S, T, S, s0);
}

// splat_kernel with the visible pairs compacted first: each warp walks
// 32-face chunks (lane = face), gathers each face's visibility over the TS
// scan points of the tile, queues the visible (face, point) pairs in shared
// memory and evaluates them 32 at a time, one per lane, instead of leaving the
// lanes of occluded pairs idle. A face hands out its points starting at a
// lane-dependent offset, so the 32 pairs of a batch fall on different
// histogram columns and their shared atomics seldom collide.
template <int TS>
__global__ void __launch_bounds__(256, 2) splat_compact_kernel(Scene sc, View3f sp, View3f so,
                                                            int has_origin,
                                                            float* __restrict__ transient, int T,
                                                            int S, float bw, float bo,
                                                            FastBins fb) {
  extern __shared__ float hist[];  // [T][TS]
  __shared__ float pts[TS][4];     // scan point, 2 |scan - origin|
  __shared__ int queue[8][64];
  const int b = blockIdx.y;
  const int s0 = blockIdx.x * TS;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < T * TS; i += blockDim.x) hist[i] = 0.f;
  if (threadIdx.x < TS && s0 + (int)threadIdx.x < S) {
    const int s = s0 + threadIdx.x;
    const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
    pts[threadIdx.x][0] = p.x;
    pts[threadIdx.x][1] = p.y;
    pts[threadIdx.x][2] = p.z;
    pts[threadIdx.x][3] =
        has_origin ? xmul(2.f, xlen(xsub3(p, mkv(so.at(b, s, 0), so.at(b, s, 1), so.at(b, s, 2)))))
                   : 0.f;
  }
  __syncthreads();
  const int n = sc.meta[b].n;
  const int nchu = (n + 31) >> 5;
  const int ts = min(TS, S - s0);
  const uint32_t* m0 = sc.mask + ((size_t)b * sc.P + s0) * sc.nch;
  const float4* shade = sc.shade + (size_t)b * sc.F * 4;
  const uint32_t below = (1u << lane) - 1u;
  int* qw = queue[warp];
  int cnt = 0;  // warp-uniform
  auto run = [&](int e) {
    const int k = e >> 4, sl = e & 15;
    const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
    const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
    const fv3 p = mkv(pts[sl][0], pts[sl][1], pts[sl][2]);
    ConfocalPair q;
    confocal_pair_filtered(s0r, s1r, s2r, p, pts[sl][3], bw, bo, fb, q);
    const float alpha = alpha_confocal(q, mkv(s3r.x, s3r.y, s3r.z), p, s0r.w);
    if (!(alpha > 0.f)) return;
    const Hist<TS> h{hist, sl, T};
    splat_tent(h, q.c, q.bin, alpha);
  };
  const int rot = lane & (TS - 1);
  for (int ch = warp; ch < nchu; ch += 8) {
    const uint32_t w = lane < ts ? __ldg(m0 + (size_t)lane * sc.nch + ch) : 0u;
    // vm: this lane's face, bit sl = visible from scan point s0 + sl; faces
    // at or past n never count, whatever the mask words hold there.
    uint32_t vm = 0u;
    for (int sl = 0; sl < ts; ++sl) vm |= ((__shfl_sync(0xffffffffu, w, sl) >> lane) & 1u) << sl;
    if (ch * 32 + lane >= n) vm = 0u;
    while (__any_sync(0xffffffffu, vm != 0u)) {
      const bool has = vm != 0u;
      int sl = 0;
      if (has) {  // next visible point, counting from this lane's offset
        const uint32_t r = ((vm >> rot) | (vm << ((TS - rot) & 31))) & ((1u << TS) - 1u);
        sl = (__ffs(r) - 1 + rot) & (TS - 1);
        vm &= ~(1u << sl);
      }
      const uint32_t take = __ballot_sync(0xffffffffu, has);
      if (has) qw[cnt + __popc(take & below)] = ((ch * 32 + lane) << 4) | sl;
      cnt += __popc(take);  // below 64: at most 31 queued before, 32 added
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
  flush_tile<TS>(hist, transient + (size_t)b * T * S, T, S, s0);
}

// The tent corners of a pair relative to its first bin, from double-float
// path lengths 2 |v_k - p| + od (bin_offset); od is the double-float origin
// term 2 |p - o| (zero without origins).
__device__ __forceinline__ void confocal_corners(const ConfocalPair& q, fv3 p, DFloat od, float bw,
                                                 float inv_bw, float bo, float x[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const DFloat d = len_df(q.v[k], p);
    x[k] = bin_offset(df_add(DFloat{2.f * d.hi, 2.f * d.lo}, od), bo, bw, inv_bw, q.bin[0]);
  }
}

// Gradient of one visible pair with respect to the three (sorted) vertices and
// the albedo, following mesh_confocal_grad_verts_optix.cu:248-314 and
// AlphaConfocalGradVerts (mesh_common.h:429-463), with the tent corners x taken
// relative to bin[0] (confocal_corners). Returns false when the pair
// contributes nothing.
__device__ __forceinline__ bool pair_grad_confocal(const ConfocalPair& q, const float x[3], fv3 c,
                                                   fv3 p, float rho, float bw,
                                                   const float* __restrict__ tg_col, int T, int S,
                                                   fv3 dv[3], float& dmat) {
  const float alpha = alpha_confocal(q, c, p, rho);
  if (!(alpha > 0.f)) return false;
  if (q.bin[0] >= T || q.bin[2] < 0) return false;
  const fv3 e1 = q.v[1] - q.v[0], e2 = q.v[2] - q.v[0];
  const fv3 n = cross(e1, e2);
  const fv3 r = c - p;
  // d log(alpha) / d v_k = J_n^T (kn n + knr r) + kr r + (knr/3) n + kw n_w
  const float kn = vdiv(-1.f, dot(n, n));
  const float kr = vdiv(-8.f, 3.f * dot(r, r));
  const float kw = vdiv(2.f, 3.f * r.z);
  const float knr = vdiv(2.f, dot(n, r));
  const fv3 w = kn * n + knr * r;
  const fv3 g1 = cross(e2, w), g2 = cross(w, e1);
  const fv3 common = kr * r + (knr * (1.f / 3.f)) * n + mkv(0.f, 0.f, kw);
  const fv3 da0 = alpha * (common - g1 - g2);
  const fv3 da1 = alpha * (common + g1);
  const fv3 da2 = alpha * (common + g2);
  const float dadm = vdiv(alpha, rho);
  if (q.bin[0] == q.bin[2]) {
    const float g = __ldg(tg_col + (size_t)q.bin[0] * S);
    dv[0] = g * da0;
    dv[1] = g * da1;
    dv[2] = g * da2;
    dmat = g * dadm;
    return true;
  }
  TentGrad tgr;
  tent_grad(tg_col, S, T, x, q.bin, tgr);
  // part1 = Ayc * dyc + A0 * dc0 + A1 * dc1 + A2 * dc2 (see TentGrad)
  const float span = x[2] - x[0];
  const float kk = vdiv(-4.f, bw * span * span);
  const fv3 r0 = q.v[0] - p, r1 = q.v[1] - p, r2 = q.v[2] - p;
  const fv3 dc0 = vdiv(2.f, bw * q.d[0]) * r0;
  const fv3 dc1 = vdiv(2.f, bw * q.d[1]) * r1;
  const fv3 dc2 = vdiv(2.f, bw * q.d[2]) * r2;
  const fv3 dyc0 = vdiv(kk, -q.d[0]) * r0;
  const fv3 dyc2 = vdiv(kk, q.d[2]) * r2;
  const fv3 p1_0 = tgr.ayc * dyc0 + tgr.a0 * dc0;
  const fv3 p1_1 = tgr.a1 * dc1;
  const fv3 p1_2 = tgr.ayc * dyc2 + tgr.a2 * dc2;
  dv[0] = tgr.part0 * da0 + alpha * p1_0;
  dv[1] = tgr.part0 * da1 + alpha * p1_1;
  dv[2] = tgr.part0 * da2 + alpha * p1_2;
  dmat = dadm * tgr.part0;
  return true;
}

// Three CTAs per SM (80 registers, a few spills): 1.46 ms against 1.51 ms at
// 128 registers and two CTAs on the differentiable step.
__global__ void __launch_bounds__(256, 3) grad_kernel(Scene sc, View3f sp, View3f so, int has_origin,
                                                   const float* __restrict__ tgrad, int T, int S,
                                                   float bw, float bo, GradOut out) {
  extern __shared__ uint32_t mcol[];  // [slice] mask words of this 32-face chunk
  __shared__ int gq[8][64];           // per-warp queue of visible scan points
  const int b = blockIdx.y;
  const int ch = blockIdx.x;
  const int n = sc.meta[b].n;
  if (ch * 32 >= n) return;
  // scan-point slice [s0, s1) of this CTA (gridDim.z slices)
  const int s0 = (int)((int64_t)S * blockIdx.z / gridDim.z);
  const int s1 = (int)((int64_t)S * (blockIdx.z + 1) / gridDim.z);
  for (int s = s0 + threadIdx.x; s < s1; s += blockDim.x)
    mcol[s - s0] = sc.mask[((size_t)b * sc.P + s) * sc.nch + ch];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const float* tgb = tgrad + (size_t)b * T * S;
  const float4* shade = sc.shade + (size_t)b * sc.F * 4;
  const float inv_bw = __frcp_rn(bw);
  for (int j = warp; j < 32; j += nw) {
    const int k = ch * 32 + j;
    if (k >= n) break;
    const float4 s0r = __ldg(shade + 4 * k), s1r = __ldg(shade + 4 * k + 1);
    const float4 s2r = __ldg(shade + 4 * k + 2), s3r = __ldg(shade + 4 * k + 3);
    const fv3 c = mkv(s3r.x, s3r.y, s3r.z);
    fv3 acc[3] = {mkv(0.f, 0.f, 0.f), mkv(0.f, 0.f, 0.f), mkv(0.f, 0.f, 0.f)};
    float accm = 0.f;
    auto run = [&](int s) {
      const fv3 p = mkv(sp.at(b, s, 0), sp.at(b, s, 1), sp.at(b, s, 2));
      float od = 0.f;
      DFloat odf{0.f, 0.f};
      if (has_origin) {
        const fv3 o = mkv(so.at(b, s, 0), so.at(b, s, 1), so.at(b, s, 2));
        od = xmul(2.f, xlen(xsub3(p, o)));
        const DFloat d = len_df(p, o);
        odf = DFloat{2.f * d.hi, 2.f * d.lo};
      }
      ConfocalPair q;
      confocal_pair(s0r, s1r, s2r, p, od, bw, bo, q);
      if (q.bin[0] >= T || q.bin[2] < 0) return;
      float x[3];
      confocal_corners(q, p, odf, bw, inv_bw, bo, x);
      fv3 dv[3];
      float dm;
      if (!pair_grad_confocal(q, x, c, p, s0r.w, bw, tgb + s, T, S, dv, dm)) return;
      add_permuted(acc, dv, q.perm);
      accm += dm;
    };
    // visible scan points are queued and evaluated 32 at a time, one per lane
    int* qw = gq[warp];
    int cnt = 0;  // warp-uniform
    for (int base = s0; base < s1; base += 32) {
      const int s = base + lane;
      const bool v = s < s1 && ((mcol[s - s0] >> j) & 1u);
      const uint32_t bits = __ballot_sync(0xffffffffu, v);
      if (v) qw[cnt + __popc(bits & ((1u << lane) - 1u))] = s;
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
    __syncwarp();
    if (lane < cnt) run(qw[lane]);
    __syncwarp();
    scatter_face_grad(out, b, s1r, s2r, s3r, acc, accm, sc.status);
  }
}

// Re-indexes mask bits from Morton order (bit k) to input face order (bit f).
__global__ void mask_unsort_kernel(Scene sc, int P, uint32_t* out) {
  const int b = blockIdx.y;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int n = sc.meta[b].n;
  if (i >= (int64_t)P * n) return;
  const int p = (int)(i / n), k = (int)(i - (int64_t)p * n);
  const uint32_t w = sc.mask[((size_t)b * sc.P + p) * sc.nch + (k >> 5)];
  if (!((w >> (k & 31)) & 1u)) return;
  const int f = __float_as_int(tri_at(sc, b, k)[3].w);
  if (!TOTRI_INDEX_OK((unsigned)f < (unsigned)sc.F, sc.status)) return;
  atomicOr(out + ((size_t)b * P + p) * sc.nch + (f >> 5), 1u << (f & 31));
}

}  // namespace

int launch_mask_unsort(const Scene& sc, int P, uint32_t* out, cudaStream_t stream) {
  TOTRI_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t) * (size_t)sc.B * P * sc.nch, stream));
  const dim3 grid((unsigned)ceil_div((int64_t)P * sc.F, 256), (unsigned)sc.B);
  TOTRI_KERNEL("mesh mask unsort", stream, mask_unsort_kernel<<<grid, 256, 0, stream>>>(sc, P, out));
  return TOTRI_OK;
}

int launch_visibility(const Scene& sc, const View3f& pts, int P, int row0, bool brute,
                      cudaStream_t stream) {
  const int64_t units = (int64_t)sc.B * P * sc.nch;
  if (units == 0) return TOTRI_OK;
  const unsigned blocks = (unsigned)ceil_div(units * 32, 256);
  if (brute) {
    TOTRI_KERNEL("mesh visibility brute", stream,
                 visibility_kernel<kVisBrute><<<blocks, 256, 0, stream>>>(sc, pts, P, row0));
  } else if (tune::get("mesh.visibility.mode") == kVisRay) {
    TOTRI_KERNEL("mesh visibility", stream,
                 visibility_kernel<kVisRay><<<blocks, 256, 0, stream>>>(sc, pts, P, row0));
  } else if (tune::get("mesh.visibility.mode") == kVisPacket) {
    TOTRI_KERNEL("mesh visibility", stream,
                 visibility_kernel<kVisPacket><<<blocks, 256, 0, stream>>>(sc, pts, P, row0));
  } else if (tune::get("mesh.visibility.mode") == kVisRayPostponed) {
    TOTRI_KERNEL("mesh visibility", stream,
                 visibility_kernel<kVisRayPostponed><<<blocks, 256, 0, stream>>>(sc, pts, P,
                                                                                  row0));
  } else {
    if (P >= (1 << 30) / 4) return fail(TOTRI_ERR_UNSUPPORTED, "too many wall points");
    const int st = launch_point_order(sc, pts, P, stream);
    if (st != TOTRI_OK) return st;
    // Chunks per CTA: up to 8 while the grid keeps 8 CTAs per SM (20,480-face
    // workload: 9.15 ms at 8, 9.3 at 4, 9.6 at 2, 10.4 at 1, 10.5 at 16).
    int chunks = tune::get("mesh.visibility.chunks");
    if (chunks <= 0) {
      const int64_t ctas = (int64_t)ceil_div(P, 32) * sc.nch * sc.B;
      chunks = (int)std::max<int64_t>(1, std::min<int64_t>(8, ctas / (8 * tune::sm_count())));
    }
    if (chunks > kMaxPatchChunks)
      return fail(TOTRI_ERR_INVALID_ARGUMENT, "at most 16 face chunks per visibility block");
    const int seed_mode = tune::get("mesh.visibility.seed");
    if (seed_mode < kSeedBack || seed_mode > kSeedFront)
      return fail(TOTRI_ERR_INVALID_ARGUMENT, "visibility seed mode must be 0..3");
    int seed_steps = tune::get("mesh.visibility.seed.steps");
    if (seed_steps <= 0) seed_steps = 48;
    // candidate capacity of the shaft search (tests lower it to force the
    // per-lane search)
    int shaft_cap = tune::get("mesh.visibility.shaft.cap");
    if (shaft_cap <= 0 || shaft_cap > kShaftCand) shaft_cap = kShaftCand;
    const dim3 grid((unsigned)ceil_div(P, 32), (unsigned)ceil_div(sc.nch, chunks),
                    (unsigned)sc.B);
    const int mode = tune::get("mesh.visibility.mode");
    if (mode == kVisPatchPacket)
      TOTRI_KERNEL("mesh visibility", stream,
                   visibility_patch_kernel<1><<<grid, 256, 0, stream>>>(
                       sc, pts, P, row0, chunks, kSeedOff, 0, 0));
    else if (mode == kVisPatchWide)
      TOTRI_KERNEL("mesh visibility", stream,
                   visibility_patch_kernel<2><<<grid, 256, 0, stream>>>(
                       sc, pts, P, row0, chunks, kSeedOff, 0, 0));
    else if (mode == kVisPatchShaft)
      TOTRI_KERNEL("mesh visibility", stream,
                   visibility_patch_kernel<3><<<grid, 256, 0, stream>>>(
                       sc, pts, P, row0, chunks, seed_mode, seed_steps, shaft_cap));
    // The default: the surface-walk prefix, then the 4-wide BVH search
    // (bvh_occluded_wide) with registers for 4 CTAs per SM (60, no spills):
    // 8.81 ms against 9.19 ms for the binary search at 5 CTAs per SM (48
    // registers, spilling) and 9.26 ms for the 4-wide search capped at 5, per
    // mesh_visibility call on the differentiable workload (build included).
    // "mesh.visibility.wide" = 2 selects the binary search.
    else if (tune::get("mesh.visibility.wide") != 2 && tune::get("mesh.visibility.queue") != 1) {
      if (tune::get("mesh.visibility.occupancy") == 5)
        TOTRI_KERNEL("mesh visibility", stream,
                     visibility_patch_kernel<4, 5><<<grid, 256, 0, stream>>>(
                         sc, pts, P, row0, chunks, seed_mode, seed_steps, 0));
      else
        TOTRI_KERNEL("mesh visibility", stream,
                     visibility_patch_kernel<4, 4><<<grid, 256, 0, stream>>>(
                         sc, pts, P, row0, chunks, seed_mode, seed_steps, 0));
    }
    // The queued BVH searches (visibility_queue_kernel) when
    // "mesh.visibility.queue" = 1; queue entries pack the target's Morton
    // position in 26 bits.
    else if (tune::get("mesh.visibility.queue") == 1 && sc.F < (1 << 26)) {
      if (tune::get("mesh.visibility.occupancy") == 4)
        TOTRI_KERNEL("mesh visibility", stream,
                     visibility_queue_kernel<4><<<grid, 256, 0, stream>>>(
                         sc, pts, P, row0, chunks, seed_mode, seed_steps));
      else
        TOTRI_KERNEL("mesh visibility", stream,
                     visibility_queue_kernel<5><<<grid, 256, 0, stream>>>(
                         sc, pts, P, row0, chunks, seed_mode, seed_steps));
    }
    // Registers capped for 5 CTAs per SM (48 a thread, 28 bytes of spills):
    // 8.84 ms against 9.33 ms uncapped (60 registers, 4 CTAs) and 9.03 ms at
    // 6 CTAs (40 registers) inside the differentiable 20,480-face step.
    else if (tune::get("mesh.visibility.occupancy") == 1)
      TOTRI_KERNEL("mesh visibility", stream,
                   visibility_patch_kernel<0, 1><<<grid, 256, 0, stream>>>(
                       sc, pts, P, row0, chunks, seed_mode, seed_steps, 0));
    else if (tune::get("mesh.visibility.occupancy") == 4)
      TOTRI_KERNEL("mesh visibility", stream,
                   visibility_patch_kernel<0, 4><<<grid, 256, 0, stream>>>(
                       sc, pts, P, row0, chunks, seed_mode, seed_steps, 0));
    else if (tune::get("mesh.visibility.occupancy") == 6)
      TOTRI_KERNEL("mesh visibility", stream,
                   visibility_patch_kernel<0, 6><<<grid, 256, 0, stream>>>(
                       sc, pts, P, row0, chunks, seed_mode, seed_steps, 0));
    else
      TOTRI_KERNEL("mesh visibility", stream,
                   visibility_patch_kernel<0, 5><<<grid, 256, 0, stream>>>(
                       sc, pts, P, row0, chunks, seed_mode, seed_steps, 0));
  }
  return TOTRI_OK;
}

template <int TS>
static int launch_splat_ts(const Scene& sc, const View3f& sp, const View3f& so, int has_origin,
                           float* transient, int T, int S, float bw, float bo,
                           cudaStream_t stream) {
  const size_t smem = sizeof(float) * (size_t)T * TS;
  const dim3 grid((unsigned)ceil_div(S, TS), (unsigned)sc.B);
  if (tune::get("mesh.confocal.splat.mode") == 1) {
    TOTRI_CUDA(tune::ensure_dynamic_smem(
        reinterpret_cast<const void*>(splat_compact_kernel<TS>), smem));
    TOTRI_KERNEL("mesh confocal splat", stream,
                 splat_compact_kernel<TS><<<grid, 256, smem, stream>>>(
                     sc, sp, so, has_origin, transient, T, S, bw, bo,
                     make_fast_bins(bw, bo, tune::get("mesh.confocal.exact") != 1)));
    return TOTRI_OK;
  }
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(splat_kernel<TS>), smem));
  TOTRI_KERNEL("mesh confocal splat", stream,
               splat_kernel<TS><<<grid, 256, smem, stream>>>(
                   sc, sp, so, has_origin, transient, T, S, bw, bo,
                   make_fast_bins(bw, bo, tune::get("mesh.confocal.exact") != 1)));
  return TOTRI_OK;
}

int launch_confocal_splat(const Scene& sc, const View3f& sp, const View3f& so, int has_origin,
                          float* transient, int T, int S, float bw, float bo,
                          cudaStream_t stream) {
  const size_t budget = 200 * 1024;
  const int want = tune::get("mesh.confocal.splat.ts");
  if (want > 0) {
    if ((size_t)T * want * 4 > budget)
      return fail(TOTRI_ERR_INVALID_ARGUMENT, "tuned scan tile too large for the bin count");
    switch (want) {
      case 1: return launch_splat_ts<1>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
      case 2: return launch_splat_ts<2>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
      case 4: return launch_splat_ts<4>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
      case 8: return launch_splat_ts<8>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
      case 16: return launch_splat_ts<16>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
      default: return fail(TOTRI_ERR_INVALID_ARGUMENT, "scan tile must be 1, 2, 4, 8 or 16");
    }
  }
  // Built-in choice: the widest scan tile that keeps the histogram within
  // 40 KB (several CTAs per SM) and still gives every SM tiles to work on.
  const size_t kTileBytes = 40 * 1024;
  if ((size_t)T * 8 * 4 <= kTileBytes && S >= 8 * 152)
    return launch_splat_ts<8>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
  if ((size_t)T * 4 * 4 <= kTileBytes && S >= 4 * 152)
    return launch_splat_ts<4>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
  if ((size_t)T * 2 * 4 <= kTileBytes && S >= 2 * 152)
    return launch_splat_ts<2>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
  if ((size_t)T * 4 <= budget)
    return launch_splat_ts<1>(sc, sp, so, has_origin, transient, T, S, bw, bo, stream);
  return fail(TOTRI_ERR_UNSUPPORTED, "number of bins too large for the shared-memory tile");
}

int launch_confocal_grad(const Scene& sc, const View3f& sp, const View3f& so, int has_origin,
                         const float* tgrad, int T, int S, float bw, float bo,
                         const GradOut& out, cudaStream_t stream) {
  constexpr int kMaxSlice = 16384;  // 64 KB of mask words per CTA
  const int split =
      tune::grad_split("mesh.confocal.grad.split", (int64_t)sc.nch * sc.B, S, kMaxSlice);
  const size_t smem = sizeof(uint32_t) * (size_t)ceil_div(S, split);
  TOTRI_CUDA(tune::ensure_dynamic_smem(
      reinterpret_cast<const void*>(grad_kernel), smem));
  const dim3 grid((unsigned)sc.nch, (unsigned)sc.B, (unsigned)split);
  TOTRI_KERNEL("mesh confocal grad", stream,
               grad_kernel<<<grid, 256, smem, stream>>>(sc, sp, so, has_origin, tgrad, T, S, bw,
                                                        bo, out));
  return TOTRI_OK;
}

}  // namespace mesh
}  // namespace totri
