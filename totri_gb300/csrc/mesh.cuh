// Mesh scene: per-batch-item face records, LBVH and visibility masks, plus
// the FP32 ray-triangle test and BVH walk used for the visibility query.
//
// The reference answers visibility with an OptiX closest-hit trace from each
// wall point to each face centroid (mesh_confocal_forward_optix.cu:42-65,
// closest-hit/miss programs :132-139). Here the same query runs over a
// linear BVH (Karras 2012 hierarchy over 30-bit Morton codes) built by
// hand-written kernels, with an explicit ray-triangle test whose FP32
// rounding is fixed so that the result equals a brute-force test over all
// faces bit for bit.
#pragma once

#include <climits>

#include "common.cuh"

namespace totri {
namespace mesh {

// ---------------------------------------------------------------------------
// Records (all 64 B, four float4, sorted by Morton code of the centroid).
//
// TriRec:   (v0.xyz, e1.x) (e1.yz, e2.xy) (e2.z, lo.xyz) (hi.xyz, face)
//           e1 = v1 - v0, e2 = v2 - v0 (FP32, original vertex order);
//           lo/hi = face AABB grown by delta: hit points must lie inside.
// ShadeRec: (v0.xyz, albedo) (v1.xyz, vi0) (v2.xyz, vi1) (c.xyz, vi2)
//           original vertices, FP32 centroid, vertex indices.
// Node:     (lo0.xy, hi0.xy) (lo1.xy, hi1.xy) (lo0.z, lo1.z, hi0.z, hi1.z) (c0, c1, -, -)
//           child >= 0: internal node, child < 0: leaf ~child. Each pair of
//           planes that one paired FMA evaluates (node_slabs) is adjacent.
// Adj:      int4 (a0, a1, a2, -): a_e = Morton position of the face sharing
//           the edge opposite vertex e (vertex indices compared), -1 if none.

struct Meta {
  int n;          // faces before the first invalid one
  int term_neg;   // 1 when the terminating face holds a negative index
  float scale;    // max |coordinate| over referenced vertices
  float delta;    // scale * 2^-12: hit-point box margin
  int cmin[3];    // ford()-encoded centroid bounds (Morton frame)
  int cmax[3];
  int pad[6];
};

struct Scene {
  int B;           // batch items
  int F;           // face capacity per item
  int nch;         // ceil(F / 32) mask words per point
  int P;           // points per item (mask rows)
  Meta* meta;      // [B]
  uint32_t* keys;  // [B][2][F] ping-pong sort buffers
  uint32_t* vals;  // [B][2][F]
  float4* tri;     // [B][F][4]
  float4* shade;   // [B][F][4]
  float4* nodes;   // [B][F][4] (F-1 used)
  float4* wide;    // [B][F][8]: 4-wide nodes at the even-depth binary nodes
  int* lparent;    // [B][F]
  int* iparent;    // [B][F]
  int* counter;    // [B][F]
  uint32_t* mask;  // [B][P][nch]
  uint32_t* pscratch;  // [4][B][P]: wall-point sort keys/values (ping-pong)
  int4* adj;       // [B][F] edge neighbours (Adj)
  unsigned long long* ekeys;  // [B][ecap] edge hash keys (build scratch)
  int2* evals;     // [B][ecap] the first two faces holding each edge
  int ecap;        // edge hash capacity per item (4 F)
  uint32_t* status;
  int sorted_buf;  // which ping-pong half holds the sorted keys (0/1)
};

// Mesh inputs of one call.
struct BuildInputs {
  View3f verts;      // [B, V, 3]
  View3i faces;      // [B, F, 3]
  View3f material;   // [B, V, M]
  int M;
  int64_t V;
  int F;             // input faces per item
};

// Workspace layout on the host.
struct Layout {
  size_t header, meta, keys, vals, tri, shade, nodes, wide, lparent, iparent, counter, adj,
      ekeys, evals, mask, pscratch, total;
};

inline Layout layout(int64_t B, int64_t F, int64_t P) {
  Layout L{};
  const int64_t Fc = F > 0 ? F : 1;
  const int64_t nch = (Fc + 31) / 32;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off = align_up(off + bytes, 256);
    return at;
  };
  L.header = take(256);
  L.meta = take(sizeof(Meta) * B);
  L.keys = take(sizeof(uint32_t) * 2 * B * Fc);
  L.vals = take(sizeof(uint32_t) * 2 * B * Fc);
  L.tri = take(64 * B * Fc);
  L.shade = take(64 * B * Fc);
  L.nodes = take(64 * B * Fc);
  L.wide = take(128 * B * Fc);
  L.lparent = take(sizeof(int) * B * Fc);
  L.iparent = take(sizeof(int) * B * Fc);
  L.counter = take(sizeof(int) * B * Fc);
  L.adj = take(sizeof(int4) * B * Fc);
  L.ekeys = take(sizeof(unsigned long long) * B * 4 * Fc);
  L.evals = take(sizeof(int2) * B * 4 * Fc);
  L.mask = take(sizeof(uint32_t) * B * P * nch);
  L.pscratch = take(sizeof(uint32_t) * 4 * B * P);
  L.total = off;
  return L;
}

inline Scene scene_from_workspace(void* ws, int64_t B, int64_t F, int64_t P) {
  const Layout L = layout(B, F, P);
  char* base = static_cast<char*>(ws);
  Scene s;
  s.B = (int)B;
  s.F = (int)(F > 0 ? F : 1);
  s.nch = (int)((s.F + 31) / 32);
  s.P = (int)P;
  s.status = reinterpret_cast<uint32_t*>(base + L.header);
  s.meta = reinterpret_cast<Meta*>(base + L.meta);
  s.keys = reinterpret_cast<uint32_t*>(base + L.keys);
  s.vals = reinterpret_cast<uint32_t*>(base + L.vals);
  s.tri = reinterpret_cast<float4*>(base + L.tri);
  s.shade = reinterpret_cast<float4*>(base + L.shade);
  s.nodes = reinterpret_cast<float4*>(base + L.nodes);
  s.wide = reinterpret_cast<float4*>(base + L.wide);
  s.lparent = reinterpret_cast<int*>(base + L.lparent);
  s.iparent = reinterpret_cast<int*>(base + L.iparent);
  s.counter = reinterpret_cast<int*>(base + L.counter);
  s.adj = reinterpret_cast<int4*>(base + L.adj);
  s.ekeys = reinterpret_cast<unsigned long long*>(base + L.ekeys);
  s.evals = reinterpret_cast<int2*>(base + L.evals);
  s.ecap = 4 * s.F;
  s.mask = reinterpret_cast<uint32_t*>(base + L.mask);
  s.pscratch = reinterpret_cast<uint32_t*>(base + L.pscratch);
  s.sorted_buf = 1;  // three 10-bit radix passes end in the second half
  return s;
}

// A scene whose BVH and face records live in `ws` (laid out for zero wall
// points) and whose visibility masks [B][P][nch] live in a separate buffer:
// the resident form, where one BVH serves many wall grids.
inline size_t mask_words_bytes(int64_t B, int64_t F, int64_t P) {
  const int64_t Fc = F > 0 ? F : 1;
  return align_up(sizeof(uint32_t) * (size_t)B * (size_t)P * (size_t)((Fc + 31) / 32), 256);
}

// Mask buffer of the resident form: the masks, then the wall-point sort scratch.
inline size_t mask_bytes(int64_t B, int64_t F, int64_t P) {
  return mask_words_bytes(B, F, P) + sizeof(uint32_t) * 4 * (size_t)B * (size_t)P;
}

inline Scene scene_with_masks(void* ws, int64_t B, int64_t F, void* masks, int64_t P) {
  Scene s = scene_from_workspace(ws, B, F, 0);
  s.P = (int)P;
  s.mask = static_cast<uint32_t*>(masks);
  s.pscratch = reinterpret_cast<uint32_t*>(static_cast<char*>(masks) + mask_words_bytes(B, F, P));
  return s;
}

// ---------------------------------------------------------------------------
// Device helpers.

__device__ __forceinline__ const float4* tri_at(const Scene& s, int b, int k) {
  return s.tri + ((size_t)b * s.F + k) * 4;
}
__device__ __forceinline__ const float4* shade_at(const Scene& s, int b, int k) {
  return s.shade + ((size_t)b * s.F + k) * 4;
}
__device__ __forceinline__ const float4* node_at(const Scene& s, int b, int i) {
  return s.nodes + ((size_t)b * s.F + i) * 4;
}
// Float index in a node record of child c's lower (hi = 0) or upper (hi = 1)
// plane on axis a; the child links are floats 12 and 13.
__host__ __device__ __forceinline__ int node_plane(int c, int hi, int a) {
  return a < 2 ? 4 * c + 2 * hi + a : 8 + 2 * hi + c;
}

// FP32 ray-triangle test (two-sided Moller-Trumbore with t in [0, tmax] and
// the hit point fma(t, d, o) inside the grown face AABB). Mirrors
// oracle/mesh.cpp tri_hit operation for operation.
__device__ __forceinline__ bool tri_hit(float4 t0, float4 t1, float4 t2, float4 t3, fv3 o,
                                        fv3 d, float tmax, float& tout) {
  const fv3 v0 = mkv(t0.x, t0.y, t0.z);
  const fv3 e1 = mkv(t0.w, t1.x, t1.y);
  const fv3 e2 = mkv(t1.z, t1.w, t2.x);
  const fv3 p = xcross(d, e2);
  const float det = xdot(e1, p);
  if (det == 0.f) return false;
  const float inv = xrcp(det);
  const fv3 tv = xsub3(o, v0);
  const float u = xmul(xdot(tv, p), inv);
  if (!(u >= 0.f && u <= 1.f)) return false;
  const fv3 q = xcross(tv, e1);
  const float v = xmul(xdot(d, q), inv);
  if (!(v >= 0.f && xadd(u, v) <= 1.f)) return false;
  const float t = xmul(xdot(e2, q), inv);
  if (!(t >= 0.f && t <= tmax)) return false;
  const float px = xfma(t, d.x, o.x);
  const float py = xfma(t, d.y, o.y);
  const float pz = xfma(t, d.z, o.z);
  if (!(px >= t2.y && px <= t3.x && py >= t2.z && py <= t3.y && pz >= t2.w && pz <= t3.z))
    return false;
  tout = t;
  return true;
}

// Slab test of a BVH box against the ray segment (-inf, limit]. Boxes carry a
// margin of at least delta beyond every accepted hit point, which dominates
// the rounding of this test, so a box holding a hit is never rejected. The
// entry distance is not clamped at 0: that only admits boxes lying wholly
// behind the wall point (none do for a mesh in front of the wall), never
// rejects one, and saves an instruction per box.
__device__ __forceinline__ bool slab(float lx, float ly, float lz, float hx, float hy,
                                     float hz, fv3 inv, fv3 oinv, float limit,
                                     float& tnear) {
  const float tx0 = fmaf(lx, inv.x, -oinv.x), tx1 = fmaf(hx, inv.x, -oinv.x);
  const float ty0 = fmaf(ly, inv.y, -oinv.y), ty1 = fmaf(hy, inv.y, -oinv.y);
  const float tz0 = fmaf(lz, inv.z, -oinv.z), tz1 = fmaf(hz, inv.z, -oinv.z);
  const float tn = fmax3(fminf(tx0, tx1), fminf(ty0, ty1), fminf(tz0, tz1));
  const float tf = fmin3(fmaxf(tx0, tx1), fmaxf(ty0, ty1), fminf(fmaxf(tz0, tz1), limit));
  tnear = tn;
  return tn <= tf;
}

__device__ __forceinline__ float safe_inv(float d) {
  return fabsf(d) < 1e-20f ? copysignf(1e20f, d) : 1.f / d;
}

// A ray's slab constants for node_slabs: 1/d and -o/d as (x, y) and (z, z)
// pairs.
struct RaySlab {
  unsigned long long ixy, izz, nxy, nzz;
};

__device__ __forceinline__ RaySlab ray_slab(fv3 inv, fv3 oinv) {
  return RaySlab{f2pack(inv.x, inv.y), f2pack(inv.z, inv.z), f2pack(-oinv.x, -oinv.y),
                 f2pack(-oinv.z, -oinv.z)};
}

// The direction octant of a ray for node_slabs: bit a set when component a of
// 1/d is negative.
__device__ __forceinline__ int ray_octant(fv3 inv) {
  return (signbit(inv.x) ? 1 : 0) | (signbit(inv.y) ? 2 : 0) | (signbit(inv.z) ? 4 : 0);
}

// Both children's slab tests of a node record (n0, n1, n2 as laid out in
// Node), each against the ray segment (-inf, limit]: the twelve plane
// distances take six paired FMAs. kOct < 8 is the ray's octant (ray_octant),
// which fixes each axis's entry and exit plane at compile time; kOct = 8 takes
// them with min/max. For a box with lo <= hi the two agree exactly (fma is
// monotone), and the test accepts the boxes slab() accepts.
template <int kOct>
__device__ __forceinline__ void node_slabs(float4 n0, float4 n1, float4 n2, const RaySlab& r,
                                           float limit, bool& h0, bool& h1, float& t0,
                                           float& t1) {
  float l0x, l0y, u0x, u0y, l1x, l1y, u1x, u1y, l0z, l1z, u0z, u1z;
  f2unpack(f2fma(f2pack(n0.x, n0.y), r.ixy, r.nxy), l0x, l0y);
  f2unpack(f2fma(f2pack(n0.z, n0.w), r.ixy, r.nxy), u0x, u0y);
  f2unpack(f2fma(f2pack(n1.x, n1.y), r.ixy, r.nxy), l1x, l1y);
  f2unpack(f2fma(f2pack(n1.z, n1.w), r.ixy, r.nxy), u1x, u1y);
  f2unpack(f2fma(f2pack(n2.x, n2.y), r.izz, r.nzz), l0z, l1z);
  f2unpack(f2fma(f2pack(n2.z, n2.w), r.izz, r.nzz), u0z, u1z);
  float a0, b0, a1, b1;  // entry / exit distance of each child
  if (kOct == 8) {
    a0 = fmax3(fminf(l0x, u0x), fminf(l0y, u0y), fminf(l0z, u0z));
    b0 = fmin3(fmaxf(l0x, u0x), fmaxf(l0y, u0y), fminf(fmaxf(l0z, u0z), limit));
    a1 = fmax3(fminf(l1x, u1x), fminf(l1y, u1y), fminf(l1z, u1z));
    b1 = fmin3(fmaxf(l1x, u1x), fmaxf(l1y, u1y), fminf(fmaxf(l1z, u1z), limit));
  } else {
    constexpr bool nx = kOct & 1, ny = kOct & 2, nz = kOct & 4;
    a0 = fmax3(nx ? u0x : l0x, ny ? u0y : l0y, nz ? u0z : l0z);
    b0 = fmin3(nx ? l0x : u0x, ny ? l0y : u0y, fminf(nz ? l0z : u0z, limit));
    a1 = fmax3(nx ? u1x : l1x, ny ? u1y : l1y, nz ? u1z : l1z);
    b1 = fmin3(nx ? l1x : u1x, ny ? l1y : u1y, fminf(nz ? l1z : u1z, limit));
  }
  h0 = a0 <= b0;
  h1 = a1 <= b1;
  t0 = a0;
  t1 = a1;
}

// The target of a visibility query: face k (Morton position) with its
// intersection record and centroid, loaded once for many wall points.
struct Target {
  int k, f;
  float4 a0, a1, a2, a3;
  fv3 c;
};

__device__ __forceinline__ Target load_target(const Scene& sc, int b, int k) {
  Target t;
  t.k = k;
  const float4* tr = tri_at(sc, b, k);
  t.a0 = __ldg(tr);
  t.a1 = __ldg(tr + 1);
  t.a2 = __ldg(tr + 2);
  t.a3 = __ldg(tr + 3);
  t.f = __float_as_int(t.a3.w);
  const float4 c4 = __ldg(shade_at(sc, b, k) + 3);
  t.c = mkv(c4.x, c4.y, c4.z);
  return t;
}

// True when the target face is the closest hit, lowest face index on ties, of
// the ray from o to its centroid within [0, 1.01 d + 1e-3]
// (mesh_confocal_forward_optix.cu:42-65). Any single occluder settles "not
// visible", so `cache` (a Morton position or -1) is tested first: callers pass
// the occluder found for a neighbouring wall point. kBrute tests every face
// instead of walking the BVH; the answer is the same by construction.
template <bool kBrute>
__device__ bool target_visible(const Scene& sc, int b, int n, const Target& tg, fv3 o, int& cache,
                               uint32_t* status) {
  const int k = tg.k;
  const fv3 D = xsub3(tg.c, o);
  const float dist = xlen(D);
  if (!(dist >= 1e-6f)) return false;
  const fv3 dir = mkv(xdiv(D.x, dist), xdiv(D.y, dist), xdiv(D.z, dist));
  const float tmax = xadd(xmul(dist, 1.01f), 1e-3f);
  const int f = tg.f;
  float tf;
  if (!tri_hit(tg.a0, tg.a1, tg.a2, tg.a3, o, dir, tmax, tf)) return false;

  auto occludes = [&](int kk) -> bool {
    if (kk == k) return false;
    if (kk < 0 || kk >= n) {
      atomicOr(status, kStatusTraversalCap);
      return false;
    }
    const float4* q = tri_at(sc, b, kk);
    const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3);
    float tq;
    if (!tri_hit(q0, q1, q2, q3, o, dir, tmax, tq)) return false;
    return tq < tf || (tq == tf && __float_as_int(q3.w) < f);
  };

  if (cache >= 0 && occludes(cache)) return false;

  if (kBrute || n == 1) {
    for (int kk = 0; kk < n; ++kk)
      if (occludes(kk)) { cache = kk; return false; }
    return true;
  }

  const fv3 inv = mkv(safe_inv(dir.x), safe_inv(dir.y), safe_inv(dir.z));
  const fv3 oinv = mkv(o.x * inv.x, o.y * inv.y, o.z * inv.z);
  int stack[64];
  int sp = 0;
  int node = 0;
  const int cap = 2 * n + 64;
  for (int it = 0; it < cap; ++it) {
    if (node < 0 || node >= n - 1) break;  // malformed tree: flagged below
    const float4* nd = node_at(sc, b, node);
    const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
    float tn0, tn1;
    bool h0 = slab(n0.x, n0.y, n2.x, n0.z, n0.w, n2.z, inv, oinv, tf, tn0);
    bool h1 = slab(n1.x, n1.y, n2.y, n1.z, n1.w, n2.w, inv, oinv, tf, tn1);
    const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
    if (h0 && c0 < 0) {
      if (occludes(~c0)) { cache = ~c0; return false; }
      h0 = false;
    }
    if (h1 && c1 < 0) {
      if (occludes(~c1)) { cache = ~c1; return false; }
      h1 = false;
    }
    if (h0 && h1) {
      const bool first0 = tn0 <= tn1;
      if (sp < 64) stack[sp++] = first0 ? c1 : c0;
      else atomicOr(status, kStatusTraversalCap);
      node = first0 ? c0 : c1;
    } else if (h0) {
      node = c0;
    } else if (h1) {
      node = c1;
    } else {
      if (sp == 0) return true;
      node = stack[--sp];
    }
  }
  atomicOr(status, kStatusTraversalCap);
  return true;
}

// Which targets try the surface walk first (the value of the tuning key
// mesh.visibility.seed; 0, the default, takes the faces seen from behind).
enum SeedMode { kSeedBack = 0, kSeedOff = 1, kSeedAll = 2, kSeedFront = 3 };

// Surface walk: a search for an occluder of the ray from o to target k that
// starts at face g (the occluder found for a neighbouring query) and moves
// across the mesh's edges. The ray's crossing with the current face's plane
// is located from barycentric coordinates in fast arithmetic (fused
// multiply-adds, approximate reciprocal); where they put it inside the face,
// up to a slack, the face gets the exact leaf test of the BVH walk, and an
// occluder found so ends the walk. Otherwise the walk crosses to the
// neighbour beyond the edge with the most negative coordinate. It stops at the
// target, at a mesh boundary, at a face whose plane the ray crosses inside the
// face without being occluded by it, or after `steps` faces. It returns an
// occluder's Morton position or -1: only the exact test can end it in "not
// visible", so the fast coordinates and any wrong turn cost time, never a
// mask bit.
__device__ __forceinline__ int surface_walk(const Scene& sc, int b, int n, int k, int f, int g,
                                            fv3 o, fv3 dir, float tmax, float tf, int steps) {
  const float4* tri = sc.tri + (size_t)b * sc.F * 4;
  const int4* adj = sc.adj + (size_t)b * sc.F;
  constexpr float kSlack = 1e-4f;
  for (int st = 0; st < steps; ++st) {
    if (g == k || (unsigned)g >= (unsigned)n) return -1;
    const float4* q = tri + (size_t)g * 4;
    const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3);
    const fv3 e1 = mkv(q0.w, q1.x, q1.y), e2 = mkv(q1.z, q1.w, q2.x);
    const fv3 pv = cross(dir, e2);
    const float inv = __fdividef(1.f, dot(e1, pv));
    const fv3 tv = o - mkv(q0.x, q0.y, q0.z);
    const float u = dot(tv, pv) * inv;
    const float v = dot(dir, cross(tv, e1)) * inv;
    const float w0 = 1.f - u - v;
    int e;
    float wm;
    if (w0 <= u && w0 <= v) {
      e = 0;
      wm = w0;
    } else if (u <= v) {
      e = 1;
      wm = u;
    } else {
      e = 2;
      wm = v;
    }
    if (wm >= -kSlack) {  // the crossing is inside the face, or close to it
      float tq;
      if (tri_hit(q0, q1, q2, q3, o, dir, tmax, tq) &&
          (tq < tf || (tq == tf && __float_as_int(q3.w) < f)))
        return g;
      if (!(wm < 0.f)) return -1;
    } else if (!(wm < 0.f)) {
      return -1;  // NaN coordinates: a degenerate face
    }
    const int4 a = __ldg(adj + g);
    g = e == 0 ? a.x : (e == 1 ? a.y : a.z);
    if (g < 0) return -1;
  }
  return -1;
}

// target_visible with postponed leaf tests (the "while-while" organisation
// of Aila and Laine, HPG 2009): a lane that reaches a leaf parks it and keeps
// walking internal nodes until no lane of the warp still walking lacks a
// parked leaf; the triangle tests, the costliest step of the walk, then run
// together. The leaves tested, and so the answer, are those of
// target_visible (any occluder settles the ray; order does not matter).
// With seed_steps > 0 and a seed face (seed >= 0), the targets that seed_mode
// selects first try surface_walk from the seed; `seed` returns the occluder
// found by either search, for the next query.
// The part of a query that needs no search: the ray to the target's centroid,
// the target's own hit and, for the targets that seed_mode selects, the
// surface walk from `seed`. Returns 1 when an occluder search must still
// decide (dir, tmax and tf set), else 0 with the answer in `vis`.
__device__ __forceinline__ int query_prefix(const Scene& sc, int b, int n, const Target& tg,
                                            fv3 o, int& seed, int seed_mode, int seed_steps,
                                            fv3& dir, float& tmax, float& tf, bool& vis) {
  vis = false;
  const fv3 D = xsub3(tg.c, o);
  const float dist = xlen(D);
  if (!(dist >= 1e-6f)) return 0;
  dir = mkv(xdiv(D.x, dist), xdiv(D.y, dist), xdiv(D.z, dist));
  tmax = xadd(xmul(dist, 1.01f), 1e-3f);
  if (!tri_hit(tg.a0, tg.a1, tg.a2, tg.a3, o, dir, tmax, tf)) return 0;
  if (n == 1) {
    vis = true;
    return 0;
  }
  if (seed_steps > 0 && seed >= 0 && seed_mode != kSeedOff) {
    bool walk = seed_mode == kSeedAll;
    if (!walk) {  // faces wound outward and seen from behind are mostly occluded
      const fv3 nrm = cross(mkv(tg.a0.w, tg.a1.x, tg.a1.y), mkv(tg.a1.z, tg.a1.w, tg.a2.x));
      walk = (dot(nrm, D) > 0.f) == (seed_mode == kSeedBack);
    }
    if (walk) {
      const int g = surface_walk(sc, b, n, tg.k, tg.f, seed, o, dir, tmax, tf, seed_steps);
      if (g >= 0) {
        seed = g;
        return 0;
      }
    }
  }
  return 1;
}

// The BVH search of target_visible_pp for rays of octant kOct (node_slabs).
template <int kOct>
__device__ __forceinline__ bool bvh_occluded_oct(const Scene& sc, int b, int n, int k, int f,
                                                 fv3 o, fv3 dir, float tmax, float tf,
                                                 const RaySlab& rs, uint32_t* status,
                                                 int& seed) {
  constexpr int kDone = INT_MIN;  // below every leaf code ~k, k < n
  int stack[64];
  int sp = 0;
  auto pop = [&]() { return sp > 0 ? stack[--sp] : kDone; };
  int node = 0;      // internal node (>= 0), leaf (~k < 0) or kDone
  int leaf = kDone;  // parked leaf
  const float4* nodes = sc.nodes + (size_t)b * sc.F * 4;
  const unsigned inner = (unsigned)(n - 1);
  int budget = 2 * n + 64;  // iteration cap: a malformed tree ends the walk
  while (node != kDone) {
    while (node >= 0) {
      if (--budget < 0 || (unsigned)node >= inner) {  // malformed tree
        atomicOr(status, kStatusTraversalCap);
        return false;
      }
      const float4* nd = nodes + node * 4;
      const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
      float tn0, tn1;
      bool h0, h1;
      node_slabs<kOct>(n0, n1, n2, rs, tf, h0, h1, tn0, tn1);
      const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
      if (h0 && h1) {
        const bool first0 = tn0 <= tn1;
        if (sp < 64) stack[sp++] = first0 ? c1 : c0;
        else atomicOr(status, kStatusTraversalCap);
        node = first0 ? c0 : c1;
      } else if (h0) {
        node = c0;
      } else if (h1) {
        node = c1;
      } else {
        node = pop();
      }
      if (node < 0 && node != kDone && leaf == kDone) {
        leaf = node;
        node = pop();
      }
      if (!__any_sync(__activemask(), leaf == kDone)) break;
    }
    while (leaf != kDone) {
      const int kk = ~leaf;
      if (kk != k) {
        if (kk < 0 || kk >= n) {
          atomicOr(status, kStatusTraversalCap);
        } else {
          const float4* q = tri_at(sc, b, kk);
          const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3);
          float tq;
          if (tri_hit(q0, q1, q2, q3, o, dir, tmax, tq) &&
              (tq < tf || (tq == tf && __float_as_int(q3.w) < f))) {
            seed = kk;
            return true;
          }
        }
      }
      leaf = kDone;
      if (node < 0 && node != kDone) {
        leaf = node;
        node = pop();
      }
    }
  }
  return false;
}

// The BVH search of target_visible_pp: true when some face other than the
// target k (original index f) hits the ray before the target's hit at tf
// (ties to the lower original index); `seed` returns that occluder. When the
// rays of all calling lanes share a direction octant with d.z >= 0 (rays
// from a wall patch towards one face mostly do), the walk with that octant's
// fixed entry and exit planes runs; otherwise the general one. Every lane of
// the warp that calls it takes the same branch.
__device__ __forceinline__ bool bvh_occluded(const Scene& sc, int b, int n, int k, int f, fv3 o,
                                             fv3 dir, float tmax, float tf, uint32_t* status,
                                             int& seed) {
  const fv3 inv = mkv(safe_inv(dir.x), safe_inv(dir.y), safe_inv(dir.z));
  const fv3 oinv = mkv(o.x * inv.x, o.y * inv.y, o.z * inv.z);
  const RaySlab rs = ray_slab(inv, oinv);
  const unsigned act = __activemask();
  const int oct = ray_octant(inv);
  const int lead = __shfl_sync(act, oct, __ffs(act) - 1);
  const int mode = __all_sync(act, oct == lead) && lead < 4 ? lead : 8;
  switch (mode) {
    case 0: return bvh_occluded_oct<0>(sc, b, n, k, f, o, dir, tmax, tf, rs, status, seed);
    case 1: return bvh_occluded_oct<1>(sc, b, n, k, f, o, dir, tmax, tf, rs, status, seed);
    case 2: return bvh_occluded_oct<2>(sc, b, n, k, f, o, dir, tmax, tf, rs, status, seed);
    case 3: return bvh_occluded_oct<3>(sc, b, n, k, f, o, dir, tmax, tf, rs, status, seed);
    default: return bvh_occluded_oct<8>(sc, b, n, k, f, o, dir, tmax, tf, rs, status, seed);
  }
}

// bvh_occluded over the 4-wide tree (see target_visible_pp4 for its records):
// one step tests the four child boxes of a record, whose planes are SoA
// float4s, with twelve paired FMAs, goes on with the nearest hit and stacks
// the others. kOct as in node_slabs. The leaves tested, and so the answer,
// are those of bvh_occluded: a leaf is reached iff its binary ancestors' boxes
// and its own all pass.
// Code of an unused slot of a 4-wide record.
constexpr int kWideEmpty = INT_MIN + 1;

template <int kOct>
__device__ __forceinline__ bool bvh_occluded_wide_oct(const Scene& sc, int b, int n, int k, int f,
                                                      fv3 o, fv3 dir, float tmax, float tf,
                                                      fv3 inv, fv3 oinv, uint32_t* status,
                                                      int& seed) {
  constexpr int kDone = INT_MIN;
  const unsigned long long ix = f2pack(inv.x, inv.x), iy = f2pack(inv.y, inv.y),
                           iz = f2pack(inv.z, inv.z);
  const unsigned long long nx = f2pack(-oinv.x, -oinv.x), ny = f2pack(-oinv.y, -oinv.y),
                           nz = f2pack(-oinv.z, -oinv.z);
  const float4* wb = sc.wide + (size_t)b * sc.F * 8;
  int stack[64];
  int sp = 0;
  auto pop = [&]() { return sp > 0 ? stack[--sp] : kDone; };
  auto push = [&](int v) {
    if (sp < 64) stack[sp++] = v;
    else atomicOr(status, kStatusTraversalCap);
  };
  int node = 0;
  int leaf = kDone;
  const unsigned inner = (unsigned)(n - 1);
  int budget = 2 * n + 64;
  while (node != kDone) {
    while (node >= 0) {
      if (--budget < 0 || (unsigned)node >= inner) {
        atomicOr(status, kStatusTraversalCap);
        return false;
      }
      const float4* w = wb + (size_t)node * 8;
      const float4 lx = __ldg(w), ly = __ldg(w + 1), lz = __ldg(w + 2);
      const float4 hx = __ldg(w + 3), hy = __ldg(w + 4), hz = __ldg(w + 5);
      const float4 cc = __ldg(w + 6);
      float lx0, lx1, lx2, lx3, ly0, ly1, ly2, ly3, lz0, lz1, lz2, lz3;
      float hx0, hx1, hx2, hx3, hy0, hy1, hy2, hy3, hz0, hz1, hz2, hz3;
      f2unpack(f2fma(f2pack(lx.x, lx.y), ix, nx), lx0, lx1);
      f2unpack(f2fma(f2pack(lx.z, lx.w), ix, nx), lx2, lx3);
      f2unpack(f2fma(f2pack(ly.x, ly.y), iy, ny), ly0, ly1);
      f2unpack(f2fma(f2pack(ly.z, ly.w), iy, ny), ly2, ly3);
      f2unpack(f2fma(f2pack(lz.x, lz.y), iz, nz), lz0, lz1);
      f2unpack(f2fma(f2pack(lz.z, lz.w), iz, nz), lz2, lz3);
      f2unpack(f2fma(f2pack(hx.x, hx.y), ix, nx), hx0, hx1);
      f2unpack(f2fma(f2pack(hx.z, hx.w), ix, nx), hx2, hx3);
      f2unpack(f2fma(f2pack(hy.x, hy.y), iy, ny), hy0, hy1);
      f2unpack(f2fma(f2pack(hy.z, hy.w), iy, ny), hy2, hy3);
      f2unpack(f2fma(f2pack(hz.x, hz.y), iz, nz), hz0, hz1);
      f2unpack(f2fma(f2pack(hz.z, hz.w), iz, nz), hz2, hz3);
      auto box = [&](float ax, float ay, float az, float bx, float by, float bz, float& t) {
        float a, e;
        if (kOct == 8) {
          a = fmax3(fminf(ax, bx), fminf(ay, by), fminf(az, bz));
          e = fmin3(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), tf));
        } else {
          constexpr bool qx = kOct & 1, qy = kOct & 2, qz = kOct & 4;
          a = fmax3(qx ? bx : ax, qy ? by : ay, qz ? bz : az);
          e = fmin3(qx ? ax : bx, qy ? ay : by, fminf(qz ? az : bz, tf));
        }
        t = a;
        return a <= e;
      };
      const int c0 = __float_as_int(cc.x), c1 = __float_as_int(cc.y);
      const int c2 = __float_as_int(cc.z), c3 = __float_as_int(cc.w);
      float t0, t1, t2, t3;
      const bool h0 = box(lx0, ly0, lz0, hx0, hy0, hz0, t0);
      const bool h1 = box(lx1, ly1, lz1, hx1, hy1, hz1, t1) && c1 != kWideEmpty;
      const bool h2 = box(lx2, ly2, lz2, hx2, hy2, hz2, t2) && c2 != kWideEmpty;
      const bool h3 = box(lx3, ly3, lz3, hx3, hy3, hz3, t3) && c3 != kWideEmpty;
      float best = INFINITY;
      int next = kDone;
      if (h0 && t0 < best) { best = t0; next = c0; }
      if (h1 && t1 < best) { best = t1; next = c1; }
      if (h2 && t2 < best) { best = t2; next = c2; }
      if (h3 && t3 < best) { best = t3; next = c3; }
      if (h3 && next != c3) push(c3);
      if (h2 && next != c2) push(c2);
      if (h1 && next != c1) push(c1);
      if (h0 && next != c0) push(c0);
      node = next != kDone ? next : pop();
      if (node < 0 && node != kDone && leaf == kDone) {
        leaf = node;
        node = pop();
      }
      if (!__any_sync(__activemask(), leaf == kDone)) break;
    }
    while (leaf != kDone) {
      const int kk = ~leaf;
      if (kk != k) {
        if (kk < 0 || kk >= n) {
          atomicOr(status, kStatusTraversalCap);
        } else {
          const float4* q = tri_at(sc, b, kk);
          const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3);
          float tq;
          if (tri_hit(q0, q1, q2, q3, o, dir, tmax, tq) &&
              (tq < tf || (tq == tf && __float_as_int(q3.w) < f))) {
            seed = kk;
            return true;
          }
        }
      }
      leaf = kDone;
      if (node < 0 && node != kDone) {
        leaf = node;
        node = pop();
      }
    }
  }
  return false;
}

// bvh_occluded through the 4-wide tree, with the same octant dispatch.
__device__ __forceinline__ bool bvh_occluded_wide(const Scene& sc, int b, int n, int k, int f,
                                                  fv3 o, fv3 dir, float tmax, float tf,
                                                  uint32_t* status, int& seed) {
  const fv3 inv = mkv(safe_inv(dir.x), safe_inv(dir.y), safe_inv(dir.z));
  const fv3 oinv = mkv(o.x * inv.x, o.y * inv.y, o.z * inv.z);
  const unsigned act = __activemask();
  const int oct = ray_octant(inv);
  const int lead = __shfl_sync(act, oct, __ffs(act) - 1);
  const int mode = __all_sync(act, oct == lead) && lead < 4 ? lead : 8;
  switch (mode) {
    case 0: return bvh_occluded_wide_oct<0>(sc, b, n, k, f, o, dir, tmax, tf, inv, oinv, status, seed);
    case 1: return bvh_occluded_wide_oct<1>(sc, b, n, k, f, o, dir, tmax, tf, inv, oinv, status, seed);
    case 2: return bvh_occluded_wide_oct<2>(sc, b, n, k, f, o, dir, tmax, tf, inv, oinv, status, seed);
    case 3: return bvh_occluded_wide_oct<3>(sc, b, n, k, f, o, dir, tmax, tf, inv, oinv, status, seed);
    default: return bvh_occluded_wide_oct<8>(sc, b, n, k, f, o, dir, tmax, tf, inv, oinv, status, seed);
  }
}

__device__ __forceinline__ bool target_visible_pp(const Scene& sc, int b, int n,
                                                  const Target& tg, fv3 o, uint32_t* status,
                                                  int& seed, int seed_mode, int seed_steps) {
  fv3 dir;
  float tmax, tf;
  bool vis;
  if (!query_prefix(sc, b, n, tg, o, seed, seed_mode, seed_steps, dir, tmax, tf, vis))
    return vis;
  return !bvh_occluded(sc, b, n, tg.k, tg.f, o, dir, tmax, tf, status, seed);
}

// Occluder candidates shared by the rays of a warp: the rays start in the box
// P (the warp's wall points) and end at the target's hit point, inside the
// target's hit-point box C, so every point of every ray segment lies in the
// convex hull of P and C, the union over s in [0, 1] of the boxes
// (1 - s) P + s C. A BVH box meets that hull iff the s-intervals of its six
// face constraints, each linear in s, intersect within [0, 1]. Both boxes are
// grown by the hit-point margin delta, far beyond the rounding of this test,
// and BVH boxes hold a delta margin around every accepted hit point, so a box
// holding an occluder of any of the rays is never rejected: the candidates
// include every occluder the rays' own BVH walks would test, and the exact
// triangle test decides.
struct Shaft {
  float plo[3], rl[3];  // lower face: Plo + s (Clo - Plo) <= box hi
  float phi[3], rh[3];  // upper face: Phi + s (Chi - Phi) >= box lo
  bool lneg[3], hneg[3];
};

__device__ __forceinline__ Shaft make_shaft(const float plo[3], const float phi[3],
                                            const float clo[3], const float chi[3]) {
  Shaft h;
  for (int a = 0; a < 3; ++a) {
    const float dl = clo[a] - plo[a], dh = chi[a] - phi[a];
    h.plo[a] = plo[a];
    h.phi[a] = phi[a];
    h.rl[a] = 1.f / dl;
    h.rh[a] = 1.f / dh;
    h.lneg[a] = dl < 0.f;
    h.hneg[a] = dh < 0.f;
  }
  return h;
}

// Box [lo, hi] against the hull; a NaN bound (a zero extent meeting a box
// face exactly) drops its constraint, which can only admit a box. Each bound
// is the difference of coordinates, then scaled: its error is an ulp of the
// coordinates over |dl|, inside the pad / |dl| that the grown boxes leave in
// s. (Scaling first, hi / dl - Plo / dl, cancels two huge terms when an axis
// of the hull is short, e.g. a target point beside the wall patch's box edge,
// and rejected boxes holding occluders.)
__device__ __forceinline__ bool shaft_box(const Shaft& h, float lx, float ly, float lz, float hx,
                                          float hy, float hz) {
  const float lo[3] = {lx, ly, lz}, hi[3] = {hx, hy, hz};
  float smin = 0.f, smax = 1.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float u = (hi[a] - h.plo[a]) * h.rl[a];  // (hi - Plo) / dl
    const float w = (lo[a] - h.phi[a]) * h.rh[a];  // (lo - Phi) / dh
    if (h.lneg[a]) smin = fmaxf(smin, u);
    else smax = fminf(smax, u);
    if (h.hneg[a]) smax = fminf(smax, w);
    else smin = fmaxf(smin, w);
  }
  return smin <= smax;
}

// Warp-collective breadth-first walk of the BVH restricted to the hull: each
// round the lanes test the children of up to 32 frontier nodes at once.
// Writes the candidate leaves (Morton positions, the target k excluded) to
// cand and returns their count, or -1 when a frontier overflows its capacity,
// the candidates exceed cap (at most kCand) or the tree is malformed (the
// caller then searches per lane). All 32 lanes must call it with the same
// arguments.
template <int kFrontier, int kCand>
__device__ __forceinline__ int shaft_candidates(const Scene& sc, int b, int n, int k,
                                                const Shaft& h, int* fr0, int* fr1, int* cand,
                                                int lane, int cap) {
  const float4* nodes = sc.nodes + (size_t)b * sc.F * 4;
  const unsigned inner = (unsigned)(n - 1);
  const unsigned lt = (1u << lane) - 1u;
  if (lane == 0) fr0[0] = 0;
  __syncwarp();
  int* cur = fr0;
  int* nxt = fr1;
  int cnt = 1, nc = 0;
  bool bad = false;
  for (int round = 0; cnt > 0; ++round) {
    if (round >= 96) return -1;
    int ncnt = 0;
    for (int base = 0; base < cnt; base += 32) {
      const int idx = base + lane;
      bool h0 = false, h1 = false;
      int c0 = 0, c1 = 0;
      if (idx < cnt) {
        const int node = cur[idx];
        if ((unsigned)node < inner) {
          const float4* nd = nodes + node * 4;
          const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2),
                       n3 = __ldg(nd + 3);
          h0 = shaft_box(h, n0.x, n0.y, n2.x, n0.z, n0.w, n2.z);
          h1 = shaft_box(h, n1.x, n1.y, n2.y, n1.z, n1.w, n2.w);
          c0 = __float_as_int(n3.x);
          c1 = __float_as_int(n3.y);
        } else {
          bad = true;
        }
      }
      const bool i0 = h0 && c0 >= 0, i1 = h1 && c1 >= 0;
      const bool l0 = h0 && c0 < 0 && ~c0 != k, l1 = h1 && c1 < 0 && ~c1 != k;
      const unsigned bi0 = __ballot_sync(0xffffffffu, i0), bi1 = __ballot_sync(0xffffffffu, i1);
      const unsigned bl0 = __ballot_sync(0xffffffffu, l0), bl1 = __ballot_sync(0xffffffffu, l1);
      int pi = ncnt + __popc(bi0 & lt) + __popc(bi1 & lt);
      if (i0) {
        if (pi < kFrontier) nxt[pi] = c0;
        ++pi;
      }
      if (i1 && pi < kFrontier) nxt[pi] = c1;
      ncnt += __popc(bi0) + __popc(bi1);
      int pl = nc + __popc(bl0 & lt) + __popc(bl1 & lt);
      if (l0) {
        if (pl < kCand) cand[pl] = ~c0;
        ++pl;
      }
      if (l1 && pl < kCand) cand[pl] = ~c1;
      nc += __popc(bl0) + __popc(bl1);
    }
    __syncwarp();
    if (__any_sync(0xffffffffu, bad) || ncnt > kFrontier || nc > cap) return -1;
    int* t = cur;
    cur = nxt;
    nxt = t;
    cnt = ncnt;
  }
  return nc;
}

// target_visible_pp over the 4-wide tree: each binary node at even depth
// holds its (up to) four grandchildren, or a child leaf in place of two, as
// one 128-byte record (boxes as four lanes of SoA float4s, then the four child
// codes; an empty slot has an inverted box). A step tests four boxes, goes on
// with the nearest hit and stacks the others, so a ray takes about half the
// dependent node fetches of the binary walk. The leaves tested, and the
// answer, are those of target_visible: a leaf is reached iff its binary
// ancestors' boxes and its own all pass, and the grandchild boxes are the same
// boxes the binary walk tests.

__device__ __forceinline__ bool target_visible_pp4(const Scene& sc, int b, int n,
                                                   const Target& tg, fv3 o, uint32_t* status) {
  constexpr int kDone = INT_MIN;
  const int k = tg.k;
  const fv3 D = xsub3(tg.c, o);
  const float dist = xlen(D);
  if (!(dist >= 1e-6f)) return false;
  const fv3 dir = mkv(xdiv(D.x, dist), xdiv(D.y, dist), xdiv(D.z, dist));
  const float tmax = xadd(xmul(dist, 1.01f), 1e-3f);
  const int f = tg.f;
  float tf;
  if (!tri_hit(tg.a0, tg.a1, tg.a2, tg.a3, o, dir, tmax, tf)) return false;
  if (n == 1) return true;
  const fv3 inv = mkv(safe_inv(dir.x), safe_inv(dir.y), safe_inv(dir.z));
  const fv3 oinv = mkv(o.x * inv.x, o.y * inv.y, o.z * inv.z);
  const float4* wb = sc.wide + (size_t)b * sc.F * 8;
  int stack[64];
  int sp = 0;
  auto push = [&](int v) {
    if (sp < 64) stack[sp++] = v;
    else atomicOr(status, kStatusTraversalCap);
  };
  auto pop = [&]() { return sp > 0 ? stack[--sp] : kDone; };
  int node = 0;
  int leaf = kDone;
  const int cap = 2 * n + 64;
  int it = 0;
  while (node != kDone) {
    while (node >= 0) {
      if (++it > cap || node >= n - 1) {
        atomicOr(status, kStatusTraversalCap);
        return true;
      }
      const float4* w = wb + (size_t)node * 8;
      const float4 lx = __ldg(w), ly = __ldg(w + 1), lz = __ldg(w + 2);
      const float4 hx = __ldg(w + 3), hy = __ldg(w + 4), hz = __ldg(w + 5);
      const float4 cc = __ldg(w + 6);
      const int c0 = __float_as_int(cc.x), c1 = __float_as_int(cc.y);
      const int c2 = __float_as_int(cc.z), c3 = __float_as_int(cc.w);
      float t0, t1, t2, t3;
      const bool h0 = slab(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, inv, oinv, tf, t0);
      const bool h1 = slab(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, inv, oinv, tf, t1) &&
                      c1 != kWideEmpty;
      const bool h2 = slab(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, inv, oinv, tf, t2) &&
                      c2 != kWideEmpty;
      const bool h3 = slab(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, inv, oinv, tf, t3) &&
                      c3 != kWideEmpty;
      // the nearest hit goes on; the other hits are stacked
      float best = INFINITY;
      int next = kDone;
      if (h0 && t0 < best) { best = t0; next = c0; }
      if (h1 && t1 < best) { best = t1; next = c1; }
      if (h2 && t2 < best) { best = t2; next = c2; }
      if (h3 && t3 < best) { best = t3; next = c3; }
      if (h3 && next != c3) push(c3);
      if (h2 && next != c2) push(c2);
      if (h1 && next != c1) push(c1);
      if (h0 && next != c0) push(c0);
      node = next != kDone ? next : pop();
      if (node < 0 && node != kDone && leaf == kDone) {
        leaf = node;
        node = pop();
      }
      if (!__any_sync(__activemask(), leaf == kDone)) break;
    }
    while (leaf != kDone) {
      const int kk = ~leaf;
      if (kk != k) {
        if (kk < 0 || kk >= n) {
          atomicOr(status, kStatusTraversalCap);
        } else {
          const float4* q = tri_at(sc, b, kk);
          const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3);
          float tq;
          if (tri_hit(q0, q1, q2, q3, o, dir, tmax, tq) &&
              (tq < tf || (tq == tf && __float_as_int(q3.w) < f)))
            return false;
        }
      }
      leaf = kDone;
      if (node < 0 && node != kDone) {
        leaf = node;
        node = pop();
      }
    }
  }
  return true;
}

// Warp-cooperative visibility of 32 targets seen from one wall point: lane i
// holds the ray from o to the centroid of its target (valid lanes only). The
// warp walks the BVH as one packet: it enters a node when the slab test of any
// still-undecided lane passes, and each lane tests a leaf triangle only when
// its own slab test of that leaf passes. Every node a lane's own walk would
// enter is entered, so each lane meets every occluder its own walk meets and
// the answer per lane is the one target_visible gives (no occluder can be
// invented: occlusion is decided by the exact triangle test alone). Node and
// leaf records are read at one address per warp; the stack is warp-uniform and
// held in registers, entry i in lane i % 32. All 32 lanes must call this.
__device__ __forceinline__ bool packet_visible(const Scene& sc, int b, int n, bool valid,
                                               const Target& tg, fv3 o, uint32_t* status) {
  constexpr uint32_t kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  bool active = false;
  fv3 dir = mkv(1.f, 0.f, 0.f);
  float tmax = 0.f, tf = 0.f;
  if (valid) {
    const fv3 D = xsub3(tg.c, o);
    const float dist = xlen(D);
    if (dist >= 1e-6f) {
      dir = mkv(xdiv(D.x, dist), xdiv(D.y, dist), xdiv(D.z, dist));
      tmax = xadd(xmul(dist, 1.01f), 1e-3f);
      active = tri_hit(tg.a0, tg.a1, tg.a2, tg.a3, o, dir, tmax, tf);
    }
  }
  if (n == 1) return active;
  bool vis = active;
  const fv3 inv = mkv(safe_inv(dir.x), safe_inv(dir.y), safe_inv(dir.z));
  const fv3 oinv = mkv(o.x * inv.x, o.y * inv.y, o.z * inv.z);
  const int k = tg.k, f = tg.f;
  auto occludes = [&](int kk) -> bool {
    if (kk == k) return false;
    if (kk < 0 || kk >= n) {
      atomicOr(status, kStatusTraversalCap);
      return false;
    }
    const float4* q = tri_at(sc, b, kk);
    const float4 q0 = __ldg(q), q1 = __ldg(q + 1), q2 = __ldg(q + 2), q3 = __ldg(q + 3);
    float tq;
    if (!tri_hit(q0, q1, q2, q3, o, dir, tmax, tq)) return false;
    return tq < tf || (tq == tf && __float_as_int(q3.w) < f);
  };
  int s_lo = 0, s_hi = 0;  // stack entries [0, 32) and [32, 64), one per lane
  int sp = 0, node = 0;
  const int cap = 2 * n + 64;
  for (int it = 0;; ++it) {
    if (__ballot_sync(kAll, active) == 0) break;
    if (it >= cap || node < 0 || node >= n - 1) {  // malformed tree (warp-uniform)
      if (lane == 0) atomicOr(status, kStatusTraversalCap);
      break;
    }
    const float4* nd = node_at(sc, b, node);
    const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3);
    float tn0 = 0.f, tn1 = 0.f;
    bool h0 = active && slab(n0.x, n0.y, n2.x, n0.z, n0.w, n2.z, inv, oinv, tf, tn0);
    bool h1 = active && slab(n1.x, n1.y, n2.y, n1.z, n1.w, n2.w, inv, oinv, tf, tn1);
    const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
    if (c0 < 0) {
      if (h0 && occludes(~c0)) active = vis = false;
      h0 = false;
    }
    if (c1 < 0) {
      if (h1 && occludes(~c1)) active = vis = false;
      h1 = false;
    }
    const uint32_t m0 = __ballot_sync(kAll, h0), m1 = __ballot_sync(kAll, h1);
    if (m0 && m1) {
      // nearer child first, by lane vote
      const uint32_t pref0 = __ballot_sync(kAll, h0 && (!h1 || tn0 <= tn1));
      const bool first0 = 2 * __popc(pref0) >= __popc(m0 | m1);
      const int later = first0 ? c1 : c0;
      if (sp < 64) {
        if (lane == (sp & 31)) {
          if (sp < 32) s_lo = later;
          else s_hi = later;
        }
        ++sp;
      } else if (lane == 0) {
        atomicOr(status, kStatusTraversalCap);
      }
      node = first0 ? c0 : c1;
    } else if (m0) {
      node = c0;
    } else if (m1) {
      node = c1;
    } else {
      if (sp == 0) break;
      --sp;
      node = __shfl_sync(kAll, sp < 32 ? s_lo : s_hi, sp & 31);
    }
  }
  return vis;
}

}  // namespace mesh
}  // namespace totri
