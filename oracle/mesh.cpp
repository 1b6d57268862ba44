// Oracle: CPU restatement of the mesh transient renderer (confocal and
// exhaustive, forward and vertex/albedo gradient).
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h). Follows, per pair:
//   forward  src/render/program/mesh_confocal_forward_optix.cu:18-129
//            src/render/program/mesh_exhaustive_forward_optix.cu:18-169
//   gradient src/render/program/mesh_confocal_grad_verts_optix.cu:18-190
//            src/render/program/mesh_exhaustive_grad_verts_optix.cu:18-248
//   math     src/render/program/mesh_common.h:28-660 (LinearInterp,
//            AreaTrapezoid, DrawTrapezoid(Grad), normal_grad_triangle,
//            Alpha{Confocal,Exhaustive}{,GradVerts,GradMaterial})
//   faces    src/common/optix.cu:18-30,55-58 (the first face holding a
//            negative index ends the face list)
//
// Visibility replaces the closed OptiX closest-hit query with an explicit FP32
// ray-triangle test (Moller-Trumbore plus a hit-point box check) evaluated by
// brute force over every face; the CUDA path must reproduce these masks
// bit-exactly through its BVH.
#include <algorithm>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle_common.h"

using namespace oracle;

namespace {

struct Tri {
  f3 v0, e1, e2;  // e1 = v1 - v0, e2 = v2 - v0 in FP32, original vertex order
  f3 lo, hi;      // face AABB grown by delta (hit points must lie inside)
};

struct Mesh {
  long n = 0;                  // number of faces before the first invalid one
  std::vector<int64_t> idx;    // [n][3]
  std::vector<f3> v[3];        // original vertex positions per face
  std::vector<f3> c;           // FP32 centroids
  std::vector<Tri> tri;
};

long count_valid_faces(const int64_t* faces, long F, long V) {
  for (long f = 0; f < F; ++f) {
    for (int k = 0; k < 3; ++k) {
      const int64_t i = faces[3 * f + k];
      if (i < 0 || i >= V) return f;
    }
  }
  return F;
}

Mesh prepare(const float* verts, long V, const int64_t* faces, long F) {
  Mesh m;
  m.n = count_valid_faces(faces, F, V);
  m.idx.assign(faces, faces + 3 * m.n);
  for (int k = 0; k < 3; ++k) m.v[k].resize(m.n);
  m.c.resize(m.n);
  m.tri.resize(m.n);
  // Scene scale: the largest coordinate magnitude of any referenced vertex.
  float scale = 0.f;
  for (long f = 0; f < m.n; ++f) {
    for (int k = 0; k < 3; ++k) {
      const float* p = verts + 3 * m.idx[3 * f + k];
      m.v[k][f] = mk(p[0], p[1], p[2]);
      for (int a = 0; a < 3; ++a) {
        const float q = std::fabs(p[a]);
        if (q > scale) scale = q;
      }
    }
  }
  const float delta = std::ldexp(scale, -12);
  for (long f = 0; f < m.n; ++f) {
    const f3 a = m.v[0][f], b = m.v[1][f], cc = m.v[2][f];
    m.c[f] = centroid_e(a, b, cc);
    Tri& t = m.tri[f];
    t.v0 = a;
    t.e1 = sub(b, a);
    t.e2 = sub(cc, a);
    t.lo = mk(std::min(std::min(a.x, b.x), cc.x) - delta,
              std::min(std::min(a.y, b.y), cc.y) - delta,
              std::min(std::min(a.z, b.z), cc.z) - delta);
    t.hi = mk(std::max(std::max(a.x, b.x), cc.x) + delta,
              std::max(std::max(a.y, b.y), cc.y) + delta,
              std::max(std::max(a.z, b.z), cc.z) + delta);
  }
  return m;
}

// FP32 ray-triangle test. Two-sided; t in [0, tmax]; the hit point
// fma(t, d, o) must lie in the face's grown AABB.
bool tri_hit(const Tri& tr, f3 o, f3 d, float tmax, float& t_out) {
  const f3 p = cross_e(d, tr.e2);
  const float det = dot_e(tr.e1, p);
  if (det == 0.f) return false;
  const float inv = 1.f / det;
  const f3 tv = sub(o, tr.v0);
  const float u = dot_e(tv, p) * inv;
  if (!(u >= 0.f && u <= 1.f)) return false;
  const f3 q = cross_e(tv, tr.e1);
  const float v = dot_e(d, q) * inv;
  if (!(v >= 0.f && u + v <= 1.f)) return false;
  const float t = dot_e(tr.e2, q) * inv;
  if (!(t >= 0.f && t <= tmax)) return false;
  const float px = std::fma(t, d.x, o.x);
  const float py = std::fma(t, d.y, o.y);
  const float pz = std::fma(t, d.z, o.z);
  if (!(px >= tr.lo.x && px <= tr.hi.x && py >= tr.lo.y && py <= tr.hi.y &&
        pz >= tr.lo.z && pz <= tr.hi.z))
    return false;
  t_out = t;
  return true;
}

// Face f is visible from wall point o iff the closest hit (lowest face index
// on equal t) of the ray o -> centroid(f) within [0, 1.01 d + 1e-3] is f
// (mesh_confocal_forward_optix.cu:42-65).
bool visible(const Mesh& m, long f, f3 o) {
  const f3 D = sub(m.c[f], o);
  const float dist = len_e(D);
  if (!(dist >= 1e-6f)) return false;
  const f3 dir = mk(D.x / dist, D.y / dist, D.z / dist);
  const float tmax = dist * 1.01f + 1e-3f;
  float tf;
  if (!tri_hit(m.tri[f], o, dir, tmax, tf)) return false;
  for (long g = 0; g < m.n; ++g) {
    if (g == f) continue;
    float tg;
    if (tri_hit(m.tri[g], o, dir, tmax, tg) && (tg < tf || (tg == tf && g < f)))
      return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// CPU BVH over the same faces. Leaf boxes are the hit-point boxes grown by
// another delta, so every accepted hit point lies at least delta inside its
// leaf box; that margin dominates the rounding of the float slab test, so the
// walk finds every occluder that the brute-force loop finds and the result is
// identical.

struct CpuNode {
  float lo[3], hi[3];
  int left, right;   // children (internal) or -1
  int first, count;  // face range in order[] (leaves)
};

struct CpuBvh {
  std::vector<CpuNode> nodes;
  std::vector<int> order;
};

int build_node(CpuBvh& b, const Mesh& m, float delta, int first, int count) {
  CpuNode nd;
  for (int a = 0; a < 3; ++a) {
    nd.lo[a] = 3.0e38f;
    nd.hi[a] = -3.0e38f;
  }
  float clo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, chi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int i = first; i < first + count; ++i) {
    const Tri& t = m.tri[b.order[i]];
    const float lo[3] = {t.lo.x - delta, t.lo.y - delta, t.lo.z - delta};
    const float hi[3] = {t.hi.x + delta, t.hi.y + delta, t.hi.z + delta};
    const f3 c = m.c[b.order[i]];
    const float cc[3] = {c.x, c.y, c.z};
    for (int a = 0; a < 3; ++a) {
      nd.lo[a] = std::min(nd.lo[a], lo[a]);
      nd.hi[a] = std::max(nd.hi[a], hi[a]);
      clo[a] = std::min(clo[a], cc[a]);
      chi[a] = std::max(chi[a], cc[a]);
    }
  }
  const int idx = (int)b.nodes.size();
  b.nodes.push_back(nd);
  if (count <= 4) {
    b.nodes[idx].left = b.nodes[idx].right = -1;
    b.nodes[idx].first = first;
    b.nodes[idx].count = count;
    return idx;
  }
  int axis = 0;
  for (int a = 1; a < 3; ++a)
    if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
  const int mid = first + count / 2;
  auto key = [&](int f) { const f3 c = m.c[f]; return axis == 0 ? c.x : (axis == 1 ? c.y : c.z); };
  std::nth_element(b.order.begin() + first, b.order.begin() + mid,
                   b.order.begin() + first + count,
                   [&](int x, int y) { return key(x) < key(y) || (key(x) == key(y) && x < y); });
  const int l = build_node(b, m, delta, first, mid - first);
  const int r = build_node(b, m, delta, mid, first + count - mid);
  b.nodes[idx].left = l;
  b.nodes[idx].right = r;
  b.nodes[idx].first = b.nodes[idx].count = 0;
  return idx;
}

CpuBvh build_bvh(const Mesh& m, float delta) {
  CpuBvh b;
  b.order.resize(m.n);
  for (long i = 0; i < m.n; ++i) b.order[i] = (int)i;
  if (m.n > 0) build_node(b, m, delta, 0, (int)m.n);
  return b;
}

float scene_delta(const Mesh& m) {
  float scale = 0.f;
  for (long f = 0; f < m.n; ++f)
    for (int k = 0; k < 3; ++k) {
      const f3 v = m.v[k][f];
      for (float q : {std::fabs(v.x), std::fabs(v.y), std::fabs(v.z)})
        if (q > scale) scale = q;
    }
  return std::ldexp(scale, -12);
}

inline bool slab_cpu(const CpuNode& nd, f3 inv, f3 o, float limit) {
  const float tx0 = (nd.lo[0] - o.x) * inv.x, tx1 = (nd.hi[0] - o.x) * inv.x;
  const float ty0 = (nd.lo[1] - o.y) * inv.y, ty1 = (nd.hi[1] - o.y) * inv.y;
  const float tz0 = (nd.lo[2] - o.z) * inv.z, tz1 = (nd.hi[2] - o.z) * inv.z;
  const float tn = std::max(std::max(std::min(tx0, tx1), std::min(ty0, ty1)),
                            std::max(std::min(tz0, tz1), 0.f));
  const float tf = std::min(std::min(std::max(tx0, tx1), std::max(ty0, ty1)),
                            std::min(std::max(tz0, tz1), limit));
  return tn <= tf;
}

inline float safe_inv(float d) {
  return std::fabs(d) < 1e-20f ? std::copysign(1e20f, d) : 1.f / d;
}

bool visible_bvh(const Mesh& m, const CpuBvh& bvh, long f, f3 o) {
  const f3 D = sub(m.c[f], o);
  const float dist = len_e(D);
  if (!(dist >= 1e-6f)) return false;
  const f3 dir = mk(D.x / dist, D.y / dist, D.z / dist);
  const float tmax = dist * 1.01f + 1e-3f;
  float tf;
  if (!tri_hit(m.tri[f], o, dir, tmax, tf)) return false;
  const f3 inv = mk(safe_inv(dir.x), safe_inv(dir.y), safe_inv(dir.z));
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const CpuNode& nd = bvh.nodes[stack[--sp]];
    if (!slab_cpu(nd, inv, o, tf)) continue;
    if (nd.left < 0) {
      for (int i = nd.first; i < nd.first + nd.count; ++i) {
        const long g = bvh.order[i];
        if (g == f) continue;
        float tg;
        if (tri_hit(m.tri[g], o, dir, tmax, tg) && (tg < tf || (tg == tf && g < f)))
          return false;
      }
    } else if (sp + 2 <= 128) {
      stack[sp++] = nd.right;
      stack[sp++] = nd.left;
    }
  }
  return true;
}

// ---------------------------------------------------------------------------
// Value arithmetic in precision T.

template <typename T>
struct v3 {
  T x, y, z;
};
template <typename T>
inline v3<T> operator+(v3<T> a, v3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
inline v3<T> operator-(v3<T> a, v3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
inline v3<T> operator*(T a, v3<T> b) { return {a * b.x, a * b.y, a * b.z}; }
template <typename T>
inline v3<T> operator/(v3<T> a, T b) { return {a.x / b, a.y / b, a.z / b}; }
template <typename T>
inline T dot(v3<T> a, v3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T>
inline v3<T> cross(v3<T> a, v3<T> b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Euclidean norm: FP32 mode stands in for CUDA's norm3df with a
// double-evaluated, once-rounded result; FP64 mode is plain sqrt.
inline float length(v3<float> a) {
  const double x = a.x, y = a.y, z = a.z;
  return (float)std::sqrt(x * x + y * y + z * z);
}
inline double length(v3<double> a) { return std::sqrt(dot(a, a)); }
template <typename T>
inline T length_sqr(v3<T> a) { return dot(a, a); }
inline float powT(float a, float e) { return std::pow(a, e); }
inline double powT(double a, double e) { return std::pow(a, e); }
template <typename T>
inline v3<T> cvt(f3 a) { return {(T)a.x, (T)a.y, (T)a.z}; }

template <typename T>
struct tri3 {  // one 3-vector per triangle vertex (reference vert3)
  v3<T> a, b, c;
};
template <typename T>
inline tri3<T> operator+(tri3<T> p, tri3<T> q) { return {p.a + q.a, p.b + q.b, p.c + q.c}; }
template <typename T>
inline tri3<T> operator-(tri3<T> p, tri3<T> q) { return {p.a - q.a, p.b - q.b, p.c - q.c}; }
template <typename T>
inline tri3<T> operator*(T s, tri3<T> p) { return {s * p.a, s * p.b, s * p.c}; }
template <typename T>
inline tri3<T> zero3() { return {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}; }
template <typename T>
inline tri3<T> same3(v3<T> v) { return {v, v, v}; }

// Jacobian-transpose of n = (v1-v0) x (v2-v0) applied to vec, per vertex
// (mesh_common.h:358-379).
template <typename T>
tri3<T> normal_grad(v3<T> a, v3<T> b, v3<T> vec) {
  tri3<T> r;
  r.a = {(b.z - a.z) * vec.y + (-b.y + a.y) * vec.z,
         (-b.z + a.z) * vec.x + (b.x - a.x) * vec.z,
         (b.y - a.y) * vec.x + (-b.x + a.x) * vec.y};
  r.b = {(-b.z) * vec.y + (b.y) * vec.z, (b.z) * vec.x + (-b.x) * vec.z,
         (-b.y) * vec.x + (b.x) * vec.y};
  r.c = {(a.z) * vec.y + (-a.y) * vec.z, (-a.z) * vec.x + (a.x) * vec.z,
         (a.y) * vec.x + (-a.x) * vec.y};
  return r;
}

// AreaTrapezoid (mesh_common.h:28-51): (b1-b0) * line(0.5*(b0+b1)).
template <typename T>
inline T area(T b0, T b1, T x0, T y0, T x1, T y1) {
  return (b1 - b0) * (y0 + (T(0.5) * (b0 + b1) - x0) / (x1 - x0) * (y1 - y0));
}

// Accumulator for one wall column (confocal: stride S; exhaustive: S*L).
template <typename T>
struct Column {
  T* base;
  long stride;
  long nbins;
  bool in(long b) const { return b >= 0 && b < nbins; }
  void add(long b, T v) const { base[b * stride] += v; }
};

// DrawTrapezoid (mesh_common.h:61-94 / 209-242) with the integer bins passed in
// (taken from the FP32 bin coordinates).
template <typename T>
void draw(const Column<T>& col, T ca, long ba, T ya, T cb, long bb, T yb) {
  if (ba == bb) {
    if (col.in(ba)) col.add(ba, T(0.5) * (cb - ca) * (ya + yb));
    return;
  }
  if (col.in(ba)) col.add(ba, area<T>(ca, T(ba + 1), ca, ya, cb, yb));
  const long lo = std::max<long>(ba + 1, 0), hi = std::min<long>(bb, col.nbins);
  for (long i = lo; i < hi; ++i) col.add(i, area<T>(T(i), T(i + 1), ca, ya, cb, yb));
  if (col.in(bb)) col.add(bb, area<T>(T(bb), cb, ca, ya, cb, yb));
}

// DrawTrapezoidGrad (mesh_common.h:104-199 / 252-347).
template <typename T, typename G>
void draw_grad(const G& grad_at, long nbins, T& p0, tri3<T>& p1, T c0, long b0,
               T y0, T c1, long b1, T y1, const tri3<T>& dc0, const tri3<T>& dc1,
               const tri3<T>& dy0, const tri3<T>& dy1) {
  auto in = [&](long b) { return b >= 0 && b < nbins; };
  const T span = c1 - c0;
  const T span2 = span * span;
  if (b0 == b1) {
    if (in(b0)) {
      const T g = grad_at(b0);
      p0 += g * (T(0.5) * (c1 - c0) * (y0 + y1));
      p1 = p1 + g * ((T(0.5) * (y0 + y1)) * (dc1 - dc0) +
                     (T(0.5) * (c1 - c0)) * (dy0 + dy1));
    }
    return;
  }
  const tri3<T> kslope = (c1 - c0) * (dy1 - dy0) - (y1 - y0) * (dc1 - dc0);
  if (in(b0)) {
    const T g = grad_at(b0);
    p0 += g * area<T>(c0, T(b0 + 1), c0, y0, c1, y1);
    const T base = T(b0 + 1) - c0;
    p1 = p1 + g * (base * dy0 - y0 * dc0 - (base * (y1 - y0) / span) * dc0 +
                   ((T(0.5) * base * base) / span2) * kslope);
  }
  const long lo = std::max<long>(b0 + 1, 0), hi = std::min<long>(b1, nbins);
  for (long i = lo; i < hi; ++i) {
    const T g = grad_at(i);
    p0 += g * area<T>(T(i), T(i + 1), c0, y0, c1, y1);
    p1 = p1 + g * (dy0 - ((y1 - y0) / span) * dc0 +
                   (((T(i) + T(0.5)) - c0) / span2) * kslope);
  }
  if (in(b1)) {
    const T g = grad_at(b1);
    p0 += g * area<T>(T(b1), c1, c0, y0, c1, y1);
    const T mid = T(0.5) * (T(b1) + c1) - c0;
    p1 = p1 + g * ((y0 + mid * (y1 - y0) / span) * dc1 +
                   (c1 - T(b1)) * (dy0 + ((y1 - y0) / span) * (T(0.5) * dc1 - dc0) +
                                   (mid / span2) * kslope));
  }
}

// Per-face albedo: mean of channel 0 over the three vertices (1 when M == 0).
template <typename T>
T albedo(const float* material, long M, const int64_t* ix) {
  if (M <= 0) return T(1);
  const float third = 1.f / 3.f;
  if (sizeof(T) == sizeof(float))
    return (T)(third * ((material[ix[0] * M] + material[ix[1] * M]) + material[ix[2] * M]));
  return (T(material[ix[0] * M]) + T(material[ix[1] * M]) + T(material[ix[2] * M])) / T(3);
}

template <typename T>
v3<T> centroid_T(const Mesh& m, long f) {
  if (sizeof(T) == sizeof(float)) return cvt<T>(m.c[f]);
  const v3<T> a = cvt<T>(m.v[0][f]), b = cvt<T>(m.v[1][f]), c = cvt<T>(m.v[2][f]);
  return (T(1) / T(3)) * ((a + b) + c);
}

// One pair (or triple) worth of geometry with its FP32 decisions taken.
template <typename T>
struct PairGeom {
  bool ok = false;
  int perm[3] = {0, 1, 2};
  long bin[3];
  T c[3];       // bin coordinates in precision T
  v3<T> v[3];   // sorted vertices
  T ds[3], dl[3];  // distances to the scan / laser point (precision T)
};

// Sorts the three vertices by FP32 path length (mesh_confocal_forward_optix.cu:86-101).
inline void sort3(float d[3], int p[3]) {
  if (d[0] > d[1]) { std::swap(d[0], d[1]); std::swap(p[0], p[1]); }
  if (d[1] > d[2]) { std::swap(d[1], d[2]); std::swap(p[1], p[2]); }
  if (d[0] > d[1]) { std::swap(d[0], d[1]); std::swap(p[0], p[1]); }
}

// Confocal geometry for face f and scan point sp with origin term od32 (FP32)
// and odT (precision T).
template <typename T>
PairGeom<T> confocal_geom(const Mesh& m, long f, f3 sp, float od32, T odT, float bw,
                          float bo) {
  PairGeom<T> g;
  float d[3];
  for (int k = 0; k < 3; ++k) d[k] = len_e(sub(m.v[k][f], sp));
  sort3(d, g.perm);
  const v3<T> s = cvt<T>(sp);
  for (int k = 0; k < 3; ++k) {
    const float cb = ((2.f * d[k] + od32) - bo) / bw;
    g.bin[k] = bin_of(cb);
    g.v[k] = cvt<T>(m.v[g.perm[k]][f]);
    if (sizeof(T) == sizeof(float)) {
      g.ds[k] = (T)d[k];
      g.c[k] = (T)cb;
    } else {
      g.ds[k] = length(g.v[k] - s);
      g.c[k] = ((T(2) * g.ds[k] + odT) - T(bo)) / T(bw);
    }
  }
  return g;
}

template <typename T>
T alpha_confocal(const v3<T> v[3], v3<T> c, v3<T> s, T rho) {
  const v3<T> n = cross(v[1] - v[0], v[2] - v[0]);
  const v3<T> r = c - s;
  const T a = T(1) / length(n) * powT(length(r), T(-8)) *
              powT(std::max(T(0), r.z), T(2)) * powT(std::fabs(dot(n, r)), T(2));
  if (sizeof(T) == sizeof(float)) return (T)(1.e2 * (double)a * (double)rho);
  return T(100) * a * rho;
}

template <typename T>
T alpha_exhaustive(const v3<T> v[3], v3<T> c, v3<T> s, v3<T> l, T rho) {
  const v3<T> n = cross(v[1] - v[0], v[2] - v[0]);
  const v3<T> rs = c - s, rl = c - l;
  const T a = T(1) / length(n) * powT(length(rs), T(-4)) * powT(length(rl), T(-4)) *
              std::max(T(0), rs.z) * std::max(T(0), rl.z) * std::fabs(dot(n, rs)) *
              std::fabs(dot(n, rl));
  if (sizeof(T) == sizeof(float)) return (T)(1.e2 * (double)a * (double)rho);
  return T(100) * a * rho;
}

// Splats the tent for one unit of work (mesh_confocal_forward_optix.cu:114-129).
template <typename T>
void splat(const Column<T>& col, const PairGeom<T>& g, T alpha) {
  if (g.bin[0] >= col.nbins || g.bin[2] < 0) return;
  if (g.bin[0] == g.bin[2]) {
    col.add(g.bin[0], alpha);
    return;
  }
  const T yc = T(2) * alpha / (g.c[2] - g.c[0]);
  draw<T>(col, g.c[0], g.bin[0], T(0), g.c[1], g.bin[1], yc);
  draw<T>(col, g.c[1], g.bin[1], yc, g.c[2], g.bin[2], T(0));
}

template <typename T>
void confocal_forward(const Mesh& m, const float* material, long M, const float* sp,
                      long S, const float* so, const uint8_t* vis, long F_stride,
                      long nbins, float bw, float bo, double* out) {
  std::vector<T> acc((size_t)nbins * S, T(0));
#pragma omp parallel for schedule(dynamic, 4)
  for (long s = 0; s < S; ++s) {
    const f3 p = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
    float od32 = 0.f;
    T odT = T(0);
    if (so) {
      const f3 o = mk(so[3 * s], so[3 * s + 1], so[3 * s + 2]);
      od32 = 2.f * len_e(sub(p, o));
      odT = (sizeof(T) == sizeof(float)) ? (T)od32 : T(2) * length(cvt<T>(p) - cvt<T>(o));
    }
    const Column<T> col{acc.data() + s, S, nbins};
    for (long f = 0; f < m.n; ++f) {
      if (!vis[s * F_stride + f]) continue;
      const PairGeom<T> g = confocal_geom<T>(m, f, p, od32, odT, bw, bo);
      const T rho = albedo<T>(material, M, &m.idx[3 * f]);
      const T alpha = alpha_confocal<T>(g.v, centroid_T<T>(m, f), cvt<T>(p), rho);
      if (!(alpha > T(0))) continue;
      splat<T>(col, g, alpha);
    }
  }
  for (size_t i = 0; i < acc.size(); ++i) out[i] = (double)acc[i];
}

// Scatters one pair's triangle gradient to the vertex and albedo gradients
// (mesh_confocal_grad_verts_optix.cu:316-332).
template <typename T>
void scatter_grad(T* vg, long vg_ch, T* mg, long M, const int64_t* ix, const int perm[3],
                  const tri3<T>& dtri, T dmat) {
  const v3<T> dv[3] = {dtri.a, dtri.b, dtri.c};
  for (int k = 0; k < 3; ++k) {
    const int64_t vi = ix[perm[k]];
    if (vg_ch > 0) {
      vg[vi * 3 + 0] += dv[k].x;
      vg[vi * 3 + 1] += dv[k].y;
      vg[vi * 3 + 2] += dv[k].z;
    }
    if (M > 0) mg[vi * M + 0] += (T(1) / T(3)) * dmat;
  }
}

template <typename T>
void confocal_grad(const Mesh& m, const float* material, long M, const float* sp, long S,
                   const float* so, const uint8_t* vis, long F_stride, long nbins, float bw,
                   float bo, const double* tgrad, long V, int want_verts, double* vgrad,
                   double* mgrad) {
  const long vg_ch = want_verts ? 3 : 0;
  std::vector<std::vector<T>> vgs, mgs;
#pragma omp parallel
  {
#pragma omp single
    {
      int nt = 1;
#ifdef _OPENMP
      nt = omp_get_num_threads();
#endif
      vgs.assign(nt, std::vector<T>(V * 3, T(0)));
      mgs.assign(nt, std::vector<T>(std::max<long>(V * M, 1), T(0)));
    }
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    T* vg = vgs[tid].data();
    T* mg = mgs[tid].data();
#pragma omp for schedule(dynamic, 4)
    for (long s = 0; s < S; ++s) {
      const f3 p = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
      const v3<T> pT = cvt<T>(p);
      float od32 = 0.f;
      T odT = T(0);
      if (so) {
        const f3 o = mk(so[3 * s], so[3 * s + 1], so[3 * s + 2]);
        od32 = 2.f * len_e(sub(p, o));
        odT = (sizeof(T) == sizeof(float)) ? (T)od32 : T(2) * length(pT - cvt<T>(o));
      }
      auto grad_at = [&](long b) { return (T)tgrad[b * S + s]; };
      for (long f = 0; f < m.n; ++f) {
        if (!vis[s * F_stride + f]) continue;
        const PairGeom<T> g = confocal_geom<T>(m, f, p, od32, odT, bw, bo);
        const T rho = albedo<T>(material, M, &m.idx[3 * f]);
        const v3<T> c = centroid_T<T>(m, f);
        const T alpha = alpha_confocal<T>(g.v, c, pT, rho);
        if (!(alpha > T(0))) continue;
        if (g.bin[0] >= nbins || g.bin[2] < 0) continue;
        // AlphaConfocalGradVerts (mesh_common.h:429-463)
        const v3<T> e1 = g.v[1] - g.v[0], e2 = g.v[2] - g.v[0];
        const v3<T> n = cross(e1, e2);
        const v3<T> r = c - pT;
        const v3<T> nw = {T(0), T(0), T(1)};
        tri3<T> lg = (T(-1) / length_sqr(n)) * normal_grad(e1, e2, n);
        lg = lg + (T(-8) / (T(3) * length_sqr(r))) * same3(r);
        lg = lg + (T(2) / (T(3) * dot(nw, r))) * same3(nw);
        lg = lg + (T(2) / dot(n, r)) * (normal_grad(e1, e2, r) + (T(1) / T(3)) * same3(n));
        const tri3<T> dalpha = alpha * lg;
        const T dalpha_dm = alpha / rho;
        tri3<T> dtri;
        T dmat;
        if (g.bin[0] == g.bin[2]) {
          const T gr = grad_at(g.bin[0]);
          dtri = gr * dalpha;
          dmat = gr * dalpha_dm;
        } else {
          T p0 = T(0);
          tri3<T> p1 = zero3<T>();
          const T span = g.c[2] - g.c[0];
          const T yc = T(2) / span;
          const T k = T(-4) / (T(bw) * span * span);
          const tri3<T> dyc = {k * ((g.v[0] - pT) / (-g.ds[0])), {0, 0, 0},
                               k * ((g.v[2] - pT) / g.ds[2])};
          tri3<T> dc0 = zero3<T>(), dc1 = zero3<T>(), dc2 = zero3<T>();
          dc0.a = (T(2) / (T(bw) * g.ds[0])) * (g.v[0] - pT);
          dc1.b = (T(2) / (T(bw) * g.ds[1])) * (g.v[1] - pT);
          dc2.c = (T(2) / (T(bw) * g.ds[2])) * (g.v[2] - pT);
          draw_grad<T>(grad_at, nbins, p0, p1, g.c[0], g.bin[0], T(0), g.c[1], g.bin[1], yc,
                       dc0, dc1, zero3<T>(), dyc);
          draw_grad<T>(grad_at, nbins, p0, p1, g.c[1], g.bin[1], yc, g.c[2], g.bin[2], T(0),
                       dc1, dc2, dyc, zero3<T>());
          dtri = p0 * dalpha + alpha * p1;
          dmat = dalpha_dm * p0;
        }
        scatter_grad<T>(vg, vg_ch, mg, M, &m.idx[3 * f], g.perm, dtri, dmat);
      }
    }
  }
  std::fill(vgrad, vgrad + V * vg_ch, 0.0);
  std::fill(mgrad, mgrad + V * M, 0.0);
  for (size_t t = 0; t < vgs.size(); ++t) {
    for (long i = 0; i < V * vg_ch; ++i) vgrad[i] += (double)vgs[t][i];
    for (long i = 0; i < V * M; ++i) mgrad[i] += (double)mgs[t][i];
  }
}

// ----------------------------- exhaustive ---------------------------------

template <typename T>
PairGeom<T> exhaustive_geom(const Mesh& m, long f, f3 sp, f3 lp, float od32, T odT,
                            float bw, float bo) {
  PairGeom<T> g;
  float d[3], ds32[3], dl32[3];
  for (int k = 0; k < 3; ++k) {
    ds32[k] = len_e(sub(m.v[k][f], sp));
    dl32[k] = len_e(sub(m.v[k][f], lp));
    d[k] = ds32[k] + dl32[k];
  }
  sort3(d, g.perm);
  const v3<T> s = cvt<T>(sp), l = cvt<T>(lp);
  for (int k = 0; k < 3; ++k) {
    const float cb = ((d[k] + od32) - bo) / bw;
    g.bin[k] = bin_of(cb);
    g.v[k] = cvt<T>(m.v[g.perm[k]][f]);
    if (sizeof(T) == sizeof(float)) {
      g.ds[k] = (T)ds32[g.perm[k]];
      g.dl[k] = (T)dl32[g.perm[k]];
      g.c[k] = (T)cb;
    } else {
      g.ds[k] = length(g.v[k] - s);
      g.dl[k] = length(g.v[k] - l);
      g.c[k] = (((g.ds[k] + g.dl[k]) + odT) - T(bo)) / T(bw);
    }
  }
  return g;
}

template <typename T>
void origin_terms(const float* sp, const float* so, long s, const float* lp,
                  const float* lo, long l, float& od32, T& odT) {
  od32 = 0.f;
  odT = T(0);
  if (so) {
    const f3 p = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
    const f3 o = mk(so[3 * s], so[3 * s + 1], so[3 * s + 2]);
    od32 = od32 + len_e(sub(p, o));
    odT = odT + ((sizeof(T) == sizeof(float)) ? (T)len_e(sub(p, o))
                                              : length(cvt<T>(p) - cvt<T>(o)));
  }
  if (lo) {
    const f3 p = mk(lp[3 * l], lp[3 * l + 1], lp[3 * l + 2]);
    const f3 o = mk(lo[3 * l], lo[3 * l + 1], lo[3 * l + 2]);
    od32 = od32 + len_e(sub(p, o));
    odT = odT + ((sizeof(T) == sizeof(float)) ? (T)len_e(sub(p, o))
                                              : length(cvt<T>(p) - cvt<T>(o)));
  }
  if (sizeof(T) == sizeof(float)) odT = (T)od32;
}

template <typename T>
void exhaustive_forward(const Mesh& m, const float* material, long M, const float* sp, long S,
                        const float* lp, long L, const float* so, const float* lo,
                        const uint8_t* vis_s, const uint8_t* vis_l, long F_stride,
                        long nbins, float bw, float bo, double* out) {
  std::vector<T> acc((size_t)nbins * S * L, T(0));
#pragma omp parallel for schedule(dynamic, 1)
  for (long s = 0; s < S; ++s) {
    const f3 p = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
    for (long l = 0; l < L; ++l) {
      const f3 q = mk(lp[3 * l], lp[3 * l + 1], lp[3 * l + 2]);
      float od32;
      T odT;
      origin_terms<T>(sp, so, s, lp, lo, l, od32, odT);
      const Column<T> col{acc.data() + s * L + l, S * L, nbins};
      for (long f = 0; f < m.n; ++f) {
        if (!vis_l[l * F_stride + f] || !vis_s[s * F_stride + f]) continue;
        const PairGeom<T> g = exhaustive_geom<T>(m, f, p, q, od32, odT, bw, bo);
        const T rho = albedo<T>(material, M, &m.idx[3 * f]);
        const T alpha =
            alpha_exhaustive<T>(g.v, centroid_T<T>(m, f), cvt<T>(p), cvt<T>(q), rho);
        if (!(alpha > T(0))) continue;  // also rejects NaN
        splat<T>(col, g, alpha);
      }
    }
  }
  for (size_t i = 0; i < acc.size(); ++i) out[i] = (double)acc[i];
}

template <typename T>
void exhaustive_grad(const Mesh& m, const float* material, long M, const float* sp, long S,
                     const float* lp, long L, const float* so, const float* lo,
                     const uint8_t* vis_s, const uint8_t* vis_l, long F_stride, long nbins,
                     float bw, float bo, const double* tgrad, long V, int want_verts,
                     double* vgrad, double* mgrad) {
  const long vg_ch = want_verts ? 3 : 0;
  std::vector<std::vector<T>> vgs, mgs;
#pragma omp parallel
  {
#pragma omp single
    {
      int nt = 1;
#ifdef _OPENMP
      nt = omp_get_num_threads();
#endif
      vgs.assign(nt, std::vector<T>(V * 3, T(0)));
      mgs.assign(nt, std::vector<T>(std::max<long>(V * M, 1), T(0)));
    }
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    T* vg = vgs[tid].data();
    T* mg = mgs[tid].data();
#pragma omp for schedule(dynamic, 1)
    for (long s = 0; s < S; ++s) {
      const f3 p = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
      const v3<T> pT = cvt<T>(p);
      for (long l = 0; l < L; ++l) {
        const f3 q = mk(lp[3 * l], lp[3 * l + 1], lp[3 * l + 2]);
        const v3<T> qT = cvt<T>(q);
        float od32;
        T odT;
        origin_terms<T>(sp, so, s, lp, lo, l, od32, odT);
        auto grad_at = [&](long b) { return (T)tgrad[(b * S + s) * L + l]; };
        for (long f = 0; f < m.n; ++f) {
          if (!vis_l[l * F_stride + f] || !vis_s[s * F_stride + f]) continue;
          const PairGeom<T> g = exhaustive_geom<T>(m, f, p, q, od32, odT, bw, bo);
          const T rho = albedo<T>(material, M, &m.idx[3 * f]);
          const v3<T> c = centroid_T<T>(m, f);
          const T alpha = alpha_exhaustive<T>(g.v, c, pT, qT, rho);
          if (!(alpha > T(0))) continue;
          if (g.bin[0] >= nbins || g.bin[2] < 0) continue;
          // AlphaExhaustiveGradVerts (mesh_common.h:549-630), including the
          // reference's swapped wall normals (both are (0,0,1)).
          const v3<T> e1 = g.v[1] - g.v[0], e2 = g.v[2] - g.v[0];
          const v3<T> n = cross(e1, e2);
          const v3<T> rs = c - pT, rl = c - qT;
          const v3<T> nw = {T(0), T(0), T(1)};
          tri3<T> lg = (T(-1) / length_sqr(n)) * normal_grad(e1, e2, n);
          lg = lg + (T(-4) / (T(3) * length_sqr(rs))) * same3(rs);
          lg = lg + (T(-4) / (T(3) * length_sqr(rl))) * same3(rl);
          lg = lg + (T(1) / (T(3) * dot(nw, rs))) * same3(nw);
          lg = lg + (T(1) / (T(3) * dot(nw, rl))) * same3(nw);
          const T dns = dot(n, rs), dnl = dot(n, rl);
          const T sgs = dns > 0 ? T(1) : (dns == 0 ? T(0) : T(-1));
          const T sgl = dnl > 0 ? T(1) : (dnl == 0 ? T(0) : T(-1));
          lg = lg + (sgs / std::fabs(dns)) * (normal_grad(e1, e2, rs) + (T(1) / T(3)) * same3(n));
          lg = lg + (sgl / std::fabs(dnl)) * (normal_grad(e1, e2, rl) + (T(1) / T(3)) * same3(n));
          const tri3<T> dalpha = alpha * lg;
          const T dalpha_dm = alpha / rho;
          tri3<T> dtri;
          T dmat;
          if (g.bin[0] == g.bin[2]) {
            const T gr = grad_at(g.bin[0]);
            dtri = gr * dalpha;
            dmat = gr * dalpha_dm;
          } else {
            T p0 = T(0);
            tri3<T> p1 = zero3<T>();
            const T span = g.c[2] - g.c[0];
            const T yc = T(2) / span;
            const T k = T(-2) / (T(bw) * span * span);
            const tri3<T> dyc = {
                k * ((g.v[0] - qT) / (-g.dl[0]) + (g.v[0] - pT) / (-g.ds[0])),
                {0, 0, 0},
                k * ((g.v[2] - qT) / g.dl[2] + (g.v[2] - pT) / g.ds[2])};
            auto dcv = [&](int i) {
              return (T(1) / (T(bw) * g.dl[i])) * (g.v[i] - qT) +
                     (T(1) / (T(bw) * g.ds[i])) * (g.v[i] - pT);
            };
            tri3<T> dc0 = zero3<T>(), dc1 = zero3<T>(), dc2 = zero3<T>();
            dc0.a = dcv(0);
            dc1.b = dcv(1);
            dc2.c = dcv(2);
            draw_grad<T>(grad_at, nbins, p0, p1, g.c[0], g.bin[0], T(0), g.c[1], g.bin[1],
                         yc, dc0, dc1, zero3<T>(), dyc);
            draw_grad<T>(grad_at, nbins, p0, p1, g.c[1], g.bin[1], yc, g.c[2], g.bin[2],
                         T(0), dc1, dc2, dyc, zero3<T>());
            dtri = p0 * dalpha + alpha * p1;
            dmat = dalpha_dm * p0;
          }
          scatter_grad<T>(vg, vg_ch, mg, M, &m.idx[3 * f], g.perm, dtri, dmat);
        }
      }
    }
  }
  std::fill(vgrad, vgrad + V * vg_ch, 0.0);
  std::fill(mgrad, mgrad + V * M, 0.0);
  for (size_t t = 0; t < vgs.size(); ++t) {
    for (long i = 0; i < V * vg_ch; ++i) vgrad[i] += (double)vgs[t][i];
    for (long i = 0; i < V * M; ++i) mgrad[i] += (double)mgs[t][i];
  }
}

}  // namespace

extern "C" {

long oracle_mesh_count_faces(const int64_t* faces, long F, long V) {
  return count_valid_faces(faces, F, V);
}

// vis[p * F + f] for every wall point p and face f (faces past the valid
// prefix are 0).
int oracle_mesh_visibility(const float* verts, long V, const int64_t* faces, long F,
                           const float* points, long P, uint8_t* vis) {
  const Mesh m = prepare(verts, V, faces, F);
  std::memset(vis, 0, (size_t)P * F);
#pragma omp parallel for collapse(2) schedule(dynamic, 64)
  for (long p = 0; p < P; ++p)
    for (long f = 0; f < m.n; ++f)
      vis[p * F + f] = visible(m, f, mk(points[3 * p], points[3 * p + 1], points[3 * p + 2]));
  return 0;
}

// Same masks as oracle_mesh_visibility, computed through a CPU BVH.
int oracle_mesh_visibility_bvh(const float* verts, long V, const int64_t* faces, long F,
                               const float* points, long P, uint8_t* vis) {
  const Mesh m = prepare(verts, V, faces, F);
  const CpuBvh bvh = build_bvh(m, scene_delta(m));
  std::memset(vis, 0, (size_t)P * F);
#pragma omp parallel for collapse(2) schedule(dynamic, 256)
  for (long p = 0; p < P; ++p)
    for (long f = 0; f < m.n; ++f)
      vis[p * F + f] =
          visible_bvh(m, bvh, f, mk(points[3 * p], points[3 * p + 1], points[3 * p + 2]));
  return 0;
}

// Visibility for an explicit list of (point, face) pairs.
int oracle_mesh_visibility_pairs(const float* verts, long V, const int64_t* faces, long F,
                                 const float* points, const int64_t* pair_p,
                                 const int64_t* pair_f, long n, uint8_t* out) {
  const Mesh m = prepare(verts, V, faces, F);
#pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < n; ++i) {
    const long p = pair_p[i], f = pair_f[i];
    out[i] = (f < m.n) ? visible(m, f, mk(points[3 * p], points[3 * p + 1], points[3 * p + 2]))
                       : 0;
  }
  return 0;
}

// transient[t * S + s]; vis[s * F + f].
int oracle_mesh_confocal_forward(const float* verts, long V, const int64_t* faces, long F,
                                 const float* material, long M, const float* scan_points,
                                 long S, const float* scan_origin, const uint8_t* vis,
                                 long nbins, float bw, float bo, int fp64, double* transient) {
  const Mesh m = prepare(verts, V, faces, F);
  if (fp64)
    confocal_forward<double>(m, material, M, scan_points, S, scan_origin, vis, F, nbins, bw,
                             bo, transient);
  else
    confocal_forward<float>(m, material, M, scan_points, S, scan_origin, vis, F, nbins, bw,
                            bo, transient);
  return 0;
}

int oracle_mesh_confocal_grad(const float* verts, long V, const int64_t* faces, long F,
                              const float* material, long M, const float* scan_points, long S,
                              const float* scan_origin, const uint8_t* vis, long nbins,
                              float bw, float bo, const double* transient_grad, int want_verts,
                              int fp64, double* verts_grad, double* material_grad) {
  const Mesh m = prepare(verts, V, faces, F);
  if (fp64)
    confocal_grad<double>(m, material, M, scan_points, S, scan_origin, vis, F, nbins, bw, bo,
                          transient_grad, V, want_verts, verts_grad, material_grad);
  else
    confocal_grad<float>(m, material, M, scan_points, S, scan_origin, vis, F, nbins, bw, bo,
                         transient_grad, V, want_verts, verts_grad, material_grad);
  return 0;
}

// transient[(t * S + s) * L + l]; vis_s[s * F + f]; vis_l[l * F + f].
int oracle_mesh_exhaustive_forward(const float* verts, long V, const int64_t* faces, long F,
                                   const float* material, long M, const float* scan_points,
                                   long S, const float* laser_points, long L,
                                   const float* scan_origin, const float* laser_origin,
                                   const uint8_t* vis_s, const uint8_t* vis_l, long nbins,
                                   float bw, float bo, int fp64, double* transient) {
  const Mesh m = prepare(verts, V, faces, F);
  if (fp64)
    exhaustive_forward<double>(m, material, M, scan_points, S, laser_points, L, scan_origin,
                               laser_origin, vis_s, vis_l, F, nbins, bw, bo, transient);
  else
    exhaustive_forward<float>(m, material, M, scan_points, S, laser_points, L, scan_origin,
                              laser_origin, vis_s, vis_l, F, nbins, bw, bo, transient);
  return 0;
}

int oracle_mesh_exhaustive_grad(const float* verts, long V, const int64_t* faces, long F,
                                const float* material, long M, const float* scan_points,
                                long S, const float* laser_points, long L,
                                const float* scan_origin, const float* laser_origin,
                                const uint8_t* vis_s, const uint8_t* vis_l, long nbins,
                                float bw, float bo, const double* transient_grad,
                                int want_verts, int fp64, double* verts_grad,
                                double* material_grad) {
  const Mesh m = prepare(verts, V, faces, F);
  if (fp64)
    exhaustive_grad<double>(m, material, M, scan_points, S, laser_points, L, scan_origin,
                            laser_origin, vis_s, vis_l, F, nbins, bw, bo, transient_grad, V,
                            want_verts, verts_grad, material_grad);
  else
    exhaustive_grad<float>(m, material, M, scan_points, S, laser_points, L, scan_origin,
                           laser_origin, vis_s, vis_l, F, nbins, bw, bo, transient_grad, V,
                           want_verts, verts_grad, material_grad);
  return 0;
}

}  // extern "C"
