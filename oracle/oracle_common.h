// Oracle: CPU restatement of the totrilib transient-rendering path.
//
// TEST INFRASTRUCTURE ONLY. This library is the checker for the CUDA kernels
// in totri_gb300/csrc; nothing in the product imports, links or calls it.
// Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it.
//
// Numerics contract shared with the CUDA path (restated here, not shared code):
//  * Every quantity that drives a discrete decision (visibility, the vertex
//    sort order, integer bin indices, branch choices) is computed in FP32 with
//    one IEEE rounding per operation, in a fixed order, with fused
//    multiply-adds only where written as fmaf(). Build flags: -ffp-contract=off.
//  * Values (path-length integrals, falloff, gradients) are computed in the
//    selected precision T (float or double) following the reference formulas.
#ifndef TOTRI_ORACLE_COMMON_H
#define TOTRI_ORACLE_COMMON_H

#include <cmath>
#include <cstdint>

namespace oracle {

struct f3 {
  float x, y, z;
};

inline f3 mk(float x, float y, float z) { return f3{x, y, z}; }
inline f3 sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline f3 add(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
// |a|^2 as fma(x, x, fma(y, y, z*z)); |a| = IEEE sqrt of that.
inline float len2_e(f3 a) {
  return std::fma(a.x, a.x, std::fma(a.y, a.y, a.z * a.z));
}
inline float len_e(f3 a) { return std::sqrt(len2_e(a)); }
// a x b with one fused product per component.
inline f3 cross_e(f3 a, f3 b) {
  return f3{std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)),
            std::fma(a.x, b.y, -(a.y * b.x))};
}
inline float dot_e(f3 a, f3 b) {
  return std::fma(a.x, b.x, std::fma(a.y, b.y, a.z * b.z));
}

// Centroid as the reference forms it: (1/3) * ((v0 + v1) + v2)
// (mesh_confocal_forward_optix.cu:40).
inline f3 centroid_e(f3 v0, f3 v1, f3 v2) {
  const float third = 1.f / 3.f;
  f3 s = add(add(v0, v1), v2);
  return f3{third * s.x, third * s.y, third * s.z};
}

// C-style int() truncation of a bin coordinate with saturation, so that
// out-of-range and NaN coordinates have a defined result on every host.
inline int bin_of(float c) {
  if (!(c == c)) return -2147483647;  // NaN: never a valid bin
  if (c >= 1.0e9f) return 1000000000;
  if (c <= -1.0e9f) return -1000000000;
  return (int)c;
}

}  // namespace oracle

#endif  // TOTRI_ORACLE_COMMON_H
