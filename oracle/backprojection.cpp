// Oracle: CPU restatement of the backprojection reconstructions.
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h). Follows
//   Velten confocal     src/reconstruct/backprojection_cuda.cu:153-194
//   Velten exhaustive   src/reconstruct/backprojection_cuda.cu:229-287
//   Arellano exhaustive src/reconstruct/backprojection_cuda.cu:11-115
// plus the adjoint of the Velten confocal backprojection.
// FP32 decisions: the nearest bin index, the Arellano sphere test and depth
// bin; values in FP64.
#include <algorithm>
#include <cstring>
#include <vector>

#include "oracle_common.h"

using namespace oracle;

namespace {

// Inclusive grid coordinate start + (i / (n - 1)) * (end - start).
inline float grid_coord(float start, float end, int n, int i) {
  return start + ((float)i / (float)(n - 1)) * (end - start);
}

inline int nearest_bin(float dist, float bw, float bo) {
  const float b = std::floor((dist - bo) / bw + 0.5f);
  if (!(b == b)) return -1;
  if (b > 2.0e9f) return 2000000000;
  if (b < -2.0e9f) return -2000000000;
  return (int)b;
}

}  // namespace

extern "C" {

// One batch item. transient [T,S], sp [S,3], so [So,3] (So = 0 or S),
// volume [D,H,W] (overwritten).
int oracle_bp_confocal_velten(const float* tr, int Tn, const float* sp, int S, const float* so,
                              int So, int D, int H, int W, const float* start, const float* end,
                              float bw, float bo, double* vol) {
#pragma omp parallel for collapse(2)
  for (int z = 0; z < D; ++z)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const f3 p = mk(grid_coord(start[0], end[0], W, x), grid_coord(start[1], end[1], H, y),
                        grid_coord(start[2], end[2], D, z));
        double value = 0.0;
        for (int s = 0; s < S; ++s) {
          const f3 q = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
          const float sv = len_e(sub(q, p));
          const float od = So > 0 ? len_e(sub(q, mk(so[3 * s], so[3 * s + 1], so[3 * s + 2]))) : 0.f;
          const int t = nearest_bin(2.f * od + 2.f * sv, bw, bo);
          if (t >= 0 && t < Tn) value += tr[(size_t)t * S + s];
        }
        vol[((size_t)z * H + y) * W + x] = value;
      }
  return 0;
}

// Adjoint of oracle_bp_confocal_velten: transient [T,S] from volume [D,H,W].
int oracle_bp_confocal_velten_adjoint(const double* vol, int D, int H, int W, const float* sp,
                                      int S, const float* so, int So, int Tn, const float* start,
                                      const float* end, float bw, float bo, double* tr) {
  std::fill(tr, tr + (size_t)Tn * S, 0.0);
#pragma omp parallel for
  for (int s = 0; s < S; ++s) {
    const f3 q = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
    const float od = So > 0 ? len_e(sub(q, mk(so[3 * s], so[3 * s + 1], so[3 * s + 2]))) : 0.f;
    for (int z = 0; z < D; ++z)
      for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
          const f3 p = mk(grid_coord(start[0], end[0], W, x), grid_coord(start[1], end[1], H, y),
                          grid_coord(start[2], end[2], D, z));
          const int t = nearest_bin(2.f * od + 2.f * len_e(sub(q, p)), bw, bo);
          if (t >= 0 && t < Tn) tr[(size_t)t * S + s] += vol[((size_t)z * H + y) * W + x];
        }
  }
  return 0;
}

// transient [T,S,L], sp [S,3], lp [L,3], so [So,3], lo [Lo,3]; volume [D,H,W].
int oracle_bp_exhaustive_velten(const float* tr, int Tn, const float* sp, int S, const float* lp,
                                int L, const float* so, int So, const float* lo, int Lo, int D,
                                int H, int W, const float* start, const float* end, float bw,
                                float bo, double* vol) {
#pragma omp parallel for collapse(2)
  for (int z = 0; z < D; ++z)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const f3 p = mk(grid_coord(start[0], end[0], W, x), grid_coord(start[1], end[1], H, y),
                        grid_coord(start[2], end[2], D, z));
        double value = 0.0;
        for (int s = 0; s < S; ++s) {
          const f3 q = mk(sp[3 * s], sp[3 * s + 1], sp[3 * s + 2]);
          const float sv = len_e(sub(q, p));
          const float sod = So > 0 ? len_e(sub(q, mk(so[3 * s], so[3 * s + 1], so[3 * s + 2]))) : 0.f;
          for (int l = 0; l < L; ++l) {
            const f3 r = mk(lp[3 * l], lp[3 * l + 1], lp[3 * l + 2]);
            const float lv = len_e(sub(r, p));
            const float lod =
                Lo > 0 ? len_e(sub(r, mk(lo[3 * l], lo[3 * l + 1], lo[3 * l + 2]))) : 0.f;
            const int t = nearest_bin(((sod + sv) + lv) + lod, bw, bo);
            if (t >= 0 && t < Tn) value += tr[((size_t)t * S + s) * L + l];
          }
        }
        vol[((size_t)z * H + y) * W + x] = value;
      }
  return 0;
}

// Arellano: transient [T,S,L]; sp [3,S]; lp [3,L]; so [3,So]; lo [3,Lo];
// volume [D,H,W] (overwritten with the deposits).
int oracle_bp_exhaustive_arellano(const float* tr, int Tn, const float* sp, int S,
                                  const float* lp, int L, const float* so, int So,
                                  const float* lo, int Lo, int D, int H, int W,
                                  const float* start, const float* end, float bw, float bo,
                                  double* vol) {
  std::fill(vol, vol + (size_t)D * H * W, 0.0);
#pragma omp parallel for collapse(2)
  for (int yi = 0; yi < H; ++yi)
    for (int xi = 0; xi < W; ++xi) {
      const float xf = start[0] + ((float)xi / (float)(W - 1)) * (end[0] - start[0]);
      const float yf = start[1] + ((float)yi / (float)(H - 1)) * (end[1] - start[1]);
      for (int s = 0; s < S; ++s) {
        const f3 sc = mk(sp[s], sp[S + s], sp[2 * S + s]);
        const float sd = So > 0 ? len_e(sub(sc, mk(so[s], so[So + s], so[2 * So + s]))) : 0.f;
        for (int l = 0; l < L; ++l) {
          const f3 lc = mk(lp[l], lp[L + l], lp[2 * L + l]);
          const float ld = Lo > 0 ? len_e(sub(lc, mk(lo[l], lo[Lo + l], lo[2 * Lo + l]))) : 0.f;
          const f3 center = mk(0.5f * (sc.x + lc.x), 0.5f * (sc.y + lc.y), 0.5f * (sc.z + lc.z));
          f3 nrm = sub(sc, lc);
          const float length = len_e(nrm);
          if (length > 1e-6f) {
            const float inv = 1.f / length;
            nrm = mk(inv * nrm.x, inv * nrm.y, inv * nrm.z);
          }
          const f3 rs = sub(mk(xf, yf, start[2]), center);
          const f3 re = sub(mk(xf, yf, end[2]), center);
          for (int t = 0; t < Tn; ++t) {
            const float value = tr[((size_t)t * S + s) * L + l];
            if (!(value > 0.f)) continue;
            const float tc = (((float)t * bw + bo) - sd) - ld;
            if (!(tc > length)) continue;
            const float r0 = tc / 2.f;
            const float r1 = std::sqrt(r0 * r0 - length * length / 4.f);
            const float scale = r1 / r0;
            const float ks = (scale - 1.f) * dot_e(rs, nrm), ke = (scale - 1.f) * dot_e(re, nrm);
            const f3 st = mk(std::fma(ks, nrm.x, rs.x), std::fma(ks, nrm.y, rs.y),
                             std::fma(ks, nrm.z, rs.z));
            const f3 et = mk(std::fma(ke, nrm.x, re.x), std::fma(ke, nrm.y, re.y),
                             std::fma(ke, nrm.z, re.z));
            f3 dir = sub(et, st);
            const float rl = len_e(dir);
            const float ir = 1.f / rl;
            dir = mk(ir * dir.x, ir * dir.y, ir * dir.z);
            const float v0 = dot_e(dir, st);
            float v1 = v0 * v0 - (dot_e(st, st) - r1 * r1);
            if (!(v1 > 0.f)) continue;
            v1 = std::sqrt(v1);
            float d = -v0 - v1;
            if (d < 0.f) d = -v0 + v1;
            // int() truncation toward zero, then the range test: (-1, D) -> [0, D)
            const float bf = d / rl * (float)D + 0.5f;
            if (!(bf > -1.f && bf < (float)D)) continue;
            const int bin = (int)bf;
            vol[((size_t)bin * H + yi) * W + xi] += (double)value;
          }
        }
      }
    }
  return 0;
}

}  // extern "C"
