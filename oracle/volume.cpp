// Oracle: CPU restatement of the voxel-volume transient renderer.
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h). Follows
//   confocal forward           src/render/volume_cuda.cu:12-66
//   transposed ("grad_volume") src/render/volume_cuda.cu:96-160
//   d/d measurement points     src/render/volume_cuda.cu:189-265
//   exhaustive forward         src/render/volume_cuda.cu:298-377
// plus the exact adjoints of both forwards (the reference's transposed
// operator differs from the adjoint at the top z slice, and its exhaustive
// gradient kernel is empty, volume_cuda.cu:428-430).
// FP32 decisions: the sphere/column test (depth^2 > 0), floor(z_hat) and its
// range test, the bin ranges; values in precision T.
#include <algorithm>
#include <cstring>
#include <vector>

#include "oracle_common.h"

using namespace oracle;

namespace {

// Column centre ((i + 0.5) * size / n + origin), FP32 as in the reference.
inline float cell_centre(float origin, float size, int n, int i) {
  return origin + ((float)i + 0.5f) * size / (float)n;
}

struct Sample {
  bool ok;
  int zi;
  float z_hat;  // FP32
  float depth;  // FP32
};

// One (point, bin, column) sample of the confocal volume renderer.
inline Sample confocal_sample(float wx, float wy, float wz, float tc, float x, float y, float oz,
                              float s, int Z) {
  Sample r{false, 0, 0.f, 0.f};
  const float dx = wx - x, dy = wy - y;
  const float d2 = (tc * tc - dx * dx) - dy * dy;
  if (!(d2 > 0.f)) return r;
  r.depth = std::sqrt(d2);
  const float z = wz + r.depth;
  r.z_hat = (z - oz) * s - 0.5f;
  const float fl = std::floor(r.z_hat);
  if (!(fl >= 0.f && fl + 1.f < (float)Z)) return r;
  r.zi = (int)fl;
  r.ok = true;
  return r;
}

template <typename T>
inline T f2_of(T depth, T tc) {
  const T q = depth / (tc * tc);
  return (q * q) * (q * q);
}

// Walks every valid sample; fn(i, t, xi, yi, zi, alpha, f2) with alpha, f2 in T.
template <typename T, typename Fn>
void for_each_sample(int X, int Y, int Z, const float* mp, int N, int Tn, const float* org,
                     const float* size, float bw, float bo, Fn&& fn) {
  const float s = (float)Z / size[2];
  for (int i = 0; i < N; ++i) {
    const float wx = mp[i], wy = mp[N + i], wz = mp[2 * N + i];
    for (int t = 0; t < Tn; ++t) {
      const float tc = (float)t * bw + bo;
      for (int xi = 0; xi < X; ++xi) {
        const float x = cell_centre(org[0], size[0], X, xi);
        for (int yi = 0; yi < Y; ++yi) {
          const float y = cell_centre(org[1], size[1], Y, yi);
          const Sample sm = confocal_sample(wx, wy, wz, tc, x, y, org[2], s, Z);
          if (!sm.ok) continue;
          T alpha, f2;
          if (sizeof(T) == sizeof(float)) {
            alpha = (T)(sm.z_hat - (float)sm.zi);
            f2 = f2_of<T>((T)sm.depth, (T)tc);
          } else {
            // values in double from the same inputs
            const T dx = (T)wx - (T)x, dy = (T)wy - (T)y, tcd = (T)t * (T)bw + (T)bo;
            const T depth = std::sqrt(std::max(T(0), tcd * tcd - dx * dx - dy * dy));
            const T zh = ((T)wz + depth - (T)org[2]) * ((T)Z / (T)size[2]) - T(0.5);
            alpha = zh - (T)sm.zi;
            f2 = f2_of<T>(depth, tcd);
          }
          fn(i, t, xi, yi, sm.zi, alpha, f2);
        }
      }
    }
  }
}

template <typename T>
void confocal_forward(const float* vol, int X, int Y, int Z, const float* mp, int N, int Tn,
                      const float* org, const float* size, float bw, float bo, double* out) {
  std::vector<T> acc((size_t)N * Tn, T(0));
  for_each_sample<T>(X, Y, Z, mp, N, Tn, org, size, bw, bo,
                     [&](int i, int t, int xi, int yi, int zi, T a, T f2) {
                       const float* col = vol + ((size_t)xi * Y + yi) * Z;
                       acc[(size_t)i * Tn + t] += ((T(1) - a) * (T)col[zi] + a * (T)col[zi + 1]) * f2;
                     });
  for (size_t k = 0; k < acc.size(); ++k) out[k] = (double)acc[k];
}

template <typename T>
void confocal_adjoint(const double* tr, int X, int Y, int Z, const float* mp, int N, int Tn,
                      const float* org, const float* size, float bw, float bo, double* vol) {
  std::vector<T> acc((size_t)X * Y * Z, T(0));
  for_each_sample<T>(X, Y, Z, mp, N, Tn, org, size, bw, bo,
                     [&](int i, int t, int xi, int yi, int zi, T a, T f2) {
                       T* col = acc.data() + ((size_t)xi * Y + yi) * Z;
                       const T g = (T)tr[(size_t)i * Tn + t] * f2;
                       col[zi] += (T(1) - a) * g;
                       col[zi + 1] += a * g;
                     });
  for (size_t k = 0; k < acc.size(); ++k) vol[k] = (double)acc[k];
}

template <typename T>
void confocal_grad_mp(const float* vol, int X, int Y, int Z, const float* mp, int N, int Tn,
                      const double* tg, const float* org, const float* size, float bw, float bo,
                      double* out) {
  std::vector<T> acc((size_t)3 * N, T(0));
  const T s = (T)Z / (T)size[2];
  for_each_sample<T>(X, Y, Z, mp, N, Tn, org, size, bw, bo,
                     [&](int i, int t, int xi, int yi, int zi, T a, T f2) {
                       const float* col = vol + ((size_t)xi * Y + yi) * Z;
                       const T v0 = col[zi], v1 = col[zi + 1];
                       const T f1 = (T(1) - a) * v0 + a * v1;
                       const T x = (T)cell_centre(org[0], size[0], X, xi);
                       const T y = (T)cell_centre(org[1], size[1], Y, yi);
                       const T wx = mp[i], wy = mp[N + i];
                       const T tc = (T)t * (T)bw + (T)bo;
                       const T depth = std::sqrt(tc * tc - (wx - x) * (wx - x) - (wy - y) * (wy - y));
                       const T dzx = -(wx - x) / depth, dzy = -(wy - y) / depth;
                       // d f2 / d depth = 4 depth^3 / tc^8
                       const T tc2 = tc * tc, tc4 = tc2 * tc2;
                       const T df2 = T(4) * depth * depth * depth / (tc4 * tc4);
                       const T g = (T)tg[(size_t)i * Tn + t];
                       acc[i] += g * (f1 * df2 * dzx + s * dzx * (v1 - v0) * f2);
                       acc[N + i] += g * (f1 * df2 * dzy + s * dzy * (v1 - v0) * f2);
                       acc[2 * N + i] += g * (s * (v1 - v0) * f2);
                     });
  for (size_t k = 0; k < acc.size(); ++k) out[k] = (double)acc[k];
}

// The reference's transposed operator, restated (volume_cuda.cu:96-160): per
// voxel, bins from ceil(tf(z - dz)) (z at slice 0) to ceil(tf(z + dz)), the
// lower/upper interpolation weight chosen by comparing with ceil(tf(z)).
template <typename T>
void confocal_transposed(const double* tr, int X, int Y, int Z, const float* mp, int N, int Tn,
                         const float* org, const float* size, float bw, float bo, double* vol) {
  const float dz = size[2] / (float)Z;
  const float s = (float)Z / size[2];
  for (int xi = 0; xi < X; ++xi)
    for (int yi = 0; yi < Y; ++yi)
      for (int zi = 0; zi < Z; ++zi) {
        const float x = cell_centre(org[0], size[0], X, xi);
        const float y = cell_centre(org[1], size[1], Y, yi);
        const float z = cell_centre(org[2], size[2], Z, zi);
        T value = 0;
        for (int i = 0; i < N; ++i) {
          const float wx = mp[i], wy = mp[N + i], wz = mp[2 * N + i];
          const float zz = zi > 0 ? dz : 0.f;
          const float dp2 = (x - wx) * (x - wx) + (y - wy) * (y - wy);
          const float ds = std::sqrt(dp2 + ((z - zz) - wz) * ((z - zz) - wz));
          const float dm = std::sqrt(dp2 + (z - wz) * (z - wz));
          const float de = std::sqrt(dp2 + ((z + dz) - wz) * ((z + dz) - wz));
          auto tbin = [&](float d) {
            const float c = std::ceil((d - bo) / bw);
            return (int)std::min(std::max(c, 0.f), (float)Tn);
          };
          const int t_start = tbin(ds), t_mid = tbin(dm), t_end = tbin(de);
          for (int t = t_start; t < t_end; ++t) {
            const float tc = (float)t * bw + bo;
            const float d2 = tc * tc - dp2;
            if (!(d2 > 0.f)) continue;
            const float depth = std::sqrt(d2);
            const float z_hat = ((wz + depth) - org[2]) * s - 0.5f;
            const float a = z_hat - std::floor(z_hat);
            const T w = (t >= t_mid) ? T(1) - (T)a : (T)a;
            value += w * f2_of<T>((T)depth, (T)tc) * (T)tr[(size_t)i * Tn + t];
          }
        }
        vol[((size_t)xi * Y + yi) * Z + zi] = (double)value;
      }
}

// Exhaustive volume renderer (volume_cuda.cu:298-377): per occupied voxel and
// (scan, laser) pair, the path-length interval of the voxel's z extent,
// box-filtered into bins. The wall-origin terms are unused by the reference
// kernel and therefore here too.
template <typename T, typename Fn>
void for_each_exhaustive(int D, int H, int W, const float* sp, int S, const float* lp, int L,
                         int Tn, const float* start, const float* end, float bw, float bo,
                         Fn&& fn) {
  for (int yi = 0; yi < H; ++yi)
    for (int xi = 0; xi < W; ++xi) {
      const float xf = start[0] + ((float)xi + 0.5f) / (float)W * (end[0] - start[0]);
      const float yf = start[1] + ((float)yi + 0.5f) / (float)H * (end[1] - start[1]);
      for (int s = 0; s < S; ++s) {
        const f3 sc = mk(sp[s], sp[S + s], sp[2 * S + s]);
        for (int l = 0; l < L; ++l) {
          const f3 lc = mk(lp[l], lp[L + l], lp[2 * L + l]);
          for (int zi = 0; zi < D; ++zi) {
            const float zf = start[2] + ((float)zi + 0.5f) / (float)D * (end[2] - start[2]);
            const float half = 0.5f / (float)D * (end[2] - start[2]);
            const float zf0 = zf - half, zf1 = zf + half;
            float d0 = len_e(sub(sc, mk(xf, yf, zf0))) + len_e(sub(lc, mk(xf, yf, zf0)));
            float d1 = len_e(sub(sc, mk(xf, yf, zf1))) + len_e(sub(lc, mk(xf, yf, zf1)));
            if (d1 < d0) std::swap(d0, d1);
            float bf0 = (d0 - bo) / bw, bf1 = (d1 - bo) / bw;
            const float range = bf1 - bf0;
            int first = (int)std::floor(bf0), last = (int)std::floor(bf1);
            if (first < 0) {
              if (last < 0) continue;
              bf0 = 0.f;
              first = 0;
            }
            if (last >= Tn) {
              if (first >= Tn) continue;
              bf1 = (float)(Tn - 1);
              last = Tn - 1;
            }
            fn(s, l, zi, yi, xi, first, last, (T)bf0, (T)bf1, (T)range);
          }
        }
      }
    }
}

}  // namespace

extern "C" {

// volume [X,Y,Z] (x-major), mp [3,N], transient [N,T].
int oracle_volume_confocal_forward(const float* vol, int X, int Y, int Z, const float* mp, int N,
                                   int Tn, const float* org, const float* size, float bw,
                                   float bo, int fp64, double* out) {
  if (fp64) confocal_forward<double>(vol, X, Y, Z, mp, N, Tn, org, size, bw, bo, out);
  else confocal_forward<float>(vol, X, Y, Z, mp, N, Tn, org, size, bw, bo, out);
  return 0;
}

int oracle_volume_confocal_adjoint(const double* tr, int X, int Y, int Z, const float* mp, int N,
                                   int Tn, const float* org, const float* size, float bw,
                                   float bo, int fp64, double* vol) {
  if (fp64) confocal_adjoint<double>(tr, X, Y, Z, mp, N, Tn, org, size, bw, bo, vol);
  else confocal_adjoint<float>(tr, X, Y, Z, mp, N, Tn, org, size, bw, bo, vol);
  return 0;
}

int oracle_volume_confocal_transposed(const double* tr, int X, int Y, int Z, const float* mp,
                                      int N, int Tn, const float* org, const float* size,
                                      float bw, float bo, int fp64, double* vol) {
  if (fp64) confocal_transposed<double>(tr, X, Y, Z, mp, N, Tn, org, size, bw, bo, vol);
  else confocal_transposed<float>(tr, X, Y, Z, mp, N, Tn, org, size, bw, bo, vol);
  return 0;
}

int oracle_volume_confocal_grad_mp(const float* vol, int X, int Y, int Z, const float* mp, int N,
                                   int Tn, const double* tg, const float* org, const float* size,
                                   float bw, float bo, int fp64, double* out) {
  if (fp64) confocal_grad_mp<double>(vol, X, Y, Z, mp, N, Tn, tg, org, size, bw, bo, out);
  else confocal_grad_mp<float>(vol, X, Y, Z, mp, N, Tn, tg, org, size, bw, bo, out);
  return 0;
}

// One batch item: volume [D,H,W], sp [3,S], lp [3,L], transient [T,S,L].
int oracle_volume_exhaustive_forward(const float* vol, int D, int H, int W, const float* sp, int S,
                                     const float* lp, int L, int Tn, const float* start,
                                     const float* end, float bw, float bo, int fp64,
                                     double* out) {
  std::vector<double> acc((size_t)Tn * S * L, 0.0);
  for_each_exhaustive<double>(D, H, W, sp, S, lp, L, Tn, start, end, bw, bo,
      [&](int s, int l, int zi, int yi, int xi, int first, int last, double bf0, double bf1,
          double range) {
        const double occ = vol[((size_t)zi * H + yi) * W + xi];
        if (occ == 0.0) return;
        double* col = acc.data() + (size_t)s * L + l;
        const size_t st = (size_t)S * L;
        if (first == last) {
          col[first * st] += occ;
          return;
        }
        const double fo = occ / range;
        col[first * st] += (1.0 - (bf0 - first)) * fo;
        for (int b = first + 1; b < last; ++b) col[b * st] += fo;
        col[last * st] += (bf1 - last) * fo;
      });
  (void)fp64;
  std::memcpy(out, acc.data(), sizeof(double) * acc.size());
  return 0;
}

// Adjoint of the exhaustive forward w.r.t. the volume (the forward is linear
// in the volume): volume_grad [D,H,W] from transient_grad [T,S,L].
int oracle_volume_exhaustive_adjoint(const double* tg, int D, int H, int W, const float* sp,
                                     int S, const float* lp, int L, int Tn, const float* start,
                                     const float* end, float bw, float bo, double* vol) {
  std::fill(vol, vol + (size_t)D * H * W, 0.0);
  for_each_exhaustive<double>(D, H, W, sp, S, lp, L, Tn, start, end, bw, bo,
      [&](int s, int l, int zi, int yi, int xi, int first, int last, double bf0, double bf1,
          double range) {
        const double* col = tg + (size_t)s * L + l;
        const size_t st = (size_t)S * L;
        double g;
        if (first == last) {
          g = col[first * st];
        } else {
          g = (1.0 - (bf0 - first)) / range * col[first * st];
          for (int b = first + 1; b < last; ++b) g += col[b * st] / range;
          g += (bf1 - last) / range * col[last * st];
        }
        vol[((size_t)zi * H + yi) * W + xi] += g;
      });
  return 0;
}

}  // extern "C"
