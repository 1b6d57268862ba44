// Oracle: CPU restatement of RBF-to-volume splatting and its gradient.
//
// TEST INFRASTRUCTURE ONLY (see oracle_common.h). Follows
//   forward  src/util/rbf2volume_cuda.cu:50-93 (Gaussian :16-30)
//   gradient src/util/rbf2volume_cuda.cu:124-201 (GaussianGradParams :32-47)
// in FP64 (no discrete decisions except the 1e-8 normalisation guard).
#include <algorithm>
#include <cmath>
#include <vector>

namespace {

inline double coord(float start, float end, int n, int i) {
  if (n == 1) return 0.5 * ((double)start + (double)end);
  return (double)start + ((double)end - (double)start) * (double)i / (double)(n - 1);
}

}  // namespace

extern "C" {

// One batch item: rbf [N, 4+A] (x, y, z, sigma, attributes);
// volume [1+A, D, H, W] (overwritten).
int oracle_rbf2volume_forward(const float* rbf, int N, int C, int D, int H, int W,
                              const float* start, const float* end, double* vol) {
  const int A = C - 4;
  const size_t V = (size_t)D * H * W;
#pragma omp parallel for collapse(2)
  for (int zi = 0; zi < D; ++zi)
    for (int yi = 0; yi < H; ++yi)
      for (int xi = 0; xi < W; ++xi) {
        const double x = coord(start[0], end[0], W, xi), y = coord(start[1], end[1], H, yi),
                     z = coord(start[2], end[2], D, zi);
        double sum = 0.0;
        std::vector<double> attr(A, 0.0);
        for (int i = 0; i < N; ++i) {
          const float* r = rbf + (size_t)i * C;
          const double dx = r[0] - x, dy = r[1] - y, dz = r[2] - z, s = r[3];
          const double w = std::exp(-0.5 * (dx * dx + dy * dy + dz * dz) / (s * s));
          sum += w;
          for (int a = 0; a < A; ++a) attr[a] += w * r[4 + a];
        }
        const size_t idx = ((size_t)zi * H + yi) * W + xi;
        vol[idx] = sum;
        const double norm = sum < 1e-8 ? 1.0 : sum;
        for (int a = 0; a < A; ++a) vol[(1 + a) * V + idx] = attr[a] / norm;
      }
  return 0;
}

// rbf_grad [N, 4+A] (overwritten) from volume and volume_grad [1+A, D, H, W].
int oracle_rbf2volume_grad(const float* rbf, int N, int C, int D, int H, int W,
                           const double* vol, const double* vgrad, const float* start,
                           const float* end, double* grad) {
  const int A = C - 4;
  const size_t V = (size_t)D * H * W;
  std::fill(grad, grad + (size_t)N * C, 0.0);
#pragma omp parallel for
  for (int i = 0; i < N; ++i) {
    const float* r = rbf + (size_t)i * C;
    double* g = grad + (size_t)i * C;
    for (int zi = 0; zi < D; ++zi)
      for (int yi = 0; yi < H; ++yi)
        for (int xi = 0; xi < W; ++xi) {
          const size_t idx = ((size_t)zi * H + yi) * W + xi;
          const double x = coord(start[0], end[0], W, xi), y = coord(start[1], end[1], H, yi),
                       z = coord(start[2], end[2], D, zi);
          const double dx = r[0] - x, dy = r[1] - y, dz = r[2] - z, s = r[3];
          const double d2 = dx * dx + dy * dy + dz * dz;
          const double w = std::exp(-0.5 * d2 / (s * s));
          const double is2 = 1.0 / (s * s);
          const double dwx = (x - r[0]) * is2 * w, dwy = (y - r[1]) * is2 * w,
                       dwz = (z - r[2]) * is2 * w, dws = d2 * is2 / s * w;
          const double dl0 = vgrad[idx];
          if (A == 0) {
            g[0] += dl0 * dwx;
            g[1] += dl0 * dwy;
            g[2] += dl0 * dwz;
            g[3] += dl0 * dws;
            continue;
          }
          double v0 = vol[idx];
          if (v0 < 1e-8) v0 = 1.0;
          const double inv = 1.0 / v0;
          double sum = 0.0;
          for (int a = 0; a < A; ++a) {
            const double dla = vgrad[(1 + a) * V + idx];
            sum += dla * (r[4 + a] - vol[(1 + a) * V + idx]);
            g[4 + a] += dla * w * inv;
          }
          sum *= inv;
          g[0] += dwx * (dl0 + sum);
          g[1] += dwy * (dl0 + sum);
          g[2] += dwz * (dl0 + sum);
          g[3] += dws * (dl0 + sum);
        }
  }
  return 0;
}

}  // extern "C"
