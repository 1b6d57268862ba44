// Orthographic depth rasteriser: the drop-in for the reference's
// UnitDepthMapRender (totri/util/depthmap.py:6-36), which rasterises a mesh
// with pytorch3d (FoVOrthographicCameras over [-xysize/2, xysize/2]^2 looking
// along +z from the origin, one face per pixel, no back-face culling) and
// returns the nearest face's depth per pixel and a coverage mask.
//
// Conventions (pytorch3d's screen space): image column j looks along the ray
// x = max_x - (j + 1/2) (max_x - min_x) / W (+x is to the left), row i along
// y = max_y - (i + 1/2) (max_y - min_y) / H (+y is up). A pixel is covered by
// a face when its centre lies inside the face's projection (edge functions
// all >= 0 or all <= 0, non-degenerate faces only); its depth is the face's z
// interpolated at the centre, kept when znear <= z <= zfar. The nearest depth
// wins, the lower face index on ties. Empty pixels hold depth -1.
//
// One thread per face walks the pixels of the face's bounding box and keeps
// (depth bits << 32 | face) with a 64-bit atomicMin per pixel (depths are
// non-negative, so their bit patterns order as the values); a second pass
// splits the words into depth and mask. FP32 with one rounding per operation
// (the CPU oracle evaluates the same expressions).
#include <cfloat>

#include "capi_common.cuh"
#include "common.cuh"

namespace totri {
namespace raster {

struct View {
  float min_x, max_x, min_y, max_y, znear, zfar;
  int H, W;
};

__device__ __forceinline__ float edge(float ax, float ay, float bx, float by, float px,
                                      float py) {
  return xsub(xmul(xsub(bx, ax), xsub(py, ay)), xmul(xsub(by, ay), xsub(px, ax)));
}

__global__ void faces_kernel(View v, const float* __restrict__ verts, int V,
                             const int64_t* __restrict__ faces, int F,
                             unsigned long long* __restrict__ zbuf) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F) return;
  int64_t idx[3];
  for (int k = 0; k < 3; ++k) {
    idx[k] = faces[3 * (int64_t)f + k];
    if (idx[k] < 0 || idx[k] >= V) return;  // not a face of this mesh
  }
  float x[3], y[3], z[3];
  for (int k = 0; k < 3; ++k) {
    x[k] = verts[3 * idx[k]];
    y[k] = verts[3 * idx[k] + 1];
    z[k] = verts[3 * idx[k] + 2];
  }
  const float area = edge(x[0], y[0], x[1], y[1], x[2], y[2]);
  if (area == 0.f || !isfinite(area)) return;  // degenerate, infinite or NaN in projection
  const float sx = xdiv(xsub(v.max_x, v.min_x), (float)v.W);
  const float sy = xdiv(xsub(v.max_y, v.min_y), (float)v.H);
  const float bx0 = fminf(fminf(x[0], x[1]), x[2]), bx1 = fmaxf(fmaxf(x[0], x[1]), x[2]);
  const float by0 = fminf(fminf(y[0], y[1]), y[2]), by1 = fmaxf(fmaxf(y[0], y[1]), y[2]);
  // columns whose centre x lies in [bx0, bx1]: j = (max_x - x) / sx - 1/2,
  // one column of slack each side (the exact test decides)
  const int j0 = max((int)floorf((v.max_x - bx1) / sx - 0.5f) - 1, 0);
  const int j1 = min((int)ceilf((v.max_x - bx0) / sx - 0.5f) + 1, v.W - 1);
  const int i0 = max((int)floorf((v.max_y - by1) / sy - 0.5f) - 1, 0);
  const int i1 = min((int)ceilf((v.max_y - by0) / sy - 0.5f) + 1, v.H - 1);
  if (!(j0 <= j1 && i0 <= i1)) return;
  for (int i = i0; i <= i1; ++i) {
    const float py = xsub(v.max_y, xmul(xadd((float)i, 0.5f), sy));
    for (int j = j0; j <= j1; ++j) {
      const float px = xsub(v.max_x, xmul(xadd((float)j, 0.5f), sx));
      const float w0 = edge(x[1], y[1], x[2], y[2], px, py);
      const float w1 = edge(x[2], y[2], x[0], y[0], px, py);
      const float w2 = edge(x[0], y[0], x[1], y[1], px, py);
      const bool in = (w0 >= 0.f && w1 >= 0.f && w2 >= 0.f) ||
                      (w0 <= 0.f && w1 <= 0.f && w2 <= 0.f);
      if (!in) continue;
      const float zz = xdiv(xadd(xadd(xmul(w0, z[0]), xmul(w1, z[1])), xmul(w2, z[2])), area);
      if (!(zz >= v.znear && zz <= v.zfar && zz >= 0.f)) continue;
      const unsigned long long key =
          ((unsigned long long)__float_as_uint(zz) << 32) | (unsigned)f;
      atomicMin(zbuf + (int64_t)i * v.W + j, key);
    }
  }
}

__global__ void finish_kernel(const unsigned long long* __restrict__ zbuf, int n,
                              float* __restrict__ depth, int* __restrict__ mask) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const unsigned long long k = zbuf[p];
  const bool hit = k != ~0ull;
  depth[p] = hit ? __uint_as_float((unsigned)(k >> 32)) : -1.f;
  mask[p] = hit ? 1 : 0;
}

}  // namespace raster
}  // namespace totri

using namespace totri;

extern "C" {

size_t totri_depth_raster_workspace(int64_t height, int64_t width) {
  return align_up(sizeof(unsigned long long) * (size_t)(height * width), 256);
}

int totri_depth_raster(const totri_array_t* verts, const totri_array_t* faces,
                       const totri_array_t* depth, const totri_array_t* mask, float min_x,
                       float max_x, float min_y, float max_y, float znear, float zfar, void* ws,
                       size_t ws_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  TOTRI_TRY(check_array(verts, "verts", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(verts, "verts", 1, 3));
  TOTRI_TRY(check_contiguous(verts, "verts"));
  TOTRI_TRY(check_array(faces, "faces", 2, TOTRI_INT64));
  TOTRI_TRY(check_dim(faces, "faces", 1, 3));
  TOTRI_TRY(check_contiguous(faces, "faces"));
  TOTRI_TRY(check_array(depth, "depth", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_contiguous(depth, "depth"));
  TOTRI_TRY(check_array(mask, "mask", 2, TOTRI_INT32));
  for (int d = 0; d < 2; ++d) TOTRI_TRY(check_dim(mask, "mask", d, depth->shape[d]));
  TOTRI_TRY(check_contiguous(mask, "mask"));
  const int64_t H = depth->shape[0], W = depth->shape[1];
  if (H > INT32_MAX / 2 || W > INT32_MAX / 2 || H * W > INT32_MAX)
    return fail(TOTRI_ERR_UNSUPPORTED, "image too large");
  if (verts->shape[0] > INT32_MAX || faces->shape[0] > INT32_MAX)
    return fail(TOTRI_ERR_UNSUPPORTED, "mesh too large");
  if (!(max_x > min_x) || !(max_y > min_y))
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "empty view window");
  if (H * W == 0) return TOTRI_OK;
  const size_t need = totri_depth_raster_workspace(H, W);
  if (!ws || ws_bytes < need)
    return fail(TOTRI_ERR_WORKSPACE, "workspace of " + std::to_string(need) + " bytes required");
  unsigned long long* zbuf = static_cast<unsigned long long*>(ws);
  TOTRI_CUDA(cudaMemsetAsync(zbuf, 0xff, sizeof(unsigned long long) * H * W, stream));
  const raster::View v{min_x, max_x, min_y, max_y, znear, zfar, (int)H, (int)W};
  const int F = (int)faces->shape[0];
  if (F > 0)
    TOTRI_KERNEL("depth raster faces", stream,
                 raster::faces_kernel<<<(unsigned)ceil_div(F, 128), 128, 0, stream>>>(
                     v, static_cast<const float*>(verts->data), (int)verts->shape[0],
                     static_cast<const int64_t*>(faces->data), F, zbuf));
  TOTRI_KERNEL("depth raster finish", stream,
               raster::finish_kernel<<<(unsigned)ceil_div(H * W, 256), 256, 0, stream>>>(
                   zbuf, (int)(H * W), static_cast<float*>(depth->data),
                   static_cast<int*>(mask->data)));
  return TOTRI_OK;
}

}  // extern "C"
