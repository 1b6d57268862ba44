// Shaded perspective rasteriser: the drop-in for the reference's preview
// renderer UnitCubeMeshRender (totri/util/render.py:17-81), which draws a
// mesh for TensorBoard images with pytorch3d: FoVPerspectiveCameras, one face
// per pixel and no blur, SoftPhongShader with one point light and vertex
// colours. pytorch3d is a third-party dependency that the reference does not
// vendor or pin; this file restates its published rasterisation, Phong
// lighting and softmax blend.
//
// Rasterisation, in normalised device coordinates (ndc): a vertex's ndc is
// (focal.x * view.x / view.z, focal.y * view.y / view.z) with its view depth
// view.z kept as z. A face is skipped when its largest z is below 0 or its
// ndc edge function area lies within +-1e-8. At a pixel centre p (inside the
// face's ndc bounding box) the screen barycentrics are
// w_i = E(p, v_{i+1}, v_{i+2}) / (E(v2, v0, v1) + 1e-8) with
// E(p, a, b) = (p - a).x (b - a).y - (p - a).y (b - a).x, corrected for
// perspective as b_i = w_i z_{i+1} z_{i+2} / max(sum of those, 1e-8); the
// pixel is covered when every b_i > 0, at depth pz = sum b_i z_i, kept when
// pz >= 0. The nearest depth wins, the lower face index on ties. All of these
// decisions are FP32 with one rounding per operation (no contraction), so the
// CPU oracle reproduces them bit for bit.
//
// Shading of a covered pixel: the barycentric interpolation of the world
// position P, of the unit vertex normals (each the normalised sum of the
// cross products (v2 - v1) x (v0 - v1) of its faces) and of the vertex
// colours C; with N = normalise(normal), L = normalise(light - P),
// E = normalise(eye - P) (each x / max(|x|, 1e-6)), c = N.L and
// R = 2 c N - L, the colour is
//   (ka la + kd ld max(c, 0)) C + ks ls (max(E.R, 0) [c > 0])^shininess.
// The blend with the background (one face per pixel) weighs the colour by
// sigmoid(d / sigma), d the squared ndc distance from the pixel centre to the
// face's nearest edge, and the background by
// max(exp((1e-10 - z_inv) / gamma), 1e-10), z_inv = (zfar - pz) / (zfar -
// znear) clamped below at 1e-10. Empty pixels hold the background.
//
// Kernels: vertex normals (a thread per face, float atomics), vertex
// projection (a thread per vertex), rasterisation (a warp per face, lanes
// over the pixels of its bounding box, a 64-bit atomicMin of
// (depth bits << 32 | face) per covered pixel), shading (a thread per pixel,
// writing the [3, H, W] image).
#include <cfloat>

#include "capi_common.cuh"
#include "common.cuh"

namespace totri {
namespace shade {

constexpr float kEps = 1e-8f;

struct Colors {
  const float* data;
  int64_t sv, sc;  // element strides over vertices and channels
  __device__ __forceinline__ float3 at(int64_t v) const {
    const float* p = data + v * sv;
    return make_float3(p[0], p[sc], p[2 * sc]);
  }
};

// pytorch3d's EdgeFunctionForward(p, a, b)
__device__ __forceinline__ float edge_fn(float px, float py, float ax, float ay, float bx,
                                         float by) {
  return xsub(xmul(xsub(px, ax), xsub(by, ay)), xmul(xsub(py, ay), xsub(bx, ax)));
}

// centre ndc of pixel index i along a side of S1 pixels (the other side S2)
__device__ __forceinline__ float pix_ndc(int i, int S1, int S2) {
  float n = xadd(-1.f, xdiv((float)(2 * i + 1), (float)S1));
  if (S1 > S2) n = xdiv(xmul(n, (float)S1), (float)S2);
  return n;
}

struct Bary {
  float b0, b1, b2;
};

// screen barycentrics of (px, py), corrected for perspective by the depths
__device__ __forceinline__ Bary bary(float px, float py, float4 a, float4 b, float4 c) {
  const float area = xadd(edge_fn(c.x, c.y, a.x, a.y, b.x, b.y), kEps);
  const float w0 = xdiv(edge_fn(px, py, b.x, b.y, c.x, c.y), area);
  const float w1 = xdiv(edge_fn(px, py, c.x, c.y, a.x, a.y), area);
  const float w2 = xdiv(edge_fn(px, py, a.x, a.y, b.x, b.y), area);
  const float t0 = xmul(xmul(w0, b.z), c.z);
  const float t1 = xmul(xmul(a.z, w1), c.z);
  const float t2 = xmul(xmul(a.z, b.z), w2);
  const float d = fmaxf(xadd(xadd(t0, t1), t2), kEps);
  return Bary{xdiv(t0, d), xdiv(t1, d), xdiv(t2, d)};
}

__device__ __forceinline__ float bary_depth(Bary w, float4 a, float4 b, float4 c) {
  return xadd(xadd(xmul(w.b0, a.z), xmul(w.b1, b.z)), xmul(w.b2, c.z));
}

__device__ __forceinline__ bool face_of(const int64_t* __restrict__ faces, int f, int V,
                                        int idx[3]) {
  for (int k = 0; k < 3; ++k) {
    const int64_t i = faces[3 * (int64_t)f + k];
    if (i < 0 || i >= V) return false;
    idx[k] = (int)i;
  }
  return true;
}

__global__ void normals_kernel(const float* __restrict__ verts, int V,
                               const int64_t* __restrict__ faces, int F, float4* nrm) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F) return;
  int idx[3];
  if (!face_of(faces, f, V, idx)) return;
  float3 x[3];
  for (int k = 0; k < 3; ++k)
    x[k] = make_float3(verts[3 * idx[k]], verts[3 * idx[k] + 1], verts[3 * idx[k] + 2]);
  const float3 e0 = make_float3(x[2].x - x[1].x, x[2].y - x[1].y, x[2].z - x[1].z);
  const float3 e1 = make_float3(x[0].x - x[1].x, x[0].y - x[1].y, x[0].z - x[1].z);
  const float3 n = make_float3(e0.y * e1.z - e0.z * e1.y, e0.z * e1.x - e0.x * e1.z,
                               e0.x * e1.y - e0.y * e1.x);
  for (int k = 0; k < 3; ++k) {
    atomicAdd(&nrm[idx[k]].x, n.x);
    atomicAdd(&nrm[idx[k]].y, n.y);
    atomicAdd(&nrm[idx[k]].z, n.z);
  }
}

__global__ void vertex_kernel(totri_shading_t s, const float* __restrict__ verts, int V,
                              float4* __restrict__ proj, float4* __restrict__ nrm) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= V) return;
  const float X = verts[3 * v], Y = verts[3 * v + 1], Z = verts[3 * v + 2];
  float view[3];
  for (int i = 0; i < 3; ++i)
    view[i] = xadd(xadd(xadd(xmul(X, s.rotation[i]), xmul(Y, s.rotation[3 + i])),
                        xmul(Z, s.rotation[6 + i])),
                   s.translation[i]);
  proj[v] = make_float4(xdiv(xmul(s.focal[0], view[0]), view[2]),
                        xdiv(xmul(s.focal[1], view[1]), view[2]), view[2], 0.f);
  const float4 n = nrm[v];
  const float inv = 1.f / fmaxf(sqrtf(n.x * n.x + n.y * n.y + n.z * n.z), 1e-6f);
  nrm[v] = make_float4(n.x * inv, n.y * inv, n.z * inv, 0.f);
}

__global__ void raster_kernel(const float4* __restrict__ proj, int V,
                              const int64_t* __restrict__ faces, int F, int H, int W,
                              unsigned long long* __restrict__ zbuf) {
  const int f = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (f >= F) return;
  int idx[3];
  if (!face_of(faces, f, V, idx)) return;
  const float4 a = proj[idx[0]], b = proj[idx[1]], c = proj[idx[2]];
  if (fmaxf(fmaxf(a.z, b.z), c.z) < 0.f) return;  // behind the camera
  const float area = edge_fn(a.x, a.y, b.x, b.y, c.x, c.y);
  if (area <= kEps && area >= -kEps) return;
  const float xmin = fminf(fminf(a.x, b.x), c.x), xmax = fmaxf(fmaxf(a.x, b.x), c.x);
  const float ymin = fminf(fminf(a.y, b.y), c.y), ymax = fmaxf(fmaxf(a.y, b.y), c.y);
  if (!(xmin <= xmax) || !(ymin <= ymax)) return;
  // pixel indices whose centre can lie in the box (ndc index i ~ (n / s + 1) S / 2 - 1/2,
  // s the side's scale), one pixel of slack each side: the exact test decides
  const float scx = W > H ? (float)W / (float)H : 1.f, scy = H > W ? (float)H / (float)W : 1.f;
  const float fx0 = fmaxf(floorf((xmin / scx + 1.f) * 0.5f * W - 0.5f) - 1.f, 0.f);
  const float fx1 = fminf(ceilf((xmax / scx + 1.f) * 0.5f * W - 0.5f) + 1.f, (float)(W - 1));
  const float fy0 = fmaxf(floorf((ymin / scy + 1.f) * 0.5f * H - 0.5f) - 1.f, 0.f);
  const float fy1 = fminf(ceilf((ymax / scy + 1.f) * 0.5f * H - 0.5f) + 1.f, (float)(H - 1));
  if (!(fx0 <= fx1) || !(fy0 <= fy1)) return;
  const int x0 = (int)fx0, y0 = (int)fy0;
  const int nx = (int)fx1 - x0 + 1, n = nx * ((int)fy1 - y0 + 1);
  for (int p = lane; p < n; p += 32) {
    const int xi = x0 + p % nx, yi = y0 + p / nx;
    const float px = pix_ndc(xi, W, H), py = pix_ndc(yi, H, W);
    if (px > xmax || px < xmin || py > ymax || py < ymin) continue;
    const Bary w = bary(px, py, a, b, c);
    const float pz = bary_depth(w, a, b, c);
    if (!(pz >= 0.f)) continue;  // behind the image plane (or NaN)
    if (!(w.b0 > 0.f && w.b1 > 0.f && w.b2 > 0.f)) continue;
    const unsigned long long key =
        ((unsigned long long)__float_as_uint(xadd(pz, 0.f)) << 32) | (unsigned)f;
    atomicMin(zbuf + (int64_t)(H - 1 - yi) * W + (W - 1 - xi), key);
  }
}

__device__ __forceinline__ float seg_dist2(float px, float py, float ax, float ay, float bx,
                                           float by) {
  const float ex = bx - ax, ey = by - ay, qx = px - ax, qy = py - ay;
  const float bot = ex * ex + ey * ey;
  float t = bot > kEps ? (ex * qx + ey * qy) / bot : 0.f;
  t = fminf(fmaxf(t, 0.f), 1.f);
  const float dx = px - ((1.f - t) * ax + t * bx), dy = py - ((1.f - t) * ay + t * by);
  return dx * dx + dy * dy;
}

__device__ __forceinline__ float3 unit(float3 v) {
  const float inv = 1.f / fmaxf(sqrtf(v.x * v.x + v.y * v.y + v.z * v.z), 1e-6f);
  return make_float3(v.x * inv, v.y * inv, v.z * inv);
}

__global__ void shade_kernel(totri_shading_t s, const float* __restrict__ verts, int V,
                             const int64_t* __restrict__ faces, Colors col,
                             const float4* __restrict__ proj, const float4* __restrict__ nrm,
                             const unsigned long long* __restrict__ zbuf, int H, int W,
                             float* __restrict__ image, int* __restrict__ pix_to_face) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= H * W) return;
  const int64_t plane = (int64_t)H * W;
  const unsigned long long key = zbuf[p];
  if (key == ~0ull) {
    for (int ch = 0; ch < 3; ++ch) image[ch * plane + p] = s.background[ch];
    if (pix_to_face) pix_to_face[p] = -1;
    return;
  }
  const int f = (int)(unsigned)(key & 0xffffffffu);
  if (pix_to_face) pix_to_face[p] = f;
  int idx[3];
  face_of(faces, f, V, idx);  // valid: only valid faces are rasterised
  const float4 a = proj[idx[0]], b = proj[idx[1]], c = proj[idx[2]];
  const int r = p / W, cidx = p % W;
  const float px = pix_ndc(W - 1 - cidx, W, H), py = pix_ndc(H - 1 - r, H, W);
  const Bary w = bary(px, py, a, b, c);
  const float pz = __uint_as_float((unsigned)(key >> 32));
  const float bw[3] = {w.b0, w.b1, w.b2};
  float3 P = make_float3(0.f, 0.f, 0.f), Nrm = P, C = P;
  for (int k = 0; k < 3; ++k) {
    const int v = idx[k];
    const float4 n = nrm[v];
    const float3 cv = col.at(v);
    P.x += bw[k] * verts[3 * v];
    P.y += bw[k] * verts[3 * v + 1];
    P.z += bw[k] * verts[3 * v + 2];
    Nrm.x += bw[k] * n.x;
    Nrm.y += bw[k] * n.y;
    Nrm.z += bw[k] * n.z;
    C.x += bw[k] * cv.x;
    C.y += bw[k] * cv.y;
    C.z += bw[k] * cv.z;
  }
  const float3 N = unit(Nrm);
  const float3 L = unit(make_float3(s.light_location[0] - P.x, s.light_location[1] - P.y,
                                    s.light_location[2] - P.z));
  const float3 E = unit(make_float3(s.camera_center[0] - P.x, s.camera_center[1] - P.y,
                                    s.camera_center[2] - P.z));
  const float cs = N.x * L.x + N.y * L.y + N.z * L.z;
  const float3 R = make_float3(2.f * cs * N.x - L.x, 2.f * cs * N.y - L.y, 2.f * cs * N.z - L.z);
  const float er = fmaxf(E.x * R.x + E.y * R.y + E.z * R.z, 0.f) * (cs > 0.f ? 1.f : 0.f);
  const float spec = powf(er, s.shininess);
  const float diff = fmaxf(cs, 0.f);
  // blend weights of the face (one per pixel) and of the background
  const float d = fminf(fminf(seg_dist2(px, py, a.x, a.y, b.x, b.y),
                              seg_dist2(px, py, b.x, b.y, c.x, c.y)),
                        seg_dist2(px, py, c.x, c.y, a.x, a.y));
  const float prob = 1.f / (1.f + expf(-d / s.sigma));
  const float zinv = fmaxf((s.zfar - pz) / (s.zfar - s.znear), 1e-10f);
  const float delta = fmaxf(expf((1e-10f - zinv) / s.gamma), 1e-10f);
  const float tex[3] = {C.x, C.y, C.z};
  for (int ch = 0; ch < 3; ++ch) {
    const float shaded = (s.material_ambient[ch] * s.light_ambient[ch] +
                          s.material_diffuse[ch] * s.light_diffuse[ch] * diff) * tex[ch] +
                         s.material_specular[ch] * s.light_specular[ch] * spec;
    image[ch * plane + p] = (prob * shaded + delta * s.background[ch]) / (prob + delta);
  }
}

}  // namespace shade
}  // namespace totri

using namespace totri;

namespace {

struct ShadeLayout {
  size_t proj, nrm, total;
};

ShadeLayout shade_layout(int64_t V, int64_t H, int64_t W) {
  ShadeLayout l;
  l.proj = align_up(sizeof(unsigned long long) * (size_t)(H * W), 256);
  l.nrm = l.proj + align_up(sizeof(float4) * (size_t)V, 256);
  l.total = l.nrm + align_up(sizeof(float4) * (size_t)V, 256);
  return l;
}

}  // namespace

extern "C" {

size_t totri_shaded_raster_workspace(int64_t num_verts, int64_t height, int64_t width) {
  return shade_layout(num_verts, height, width).total;
}

int totri_shaded_raster(const totri_array_t* verts, const totri_array_t* faces,
                        const totri_array_t* colors, const totri_shading_t* shading,
                        const totri_array_t* image, const totri_array_t* pix_to_face, void* ws,
                        size_t ws_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  TOTRI_TRY(check_array(verts, "verts", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(verts, "verts", 1, 3));
  TOTRI_TRY(check_contiguous(verts, "verts"));
  TOTRI_TRY(check_array(faces, "faces", 2, TOTRI_INT64));
  TOTRI_TRY(check_dim(faces, "faces", 1, 3));
  TOTRI_TRY(check_contiguous(faces, "faces"));
  TOTRI_TRY(check_array(colors, "colors", 2, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(colors, "colors", 0, verts->shape[0]));
  TOTRI_TRY(check_dim(colors, "colors", 1, 3));
  TOTRI_TRY(check_array(image, "image", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(image, "image", 0, 3));
  TOTRI_TRY(check_contiguous(image, "image"));
  const int64_t H = image->shape[1], W = image->shape[2];
  if (pix_to_face) {
    TOTRI_TRY(check_array(pix_to_face, "pix_to_face", 2, TOTRI_INT32));
    TOTRI_TRY(check_dim(pix_to_face, "pix_to_face", 0, H));
    TOTRI_TRY(check_dim(pix_to_face, "pix_to_face", 1, W));
    TOTRI_TRY(check_contiguous(pix_to_face, "pix_to_face"));
  }
  if (!shading) return fail(TOTRI_ERR_INVALID_ARGUMENT, "shading settings are missing");
  if (H > (1 << 20) || W > (1 << 20) || H * W > INT32_MAX)
    return fail(TOTRI_ERR_UNSUPPORTED, "image too large");
  if (verts->shape[0] > INT32_MAX || faces->shape[0] > INT32_MAX / 32)
    return fail(TOTRI_ERR_UNSUPPORTED, "mesh too large");
  if (!(shading->zfar != shading->znear) || !(shading->sigma > 0.f) || !(shading->gamma > 0.f))
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "znear == zfar or non-positive sigma/gamma");
  if (H * W == 0) return TOTRI_OK;
  const int V = (int)verts->shape[0], F = (int)faces->shape[0];
  const ShadeLayout l = shade_layout(V, H, W);
  if (!ws || ws_bytes < l.total)
    return fail(TOTRI_ERR_WORKSPACE,
                "workspace of " + std::to_string(l.total) + " bytes required");
  char* base = static_cast<char*>(ws);
  unsigned long long* zbuf = reinterpret_cast<unsigned long long*>(base);
  float4* proj = reinterpret_cast<float4*>(base + l.proj);
  float4* nrm = reinterpret_cast<float4*>(base + l.nrm);
  const float* vp = static_cast<const float*>(verts->data);
  const int64_t* fp = static_cast<const int64_t*>(faces->data);
  TOTRI_CUDA(cudaMemsetAsync(zbuf, 0xff, sizeof(unsigned long long) * H * W, stream));
  if (V > 0) {
    TOTRI_CUDA(cudaMemsetAsync(nrm, 0, sizeof(float4) * V, stream));
    if (F > 0)
      TOTRI_KERNEL("shade normals", stream,
                   shade::normals_kernel<<<(unsigned)ceil_div(F, 256), 256, 0, stream>>>(
                       vp, V, fp, F, nrm));
    TOTRI_KERNEL("shade vertices", stream,
                 shade::vertex_kernel<<<(unsigned)ceil_div(V, 256), 256, 0, stream>>>(
                     *shading, vp, V, proj, nrm));
    if (F > 0)
      TOTRI_KERNEL("shade raster", stream,
                   shade::raster_kernel<<<(unsigned)ceil_div((int64_t)F * 32, 256), 256, 0,
                                          stream>>>(proj, V, fp, F, (int)H, (int)W, zbuf));
  }
  const shade::Colors col{static_cast<const float*>(colors->data), colors->strides[0],
                          colors->strides[1]};
  TOTRI_KERNEL("shade pixels", stream,
               shade::shade_kernel<<<(unsigned)ceil_div(H * W, 256), 256, 0, stream>>>(
                   *shading, vp, V, fp, col, proj, nrm, zbuf, (int)H, (int)W,
                   static_cast<float*>(image->data),
                   pix_to_face ? static_cast<int*>(pix_to_face->data) : nullptr));
  return TOTRI_OK;
}

}  // extern "C"
