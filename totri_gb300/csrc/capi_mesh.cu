// C ABI entry points of the mesh renderer (confocal and exhaustive).
#include <string>

#include "capi_common.cuh"
#include "mesh.cuh"
#include "mesh_kernels.cuh"

namespace totri {

thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg) {
  set_error(msg);
  return status;
}

int cuda_status(cudaError_t e, const char* what) {
  return fail(TOTRI_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

__global__ void zero3_kernel(float* p, int64_t sb, int64_t sv, int64_t sc, int64_t B, int64_t V,
                             int64_t C) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B * V * C) return;
  const int64_t c = i % C, v = (i / C) % V, b = i / (C * V);
  p[b * sb + v * sv + c * sc] = 0.f;
}

int zero3(const totri_array_t* a, cudaStream_t stream) {
  const int64_t n = numel(a);
  if (n == 0) return TOTRI_OK;
  if (is_contiguous(a)) {
    TOTRI_CUDA(cudaMemsetAsync(a->data, 0, sizeof(float) * n, stream));
    return TOTRI_OK;
  }
  TOTRI_KERNEL("zero gradient", stream,
               zero3_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, stream>>>(
                   static_cast<float*>(a->data), a->strides[0], a->strides[1], a->strides[2],
                   a->shape[0], a->shape[1], a->shape[2]));
  return TOTRI_OK;
}

struct MeshArgs {
  int64_t B, V, F, M;
  mesh::BuildInputs in;
};

// verts [B,V,3] f32, faces [B|1,F,3] i32/i64, material [B,V,M] f32 (M <= 4).
int check_mesh(const totri_array_t* verts, const totri_array_t* faces,
               const totri_array_t* material, MeshArgs& a) {
  TOTRI_TRY(check_array(verts, "verts", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(verts, "verts", 2, 3));
  a.B = verts->shape[0];
  a.V = verts->shape[1];
  TOTRI_TRY(check_array(faces, "faces", 3, -1));
  if (faces->dtype != TOTRI_INT32 && faces->dtype != TOTRI_INT64)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "faces must be int32 or int64");
  TOTRI_TRY(check_dim(faces, "faces", 2, 3));
  if (faces->shape[0] != a.B && faces->shape[0] != 1)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "faces batch size does not match verts");
  a.F = faces->shape[1];
  TOTRI_TRY(check_array(material, "material", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(material, "material", 0, a.B));
  TOTRI_TRY(check_dim(material, "material", 1, a.V));
  a.M = material->shape[2];
  if (a.M > 4) return fail(TOTRI_ERR_INVALID_ARGUMENT, "material may have at most 4 channels");
  if (a.F >= (int64_t)1 << 30 || a.V >= (int64_t)1 << 31)
    return fail(TOTRI_ERR_UNSUPPORTED, "too many faces or vertices");
  a.in.verts = view3f(verts);
  a.in.faces = mesh::BuildInputs{}.faces;
  a.in.faces.p = faces->data;
  a.in.faces.sb = faces->shape[0] == 1 ? 0 : faces->strides[0];
  a.in.faces.sn = faces->strides[1];
  a.in.faces.sc = faces->strides[2];
  a.in.faces.is64 = faces->dtype == TOTRI_INT64;
  a.in.material = view3f(material);
  a.in.M = (int)a.M;
  a.in.V = a.V;
  a.in.F = (int)a.F;
  return TOTRI_OK;
}

// points [B,N,3] f32 (N may be 0 for origins when allow_empty).
int check_points(const totri_array_t* p, const char* name, int64_t B, int64_t& N) {
  TOTRI_TRY(check_array(p, name, 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(p, name, 0, B));
  TOTRI_TRY(check_dim(p, name, 2, 3));
  N = p->shape[1];
  return TOTRI_OK;
}

int check_origin(const totri_array_t* o, const char* name, int64_t B, int64_t N, int& has) {
  int64_t No;
  TOTRI_TRY(check_points(o, name, B, No));
  if (No != 0 && No != N)
    return fail(TOTRI_ERR_INVALID_ARGUMENT,
                std::string(name) + " must have as many points as its wall points, or none");
  has = No > 0;
  return TOTRI_OK;
}

int check_workspace(void* ws, size_t bytes, size_t need) {
  if (need == 0) return TOTRI_OK;
  if (!ws || bytes < need)
    return fail(TOTRI_ERR_WORKSPACE, "workspace of " + std::to_string(need) +
                                         " bytes required, got " + std::to_string(bytes));
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0)
    return fail(TOTRI_ERR_WORKSPACE, "workspace must be 256-byte aligned");
  return TOTRI_OK;
}

int check_grads(const totri_array_t* vg, const totri_array_t* mg, const MeshArgs& a,
                mesh::GradOut& out) {
  TOTRI_TRY(check_array(vg, "verts_grad", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(vg, "verts_grad", 0, a.B));
  TOTRI_TRY(check_dim(vg, "verts_grad", 1, a.V));
  if (vg->shape[2] != 3 && vg->shape[2] != 0)
    return fail(TOTRI_ERR_INVALID_ARGUMENT, "verts_grad must be [B,V,3] or [B,V,0]");
  TOTRI_TRY(check_array(mg, "material_grad", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(mg, "material_grad", 0, a.B));
  TOTRI_TRY(check_dim(mg, "material_grad", 1, a.V));
  if (mg->shape[2] > 4) return fail(TOTRI_ERR_INVALID_ARGUMENT, "material_grad has > 4 channels");
  out.V = a.V;
  out.vg = vg->shape[2] == 3 ? static_cast<float*>(vg->data) : nullptr;
  out.vsb = vg->strides[0];
  out.vsv = vg->strides[1];
  out.vsc = vg->strides[2];
  out.mg = mg->shape[2] > 0 ? static_cast<float*>(mg->data) : nullptr;
  out.msb = mg->strides[0];
  out.msv = mg->strides[1];
  out.msc = mg->strides[2];
  return TOTRI_OK;
}

// Mask buffer of a prepared scene: [B][P][ceil(F/32)] words, 256-byte aligned.
int check_masks(const void* masks, size_t bytes, int64_t B, int64_t F, int64_t P) {
  const size_t need = mesh::mask_bytes(B, F, P);
  if (!masks || bytes < need)
    return fail(TOTRI_ERR_WORKSPACE, "mask buffer of " + std::to_string(need) +
                                         " bytes required, got " + std::to_string(bytes));
  if ((reinterpret_cast<uintptr_t>(masks) & 255) != 0)
    return fail(TOTRI_ERR_WORKSPACE, "mask buffer must be 256-byte aligned");
  return TOTRI_OK;
}

// Every (point, face) pair visible: the masks of the unoccluded renders.
int all_visible(const mesh::Scene& sc, int64_t P, cudaStream_t stream) {
  TOTRI_CUDA(cudaMemsetAsync(sc.mask, 0xff, sizeof(uint32_t) * (size_t)sc.B * P * sc.nch,
                             stream));
  return TOTRI_OK;
}

int confocal_grad_impl(const totri_array_t* verts, const totri_array_t* faces,
                       const totri_array_t* material, const totri_array_t* scan_points,
                       const totri_array_t* scan_origin, const totri_array_t* transient_grad,
                       const totri_array_t* verts_grad, const totri_array_t* material_grad,
                       float bin_width, float bin_offset, void* ws, size_t ws_bytes,
                       void* stream_, bool reuse, void* masks = nullptr,
                       size_t masks_bytes = 0, bool occluded = true) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  MeshArgs a;
  TOTRI_TRY(check_mesh(verts, faces, material, a));
  int64_t S;
  int has_origin;
  TOTRI_TRY(check_points(scan_points, "scan_points", a.B, S));
  TOTRI_TRY(check_origin(scan_origin, "scan_origin", a.B, S, has_origin));
  TOTRI_TRY(check_array(transient_grad, "transient_grad", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient_grad, "transient_grad", 0, a.B));
  TOTRI_TRY(check_dim(transient_grad, "transient_grad", 2, S));
  TOTRI_TRY(check_contiguous(transient_grad, "transient_grad"));
  const int64_t T = transient_grad->shape[1];
  mesh::GradOut out;
  TOTRI_TRY(check_grads(verts_grad, material_grad, a, out));
  TOTRI_TRY(zero3(verts_grad, stream));
  TOTRI_TRY(zero3(material_grad, stream));
  if (a.F == 0 || S == 0 || T == 0 || a.B == 0 || (!out.vg && !out.mg)) return TOTRI_OK;
  mesh::Scene sc;
  if (masks) {  // prepared scene, masks from totri_mesh_prepared_visibility
    TOTRI_TRY(check_workspace(ws, ws_bytes, mesh::layout(a.B, a.F, 0).total));
    TOTRI_TRY(check_masks(masks, masks_bytes, a.B, a.F, S));
    sc = mesh::scene_with_masks(ws, a.B, a.F, masks, S);
  } else {
    TOTRI_TRY(check_workspace(ws, ws_bytes, mesh::layout(a.B, a.F, S).total));
    sc = mesh::scene_from_workspace(ws, a.B, a.F, S);
  }
  if (!reuse && !masks) {
    TOTRI_TRY(mesh::build_scene(sc, a.in, stream));
    if (occluded)
      TOTRI_TRY(mesh::launch_visibility(sc, view3f(scan_points), (int)S, 0, false, stream));
    else
      TOTRI_TRY(all_visible(sc, S, stream));
  }
  return mesh::launch_confocal_grad(sc, view3f(scan_points), view3f(scan_origin), has_origin,
                                    static_cast<const float*>(transient_grad->data), (int)T,
                                    (int)S, bin_width, bin_offset, out, stream);
}

struct ExhArgs {
  MeshArgs m;
  int64_t S, L, T;
  mesh::Origins org;
};

int check_exhaustive(const totri_array_t* verts, const totri_array_t* faces,
                     const totri_array_t* material, const totri_array_t* scan_points,
                     const totri_array_t* laser_points, const totri_array_t* scan_origin,
                     const totri_array_t* laser_origin, const totri_array_t* tr, const char* tname,
                     ExhArgs& e) {
  TOTRI_TRY(check_mesh(verts, faces, material, e.m));
  TOTRI_TRY(check_points(scan_points, "scan_points", e.m.B, e.S));
  TOTRI_TRY(check_points(laser_points, "laser_points", e.m.B, e.L));
  TOTRI_TRY(check_origin(scan_origin, "scan_origin", e.m.B, e.S, e.org.has_so));
  TOTRI_TRY(check_origin(laser_origin, "laser_origin", e.m.B, e.L, e.org.has_lo));
  e.org.so = view3f(scan_origin);
  e.org.lo = view3f(laser_origin);
  TOTRI_TRY(check_array(tr, tname, 4, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(tr, tname, 0, e.m.B));
  TOTRI_TRY(check_dim(tr, tname, 2, e.S));
  TOTRI_TRY(check_dim(tr, tname, 3, e.L));
  TOTRI_TRY(check_contiguous(tr, tname));
  e.T = tr->shape[1];
  if (e.S + e.L >= (int64_t)1 << 30 || e.T >= (int64_t)1 << 30)
    return fail(TOTRI_ERR_UNSUPPORTED, "too many wall points or bins");
  return TOTRI_OK;
}

int exhaustive_grad_impl(const totri_array_t* verts, const totri_array_t* faces,
                         const totri_array_t* material, const totri_array_t* scan_points,
                         const totri_array_t* laser_points, const totri_array_t* scan_origin,
                         const totri_array_t* laser_origin, const totri_array_t* transient_grad,
                         const totri_array_t* verts_grad, const totri_array_t* material_grad,
                         float bw, float bo, void* ws, size_t ws_bytes, void* stream_,
                         bool reuse) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  ExhArgs e;
  TOTRI_TRY(check_exhaustive(verts, faces, material, scan_points, laser_points, scan_origin,
                             laser_origin, transient_grad, "transient_grad", e));
  mesh::GradOut out;
  TOTRI_TRY(check_grads(verts_grad, material_grad, e.m, out));
  TOTRI_TRY(zero3(verts_grad, stream));
  TOTRI_TRY(zero3(material_grad, stream));
  if (e.m.F == 0 || e.S == 0 || e.L == 0 || e.T == 0 || e.m.B == 0 || (!out.vg && !out.mg))
    return TOTRI_OK;
  const int64_t P = e.S + e.L;
  const size_t base = mesh::layout(e.m.B, e.m.F, P).total;
  TOTRI_TRY(check_workspace(ws, ws_bytes, base));
  const mesh::Scene sc = mesh::scene_from_workspace(ws, e.m.B, e.m.F, P);
  if (!reuse) {
    TOTRI_TRY(mesh::build_scene(sc, e.m.in, stream));
    TOTRI_TRY(mesh::launch_visibility(sc, view3f(scan_points), (int)e.S, 0, false, stream));
    TOTRI_TRY(
        mesh::launch_visibility(sc, view3f(laser_points), (int)e.L, (int)e.S, false, stream));
  }
  // the bytes past the mesh layout (256-aligned) are the optional scratch
  void* scratch = ws_bytes > base ? static_cast<char*>(ws) + base : nullptr;
  return mesh::launch_exhaustive_grad(sc, view3f(scan_points), view3f(laser_points), e.org,
                                      (int)e.S, (int)e.L,
                                      static_cast<const float*>(transient_grad->data), (int)e.T,
                                      bw, bo, out, scratch, scratch ? ws_bytes - base : 0,
                                      stream);
}

}  // namespace
}  // namespace totri

using namespace totri;

extern "C" {

const char* totri_version(void) { return "totri_gb300 0.1.0 (sm_103a)"; }

const char* totri_last_error(void) { return g_last_error.c_str(); }

size_t totri_mesh_workspace(int64_t batch, int64_t num_verts, int64_t num_faces,
                            int64_t num_points) {
  (void)num_verts;
  if (batch <= 0 || num_faces <= 0 || num_points < 0) return 0;
  return mesh::layout(batch, num_faces, num_points).total;
}

size_t totri_mesh_exhaustive_grad_scratch(int64_t num_scan_points, int64_t num_laser_points,
                                          int64_t num_bins) {
  return mesh::exh_grad_scratch_bytes(num_scan_points, num_laser_points, num_bins);
}

static int confocal_forward_impl(const totri_array_t* verts, const totri_array_t* faces,
                                 const totri_array_t* material,
                                 const totri_array_t* scan_points,
                                 const totri_array_t* scan_origin,
                                 const totri_array_t* transient, float bin_width,
                                 float bin_offset, void* ws, size_t ws_bytes, void* stream_,
                                 bool occluded) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  MeshArgs a;
  TOTRI_TRY(check_mesh(verts, faces, material, a));
  int64_t S;
  int has_origin;
  TOTRI_TRY(check_points(scan_points, "scan_points", a.B, S));
  TOTRI_TRY(check_origin(scan_origin, "scan_origin", a.B, S, has_origin));
  TOTRI_TRY(check_array(transient, "transient", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient, "transient", 0, a.B));
  TOTRI_TRY(check_dim(transient, "transient", 2, S));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  const int64_t T = transient->shape[1];
  if (numel(transient) == 0) return TOTRI_OK;
  if (a.F == 0) {
    TOTRI_CUDA(cudaMemsetAsync(transient->data, 0, sizeof(float) * numel(transient), stream));
    return TOTRI_OK;
  }
  if (S >= (int64_t)1 << 30 || T >= (int64_t)1 << 30)
    return fail(TOTRI_ERR_UNSUPPORTED, "too many scan points or bins");
  const mesh::Layout L = mesh::layout(a.B, a.F, S);
  TOTRI_TRY(check_workspace(ws, ws_bytes, L.total));
  const mesh::Scene sc = mesh::scene_from_workspace(ws, a.B, a.F, S);
  TOTRI_TRY(mesh::build_scene(sc, a.in, stream));
  if (occluded)
    TOTRI_TRY(mesh::launch_visibility(sc, view3f(scan_points), (int)S, 0, false, stream));
  else
    TOTRI_TRY(all_visible(sc, S, stream));
  return mesh::launch_confocal_splat(sc, view3f(scan_points), view3f(scan_origin), has_origin,
                                     static_cast<float*>(transient->data), (int)T, (int)S,
                                     bin_width, bin_offset, stream);
}

int totri_mesh_confocal_forward(const totri_array_t* verts, const totri_array_t* faces,
                                const totri_array_t* material,
                                const totri_array_t* scan_points,
                                const totri_array_t* scan_origin,
                                const totri_array_t* transient, float bin_width,
                                float bin_offset, int model, void* ws, size_t ws_bytes,
                                void* stream) {
  (void)model;
  return confocal_forward_impl(verts, faces, material, scan_points, scan_origin, transient,
                               bin_width, bin_offset, ws, ws_bytes, stream, true);
}

int totri_mesh_confocal_forward_unoccluded(const totri_array_t* verts,
                                           const totri_array_t* faces,
                                           const totri_array_t* material,
                                           const totri_array_t* scan_points,
                                           const totri_array_t* scan_origin,
                                           const totri_array_t* transient, float bin_width,
                                           float bin_offset, int model, void* ws,
                                           size_t ws_bytes, void* stream) {
  (void)model;
  return confocal_forward_impl(verts, faces, material, scan_points, scan_origin, transient,
                               bin_width, bin_offset, ws, ws_bytes, stream, false);
}

int totri_mesh_confocal_grad_verts_unoccluded(
    const totri_array_t* verts, const totri_array_t* faces, const totri_array_t* material,
    const totri_array_t* scan_points, const totri_array_t* scan_origin,
    const totri_array_t* transient_grad, const totri_array_t* verts_grad,
    const totri_array_t* material_grad, float bin_width, float bin_offset, int model, void* ws,
    size_t ws_bytes, void* stream) {
  (void)model;
  return confocal_grad_impl(verts, faces, material, scan_points, scan_origin, transient_grad,
                            verts_grad, material_grad, bin_width, bin_offset, ws, ws_bytes,
                            stream, false, nullptr, 0, false);
}

int totri_mesh_confocal_grad_verts(const totri_array_t* verts, const totri_array_t* faces,
                                   const totri_array_t* material,
                                   const totri_array_t* scan_points,
                                   const totri_array_t* scan_origin,
                                   const totri_array_t* transient_grad,
                                   const totri_array_t* verts_grad,
                                   const totri_array_t* material_grad, float bin_width,
                                   float bin_offset, int model, void* ws, size_t ws_bytes,
                                   void* stream) {
  (void)model;
  return confocal_grad_impl(verts, faces, material, scan_points, scan_origin, transient_grad,
                            verts_grad, material_grad, bin_width, bin_offset, ws, ws_bytes,
                            stream, false);
}

int totri_mesh_confocal_grad_verts_reuse(const totri_array_t* verts, const totri_array_t* faces,
                                         const totri_array_t* material,
                                         const totri_array_t* scan_points,
                                         const totri_array_t* scan_origin,
                                         const totri_array_t* transient_grad,
                                         const totri_array_t* verts_grad,
                                         const totri_array_t* material_grad, float bin_width,
                                         float bin_offset, int model, void* ws,
                                         size_t ws_bytes, void* stream) {
  (void)model;
  return confocal_grad_impl(verts, faces, material, scan_points, scan_origin, transient_grad,
                            verts_grad, material_grad, bin_width, bin_offset, ws, ws_bytes,
                            stream, true);
}

int totri_mesh_exhaustive_forward(const totri_array_t* verts, const totri_array_t* faces,
                                  const totri_array_t* material,
                                  const totri_array_t* scan_points,
                                  const totri_array_t* laser_points,
                                  const totri_array_t* scan_origin,
                                  const totri_array_t* laser_origin,
                                  const totri_array_t* transient, float bw, float bo, int model,
                                  void* ws, size_t ws_bytes, void* stream_) {
  (void)model;
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  ExhArgs e;
  TOTRI_TRY(check_exhaustive(verts, faces, material, scan_points, laser_points, scan_origin,
                             laser_origin, transient, "transient", e));
  if (numel(transient) == 0) return TOTRI_OK;
  if (e.m.F == 0) {
    TOTRI_CUDA(cudaMemsetAsync(transient->data, 0, sizeof(float) * numel(transient), stream));
    return TOTRI_OK;
  }
  const int64_t P = e.S + e.L;
  TOTRI_TRY(check_workspace(ws, ws_bytes, mesh::layout(e.m.B, e.m.F, P).total));
  const mesh::Scene sc = mesh::scene_from_workspace(ws, e.m.B, e.m.F, P);
  TOTRI_TRY(mesh::build_scene(sc, e.m.in, stream));
  TOTRI_TRY(mesh::launch_visibility(sc, view3f(scan_points), (int)e.S, 0, false, stream));
  TOTRI_TRY(mesh::launch_visibility(sc, view3f(laser_points), (int)e.L, (int)e.S, false, stream));
  return mesh::launch_exhaustive_splat(sc, view3f(scan_points), view3f(laser_points), e.org,
                                       (int)e.S, (int)e.L, static_cast<float*>(transient->data),
                                       (int)e.T, bw, bo, stream);
}

int totri_mesh_exhaustive_grad_verts(const totri_array_t* verts, const totri_array_t* faces,
                                     const totri_array_t* material,
                                     const totri_array_t* scan_points,
                                     const totri_array_t* laser_points,
                                     const totri_array_t* scan_origin,
                                     const totri_array_t* laser_origin,
                                     const totri_array_t* transient_grad,
                                     const totri_array_t* verts_grad,
                                     const totri_array_t* material_grad, float bw, float bo,
                                     int model, void* ws, size_t ws_bytes, void* stream) {
  (void)model;
  return exhaustive_grad_impl(verts, faces, material, scan_points, laser_points, scan_origin,
                              laser_origin, transient_grad, verts_grad, material_grad, bw, bo, ws,
                              ws_bytes, stream, false);
}

int totri_mesh_exhaustive_grad_verts_reuse(
    const totri_array_t* verts, const totri_array_t* faces, const totri_array_t* material,
    const totri_array_t* scan_points, const totri_array_t* laser_points,
    const totri_array_t* scan_origin, const totri_array_t* laser_origin,
    const totri_array_t* transient_grad, const totri_array_t* verts_grad,
    const totri_array_t* material_grad, float bw, float bo, int model, void* ws, size_t ws_bytes,
    void* stream) {
  (void)model;
  return exhaustive_grad_impl(verts, faces, material, scan_points, laser_points, scan_origin,
                              laser_origin, transient_grad, verts_grad, material_grad, bw, bo, ws,
                              ws_bytes, stream, true);
}

int totri_mesh_visibility(const totri_array_t* verts, const totri_array_t* faces,
                          const totri_array_t* points, const totri_array_t* mask,
                          int brute_force, void* ws, size_t ws_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  const totri_array_t* material = nullptr;
  // Visibility needs no material: use an empty [B,V,0] view.
  TOTRI_TRY(check_array(verts, "verts", 3, TOTRI_FLOAT32));
  totri_array_t empty{};
  empty.data = verts->data;
  empty.dtype = TOTRI_FLOAT32;
  empty.ndim = 3;
  empty.shape[0] = verts->shape[0];
  empty.shape[1] = verts->shape[1];
  empty.shape[2] = 0;
  empty.strides[0] = 0;
  empty.strides[1] = 0;
  empty.strides[2] = 1;
  material = &empty;
  MeshArgs a;
  TOTRI_TRY(check_mesh(verts, faces, material, a));
  int64_t P;
  TOTRI_TRY(check_points(points, "points", a.B, P));
  const int64_t nch = (a.F + 31) / 32;
  TOTRI_TRY(check_array(mask, "mask", 3, TOTRI_INT32));
  TOTRI_TRY(check_dim(mask, "mask", 0, a.B));
  TOTRI_TRY(check_dim(mask, "mask", 1, P));
  TOTRI_TRY(check_dim(mask, "mask", 2, nch));
  TOTRI_TRY(check_contiguous(mask, "mask"));
  if (a.F == 0 || P == 0 || a.B == 0) return TOTRI_OK;
  const mesh::Layout L = mesh::layout(a.B, a.F, P);
  TOTRI_TRY(check_workspace(ws, ws_bytes, L.total));
  const mesh::Scene sc = mesh::scene_from_workspace(ws, a.B, a.F, P);
  TOTRI_TRY(mesh::build_scene(sc, a.in, stream));
  TOTRI_TRY(mesh::launch_visibility(sc, view3f(points), (int)P, 0, brute_force != 0, stream));
  return mesh::launch_mask_unsort(sc, (int)P, static_cast<uint32_t*>(mask->data), stream);
}

size_t totri_mesh_mask_bytes(int64_t batch, int64_t num_faces, int64_t num_points) {
  if (batch <= 0 || num_faces <= 0 || num_points < 0) return 0;
  return mesh::mask_bytes(batch, num_faces, num_points);
}

int totri_mesh_prepare(const totri_array_t* verts, const totri_array_t* faces,
                       const totri_array_t* material, void* ws, size_t ws_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  MeshArgs a;
  TOTRI_TRY(check_mesh(verts, faces, material, a));
  if (a.F == 0 || a.B == 0) return TOTRI_OK;
  TOTRI_TRY(check_workspace(ws, ws_bytes, mesh::layout(a.B, a.F, 0).total));
  return mesh::build_scene(mesh::scene_from_workspace(ws, a.B, a.F, 0), a.in, stream);
}

int totri_mesh_prepared_visibility(const totri_array_t* verts, const totri_array_t* faces,
                                   const totri_array_t* material, const totri_array_t* points,
                                   const void* ws, size_t ws_bytes, void* masks,
                                   size_t masks_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  MeshArgs a;
  TOTRI_TRY(check_mesh(verts, faces, material, a));
  int64_t P;
  TOTRI_TRY(check_points(points, "points", a.B, P));
  if (a.F == 0 || P == 0 || a.B == 0) return TOTRI_OK;
  if (P >= (int64_t)1 << 30) return fail(TOTRI_ERR_UNSUPPORTED, "too many points");
  TOTRI_TRY(check_workspace(const_cast<void*>(ws), ws_bytes, mesh::layout(a.B, a.F, 0).total));
  TOTRI_TRY(check_masks(masks, masks_bytes, a.B, a.F, P));
  const mesh::Scene sc = mesh::scene_with_masks(const_cast<void*>(ws), a.B, a.F, masks, P);
  return mesh::launch_visibility(sc, view3f(points), (int)P, 0, false, stream);
}

int totri_mesh_prepared_confocal_forward(const totri_array_t* verts, const totri_array_t* faces,
                                         const totri_array_t* material,
                                         const totri_array_t* scan_points,
                                         const totri_array_t* scan_origin,
                                         const totri_array_t* transient, float bin_width,
                                         float bin_offset, const void* ws, size_t ws_bytes,
                                         const void* masks, size_t masks_bytes, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  MeshArgs a;
  TOTRI_TRY(check_mesh(verts, faces, material, a));
  int64_t S;
  int has_origin;
  TOTRI_TRY(check_points(scan_points, "scan_points", a.B, S));
  TOTRI_TRY(check_origin(scan_origin, "scan_origin", a.B, S, has_origin));
  TOTRI_TRY(check_array(transient, "transient", 3, TOTRI_FLOAT32));
  TOTRI_TRY(check_dim(transient, "transient", 0, a.B));
  TOTRI_TRY(check_dim(transient, "transient", 2, S));
  TOTRI_TRY(check_contiguous(transient, "transient"));
  const int64_t T = transient->shape[1];
  if (numel(transient) == 0) return TOTRI_OK;
  if (a.F == 0) {
    TOTRI_CUDA(cudaMemsetAsync(transient->data, 0, sizeof(float) * numel(transient), stream));
    return TOTRI_OK;
  }
  if (S >= (int64_t)1 << 30 || T >= (int64_t)1 << 30)
    return fail(TOTRI_ERR_UNSUPPORTED, "too many scan points or bins");
  TOTRI_TRY(check_workspace(const_cast<void*>(ws), ws_bytes, mesh::layout(a.B, a.F, 0).total));
  TOTRI_TRY(check_masks(masks, masks_bytes, a.B, a.F, S));
  const mesh::Scene sc =
      mesh::scene_with_masks(const_cast<void*>(ws), a.B, a.F, const_cast<void*>(masks), S);
  return mesh::launch_confocal_splat(sc, view3f(scan_points), view3f(scan_origin), has_origin,
                                     static_cast<float*>(transient->data), (int)T, (int)S,
                                     bin_width, bin_offset, stream);
}

int totri_mesh_prepared_confocal_grad_verts(
    const totri_array_t* verts, const totri_array_t* faces, const totri_array_t* material,
    const totri_array_t* scan_points, const totri_array_t* scan_origin,
    const totri_array_t* transient_grad, const totri_array_t* verts_grad,
    const totri_array_t* material_grad, float bin_width, float bin_offset, const void* ws,
    size_t ws_bytes, const void* masks, size_t masks_bytes, void* stream) {
  if (!masks) return fail(TOTRI_ERR_WORKSPACE, "mask buffer missing");
  return confocal_grad_impl(verts, faces, material, scan_points, scan_origin, transient_grad,
                            verts_grad, material_grad, bin_width, bin_offset,
                            const_cast<void*>(ws), ws_bytes, stream, true,
                            const_cast<void*>(masks), masks_bytes);
}

int totri_mesh_workspace_status(const void* ws, size_t ws_bytes, uint32_t* flags, void* stream_) {
  cudaStream_t stream = static_cast<cudaStream_t>(stream_);
  if (!ws || ws_bytes < 256) return fail(TOTRI_ERR_WORKSPACE, "workspace missing");
  uint32_t h = 0;
  TOTRI_CUDA(cudaMemcpyAsync(&h, ws, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
  TOTRI_CUDA(cudaStreamSynchronize(stream));
  if (flags) *flags = h;
  if (h != 0) return fail(TOTRI_ERR_DEVICE, "device status flags " + std::to_string(h));
  return TOTRI_OK;
}

}  // extern "C"
