// Runs the reference's four OptiX ray-generation programs
// (src/render/program/mesh_{confocal,exhaustive}_{forward,grad_verts}_optix.cu,
// compiled for the CPU from the reference tree with stub headers) over every
// (face, scan point[, laser point]) launch index. optixTrace is answered from
// visibility masks passed in by the caller. Test infrastructure only.
#include "cuda_host_shim.h"

#include <torch/extension.h>

#include "render/program/mesh_confocal_forward.h"
#include "render/program/mesh_confocal_grad_verts.h"
#include "render/program/mesh_exhaustive_forward.h"
#include "render/program/mesh_exhaustive_grad_verts.h"

using namespace totri::render;

extern "C" {
MeshConfocalForwardLaunchParams mesh_confocal_forward_launch_params;
MeshConfocalGradVertsLaunchParams mesh_confocal_grad_verts_launch_params;
MeshExhaustiveForwardLaunchParams mesh_exhaustive_forward_launch_params;
MeshExhaustiveGradVertsLaunchParams mesh_exhaustive_grad_verts_launch_params;
void ref_mcf_rg();
void ref_mcg_rg();
void ref_mef_rg();
void ref_meg_rg();
}

namespace {
thread_local const uint8_t* t_vis_s = nullptr;  // [S][F]
thread_local const uint8_t* t_vis_l = nullptr;  // [L][F]
thread_local int t_calls = 0;
thread_local long t_F = 0;

unsigned int trace_confocal(float3, float3, float, float) {
  const uint3 i = refshim::launch_index;
  return t_vis_s[(long)i.y * t_F + i.x] ? i.x : 4294967295u;
}
// The exhaustive programs trace from the laser point first, then from the
// scan point (mesh_exhaustive_forward_optix.cu:47-94).
unsigned int trace_exhaustive(float3, float3, float, float) {
  const uint3 i = refshim::launch_index;
  const bool vis = (t_calls++ == 0) ? t_vis_l[(long)i.z * t_F + i.x] : t_vis_s[(long)i.y * t_F + i.x];
  return vis ? i.x : 4294967295u;
}

std::vector<uint3> faces_buffer(const int32_t* faces, int F) {
  std::vector<uint3> out(F);
  for (int f = 0; f < F; ++f)
    out[f] = make_uint3((unsigned)faces[3 * f], (unsigned)faces[3 * f + 1], (unsigned)faces[3 * f + 2]);
  return out;
}

template <typename Fn>
void run(int F, int S, int L, Fn&& fn) {
#pragma omp parallel for schedule(dynamic, 8)
  for (int f = 0; f < F; ++f)
    for (int s = 0; s < S; ++s)
      for (int l = 0; l < L; ++l) {
        refshim::launch_index = make_uint3(f, s, l);
        t_calls = 0;
        fn();
      }
}
}  // namespace

extern "C" {

int ref_mesh_confocal_forward(float* verts, int V, const int32_t* faces, int F, float* material,
                              int M, float* sp, int S, float* so, int So, const uint8_t* vis,
                              float* transient, int T, float bw, float bo) {
  std::vector<uint3> fb = faces_buffer(faces, F);
  auto& p = mesh_confocal_forward_launch_params;
  p.verts = at::make_accessor<float, 3>(verts, {1, V, 3});
  p.material = at::make_accessor<float, 3>(material, {1, V, M});
  p.scan_points = at::make_accessor<float, 3>(sp, {1, S, 3});
  p.scan_origin = at::make_accessor<float, 3>(so, {1, So, 3});
  p.transient = at::make_accessor<float, 3>(transient, {1, T, S});
  p.faces = fb.data();
  p.bin_width = bw;
  p.bin_offset = bo;
  p.model = 0;
  p.b = 0;
  run(F, S, 1, [&] {
    t_vis_s = vis;
    t_F = F;
    refshim::trace_fn = trace_confocal;
    ref_mcf_rg();
  });
  return 0;
}

int ref_mesh_confocal_grad(float* verts, int V, const int32_t* faces, int F, float* material,
                           int M, float* sp, int S, float* so, int So, const uint8_t* vis,
                           float* tgrad, int T, float* vgrad, int vch, float* mgrad, int mch,
                           float bw, float bo) {
  std::vector<uint3> fb = faces_buffer(faces, F);
  auto& p = mesh_confocal_grad_verts_launch_params;
  p.verts = at::make_accessor<float, 3>(verts, {1, V, 3});
  p.material = at::make_accessor<float, 3>(material, {1, V, M});
  p.scan_points = at::make_accessor<float, 3>(sp, {1, S, 3});
  p.scan_origin = at::make_accessor<float, 3>(so, {1, So, 3});
  p.transient_grad = at::make_accessor<float, 3>(tgrad, {1, T, S});
  p.verts_grad = at::make_accessor<float, 3>(vgrad, {1, V, vch});
  p.material_grad = at::make_accessor<float, 3>(mgrad, {1, V, mch});
  p.faces = fb.data();
  p.bin_width = bw;
  p.bin_offset = bo;
  p.model = 0;
  p.b = 0;
  run(F, S, 1, [&] {
    t_vis_s = vis;
    t_F = F;
    refshim::trace_fn = trace_confocal;
    ref_mcg_rg();
  });
  return 0;
}

int ref_mesh_exhaustive_forward(float* verts, int V, const int32_t* faces, int F, float* material,
                                int M, float* sp, int S, float* lp, int L, float* so, int So,
                                float* lo, int Lo, const uint8_t* vis_s, const uint8_t* vis_l,
                                float* transient, int T, float bw, float bo) {
  std::vector<uint3> fb = faces_buffer(faces, F);
  auto& p = mesh_exhaustive_forward_launch_params;
  p.verts = at::make_accessor<float, 3>(verts, {1, V, 3});
  p.material = at::make_accessor<float, 3>(material, {1, V, M});
  p.scan_points = at::make_accessor<float, 3>(sp, {1, S, 3});
  p.laser_points = at::make_accessor<float, 3>(lp, {1, L, 3});
  p.scan_origin = at::make_accessor<float, 3>(so, {1, So, 3});
  p.laser_origin = at::make_accessor<float, 3>(lo, {1, Lo, 3});
  p.transient = at::make_accessor<float, 4>(transient, {1, T, S, L});
  p.faces = fb.data();
  p.bin_width = bw;
  p.bin_offset = bo;
  p.model = 0;
  p.b = 0;
  run(F, S, L, [&] {
    t_vis_s = vis_s;
    t_vis_l = vis_l;
    t_F = F;
    refshim::trace_fn = trace_exhaustive;
    ref_mef_rg();
  });
  return 0;
}

int ref_mesh_exhaustive_grad(float* verts, int V, const int32_t* faces, int F, float* material,
                             int M, float* sp, int S, float* lp, int L, float* so, int So,
                             float* lo, int Lo, const uint8_t* vis_s, const uint8_t* vis_l,
                             float* tgrad, int T, float* vgrad, int vch, float* mgrad, int mch,
                             float bw, float bo) {
  std::vector<uint3> fb = faces_buffer(faces, F);
  auto& p = mesh_exhaustive_grad_verts_launch_params;
  p.verts = at::make_accessor<float, 3>(verts, {1, V, 3});
  p.material = at::make_accessor<float, 3>(material, {1, V, M});
  p.scan_points = at::make_accessor<float, 3>(sp, {1, S, 3});
  p.laser_points = at::make_accessor<float, 3>(lp, {1, L, 3});
  p.scan_origin = at::make_accessor<float, 3>(so, {1, So, 3});
  p.laser_origin = at::make_accessor<float, 3>(lo, {1, Lo, 3});
  p.transient_grad = at::make_accessor<float, 4>(tgrad, {1, T, S, L});
  p.verts_grad = at::make_accessor<float, 3>(vgrad, {1, V, vch});
  p.material_grad = at::make_accessor<float, 3>(mgrad, {1, V, mch});
  p.faces = fb.data();
  p.bin_width = bw;
  p.bin_offset = bo;
  p.model = 0;
  p.b = 0;
  run(F, S, L, [&] {
    t_vis_s = vis_s;
    t_vis_l = vis_l;
    t_F = F;
    refshim::trace_fn = trace_exhaustive;
    ref_meg_rg();
  });
  return 0;
}

}  // extern "C"
