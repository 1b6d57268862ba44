// Entry points whose kernels are not built yet: they fail loudly.
#include "capi_common.cuh"

using namespace totri;

namespace {
int pending(const char* name) {
  return fail(TOTRI_ERR_UNSUPPORTED, std::string(name) + " is not implemented in this build");
}
}  // namespace

extern "C" {

int totri_mesh_exhaustive_forward(const totri_array_t*, const totri_array_t*,
                                  const totri_array_t*, const totri_array_t*,
                                  const totri_array_t*, const totri_array_t*,
                                  const totri_array_t*, const totri_array_t*, float, float, int,
                                  void*, size_t, void*) {
  return pending("mesh_exhaustive_forward");
}

int totri_mesh_exhaustive_grad_verts(const totri_array_t*, const totri_array_t*,
                                     const totri_array_t*, const totri_array_t*,
                                     const totri_array_t*, const totri_array_t*,
                                     const totri_array_t*, const totri_array_t*,
                                     const totri_array_t*, const totri_array_t*, float, float,
                                     int, void*, size_t, void*) {
  return pending("mesh_exhaustive_grad_verts");
}

int totri_mesh_exhaustive_grad_verts_reuse(const totri_array_t*, const totri_array_t*,
                                           const totri_array_t*, const totri_array_t*,
                                           const totri_array_t*, const totri_array_t*,
                                           const totri_array_t*, const totri_array_t*,
                                           const totri_array_t*, const totri_array_t*, float,
                                           float, int, void*, size_t, void*) {
  return pending("mesh_exhaustive_grad_verts_reuse");
}

int totri_volume_confocal_forward(const totri_array_t*, const totri_array_t*,
                                  const totri_array_t*, const float*, const float*, float, float,
                                  void*) {
  return pending("volume_confocal_forward");
}

int totri_volume_confocal_grad_volume(const totri_array_t*, const totri_array_t*,
                                      const totri_array_t*, const float*, const float*, float,
                                      float, void*) {
  return pending("volume_confocal_grad_volume");
}

int totri_volume_confocal_adjoint(const totri_array_t*, const totri_array_t*,
                                  const totri_array_t*, const float*, const float*, float, float,
                                  void*) {
  return pending("volume_confocal_adjoint");
}

int totri_volume_confocal_grad_measurement_points(const totri_array_t*, const totri_array_t*,
                                                  const totri_array_t*, const totri_array_t*,
                                                  const float*, const float*, float, float,
                                                  void*) {
  return pending("volume_confocal_grad_measurement_points");
}

int totri_volume_exhaustive_forward(const totri_array_t*, const totri_array_t*,
                                    const totri_array_t*, const totri_array_t*,
                                    const totri_array_t*, const totri_array_t*, const float*,
                                    const float*, float, float, void*) {
  return pending("volume_exhaustive_forward");
}

int totri_volume_exhaustive_grad_volume(const totri_array_t*, const totri_array_t*,
                                        const totri_array_t*, const totri_array_t*,
                                        const totri_array_t*, const totri_array_t*,
                                        const float*, const float*, float, float, void*) {
  return pending("volume_exhaustive_grad_volume");
}

int totri_backprojection_confocal_velten_forward(const totri_array_t*, const totri_array_t*,
                                                 const totri_array_t*, const totri_array_t*,
                                                 const float*, const float*, float, float,
                                                 void*) {
  return pending("backprojection_confocal_velten_forward");
}

int totri_backprojection_confocal_velten_adjoint(const totri_array_t*, const totri_array_t*,
                                                 const totri_array_t*, const totri_array_t*,
                                                 const float*, const float*, float, float,
                                                 void*) {
  return pending("backprojection_confocal_velten_adjoint");
}

int totri_backprojection_exhaustive_velten_forward(const totri_array_t*, const totri_array_t*,
                                                   const totri_array_t*, const totri_array_t*,
                                                   const totri_array_t*, const totri_array_t*,
                                                   const float*, const float*, float, float,
                                                   void*) {
  return pending("backprojection_exhaustive_velten_forward");
}

int totri_backprojection_exhaustive_arellano_forward(const totri_array_t*, const totri_array_t*,
                                                     const totri_array_t*, const totri_array_t*,
                                                     const totri_array_t*, const totri_array_t*,
                                                     const float*, const float*, float, float,
                                                     void*) {
  return pending("backprojection_exhaustive_arellano_forward");
}

int totri_rbf2volume_gaussian_forward(const totri_array_t*, const totri_array_t*, const float*,
                                      const float*, void*) {
  return pending("rbf2volume_gaussian_forward");
}

int totri_rbf2volume_gaussian_grad(const totri_array_t*, const totri_array_t*,
                                   const totri_array_t*, const totri_array_t*, const float*,
                                   const float*, void*) {
  return pending("rbf2volume_gaussian_grad");
}

}  // extern "C"
