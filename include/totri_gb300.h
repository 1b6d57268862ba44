/*
 * totri_gb300 C ABI: GB300-native (sm_103a) transient rendering, backprojection
 * and RBF-to-volume kernels of totrilib behind plain C entry points.
 *
 * Every entry point replaces one function of the reference's pybind11 module
 * `totri_cpp` (src/totri.cpp:13-54) with the same argument order and tensor
 * layouts. Tensors cross the boundary as `totri_array_t` descriptors (device
 * pointer, dtype, shape, strides in elements) instead of at::Tensor; scalars
 * keep their reference types. Nothing here allocates device memory: callers
 * query the scratch size with the matching *_workspace() function and pass a
 * device buffer of at least that many bytes (NULL when the size is 0).
 * Kernels are enqueued on `stream` (a cudaStream_t) and the call returns
 * without synchronising. All functions return TOTRI_OK (0) or an error code;
 * totri_last_error() describes the last failure on the calling thread.
 *
 * Layout rules: small per-point/per-vertex arrays (verts, faces, material,
 * points, origins, rbf parameters) accept arbitrary strides (including 0 for
 * broadcast dimensions, as produced by torch expand()); dense outputs and
 * dense gradients (transients, volumes) must be C-contiguous.
 */
#ifndef TOTRI_GB300_H
#define TOTRI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------- */
/* Status codes, dtypes, descriptors                                        */

enum totri_status {
  TOTRI_OK = 0,
  TOTRI_ERR_INVALID_ARGUMENT = 1, /* bad shape/dtype/stride (ValueError)   */
  TOTRI_ERR_WORKSPACE = 2,        /* workspace missing or too small         */
  TOTRI_ERR_CUDA = 3,             /* a CUDA runtime call failed             */
  TOTRI_ERR_UNSUPPORTED = 4,      /* valid in the reference, not supported  */
  TOTRI_ERR_DEVICE = 5            /* a kernel reported an error status     */
};

enum totri_dtype {
  TOTRI_FLOAT32 = 0,
  TOTRI_FLOAT64 = 1,
  TOTRI_INT32 = 2,
  TOTRI_INT64 = 3
};

#define TOTRI_MAX_DIMS 5

typedef struct totri_array {
  void* data;                       /* device pointer (may be NULL if numel 0) */
  int32_t dtype;                    /* enum totri_dtype                         */
  int32_t ndim;                     /* number of dimensions (<= 5)              */
  int64_t shape[TOTRI_MAX_DIMS];    /* sizes                                    */
  int64_t strides[TOTRI_MAX_DIMS];  /* strides in elements                      */
} totri_array_t;

/* Library version string. */
const char* totri_version(void);
/* Message describing the last failure on the calling thread ("" if none). */
const char* totri_last_error(void);

/* Launch accounting (no reference counterpart). Every kernel launch is
 * counted per kernel name; while enabled, launches are also bracketed by CUDA
 * events on their stream. totri_profile_read synchronises on those events and
 * reports, per kernel name (64-byte NUL-terminated slots in `names`), the
 * launches since the last reset, how many of them were timed, and their total
 * device time in milliseconds. */
int totri_profile_enable(int on);
void totri_profile_reset(void);
int totri_profile_read(int max_entries, char* names, int64_t* launches, int64_t* timed,
                       double* total_ms, int* n_entries);

/* Tile-shape overrides chosen by the autotuner (no reference counterpart).
 * Keys: "mesh.confocal.splat.ts" (scan points per confocal splat CTA: 1, 2,
 * 4, 8, 16), "mesh.exhaustive.splat.lt" (laser points per exhaustive splat
 * CTA: 1, 4, 8, 16, 32). 0 restores the built-in heuristic. */
int totri_tune_set(const char* key, int value);
int totri_tune_get(const char* key);

/* ----------------------------------------------------------------------- */
/* render: meshes                                                           */

/* Scratch bytes for the mesh entry points: one BVH, one visibility mask per
 * batch item. num_points is S (confocal) or S + L (exhaustive). */
size_t totri_mesh_workspace(int64_t batch, int64_t num_verts, int64_t num_faces,
                            int64_t num_points);

/* Optional extra scratch for totri_mesh_exhaustive_grad_verts(_reuse), no
 * reference counterpart: given a workspace of at least
 * totri_mesh_workspace(B, V, F, S + L) + this many bytes, the gradient reads
 * transient_grad through bins-last copies ([s][l][t] order, one batch item and
 * at most 2 GiB of scan points at a time) instead of in place; the results are
 * the same up to FP32 summation order. 0 when one scan point's L x T floats
 * exceed 2 GiB (the gradient then always reads in place). */
size_t totri_mesh_exhaustive_grad_scratch(int64_t num_scan_points, int64_t num_laser_points,
                                          int64_t num_bins);

/* Replaces totri_cpp.render.mesh_confocal_forward
 * (src/render/mesh.h:10-18, src/render/mesh.cpp:9-20).
 * verts [B,V,3] f32, faces [B|1,F,3] i32/i64 (-1 padded: the first face with a
 * negative index ends the list), material [B,V,M] f32 (M<=4, M==0 -> albedo 1),
 * scan_points [B,S,3] f32, scan_origin [B,S,3] or [B,0,3] f32,
 * transient [B,T,S] f32 (written, not accumulated). `model` is ignored, as in
 * the reference. */
int totri_mesh_confocal_forward(const totri_array_t* verts, const totri_array_t* faces,
                                const totri_array_t* material,
                                const totri_array_t* scan_points,
                                const totri_array_t* scan_origin,
                                const totri_array_t* transient, float bin_width,
                                float bin_offset, int model, void* workspace,
                                size_t workspace_bytes, void* stream);

/* totri_mesh_confocal_forward without a caller-provided workspace. It has no
 * counterpart in the reference. It exists for callers that cannot allocate
 * device memory: hosts that own all device memory through a fixed pool,
 * loops that must not pay the device synchronisation of an allocation, and
 * foreign-language hosts that bind only this C ABI. Its scratch is one static
 * 24 MiB device array inside the library (held on every GPU the library runs
 * on until exit); inputs whose scratch would exceed it (see
 * totri_mesh_workspace) fail with TOTRI_ERR_WORKSPACE before any work is
 * enqueued. All calls share that array: calls that overlap on the GPU race
 * and must be serialised by the caller. The first call on each device looks
 * up the array's device address; make it before any stream capture, and do
 * not call this entry point again on a device after cudaDeviceReset in the
 * same process (the address it keeps would be stale). It reports no device
 * status: a face index outside [0, V) ends the face list as in
 * totri_mesh_confocal_forward, and a BVH search reaching its step limit
 * (which a valid mesh does not reach) goes unreported; callers that need
 * totri_mesh_workspace_status use totri_mesh_confocal_forward. */
int totri_mesh_confocal_forward_noalloc(const totri_array_t* verts, const totri_array_t* faces,
                                        const totri_array_t* material,
                                        const totri_array_t* scan_points,
                                        const totri_array_t* scan_origin,
                                        const totri_array_t* transient, float bin_width,
                                        float bin_offset, int model, void* stream);

/* Replaces totri_cpp.render.mesh_confocal_grad_verts
 * (src/render/mesh.h:20-29, src/render/mesh.cpp:22-36).
 * transient_grad [B,T,S]; verts_grad [B,V,3] or [B,V,0]; material_grad
 * [B,V,M] or [B,V,0]; both gradients are overwritten. */
int totri_mesh_confocal_grad_verts(const totri_array_t* verts, const totri_array_t* faces,
                                   const totri_array_t* material,
                                   const totri_array_t* scan_points,
                                   const totri_array_t* scan_origin,
                                   const totri_array_t* transient_grad,
                                   const totri_array_t* verts_grad,
                                   const totri_array_t* material_grad, float bin_width,
                                   float bin_offset, int model, void* workspace,
                                   size_t workspace_bytes, void* stream);

/* Same as totri_mesh_confocal_grad_verts, but reuses the BVH and visibility
 * masks left in `workspace` by a totri_mesh_confocal_forward call on the same
 * inputs (the autograd path keeps that workspace between forward and
 * backward). No reference counterpart: the reference rebuilds both
 * (src/render/mesh_cuda.cu:78). */
int totri_mesh_confocal_grad_verts_reuse(const totri_array_t* verts,
                                         const totri_array_t* faces,
                                         const totri_array_t* material,
                                         const totri_array_t* scan_points,
                                         const totri_array_t* scan_origin,
                                         const totri_array_t* transient_grad,
                                         const totri_array_t* verts_grad,
                                         const totri_array_t* material_grad,
                                         float bin_width, float bin_offset, int model,
                                         void* workspace, size_t workspace_bytes,
                                         void* stream);

/* The confocal forward and gradient with every (scan point, face) pair
 * counted as visible: the unoccluded three-bounce render (arguments, layouts
 * and workspace as for totri_mesh_confocal_forward / _grad_verts; a
 * totri_mesh_confocal_grad_verts_reuse call after the unoccluded forward
 * reuses its all-visible masks). No reference counterpart: the reference
 * always tests visibility (mesh_confocal_forward_optix.cu:50-66). */
int totri_mesh_confocal_forward_unoccluded(const totri_array_t* verts,
                                           const totri_array_t* faces,
                                           const totri_array_t* material,
                                           const totri_array_t* scan_points,
                                           const totri_array_t* scan_origin,
                                           const totri_array_t* transient, float bin_width,
                                           float bin_offset, int model, void* workspace,
                                           size_t workspace_bytes, void* stream);
int totri_mesh_confocal_grad_verts_unoccluded(
    const totri_array_t* verts, const totri_array_t* faces, const totri_array_t* material,
    const totri_array_t* scan_points, const totri_array_t* scan_origin,
    const totri_array_t* transient_grad, const totri_array_t* verts_grad,
    const totri_array_t* material_grad, float bin_width, float bin_offset, int model,
    void* workspace, size_t workspace_bytes, void* stream);

/* Replaces totri_cpp.render.mesh_exhaustive_forward
 * (src/render/mesh.h:31-42, src/render/mesh.cpp:38-52).
 * laser_points [B,L,3], laser_origin [B,L,3] or [B,0,3]; transient [B,T,S,L]. */
int totri_mesh_exhaustive_forward(const totri_array_t* verts, const totri_array_t* faces,
                                  const totri_array_t* material,
                                  const totri_array_t* scan_points,
                                  const totri_array_t* laser_points,
                                  const totri_array_t* scan_origin,
                                  const totri_array_t* laser_origin,
                                  const totri_array_t* transient, float bin_width,
                                  float bin_offset, int model, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* Replaces totri_cpp.render.mesh_exhaustive_grad_verts
 * (src/render/mesh.h:44-56, src/render/mesh.cpp:54-71). */
int totri_mesh_exhaustive_grad_verts(const totri_array_t* verts, const totri_array_t* faces,
                                     const totri_array_t* material,
                                     const totri_array_t* scan_points,
                                     const totri_array_t* laser_points,
                                     const totri_array_t* scan_origin,
                                     const totri_array_t* laser_origin,
                                     const totri_array_t* transient_grad,
                                     const totri_array_t* verts_grad,
                                     const totri_array_t* material_grad, float bin_width,
                                     float bin_offset, int model, void* workspace,
                                     size_t workspace_bytes, void* stream);

/* Exhaustive gradient reusing the BVH and masks of a forward call's
 * workspace (no reference counterpart; see the confocal variant). */
int totri_mesh_exhaustive_grad_verts_reuse(
    const totri_array_t* verts, const totri_array_t* faces, const totri_array_t* material,
    const totri_array_t* scan_points, const totri_array_t* laser_points,
    const totri_array_t* scan_origin, const totri_array_t* laser_origin,
    const totri_array_t* transient_grad, const totri_array_t* verts_grad,
    const totri_array_t* material_grad, float bin_width, float bin_offset, int model,
    void* workspace, size_t workspace_bytes, void* stream);

/* Visibility masks only (testing and diagnostics; no reference counterpart).
 * mask [B,P,ceil(F/32)] int32 words: bit f%32 of word f/32 is set when face f
 * is the closest hit of the ray from point p to the centroid of f.
 * brute_force != 0 tests every face instead of walking the BVH. */
int totri_mesh_visibility(const totri_array_t* verts, const totri_array_t* faces,
                          const totri_array_t* points, const totri_array_t* mask,
                          int brute_force, void* workspace, size_t workspace_bytes,
                          void* stream);

/* Reads the device status word of a mesh workspace (synchronises `stream`).
 * Returns TOTRI_OK when no kernel reported a problem, else TOTRI_ERR_DEVICE
 * and *flags receives the bit set (1: a face index >= V ended a face list,
 * 2: a BVH walk hit its iteration cap). */
int totri_mesh_workspace_status(const void* workspace, size_t workspace_bytes,
                                uint32_t* flags, void* stream);

/* Resident (prepared) meshes. No counterpart in the reference, which builds
 * its acceleration structure inside every call; these keep one BVH per mesh
 * batch on the device and visibility masks per wall grid, so that repeated
 * renders and gradients of the same mesh skip the build and, on a known grid,
 * the visibility walk. The prepared workspace is totri_mesh_workspace(B, V, F,
 * 0) bytes and holds the face records, albedo included: a prepared mesh whose
 * vertices or material change must be prepared again. Mask buffers are
 * totri_mesh_mask_bytes(B, F, P) bytes, 256-byte aligned, opaque. */
size_t totri_mesh_mask_bytes(int64_t batch, int64_t num_faces, int64_t num_points);

/* Builds the BVH and face records of verts/faces/material into workspace. */
int totri_mesh_prepare(const totri_array_t* verts, const totri_array_t* faces,
                       const totri_array_t* material, void* workspace, size_t workspace_bytes,
                       void* stream);

/* Visibility masks of a prepared mesh batch for points [B,P,3]. */
int totri_mesh_prepared_visibility(const totri_array_t* verts, const totri_array_t* faces,
                                   const totri_array_t* material, const totri_array_t* points,
                                   const void* workspace, size_t workspace_bytes, void* masks,
                                   size_t masks_bytes, void* stream);

/* totri_mesh_confocal_forward of a prepared mesh batch with masks computed
 * for the same scan points (arguments as there; no build, no walk). */
int totri_mesh_prepared_confocal_forward(const totri_array_t* verts, const totri_array_t* faces,
                                         const totri_array_t* material,
                                         const totri_array_t* scan_points,
                                         const totri_array_t* scan_origin,
                                         const totri_array_t* transient, float bin_width,
                                         float bin_offset, const void* workspace,
                                         size_t workspace_bytes, const void* masks,
                                         size_t masks_bytes, void* stream);

/* totri_mesh_confocal_grad_verts of a prepared mesh batch with masks. */
int totri_mesh_prepared_confocal_grad_verts(
    const totri_array_t* verts, const totri_array_t* faces, const totri_array_t* material,
    const totri_array_t* scan_points, const totri_array_t* scan_origin,
    const totri_array_t* transient_grad, const totri_array_t* verts_grad,
    const totri_array_t* material_grad, float bin_width, float bin_offset, const void* workspace,
    size_t workspace_bytes, const void* masks, size_t masks_bytes, void* stream);

/* ----------------------------------------------------------------------- */
/* render: volumes                                                          */

/* Scratch bytes for the volume entry points that list occupied voxels
 * (confocal forward, measurement-point gradient, exhaustive forward):
 * num_voxels = X*Y*Z (or D*H*W of one batch item). A 256-byte header, then
 * 16 bytes per voxel (the confocal entry points keep one record per occupied
 * voxel: column centre, value and cell). */
size_t totri_volume_workspace(int64_t num_voxels);

/* Replaces totri_cpp.render.volume_confocal_forward
 * (src/render/volume.h:10-16, src/render/volume.cpp:7-23).
 * volume [X,Y,Z], measurement_points [3,N], transient [N,T] (overwritten);
 * volume_origin/volume_size are 3-vectors. float32 (the reference also
 * dispatches float64; that is refused with TOTRI_ERR_UNSUPPORTED). */
int totri_volume_confocal_forward(const totri_array_t* volume,
                                  const totri_array_t* measurement_points,
                                  const totri_array_t* transient, const float volume_origin[3],
                                  const float volume_size[3], float bin_width,
                                  float bin_offset, void* workspace, size_t workspace_bytes,
                                  void* stream);

/* Replaces totri_cpp.render.volume_confocal_grad_volume
 * (src/render/volume.h:18-24, src/render/volume.cpp:25-41): the transposed
 * operator, transient [N,T] -> volume [X,Y,Z] (overwritten). */
int totri_volume_confocal_grad_volume(const totri_array_t* volume,
                                      const totri_array_t* measurement_points,
                                      const totri_array_t* transient,
                                      const float volume_origin[3],
                                      const float volume_size[3], float bin_width,
                                      float bin_offset, void* stream);

/* The exact adjoint of totri_volume_confocal_forward (no reference
 * counterpart: the reference transposed operator includes samples in the top
 * slice that the forward drops, src/render/volume_cuda.cu:49 vs :127). */
int totri_volume_confocal_adjoint(const totri_array_t* volume,
                                  const totri_array_t* measurement_points,
                                  const totri_array_t* transient,
                                  const float volume_origin[3], const float volume_size[3],
                                  float bin_width, float bin_offset, void* stream);

/* Replaces totri_cpp.render.volume_confocal_grad_measurement_points
 * (src/render/volume.h:26-32, src/render/volume.cpp:43-81).
 * measurement_points_grad [3,N] (overwritten). */
int totri_volume_confocal_grad_measurement_points(
    const totri_array_t* measurement_points_grad, const totri_array_t* volume,
    const totri_array_t* measurement_points, const totri_array_t* transient_grad,
    const float volume_origin[3], const float volume_size[3], float bin_width,
    float bin_offset, void* workspace, size_t workspace_bytes, void* stream);

/* Replaces totri_cpp.render.volume_render_exhaustive_forward
 * (src/render/volume.h:34-43, src/render/volume.cpp:83-96).
 * volume [B,D,H,W]; scan_points [B,3,S]; laser_points [B,3,L];
 * scan_origin [B,3,S|0]; laser_origin [B,3,L|0]; transient [B,T,S,L]
 * (overwritten). */
int totri_volume_exhaustive_forward(const totri_array_t* volume,
                                    const totri_array_t* scan_points,
                                    const totri_array_t* laser_points,
                                    const totri_array_t* scan_origin,
                                    const totri_array_t* laser_origin,
                                    const totri_array_t* transient,
                                    const float volume_start[3], const float volume_end[3],
                                    float bin_width, float bin_offset, void* workspace,
                                    size_t workspace_bytes, void* stream);

/* Replaces totri_cpp.render.volume_render_exhaustive_grad_volume
 * (src/render/volume.h:45-54, src/render/volume.cpp:98-111), whose kernel
 * body is empty in the reference (src/render/volume_cuda.cu:428-430). This is
 * the true adjoint of totri_volume_exhaustive_forward, which is linear in the
 * volume (skipping empty voxels there changes nothing). volume_grad
 * [B,D,H,W] (overwritten). */
int totri_volume_exhaustive_grad_volume(const totri_array_t* transient_grad,
                                        const totri_array_t* scan_points,
                                        const totri_array_t* laser_points,
                                        const totri_array_t* scan_origin,
                                        const totri_array_t* laser_origin,
                                        const totri_array_t* volume_grad,
                                        const float volume_start[3],
                                        const float volume_end[3], float bin_width,
                                        float bin_offset, void* stream);

/* ----------------------------------------------------------------------- */
/* reconstruct: backprojection                                              */

/* Replaces totri_cpp.reconstruct.backprojection_confocal_velten_forward
 * (src/reconstruct/backprojection.h:21-29, backprojection.cpp:22-34).
 * transient [B,T,S]; scan_points [B,S,3]; scan_origin [B,S|0,3];
 * volume [B,D,H,W] (overwritten). */
int totri_backprojection_confocal_velten_forward(
    const totri_array_t* transient, const totri_array_t* scan_points,
    const totri_array_t* scan_origin, const totri_array_t* volume,
    const float volume_start[3], const float volume_end[3], float bin_width,
    float bin_offset, void* stream);

/* The adjoint of the Velten confocal backprojection: volume [B,D,H,W] ->
 * transient [B,T,S] (overwritten). No reference counterpart. */
int totri_backprojection_confocal_velten_adjoint(
    const totri_array_t* volume, const totri_array_t* scan_points,
    const totri_array_t* scan_origin, const totri_array_t* transient,
    const float volume_start[3], const float volume_end[3], float bin_width,
    float bin_offset, void* stream);

/* Replaces totri_cpp.reconstruct.backprojection_exhaustive_velten_forward
 * (src/reconstruct/backprojection.h:31-39, backprojection.cpp:36-49).
 * transient [B,T,S,L]; scan_points [B,S,3]; laser_points [B,L,3]. */
int totri_backprojection_exhaustive_velten_forward(
    const totri_array_t* transient, const totri_array_t* scan_points,
    const totri_array_t* laser_points, const totri_array_t* scan_origin,
    const totri_array_t* laser_origin, const totri_array_t* volume,
    const float volume_start[3], const float volume_end[3], float bin_width,
    float bin_offset, void* stream);

/* Replaces totri_cpp.reconstruct.backprojection_exhaustive_arellano_forward
 * (src/reconstruct/backprojection.h:10-19, backprojection.cpp:8-20).
 * transient [B,T,S,L]; points [B,3,S] / [B,3,L]; volume [B,D,H,W]
 * (accumulated into, as the reference does; callers pass zeros). */
int totri_backprojection_exhaustive_arellano_forward(
    const totri_array_t* transient, const totri_array_t* scan_points,
    const totri_array_t* laser_points, const totri_array_t* scan_origin,
    const totri_array_t* laser_origin, const totri_array_t* volume,
    const float volume_start[3], const float volume_end[3], float bin_width,
    float bin_offset, void* stream);

/* ----------------------------------------------------------------------- */
/* util: RBF to volume                                                      */

/* Replaces totri_cpp.util.rbf2volume_gaussian_forward
 * (src/util/rbf2volume.h:10-14, src/util/rbf2volume.cpp:7-15).
 * rbf [B,N,4+A] (A<=8); volume [B,1+A,D,H,W] (overwritten). */
int totri_rbf2volume_gaussian_forward(const totri_array_t* rbf, const totri_array_t* volume,
                                      const float volume_start[3],
                                      const float volume_end[3], void* stream);

/* Replaces totri_cpp.util.rbf2volume_gaussian_grad
 * (src/util/rbf2volume.h:16-22, src/util/rbf2volume.cpp:17-28).
 * rbf_grad [B,N,4+A] is accumulated into (callers pass zeros, as the
 * reference's Python layer does). */
int totri_rbf2volume_gaussian_grad(const totri_array_t* rbf, const totri_array_t* volume,
                                   const totri_array_t* volume_grad,
                                   const totri_array_t* rbf_grad,
                                   const float volume_start[3], const float volume_end[3],
                                   void* stream);

/* ----------------------------------------------------------------------- */
/* reconstruct: f-k migration                                               */

/* The three kernels of totri.reconstruct.FkMigration (reference
 * totri/reconstruct/fk_migration.py:88-120, plain PyTorch there); the caller
 * runs the forward and inverse 3-D FFTs between them. Complex arrays are
 * float32 with a trailing dimension of 2 (re, im).
 *   _prepare: transient [N,D,H,W] -> out [N,2D,H,W,2]: sqrt(t) x
 *             linspace(0,1,D)[d] for d < D, zero for the padding bins;
 *   _stolt:   Stolt resampling (StoltInterpolation, fk_migration.py:5-86) of
 *             fourier [M,2D,H,W,2] into out (not in place); input_centred 0
 *             reads an un-centred FFT as if fftshift had been applied,
 *             output_centred 0 writes the result ifftshift-ed;
 *   _finish:  volume [N,2D,H,W,2] -> out [N,D,H,W] = |volume| of the first D
 *             bins. */
int totri_fk_prepare(const totri_array_t* transient, const totri_array_t* out, void* stream);
int totri_fk_stolt(const totri_array_t* fourier, const totri_array_t* out, float depth,
                   float height, float width, int input_centred, int output_centred,
                   void* stream);
int totri_fk_finish(const totri_array_t* volume, const totri_array_t* out, void* stream);

/* ----------------------------------------------------------------------- */
/* util: orthographic depth rasteriser                                      */

/* Replaces totri.util.UnitDepthMapRender (totri/util/depthmap.py:6-36, a
 * pytorch3d orthographic rasteriser): verts [V,3] float32, faces [F,3] int64
 * -> depth [H,W] float32 (nearest face's z at each pixel centre within
 * [znear, zfar], -1 where empty) and mask [H,W] int32 (1 where covered).
 * Column j looks along x = max_x - (j + 1/2) (max_x - min_x) / W, row i along
 * y = max_y - (i + 1/2) (max_y - min_y) / H, both faces counted. Scratch:
 * totri_depth_raster_workspace(H, W) bytes. */
size_t totri_depth_raster_workspace(int64_t height, int64_t width);
int totri_depth_raster(const totri_array_t* verts, const totri_array_t* faces,
                       const totri_array_t* depth, const totri_array_t* mask, float min_x,
                       float max_x, float min_y, float max_y, float znear, float zfar,
                       void* workspace, size_t workspace_bytes, void* stream);

/* ----------------------------------------------------------------------- */
/* util: shaded perspective preview renderer                                */

/* Camera, light, material and blend settings of totri_shaded_raster. View
 * coordinates are row vectors: view = world @ rotation + translation
 * (rotation row-major [3][3]); normalised device coordinates are
 * ndc.x = focal[0] * view.x / view.z, ndc.y = focal[1] * view.y / view.z. */
typedef struct totri_shading {
  float rotation[9];
  float translation[3];
  float focal[2];
  float znear, zfar;          /* depth range of the blend weights            */
  float camera_center[3];     /* world position of the eye (specular term)   */
  float light_location[3];    /* one point light                             */
  float light_ambient[3], light_diffuse[3], light_specular[3];
  float material_ambient[3], material_diffuse[3], material_specular[3];
  float shininess;
  float background[3];
  float sigma, gamma;         /* blend sharpness (coverage, depth)           */
} totri_shading_t;

/* Replaces totri.util.render.UnitCubeMeshRender.apply (totri/util/render.py:
 * 17-81: pytorch3d FoVPerspectiveCameras, one face per pixel without blur,
 * SoftPhongShader with a point light and vertex colours): verts [V,3] float32,
 * faces [F,3] int64 (a face with an index outside [0, V) is skipped), colors
 * [V,3] float32 (any strides, e.g. a broadcast row) -> image [3,H,W] float32,
 * and when pix_to_face is not NULL the winning face per pixel [H,W] int32
 * (-1 where empty). Pixel (row r, column c) samples ndc
 * x = -1 + (2 (W-1-c) + 1) / W, y = -1 + (2 (H-1-r) + 1) / H (the longer side
 * scaled by its ratio to the shorter). Scratch:
 * totri_shaded_raster_workspace(V, H, W) bytes. */
size_t totri_shaded_raster_workspace(int64_t num_verts, int64_t height, int64_t width);
int totri_shaded_raster(const totri_array_t* verts, const totri_array_t* faces,
                        const totri_array_t* colors, const totri_shading_t* shading,
                        const totri_array_t* image, const totri_array_t* pix_to_face,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ----------------------------------------------------------------------- */
/* util: differentiable marching cubes                                      */

/* Replaces tomcubes.MarchingCubesFunction (an un-vendored submodule of the
 * reference, .gitmodules:4-6; called at totri/fitting/rbf.py:88-98 as
 * apply(volume [B,1+A,D,H,W], iso, volume_def.start, volume_def.end) and
 * rendered as consecutive vertex triples, rbf.py:719). Three calls share one
 * workspace of totri_marching_cubes_workspace(B, D, H, W) bytes:
 *   _count: classifies the cells of channel 0 against iso (a grid point is
 *           inside when its value is above iso) and writes the triangles of
 *           every batch item to `triangles` [B] int64 (device memory);
 *   _emit:  writes the triangle soup verts [B,N,3+A] (x, y, z, then the
 *           attribute channels 1.. interpolated along the same edges) and
 *           edges [B,N] int64 (12 x cell + edge, the record the gradient
 *           needs) for N >= 3 x max(triangles); rows past an item's vertices
 *           are left as the caller filled them (zeros / -1);
 *   _grad:  accumulates d loss / d volume into volume_grad [B,1+A,D,H,W]
 *           from verts_grad [B,N,3+A] (rows whose edge record is < 0 are
 *           skipped), with the case table held constant.
 * Grid point (x, y, z) sits at start + ((end - start) i) / (n - 1) per axis,
 * as in totri_rbf2volume_gaussian_forward. */
size_t totri_marching_cubes_workspace(int64_t batch, int64_t depth, int64_t height,
                                      int64_t width);
int totri_marching_cubes_count(const totri_array_t* volume, float iso,
                               const totri_array_t* triangles, void* workspace,
                               size_t workspace_bytes, void* stream);
int totri_marching_cubes_emit(const totri_array_t* volume, float iso,
                              const float volume_start[3], const float volume_end[3],
                              const totri_array_t* verts, const totri_array_t* edges,
                              void* workspace, size_t workspace_bytes, void* stream);
int totri_marching_cubes_grad(const totri_array_t* volume, float iso,
                              const float volume_start[3], const float volume_end[3],
                              const totri_array_t* edges, const totri_array_t* verts_grad,
                              const totri_array_t* volume_grad, void* stream);
/* The case table (host memory, no GPU needed): ntri[256] triangles per case
 * (bit i of the case = corner (i & 1, i >> 1 & 1, i >> 2) inside) and
 * edges[256 * 15] edge ids (4 x axis + the other two corner bits), -1 padded. */
int totri_marching_cubes_table(uint8_t* ntri, int8_t* edges);

/* Fills out[0..n) with standard normal values drawn from `seed`; element i
 * depends only on (seed, i) (counter-based), so repeated and graph-captured
 * fills agree. No counterpart in the reference: the batched benchmark's
 * seeded N(0,1) d loss / d transient. */
int totri_fill_normal(float* out, int64_t n, uint64_t seed, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TOTRI_GB300_H */
