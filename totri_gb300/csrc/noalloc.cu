// Allocation-free confocal mesh forward.
//
// Some callers cannot call cudaMalloc: hosts that own every byte of device
// memory through their own fixed pool (a serving process or engine that
// reserves the GPU at start-up), latency-critical loops that must not hit the
// implicit device synchronisation of an allocation, and foreign-language hosts
// that bind only this C ABI and have no device allocator at all. They cannot
// provide the scratch buffer that totri_mesh_confocal_forward needs for its
// BVH and visibility masks. This entry point takes that scratch from one
// file-scope device array that is part of the library image instead.
//
// Limits and sharing rules:
//  * The array holds kNoAllocScratchBytes (24 MiB); calls whose scratch would
//    exceed it are rejected with TOTRI_ERR_WORKSPACE before anything is
//    enqueued. 24 MiB covers, for example, one 20,480-face mesh seen from
//    4,096 scan points.
//  * Every GPU on which the library runs a kernel holds the array until the
//    process exits.
//  * All calls share the array and it keeps the previous call's contents; the
//    pipeline resets everything it reads before reading it. Calls that overlap
//    on the GPU (different streams, or different host threads without
//    ordering) race on the array and must be serialised by the caller.
//  * The device address of the array is looked up once per device, on the
//    first call made while that device is current; make that first call before
//    any stream capture. The address is kept for the life of the process, so
//    the entry point must not be used on a device after cudaDeviceReset.
//  * The device status word (totri_mesh_workspace_status) lives in the scratch
//    and is not reported to the caller.
#include <mutex>
#include <string>

#include "common.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = 24u << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once per
// device; host code must never use the symbol itself as a pointer).
int noalloc_scratch(void** out) {
  int dev = -1;
  TOTRI_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices)
    return totri::fail(TOTRI_ERR_UNSUPPORTED, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    TOTRI_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = p;
  }
  *out = g_noalloc_ptr[dev];
  return TOTRI_OK;
}

}  // namespace

extern "C" {

int totri_mesh_confocal_forward_noalloc(const totri_array_t* verts, const totri_array_t* faces,
                                        const totri_array_t* material,
                                        const totri_array_t* scan_points,
                                        const totri_array_t* scan_origin,
                                        const totri_array_t* transient, float bin_width,
                                        float bin_offset, int model, void* stream) {
  if (!verts || !faces || !scan_points || verts->ndim != 3 || faces->ndim != 3 ||
      scan_points->ndim != 3)
    return totri::fail(TOTRI_ERR_INVALID_ARGUMENT,
                       "verts, faces and scan_points must be 3-dimensional arrays");
  const size_t need = totri_mesh_workspace(verts->shape[0], verts->shape[1], faces->shape[1],
                                           scan_points->shape[1]);
  if (need > kNoAllocScratchBytes)
    return totri::fail(TOTRI_ERR_WORKSPACE,
                       "mesh_confocal_forward_noalloc needs " + std::to_string(need) +
                           " bytes of scratch; its static scratch holds " +
                           std::to_string(kNoAllocScratchBytes) +
                           " bytes (use totri_mesh_confocal_forward with a caller buffer)");
  void* scratch = nullptr;
  if (need > 0) {
    const int st = noalloc_scratch(&scratch);
    if (st != TOTRI_OK) return st;
  }
  return totri_mesh_confocal_forward(verts, faces, material, scan_points, scan_origin, transient,
                                     bin_width, bin_offset, model, scratch,
                                     need > 0 ? kNoAllocScratchBytes : 0, stream);
}

}  // extern "C"
