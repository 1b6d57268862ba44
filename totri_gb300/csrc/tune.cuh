// Tile-shape overrides (see tune.cu). Keys:
//   "mesh.confocal.splat.ts"    scan points per confocal splat CTA (1,2,4,8,16)
//   "mesh.exhaustive.splat.lt"  laser points per exhaustive splat CTA (1,4,8,16,32)
//   "volume.exhaustive.lt"      laser points per exhaustive volume CTA (1,8,32)
//   "mesh.visibility.mode"      1 per-lane BVH walk, 2 warp-packet walk
//   "mesh.visibility.queue"     1: queued BVH searches (visibility_queue_kernel)
//   "mesh.visibility.wide"      2: binary BVH search after the surface-walk prefix
//                               (the default is the 4-wide search)
//   "mesh.confocal.grad.split"  scan-point slices per confocal gradient chunk
//   "mesh.exhaustive.grad.split" scan-point slices per exhaustive gradient chunk
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace totri {
namespace tune {
int get(const char* key);  // 0 when unset
int sm_count();            // multiprocessors of the current device
// Slices of the scan-point loop for a gradient grid of `ctas` CTAs: enough for
// 32 CTAs per SM in total, at most one per 64 points (tuned value first),
// and never fewer than make each slice at most `max_slice` points long.
int grad_split(const char* key, int64_t ctas, int S, int max_slice);
// Raises the dynamic shared-memory limit of kernel `func` to at least `bytes`
// on the current device. The limit belongs to the (kernel, device) pair, so
// the value set is remembered per pair (under a lock: launches come from
// several host threads) and set again only when a launch needs more.
cudaError_t ensure_dynamic_smem(const void* func, size_t bytes);
}  // namespace tune
}  // namespace totri
