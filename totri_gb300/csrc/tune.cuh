// Tile-shape and kernel-variant overrides (see tune.cu); 0 (unset) takes the
// default. Keys:
//   "mesh.confocal.splat.ts"    scan points per confocal splat CTA (1,2,4,8,16)
//   "mesh.confocal.splat.mode"  confocal splat variant (at its launcher)
//   "mesh.confocal.exact"       1: every confocal sample takes the exact chain
//   "mesh.confocal.grad.split"  scan-point slices per confocal gradient chunk
//   "mesh.exhaustive.splat.lt"  laser points per exhaustive splat CTA (1,4,8,16,32)
//   "mesh.exhaustive.splat.mode", "mesh.exhaustive.splat.occupancy"
//                               exhaustive splat variant / 1: uncapped registers
//   "mesh.exhaustive.splat.cluster" 1: tiles under 8 lasers flush alone (default:
//                               through a cluster, in whole 32-byte sectors)
//   "mesh.exhaustive.exact"     1: every exhaustive sample takes the exact chain
//   "mesh.exhaustive.grad.mode" 1 per-lane mask tests, 2 compacted triples
//                               (default: per-face point records)
//   "mesh.exhaustive.grad.faces" faces per CTA of the point-record gradient (8)
//   "mesh.exhaustive.grad.occupancy" 4: that kernel capped for 4 CTAs/SM (64
//                               registers) instead of 3
//   "mesh.exhaustive.grad.lchunk", ".sslice" lasers / scan points per CTA of the
//                               point-record gradient (at most 256 each)
//   "mesh.exhaustive.grad.layout" 2: read transient_grad in place even when the
//                               workspace holds the bins-last scratch
//   "mesh.exhaustive.grad.chunk" most scan points per bins-last copy
//   "mesh.exhaustive.grad.split" scan-point slices per exhaustive gradient chunk
//   "mesh.visibility.mode"      1 per-lane BVH walk, 2 warp-packet walk, 7 one hull
//                               per target (at its launcher)
//   "mesh.visibility.queue"     1: queued BVH searches (visibility_queue_kernel)
//   "mesh.visibility.wide"      2: binary BVH search after the surface-walk prefix
//                               (the default is the 4-wide search)
//   "mesh.visibility.occupancy", ".chunks", ".seed", ".seed.steps", ".shaft.cap"
//                               visibility launch shape and prefix (at its launcher)
//   "volume.exact"              1: every volume sample takes the exact chain
//   "volume.adjoint.mode"       0 lanes over 32 columns (default), 1 shared-memory
//                               atomics, 2 lane-owned cells (up to 256 cells)
//   "volume.adjoint.warps"      warps per CTA of the lanes-over-columns adjoint
//   "volume.adjoint.slabs"      z slabs of its columns (default: slabs of <= 64 cells)
//   "volume.exhaustive.lt"      laser points per exhaustive volume CTA (1,8,32)
//   "backprojection.velten.mode", ".occupancy", ".vz", ".groups", ".pair"
//                               Velten kernel variant, 1: uncapped registers (5: capped for
//                               5 CTAs per SM), slab depth, bin windows (1 one per tile, 2 per
//                               point group; 0: by the voxel block's span in bins), 2: bins
//                               one voxel at a time instead of paired
//   "rbf.cull"                  1: RBF kernels without the underflow cull
//   "rbf.forward.vz"            1: one voxel per thread in the RBF forward (default two)
//   "rbf.grad.pair"             2: one Gaussian per warp iteration in the RBF gradient
//                               (default two)
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
