// Stand-in for the OptiX API surface used by the reference's ray-generation
// programs. optixTrace is answered by a callback supplied by the harness (the
// visibility masks of the oracle), since OptiX's own intersection is closed.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

typedef unsigned long long OptixTraversableHandle;
typedef unsigned int OptixVisibilityMask;
enum { OPTIX_RAY_FLAG_NONE = 0 };

namespace refshim {
inline thread_local uint3 launch_index;
// returns the closest-hit primitive index or 4294967295 (miss)
inline thread_local unsigned int (*trace_fn)(float3 origin, float3 dir, float tmin, float tmax) =
    nullptr;
}  // namespace refshim

inline uint3 optixGetLaunchIndex() { return refshim::launch_index; }
inline void optixTrace(OptixTraversableHandle, float3 origin, float3 dir, float tmin, float tmax,
                       float, OptixVisibilityMask, unsigned int, unsigned int, unsigned int,
                       unsigned int, unsigned int& p0) {
  p0 = refshim::trace_fn(origin, dir, tmin, tmax);
}
inline unsigned int optixGetPrimitiveIndex() { return 0; }
inline void optixSetPayload_0(unsigned int) {}
