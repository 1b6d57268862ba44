// Stand-in for the reference's OptiX pipeline base class (declarations only).
#pragma once
#include "common/optix.h"
namespace totri {
namespace render {
struct EmptyRaygenRecord {};
struct EmptyMissRecord {};
struct EmptyHitgroupRecord {};
class MeshProgramBase {};
}  // namespace render
}  // namespace totri
