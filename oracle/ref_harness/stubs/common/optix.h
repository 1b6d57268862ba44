// Stand-in for the reference's OptiX context header (nothing is needed from it).
#pragma once
#include "optix.h"
#include "common/buffer.h"
