#pragma once
#include <cstdint>
#include <vector>

#include "../../../include/barnacle_gpu.h"
#include "host_math.hpp"

namespace bnh {
// Reference-compatible BVHNode.Build; see bvh_build.cpp.  Returns false when a leaf would hold
// more items than the reference's int8 count field.
bool bvh_build(const float* bounds, int32_t n, std::vector<bn_bvh_node>* nodes, std::vector<int32_t>* perm);
}  // namespace bnh
