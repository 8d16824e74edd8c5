// Oracle (test infrastructure only): CPU restatement of parry3d's convex contact queries.
// Filled in alongside the GJK/EPA kernels.
#pragma once
#include "bvh.hpp"
#include <atomic>
