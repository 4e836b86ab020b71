// SAH BVH built on the GPU: the reference's BVH::_divide / _build
// (src/hierarchy/bvh.cpp:5-70) computed level by level over all nodes of a
// level at once, for scenes where the host build's setup time matters.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "host_scene.h"

namespace nr {

// Builds the same kind of tree as build_bvh (host_scene.h) from `n`
// triangles (pos: 9 floats each, host memory): primitives ordered by pMax
// along each axis, the reference's surface-area cost at every split
// position, leaves of at most 5 triangles, nodes depth-first with the left
// child first. Where no two triangles share a pMax coordinate the tree is
// the reference's tree; among equal keys the order here is stable (by
// loader index) while the reference's std::sort leaves it unspecified, so
// trees of such scenes can differ (the closest hits differ only on exact
// ties). Past depth_limit it stops as build_bvh does (no nodes, max_depth =
// depth_limit + 1). Returns "" or an error message.
std::string build_bvh_gpu(const float* pos, int n, Bvh& out, cudaStream_t st, double* device_ms = nullptr,
                          int depth_limit = 2048);

}  // namespace nr
