// Allocation-free closest-hit queries (noalloc.cu).
#pragma once
#include <string>

#include "nr_types.h"

// Rays per nr_intersect_noalloc call: NR_NOALLOC_MAX_RAYS of include/nuray.h
// (the one definition; the static device scratch holds that many rays and
// results, 40 bytes each, 2.6 MB per device in all).
#define NR_NOALLOC_MAX_DEVICES 64

namespace nr {

// Closest hits for n host rays staged through the static scratch on `st`;
// returns "" or an error message. Blocks until the results are on the host.
// Loads the module that holds the static scratch on `device` (the current
// device) and looks up its device address, so that no later
// nr_intersect_noalloc call on that device loads anything. Called when a
// scene is created; returns "" or an error message.
std::string noalloc_prepare(int device);

std::string noalloc_intersect(const DeviceScene& S, int device, cudaStream_t st, int n, const float* o, const float* d,
                              int32_t* tri, float* t, float* b1, float* b2);

}  // namespace nr
