// Allocation-free closest-hit queries (noalloc.cu).
#pragma once
#include <string>

#include "nr_types.h"

// Rays per nr_intersect_noalloc call: the static device scratch holds this
// many rays and results (40 bytes each, 2.6 MB per device in all).
#ifndef NR_NOALLOC_MAX_RAYS
#define NR_NOALLOC_MAX_RAYS 65536
#endif
#define NR_NOALLOC_MAX_DEVICES 64

namespace nr {

// Closest hits for n host rays staged through the static scratch on `st`;
// returns "" or an error message. Blocks until the results are on the host.
std::string noalloc_intersect(const DeviceScene& S, int device, cudaStream_t st, int n, const float* o, const float* d,
                              int32_t* tri, float* t, float* b1, float* b2);

}  // namespace nr
