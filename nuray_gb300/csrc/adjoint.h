// Path-replay adjoint (adjoint.cu).
#pragma once
#include "nr_types.h"

namespace nr {

struct AdjArgs {
    DeviceScene S;
    Policy pol;
    nr_camera cam;
    float film_h;
    int32_t npix;      // full frame: imgw * imgh
    uint32_t sample0;
    int32_t spp;
};

// grad: num_mats * 7 floats (albedo rgb, roughness, emission rgb), added to.
// image_sum (may be null): per-pixel sum over samples of max(0, L).
void adjoint_setup();
void launch_adjoint(const AdjArgs& A, const float* dldi, float* grad, float* image_sum, int num_sms, cudaStream_t st);

}  // namespace nr
