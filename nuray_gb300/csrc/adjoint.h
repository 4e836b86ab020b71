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
// Lbuf: each path's max(0, L) at [(pixel * spp + sample) * 3] (pixel =
// y * imgw + x), as the wavefront renderer collects it.
void adjoint_setup();
void launch_adjoint(const AdjArgs& A, const float* dldi, float* grad, const float* Lbuf, int num_sms, cudaStream_t st);
// image_sum: per-pixel sum over samples of Lbuf.
void launch_image_from_L(const float* Lbuf, int npix, int spp, float* image_sum, cudaStream_t st);

}  // namespace nr
