// Path-replay adjoint (adjoint.cu).
#pragma once
#include "integrator.h"
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

// Per-slot state of the wavefront replay: each path's radiance and gradient
// weight, its pending BSDF-factor terms (albedo terms and material in pk, w =
// -1 for none; roughness terms and d fac / d alpha in pa), and per shadow ray
// the light sample's gradient terms (sg0: albedo, roughness; sg1: emission,
// w = material | light material << 16).
// The adjoint's per-slot state in pairs that are read together, one
// 32-byte sector per slot and pair (SlotField): (L, delta), (pk, pa), and
// per shadow-queue entry (sg0, sg1).
struct AdjWave {
    SlotField<float4> L;
    SlotField<float4> delta;
    SlotField<float4> pk;
    SlotField<float4> pa;
    SlotField<float4> sg0;
    SlotField<float4> sg1;
};
// W: the wave (its layout as rendered); the radiance buffer and dldi are
// indexed by scanline pixel, Lbuf as (pixel * spp + sample) * 3.
void launch_adj_init(const PathState& P, const AdjWave& J, const WaveDesc& W, int imgw, int spp, const float* Lbuf,
                     const float* dldi, cudaStream_t st);
// Shading of one bounce (after launch_trace or launch_sort_recorded), adding
// to grad. vis: the bounce's light-sample visibility recorded by the first
// pass, or null to trace the shadow rays here. Returns the kernels launched.
int launch_adj_bounce_shading(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity,
                              const AdjWave& J, const uint8_t* vis, float* grad, int num_sms, int shadow_blocks,
                              cudaStream_t st);

// grad: num_mats * 7 floats (albedo rgb, roughness, emission rgb), added to.
// Lbuf: each path's max(0, L) at [(pixel * spp + sample) * 3] (pixel =
// y * imgw + x), as the wavefront renderer collects it.
void adjoint_setup();
void launch_adjoint(const AdjArgs& A, const float* dldi, float* grad, const float* Lbuf, int num_sms, cudaStream_t st);
// image_sum: per-pixel sum over samples of Lbuf.
void launch_image_from_L(const float* Lbuf, int npix, int spp, float* image_sum, cudaStream_t st);

}  // namespace nr
