// Neural radiance cache MLP (nrc.cu): layout constants and launchers.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#define NRC_IN 80        // encoded input width (see nrc_encode in nr_material.cuh)
#define NRC_H 64         // hidden width, 4 hidden layers
#define NRC_OUT 3        // RGB
#define NRC_OUT_PAD 8    // output rows padded to one mma n-tile

#define NRC_OFF_W0 0
#define NRC_OFF_B0 (NRC_OFF_W0 + NRC_H * NRC_IN)
#define NRC_OFF_W1 (NRC_OFF_B0 + NRC_H)
#define NRC_OFF_B1 (NRC_OFF_W1 + NRC_H * NRC_H)
#define NRC_OFF_W2 (NRC_OFF_B1 + NRC_H)
#define NRC_OFF_B2 (NRC_OFF_W2 + NRC_H * NRC_H)
#define NRC_OFF_W3 (NRC_OFF_B2 + NRC_H)
#define NRC_OFF_B3 (NRC_OFF_W3 + NRC_H * NRC_H)
#define NRC_OFF_W4 (NRC_OFF_B3 + NRC_H)
#define NRC_OFF_B4 (NRC_OFF_W4 + NRC_OUT_PAD * NRC_H)
#define NRC_NUM_PARAMS (NRC_OFF_B4 + NRC_OUT_PAD)

namespace nr {

// Device buffers of one cache: FP32 master parameters, gradient, Adam
// moments and the BF16 copy the kernels read.
struct NrcDev {
    float* params;
    float* grad;
    float* m;
    float* v;
    __nv_bfloat16* wb;
    // exponential moving average of the parameters for inference in renders:
    // ema (running sum), pinf = ema / (1 - beta^t) and its BF16 copy
    float* ema;
    float* pinf;
    __nv_bfloat16* wb_inf;
};

void nrc_setup();
// out [M][3] FP32; acts [4][M][64] BF16 or null.
void nrc_launch_forward(const NrcDev& N, const __nv_bfloat16* x, int M, float* out, __nv_bfloat16* acts, int num_sms,
                        cudaStream_t st);
// Accumulates the gradient of the mean relative L2 loss into N.grad;
// dz: [5][M][64] BF16 scratch; loss_sum (device float, may be null) gets the summed loss.
void nrc_launch_backward(const NrcDev& N, const __nv_bfloat16* x, const float* out, const float* y,
                         const __nv_bfloat16* acts, __nv_bfloat16* dz, int M, float* loss_sum, int num_sms,
                         cudaStream_t st);
// ema_beta 0 keeps pinf / wb_inf equal to the current parameters.
void nrc_launch_adam(const NrcDev& N, float lr, float b1, float b2, float eps, int step, float ema_beta, cudaStream_t st);
// Forward with the inference copy (pinf / wb_inf).
void nrc_launch_forward_inf(const NrcDev& N, const __nv_bfloat16* x, int M, float* out, int num_sms, cudaStream_t st);
void nrc_launch_to_bf16(const float* a, __nv_bfloat16* b, size_t n, cudaStream_t st);

}  // namespace nr
