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

// The rows one launch works on. With count == nullptr they are [0, n). With
// a device counter they are chunk `step` of `steps` equal chunks of
// min(*count, n) rows, so a whole training sequence can be issued before
// the host knows how many rows there are. Per-row arrays (x, y, out) are
// indexed from the first row of the chunk; acts and dz hold one chunk with
// `ld` rows per layer.
struct NrcRows {
    const uint32_t* count;
    int n;
    int step, steps;
    int ld;
};
inline NrcRows nrc_rows(int n) { return NrcRows{nullptr, n, 0, 1, n}; }
inline NrcRows nrc_rows_counted(const uint32_t* count, int n, int step, int steps) {
    return NrcRows{count, n, step, steps, (n + steps - 1) / steps};
}

void nrc_setup();
// out [rows][3] FP32; acts [4][ld][64] BF16 or null.
void nrc_launch_forward(const NrcDev& N, const __nv_bfloat16* x, const NrcRows& R, float* out, __nv_bfloat16* acts,
                        int num_sms, cudaStream_t st);
// Accumulates the gradient of the mean relative L2 loss of the chunk into
// N.grad; dz: [5][ld][64] BF16 scratch; loss_sum (device float, may be null)
// gets the chunk's mean loss added.
void nrc_launch_backward(const NrcDev& N, const __nv_bfloat16* x, const float* out, const float* y,
                         const __nv_bfloat16* acts, __nv_bfloat16* dz, const NrcRows& R, float* loss_sum, int num_sms,
                         cudaStream_t st);
// ema_beta 0 keeps pinf / wb_inf equal to the current parameters. A counted
// chunk without rows leaves the parameters unchanged, and so does a nonzero
// error word `err` (device, may be null): a kernel of the step failed.
void nrc_launch_adam(const NrcDev& N, float lr, float b1, float b2, float eps, int step, float ema_beta,
                     const NrcRows& R, cudaStream_t st, const uint32_t* err = nullptr);
// Forward with the inference copy (pinf / wb_inf).
void nrc_launch_forward_inf(const NrcDev& N, const __nv_bfloat16* x, const NrcRows& R, float* out, int num_sms,
                            cudaStream_t st);
void nrc_launch_to_bf16(const float* a, __nv_bfloat16* b, size_t n, cudaStream_t st);

// Polls of the tensor-core kernels' bounded mbarrier waits (about 40 ms of
// polling on the GB300 before a wait counts as timed out).
#ifndef NR_TC_FIRST_WAIT_LIMIT
#define NR_TC_FIRST_WAIT_LIMIT (1u << 22)
#endif

// The forward on the tcgen05 tensor cores (nrc_tc.cu) with the BF16 weights
// wb and the FP32 biases of params (either copy of a cache): out [rows][3].
// err (device word) gets bit 8 when a tensor-core wait timed out (the CTA
// then waits again, bounded, for the MMAs in flight, frees its tensor memory
// and returns) and bit 32 as well when that second wait ran out too.
// first_wait: the bound of the first wait of each layer.
void nrc_tc_setup();
void nrc_launch_forward_tc(const __nv_bfloat16* wb, const float* params, const __nv_bfloat16* x, const NrcRows& R,
                           float* out, int num_sms, uint32_t* err, cudaStream_t st, __nv_bfloat16* acts = nullptr,
                           uint32_t first_wait = NR_TC_FIRST_WAIT_LIMIT);
// The same over compact query records (nrc_encode.cuh, [rows][2]), expanded
// in shared memory: 32 bytes read per row instead of 160.
void nrc_launch_forward_tc_records(const __nv_bfloat16* wb, const float* params, const uint4* rec, const NrcRows& R,
                                   float* out, int num_sms, uint32_t* err, cudaStream_t st,
                                   uint32_t first_wait = NR_TC_FIRST_WAIT_LIMIT);
// Compact records -> BF16 rows [rows][80] (for the mma.sync forward).
void nrc_launch_expand(const uint4* rec, const NrcRows& R, __nv_bfloat16* x, int num_sms, cudaStream_t st);
// After error bit 32 the process stops launching the tensor-core kernels
// (their tensor memory may have been freed under running MMAs): every cache
// falls back to the mma.sync kernels of nrc.cu.
void nrc_tc_disable();
bool nrc_tc_enabled();
// Training on the tensor cores: the data gradients (dz [5][ld][64], loss)
// of k_nrc_backward_data by tcgen05.mma; the weight gradients then come
// from nrc_launch_backward_weight.
// wt_img: nrc_wt_image_bytes() of device scratch for the packed transposed
// weights.
void nrc_launch_backward_data_tc(const __nv_bfloat16* wb, const float* out, const float* y, const __nv_bfloat16* acts,
                                 __nv_bfloat16* dz, const NrcRows& R, float* loss_sum, int num_sms, void* wt_img,
                                 uint32_t* err, cudaStream_t st, uint32_t first_wait = NR_TC_FIRST_WAIT_LIMIT);
size_t nrc_wt_image_bytes();
// The weight-gradient half of nrc_launch_backward (k_nrc_backward_weight).
void nrc_launch_backward_weight(const NrcDev& N, const __nv_bfloat16* x, const __nv_bfloat16* dz,
                                const __nv_bfloat16* acts, const NrcRows& R, int num_sms, cudaStream_t st);

}  // namespace nr
