// Neural radiance cache: a fully fused 80-64-64-64-64-3 ReLU MLP on the
// BF16 tensor cores (mma.sync m16n8k16, FP32 accumulation), its backward
// pass, and Adam on FP32 master weights.
//
// Replaces the per-neuron MLP of the reference's nrc renderer
// (NNNodeMultiLayerPerceptron::eval / train, src/nn/nnnode.cpp:175-201) with
// a batched, fused design: one warp carries 16 rows through every layer in
// registers; the C fragment of layer l becomes the A fragment of layer l+1
// without leaving the register file.
//
// Parameter vector (FP32 master copy, gradients, Adam moments share it):
//   W0 [64][80] b0 [64] | W1 [64][64] b1 | W2 [64][64] b2 | W3 [64][64] b3 |
//   W4 [8][64] (rows 3..7 stay zero) b4 [8]
// The kernels read a BF16 copy of the whole vector and the FP32 biases.
#include <cuda_bf16.h>

#include "nrc.h"

namespace nr {

namespace {

constexpr int IN = NRC_IN, H = NRC_H, OP = NRC_OUT_PAD;
constexpr int S0 = IN + 8;  // padded smem row strides (bank-conflict free)
constexpr int SH = H + 8;

// smem layout of the weights (BF16)
constexpr int SM_W0 = 0;
constexpr int SM_W1 = SM_W0 + H * S0;
constexpr int SM_W2 = SM_W1 + H * SH;
constexpr int SM_W3 = SM_W2 + H * SH;
constexpr int SM_W4 = SM_W3 + H * SH;       // 16 rows: 8 real (3 used) + 8 zero
constexpr int SM_WEND = SM_W4 + 16 * SH;

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack2h(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ float bf(const __nv_bfloat16 x) { return __bfloat162float(x); }

// First row and row count of a launch (see NrcRows).
__device__ __forceinline__ void row_range(const NrcRows& R, int& m0, int& M) {
    if (!R.count) { m0 = 0; M = R.n; return; }
    const int total = min((int)*R.count, R.n);
    const int chunk = (total + R.steps - 1) / R.steps;
    m0 = R.step * chunk;
    M = max(0, min(chunk, total - m0));
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Copies the BF16 weights into shared memory with padded strides; rows
// 8..15 of W4 are zero.
__device__ void load_weights(const __nv_bfloat16* __restrict__ wb, __nv_bfloat16* sm) {
    const __nv_bfloat16 z = __float2bfloat16(0.f);
    for (int i = threadIdx.x; i < H * IN; i += blockDim.x) sm[SM_W0 + (i / IN) * S0 + i % IN] = wb[NRC_OFF_W0 + i];
    for (int l = 0; l < 3; ++l) {
        const int src = l == 0 ? NRC_OFF_W1 : (l == 1 ? NRC_OFF_W2 : NRC_OFF_W3);
        const int dst = l == 0 ? SM_W1 : (l == 1 ? SM_W2 : SM_W3);
        for (int i = threadIdx.x; i < H * H; i += blockDim.x) sm[dst + (i / H) * SH + i % H] = wb[src + i];
    }
    for (int i = threadIdx.x; i < 16 * H; i += blockDim.x) {
        int r = i / H;
        sm[SM_W4 + r * SH + i % H] = r < OP ? wb[NRC_OFF_W4 + i] : z;
    }
}

// One 16-row tile through a hidden layer: acc = bias + A x W^T, K = 16 * KS.
template <int KS>
__device__ __forceinline__ void layer_fwd(float (&acc)[8][4], const uint32_t (&a)[KS][4], const __nv_bfloat16* W,
                                          int stride, const float* __restrict__ bias, int g, int t) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        float b0 = bias[8 * j + 2 * t], b1 = bias[8 * j + 2 * t + 1];
        acc[j][0] = b0; acc[j][1] = b1; acc[j][2] = b0; acc[j][3] = b1;
    }
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const __nv_bfloat16* row = W + (8 * j + g) * stride + 16 * ks + 2 * t;
            uint32_t b0 = *reinterpret_cast<const uint32_t*>(row);
            uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 8);
            mma16816(acc[j], a[ks], b0, b1);
        }
    }
}

// ReLU, optional store of the activations, and conversion of the C
// fragments into the A fragments of the next layer.
__device__ __forceinline__ void relu_to_a(float (&acc)[8][4], uint32_t (&a)[4][4], __nv_bfloat16* act, int row0, int M,
                                          int g, int t) {
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[j][e] = fmaxf(acc[j][e], 0.f);
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        a[s][0] = pack2(acc[2 * s][0], acc[2 * s][1]);
        a[s][1] = pack2(acc[2 * s][2], acc[2 * s][3]);
        a[s][2] = pack2(acc[2 * s + 1][0], acc[2 * s + 1][1]);
        a[s][3] = pack2(acc[2 * s + 1][2], acc[2 * s + 1][3]);
    }
    if (act) {
        int r0 = row0 + g, r1 = row0 + g + 8;
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            if (r0 < M) {
                *reinterpret_cast<uint32_t*>(act + (size_t)r0 * H + 16 * s + 2 * t) = a[s][0];
                *reinterpret_cast<uint32_t*>(act + (size_t)r0 * H + 16 * s + 8 + 2 * t) = a[s][2];
            }
            if (r1 < M) {
                *reinterpret_cast<uint32_t*>(act + (size_t)r1 * H + 16 * s + 2 * t) = a[s][1];
                *reinterpret_cast<uint32_t*>(act + (size_t)r1 * H + 16 * s + 8 + 2 * t) = a[s][3];
            }
        }
    }
}

}  // namespace

// Forward over M rows of BF16 inputs [M][80]. out: [M][3] FP32. acts (may be
// null): [4][M][64] BF16 post-ReLU activations of the hidden layers, kept for
// the backward pass.
__global__ void __launch_bounds__(128) k_nrc_forward(const __nv_bfloat16* __restrict__ wb, const float* __restrict__ params,
                                                     const __nv_bfloat16* __restrict__ x, NrcRows R, float* __restrict__ out,
                                                     __nv_bfloat16* __restrict__ acts) {
    int m0, M;
    row_range(R, m0, M);
    if (M <= 0 || (int)blockIdx.x * 64 >= M) return;
    x += (size_t)m0 * IN;
    out += (size_t)m0 * 3;
    const size_t LS = (size_t)R.ld * H;  // one layer of acts
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    float* sb = reinterpret_cast<float*>(sw + SM_WEND);
    load_weights(wb, sw);
    for (int i = threadIdx.x; i < 4 * H + OP; i += blockDim.x) {
        int l = i / H, k = i % H;
        const int offs[5] = {NRC_OFF_B0, NRC_OFF_B1, NRC_OFF_B2, NRC_OFF_B3, NRC_OFF_B4};
        sb[i] = l < 4 ? params[offs[l] + k] : params[NRC_OFF_B4 + (i - 4 * H)];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int tiles = (M + 15) / 16;
    for (int tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
        const int row0 = tile * 16;
        const int r0 = row0 + g, r1 = row0 + g + 8;
        uint32_t a0[5][4];
#pragma unroll
        for (int ks = 0; ks < 5; ++ks) {
            const int c = 16 * ks + 2 * t;
            a0[ks][0] = r0 < M ? *reinterpret_cast<const uint32_t*>(x + (size_t)r0 * IN + c) : 0u;
            a0[ks][1] = r1 < M ? *reinterpret_cast<const uint32_t*>(x + (size_t)r1 * IN + c) : 0u;
            a0[ks][2] = r0 < M ? *reinterpret_cast<const uint32_t*>(x + (size_t)r0 * IN + c + 8) : 0u;
            a0[ks][3] = r1 < M ? *reinterpret_cast<const uint32_t*>(x + (size_t)r1 * IN + c + 8) : 0u;
        }
        float acc[8][4];
        uint32_t a[4][4];
        layer_fwd<5>(acc, a0, sw + SM_W0, S0, sb, g, t);
        relu_to_a(acc, a, acts ? acts + 0 * LS : nullptr, row0, M, g, t);
        layer_fwd<4>(acc, a, sw + SM_W1, SH, sb + H, g, t);
        relu_to_a(acc, a, acts ? acts + 1 * LS : nullptr, row0, M, g, t);
        layer_fwd<4>(acc, a, sw + SM_W2, SH, sb + 2 * H, g, t);
        relu_to_a(acc, a, acts ? acts + 2 * LS : nullptr, row0, M, g, t);
        layer_fwd<4>(acc, a, sw + SM_W3, SH, sb + 3 * H, g, t);
        relu_to_a(acc, a, acts ? acts + 3 * LS : nullptr, row0, M, g, t);
        // output layer, one n-tile of 8 (3 used)
        float o[4] = {sb[4 * H + 2 * t], sb[4 * H + 2 * t + 1], sb[4 * H + 2 * t], sb[4 * H + 2 * t + 1]};
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            const __nv_bfloat16* row = sw + SM_W4 + g * SH + 16 * ks + 2 * t;
            mma16816(o, a[ks], *reinterpret_cast<const uint32_t*>(row), *reinterpret_cast<const uint32_t*>(row + 8));
        }
        const int c = 2 * t;
        if (r0 < M) {
            if (c < 3) out[(size_t)r0 * 3 + c] = o[0];
            if (c + 1 < 3) out[(size_t)r0 * 3 + c + 1] = o[1];
        }
        if (r1 < M) {
            if (c < 3) out[(size_t)r1 * 3 + c] = o[2];
            if (c + 1 < 3) out[(size_t)r1 * 3 + c + 1] = o[3];
        }
    }
}

// Backward through the layers for M rows: loss gradient of the relative L2
// loss (o - y)^2 / (o^2 + 0.01) (o held constant in the denominator), then
// dZ_l for every layer, stored as BF16 [5][ld][64] (layer 4 uses 8 columns).
// loss_sum (FP32, may be null) receives the mean loss over the rows.
__global__ void __launch_bounds__(128) k_nrc_backward_data(const __nv_bfloat16* __restrict__ wb,
                                                           const float* __restrict__ out, const float* __restrict__ y,
                                                           const __nv_bfloat16* __restrict__ acts, NrcRows R,
                                                           __nv_bfloat16* __restrict__ dz, float* loss_sum) {
    int m0, M;
    row_range(R, m0, M);
    if (M <= 0 || (int)blockIdx.x * 64 >= M) return;
    out += (size_t)m0 * 3;
    y += (size_t)m0 * 3;
    const float inv_n = 1.0f / (3.0f * (float)M);
    const size_t LS = (size_t)R.ld * H;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    load_weights(wb, sw);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int tiles = (M + 15) / 16;
    float loss = 0.f;
    for (int tile = blockIdx.x * 4 + warp; tile < tiles; tile += gridDim.x * 4) {
        const int row0 = tile * 16;
        const int rr[2] = {row0 + g, row0 + g + 8};
        // dOut in C layout: rows g / g+8, columns 2t, 2t+1
        float d4[4];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                int c = 2 * t + e, r = rr[h];
                float v = 0.f;
                if (c < 3 && r < M) {
                    float o = out[(size_t)r * 3 + c], target = y[(size_t)r * 3 + c];
                    float den = o * o + 0.01f;
                    float diff = o - target;
                    loss += diff * diff / den;
                    v = 2.f * diff / den * inv_n;
                }
                d4[2 * h + e] = v;
            }
        __nv_bfloat16* dz4 = dz + 4 * LS;
        for (int h = 0; h < 2; ++h)
            if (rr[h] < M) *reinterpret_cast<uint32_t*>(dz4 + (size_t)rr[h] * H + 2 * t) = pack2(d4[2 * h], d4[2 * h + 1]);
        // dA3 = dOut x W4 (contraction over the 16 padded outputs)
        uint32_t a[4][4];
        a[0][0] = pack2(d4[0], d4[1]);
        a[0][1] = pack2(d4[2], d4[3]);
        a[0][2] = 0u;
        a[0][3] = 0u;
        float acc[8][4];
        const __nv_bfloat16* W4 = sw + SM_W4;
#pragma unroll
        for (int jt = 0; jt < 8; ++jt) {
            acc[jt][0] = acc[jt][1] = acc[jt][2] = acc[jt][3] = 0.f;
            const int k = 8 * jt + g;
            uint32_t b0 = pack2h(W4[(2 * t) * SH + k], W4[(2 * t + 1) * SH + k]);
            uint32_t b1 = pack2h(W4[(2 * t + 8) * SH + k], W4[(2 * t + 9) * SH + k]);
            mma16816(acc[jt], a[0], b0, b1);
        }
        // hidden layers 3, 2, 1, 0: dZ_l = dA_l * (A_l > 0); dA_{l-1} = dZ_l x W_l
#pragma unroll 1
        for (int l = 3; l >= 0; --l) {
            const __nv_bfloat16* act = acts + (size_t)l * LS;
            __nv_bfloat16* dzl = dz + (size_t)l * LS;
#pragma unroll
            for (int jt = 0; jt < 8; ++jt)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    int r = rr[h];
                    uint32_t av = r < M ? *reinterpret_cast<const uint32_t*>(act + (size_t)r * H + 8 * jt + 2 * t) : 0u;
                    __nv_bfloat16 lo = __ushort_as_bfloat16((unsigned short)(av & 0xffff));
                    __nv_bfloat16 hi = __ushort_as_bfloat16((unsigned short)(av >> 16));
                    if (!(bf(lo) > 0.f)) acc[jt][2 * h] = 0.f;
                    if (!(bf(hi) > 0.f)) acc[jt][2 * h + 1] = 0.f;
                    if (r < M) *reinterpret_cast<uint32_t*>(dzl + (size_t)r * H + 8 * jt + 2 * t) = pack2(acc[jt][2 * h], acc[jt][2 * h + 1]);
                }
            if (l == 0) break;
#pragma unroll
            for (int s = 0; s < 4; ++s) {
                a[s][0] = pack2(acc[2 * s][0], acc[2 * s][1]);
                a[s][1] = pack2(acc[2 * s][2], acc[2 * s][3]);
                a[s][2] = pack2(acc[2 * s + 1][0], acc[2 * s + 1][1]);
                a[s][3] = pack2(acc[2 * s + 1][2], acc[2 * s + 1][3]);
            }
            const __nv_bfloat16* W = sw + (l == 3 ? SM_W3 : (l == 2 ? SM_W2 : SM_W1));
#pragma unroll
            for (int jt = 0; jt < 8; ++jt) {
                acc[jt][0] = acc[jt][1] = acc[jt][2] = acc[jt][3] = 0.f;
                const int k = 8 * jt + g;
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const int n = 16 * s + 2 * t;
                    uint32_t b0 = pack2h(W[n * SH + k], W[(n + 1) * SH + k]);
                    uint32_t b1 = pack2h(W[(n + 8) * SH + k], W[(n + 9) * SH + k]);
                    mma16816(acc[jt], a[s], b0, b1);
                }
            }
        }
    }
    if (loss_sum) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
        if (lane == 0) atomicAdd(loss_sum, loss * (1.0f / (3.0f * (float)M)));
    }
}

// Weight gradients of all five layers in one launch (blockIdx.y = layer):
// gW[n][k] += sum_m dZ[m][n] X[m][k] and gb[n] += sum_m dZ[m][n], split
// over CTAs in 64-row chunks. N is 64 (hidden) or 8 (output); K is 80 (input
// layer) or 64. X rows have stride K, dZ rows stride 64.
__global__ void __launch_bounds__(128) k_nrc_backward_weight(const __nv_bfloat16* __restrict__ dz_all,
                                                             const __nv_bfloat16* __restrict__ x,
                                                             const __nv_bfloat16* __restrict__ acts, NrcRows R,
                                                             float* __restrict__ grad) {
    int row0, M;
    row_range(R, row0, M);
    if (M <= 0 || (int)blockIdx.x * 64 >= M) return;
    const int l = blockIdx.y;
    const size_t LS = (size_t)R.ld * H;
    const int N = l == 4 ? OP : H, K = l == 0 ? IN : H;
    const __nv_bfloat16* dz = dz_all + (size_t)l * LS;
    const __nv_bfloat16* xin = l == 0 ? x + (size_t)row0 * IN : acts + (size_t)(l - 1) * LS;
    const int woff = l == 0 ? NRC_OFF_W0 : (l == 1 ? NRC_OFF_W1 : (l == 2 ? NRC_OFF_W2 : (l == 3 ? NRC_OFF_W3 : NRC_OFF_W4)));
    const int boff = l == 0 ? NRC_OFF_B0 : (l == 1 ? NRC_OFF_B1 : (l == 2 ? NRC_OFF_B2 : (l == 3 ? NRC_OFF_B3 : NRC_OFF_B4)));
    float* gW = grad + woff;
    float* gb = grad + boff;
    __shared__ __align__(16) __nv_bfloat16 sdz[64 * (H + 8)];
    __shared__ __align__(16) __nv_bfloat16 sx[64 * (IN + 8)];
    __shared__ float sbias[64];
    const int SD = H + 8, SX = K + 8;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int n0 = 16 * warp;
    const bool active = n0 < N;
    const int KT = K / 8;
    float acc[10][4];
#pragma unroll
    for (int j = 0; j < 10; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    // bias gradient: thread (column tid % 64, rows of half tid / 64) sums its
    // column over the chunks, the halves meet in shared memory at the end
    float bsum = 0.f;
    const int bc = threadIdx.x & 63, bh = threadIdx.x >> 6;
    if (threadIdx.x < 64) sbias[threadIdx.x] = 0.f;
    for (int m0 = blockIdx.x * 64; m0 < M; m0 += gridDim.x * 64) {
        __syncthreads();
        // 16-byte loads: rows of dZ (64 columns, those past N zero) and of X
        for (int i = threadIdx.x; i < 64 * (H / 8); i += blockDim.x) {
            const int r = i / (H / 8), c = 8 * (i % (H / 8));
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (m0 + r < M && c < N) v = *reinterpret_cast<const uint4*>(dz + (size_t)(m0 + r) * H + c);
            *reinterpret_cast<uint4*>(&sdz[r * SD + c]) = v;
        }
        for (int i = threadIdx.x; i < 64 * (K / 8); i += blockDim.x) {
            const int r = i / (K / 8), c = 8 * (i % (K / 8));
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (m0 + r < M) v = *reinterpret_cast<const uint4*>(xin + (size_t)(m0 + r) * K + c);
            *reinterpret_cast<uint4*>(&sx[r * SX + c]) = v;
        }
        __syncthreads();
        if (bc < N)
            for (int r = 32 * bh; r < 32 * bh + 32; ++r) bsum += bf(sdz[r * SD + bc]);
        if (!active) continue;
#pragma unroll
        for (int ms = 0; ms < 4; ++ms) {
            const int m = 16 * ms + 2 * t;
            uint32_t a[4];
            a[0] = pack2h(sdz[m * SD + n0 + g], sdz[(m + 1) * SD + n0 + g]);
            a[1] = pack2h(sdz[m * SD + n0 + g + 8], sdz[(m + 1) * SD + n0 + g + 8]);
            a[2] = pack2h(sdz[(m + 8) * SD + n0 + g], sdz[(m + 9) * SD + n0 + g]);
            a[3] = pack2h(sdz[(m + 8) * SD + n0 + g + 8], sdz[(m + 9) * SD + n0 + g + 8]);
#pragma unroll
            for (int jt = 0; jt < 10; ++jt) {
                if (jt >= KT) break;
                const int k = 8 * jt + g;
                uint32_t b0 = pack2h(sx[m * SX + k], sx[(m + 1) * SX + k]);
                uint32_t b1 = pack2h(sx[(m + 8) * SX + k], sx[(m + 9) * SX + k]);
                mma16816(acc[jt], a, b0, b1);
            }
        }
    }
    if (bc < N) atomicAdd(&sbias[bc], bsum);
    __syncthreads();
    if (threadIdx.x < N) atomicAdd(&gb[threadIdx.x], sbias[threadIdx.x]);
    if (!active) return;
#pragma unroll
    for (int jt = 0; jt < 10; ++jt) {
        if (jt >= KT) break;
        const int c = 8 * jt + 2 * t;
        if (n0 + g < N) {
            atomicAdd(&gW[(n0 + g) * K + c], acc[jt][0]);
            atomicAdd(&gW[(n0 + g) * K + c + 1], acc[jt][1]);
        }
        if (n0 + g + 8 < N) {
            atomicAdd(&gW[(n0 + g + 8) * K + c], acc[jt][2]);
            atomicAdd(&gW[(n0 + g + 8) * K + c + 1], acc[jt][3]);
        }
    }
}

// Adam on the FP32 master parameters (Kingma & Ba), refreshing the BF16 copy
// and clearing the gradient.
// Also advances the moving average used for inference: ema = beta ema +
// (1 - beta) p, read with the start-up correction 1 / (1 - beta^t).
__global__ void k_nrc_adam(float* __restrict__ p, float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                           __nv_bfloat16* __restrict__ wb, float* __restrict__ ema, float* __restrict__ pinf,
                           __nv_bfloat16* __restrict__ wb_inf, int n, float lr, float b1, float b2, float eps, float c1,
                           float c2, float beta, float cema, NrcRows R, const uint32_t* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (err && *err) return;  // a kernel of this step failed: its gradient is not applied
    int r0, rows;
    row_range(R, r0, rows);
    if (rows <= 0) return;  // an empty counted chunk: no step
    float gr = grad[i];
    float mi = b1 * m[i] + (1.f - b1) * gr;
    float vi = b2 * v[i] + (1.f - b2) * gr * gr;
    m[i] = mi;
    v[i] = vi;
    float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    wb[i] = __float2bfloat16(pi);
    grad[i] = 0.f;
    float e = beta * ema[i] + (1.f - beta) * pi;
    ema[i] = e;
    float q = beta > 0.f ? e / cema : pi;
    pinf[i] = q;
    wb_inf[i] = __float2bfloat16(q);
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, __nv_bfloat16* __restrict__ b, size_t n) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = __float2bfloat16(a[i]);
}

// ------------------------------------------------------------------ launchers
size_t nrc_forward_smem() { return (size_t)SM_WEND * 2 + (4 * H + OP) * 4; }
size_t nrc_backward_smem() { return (size_t)SM_WEND * 2; }

void nrc_setup() {
    cudaFuncSetAttribute(k_nrc_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nrc_forward_smem());
    cudaFuncSetAttribute(k_nrc_backward_data, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nrc_backward_smem());
}

static int grid_for(int tiles, int num_sms) {
    int blocks = (tiles + 3) / 4;
    int cap = num_sms * 4;
    return blocks < 1 ? 1 : (blocks > cap ? cap : blocks);
}

// Largest number of rows a launch over R can see.
static int max_rows(const NrcRows& R) { return R.count ? (R.n + R.steps - 1) / R.steps : R.n; }

void nrc_launch_forward(const NrcDev& N, const __nv_bfloat16* x, const NrcRows& R, float* out, __nv_bfloat16* acts,
                        int num_sms, cudaStream_t st) {
    const int M = max_rows(R);
    if (M <= 0) return;
    k_nrc_forward<<<grid_for((M + 15) / 16, num_sms), 128, nrc_forward_smem(), st>>>(N.wb, N.params, x, R, out, acts);
}

void nrc_launch_backward(const NrcDev& N, const __nv_bfloat16* x, const float* out, const float* y,
                         const __nv_bfloat16* acts, __nv_bfloat16* dz, const NrcRows& R, float* loss_sum, int num_sms,
                         cudaStream_t st) {
    const int M = max_rows(R);
    if (M <= 0) return;
    k_nrc_backward_data<<<grid_for((M + 15) / 16, num_sms), 128, nrc_backward_smem(), st>>>(N.wb, out, y, acts, R, dz,
                                                                                          loss_sum);
    int blocks = (M + 63) / 64;
    if (blocks > num_sms * 2) blocks = num_sms * 2;
    k_nrc_backward_weight<<<dim3(blocks, 5), 128, 0, st>>>(dz, x, acts, R, N.grad);
}

void nrc_launch_backward_weight(const NrcDev& N, const __nv_bfloat16* x, const __nv_bfloat16* dz,
                                const __nv_bfloat16* acts, const NrcRows& R, int num_sms, cudaStream_t st) {
    const int M = max_rows(R);
    if (M <= 0) return;
    int blocks = (M + 63) / 64;
    if (blocks > num_sms * 2) blocks = num_sms * 2;
    k_nrc_backward_weight<<<dim3(blocks, 5), 128, 0, st>>>(dz, x, acts, R, N.grad);
}

void nrc_launch_adam(const NrcDev& N, float lr, float b1, float b2, float eps, int step, float ema_beta,
                     const NrcRows& R, cudaStream_t st, const uint32_t* err) {
    float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
    float cema = 1.f - powf(ema_beta, (float)step);
    k_nrc_adam<<<(NRC_NUM_PARAMS + 255) / 256, 256, 0, st>>>(N.params, N.grad, N.m, N.v, N.wb, N.ema, N.pinf, N.wb_inf,
                                                            NRC_NUM_PARAMS, lr, b1, b2, eps, c1, c2, ema_beta, cema, R,
                                                            err);
}

void nrc_launch_forward_inf(const NrcDev& N, const __nv_bfloat16* x, const NrcRows& R, float* out, int num_sms,
                            cudaStream_t st) {
    const int M = max_rows(R);
    if (M <= 0) return;
    k_nrc_forward<<<grid_for((M + 15) / 16, num_sms), 128, nrc_forward_smem(), st>>>(N.wb_inf, N.pinf, x, R, out, nullptr);
}

void nrc_launch_to_bf16(const float* a, __nv_bfloat16* b, size_t n, cudaStream_t st) {
    if (n == 0) return;
    k_f32_to_bf16<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, b, n);
}

}  // namespace nr
