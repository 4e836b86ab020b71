// The cache's MLP on the 5th-generation tensor cores: the 80-64-64-64-64-3
// network of nrc.cu as chains of tcgen05.mma (kind::f16, BF16 operands,
// FP32 accumulators in tensor memory), 128 rows per CTA tile. The forward
// kernel serves inference and, storing the hidden activations, training;
// the data-gradient kernel runs the same chain backwards against the
// transposed weights (its own comment below). Weight gradients and Adam
// stay in nrc.cu.
//
// Per tile: the 128 input rows go to shared memory in the canonical K-major
// layout without swizzle (8-row x 16-byte core matrices; the leading byte
// offset steps between core matrices along K, the stride byte offset between
// 8-row groups); one thread issues the layer's MMAs (K = 16 each) and
// commits them to an mbarrier; every thread then reads its row of the
// 128 x N accumulator from tensor memory (tcgen05.ld 32x32b, warp w owns
// lanes 32w..32w+31), adds the bias, applies ReLU, rounds to BF16 and writes
// the row back to shared memory as the next layer's A operand. The weights
// stay in shared memory for all tiles of the CTA. Every wait on the mbarrier
// is bounded; a timeout sets an error bit, the CTA stops, frees its tensor
// memory and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>

#include "nrc.h"
#include "nrc_encode.cuh"
#include "nr_types.h"

namespace nr {

namespace {

constexpr int IN = NRC_IN, H = NRC_H;
constexpr int TM = 128;           // rows per tile (MMA M)
constexpr int KC_IN = IN / 8;     // 16-byte chunks per input row (10)
constexpr int KC_H = H / 8;       // 8
// shared memory regions (bytes), each a multiple of 128
constexpr int SM_W0 = 0;                              // 64 x 80
constexpr int SM_W1 = SM_W0 + (H / 8) * KC_IN * 128;  // 64 x 64 each
constexpr int SM_W2 = SM_W1 + (H / 8) * KC_H * 128;
constexpr int SM_W3 = SM_W2 + (H / 8) * KC_H * 128;
constexpr int SM_W4 = SM_W3 + (H / 8) * KC_H * 128;   // 16 x 64 (rows 3..15 zero)
constexpr int SM_A = SM_W4 + 2 * KC_H * 128;          // 128 x 80 (hidden layers use 128 x 64)
constexpr int SM_BIAS = SM_A + (TM / 8) * KC_IN * 128;
constexpr int SM_BAR = SM_BIAS + (4 * H + 16) * 4;
constexpr int SM_TOTAL = SM_BAR + 16;
constexpr uint32_t TMEM_COLS = 64;
// Polls of one bounded mbarrier wait. The first wait of a layer takes the
// caller's bound (NR_TC_FIRST_WAIT_LIMIT by default; a cache created with
// tc_first_wait=0 makes it run out at once, which tests the timeout path);
// the wait after a timeout, for the MMAs still in flight, always takes this one.
constexpr uint32_t WAIT_LIMIT = NR_TC_FIRST_WAIT_LIMIT;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory descriptor: start, leading and stride byte offsets
// (all >> 4), the fixed 0b001 at bits 46-48, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// kind::f16 instruction descriptor: FP32 D, BF16 A and B, both K-major, N, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}
// Bounded wait for the mbarrier phase; false on timeout.
__device__ __forceinline__ bool wait_phase(uint32_t bar, uint32_t phase, uint32_t limit) {
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's lane; the wait for the load
// sits in the same statement, so no register is read before it lands.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// W [n][k] (row-major, k contiguous) into the canonical K-major layout.
__device__ void load_w(unsigned char* sm, int off, const __nv_bfloat16* __restrict__ w, int rows, int rows_real, int k) {
    const int kc = k / 8;
    for (int i = threadIdx.x; i < rows * kc; i += blockDim.x) {
        const int n = i / kc, c = i % kc;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (n < rows_real) v = *reinterpret_cast<const uint4*>(w + (size_t)n * k + 8 * c);
        *reinterpret_cast<uint4*>(sm + off + (n / 8) * (kc * 128) + c * 128 + (n % 8) * 16) = v;
    }
}

}  // namespace

// Forward of the rows R over BF16 inputs [rows][80] with the BF16 weights
// `wb` and the biases of `params`; out [rows][3] FP32; acts (may be null):
// the hidden layers' post-ReLU BF16 activations [4][R.ld][64] for the
// backward pass. err bit 8 on a tensor-core wait that timed out.
//
// NWG warpgroups per CTA, each an independent tile pipeline over the one
// copy of the weights in shared memory: its own 128-row A buffer, mbarrier
// and 64 tensor-memory columns, synchronised by its own named barrier. One
// tile's five layers are a dependent chain (MMA, commit, wait, tensor-memory
// read, epilogue), so tiles in flight are what hides that latency: with
// NWG = 3 two CTAs fit an SM (98 KB of shared memory each, 256 tensor-memory
// columns each), six tiles in flight per SM against three with one
// warpgroup per CTA.
namespace {
constexpr int FW_A_BYTES = (TM / 8) * KC_IN * 128;          // 128 x 80 BF16, canonical layout
constexpr int FW_BIAS = SM_A;                               // biases right after the weights
constexpr int FW_ABUF = ((FW_BIAS + (4 * H + 16) * 4) + 127) / 128 * 128;
__host__ __device__ constexpr int fw_smem(int nwg) { return FW_ABUF + nwg * FW_A_BYTES + 16 * nwg; }
__host__ __device__ constexpr uint32_t fw_tmem_cols(int nwg) { return nwg == 1 ? 64u : (nwg == 2 ? 128u : 256u); }

// Named barrier `id` over the 128 threads of one warpgroup.
__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;\n" ::"r"(id) : "memory"); }
// The same with an OR of v over the warpgroup.
__device__ __forceinline__ bool wg_sync_or(int id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n barrier.cta.red.or.pred p, %2, 128, q;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id)
        : "memory");
    return r != 0;
}
}  // namespace

// rec (or null): compact records [rows][2] (nrc_encode.cuh) expanded into
// the A tile in place of rows of x.
template <int NWG>
__global__ void __launch_bounds__(128 * NWG) k_nrc_forward_tc(const __nv_bfloat16* __restrict__ wb,
                                                              const float* __restrict__ params,
                                                              const __nv_bfloat16* __restrict__ x,
                                                              const uint4* __restrict__ rec, NrcRows R,
                                                              float* __restrict__ out, __nv_bfloat16* __restrict__ acts,
                                                              uint32_t* err, uint32_t first_wait) {
    int m0, M;
    if (!R.count) {
        m0 = 0;
        M = R.n;
    } else {
        const int total = min((int)*R.count, R.n);
        const int chunk = (total + R.steps - 1) / R.steps;
        m0 = R.step * chunk;
        M = max(0, min(chunk, total - m0));
    }
    const int tiles = (M + TM - 1) / TM;
    if ((int)blockIdx.x * NWG >= tiles) return;  // no warpgroup of this CTA has a tile: no tensor memory taken
    if (rec) rec += 2 * (size_t)m0;
    else x += (size_t)m0 * IN;
    out += (size_t)m0 * 3;
    const size_t LS = (size_t)R.ld * H;  // one layer of acts

    extern __shared__ __align__(1024) unsigned char sm[];
    float* sbias = reinterpret_cast<float*>(sm + FW_BIAS);
    __shared__ uint32_t s_taddr;
    __shared__ int s_abort[NWG];
    const int tid = threadIdx.x, warp = tid >> 5, wg = tid >> 7, wtid = tid & 127;
    const int bar_id = 1 + wg;  // named barrier of this warpgroup (0 is __syncthreads)

    load_w(sm, SM_W0, wb + NRC_OFF_W0, H, H, IN);
    load_w(sm, SM_W1, wb + NRC_OFF_W1, H, H, H);
    load_w(sm, SM_W2, wb + NRC_OFF_W2, H, H, H);
    load_w(sm, SM_W3, wb + NRC_OFF_W3, H, H, H);
    load_w(sm, SM_W4, wb + NRC_OFF_W4, 16, NRC_OUT_PAD, H);
    for (int i = tid; i < 4 * H + 16; i += blockDim.x) {
        const int offs[4] = {NRC_OFF_B0, NRC_OFF_B1, NRC_OFF_B2, NRC_OFF_B3};
        sbias[i] = i < 4 * H ? params[offs[i / H] + i % H]
                             : (i - 4 * H < NRC_OUT_PAD ? params[NRC_OFF_B4 + i - 4 * H] : 0.f);
    }
    unsigned char* abuf = sm + FW_ABUF + wg * FW_A_BYTES;
    const uint32_t bar = smem_u32(sm + FW_ABUF + NWG * FW_A_BYTES + 16 * wg);
    if (wtid == 0) {
        s_abort[wg] = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_taddr)),
                     "r"(fw_tmem_cols(NWG))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    // this warpgroup's 64 columns; a warp reads the tensor-memory lanes of its quarter
    const uint32_t tmem = s_taddr + 64u * (uint32_t)wg;
    const uint32_t lane_base = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    uint32_t phase = 0;

    const uint32_t a_addr = smem_u32(abuf);
    const uint32_t w_addr[5] = {smem_u32(sm + SM_W0), smem_u32(sm + SM_W1), smem_u32(sm + SM_W2), smem_u32(sm + SM_W3),
                                smem_u32(sm + SM_W4)};

    for (int tile = blockIdx.x * NWG + wg; tile < tiles; tile += gridDim.x * NWG) {
        {  // input rows -> A (K = 80)
            const int r = wtid, row = tile * TM + r;
            unsigned char* dst = abuf + (r / 8) * (KC_IN * 128) + (r % 8) * 16;
            if (rec) {
                uint32_t w[40];
                if (row < M) {
                    const uint4 a = rec[2 * (size_t)row], b = rec[2 * (size_t)row + 1];
                    const uint32_t q[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
                    nrc_expand(q, w);
                } else {
#pragma unroll
                    for (int i = 0; i < 40; ++i) w[i] = 0u;
                }
#pragma unroll
                for (int c = 0; c < KC_IN; ++c)
                    *reinterpret_cast<uint4*>(dst + c * 128) = make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
            } else {
#pragma unroll
                for (int c = 0; c < KC_IN; ++c) {
                    uint4 v = make_uint4(0u, 0u, 0u, 0u);
                    if (row < M) v = *reinterpret_cast<const uint4*>(x + (size_t)row * IN + 8 * c);
                    *reinterpret_cast<uint4*>(dst + c * 128) = v;
                }
            }
        }
        for (int layer = 0; layer < 5; ++layer) {
            const int k = layer == 0 ? IN : H;
            const uint32_t sbo = (uint32_t)(k / 8) * 128u;
            const uint32_t n = layer == 4 ? 16u : (uint32_t)H;
            fence_async_smem();
            fence_before();
            wg_sync(bar_id);
            if (wtid == 0) {
                fence_after();
#pragma unroll 1
                for (int ks = 0; ks < k / 16; ++ks) {
                    const uint64_t ad = sdesc(a_addr + (uint32_t)ks * 256u, 128u, sbo);
                    const uint64_t bd = sdesc(w_addr[layer] + (uint32_t)ks * 256u, 128u, sbo);
                    mma(tmem, ad, bd, idesc_bf16(n), ks > 0 ? 1u : 0u);
                }
                commit(bar);
            }
            const bool ok = wait_phase(bar, phase, first_wait);
            if (wg_sync_or(bar_id, !ok)) {
                if (wtid == 0) {
                    s_abort[wg] = 1;
                    // the MMAs may still write the tensor memory freed below:
                    // one more bounded wait for their commit; if that runs
                    // out too, bit 32 tells the host to stop using these kernels
                    const bool done = wait_phase(bar, phase, WAIT_LIMIT);
                    atomicOr(err, done ? (uint32_t)NR_ERRBIT_TC_WAIT : (uint32_t)(NR_ERRBIT_TC_WAIT | NR_ERRBIT_TC_LOST));
                }
                break;
            }
            phase ^= 1u;
            fence_after();
            const int r = wtid, row = tile * TM + r;
            if (layer < 4) {
                unsigned char* dst = abuf + (r / 8) * (KC_H * 128) + (r % 8) * 16;
                const float* b = sbias + layer * H;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float v[16];
                    tmem_ld16(lane_base + (uint32_t)(16 * q), v);
#pragma unroll
                    for (int h2 = 0; h2 < 2; ++h2) {
                        uint4 pk;
                        const int c0 = 16 * q + 8 * h2;
                        pk.x = pack_bf16(fmaxf(v[8 * h2 + 0] + b[c0 + 0], 0.f), fmaxf(v[8 * h2 + 1] + b[c0 + 1], 0.f));
                        pk.y = pack_bf16(fmaxf(v[8 * h2 + 2] + b[c0 + 2], 0.f), fmaxf(v[8 * h2 + 3] + b[c0 + 3], 0.f));
                        pk.z = pack_bf16(fmaxf(v[8 * h2 + 4] + b[c0 + 4], 0.f), fmaxf(v[8 * h2 + 5] + b[c0 + 5], 0.f));
                        pk.w = pack_bf16(fmaxf(v[8 * h2 + 6] + b[c0 + 6], 0.f), fmaxf(v[8 * h2 + 7] + b[c0 + 7], 0.f));
                        *reinterpret_cast<uint4*>(dst + (c0 / 8) * 128) = pk;
                        if (acts && row < M)
                            *reinterpret_cast<uint4*>(acts + (size_t)layer * LS + (size_t)row * H + c0) = pk;
                    }
                }
            } else {
                float v[16];
                tmem_ld16(lane_base, v);
                if (row < M) {
                    out[(size_t)row * 3 + 0] = v[0] + sbias[4 * H + 0];
                    out[(size_t)row * 3 + 1] = v[1] + sbias[4 * H + 1];
                    out[(size_t)row * 3 + 2] = v[2] + sbias[4 * H + 2];
                }
            }
        }
        wg_sync(bar_id);
        if (s_abort[wg]) break;
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(s_taddr), "r"(fw_tmem_cols(NWG))
                     : "memory");
    }
}

// Data gradients on the tensor cores for the rows R: the relative L2
// loss's gradient dOut (o - y) 2 / (o^2 + 0.01) / (3 rows), then per tile
// of 128 rows the chain dA3 = dOut W4, dZ3 = dA3 (A3 > 0), dA2 = dZ3 W3, ...,
// dZ0, each product one group of tcgen05.mma with the transposed weight
// (B[n][k] = W[k][n]) in shared memory. dz [5][R.ld][64] BF16 as
// k_nrc_backward_data writes it (layer 4: 8 columns), for
// k_nrc_backward_weight; loss_sum (may be null) += the mean loss.
namespace {
constexpr int BK_W4T = 0;                                  // 64 x 16
constexpr int BK_W3T = BK_W4T + (H / 8) * 2 * 128;         // 64 x 64 each
constexpr int BK_W2T = BK_W3T + (H / 8) * KC_H * 128;
constexpr int BK_W1T = BK_W2T + (H / 8) * KC_H * 128;
constexpr int BK_A = BK_W1T + (H / 8) * KC_H * 128;        // 128 x 64 (the first product uses 128 x 16)
constexpr int BK_BAR = BK_A + (TM / 8) * KC_H * 128;
constexpr int BK_TOTAL = BK_BAR + 16;

// W [k][n] (row-major, `n_in` columns, `k_real` rows, the rest zero) into
// the canonical K-major layout of B[n][k] with K = kk, at dst + off.
__device__ void load_wt(unsigned char* sm, int off, const __nv_bfloat16* __restrict__ w, int n_in, int k_real, int kk) {
    const int kc = kk / 8;
    // consecutive threads read consecutive elements of a row of W
    for (int i = threadIdx.x; i < n_in * kk; i += blockDim.x) {
        const int k = i / n_in, n = i % n_in;
        const __nv_bfloat16 v = k < k_real ? w[(size_t)k * n_in + n] : __float2bfloat16(0.f);
        *reinterpret_cast<__nv_bfloat16*>(sm + off + (n / 8) * (kc * 128) + (k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2) = v;
    }
}
}  // namespace

// The four transposed weight images of k_nrc_backward_data_tc (one per
// block), packed once per pass into `img` (BK_A bytes) from which every CTA
// copies them.
__global__ void k_nrc_pack_wt(const __nv_bfloat16* __restrict__ wb, unsigned char* __restrict__ img) {
    switch (blockIdx.x) {
        case 0: load_wt(img, BK_W4T, wb + NRC_OFF_W4, H, NRC_OUT_PAD, 16); break;
        case 1: load_wt(img, BK_W3T, wb + NRC_OFF_W3, H, H, H); break;
        case 2: load_wt(img, BK_W2T, wb + NRC_OFF_W2, H, H, H); break;
        default: load_wt(img, BK_W1T, wb + NRC_OFF_W1, H, H, H); break;
    }
}

__global__ void __launch_bounds__(128) k_nrc_backward_data_tc(const __nv_bfloat16* __restrict__ wb,
                                                              const float* __restrict__ out,
                                                              const float* __restrict__ y,
                                                              const __nv_bfloat16* __restrict__ acts, NrcRows R,
                                                              __nv_bfloat16* __restrict__ dz, float* loss_sum,
                                                              const unsigned char* __restrict__ wt_img,
                                                              uint32_t* err, uint32_t first_wait) {
    int m0, M;
    if (!R.count) {
        m0 = 0;
        M = R.n;
    } else {
        const int total = min((int)*R.count, R.n);
        const int chunk = (total + R.steps - 1) / R.steps;
        m0 = R.step * chunk;
        M = max(0, min(chunk, total - m0));
    }
    const int tiles = (M + TM - 1) / TM;
    if ((int)blockIdx.x >= tiles) return;
    out += (size_t)m0 * 3;
    y += (size_t)m0 * 3;
    const size_t LS = (size_t)R.ld * H;
    const float inv_n = 1.0f / (3.0f * (float)M);

    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ uint32_t s_taddr;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < BK_A / 16; i += blockDim.x)
        reinterpret_cast<uint4*>(sm)[i] = reinterpret_cast<const uint4*>(wt_img)[i];
    const uint32_t bar = smem_u32(sm + BK_BAR);
    if (tid == 0) {
        s_abort = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_taddr)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s_taddr;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0;
    const uint32_t a_addr = smem_u32(sm + BK_A);
    const uint32_t wt_addr[4] = {smem_u32(sm + BK_W4T), smem_u32(sm + BK_W3T), smem_u32(sm + BK_W2T),
                                 smem_u32(sm + BK_W1T)};
    float loss = 0.f;

    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int r = tid, row = tile * TM + r;
        {  // dOut of this row -> A (K = 16) and dz[4]
            float d[3] = {0.f, 0.f, 0.f};
            if (row < M) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float o = out[(size_t)row * 3 + c], target = y[(size_t)row * 3 + c];
                    const float den = o * o + 0.01f, diff = o - target;
                    loss += diff * diff / den;
                    d[c] = 2.f * diff / den * inv_n;
                }
            }
            const uint4 pk = make_uint4(pack_bf16(d[0], d[1]), pack_bf16(d[2], 0.f), 0u, 0u);
            unsigned char* dst = sm + BK_A + (r / 8) * (2 * 128) + (r % 8) * 16;
            *reinterpret_cast<uint4*>(dst) = pk;
            *reinterpret_cast<uint4*>(dst + 128) = make_uint4(0u, 0u, 0u, 0u);
            if (row < M) *reinterpret_cast<uint4*>(dz + 4 * LS + (size_t)row * H) = pk;
        }
        // products with W4, W3, W2, W1; the epilogue of each gives dZ3, dZ2, dZ1, dZ0
        for (int g = 0; g < 4; ++g) {
            const int k = g == 0 ? 16 : H;
            const uint32_t sbo = (uint32_t)(k / 8) * 128u;
            fence_async_smem();
            fence_before();
            __syncthreads();
            if (tid == 0) {
                fence_after();
#pragma unroll 1
                for (int ks = 0; ks < k / 16; ++ks) {
                    const uint64_t ad = sdesc(a_addr + (uint32_t)ks * 256u, 128u, sbo);
                    const uint64_t bd = sdesc(wt_addr[g] + (uint32_t)ks * 256u, 128u, sbo);
                    mma(tmem, ad, bd, idesc_bf16((uint32_t)H), ks > 0 ? 1u : 0u);
                }
                commit(bar);
            }
            const bool ok = wait_phase(bar, phase, first_wait);
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    s_abort = 1;
                    // the MMAs may still write the tensor memory freed below:
                    // one more bounded wait for their commit; if that runs
                    // out too, bit 32 tells the host to stop using these kernels
                    const bool done = wait_phase(bar, phase, WAIT_LIMIT);
                    atomicOr(err, done ? (uint32_t)NR_ERRBIT_TC_WAIT : (uint32_t)(NR_ERRBIT_TC_WAIT | NR_ERRBIT_TC_LOST));
                }
                break;
            }
            phase ^= 1u;
            fence_after();
            const int l = 3 - g;  // the layer whose dZ this epilogue forms
            unsigned char* dst = sm + BK_A + (r / 8) * (KC_H * 128) + (r % 8) * 16;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float v[16];
                tmem_ld16(lane_base + (uint32_t)(16 * q), v);
#pragma unroll
                for (int h2 = 0; h2 < 2; ++h2) {
                    const int c0 = 16 * q + 8 * h2;
                    uint4 av = make_uint4(0u, 0u, 0u, 0u);
                    if (row < M) av = *reinterpret_cast<const uint4*>(acts + (size_t)l * LS + (size_t)row * H + c0);
                    const uint32_t aw[4] = {av.x, av.y, av.z, av.w};
                    uint32_t pw[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float lo = __uint_as_float(aw[e] << 16), hi = __uint_as_float(aw[e] & 0xffff0000u);
                        pw[e] = pack_bf16(lo > 0.f ? v[8 * h2 + 2 * e] : 0.f, hi > 0.f ? v[8 * h2 + 2 * e + 1] : 0.f);
                    }
                    const uint4 pk = make_uint4(pw[0], pw[1], pw[2], pw[3]);
                    *reinterpret_cast<uint4*>(dst + (c0 / 8) * 128) = pk;
                    if (row < M) *reinterpret_cast<uint4*>(dz + (size_t)l * LS + (size_t)row * H + c0) = pk;
                }
            }
        }
        __syncthreads();
        if (s_abort) break;
    }
    if (loss_sum) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
        if ((tid & 31) == 0) atomicAdd(loss_sum, loss * (1.0f / (3.0f * (float)M)));
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// Warpgroups per CTA of the forward kernel (NR_NRC_FW_WG: 1, 2 or 3).
#ifndef NR_NRC_FW_WG
#define NR_NRC_FW_WG 3
#endif
constexpr int kFwWg = NR_NRC_FW_WG;
static_assert(kFwWg >= 1 && kFwWg <= 3, "1 to 3 warpgroups per forward CTA");
size_t nrc_forward_tc_smem() { return (size_t)fw_smem(kFwWg); }

namespace {
std::atomic<bool> g_tc_disabled{false};
}
void nrc_tc_disable() { g_tc_disabled.store(true); }
bool nrc_tc_enabled() { return !g_tc_disabled.load(); }

void nrc_tc_setup() {
    cudaFuncSetAttribute(k_nrc_forward_tc<kFwWg>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nrc_forward_tc_smem());
    cudaFuncSetAttribute(k_nrc_backward_data_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, BK_TOTAL);
}

namespace {
void launch_forward_tc(const __nv_bfloat16* wb, const float* params, const __nv_bfloat16* x, const uint4* rec,
                       const NrcRows& R, float* out, int num_sms, uint32_t* err, cudaStream_t st, __nv_bfloat16* acts,
                       uint32_t first_wait) {
    const int M = R.count ? (R.n + R.steps - 1) / R.steps : R.n;
    if (M <= 0) return;
    const int tiles = (M + TM - 1) / TM;
    int blocks = (tiles + kFwWg - 1) / kFwWg;
    // resident CTAs per SM by shared memory: 3 with one warpgroup (58 KB), 2 with two or three
    const int cap = num_sms * (kFwWg == 1 ? 3 : 2);
    if (blocks > cap) blocks = cap;
    k_nrc_forward_tc<kFwWg><<<blocks, 128 * kFwWg, nrc_forward_tc_smem(), st>>>(wb, params, x, rec, R, out, acts, err,
                                                                              first_wait);
}

// Compact records -> BF16 rows of 80 (for the mma.sync forward).
__global__ void k_nrc_expand(const uint4* __restrict__ rec, NrcRows R, __nv_bfloat16* __restrict__ x) {
    const int total = R.count ? min((int)*R.count, R.n) : R.n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const uint4 a = rec[2 * (size_t)i], b = rec[2 * (size_t)i + 1];
        const uint32_t q[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
        uint32_t w[40];
        nrc_expand(q, w);
        nrc_store_row(reinterpret_cast<uint32_t*>(x + (size_t)i * IN), w);
    }
}
}  // namespace

void nrc_launch_forward_tc(const __nv_bfloat16* wb, const float* params, const __nv_bfloat16* x, const NrcRows& R,
                           float* out, int num_sms, uint32_t* err, cudaStream_t st, __nv_bfloat16* acts,
                           uint32_t first_wait) {
    launch_forward_tc(wb, params, x, nullptr, R, out, num_sms, err, st, acts, first_wait);
}

void nrc_launch_forward_tc_records(const __nv_bfloat16* wb, const float* params, const uint4* rec, const NrcRows& R,
                                   float* out, int num_sms, uint32_t* err, cudaStream_t st, uint32_t first_wait) {
    launch_forward_tc(wb, params, nullptr, rec, R, out, num_sms, err, st, nullptr, first_wait);
}

void nrc_launch_expand(const uint4* rec, const NrcRows& R, __nv_bfloat16* x, int num_sms, cudaStream_t st) {
    if (R.n <= 0) return;
    const int blocks = std::min((R.n + 255) / 256, num_sms * 8);
    k_nrc_expand<<<blocks, 256, 0, st>>>(rec, R, x);
}

size_t nrc_wt_image_bytes() { return (size_t)BK_A; }

void nrc_launch_backward_data_tc(const __nv_bfloat16* wb, const float* out, const float* y, const __nv_bfloat16* acts,
                                 __nv_bfloat16* dz, const NrcRows& R, float* loss_sum, int num_sms, void* wt_img,
                                 uint32_t* err, cudaStream_t st, uint32_t first_wait) {
    const int M = R.count ? (R.n + R.steps - 1) / R.steps : R.n;
    if (M <= 0) return;
    k_nrc_pack_wt<<<4, 256, 0, st>>>(wb, static_cast<unsigned char*>(wt_img));
    int blocks = (M + TM - 1) / TM;
    const int cap = num_sms * 4;  // 43 KB of shared memory and 64 tensor-memory columns per CTA
    if (blocks > cap) blocks = cap;
    k_nrc_backward_data_tc<<<blocks, 128, BK_TOTAL, st>>>(wb, out, y, acts, R, dz, loss_sum,
                                                          static_cast<const unsigned char*>(wt_img), err, first_wait);
}

}  // namespace nr
