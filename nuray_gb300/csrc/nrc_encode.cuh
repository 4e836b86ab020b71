// The cache's input encoding, shared by the shading kernels (which write
// query and training records) and the tensor-core forward (which expands
// compact query records in shared memory).
//
// 80 BF16 values in 40 words: position in the scene box with 12
// frequencies of sin/cos per axis (words 0-35), outgoing direction and
// shading normal as (phi / 2pi + 0.5, theta / pi) (36, 37), roughness and
// albedo (38, 39).
//
// A compact query record (32 bytes, 8 words) holds the position in the
// scene box as three floats, words 36-39 of the encoding, and a zero word:
// 32 bytes written by the shading kernel and read by the forward instead of
// 160, the 36 frequency words rebuilt from the position bit for bit.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace nr {

// sin and cos of pi x as one BF16 pair: x reduced exactly to r in [-1, 1] of
// the same period-2 class (h - rint(h) is exact for |h| < 2^23), then the
// SFU's sin / cos of pi r (absolute error about 4e-7 on [-pi, pi], far below
// the BF16 step the values are stored with).
__device__ __forceinline__ uint32_t nrc_sincospi_bf16(float x) {
    const float h = 0.5f * x;
    float sv, cv;
    __sincosf((h - rintf(h)) * 6.28318530718f, &sv, &cv);
    __nv_bfloat162 v = __floats2bfloat162_rn(sv, cv);
    return *reinterpret_cast<uint32_t*>(&v);
}

// The 40 words of the encoding from a compact record.
__device__ __forceinline__ void nrc_expand(const uint32_t rec[8], uint32_t w[40]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float p = __uint_as_float(rec[a]);
        float f = 1.f;
#pragma unroll
        for (int k = 0; k < 12; ++k) {
            w[a * 12 + k] = nrc_sincospi_bf16(p * f);
            f *= 2.f;
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) w[36 + i] = rec[3 + i];
}

// The 40 words as ten 16-byte stores (dst 16-byte aligned).
__device__ __forceinline__ void nrc_store_row(uint32_t* dst, const uint32_t w[40]) {
    uint4* d4 = reinterpret_cast<uint4*>(dst);
#pragma unroll
    for (int i = 0; i < 10; ++i) d4[i] = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
}

}  // namespace nr
