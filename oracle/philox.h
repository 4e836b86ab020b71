// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw,
// "Parallel Random Numbers: As Easy as 1, 2, 3", SC'11), restated from the
// published round function for the oracle and the CPU restatement.
//
// Stream layout shared with the GPU kernels: a path is keyed by
// (pixel, sample); its n-th uniform draw comes from lane n%4 of the block
// with counter (pixel, sample, n/4, 0x6e755279) and key (seed_lo, seed_hi).
// A uniform is (x >> 8) * 2^-24, in [0, 1).
#pragma once
#include <stdint.h>

static inline void nr_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

#define NR_STREAM_TAG 0x6e755279u

typedef struct {
    uint32_t key[2];
    uint32_t pixel, sample;
    uint32_t n;       // draws taken so far
    uint32_t buf[4];
} nr_path_stream;

static inline void nr_stream_init(nr_path_stream* s, uint64_t seed, uint32_t pixel, uint32_t sample, uint32_t first_draw) {
    s->key[0] = (uint32_t)seed;
    s->key[1] = (uint32_t)(seed >> 32);
    s->pixel = pixel;
    s->sample = sample;
    s->n = first_draw;
    uint32_t ctr[4] = {pixel, sample, first_draw >> 2, NR_STREAM_TAG};
    nr_philox4x32_10(ctr, s->key, s->buf);
}

static inline float nr_u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

static inline float nr_stream_next(nr_path_stream* s) {
    if ((s->n & 3u) == 0u && s->n != 0u) {
        uint32_t ctr[4] = {s->pixel, s->sample, s->n >> 2, NR_STREAM_TAG};
        nr_philox4x32_10(ctr, s->key, s->buf);
    }
    float u = nr_u01(s->buf[s->n & 3u]);
    s->n++;
    return u;
}
