// Launchers of the ptnee wavefront kernels (integrator.cu).
#pragma once
#include "nr_types.h"

namespace nr {

// One wavefront batch: global path indices [base, base + count) with
// g = (sample - sample0) * npix + pixel_index.
struct WaveDesc {
    uint64_t base;
    int32_t count;
    int32_t npix;
    uint32_t sample0;
    const int32_t* pix_xy;  // device (x, y) list, or null for the full frame
    int32_t tiled;          // 0 scanline; 1 full frame in 8x4 pixel tiles (frame_pixel); 2 a warp of paths
                            // holds g_s consecutive samples of a g_w x g_h pixel tile (g_s g_w g_h = 32)
    int32_t g_s, g_w, g_h;
};

#ifdef __CUDACC__
// Full-frame pixel of path index p: row-major, or in 8x4 tiles (one warp of
// consecutive paths covers a compact patch) when the frame divides into them.
__device__ __forceinline__ void frame_pixel(uint32_t p, int w, int tiled, int& x, int& y) {
    if (tiled) {
        uint32_t tile = p >> 5, j = p & 31u, tiles_x = (uint32_t)w >> 3;
        x = (int)((tile % tiles_x) * 8u + (j & 7u));
        y = (int)((tile / tiles_x) * 4u + (j >> 3));
    } else {
        x = (int)(p % (uint32_t)w);
        y = (int)(p / (uint32_t)w);
    }
}

// tiled == 2: paths come in groups of g_s samples of every pixel; within a
// group, 32 consecutive paths are samples 0..g_s-1 of a g_w x g_h pixel
// tile (lane = sample * g_w * g_h + pixel in the tile, row-major), tiles in
// row-major order.
__device__ __forceinline__ void tile2_path(const WaveDesc& W, uint64_t g, int w, int& x, int& y, uint32_t& srel) {
    const uint32_t tp = (uint32_t)(W.g_w * W.g_h);
    const uint64_t per = (uint64_t)W.g_s * W.npix;
    const uint32_t grp = (uint32_t)(g / per), l = (uint32_t)(g % per);
    const uint32_t tile = l >> 5, lane = l & 31u, pit = lane % tp, tiles_x = (uint32_t)w / (uint32_t)W.g_w;
    x = (int)((tile % tiles_x) * (uint32_t)W.g_w + pit % (uint32_t)W.g_w);
    y = (int)((tile / tiles_x) * (uint32_t)W.g_h + pit / (uint32_t)W.g_w);
    srel = grp * (uint32_t)W.g_s + lane / tp;
}
// path index of sample srel of the pixel with film-thread index p (p / tile
// pixels: the tile, the rest: the pixel in it)
__device__ __forceinline__ uint64_t tile2_index(const WaveDesc& W, uint32_t p, uint32_t srel) {
    const uint32_t tp = (uint32_t)(W.g_w * W.g_h);
    return (uint64_t)(srel / (uint32_t)W.g_s) * (uint32_t)W.g_s * W.npix + (uint64_t)(p / tp) * 32u +
           (srel % (uint32_t)W.g_s) * tp + p % tp;
}

// Pixel (x, y) of wave path g (global index) and its sample relative to
// sample0, for a wave without a pixel list.
__device__ __forceinline__ void wave_path(const WaveDesc& W, uint64_t g, int imgw, int& x, int& y, uint32_t& srel) {
    if (W.tiled == 2) {
        tile2_path(W, g, imgw, x, y, srel);
        return;
    }
    srel = (uint32_t)(g / (uint64_t)W.npix);
    frame_pixel((uint32_t)(g % (uint64_t)W.npix), imgw, W.tiled, x, y);
}
#endif

void launch_setup(int num_sms);
void launch_raygen(const PathState& P, const WaveDesc& W, const nr_camera& cam, float film_h, const Policy& pol,
                   cudaStream_t st);
// trace + sort, shade (for waves above 2^22 paths one kernel per shading
// category the scene's materials can produce, else one for all), shadow,
// (envis: the environment samples' fold), advance: bounce_launches(capacity,
// envis, scene category mask) kernels. ev (optional) receives 4 events.
constexpr int SHADE_SPLIT_MIN = 1 << 22;
inline int bounce_launches(int capacity, bool envis, uint32_t cat_mask) {
    return (capacity > SHADE_SPLIT_MIN ? 3 + __builtin_popcount(cat_mask) : 4) + (envis ? 1 : 0);
}
void launch_bounce(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity, int max_count,
                   cudaStream_t st, cudaEvent_t* ev, bool count, const NrcCtx* nrc);
// Query and training-record counts are read from C.counters on the device.
void launch_nrc_apply(const PathState& P, const NrcCtx& C, const float* pred, int cap, cudaStream_t st);
void launch_nrc_targets(const PathState& P, const NrcCtx& C, float* y, float clamp_max, cudaStream_t st);
void launch_reset_counters(uint32_t* counters, cudaStream_t st);
// The closest-hit + material-sort and advance steps alone, for wavefronts
// that shade with kernels of their own (the adjoint replay).
void launch_trace(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity, cudaStream_t st);
void launch_advance(uint32_t* counters, cudaStream_t st);
// Every live path of queue_in to its end in one launch (after some
// wavefront bounces of a small wave); capacity bounds the live count.
void launch_tail(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity, const NrcCtx* nrc,
                 cudaStream_t st);
// k_trace's sort by shading category for hits recorded in P.hit by an earlier pass
void launch_sort_recorded(const PathState& P, const DeviceScene& S, int capacity, cudaStream_t st);
int shadow_grid();  // blocks of the persistent shadow-ray kernels
void launch_film(const PathState& P, const WaveDesc& W, float4* film, int imgw, cudaStream_t st);
void launch_collect(const PathState& P, const WaveDesc& W, float* out, int spp, int imgw, cudaStream_t st);
void launch_finish(const float4* film, int npix, float inv_spp, float* hdr, uint8_t* rgb8, cudaStream_t st);
void launch_intersect(const DeviceScene& S, int n, const float* o, const float* d, int* tri, float* t, float* b1,
                      float* b2, uint32_t* err, cudaStream_t st);
void launch_material_probe(const DeviceScene& S, int mat, int n, const float* wo, const float* nrm, const float* wi,
                           const float* uv, const float* u, float* f, float* pdf, float* wi_s, cudaStream_t st);

}  // namespace nr
