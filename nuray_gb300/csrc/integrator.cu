// The ptnee wavefront: ray generation, closest-hit traversal with the
// material sort, shading with NEE / MIS / Russian roulette, shadow
// traversal, film accumulation. One path per (pixel, sample); its random
// numbers come from a Philox stream keyed by (pixel, sample) so any batch
// split and any thread order give the same image.
//
// Per path and vertex this is RendererPTLS::trace
// (src/renderer/rendererptls.cpp:13-94) unrolled into an iteration:
//   L += T * (NEE term);  T *= |wi.n| f / pdf / prr;  emitter hit: L += T * Ke * fac
// which is the reference's recursion result = NEE + Li * |wi.n| f / pdf / prr.
#include "nr_material.cuh"
#include "integrator.h"

namespace nr {

// Warp-aggregated append: every active lane with `want` gets a unique index
// in the queue behind *counter; one atomic per warp.
__device__ __forceinline__ int warp_append(bool want, uint32_t* counter) {
    unsigned active = __activemask();
    unsigned m = __ballot_sync(active, want);
    if (!want) return -1;
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int rank = __popc(m & ((1u << lane) - 1u));
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return (int)(base + rank);
}

// Append keyed by a small category: lanes sharing a key share one atomic.
__device__ __forceinline__ int warp_append_keyed(int key, uint32_t* counters) {
    unsigned active = __activemask();
    unsigned m = __match_any_sync(active, key);
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int rank = __popc(m & ((1u << lane) - 1u));
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&counters[key], (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return (int)(base + rank);
}

// ---------------------------------------------------------------- ray generation
// RendererPTLS::render per-sample body (src/renderer/rendererptls.cpp:170-173):
// jitter x, jitter y, Camera::generateRay.
__global__ void k_raygen(PathState P, WaveDesc W, nr_camera cam, float film_h, Policy pol) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W.count) return;
    uint64_t g = W.base + (uint64_t)i;
    uint32_t srel = (uint32_t)(g / (uint64_t)W.npix);
    const uint32_t pidx = (uint32_t)(g % (uint64_t)W.npix);
    int x, y;
    if (W.pix_xy) { x = W.pix_xy[2 * pidx]; y = W.pix_xy[2 * pidx + 1]; }
    else wave_path(W, g, pol.imgw, x, y, srel);
    uint32_t key = (uint32_t)y * (uint32_t)pol.imgw + (uint32_t)x;
    uint32_t sample = W.sample0 + srel;
    Stream s;
    s.init(pol.seed_lo, pol.seed_hi, key, sample, 0);
    float jx = s.next();
    float jy = s.next();
    f3 d = camera_ray(cam, film_h, (float)x + jx, (float)y + jy, (float)pol.imgw, (float)pol.imgh);
    uint32_t flags = pol.force_train ? NR_META_TRAIN : 0u;
    if (pol.coin && (double)s.next() < 0.2) flags = NR_META_TRAIN;  // sampler.random() < 0.2 (renderernrc.cpp:255)
    P.ray_o[i] = make_float4(cam.pos[0], cam.pos[1], cam.pos[2], 0.f);
    P.ray_d[i] = make_float4(d.x, d.y, d.z, 0.f);
    P.thr[i] = make_float4(1.f, 1.f, 1.f, 1.f);
    P.rad[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.meta[i] = make_uint4(key, sample, s.n, flags);
    P.queue_in[i] = i;
    if (i == 0) P.counters[CNT_IN] = (uint32_t)W.count;
}

// ---------------------------------------------------------------- closest hit + sort
// Persistent: warps take 32 queue entries at a time from a shared cursor.
// Writes the hit record and buckets the slot by shading category
// (material type of the hit, or CAT_MISS) for the shading pass.
// Adds a per-thread count into a 64-bit device counter, one atomic per warp.
__device__ __forceinline__ void warp_count(uint32_t v, uint32_t* lohi) {
    unsigned long long x = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(reinterpret_cast<unsigned long long*>(lohi), x);
}

// Closest hit, persistent: warps take 32 queue entries at a time from a
// shared cursor, one ray per lane to completion (closest_hit), then the slot
// is bucketed by shading category (material type of the hit, or CAT_MISS).
// FAST (trav=1) walks the widened boxes with the one-FMA test alone and
// tests triangles with the fast test and its exact fallback; !FAST (trav=0)
// walks the reference's boxes with its exact arithmetic. The widened boxes
// accept every box the exact test accepts, so trav=1 reaches every triangle
// trav=0 reaches (the same hits but where a ray passes within about 1e-6 of
// a box face and hits a triangle there that the exact test's rounding
// excludes). Measured on the 1M-triangle frame: 757.5 Mpaths/s with the
// margin-and-fallback box test on the reference's boxes, 866.4 with the
// one-FMA test alone (not conservative), 831.3 with that test widened by its
// error bound at run time. (Measured and dropped: a variant that
// refilled idle lanes from the queue with separate node and leaf phases,
// 28 % slower; a four-wide tree collapsed from this one, no faster.)
// Minimum resident 128-thread blocks per SM requested from the register
// allocator for the two traversal kernels (NR_TRACE_MINB, NR_SHADOW_MINB
// below). Traversal is bound by dependent L2 latency, so extra warps pay:
// measured on GB300 for the 1M-triangle frame with the if-if loops, 566
// Mpaths/s at 10 blocks (48 registers, 40 warps) against 530 with no cap
// (53 registers, 36 warps) and 541 at 12 (40 registers, with spills); the
// current loops and caps below.
// Loop shape (NR_WW bits): 1 closest hit while-while with postponed leaves
// (closest_hit_ww), 8 the same without postponing; 2 / 4 any hit likewise;
// 0 the if-if loops (closest_hit, any_hit). Measured for the 1M-triangle
// frame: if-if 585.5 Mpaths/s; postponed leaves in both 591.9 (k_trace
// -14 %, k_shadow slower: its first leaf often holds the occluder); in
// closest hit only 636.6; with any hit while-while without postponing 645.4;
// closest hit without postponing too 606.6. With this shape the caps were
// best at 10 / 10 (trace 8: 621.8, 12: 629.6; shadow 8: 639.9, 12: 603.1).
// Once the closest-hit walk lost its step budget (one register less) and
// took the folded box test, 12 blocks (40 registers, 28 bytes of spills)
// overtook 10 for it: 912.2 against 901.4 Mpaths/s, 9 blocks 879.9; the
// shadow kernel stays at 10 (8: 906.8, 12: 909.7, 10: 912.1).
// Also measured and dropped for the shadow rays: dynamic fetch of new rays
// into idle lanes (Aila and Laine 2009) at 4, 8 or 16 idle lanes, 571;
// the shadow queue sorted by light (counting sort, 257 buckets) before the
// shadow kernel, 541: rays from neighbouring pixels to different lights
// share more of their walk than rays to one light from across the frame.
// Likewise within a warp's window of 128 or 256 queued rays, grouped by the
// cell of a 4x4x4 grid holding the ray's end point (counting sort in shared
// memory): 756.1 and 743.3 against 772.1.
#ifndef NR_TRACE_MINB
#define NR_TRACE_MINB 12
#endif
#ifndef NR_SHADOW_MINB
#define NR_SHADOW_MINB 10
#endif
#ifndef NR_WW
#define NR_WW 5
#endif
// Entries of each traversal stack kept in shared memory (a power of two; 0:
// all in local memory). Measured on the 1M-triangle frame: K = 4 704.2 and
// K = 8 706.1 against 757.5 Mpaths/s with the whole stack in local memory
// (L1-resident already; the ring's index arithmetic costs issue slots).
#ifndef NR_SMEM_STACK
#define NR_SMEM_STACK 0
#endif

template <bool COUNT, bool FAST>
__global__ void __launch_bounds__(128, NR_TRACE_MINB) k_trace(PathState P, DeviceScene S, int capacity) {
    const uint32_t n = P.counters[CNT_IN];
    const int lane = threadIdx.x & 31;
    uint32_t nv = 0, nt = 0;
#if NR_SMEM_STACK
    __shared__ int2 ring[NR_SMEM_STACK * 128];
#else
    int2* ring = nullptr;
#endif
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&P.counters[CNT_WORK], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        uint32_t idx = base + lane;
        if (idx < n) {
            int slot = P.queue_in[idx];
            f3 o = xyz(P.ray_o[slot]), d = xyz(P.ray_d[slot]);
            float t, b1, b2;
            int tri = (NR_WW & 9) ? closest_hit_ww<FAST ? 2 : 0, (NR_WW & 1) != 0, NR_SMEM_STACK>(
                                        S, o, d, t, b1, b2, &P.counters[CNT_ERR], COUNT ? &nv : nullptr,
                                        COUNT ? &nt : nullptr, ring)
                            : closest_hit<FAST>(S, o, d, t, b1, b2, &P.counters[CNT_ERR], COUNT ? &nv : nullptr,
                                                COUNT ? &nt : nullptr);
            P.hit[slot] = make_float4(t, b1, b2, __int_as_float(tri));
            int cat = CAT_MISS;
            if (tri >= 0) cat = S.mats[__float_as_int(__ldg(&S.tri_geo[3 * tri + 1]).w)].type;
            int pos = warp_append_keyed(cat, &P.counters[CNT_CAT]);
            P.sorted[(size_t)cat * capacity + pos] = slot;
        }
    }
    if (COUNT) {
        warp_count(nv, &P.counters[CNT_NODES]);
        warp_count(nt, &P.counters[CNT_TRIS]);
    }
}

// The sort of k_trace for hits recorded by an earlier pass over the same
// paths (P.hit pointing at that bounce's record): no traversal.
__global__ void k_sort_recorded(PathState P, DeviceScene S, int capacity) {
    const uint32_t n = P.counters[CNT_IN];
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int slot = P.queue_in[idx];
        const int tri = __float_as_int(P.hit[slot].w);
        int cat = CAT_MISS;
        if (tri >= 0) cat = S.mats[__float_as_int(__ldg(&S.tri_geo[3 * tri + 1]).w)].type;
        const int pos = warp_append_keyed(cat, &P.counters[CNT_CAT]);
        P.sorted[(size_t)cat * capacity + pos] = slot;
    }
}

// Shadow rays, persistent like k_trace: occluded when any reachable triangle
// has t <= the ray's limit (any_hit); unoccluded rays add their NEE term.
template <bool COUNT, bool FAST>
__global__ void __launch_bounds__(128, NR_SHADOW_MINB) k_shadow(PathState P, DeviceScene S, float4* t_before) {
    // (a full queue drops rays with an error bit but still counts them)
    const uint32_t n = min(P.counters[CNT_SHADOW], (uint32_t)P.sh_cap);
    const int lane = threadIdx.x & 31;
    uint32_t nv = 0, nt = 0;
#if NR_SMEM_STACK
    __shared__ int ring[NR_SMEM_STACK * 128];
#else
    int* ring = nullptr;
#endif
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&P.counters[CNT_WORK_SH], 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        uint32_t idx = base + lane;
        if (idx < n) {
            float4 o = P.sh_o[idx], d = P.sh_d[idx];
            const bool env = o.w < 0.f;  // an environment sample: k_env_fold adds it
            const float tmax = env ? -o.w : o.w;
            const bool occluded =
                (NR_WW & 6) ? any_hit_ww<FAST ? 2 : 0, (NR_WW & 2) != 0, NR_SMEM_STACK>(
                                  S, xyz(o), xyz(d), tmax, &P.counters[CNT_ERR], COUNT ? &nv : nullptr,
                                  COUNT ? &nt : nullptr, ring)
                      : any_hit<FAST>(S, xyz(o), xyz(d), tmax, &P.counters[CNT_ERR], COUNT ? &nv : nullptr,
                                      COUNT ? &nt : nullptr);
            if (P.vis) P.vis[__float_as_int(d.w)] = occluded ? 0 : 1;
            if (env) {
                if (occluded) P.sh_c[idx].x = P.sh_c[idx].y = P.sh_c[idx].z = 0.f;
            } else if (!occluded) {
                int slot = __float_as_int(d.w);
                float4 c = P.sh_c[idx];
                float4 r = P.rad[slot];
                P.rad[slot] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.f);
                // a cache training record that excludes its vertex's light sample
                const int rec = __float_as_int(c.w);
                if (t_before && rec >= 0) {
                    float4 b = t_before[rec];
                    t_before[rec] = make_float4(b.x + c.x, b.y + c.y, b.z + c.z, 0.f);
                }
            }
        }
    }
    if (COUNT) {
        warp_count(nv, &P.counters[CNT_SH_NODES]);
        warp_count(nt, &P.counters[CNT_SH_TRIS]);
    }
}

// After k_shadow: every environment sample of the bounce adds its
// contribution (zero if occluded) to its path, after the path's area-light
// sample; one environment sample per path, so one writer per slot.
__global__ void k_env_fold(PathState P, float4* t_before) {
    const uint32_t n = min(P.counters[CNT_SHADOW], (uint32_t)P.sh_cap);
    for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        if (!(P.sh_o[idx].w < 0.f)) continue;
        const int slot = __float_as_int(P.sh_d[idx].w);
        const float4 c = P.sh_c[idx], r = P.rad[slot];
        P.rad[slot] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.f);
        const int rec = __float_as_int(c.w);
        if (t_before && rec >= 0) {
            const float4 b = t_before[rec];
            t_before[rec] = make_float4(b.x + c.x, b.y + c.y, b.z + c.z, 0.f);
        }
    }
}

// ---------------------------------------------------------------- shading
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
// Training paths of the online cache: a fixed hash of (pixel, sample).
__device__ __forceinline__ bool nrc_is_training(uint32_t pixel, uint32_t sample, uint32_t stride) {
    return hash32(pixel ^ hash32(sample + 0x9e3779b9u)) % stride == 0u;
}

// Queues a shadow ray (or, when no hit can come before the limit, adds its
// contribution at once). rec: the training record whose target leaves this
// light sample out, or -1.
// TAIL: trace the shadow ray here (the any-hit walk of k_shadow) instead of
// queueing it. env: the vertex's environment sample, queued with its limit
// negated: k_shadow leaves its contribution in the queue entry (zero when
// occluded) and k_env_fold adds it after the area-light samples, so each
// path's radiance has one writer at a time and the restatement's order.
template <bool NRC, bool TAIL = false>
__device__ __forceinline__ void emit_shadow(const PathState& P, const DeviceScene& S, const Policy& pol,
                                            const NrcCtx& C, int slot, int rec, f3 so, f3 d, float tmax, f3 c,
                                            bool env = false) {
    if (TAIL && tmax > 0.f) {
        const bool occluded = pol.trav ? any_hit_ww<2, (NR_WW & 2) != 0>(S, so, d, tmax, &P.counters[CNT_ERR])
                                       : any_hit_ww<0, (NR_WW & 2) != 0>(S, so, d, tmax, &P.counters[CNT_ERR]);
        if (occluded) return;
        tmax = 0.f;  // unoccluded: added below
    }
    if (tmax > 0.f) {
        int q = warp_append(true, &P.counters[CNT_SHADOW]);
        if (q >= P.sh_cap) { atomicOr(&P.counters[CNT_ERR], 4u); return; }
        P.sh_o[q] = make_float4(so.x, so.y, so.z, env ? -tmax : tmax);
        P.sh_d[q] = make_float4(d.x, d.y, d.z, __int_as_float(slot));
        P.sh_c[q] = make_float4(c.x, c.y, c.z, __int_as_float(rec));
    } else {
        float4 r = P.rad[slot];
        P.rad[slot] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.f);
        if (NRC && rec >= 0) {
            float4 b = C.t_before[rec];
            C.t_before[rec] = make_float4(b.x + c.x, b.y + c.y, b.z + c.z, 0.f);
        }
    }
}

// MT: the shading category when it is known at compile time (a material
// type, or CAT_MISS), -1 for any. TAIL: light samples traced here and the
// continuing path not queued. Returns whether the path goes on.
template <bool NRC, int MT = -1, bool TAIL = false>
__device__ __forceinline__ bool shade_one(const PathState& P, const DeviceScene& S, const Policy& pol, int slot,
                                          const NrcCtx& C) {
    float4 h = P.hit[slot];
    float4 thr = P.thr[slot];
    uint4 meta = P.meta[slot];
    const float4 dir4 = P.ray_d[slot];
    f3 dir = xyz(dir4);
    f3 T = xyz(thr);
    int tri = __float_as_int(h.w);
    if (MT == CAT_MISS || (MT < 0 && tri < 0)) {
        if (S.env_tex >= 0) {
            float4 r = P.rad[slot];
            f3 e = env_lookup(S, dir);
            // envis: the previous vertex also sampled the environment; dir4.w
            // holds the BSDF density of this direction (balance heuristic)
            if (dir4.w > 0.f && S.env_weight) e = e * (dir4.w / (dir4.w + env_pdf(S, dir)));
            P.rad[slot] = make_float4(r.x + T.x * e.x, r.y + T.y * e.y, r.z + T.z * e.z, 0.f);
        }
        return false;
    }
    float b1 = h.y, b2 = h.z;
    float4 s0 = __ldg(&S.tri_shade[4 * tri]), s1 = __ldg(&S.tri_shade[4 * tri + 1]);
    float4 s2 = __ldg(&S.tri_shade[4 * tri + 2]), s3 = __ldg(&S.tri_shade[4 * tri + 3]);
    int mat = __float_as_int(s3.w);
    // Triangle::getNormal / getTexCoords (src/scene/triangle.cpp:35-43)
    float w0 = 1.0f - b1 - b2;
    f3 normal = normalized(w0 * xyz(s0) + b1 * xyz(s1) + b2 * xyz(s2));
    f3 wo = -dir;
    const int type = MT >= 0 ? MT : S.mats[mat].type;
    if (type == NR_MAT_LIGHT) {  // emitter: Ke * light_fac (rendererptls.cpp:33-36)
        const nr_material& M = S.mats[mat];
        float4 r = P.rad[slot];
        float lf = thr.w;
        P.rad[slot] = make_float4(r.x + T.x * M.c0[0] * lf, r.y + T.y * M.c0[1] * lf, r.z + T.z * M.c0[2] * lf, 0.f);
        return false;
    }
    // opaque back faces end the path (rendererptls.cpp:41-42)
    if (dot(normal, dir) > 0.f && !mat_transmissive(type)) return false;
    // texture coordinates: t0 = (s0.w, s1.w), t1 = (s2.w, s3.x), t2 = (s3.y, s3.z)
    f3 uv = mk(w0 * s0.w + b1 * s2.w + b2 * s3.y, w0 * s1.w + b1 * s3.x + b2 * s3.z, 0.f);
    MatView M = load_mat(S, mat, uv);
    if (MT >= 0) M.type = MT;  // the switch over material types folds to one case
    f3 o = xyz(P.ray_o[slot]);
    f3 hit_pos = o + dir * h.x;
    Stream rng;
    rng.init(pol.seed_lo, pol.seed_hi, meta.x, meta.y, meta.z);
    float fac = 1.0f;
    const int depth = (int)(meta.w & NR_META_DEPTH_MASK);
    uint32_t flags = meta.w & NR_META_SEEN_DIFFUSE;
    const uint32_t train_flag = meta.w & NR_META_TRAIN;
    bool query_here = false;
    int rec = -1;  // training record whose target leaves out this vertex's light sample
    if (NRC) {
        const bool train = pol.excl ? train_flag != 0 : nrc_is_training(meta.x, meta.y, C.train_stride);
        // Past the first diffuse bounce the cache stands in for the rest of the
        // path: from depth min_depth on, or for training paths from
        // train_depth on (their earlier vertices then learn from it).
        // renderer=nrc asks at any vertex: depth >= path_lim, or
        // path_lim_train on training paths (renderernrc.cpp:130).
        const bool end_here = train ? (C.train_depth > 0 && depth >= C.train_depth) : depth >= C.min_depth;
        const bool diffuse_here = C.first && nrc_diffuse(M, C.rough);
        if ((flags || diffuse_here || pol.excl) && C.query && end_here) {
            int q = warp_append(true, &C.counters[0]);
            C.q_slot[q] = slot;
            C.q_thr[q] = make_float4(T.x, T.y, T.z, 0.f);
            uint32_t qr[8];
            nrc_record(qr, C.lo, C.inv_ext, hit_pos, wo, normal, nrc_roughness(M), M.c0);
            C.q_rec[2 * (size_t)q] = make_uint4(qr[0], qr[1], qr[2], qr[3]);
            C.q_rec[2 * (size_t)q + 1] = make_uint4(qr[4], qr[5], qr[6], qr[7]);
            if (!C.direct) return false;
            query_here = true;  // the light sample below stays explicit
        } else if (train) {
            int r = warp_append(true, &C.counters[1]);
            if (r < C.tcap) {
                C.t_slot[r] = slot;
                C.t_thr[r] = make_float4(T.x, T.y, T.z, 0.f);
                C.t_before[r] = P.rad[slot];
                nrc_encode(reinterpret_cast<uint32_t*>(C.t_x) + (size_t)r * 40, C.lo, C.inv_ext, hit_pos, wo, normal,
                           nrc_roughness(M), M.c0);
                if (C.direct) rec = r;
            }
        }
        if (nrc_diffuse(M, C.rough)) flags = NR_META_SEEN_DIFFUSE;
    }

    // next-event estimation (rendererptls.cpp:49-78)
    if (pol.excl && pol.nee && mat_nee(type)) fac = 0.0f;  // is_light_sampled (renderernrc.cpp:139)
    if (pol.nee && mat_nee(type) && S.num_lights > 0) {
        const int li = pick_light(S, rng.next());
        const float4* L = S.lights + 6 * li;
        float4 l0 = __ldg(&L[0]), l1 = __ldg(&L[1]), l2 = __ldg(&L[2]);
        float4 n0 = __ldg(&L[3]), n1 = __ldg(&L[4]), n2 = __ldg(&L[5]);
        // Triangle::sample (src/scene/triangle.cpp:45-55)
        float r1 = rng.next();
        float r2 = rng.next();
        if (r1 + r2 > 1.f) { r1 = 1.f - r1; r2 = 1.f - r2; }
        float lw = 1.f - r1 - r2;
        f3 light_pos = lw * xyz(l0) + r1 * xyz(l1) + r2 * xyz(l2);
        f3 light_normal = normalized(lw * xyz(n0) + r1 * xyz(n1) + r2 * xyz(n2));
        f3 light_vec = light_pos - hit_pos;
        f3 wl = normalized(light_vec);
        f3 Ke = mk(l0.w, l1.w, l2.w);
        float light_pdf = S.light_p;
        float cos_l = dot(light_normal, -wl);
        float light_omega_pdf = light_pdf * dot(light_vec, light_vec) / smax(1e-6f, cos_l);
        float brdf_omega_pdf = mat_pdf(M, wo, normal, wl);
        float mis = light_omega_pdf / (light_omega_pdf + brdf_omega_pdf);
        if (!pol.mis) mis = 0.5f;
        if (pol.excl) mis = 1.0f;  // renderernrc.cpp:155: no MIS weight
        else fac = 1.0f - mis;
        f3 brdf = mat_bxdf(M, wo, normal, wl);
        f3 Ll = Ke / norm2(light_vec) * smax(0.f, cos_l) / light_pdf;
        const float geo = smax(0.f, dot(normal, normalized(light_pos - hit_pos)));
        f3 c = Ll * brdf * geo * mis;
        c = c * T;
        if (c.x != 0.f || c.y != 0.f || c.z != 0.f || (pol.adj && cos_l > 0.f && geo > 0.f && mis > 0.f)) {
            // Visible iff the closest t satisfies t + 2e-3 > |light_vec| (in
            // double there), i.e. occluded iff some hit has t <= |lv| - 2e-3.
            double lim = (double)norm(light_vec) - 2e-3;
            float tmax = lim > 0.0 ? __double2float_rd(lim) : 0.0f;
            emit_shadow<NRC, TAIL>(P, S, pol, C, slot, rec, hit_pos + wl * 1e-3f, wl, tmax, c);
        }
    }
    // envis: one environment light sample more (no counterpart in the
    // reference), weighted against the BSDF-sampled miss by the balance
    // heuristic; its two draws follow the area-light draws
    bool env_sampled = false;
    if (pol.envis && pol.nee && mat_nee(type) && S.env_weight) {
        env_sampled = true;
        const float r1 = rng.next(), r2 = rng.next();
        f3 we;
        float pe;
        if (env_sample(S, r1, r2, we, pe)) {
            const float cosn = dot(normal, we);
            if (cosn > 0.f) {
                // at the depth limit no BSDF sample follows: the light sample takes the full weight
                const bool last = pol.maxdepth > 0 && depth + 1 >= pol.maxdepth;
                const float pb = last ? 0.f : mat_pdf(M, wo, normal, we);
                const f3 c = T * mat_bxdf(M, wo, normal, we) * env_lookup(S, we) * (cosn / (pe + pb));
                if (c.x != 0.f || c.y != 0.f || c.z != 0.f)
                    emit_shadow<NRC, TAIL>(P, S, pol, C, slot, rec, hit_pos + we * 1e-3f, we, 3.0e38f, c, true);
            }
        }
    }
    if (NRC && query_here) return false;
    if (pol.maxdepth > 0 && depth + 1 >= pol.maxdepth) return false;
    // Russian roulette (rendererptls.cpp:80-83)
    float prr = depth < pol.rrdepth ? 1.0f : pol.prr;
    float u = rng.next();
    if (depth >= pol.rrdepth && (pol.excl ? !(u < prr) : u > prr)) return false;  // renderernrc.cpp:162: go on while u < prr
    f3 wi = mat_sample(M, rng, wo, normal);
    float pdf = mat_pdf(M, wo, normal, wi);
    f3 brdf = mat_bxdf(M, wo, normal, wi);
    // contri = Li * |wi.n| * brdf / pdf / prr (rendererptls.cpp:90)
    f3 Tn = T * fabsf(dot(wi, normal)) * brdf / pdf / prr;
    f3 no = hit_pos + wi * 1e-3f;
    if (!TAIL) {
        int q = warp_append(true, &P.counters[CNT_OUT]);
        P.queue_out[q] = slot;
    }
    P.ray_o[slot] = make_float4(no.x, no.y, no.z, 0.f);
    P.ray_d[slot] = make_float4(wi.x, wi.y, wi.z, env_sampled ? pdf : 0.f);
    P.thr[slot] = make_float4(Tn.x, Tn.y, Tn.z, fac);
    P.meta[slot] = make_uint4(meta.x, meta.y, rng.n, (uint32_t)(depth + 1) | flags | train_flag);
    return true;
}

// Shading: one kernel per shading category of the bucketed queue (the five
// material types, emitters, misses), each compiled with its category fixed
// so the material switch folds to one case and the kernel keeps only that
// material's registers. All seven are launched per bounce; each strides
// over its device-side count with at most 32 rounds of resident blocks.
// Measured on the 1M-triangle frame (Mpaths/s): one kernel for all
// categories 761.6, per category 771.3 (C3, mixed materials: 751.4 ->
// 761.2); 8, 32 or 128 rounds of blocks 769.9, 771.3, (C3) 759.7.
// Blocks per SM asked of the register allocator: 8 (64 registers). For the
// single kernel before: 646.3 uncapped (94 registers), 651.8 at 6, 657.4
// at 8, 647.3 at 10, 629.7 at 12; per category 6 gives 763.3 against 771.3;
// re-checked with the tail kernel and the category mask: 6 / 8 / 10 give
// 766.0 / 773.9 / 768.6.
#ifndef NR_SHADE_MINB
#define NR_SHADE_MINB 8
#endif
#ifndef NR_SHADE_ROUNDS
#define NR_SHADE_ROUNDS 32
#endif
template <bool NRC, int MT>
__global__ void __launch_bounds__(128, NR_SHADE_MINB) k_shade(PathState P, DeviceScene S, Policy pol, int capacity,
                                                              NrcCtx C) {
    if (MT >= 0) {
        const uint32_t n = P.counters[CNT_CAT + (MT >= 0 ? MT : 0)];
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            shade_one<NRC, MT>(P, S, pol, P.sorted[(size_t)MT * capacity + i], C);
        return;
    }
    // MT = -1: every category in one kernel (categories are contiguous, so
    // a warp mostly runs one material's code)
    uint32_t start[NUM_CAT];
    uint32_t total = 0;
#pragma unroll
    for (int c = 0; c < NUM_CAT; ++c) { start[c] = total; total += P.counters[CNT_CAT + c]; }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        int c = 0;
#pragma unroll
        for (int k = 1; k < NUM_CAT; ++k) if (i >= start[k]) c = k;
        shade_one<NRC>(P, S, pol, P.sorted[(size_t)c * capacity + (i - start[c])], C);
    }
}
// Waves of at most SHADE_SPLIT_MIN paths shade with the one kernel for all
// categories: their bounces are short, and six mostly empty launches per
// bounce cost more than the split saves (time to relMSE 1e-3 with 960x540
// frames of 1 spp: 10.40 s with one kernel, 11.34 s with seven).
template <bool NRC>
static void launch_shade(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity, int blocks,
                         const NrcCtx& C, cudaStream_t st) {
    if (capacity <= SHADE_SPLIT_MIN) {
        k_shade<NRC, -1><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
        return;
    }
    // categories of material types absent from the scene can hold no path
    if (S.cat_mask & (1u << NR_MAT_LAMBERT)) k_shade<NRC, NR_MAT_LAMBERT><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
    if (S.cat_mask & (1u << NR_MAT_GGXR)) k_shade<NRC, NR_MAT_GGXR><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
    if (S.cat_mask & (1u << NR_MAT_GGX)) k_shade<NRC, NR_MAT_GGX><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
    if (S.cat_mask & (1u << NR_MAT_GLASS)) k_shade<NRC, NR_MAT_GLASS><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
    if (S.cat_mask & (1u << NR_MAT_BLINNPHONG))
        k_shade<NRC, NR_MAT_BLINNPHONG><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
    if (S.cat_mask & (1u << NR_MAT_LIGHT)) k_shade<NRC, NR_MAT_LIGHT><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
    k_shade<NRC, CAT_MISS><<<blocks, 128, 0, st>>>(P, S, pol, capacity, C);
}

// The rest of every live path in one launch, one thread per path: closest
// hit, then shade_one in its TAIL form (light samples traced inline), until
// the path ends. For small waves, whose last bounces hold few rays: the
// bounce-by-bounce wavefront waits at each bounce for its slowest ray, this
// kernel only for the slowest path. Same functions, same results.
#ifndef NR_TAIL_MAX_BOUNCES
#define NR_TAIL_MAX_BOUNCES 4096
#endif
// Resident blocks per SM requested for the tail kernel. Its paths wait on
// dependent traversal loads with few live lanes, so warps in flight pay more
// than the registers' spills cost: 960x540 frames of 1 spp take 1.543 ms at 4
// blocks (89 registers), 1.536 at 6, 1.463 at 8 (64 registers, 176 bytes
// spilled), 1.459 at 10, 1.476 at 12 and 1.535 at 16 (40 and 32 registers,
// kilobytes spilled).
#ifndef NR_TAIL_MINB
#define NR_TAIL_MINB 8
#endif
template <bool NRC, bool FAST>
__global__ void __launch_bounds__(128, NR_TAIL_MINB) k_tail(PathState P, DeviceScene S, Policy pol, NrcCtx C) {
    const uint32_t n = P.counters[CNT_IN];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int slot = P.queue_in[i];
    for (int b = 0; b < NR_TAIL_MAX_BOUNCES; ++b) {
        const f3 o = xyz(P.ray_o[slot]), d = xyz(P.ray_d[slot]);
        float t, b1, b2;
        const int tri = closest_hit_ww<FAST ? 2 : 0>(S, o, d, t, b1, b2, &P.counters[CNT_ERR]);
        P.hit[slot] = make_float4(t, b1, b2, __int_as_float(tri));
        if (!shade_one<NRC, -1, true>(P, S, pol, slot, C)) return;
    }
    atomicOr(&P.counters[CNT_ERR], 16u);  // bounce cap: the path did not end
}

// ---------------------------------------------------------------- shadow rays
// Moves the continuation queue into place for the next bounce and clears the
// per-bounce counters; also keeps the 64-bit ray totals.
__global__ void k_advance(uint32_t* counters) {
    uint32_t in = counters[CNT_IN], sh = counters[CNT_SHADOW];
    unsigned long long* rays = reinterpret_cast<unsigned long long*>(counters + CNT_RAYS);
    unsigned long long* shr = reinterpret_cast<unsigned long long*>(counters + CNT_SHRAYS);
    *rays += in;
    *shr += sh;
    counters[CNT_IN] = counters[CNT_OUT];
    counters[CNT_OUT] = 0;
    counters[CNT_SHADOW] = 0;
    counters[CNT_WORK] = 0;
    counters[CNT_WORK_SH] = 0;
    for (int c = 0; c < NUM_CAT; ++c) counters[CNT_CAT + c] = 0;
}

// Clears the per-wave counters; the error word and the totals from
// CNT_RAYS on are kept for the whole render.
__global__ void k_reset_counters(uint32_t* counters) {
    int i = threadIdx.x;
    if (i < CNT_RAYS && i != CNT_ERR) counters[i] = 0;
}

// ---------------------------------------------------------------- film
// For every pixel of the wave, adds max(0, L) of its samples in sample order
// (rendererptls.cpp:173). film holds npix float4 sums.
__global__ void k_film(PathState P, WaveDesc W, float4* film, int imgw) {
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint32_t)W.npix) return;
    int x, y;
    const uint64_t end = W.base + (uint64_t)W.count;
    if (W.tiled == 2) {
        const uint32_t tp = (uint32_t)(W.g_w * W.g_h), tile = p / tp, tiles_x = (uint32_t)imgw / (uint32_t)W.g_w;
        x = (int)((tile % tiles_x) * (uint32_t)W.g_w + (p % tp) % (uint32_t)W.g_w);
        y = (int)((tile / tiles_x) * (uint32_t)W.g_h + (p % tp) / (uint32_t)W.g_w);
        const uint32_t pix = (uint32_t)y * (uint32_t)imgw + (uint32_t)x;
        // this pixel's samples in the wave, in sample order
        uint32_t s = (uint32_t)(W.base / ((uint64_t)W.g_s * W.npix)) * (uint32_t)W.g_s;
        float4 acc = film[pix];
        bool any = false;
        for (;; ++s) {
            const uint64_t g = tile2_index(W, p, s);
            if (g >= end) break;
            if (g < W.base) continue;
            const float4 r = P.rad[g - W.base];
            acc.x += smax(0.f, r.x);
            acc.y += smax(0.f, r.y);
            acc.z += smax(0.f, r.z);
            any = true;
        }
        if (any) film[pix] = acc;
        return;
    }
    frame_pixel(p, imgw, W.tiled, x, y);
    const uint32_t pix = (uint32_t)y * (uint32_t)imgw + (uint32_t)x;
    uint64_t s_first = W.base / (uint64_t)W.npix;
    uint64_t g = s_first * (uint64_t)W.npix + p;
    if (g < W.base) g += (uint64_t)W.npix;
    if (g >= end) return;
    float4 acc = film[pix];
    for (; g < end; g += (uint64_t)W.npix) {
        float4 r = P.rad[g - W.base];
        acc.x += smax(0.f, r.x);
        acc.y += smax(0.f, r.y);
        acc.z += smax(0.f, r.z);
    }
    film[pix] = acc;
}

// Copies per-sample max(0, L) to out[(pixel * spp + sample) * 3], pixel the
// index in the pixel list, or y * imgw + x for a full frame.
__global__ void k_collect(PathState P, WaveDesc W, float* out, int spp, int imgw) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W.count) return;
    uint64_t g = W.base + (uint64_t)i;
    uint64_t srel = g / (uint64_t)W.npix, pidx = g % (uint64_t)W.npix;
    if (!W.pix_xy && W.tiled) {
        int x, y;
        uint32_t s;
        wave_path(W, g, imgw, x, y, s);
        srel = s;
        pidx = (uint64_t)y * (uint64_t)imgw + (uint64_t)x;
    }
    float4 r = P.rad[i];
    float* o = out + (pidx * (uint64_t)spp + srel) * 3;
    o[0] = smax(0.f, r.x); o[1] = smax(0.f, r.y); o[2] = smax(0.f, r.z);
}

// Mean, gamma and 8-bit conversion (rendererptls.cpp:175-180).
__global__ void k_finish(const float4* film, int npix, float inv_spp, float* hdr, uint8_t* rgb8) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float4 a = film[p];
    float m[3] = {a.x * inv_spp, a.y * inv_spp, a.z * inv_spp};
    for (int k = 0; k < 3; ++k) {
        if (hdr) hdr[3 * p + k] = m[k];
        if (rgb8) {
            float g = powf(m[k], (float)(1.0 / 2.2)) * 255.0f;
            g = smin(255.0f, smax(0.0f, g));
            rgb8[3 * p + k] = (uint8_t)(int)g;
        }
    }
}

// ---------------------------------------------------------------- online cache
// Adds the cache prediction of each query: L += T * max(0, nrc(x)).
__global__ void k_nrc_apply(PathState P, NrcCtx C, const float* __restrict__ pred) {
    const int n = (int)C.counters[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int slot = C.q_slot[i];
        float4 t = C.q_thr[i], r = P.rad[slot];
        const float* o = pred + 3 * (size_t)i;
        P.rad[slot] = make_float4(r.x + t.x * fmaxf(0.f, o[0]), r.y + t.y * fmaxf(0.f, o[1]), r.z + t.z * fmaxf(0.f, o[2]), 0.f);
    }
}

// Training targets: radiance the path gathered from the vertex on, divided by
// the throughput that reached the vertex; channels with negligible
// throughput copy the luminance-weighted value, and targets are clamped.
__global__ void k_nrc_targets(PathState P, NrcCtx C, float* __restrict__ y, float clamp_max) {
    const int n = min((int)C.counters[1], C.tcap);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int slot = C.t_slot[i];
        float4 a = P.rad[slot], b = C.t_before[i], t = C.t_thr[i];
        float d[3] = {a.x - b.x, a.y - b.y, a.z - b.z}, tt[3] = {t.x, t.y, t.z};
        float tsum = tt[0] + tt[1] + tt[2], dsum = d[0] + d[1] + d[2];
        for (int k = 0; k < 3; ++k) {
            float v = tt[k] > 1e-4f ? d[k] / tt[k] : (tsum > 1e-4f ? dsum / tsum : 0.f);
            if (!(v >= 0.f)) v = 0.f;  // NaN or negative
            y[3 * (size_t)i + k] = fminf(v, clamp_max);
        }
    }
}

// ---------------------------------------------------------------- single queries
__global__ void k_intersect(DeviceScene S, int n, const float* o, const float* d, int* tri, float* t, float* b1,
                            float* b2, uint32_t* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float tt, u, v;
    int k = closest_hit(S, mk(o[3 * i], o[3 * i + 1], o[3 * i + 2]), mk(d[3 * i], d[3 * i + 1], d[3 * i + 2]), tt, u, v, err);
    tri[i] = k >= 0 ? __float_as_int(__ldg(&S.tri_geo[3 * k]).w) : -1;
    t[i] = tt; b1[i] = u; b2[i] = v;
}

struct ListRng {
    const float* u;
    int i;
    __device__ float next() { return i < 4 ? u[i++] : 0.5f; }
};

__global__ void k_material_probe(DeviceScene S, int mat, int n, const float* wo, const float* nrm, const float* wi,
                                 const float* uv, const float* u, float* f, float* pdf, float* wi_s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 a = mk(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), nn = mk(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
    f3 b = mk(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    MatView M = load_mat(S, mat, mk(uv[3 * i], uv[3 * i + 1], uv[3 * i + 2]));
    f3 ff = mat_bxdf(M, a, nn, b);
    pdf[i] = mat_pdf(M, a, nn, b);
    ListRng r{u + 4 * i, 0};
    f3 ws = mat_sample(M, r, a, nn);
    f[3 * i] = ff.x; f[3 * i + 1] = ff.y; f[3 * i + 2] = ff.z;
    wi_s[3 * i] = ws.x; wi_s[3 * i + 1] = ws.y; wi_s[3 * i + 2] = ws.z;
}

// ---------------------------------------------------------------- launchers
static int g_trace_blocks = 0, g_shadow_blocks = 0, g_num_sms = 1;

void launch_setup(int num_sms) {
    g_num_sms = num_sms > 0 ? num_sms : 1;
    int b1 = 0, b2 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_trace<false, true>, 128, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_shadow<false, true>, 128, 0);
    g_trace_blocks = num_sms * (b1 > 0 ? b1 : 1);
    g_shadow_blocks = num_sms * (b2 > 0 ? b2 : 1);
}

void launch_raygen(const PathState& P, const WaveDesc& W, const nr_camera& cam, float film_h, const Policy& pol,
                   cudaStream_t st) {
    k_raygen<<<(W.count + 255) / 256, 256, 0, st>>>(P, W, cam, film_h, pol);
}

static int count_grid(int cap);

void launch_bounce(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity, int max_count,
                   cudaStream_t st, cudaEvent_t* ev, bool count, const NrcCtx* nrc) {
    if (ev) cudaEventRecord(ev[0], st);
    switch ((count ? 2 : 0) + pol.trav) {
        case 0: k_trace<false, false><<<g_trace_blocks, 128, 0, st>>>(P, S, capacity); break;
        case 1: k_trace<false, true><<<g_trace_blocks, 128, 0, st>>>(P, S, capacity); break;
        case 2: k_trace<true, false><<<g_trace_blocks, 128, 0, st>>>(P, S, capacity); break;
        default: k_trace<true, true><<<g_trace_blocks, 128, 0, st>>>(P, S, capacity); break;
    }
    if (ev) cudaEventRecord(ev[1], st);
    // the shading kernels stride over their device counts; max_count (an
    // upper bound of their sum) and NR_SHADE_ROUNDS size the grids
    int shade_blocks = (max_count + 127) / 128;
    if (shade_blocks < 1) shade_blocks = 1;
    const int most = g_num_sms * NR_SHADE_MINB * NR_SHADE_ROUNDS;
    if (shade_blocks > most) shade_blocks = most;
    if (nrc) launch_shade<true>(P, S, pol, capacity, shade_blocks, *nrc, st);
    else launch_shade<false>(P, S, pol, capacity, shade_blocks, NrcCtx{}, st);
    if (ev) cudaEventRecord(ev[2], st);
    float4* tb = (nrc && nrc->direct) ? nrc->t_before : nullptr;
    switch ((count ? 2 : 0) + pol.trav) {
        case 0: k_shadow<false, false><<<g_shadow_blocks, 128, 0, st>>>(P, S, tb); break;
        case 1: k_shadow<false, true><<<g_shadow_blocks, 128, 0, st>>>(P, S, tb); break;
        case 2: k_shadow<true, false><<<g_shadow_blocks, 128, 0, st>>>(P, S, tb); break;
        default: k_shadow<true, true><<<g_shadow_blocks, 128, 0, st>>>(P, S, tb); break;
    }
    if (pol.envis) k_env_fold<<<count_grid(P.sh_cap), 256, 0, st>>>(P, tb);
    if (ev) cudaEventRecord(ev[3], st);
    k_advance<<<1, 1, 0, st>>>(P.counters);
}

void launch_tail(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity, const NrcCtx* nrc,
                 cudaStream_t st) {
    const int blocks = (capacity + 127) / 128;
    if (nrc) {
        if (pol.trav) k_tail<true, true><<<blocks, 128, 0, st>>>(P, S, pol, *nrc);
        else k_tail<true, false><<<blocks, 128, 0, st>>>(P, S, pol, *nrc);
    } else {
        if (pol.trav) k_tail<false, true><<<blocks, 128, 0, st>>>(P, S, pol, NrcCtx{});
        else k_tail<false, false><<<blocks, 128, 0, st>>>(P, S, pol, NrcCtx{});
    }
}

void launch_trace(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity, cudaStream_t st) {
    if (pol.trav) k_trace<false, true><<<g_trace_blocks, 128, 0, st>>>(P, S, capacity);
    else k_trace<false, false><<<g_trace_blocks, 128, 0, st>>>(P, S, capacity);
}
void launch_advance(uint32_t* counters, cudaStream_t st) { k_advance<<<1, 1, 0, st>>>(counters); }
int shadow_grid() { return g_shadow_blocks; }

void launch_reset_counters(uint32_t* counters, cudaStream_t st) { k_reset_counters<<<1, 32, 0, st>>>(counters); }

// The counts live on the device: grid-stride loops over a grid sized for
// the capacity, at most eight 256-thread blocks per SM.
static int count_grid(int cap) {
    int b = (cap + 255) / 256;
    const int most = 8 * g_num_sms;
    return b < 1 ? 1 : (b > most ? most : b);
}
void launch_sort_recorded(const PathState& P, const DeviceScene& S, int capacity, cudaStream_t st) {
    k_sort_recorded<<<count_grid(capacity), 256, 0, st>>>(P, S, capacity);
}
void launch_nrc_apply(const PathState& P, const NrcCtx& C, const float* pred, int cap, cudaStream_t st) {
    k_nrc_apply<<<count_grid(cap), 256, 0, st>>>(P, C, pred);
}
void launch_nrc_targets(const PathState& P, const NrcCtx& C, float* y, float clamp_max, cudaStream_t st) {
    k_nrc_targets<<<count_grid(C.tcap), 256, 0, st>>>(P, C, y, clamp_max);
}

void launch_film(const PathState& P, const WaveDesc& W, float4* film, int imgw, cudaStream_t st) {
    k_film<<<(W.npix + 255) / 256, 256, 0, st>>>(P, W, film, imgw);
}

void launch_collect(const PathState& P, const WaveDesc& W, float* out, int spp, int imgw, cudaStream_t st) {
    k_collect<<<(W.count + 255) / 256, 256, 0, st>>>(P, W, out, spp, imgw);
}

void launch_finish(const float4* film, int npix, float inv_spp, float* hdr, uint8_t* rgb8, cudaStream_t st) {
    k_finish<<<(npix + 255) / 256, 256, 0, st>>>(film, npix, inv_spp, hdr, rgb8);
}

void launch_intersect(const DeviceScene& S, int n, const float* o, const float* d, int* tri, float* t, float* b1,
                      float* b2, uint32_t* err, cudaStream_t st) {
    k_intersect<<<(n + 127) / 128, 128, 0, st>>>(S, n, o, d, tri, t, b1, b2, err);
}

void launch_material_probe(const DeviceScene& S, int mat, int n, const float* wo, const float* nrm, const float* wi,
                           const float* uv, const float* u, float* f, float* pdf, float* wi_s, cudaStream_t st) {
    k_material_probe<<<(n + 127) / 128, 128, 0, st>>>(S, mat, n, wo, nrm, wi, uv, u, f, pdf, wi_s);
}

}  // namespace nr
