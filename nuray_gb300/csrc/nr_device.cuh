// Device building blocks of the ptnee wavefront: vector helpers, the Philox
// path stream, the reference-exact ray/box and ray/triangle tests and the
// BVH traversals. Included by the .cu files of libnuray_gpu.so only.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

#include "nr_types.h"

namespace nr {

// ------------------------------------------------------------------ vectors
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 mk(float s) { return {s, s, s}; }
__device__ __forceinline__ f3 xyz(float4 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float norm2(f3 a) { return dot(a, a); }
__device__ __forceinline__ float norm(f3 a) { return sqrtf(norm2(a)); }
// vec3::normalized divides by |a| + 1e-8 (src/math/vec3.cpp:70-73)
__device__ __forceinline__ f3 normalized(f3 a) { return a / (norm(a) + 1e-8f); }
// std::max / std::min semantics (first argument kept unless strictly beaten)
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }

// Rounded-to-nearest float ops that the compiler may not fuse; used where the
// reference's FP32 results have to be reproduced bit for bit.
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ f3 rsub3(f3 a, f3 b) { return {rsub(a.x, b.x), rsub(a.y, b.y), rsub(a.z, b.z)}; }
__device__ __forceinline__ float rdot(f3 a, f3 b) { return radd(radd(rmul(a.x, b.x), rmul(a.y, b.y)), rmul(a.z, b.z)); }
__device__ __forceinline__ f3 rcross(f3 a, f3 b) {
    return {rsub(rmul(a.y, b.z), rmul(a.z, b.y)), rsub(rmul(a.z, b.x), rmul(a.x, b.z)),
            rsub(rmul(a.x, b.y), rmul(a.y, b.x))};
}

// Correctly rounded a / b given rb = RN(1/b): one residual correction of
// the product a * rb (Markstein). Exact for finite, non-denormal results.
__device__ __forceinline__ float qdiv(float a, float b, float rb) {
    float q0 = __fmul_rn(a, rb);
    float r = __fmaf_rn(-q0, b, a);
    return __fmaf_rn(r, rb, q0);
}

// RN_float(x + 1e-6) where 1e-6 is the double literal of the reference's
// `s1.dot(e1) + 1e-6` (src/scene/triangle.cpp:31): a float TwoSum with the
// split constant hi + lo. Differs from the double evaluation only when the
// exact sum lies within 2^-48 of a float rounding boundary.
__device__ __forceinline__ float add_1e6(float x) {
    const float hi = 9.99999997475242708e-07f;
    const float lo = (float)(1e-6 - (double)9.99999997475242708e-07f);
    float s = __fadd_rn(x, hi);
    float bb = __fsub_rn(s, x);
    float e = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(hi, bb));
    return __fadd_rn(s, __fadd_rn(e, lo));
}

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon et al., SC'11). Path stream: draw n of path
// (pixel, sample) is lane n%4 of philox(ctr = (pixel, sample, n/4, tag),
// key = seed); uniform = (x >> 8) * 2^-24.
#define NR_STREAM_TAG 0x6e755279u
__device__ __forceinline__ uint4 philox10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

struct Stream {
    uint2 key;
    uint32_t pixel, sample, n;
    uint4 buf;
    __device__ __forceinline__ void init(uint32_t seed_lo, uint32_t seed_hi, uint32_t px, uint32_t smp, uint32_t first) {
        key = make_uint2(seed_lo, seed_hi);
        pixel = px; sample = smp; n = first;
        buf = philox10(make_uint4(pixel, sample, n >> 2, NR_STREAM_TAG), key);
    }
    __device__ __forceinline__ float next() {
        if ((n & 3u) == 0u && n != 0u) buf = philox10(make_uint4(pixel, sample, n >> 2, NR_STREAM_TAG), key);
        uint32_t lane = n & 3u;
        uint32_t x = lane == 0 ? buf.x : (lane == 1 ? buf.y : (lane == 2 ? buf.z : buf.w));
        ++n;
        return (float)(x >> 8) * (1.0f / 16777216.0f);
    }
};

// ------------------------------------------------------------------ intersection
// Ray prepared for the exact slab test: denominators d + 1e-9f and their
// correctly rounded reciprocals (src/hierarchy/bvhnode.cpp:41).
struct SlabRay {
    float ox, oy, oz;
    float dx, dy, dz;     // d + 1e-9f
    float rx, ry, rz;     // RN(1 / (d + 1e-9f))
    float cx, cy, cz;     // RN(-o * r), for the one-FMA approximate quotient
    float abs_err;        // bound on |fma(b, r, c) - (b - o) r| from rounding c
};
__device__ __forceinline__ SlabRay make_slab_ray(f3 o, f3 d) {
    SlabRay r;
    r.ox = o.x; r.oy = o.y; r.oz = o.z;
    r.dx = __fadd_rn(d.x, 1e-9f); r.dy = __fadd_rn(d.y, 1e-9f); r.dz = __fadd_rn(d.z, 1e-9f);
    r.rx = __frcp_rn(r.dx); r.ry = __frcp_rn(r.dy); r.rz = __frcp_rn(r.dz);
    r.cx = -o.x * r.rx; r.cy = -o.y * r.ry; r.cz = -o.z * r.rz;
    // |c| * 2^-24 (rounding of c) with headroom: 2^-22
    r.abs_err = 2.4e-7f * fmaxf(fabsf(r.cx), fmaxf(fabsf(r.cy), fabsf(r.cz)));
    return r;
}

// BVHNode::intersect (src/hierarchy/bvhnode.cpp:35-48) with the same
// rounding: t = (bound - o) / (d + 1e-9f), swap, std::max / std::min.
// Returns the entry distance in *tin when accepted.
__device__ __forceinline__ bool slab_axis(float lo, float hi, float o, float d, float rd, float& tin, float& tout) {
    float t1 = qdiv(__fsub_rn(lo, o), d, rd);
    float t2 = qdiv(__fsub_rn(hi, o), d, rd);
    if (t1 > t2) { float s = t1; t1 = t2; t2 = s; }
    tin = smax(tin, t1);
    tout = smin(tout, t2);
    return true;
}
__device__ __forceinline__ bool box_test(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz,
                                         float& t_entry) {
    float tin = -1e18f, tout = 1e18f;
    slab_axis(lx, hx, r.ox, r.dx, r.rx, tin, tout);
    slab_axis(ly, hy, r.oy, r.dy, r.ry, tin, tout);
    slab_axis(lz, hz, r.oz, r.dz, r.rz, tin, tout);
    t_entry = tin;
    return tin <= tout && tout >= 0.0f;
}

// The same decision from approximate quotients (b - o) * RN(1/d): each is
// within 2^-22.4 of the exact quotient, and the sign is exact, so the result
// can only differ from the exact test when the entry and exit distances lie
// within that error of each other; those cases are recomputed exactly.
__device__ __forceinline__ bool box_test_fast(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz,
                                              float& t_entry) {
    // one FMA per bound: fma(b, r, -o r) is within 2^-22.4 |q| + abs_err of
    // the exact quotient q = (b - o) / d
    float x1 = __fmaf_rn(lx, r.rx, r.cx), x2 = __fmaf_rn(hx, r.rx, r.cx);
    float y1 = __fmaf_rn(ly, r.ry, r.cy), y2 = __fmaf_rn(hy, r.ry, r.cy);
    float z1 = __fmaf_rn(lz, r.rz, r.cz), z2 = __fmaf_rn(hz, r.rz, r.cz);
    float tin = fmaxf(fmaxf(fminf(x1, x2), fminf(y1, y2)), fmaxf(fminf(z1, z2), -1e18f));
    float tout = fminf(fminf(fmaxf(x1, x2), fmaxf(y1, y2)), fminf(fmaxf(z1, z2), 1e18f));
    float margin = 1e-6f * fmaxf(fabsf(tin), fabsf(tout)) + r.abs_err;
    if (tout < -margin) return false;
    if (tin + margin < tout && tout > margin) { t_entry = tin; return true; }
    if (tin > tout + margin) return false;
    return box_test(r, lx, hx, ly, hy, lz, hz, t_entry);
}

// The one-FMA test alone, for boxes widened on the host (DeviceScene::
// nodes_fast): each bound is moved outward by more than the error of these
// quotients and of the reference's own rounding for every ray origin within
// DeviceScene::fast_origin_bound, so the test accepts every box the exact
// test accepts for the unwidened box (and a sliver more around it) without
// a margin or a fallback.
__device__ __forceinline__ bool box_test_plain(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz,
                                               float& t_entry) {
    float x1 = __fmaf_rn(lx, r.rx, r.cx), x2 = __fmaf_rn(hx, r.rx, r.cx);
    float y1 = __fmaf_rn(ly, r.ry, r.cy), y2 = __fmaf_rn(hy, r.ry, r.cy);
    float z1 = __fmaf_rn(lz, r.rz, r.cz), z2 = __fmaf_rn(hz, r.rz, r.cz);
    float tin = fmaxf(fmaxf(fminf(x1, x2), fminf(y1, y2)), fmaxf(fminf(z1, z2), -1e18f));
    float tout = fminf(fminf(fmaxf(x1, x2), fmaxf(y1, y2)), fminf(fmaxf(z1, z2), 1e18f));
    t_entry = tin;
    return tin <= tout && tout >= 0.0f;
}

// box_test_plain with the pruning limit folded in: the box is kept when
// max(entry, 0) <= min(exit, lim), which for 0 <= lim <= 1e18 is
// box_test_plain's acceptance together with entry <= lim. t_entry receives
// max(entry, 0); only the visiting order of boxes that hold the origin sees
// the difference.
__device__ __forceinline__ bool box_test_clip(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz,
                                              float lim, float& t_entry) {
    float x1 = __fmaf_rn(lx, r.rx, r.cx), x2 = __fmaf_rn(hx, r.rx, r.cx);
    float y1 = __fmaf_rn(ly, r.ry, r.cy), y2 = __fmaf_rn(hy, r.ry, r.cy);
    float z1 = __fmaf_rn(lz, r.rz, r.cz), z2 = __fmaf_rn(hz, r.rz, r.cz);
    float tin = fmaxf(fmaxf(fminf(x1, x2), fminf(y1, y2)), fmaxf(fminf(z1, z2), 0.0f));
    float tout = fminf(fminf(fmaxf(x1, x2), fmaxf(y1, y2)), fminf(fmaxf(z1, z2), lim));
    t_entry = tin;
    return tin <= tout;
}

// Box test of traversal mode MODE: 0 the reference's exact arithmetic, 1 the
// one-FMA test with its error margin and exact fallback (the same answers),
// 2 box_test_plain on the widened boxes.
template <int MODE>
__device__ __forceinline__ bool box_test_mode(const SlabRay& r, float lx, float hx, float ly, float hy, float lz, float hz,
                                              float& t_entry) {
    if (MODE == 0) return box_test(r, lx, hx, ly, hy, lz, hz, t_entry);
    if (MODE == 1) return box_test_fast(r, lx, hx, ly, hy, lz, hz, t_entry);
    return box_test_plain(r, lx, hx, ly, hy, lz, hz, t_entry);
}

// Triangle::intersection (src/scene/triangle.cpp:27-33) followed by the leaf
// acceptance test of BVHNode::getIntersection (src/hierarchy/bvhnode.cpp:55-63):
// t < limit && t > 0 && b1 >= 0 && b2 >= 0 && b1 + b2 <= 1.
__device__ __forceinline__ bool tri_test(f3 o, f3 d, float4 g0, float4 g1, float4 g2, float limit, float& t, float& b1,
                                         float& b2) {
    f3 p0 = xyz(g0), e1 = xyz(g1), e2 = xyz(g2);
    f3 s = rsub3(o, p0);
    f3 s1 = rcross(d, e2);
    f3 s2 = rcross(s, e1);
    float tt = rdot(s2, e2);
    float q = add_1e6(rdot(s1, e1));
    // t = tt / q > 0 needs equal signs and tt != 0; anything else is rejected.
    if (tt == 0.0f || ((__float_as_uint(tt) ^ __float_as_uint(q)) & 0x80000000u)) return false;
    float rq = __frcp_rn(q);
    t = qdiv(tt, q, rq);
    if (!(t < limit && t > 0.0f)) return false;
    b1 = qdiv(rdot(s1, s), q, rq);
    b2 = qdiv(rdot(s2, d), q, rq);
    return b1 >= 0.0f && b2 >= 0.0f && __fadd_rn(b1, b2) <= 1.0f;
}

// tri_test with an approximate reciprocal of q: the decision is taken from
// quotients within 2^-21 of the exact ones when every comparison clears that
// margin, and recomputed with the exact division otherwise, so the accepted
// set and the returned t, b1, b2 equal tri_test's.
__device__ __forceinline__ bool tri_test_fast(f3 o, f3 d, float4 g0, float4 g1, float4 g2, float limit, float& t,
                                              float& b1, float& b2) {
    f3 p0 = xyz(g0), e1 = xyz(g1), e2 = xyz(g2);
    const float e = 1e-6f, tiny = 1e-30f;
    // The rejections in the order of what they need, so a miss on the first
    // barycentric skips the second cross product: the same rejections as the
    // exact test's, all of them checked before a hit is kept (1M-triangle
    // frame: 706.1 -> 717.1 Mpaths/s against computing all before rejecting).
    f3 s1 = rcross(d, e2);
    float q = add_1e6(rdot(s1, e1));
    f3 s = rsub3(o, p0);
    float u = rdot(s1, s);
    // quotients from an approximate reciprocal (2 ulp): within 2^-21 of the exact ones
    float rq = __fdividef(1.0f, q);
    float ua = u * rq;
    // with va >= -tiny, ua > 1 + 2e already puts the rounded ua + va above 1 + 2e
    if (ua < -tiny || ua > 1.0f + 2.0f * e) return false;
    f3 s2 = rcross(s, e1);
    float v = rdot(s2, d);
    float va = v * rq;
    if (va < -tiny || ua + va > 1.0f + 2.0f * e) return false;
    float tt = rdot(s2, e2);
    // t = tt / q > 0 needs equal signs and tt != 0 (exact)
    if (tt == 0.0f || ((__float_as_uint(tt) ^ __float_as_uint(q)) & 0x80000000u)) return false;
    float ta = tt * rq;
    if (ta > limit * (1.0f + e)) return false;
    float rqe = __frcp_rn(q);
    if (ta < limit * (1.0f - e) && ta > tiny && ua > tiny && va > tiny && ua + va < 1.0f - 2.0f * e) {
        t = qdiv(tt, q, rqe);
        b1 = qdiv(u, q, rqe);
        b2 = qdiv(v, q, rqe);
        return true;
    }
    // close to an edge, the far limit or zero: decide with the exact quotients
    t = qdiv(tt, q, rqe);
    if (!(t < limit && t > 0.0f)) return false;
    b1 = qdiv(u, q, rqe);
    b2 = qdiv(v, q, rqe);
    return b1 >= 0.0f && b2 >= 0.0f && __fadd_rn(b1, b2) <= 1.0f;
}

// Pruning: a subtree whose entry distance exceeds the best hit so far (or a
// shadow ray's limit) times S.prune_k is skipped; the reference prunes
// nothing (src/hierarchy/bvh.cpp:116-117). The default factor is
// 1 + NR_PRUNE_MARGIN. The reference's biased determinant (q + 1e-6,
// src/scene/triangle.cpp:31) reports t' = t q / (q + 1e-6) and accepts the
// triangle scaled about p0 by (q + 1e-6) / q, so a triangle crossed at a
// grazing angle (0 < q < 1e-6 / margin, or |q| < 1e-6) can report a t
// below its box's entry distance, even below the best hit of another
// subtree; no bound from the boxes excludes it. Such rays need the plane
// of a triangle to hold the ray to about 1e-6 of its length; prune=0
// (S.prune_k = infinity) visits every node whose box the ray enters, as
// the reference does, and returns the reference's hits for them too.
// LightSampler::sampleLight (src/sampler/lightsampler.cpp:56): the first
// emitter whose CDF entry is >= r (lower_bound), or the last one. The guide
// table narrows the search to the emitters between the lower bounds of
// floor(r K) / K and (floor(r K) + 1) / K, which enclose the answer.
__device__ __forceinline__ int pick_light(const DeviceScene& S, float r) {
    const int k = S.light_guide_k;
    int b = (int)(r * (float)k);
    b = b < 0 ? 0 : (b > k - 1 ? k - 1 : b);
    int lo = __ldg(&S.light_guide[b]), hi = __ldg(&S.light_guide[b + 1]);
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&S.light_cdf[mid]) < r) lo = mid + 1; else hi = mid;
    }
    return lo < S.num_lights ? lo : S.num_lights - 1;
}

#define NR_STACK NR_STACK_LIMIT

// Closest hit with the reference's exhaustive semantics (BVH::_traversal,
// src/hierarchy/bvh.cpp:99-127): the minimum t over reachable triangles;
// equal t resolved towards the later leaf in depth-first order (the
// reference keeps the right subtree unless the left is strictly nearer) and,
// within a leaf, towards the earlier triangle. Visits children near-first
// and prunes with the margin above. Returns the flattened triangle index or
// -1; err is set on a stack overflow.
template <bool FAST = true>
__device__ __forceinline__ int closest_hit(const DeviceScene& S, f3 o, f3 d, float& best_t, float& best_b1,
                                           float& best_b2, uint32_t* err, uint32_t* nodes_visited = nullptr,
                                           uint32_t* tris_tested = nullptr) {
    best_t = 1e18f; best_b1 = 0.f; best_b2 = 0.f;
    int best = -1, best_leaf = -1;
    if (S.root_ref == INT32_MIN) return -1;
    SlabRay R = make_slab_ray(o, d);
    float te;
    if (!box_test(R, S.root_lo[0], S.root_hi[0], S.root_lo[1], S.root_hi[1], S.root_lo[2], S.root_hi[2], te)) return -1;
    // (subtree reference, entry distance) pairs: one 8-byte local access per push / pop
    int2 stack[NR_STACK];
    int sp = 0;
    int ref = S.root_ref;
    uint32_t nv = 0, nt = 0;
    // every node is entered at most once per ray; the cap only guards against
    // a corrupted node array
    int budget = 2 * S.num_nodes + 8;
    while (true) {
        if (--budget < 0) { atomicOr(err, 2u); break; }
        if (ref >= 0) {
            const GpuNode& N = S.nodes[ref];
            float4 a = __ldg(&N.a), b = __ldg(&N.b), c = __ldg(&N.c);
            int4 k = __ldg(&N.d);
            ++nv;
            float t0, t1;
            bool h0 = FAST ? box_test_fast(R, a.x, a.y, a.z, a.w, c.x, c.y, t0) : box_test(R, a.x, a.y, a.z, a.w, c.x, c.y, t0);
            bool h1 = FAST ? box_test_fast(R, b.x, b.y, b.z, b.w, c.z, c.w, t1) : box_test(R, b.x, b.y, b.z, b.w, c.z, c.w, t1);
            float lim = best_t * S.prune_k;
            h0 = h0 && t0 <= lim;
            h1 = h1 && t1 <= lim;
            if (h0 && h1) {
                int nr = k.x, fr = k.y;
                float ft = t1;
                if (t1 < t0) { nr = k.y; fr = k.x; ft = t0; }
                if (sp >= NR_STACK) { atomicOr(err, 1u); break; }
                stack[sp] = make_int2(fr, __float_as_int(ft)); ++sp;
                ref = nr;
                continue;
            }
            if (h0) { ref = k.x; continue; }
            if (h1) { ref = k.y; continue; }
        } else {
            int first = leaf_first(ref), cnt = leaf_count(ref);
            float lt = 1e18f;
            int li = -1;
            for (int i = 0; i < cnt; ++i) {
                int ti = first + i;
                float4 g0 = __ldg(&S.tri_geo[3 * ti]), g1 = __ldg(&S.tri_geo[3 * ti + 1]), g2 = __ldg(&S.tri_geo[3 * ti + 2]);
                ++nt;
                float t, u, v;
                if (FAST ? tri_test_fast(o, d, g0, g1, g2, lt, t, u, v) : tri_test(o, d, g0, g1, g2, lt, t, u, v)) {
                    lt = t; li = ti;
                }
            }
            if (li >= 0 && (lt < best_t || (lt == best_t && first > best_leaf))) {
                best_t = lt; best = li; best_leaf = first;
            }
        }
        // pop the next subtree that can still hold a hit
        bool found = false;
        while (sp > 0) {
            --sp;
            const int2 e = stack[sp];
            if (__int_as_float(e.y) <= best_t * S.prune_k) { ref = e.x; found = true; break; }
        }
        if (!found) break;
    }
    if (nodes_visited) *nodes_visited += nv;
    if (tris_tested) *tris_tested += nt;
    if (best >= 0) {
        // barycentrics of the winner, recomputed rather than carried through
        // the loop (fewer live registers): both tests return the correctly
        // rounded quotients, so these equal the values found in the leaf
        float4 g0 = __ldg(&S.tri_geo[3 * best]), g1 = __ldg(&S.tri_geo[3 * best + 1]), g2 = __ldg(&S.tri_geo[3 * best + 2]);
        float t;
        tri_test(o, d, g0, g1, g2, 3.0e38f, t, best_b1, best_b2);
    }
    return best;
}

// Shadow query: true when some reachable triangle has a reference hit with
// t <= tmax (the complement of `t + 2e-3 > |light_vec|` of
// src/renderer/rendererptls.cpp:71 for the closest hit).
// While-while traversal with postponed leaves (Aila and Laine, "Understanding
// the efficiency of ray traversal on GPUs", HPG 2009): a lane that reaches a
// leaf keeps it aside and goes on through inner nodes until every active lane
// of its warp holds a leaf; then the warp tests leaves together. Same hits as
// closest_hit: the winner is the minimum t, ties to the larger leaf start and
// then the earlier triangle of the leaf, whatever the visiting order, and a
// subtree is only skipped when its entry distance exceeds the pruning limit
// of the best hit so far, which never undercuts the final one.
// Refs: inner nodes >= 0, leaves < 0; NR_TRAV_END (no node) ends the walk.
#define NR_TRAV_END 0x7fffffff

// Traversal stacks. The default keeps every entry in per-thread local
// memory (L1-resident). With K > 0 the top K entries of each thread live in
// a shared-memory ring (entry i at ring[(i % K) * blockDim.x]: threads of a
// warp in adjacent banks) and only deeper entries go to local memory, moved
// there when the ring is full and back when it drains.
template <class E, int K>
struct TravStack {
    E spill[NR_STACK];
    E* ring;  // this thread's column of the block's ring, or null
    int sp = 0;
    __device__ __forceinline__ void init(E* block_ring) { ring = block_ring ? block_ring + threadIdx.x : nullptr; }
    __device__ __forceinline__ bool full() const { return sp >= NR_STACK; }
    __device__ __forceinline__ bool empty() const { return sp == 0; }
    __device__ __forceinline__ void push(E e) {
        if (K == 0) { spill[sp++] = e; return; }
        E* slot = ring + (sp & (K - 1)) * blockDim.x;
        if (sp >= K) spill[sp - K] = *slot;  // the entry K below the top leaves the ring
        *slot = e;
        ++sp;
    }
    __device__ __forceinline__ E pop() {
        --sp;
        if (K == 0) return spill[sp];
        E* slot = ring + (sp & (K - 1)) * blockDim.x;
        const E e = *slot;
        if (sp >= K) *slot = spill[sp - K];  // the entry K below comes back into the ring
        return e;
    }
};

// MODE 2 takes box_test_clip with the pruning limit folded into the slab
// test (1M-triangle frame: 876.0 against 863.2 Mpaths/s with the limit
// compared apart; keeping the limit in a register updated with each new best
// hit instead of recomputing it per node spills: 736).
template <int MODE, bool SPEC = true, int K = 0>
__device__ __forceinline__ int closest_hit_ww(const DeviceScene& S, f3 o, f3 d, float& best_t, float& best_b1,
                                              float& best_b2, uint32_t* err, uint32_t* nodes_visited = nullptr,
                                              uint32_t* tris_tested = nullptr, int2* ring = nullptr) {
    best_t = 1e18f; best_b1 = 0.f; best_b2 = 0.f;
    int best = -1, best_leaf = -1;
    if (S.root_ref == INT32_MIN) return -1;
    SlabRay R = make_slab_ray(o, d);
    float te;
    if (!box_test(R, S.root_lo[0], S.root_hi[0], S.root_lo[1], S.root_hi[1], S.root_lo[2], S.root_hi[2], te)) return -1;
    TravStack<int2, K> stack;
    stack.init(ring);
    int ref = S.root_ref;
    int leaf = 0;  // postponed leaf (< 0), or none (>= 0)
    uint32_t nv = 0, nt = 0;
    // No step budget and no stack-full test here: the host accepts only
    // trees in which every inner node has at most one parent, of a smaller
    // index, and whose depth leaves the stack room (upload_scene and
    // finish_scene), so a walk visits each node at most once and its stack
    // holds at most one entry per level. 1M-triangle frame with the folded
    // slab test: 876.0 Mpaths/s with the two tests, 897.7 without them here,
    // 893.0 without them in the any-hit walk as well (which keeps them).
    // the next stacked subtree that can still hold a hit, or NR_TRAV_END
    auto pop = [&]() {
        while (!stack.empty()) {
            const int2 e = stack.pop();
            if (__int_as_float(e.y) <= best_t * S.prune_k) return e.x;
        }
        return (int)NR_TRAV_END;
    };
    while (ref != NR_TRAV_END) {
        while ((unsigned)ref < (unsigned)NR_TRAV_END) {
            const GpuNode& N = (MODE == 2 ? S.nodes_fast : S.nodes)[ref];
            float4 a = __ldg(&N.a), b = __ldg(&N.b), c = __ldg(&N.c);
            int4 k = __ldg(&N.d);
            ++nv;
            float t0, t1;
            bool h0, h1;
            if (MODE == 2) {
                const float lim = fminf(best_t * S.prune_k, 1e18f);
                h0 = box_test_clip(R, a.x, a.y, a.z, a.w, c.x, c.y, lim, t0);
                h1 = box_test_clip(R, b.x, b.y, b.z, b.w, c.z, c.w, lim, t1);
            } else {
                h0 = box_test_mode<MODE>(R, a.x, a.y, a.z, a.w, c.x, c.y, t0);
                h1 = box_test_mode<MODE>(R, b.x, b.y, b.z, b.w, c.z, c.w, t1);
                const float lim = best_t * S.prune_k;
                h0 = h0 && t0 <= lim;
                h1 = h1 && t1 <= lim;
            }
            if (h0 && h1) {
                int nr = k.x, fr = k.y;
                float ft = t1;
                if (t1 < t0) { nr = k.y; fr = k.x; ft = t0; }
                stack.push(make_int2(fr, __float_as_int(ft)));
                ref = nr;
            } else if (h0) {
                ref = k.x;
            } else if (h1) {
                ref = k.y;
            } else {
                ref = pop();
            }
            if (SPEC) {
                if (ref < 0 && leaf >= 0) {  // first leaf: keep it aside, go on
                    leaf = ref;
                    ref = pop();
                }
                if (!__any_sync(__activemask(), leaf >= 0)) break;
            }
        }
        if (!SPEC && ref < 0) {
            leaf = ref;
            ref = pop();
        }
        while (leaf < 0) {
            int first = leaf_first(leaf), cnt = leaf_count(leaf);
            float lt = 1e18f;
            int li = -1;
            for (int i = 0; i < cnt; ++i) {
                int ti = first + i;
                float4 g0 = __ldg(&S.tri_geo[3 * ti]), g1 = __ldg(&S.tri_geo[3 * ti + 1]), g2 = __ldg(&S.tri_geo[3 * ti + 2]);
                ++nt;
                float t, u, v;
                // t < lt within the leaf, and t <= best_t (a tie with the best
                // so far still decides by leaf order): the next float above
                // best_t as the limit rejects farther hits before the exact
                // quotients (770.9 -> 772.8 Mpaths/s)
                const float cap = fminf(lt, __uint_as_float(__float_as_uint(best_t) + 1u));
                if (MODE ? tri_test_fast(o, d, g0, g1, g2, cap, t, u, v) : tri_test(o, d, g0, g1, g2, cap, t, u, v)) {
                    lt = t; li = ti;
                }
            }
            if (li >= 0 && (lt < best_t || (lt == best_t && first > best_leaf))) {
                best_t = lt; best = li; best_leaf = first;
            }
            // a second leaf reached while this one waited goes next
            leaf = ref;
            if (ref < 0) ref = pop();
        }
    }
    if (nodes_visited) *nodes_visited += nv;
    if (tris_tested) *tris_tested += nt;
    if (best >= 0) {
        float4 g0 = __ldg(&S.tri_geo[3 * best]), g1 = __ldg(&S.tri_geo[3 * best + 1]), g2 = __ldg(&S.tri_geo[3 * best + 2]);
        float t;
        tri_test(o, d, g0, g1, g2, 3.0e38f, t, best_b1, best_b2);
    }
    return best;
}

// Any hit with t <= tmax, traversed as closest_hit_ww (SPEC), or while-while
// without postponing: a lane's inner-node loop ends at its first leaf.
template <int MODE, bool SPEC, int K = 0>
__device__ __forceinline__ bool any_hit_ww(const DeviceScene& S, f3 o, f3 d, float tmax, uint32_t* err,
                                           uint32_t* nodes_visited = nullptr, uint32_t* tris_tested = nullptr,
                                           int* ring = nullptr) {
    if (S.root_ref == INT32_MIN) return false;
    SlabRay R = make_slab_ray(o, d);
    float te;
    if (!box_test(R, S.root_lo[0], S.root_hi[0], S.root_lo[1], S.root_hi[1], S.root_lo[2], S.root_hi[2], te)) return false;
    const float lim = tmax * S.prune_k;
    const float lim_clip = fminf(lim, 1e18f);
    TravStack<int, K> stack;
    stack.init(ring);
    int ref = S.root_ref;
    int leaf = 0;
    const float limit = fminf(1e18f, __uint_as_float(__float_as_uint(tmax) + 1u));  // accepts t <= tmax
    int budget = 2 * S.num_nodes + 8;
    while (ref != NR_TRAV_END) {
        while ((unsigned)ref < (unsigned)NR_TRAV_END) {
            if (--budget < 0) { atomicOr(err, 2u); return false; }
            const GpuNode& N = (MODE == 2 ? S.nodes_fast : S.nodes)[ref];
            float4 a = __ldg(&N.a), b = __ldg(&N.b), c = __ldg(&N.c);
            int4 k = __ldg(&N.d);
            if (nodes_visited) ++*nodes_visited;
            float t0, t1;
            bool h0, h1;
            if (MODE == 2) {
                h0 = box_test_clip(R, a.x, a.y, a.z, a.w, c.x, c.y, lim_clip, t0);
                h1 = box_test_clip(R, b.x, b.y, b.z, b.w, c.z, c.w, lim_clip, t1);
            } else {
                h0 = box_test_mode<MODE>(R, a.x, a.y, a.z, a.w, c.x, c.y, t0) && t0 <= lim;
                h1 = box_test_mode<MODE>(R, b.x, b.y, b.z, b.w, c.z, c.w, t1) && t1 <= lim;
            }
            if (h0 && h1) {
                int nr = k.x, fr = k.y;
                // far child first: the near one holds the surface the shadow
                // ray leaves and its neighbours, which seldom occlude it
                // (1M-triangle frame: 722.5 Mpaths/s near first, 759.8 far first)
                if (t1 > t0) { nr = k.y; fr = k.x; }
                if (stack.full()) { atomicOr(err, 1u); return false; }
                stack.push(fr);
                ref = nr;
            } else if (h0) {
                ref = k.x;
            } else if (h1) {
                ref = k.y;
            } else {
                ref = stack.empty() ? NR_TRAV_END : stack.pop();
            }
            if (SPEC) {
                if (ref < 0 && leaf >= 0) {
                    leaf = ref;
                    ref = stack.empty() ? NR_TRAV_END : stack.pop();
                }
                if (!__any_sync(__activemask(), leaf >= 0)) break;
            }
        }
        if (!SPEC && ref < 0) {  // the leaf reached: tested at once
            leaf = ref;
            ref = stack.empty() ? NR_TRAV_END : stack.pop();
        }
        while (leaf < 0) {
            int first = leaf_first(leaf), cnt = leaf_count(leaf);
            for (int i = 0; i < cnt; ++i) {
                int ti = first + i;
                float4 g0 = __ldg(&S.tri_geo[3 * ti]), g1 = __ldg(&S.tri_geo[3 * ti + 1]), g2 = __ldg(&S.tri_geo[3 * ti + 2]);
                if (tris_tested) ++*tris_tested;
                float t, u, v;
                if (MODE ? tri_test_fast(o, d, g0, g1, g2, limit, t, u, v) : tri_test(o, d, g0, g1, g2, limit, t, u, v)) return true;
            }
            leaf = ref;
            if (ref < 0) ref = stack.empty() ? NR_TRAV_END : stack.pop();
        }
    }
    return false;
}

template <bool FAST = true>
__device__ __forceinline__ bool any_hit(const DeviceScene& S, f3 o, f3 d, float tmax, uint32_t* err,
                                        uint32_t* nodes_visited = nullptr, uint32_t* tris_tested = nullptr) {
    if (S.root_ref == INT32_MIN) return false;
    SlabRay R = make_slab_ray(o, d);
    float te;
    if (!box_test(R, S.root_lo[0], S.root_hi[0], S.root_lo[1], S.root_hi[1], S.root_lo[2], S.root_hi[2], te)) return false;
    const float lim = tmax * S.prune_k;
    int stack[NR_STACK];
    int sp = 0;
    int ref = S.root_ref;
    const float limit = fminf(1e18f, __uint_as_float(__float_as_uint(tmax) + 1u));  // accepts t <= tmax
    int budget = 2 * S.num_nodes + 8;
    while (true) {
        if (--budget < 0) { atomicOr(err, 2u); return false; }
        if (ref >= 0) {
            const GpuNode& N = S.nodes[ref];
            float4 a = __ldg(&N.a), b = __ldg(&N.b), c = __ldg(&N.c);
            int4 k = __ldg(&N.d);
            if (nodes_visited) ++*nodes_visited;
            float t0, t1;
            bool h0 = (FAST ? box_test_fast(R, a.x, a.y, a.z, a.w, c.x, c.y, t0) : box_test(R, a.x, a.y, a.z, a.w, c.x, c.y, t0)) && t0 <= lim;
            bool h1 = (FAST ? box_test_fast(R, b.x, b.y, b.z, b.w, c.z, c.w, t1) : box_test(R, b.x, b.y, b.z, b.w, c.z, c.w, t1)) && t1 <= lim;
            if (h0 && h1) {
                int nr = k.x, fr = k.y;
                if (t1 < t0) { nr = k.y; fr = k.x; }
                if (sp >= NR_STACK) { atomicOr(err, 1u); return false; }
                stack[sp++] = fr;
                ref = nr;
                continue;
            }
            if (h0) { ref = k.x; continue; }
            if (h1) { ref = k.y; continue; }
        } else {
            int first = leaf_first(ref), cnt = leaf_count(ref);
            for (int i = 0; i < cnt; ++i) {
                int ti = first + i;
                float4 g0 = __ldg(&S.tri_geo[3 * ti]), g1 = __ldg(&S.tri_geo[3 * ti + 1]), g2 = __ldg(&S.tri_geo[3 * ti + 2]);
                if (tris_tested) ++*tris_tested;
                float t, u, v;
                if (FAST ? tri_test_fast(o, d, g0, g1, g2, limit, t, u, v) : tri_test(o, d, g0, g1, g2, limit, t, u, v)) return true;
            }
        }
        if (sp == 0) break;
        ref = stack[--sp];
    }
    return false;
}

}  // namespace nr
