// Path-replay adjoint of the ptnee estimator: d(loss)/d(per-material albedo,
// roughness, emission) for a loss whose image gradient dL/dI the caller
// provides. No per-vertex tape is kept: each path is traced twice from its
// Philox key (pixel, sample). Pass 1 yields the path radiance L; pass 2
// replays the same path and, at every factor that depends on a parameter,
// adds delta . (d factor / d theta) . (radiance that factor multiplies), where
// delta = dL/dI[pixel] / spp on the channels with L > 0 (the per-sample
// max(0, .) of src/renderer/rendererptls.cpp:173) and the radiance after a
// vertex is L minus what was accumulated before it (path replay
// backpropagation, Vicini, Speierer and Jakob, SIGGRAPH 2021).
//
// Derivative terms (the estimator of RendererPTLS::trace, rendererptls.cpp:13-94):
//  * albedo: f is affine in each channel of Kd (Lambert, GGXRefl F0, GGX F0,
//    BlinnPhong Kd, glass F0), so d f_c / d Kd_c = f_c(Kd + 1) - f_c(Kd)
//    exactly. Textured albedo has no gradient.
//  * roughness: the sampled directions are held fixed (detached sampling:
//    the 1/pdf of the sampling density is not differentiated, which keeps
//    the estimator of d E[L] / d alpha unbiased); d f / d alpha and the
//    derivative of the MIS weight through the BSDF pdf, including the
//    (1 - mis) factor that weights the next emitter hit, use central
//    differences of the device BSDF in alpha.
//  * emission: linear; d/dKe of an emitter hit is T * fac, of an NEE term
//    T * f * cos * mis / |lv|^2 * cos_l / p_light.
#include "nr_material.cuh"
#include "adjoint.h"

namespace nr {

namespace {

struct GradAcc {
    float* g;  // shared memory, num_mats * 7
    __device__ void add(int m, int k, float v) {
        if (v != 0.f) atomicAdd(&g[m * 7 + k], v);
    }
};

__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// Material calls out of line: the two replays call them at about twenty
// sites, and inlining every copy of the six-material code made the kernel
// front-end bound (ncu: "no instruction" stalls led, 151 registers).
#ifndef NR_ADJ_NOINLINE
#define NR_ADJ_NOINLINE 1
#endif
#if NR_ADJ_NOINLINE
__device__ __noinline__ f3 adj_bxdf(const MatView& M, f3 wo, f3 n, f3 wi) { return mat_bxdf(M, wo, n, wi); }
__device__ __noinline__ float adj_pdf(const MatView& M, f3 wo, f3 n, f3 wi) { return mat_pdf(M, wo, n, wi); }
__device__ __noinline__ f3 adj_sample(const MatView& M, Stream& rng, f3 wo, f3 n) { return mat_sample(M, rng, wo, n); }
#else
__device__ __forceinline__ f3 adj_bxdf(const MatView& M, f3 wo, f3 n, f3 wi) { return mat_bxdf(M, wo, n, wi); }
__device__ __forceinline__ float adj_pdf(const MatView& M, f3 wo, f3 n, f3 wi) { return mat_pdf(M, wo, n, wi); }
__device__ __forceinline__ f3 adj_sample(const MatView& M, Stream& rng, f3 wo, f3 n) { return mat_sample(M, rng, wo, n); }
#endif

// d f / d Kd per channel (f is affine in Kd).
__device__ __forceinline__ f3 df_dkd(const MatView& M, f3 wo, f3 n, f3 wi, f3 f0) {
    MatView P = M;
    P.c0 = M.c0 + mk(1.f);
    return adj_bxdf(P, wo, n, wi) - f0;
}

__device__ __forceinline__ bool has_alpha(const MatView& M) { return M.type == NR_MAT_GGXR || M.type == NR_MAT_GGX; }

__device__ __forceinline__ float alpha_step(float a) { return fmaxf(1e-3f * a, 1e-5f); }

__device__ __forceinline__ f3 df_dalpha(const MatView& M, f3 wo, f3 n, f3 wi) {
    MatView P = M, Q = M;
    float h = alpha_step(M.alpha);
    P.alpha = M.alpha + h;
    Q.alpha = M.alpha - h;
    return (adj_bxdf(P, wo, n, wi) - adj_bxdf(Q, wo, n, wi)) / (2.f * h);
}

__device__ __forceinline__ float dpdf_dalpha(const MatView& M, f3 wo, f3 n, f3 wi) {
    MatView P = M, Q = M;
    float h = alpha_step(M.alpha);
    P.alpha = M.alpha + h;
    Q.alpha = M.alpha - h;
    float a = adj_pdf(P, wo, n, wi), b = adj_pdf(Q, wo, n, wi);
    if (a >= 1e17f || b >= 1e17f) return 0.f;  // the pdf's 1e18 sentinel branch
    return (a - b) / (2.f * h);
}

// One path of the estimator. ADJ = false: returns its radiance. ADJ = true:
// replays it and accumulates the parameter gradient into acc.
template <bool ADJ>
__device__ f3 replay(const AdjArgs& A, uint32_t key, uint32_t sample, int x, int y, f3 Ltot, f3 delta, GradAcc acc) {
    const DeviceScene& S = A.S;
    const Policy& pol = A.pol;
    Stream rng;
    rng.init(pol.seed_lo, pol.seed_hi, key, sample, 0);
    float jx = rng.next();
    float jy = rng.next();
    f3 d = camera_ray(A.cam, A.film_h, (float)x + jx, (float)y + jy, (float)pol.imgw, (float)pol.imgh);
    f3 o = mk(A.cam.pos[0], A.cam.pos[1], A.cam.pos[2]);
    f3 T = mk(1.f), Lacc = mk(0.f);
    float fac = 1.f, dfac_da = 0.f;
    int prev_m = -1;
    uint32_t dummy_err = 0;
    for (int depth = 0;; ++depth) {
        float t, b1, b2;
        int tri = closest_hit(S, o, d, t, b1, b2, &dummy_err);
        if (tri < 0) {
            if (S.env_tex >= 0) Lacc = Lacc + T * env_lookup(S, d);
            break;
        }
        float4 s0 = __ldg(&S.tri_shade[4 * tri]), s1 = __ldg(&S.tri_shade[4 * tri + 1]);
        float4 s2 = __ldg(&S.tri_shade[4 * tri + 2]), s3 = __ldg(&S.tri_shade[4 * tri + 3]);
        const int m = __float_as_int(s3.w);
        float w0 = 1.0f - b1 - b2;
        f3 normal = normalized(w0 * xyz(s0) + b1 * xyz(s1) + b2 * xyz(s2));
        f3 wo = -d;
        const int type = S.mats[m].type;
        if (type == NR_MAT_LIGHT) {
            const nr_material& E = S.mats[m];
            f3 Ke = mk(E.c0[0], E.c0[1], E.c0[2]);
            if (ADJ) {
                f3 w = T * fac;
                acc.add(m, 4, delta.x * w.x);
                acc.add(m, 5, delta.y * w.y);
                acc.add(m, 6, delta.z * w.z);
                if (prev_m >= 0) acc.add(prev_m, 3, dot3(delta, T * Ke) * dfac_da);
            }
            Lacc = Lacc + T * Ke * fac;
            break;
        }
        if (dot(normal, d) > 0.f && !mat_transmissive(type)) break;
        f3 uv = mk(w0 * s0.w + b1 * s2.w + b2 * s3.y, w0 * s1.w + b1 * s3.x + b2 * s3.z, 0.f);
        MatView M = load_mat(S, m, uv);
        const bool textured = S.mats[m].tex0 >= 0;
        f3 hit_pos = o + d * t;
        fac = 1.f;
        dfac_da = 0.f;
        prev_m = m;
        if (pol.nee && mat_nee(type) && S.num_lights > 0) {
            const int li = pick_light(S, rng.next());
            const float4* L = S.lights + 6 * li;
            float4 l0 = __ldg(&L[0]), l1 = __ldg(&L[1]), l2 = __ldg(&L[2]);
            float4 n0 = __ldg(&L[3]), n1 = __ldg(&L[4]), n2 = __ldg(&L[5]);
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
            float lop = light_pdf * dot(light_vec, light_vec) / smax(1e-6f, cos_l);
            float bop = adj_pdf(M, wo, normal, wl);
            float mis = lop / (lop + bop);
            float dmis = 0.f;
            if (ADJ && pol.mis && has_alpha(M)) dmis = -lop / ((lop + bop) * (lop + bop)) * dpdf_dalpha(M, wo, normal, wl);
            if (!pol.mis) mis = 0.5f;
            fac = 1.0f - mis;
            dfac_da = -dmis;
            f3 fl = adj_bxdf(M, wo, normal, wl);
            float unit = 1.f / norm2(light_vec) * smax(0.f, cos_l) / light_pdf;
            f3 Ll = Ke * unit;
            float geo = smax(0.f, dot(normal, normalized(light_pos - hit_pos)));
            f3 c = T * (Ll * fl * geo * mis);
            // (pass 2 also needs visibility where c vanishes only through a zero albedo channel)
            if (c.x != 0.f || c.y != 0.f || c.z != 0.f || (ADJ && cos_l > 0.f && geo > 0.f && mis > 0.f)) {
                double lim = (double)norm(light_vec) - 2e-3;
                float tmax = lim > 0.0 ? __double2float_rd(lim) : 0.0f;
                bool visible = tmax <= 0.f || !any_hit(S, hit_pos + wl * 1e-3f, wl, tmax, &dummy_err);
                if (visible) {
                    if (ADJ) {
                        if (!textured) {
                            f3 dk = T * Ll * df_dkd(M, wo, normal, wl, fl) * (geo * mis);
                            acc.add(m, 0, delta.x * dk.x);
                            acc.add(m, 1, delta.y * dk.y);
                            acc.add(m, 2, delta.z * dk.z);
                        }
                        if (has_alpha(M)) {
                            f3 da = T * Ll * (df_dalpha(M, wo, normal, wl) * mis + fl * dmis) * geo;
                            acc.add(m, 3, dot3(delta, da));
                        }
                        // the light's emission, material of the emitter triangle
                        const int lm = __ldg(&S.light_mat[li]);
                        f3 de = T * fl * (unit * geo * mis);
                        acc.add(lm, 4, delta.x * de.x);
                        acc.add(lm, 5, delta.y * de.y);
                        acc.add(lm, 6, delta.z * de.z);
                    }
                    Lacc = Lacc + c;
                }
            }
        }
        if (pol.maxdepth > 0 && depth + 1 >= pol.maxdepth) break;
        float prr = depth < pol.rrdepth ? 1.0f : pol.prr;
        float u = rng.next();
        if (depth >= pol.rrdepth && u > prr) break;
        f3 wi = adj_sample(M, rng, wo, normal);
        float pdf = adj_pdf(M, wo, normal, wi);
        f3 f = adj_bxdf(M, wo, normal, wi);
        if (ADJ) {
            f3 after = Ltot - Lacc;  // radiance of the events this factor multiplies
            if (!textured) {
                f3 dk = df_dkd(M, wo, normal, wi, f);
                if (f.x != 0.f) acc.add(m, 0, delta.x * after.x * dk.x / f.x);
                if (f.y != 0.f) acc.add(m, 1, delta.y * after.y * dk.y / f.y);
                if (f.z != 0.f) acc.add(m, 2, delta.z * after.z * dk.z / f.z);
            }
            if (has_alpha(M)) {
                f3 da = df_dalpha(M, wo, normal, wi);
                float g = 0.f;
                if (f.x != 0.f) g += delta.x * after.x * da.x / f.x;
                if (f.y != 0.f) g += delta.y * after.y * da.y / f.y;
                if (f.z != 0.f) g += delta.z * after.z * da.z / f.z;
                acc.add(m, 3, g);
            }
        }
        T = T * fabsf(dot(wi, normal)) * f / pdf / prr;
        o = hit_pos + wi * 1e-3f;
        d = wi;
    }
    return Lacc;
}

// ------------------------------------------------------------ wavefront replay
// The same replay as replay<true>, spread over the wavefront: k_trace sorts
// the vertices by material, k_shade_adj shades them one thread per path, and
// k_shadow_adj resolves the light samples. Two terms move in time: a light
// sample's gradient is only known to count once its shadow ray is found
// unoccluded, so it rides with the shadow ray; and the gradient of a
// vertex's BSDF factor needs the radiance gathered after it (L minus the
// radiance so far, light samples included), so it is held per path and
// settled when the path's next vertex is shaded.

__device__ __forceinline__ int adj_append(bool want, uint32_t* counter) {
    unsigned active = __activemask();
    unsigned m = __ballot_sync(active, want);
    if (!want) return -1;
    int lane = threadIdx.x & 31, leader = __ffs(m) - 1, rank = __popc(m & ((1u << lane) - 1u));
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return (int)(base + rank);
}

__device__ void shade_adj(const PathState& P, const DeviceScene& S, const Policy& pol, const AdjWave& J,
                          const uint8_t* __restrict__ vis, int slot, GradAcc acc) {
    const float4 h = P.hit[slot], thr = P.thr[slot];
    const uint4 meta = P.meta[slot];
    const f3 dir = xyz(P.ray_d[slot]);
    const f3 T = xyz(thr);
    const f3 Ltot = xyz(J.L[slot]), delta = xyz(J.delta[slot]);
    const float4 pk = J.pk[slot], pa = J.pa[slot];
    const int pm = __float_as_int(pk.w);
    if (pm >= 0) {  // the previous vertex's BSDF factor multiplies all radiance from here on
        const f3 after = Ltot - xyz(P.rad[slot]);
        acc.add(pm, 0, pk.x * after.x);
        acc.add(pm, 1, pk.y * after.y);
        acc.add(pm, 2, pk.z * after.z);
        acc.add(pm, 3, pa.x * after.x + pa.y * after.y + pa.z * after.z);
    }
    const int tri = __float_as_int(h.w);
    if (tri < 0) return;
    const float b1 = h.y, b2 = h.z;
    const float4 s0 = __ldg(&S.tri_shade[4 * tri]), s1 = __ldg(&S.tri_shade[4 * tri + 1]);
    const float4 s2 = __ldg(&S.tri_shade[4 * tri + 2]), s3 = __ldg(&S.tri_shade[4 * tri + 3]);
    const int m = __float_as_int(s3.w);
    const float w0 = 1.0f - b1 - b2;
    const f3 normal = normalized(w0 * xyz(s0) + b1 * xyz(s1) + b2 * xyz(s2));
    const f3 wo = -dir;
    const int type = S.mats[m].type;
    if (type == NR_MAT_LIGHT) {
        const nr_material& E = S.mats[m];
        const f3 Ke = mk(E.c0[0], E.c0[1], E.c0[2]);
        const f3 w = T * thr.w;
        acc.add(m, 4, delta.x * w.x);
        acc.add(m, 5, delta.y * w.y);
        acc.add(m, 6, delta.z * w.z);
        if (pm >= 0) acc.add(pm, 3, dot3(delta, T * Ke) * pa.w);
        return;
    }
    if (dot(normal, dir) > 0.f && !mat_transmissive(type)) return;
    const f3 uv = mk(w0 * s0.w + b1 * s2.w + b2 * s3.y, w0 * s1.w + b1 * s3.x + b2 * s3.z, 0.f);
    const MatView M = load_mat(S, m, uv);
    const bool textured = S.mats[m].tex0 >= 0;
    const f3 hit_pos = xyz(P.ray_o[slot]) + dir * h.x;
    Stream rng;
    rng.init(pol.seed_lo, pol.seed_hi, meta.x, meta.y, meta.z);
    const int depth = (int)(meta.w & NR_META_DEPTH_MASK);
    float fac = 1.f, dfac_da = 0.f;
    if (pol.nee && mat_nee(type) && S.num_lights > 0) {
        const int li = pick_light(S, rng.next());
        const float4* Lt = S.lights + 6 * li;
        const float4 l0 = __ldg(&Lt[0]), l1 = __ldg(&Lt[1]), l2 = __ldg(&Lt[2]);
        const float4 n0 = __ldg(&Lt[3]), n1 = __ldg(&Lt[4]), n2 = __ldg(&Lt[5]);
        float r1 = rng.next();
        float r2 = rng.next();
        if (r1 + r2 > 1.f) { r1 = 1.f - r1; r2 = 1.f - r2; }
        const float lw = 1.f - r1 - r2;
        const f3 light_pos = lw * xyz(l0) + r1 * xyz(l1) + r2 * xyz(l2);
        const f3 light_normal = normalized(lw * xyz(n0) + r1 * xyz(n1) + r2 * xyz(n2));
        const f3 light_vec = light_pos - hit_pos;
        const f3 wl = normalized(light_vec);
        const f3 Ke = mk(l0.w, l1.w, l2.w);
        const float light_pdf = S.light_p;
        const float cos_l = dot(light_normal, -wl);
        const float lop = light_pdf * dot(light_vec, light_vec) / smax(1e-6f, cos_l);
        const float bop = adj_pdf(M, wo, normal, wl);
        float mis = lop / (lop + bop);
        float dmis = 0.f;
        if (pol.mis && has_alpha(M)) dmis = -lop / ((lop + bop) * (lop + bop)) * dpdf_dalpha(M, wo, normal, wl);
        if (!pol.mis) mis = 0.5f;
        fac = 1.0f - mis;
        dfac_da = -dmis;
        const f3 fl = adj_bxdf(M, wo, normal, wl);
        const float unit = 1.f / norm2(light_vec) * smax(0.f, cos_l) / light_pdf;
        const f3 Ll = Ke / norm2(light_vec) * smax(0.f, cos_l) / light_pdf;
        const float geo = smax(0.f, dot(normal, normalized(light_pos - hit_pos)));
        f3 c = Ll * fl * geo * mis;  // the renderer's expression order, so rad follows its L exactly
        c = c * T;
        // traced by the renderer's first pass under pol.adj, which recorded vis
        if (c.x != 0.f || c.y != 0.f || c.z != 0.f || (cos_l > 0.f && geo > 0.f && mis > 0.f)) {
            f3 gk = mk(0.f), ge;
            float ga = 0.f;
            if (!textured) gk = delta * (T * Ll * df_dkd(M, wo, normal, wl, fl) * (geo * mis));
            if (has_alpha(M)) ga = dot3(delta, T * Ll * (df_dalpha(M, wo, normal, wl) * mis + fl * dmis) * geo);
            ge = delta * (T * fl * (unit * geo * mis));
            const int lm = __ldg(&S.light_mat[li]);
            const double lim = (double)norm(light_vec) - 2e-3;
            const float tmax = lim > 0.0 ? __double2float_rd(lim) : 0.0f;
            if (tmax > 0.f && !vis) {
                const int q = adj_append(true, &P.counters[CNT_SHADOW]);
                if (q >= P.sh_cap) { atomicOr(&P.counters[CNT_ERR], 4u); return; }
                const f3 so = hit_pos + wl * 1e-3f;
                P.sh_o[q] = make_float4(so.x, so.y, so.z, tmax);
                P.sh_d[q] = make_float4(wl.x, wl.y, wl.z, __int_as_float(slot));
                P.sh_c[q] = make_float4(c.x, c.y, c.z, 0.f);
                J.sg0[q] = make_float4(gk.x, gk.y, gk.z, ga);
                J.sg1[q] = make_float4(ge.x, ge.y, ge.z, __int_as_float(m | (lm << 16)));
            } else if (tmax <= 0.f || vis[slot]) {  // recorded unoccluded, or nothing can occlude
                const float4 rr = P.rad[slot];
                P.rad[slot] = make_float4(rr.x + c.x, rr.y + c.y, rr.z + c.z, 0.f);
                acc.add(m, 0, gk.x); acc.add(m, 1, gk.y); acc.add(m, 2, gk.z); acc.add(m, 3, ga);
                acc.add(lm, 4, ge.x); acc.add(lm, 5, ge.y); acc.add(lm, 6, ge.z);
            }
        }
    }
    if (pol.maxdepth > 0 && depth + 1 >= pol.maxdepth) return;
    const float prr = depth < pol.rrdepth ? 1.0f : pol.prr;
    const float u = rng.next();
    if (depth >= pol.rrdepth && u > prr) return;
    const f3 wi = adj_sample(M, rng, wo, normal);
    const float pdf = adj_pdf(M, wo, normal, wi);
    const f3 f = adj_bxdf(M, wo, normal, wi);
    f3 gk = mk(0.f), gr = mk(0.f);
    if (!textured) {
        const f3 dk = df_dkd(M, wo, normal, wi, f);
        gk = mk(f.x != 0.f ? delta.x * dk.x / f.x : 0.f, f.y != 0.f ? delta.y * dk.y / f.y : 0.f,
                f.z != 0.f ? delta.z * dk.z / f.z : 0.f);
    }
    if (has_alpha(M)) {
        const f3 da = df_dalpha(M, wo, normal, wi);
        gr = mk(f.x != 0.f ? delta.x * da.x / f.x : 0.f, f.y != 0.f ? delta.y * da.y / f.y : 0.f,
                f.z != 0.f ? delta.z * da.z / f.z : 0.f);
    }
    J.pk[slot] = make_float4(gk.x, gk.y, gk.z, __int_as_float(m));
    J.pa[slot] = make_float4(gr.x, gr.y, gr.z, dfac_da);
    const f3 Tn = T * fabsf(dot(wi, normal)) * f / pdf / prr;
    const f3 no = hit_pos + wi * 1e-3f;
    const int q = adj_append(true, &P.counters[CNT_OUT]);
    P.queue_out[q] = slot;
    P.ray_o[slot] = make_float4(no.x, no.y, no.z, 0.f);
    P.ray_d[slot] = make_float4(wi.x, wi.y, wi.z, 0.f);
    P.thr[slot] = make_float4(Tn.x, Tn.y, Tn.z, fac);
    P.meta[slot] = make_uint4(meta.x, meta.y, rng.n, (uint32_t)(depth + 1));
}

}  // namespace

// Per wave, after ray generation: each path's radiance and gradient weight;
// paths whose gradient weight is zero are left out of the queue.
__global__ void k_adj_init(PathState P, AdjWave J, WaveDesc W, int imgw, int spp, const float* __restrict__ Lbuf,
                           const float* __restrict__ dldi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W.count) return;
    int x, y;
    uint32_t srel;
    wave_path(W, W.base + (uint64_t)i, imgw, x, y, srel);
    const uint64_t pidx = (uint64_t)y * (uint64_t)imgw + (uint64_t)x;
    const float* l = Lbuf + (pidx * (uint64_t)spp + srel) * 3;
    const float inv = 1.0f / (float)spp;
    const f3 d = mk(l[0] > 0.f ? dldi[3 * pidx] * inv : 0.f, l[1] > 0.f ? dldi[3 * pidx + 1] * inv : 0.f,
                    l[2] > 0.f ? dldi[3 * pidx + 2] * inv : 0.f);
    J.L[i] = make_float4(l[0], l[1], l[2], 0.f);
    J.delta[i] = make_float4(d.x, d.y, d.z, 0.f);
    J.pk[i] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    J.pa[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool live = d.x != 0.f || d.y != 0.f || d.z != 0.f;
    const int q = adj_append(live, &P.counters[CNT_WORK]);
    if (live) P.queue_in[q] = i;
}
__global__ void k_adj_setin(uint32_t* counters) {
    counters[CNT_IN] = counters[CNT_WORK];
    counters[CNT_WORK] = 0;
}

// 8 resident blocks per SM asked of the register allocator (64 registers,
// some spills, against 128 registers and 4 blocks uncapped): C5 552.1
// against 535.1 Mpaths/s on one box, 534.8 at 6.
#ifndef NR_ADJ_SHADE_MINB
#define NR_ADJ_SHADE_MINB 8
#endif
__global__ void __launch_bounds__(128, NR_ADJ_SHADE_MINB) k_shade_adj(PathState P, DeviceScene S, Policy pol, int capacity, AdjWave J,
                                                   const uint8_t* __restrict__ vis, float* __restrict__ grad) {
    extern __shared__ float sg[];
    const int NG = S.num_mats * 7;
    for (int i = threadIdx.x; i < NG; i += blockDim.x) sg[i] = 0.f;
    __syncthreads();
    GradAcc acc{sg};
    uint32_t cnt[NUM_CAT], start[NUM_CAT];
    uint32_t total = 0;
#pragma unroll
    for (int c = 0; c < NUM_CAT; ++c) { cnt[c] = P.counters[CNT_CAT + c]; start[c] = total; total += cnt[c]; }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        int c = 0;
#pragma unroll
        for (int k = 1; k < NUM_CAT; ++k) if (i >= start[k]) c = k;
        shade_adj(P, S, pol, J, vis, P.sorted[(size_t)c * capacity + (i - start[c])], acc);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NG; i += blockDim.x)
        if (sg[i] != 0.f) atomicAdd(&grad[i], sg[i]);
}

__global__ void __launch_bounds__(128) k_shadow_adj(PathState P, DeviceScene S, AdjWave J, float* __restrict__ grad) {
    extern __shared__ float sg[];
    const int NG = S.num_mats * 7;
    for (int i = threadIdx.x; i < NG; i += blockDim.x) sg[i] = 0.f;
    __syncthreads();
    GradAcc acc{sg};
    const uint32_t n = min(P.counters[CNT_SHADOW], (uint32_t)P.sh_cap);
    const int lane = threadIdx.x & 31;
    while (true) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(&P.counters[CNT_WORK_SH], 32u);
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b >= n) break;
        const uint32_t idx = b + lane;
        if (idx < n) {
            const float4 o = P.sh_o[idx], d = P.sh_d[idx];
            if (!any_hit_ww<true, false>(S, xyz(o), xyz(d), o.w, &P.counters[CNT_ERR])) {
                const int slot = __float_as_int(d.w);
                const float4 c = P.sh_c[idx], r = P.rad[slot];
                P.rad[slot] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.f);
                const float4 g0 = J.sg0[idx], g1 = J.sg1[idx];
                const int mm = __float_as_int(g1.w), m = mm & 0xffff, lm = mm >> 16;
                acc.add(m, 0, g0.x); acc.add(m, 1, g0.y); acc.add(m, 2, g0.z); acc.add(m, 3, g0.w);
                acc.add(lm, 4, g1.x); acc.add(lm, 5, g1.y); acc.add(lm, 6, g1.z);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NG; i += blockDim.x)
        if (sg[i] != 0.f) atomicAdd(&grad[i], sg[i]);
}

void launch_adj_init(const PathState& P, const AdjWave& J, const WaveDesc& W, int imgw, int spp, const float* Lbuf,
                     const float* dldi, cudaStream_t st) {
    k_adj_init<<<(W.count + 255) / 256, 256, 0, st>>>(P, J, W, imgw, spp, Lbuf, dldi);
    k_adj_setin<<<1, 1, 0, st>>>(P.counters);
}
int launch_adj_bounce_shading(const PathState& P, const DeviceScene& S, const Policy& pol, int capacity,
                              const AdjWave& J, const uint8_t* vis, float* grad, int num_sms, int shadow_blocks,
                              cudaStream_t st) {
    const size_t smem = (size_t)S.num_mats * 7 * sizeof(float);
    k_shade_adj<<<num_sms * 8, 128, smem, st>>>(P, S, pol, capacity, J, vis, grad);
    if (vis) return 1;
    k_shadow_adj<<<shadow_blocks, 128, smem, st>>>(P, S, J, grad);
    return 2;
}

// One thread per path: the adjoint replay, given each path's radiance L
// from the wavefront renderer (Lbuf[(pixel * spp + sample) * 3], max(0, L)
// per channel). Block-level gradient histogram in shared memory, flushed
// with one atomic per entry.
// 8 resident blocks per SM (64 registers, with spills): measured 62.7
// Mpaths/s on the 200k-triangle adjoint workload, against 56.7 at 6 blocks,
// 54.9 at 7, 50.8 at 4, 50.3 uncapped (123 registers) and 36.8 with the
// material code inlined.
#ifndef NR_ADJ_MINB
#define NR_ADJ_MINB 8
#endif
__global__ void __launch_bounds__(128, NR_ADJ_MINB) k_adjoint(AdjArgs A, const float* __restrict__ dldi, float* __restrict__ grad,
                                                 const float* __restrict__ Lbuf) {
    extern __shared__ float sg[];
    const int NG = A.S.num_mats * 7;
    for (int i = threadIdx.x; i < NG; i += blockDim.x) sg[i] = 0.f;
    __syncthreads();
    GradAcc acc{sg};
    const uint64_t total = (uint64_t)A.npix * (uint64_t)A.spp;
    const float inv_spp = 1.0f / (float)A.spp;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t pidx = (uint32_t)(g % (uint64_t)A.npix);
        uint32_t srel = (uint32_t)(g / (uint64_t)A.npix);
        int x = (int)(pidx % (uint32_t)A.pol.imgw), y = (int)(pidx / (uint32_t)A.pol.imgw);
        uint32_t key = (uint32_t)y * (uint32_t)A.pol.imgw + (uint32_t)x;
        uint32_t sample = A.sample0 + srel;
        const float* l = Lbuf + ((uint64_t)pidx * (uint64_t)A.spp + srel) * 3;
        const f3 L = mk(l[0], l[1], l[2]);
        f3 delta = mk(L.x > 0.f ? dldi[3 * pidx] * inv_spp : 0.f, L.y > 0.f ? dldi[3 * pidx + 1] * inv_spp : 0.f,
                      L.z > 0.f ? dldi[3 * pidx + 2] * inv_spp : 0.f);
        if (delta.x == 0.f && delta.y == 0.f && delta.z == 0.f) continue;
        replay<true>(A, key, sample, x, y, L, delta, acc);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < NG; i += blockDim.x)
        if (sg[i] != 0.f) atomicAdd(&grad[i], sg[i]);
}

// image_sum[pixel] = sum over its samples of max(0, L), in sample order.
__global__ void k_image_from_L(const float* __restrict__ Lbuf, int npix, int spp, float* __restrict__ image_sum) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    float a = 0.f, b = 0.f, c = 0.f;
    for (int s = 0; s < spp; ++s) {
        const float* l = Lbuf + ((size_t)p * spp + s) * 3;
        a += l[0]; b += l[1]; c += l[2];
    }
    image_sum[3 * p] = a; image_sum[3 * p + 1] = b; image_sum[3 * p + 2] = c;
}

void adjoint_setup() {
    cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_shade_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_shadow_adj, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

void launch_image_from_L(const float* Lbuf, int npix, int spp, float* image_sum, cudaStream_t st) {
    k_image_from_L<<<(npix + 255) / 256, 256, 0, st>>>(Lbuf, npix, spp, image_sum);
}

void launch_adjoint(const AdjArgs& A, const float* dldi, float* grad, const float* Lbuf, int num_sms, cudaStream_t st) {
    const uint64_t total = (uint64_t)A.npix * (uint64_t)A.spp;
    uint64_t blocks = (total + 127) / 128;
    uint64_t cap = (uint64_t)num_sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    size_t smem = (size_t)A.S.num_mats * 7 * sizeof(float);
    k_adjoint<<<(unsigned)blocks, 128, smem, st>>>(A, dldi, grad, Lbuf);
}

}  // namespace nr
