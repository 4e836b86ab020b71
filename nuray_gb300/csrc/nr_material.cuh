// Device versions of the reference materials, textures, camera and
// environment lookup used by the ptnee shading kernel. FP32 throughout; the
// reference evaluates some sub-expressions in double through C++ promotion
// (double literals, C libm calls on floats), which these restate in float.
#pragma once
#include <cuda_bf16.h>

#include "nr_device.cuh"
#include "nrc_encode.cuh"

namespace nr {

#define NR_PI_F 3.14159f    // the reference writes pi as 3.14159 everywhere
#define NR_INV_PI_F 0.318310155f  // 1.0 / 3.14159

// Texture::pixel (black outside), ::pixelBi and ::pixelUV
// (src/scene/texture.cpp:54-72): bilinear over integer texel corners,
// u wrapped, v flipped.
__device__ __forceinline__ f3 texel(const DeviceScene& S, int4 info, int x, int y) {
    if (x < 0 || y < 0 || x >= info.x || y >= info.y) return mk(0.f);
    float4 v = __ldg(&S.tex_texels[(size_t)info.z + (size_t)y * info.x + x]);
    return xyz(v);
}
__device__ __forceinline__ f3 tex_uv(const DeviceScene& S, int tex, float u, float v) {
    int4 info = __ldg(&S.tex_info[tex]);
    float fu = fmodf(fmodf(u, 1.0f) + 1.0f, 1.0f) * (float)info.x;
    float fv = fmodf(fmodf(1.0f - v, 1.0f) + 1.0f, 1.0f) * (float)info.y;
    int x0 = (int)floorf(fu), y0 = (int)floorf(fv);
    int x1 = x0 + 1, y1 = y0 + 1;
    float ax = fu - (float)x0, ay = fv - (float)y0, bx = (float)x1 - fu, by = (float)y1 - fv;
    return texel(S, info, x1, y1) * ax * ay + texel(S, info, x1, y0) * ax * by + texel(S, info, x0, y1) * bx * ay +
           texel(S, info, x0, y0) * bx * by;
}

// Environment lookup on a miss (src/renderer/rendererptls.cpp:24-26,
// src/scene/envmap.cpp:17-24).
__device__ __forceinline__ f3 env_lookup(const DeviceScene& S, f3 dir) {
    float v = 1.0f - acosf(dir.y) / NR_PI_F;
    float u = atan2f(dir.z, dir.x) / 2.0f / NR_PI_F + 0.5f;
    return tex_uv(S, S.env_tex, u, v) * S.env_gain;
}

// Environment light sampling (envis=1; no counterpart in the reference):
// a cell of the sampling table by its row and column CDFs, a uniform point
// in the cell, the direction env_lookup maps that point from, and the
// solid-angle density, table density * w * h / (2 pi^2 sin theta) (with
// the reference's pi of 3.14159, the one the lookup uses).
__device__ __forceinline__ int cdf_upper(const float* cdf, int n, float r) {  // first i with cdf[i] > r
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(&cdf[mid]) > r) hi = mid; else lo = mid + 1;
    }
    return lo < n ? lo : n - 1;
}
__device__ __forceinline__ bool env_sample(const DeviceScene& S, float r1, float r2, f3& dir, float& pdf) {
    const int4 info = __ldg(&S.tex_info[S.env_tex]);
    const int w = info.x, h = info.y;
    const int y = cdf_upper(S.env_row_cdf, h, r1);
    const float c0 = y ? __ldg(&S.env_row_cdf[y - 1]) : 0.f, c1 = __ldg(&S.env_row_cdf[y]);
    const float fy = fminf(fmaxf(c1 > c0 ? (r1 - c0) / (c1 - c0) : 0.5f, 0.f), 0.99999994f);
    const float* col = S.env_col_cdf + (size_t)y * w;
    const int x = cdf_upper(col, w, r2);
    const float d0 = x ? __ldg(&col[x - 1]) : 0.f, d1 = __ldg(&col[x]);
    const float fx = fminf(fmaxf(d1 > d0 ? (r2 - d0) / (d1 - d0) : 0.5f, 0.f), 0.99999994f);
    const float wt = __ldg(&S.env_weight[(size_t)y * w + x]);
    if (!(wt > 0.f) || !(S.env_total > 0.f)) return false;
    const float theta = ((float)y + fy) / (float)h * NR_PI_F;
    const float phi = (((float)x + fx) / (float)w - 0.5f) * 2.0f * NR_PI_F;
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    if (st < 1e-6f) return false;
    dir = mk(st * cp, ct, st * sp);
    pdf = wt / S.env_total * ((float)w * (float)h) / (2.0f * NR_PI_F * NR_PI_F * st);
    return true;
}
// Density env_sample gives a direction (0 outside the sampled domain).
__device__ __forceinline__ float env_pdf(const DeviceScene& S, f3 dir) {
    const int4 info = __ldg(&S.tex_info[S.env_tex]);
    const int w = info.x, h = info.y;
    const float theta = acosf(fminf(fmaxf(dir.y, -1.f), 1.f));
    const float fv = theta / NR_PI_F * (float)h;
    const float fu = (atan2f(dir.z, dir.x) / 2.0f / NR_PI_F + 0.5f) * (float)w;
    if (!(fv >= 0.f && fv < (float)h && fu >= 0.f && fu < (float)w)) return 0.f;
    const int y = (int)fv, x = (int)fu;
    const float st = sinf(theta);
    if (st < 1e-6f || !(S.env_total > 0.f)) return 0.f;
    return __ldg(&S.env_weight[(size_t)y * w + x]) / S.env_total * ((float)w * (float)h) /
           (2.0f * NR_PI_F * NR_PI_F * st);
}

struct MatView {
    int type;
    f3 c0, c1;
    float alpha, ior, ns;
};

__device__ __forceinline__ MatView load_mat(const DeviceScene& S, int m, f3 uv) {
    const nr_material& M = S.mats[m];
    MatView v;
    v.type = M.type;
    v.c0 = mk(M.c0[0], M.c0[1], M.c0[2]);
    v.c1 = mk(M.c1[0], M.c1[1], M.c1[2]);
    v.alpha = M.alpha; v.ior = M.ior; v.ns = M.ns;
    if (M.tex0 >= 0) v.c0 = tex_uv(S, M.tex0, uv.x, uv.y);
    if (M.tex1 >= 0) v.c1 = tex_uv(S, M.tex1, uv.x, uv.y);
    return v;
}

__device__ __forceinline__ bool mat_transmissive(int type) { return type == NR_MAT_GGX || type == NR_MAT_GLASS || type == NR_MAT_LIGHT; }
__device__ __forceinline__ bool mat_nee(int type) { return type == NR_MAT_LAMBERT || type == NR_MAT_GGXR || type == NR_MAT_BLINNPHONG; }

// Tangent frame of the samplers (e.g. src/material/matlambert.cpp:12-14).
__device__ __forceinline__ void frame(f3 n, f3& ax1, f3& ax2) {
    f3 ax0 = fabsf(n.x) < 0.8f ? mk(1.f, 0.f, 0.f) : mk(0.f, 1.f, 0.f);
    ax1 = normalized(cross(ax0, n));
    ax2 = normalized(cross(n, ax1));
}

__device__ __forceinline__ float pow5(float x) { float x2 = x * x; return x2 * x2 * x; }

// GGX D with the reference's alpha^2 / pi / (cos^2 (alpha^2 - 1) + 1)^2.
__device__ __forceinline__ float ggx_D(float alpha, float cosnh) {
    float a2 = alpha * alpha;
    float k = cosnh * cosnh * (a2 - 1.0f) + 1.0f;
    return a2 / NR_PI_F / (k * k);
}

// MatGGX helpers (src/material/matggx.cpp:50-105)
__device__ __forceinline__ f3 ggx_F(f3 v, f3 m, f3 Kd) {
    float vm = dot(v, m);
    if (vm < 0.f) return mk(0.f);
    return Kd + (mk(1.f) - Kd) * pow5(1.f - vm);
}
__device__ __forceinline__ float ggx_G1(float alpha, f3 v, f3 m, f3 n) {
    float vm = dot(v, m), vn = dot(v, n);
    if (vm * vn < 0.f) return 0.f;
    float tn = tanf(acosf(vn));
    float r2 = 1.0f + (alpha * tn) * (alpha * tn);
    return 2.0f / (1.0f + sqrtf(r2));
}
__device__ __forceinline__ float ggx_Dm(float alpha, f3 m, f3 n) {
    float c = dot(n, m);
    if (c < 0.f) return 0.f;
    return ggx_D(alpha, c);
}
__device__ __forceinline__ f3 ggx_fr(const MatView& M, f3 i, f3 o, f3 n) {
    if (dot(n, i) * dot(n, o) < 0.f) return mk(0.f);
    f3 h = normalized(i + o);
    f3 nn = dot(i, n) > 0.f ? n : -n;
    f3 f = ggx_F(i, h, M.c0);
    float g = ggx_G1(M.alpha, i, h, nn) * ggx_G1(M.alpha, o, h, nn);
    float d = ggx_Dm(M.alpha, h, nn);
    float denom = 4.0f * dot(i, nn) * dot(o, nn);
    return f * g * d / (denom + 1e-6f);
}
__device__ __forceinline__ f3 ggx_ft(const MatView& M, f3 i, f3 o, f3 n) {
    if (dot(n, i) * dot(n, o) > 0.f) return mk(0.f);
    float eta = dot(i, n) > 0.f ? M.ior : 1.0f / M.ior;
    f3 h = -normalized(i + eta * o);
    float A = fabsf(dot(i, h) * dot(o, h) / dot(i, n) / dot(o, n));
    f3 f = ggx_F(i, h, M.c0);
    float g = ggx_G1(M.alpha, i, h, n) * ggx_G1(M.alpha, o, h, n);
    float d = ggx_Dm(M.alpha, h, n);
    f3 numer = (eta * eta) * (mk(1.f) - f) * g * d;
    float x = dot(i, h) + eta * dot(o, h);
    return A * numer / (x * x + 1e-8f);
}

// Material::bxdf
__device__ __forceinline__ f3 mat_bxdf(const MatView& M, f3 wo, f3 n, f3 wi) {
    switch (M.type) {
        case NR_MAT_LAMBERT:  // src/material/matlambert.cpp:20-31
            if (dot(wi, n) * dot(wo, n) < 0.f) return mk(0.f);
            return M.c0 / NR_PI_F;
        case NR_MAT_GGXR: {  // src/material/matggxrefl.cpp:35-52
            float ni = dot(n, wi), no = dot(n, wo);
            if (ni * no < 0.f) return mk(0.f);
            f3 wh = normalized(wo + wi);
            float D = ggx_D(M.alpha, dot(n, wh));
            float k = M.alpha * 0.5f + 0.5f, k2 = k * k;
            float Gl = 2.f * ni / (ni + sqrtf(k2 + (1.f - k2 * ni * ni)));
            float Gv = 2.f * no / (no + sqrtf(k2 + (1.f - k2 * no * no)));
            f3 F = M.c0 + (mk(1.f) - M.c0) * pow5(1.0f - dot(wh, wi));
            return F * (D * Gl * Gv) / 4.0f / (no + 1e-6f) / (ni + 1e-6f);
        }
        case NR_MAT_GGX: {  // src/material/matggx.cpp:107-121
            if (dot(wi, n) * dot(wo, n) >= 0.f) return ggx_fr(M, wi, wo, n);
            return ggx_ft(M, wi, wo, n);
        }
        case NR_MAT_GLASS: {  // src/material/matglass.cpp:26-43
            if (fabsf(dot(wi, n)) < 1e-3f) return mk(0.f);
            f3 F = M.c0 + (mk(1.f) - M.c0) * pow5(1.f - fabsf(dot(n, wo)));
            if (dot(wi, n) * dot(wo, n) > 0.f) return F;
            float I = dot(wo, n) > 0.f ? 1.0f / M.ior : M.ior;
            return (mk(1.f) - F) * (I * I);
        }
        case NR_MAT_BLINNPHONG: {  // src/material/matblinnphong.cpp:39-51
            float ni = dot(wi, n), no = dot(wo, n);
            if (ni * no < 0.f) return mk(0.f);
            if (ni <= 1e-4f || no <= 1e-4f) return mk(0.f);
            f3 h = normalized(wo + wi);
            f3 spec = ((M.ns + 2.f) / NR_PI_F / 8.f) * M.c1 * powf(dot(n, h), M.ns);
            return M.c0 / NR_PI_F + spec;
        }
        default:
            return mk(0.f);
    }
}

// Material::pdf
__device__ __forceinline__ float mat_pdf(const MatView& M, f3 wo, f3 n, f3 wi) {
    switch (M.type) {
        case NR_MAT_LAMBERT:  // src/material/matlambert.cpp:33-37
            return NR_INV_PI_F * (fabsf(dot(wi, n)) + 1e-4f);
        case NR_MAT_GGXR: {  // src/material/matggxrefl.cpp:54-64
            if (dot(wi, n) <= 1e-4f || dot(wo, n) <= 1e-4f) return 1e18f;
            f3 wh = normalized(wo + wi);
            float c = dot(n, wh);
            return ggx_D(M.alpha, c) * c / 4.0f + 1e-8f;
        }
        case NR_MAT_GGX: {  // src/material/matggx.cpp:123-148
            if (dot(wi, n) * dot(wo, n) > 0.f) {
                f3 wh = normalized(wo + wi);
                float d = ggx_Dm(M.alpha, wh, n);
                if (d < 1e-9f) return 1e18f;
                return d * dot(n, wh) / 4.0f;
            }
            float eta = dot(wi, n) > 0.f ? M.ior : 1.0f / M.ior;
            f3 wh = -normalized(wi + eta * wo);
            if (dot(wh, n) < 0.f) wh = -wh;
            float d = ggx_Dm(M.alpha, wh, n);
            if (d < 1e-6f) return 1e18f;
            return smax(d * dot(n, wh) / 4.0f, 1.0f);
        }
        case NR_MAT_GLASS:
            return 0.5f;
        case NR_MAT_BLINNPHONG: {  // src/material/matblinnphong.cpp:53-62
            if (dot(wi, n) <= 1e-4f || dot(wo, n) <= 1e-4f) return 1e-18f;
            float pd = NR_INV_PI_F * (fabsf(dot(wi, n)) + 1e-6f);
            f3 h = normalized(wo + wi);
            float ps = (M.ns + 2.f) / NR_PI_F / 8.f * powf(fabsf(dot(n, h)), M.ns + 1.f);
            return 0.5f * pd + 0.5f * ps;
        }
        default:
            return NR_INV_PI_F;
    }
}

// Material::sampleBxdf; the draw order matches the reference exactly.
template <class RNG>
__device__ __forceinline__ f3 mat_sample(const MatView& M, RNG& s, f3 wo, f3 n) {
    switch (M.type) {
        case NR_MAT_LAMBERT: {  // src/material/matlambert.cpp:5-18
            float r2 = s.next() * 0.99f;
            float phi = s.next() * (NR_PI_F * 2.0f);
            float r = sqrtf(r2), h = sqrtf(1.f - r2);
            f3 ax1, ax2; frame(n, ax1, ax2);
            float sp, cp; sincosf(phi, &sp, &cp);
            return h * n + (r * cp) * ax1 + (r * sp) * ax2;
        }
        case NR_MAT_GGXR: {  // src/material/matggxrefl.cpp:5-33
            f3 ax1, ax2; frame(n, ax1, ax2);
            float r1 = s.next(), r2 = s.next();
            float theta = atanf(M.alpha * sqrtf(r1 / (1.f - r1))) * 0.9999f;
            float phi = 2.0f * 3.14159f * r2;
            float st, ct, sp, cp; sincosf(theta, &st, &ct); sincosf(phi, &sp, &cp);
            f3 h = ct * n + (st * cp) * ax1 + (st * sp) * ax2;
            return (2.0f * dot(h, wo)) * h - wo;
        }
        case NR_MAT_GGX: {  // src/material/matggx.cpp:5-48
            f3 ax1, ax2; frame(n, ax1, ax2);
            float r1 = s.next(), r2 = s.next();
            float cos_theta = sqrtf((1.f - r1) / (1.f + (M.alpha * M.alpha - 1.f) * r1));
            float theta = acosf(cos_theta) * 0.9999f;
            float phi = 2.0f * 3.14159f * r2;
            float st, ct, sp, cp; sincosf(theta, &st, &ct); sincosf(phi, &sp, &cp);
            f3 h = ct * n + (st * cp) * ax1 + (st * sp) * ax2;
            f3 wi;
            if (s.next() < 0.5f) {
                wi = (2.0f * dot(h, wo)) * h - wo;
            } else {
                float eta = 1.0f / M.ior;  // the reference tests the still-zero wi (matggx.cpp:43)
                float nh = fabsf((eta + 1.0f) * dot(wo, h));
                wi = (-eta) * wo - h * nh;
            }
            return normalized(wi);
        }
        case NR_MAT_GLASS: {  // src/material/matglass.cpp:5-24
            bool refract = s.next() < 0.5f;
            float c = dot(wo, n);
            f3 nn = c > 0.f ? n : -n;
            if (refract) {
                float I = c > 0.f ? 1.0f / M.ior : M.ior;
                f3 t = normalized(cross(cross(nn, wo), nn));
                float sin_i = smin(dot(wo, t) * I, 1.0f);
                float cos_i = sqrtf(1.0f - sin_i * sin_i);
                return -(cos_i * nn + sin_i * t);
            }
            return (2.0f * dot(wo, nn)) * nn - wo;
        }
        case NR_MAT_BLINNPHONG: {  // src/material/matblinnphong.cpp:5-37
            float r0 = s.next();
            f3 ax1, ax2; frame(n, ax1, ax2);
            if (r0 < 0.5f) {
                float r2 = s.next() * 0.99f;
                float phi = s.next() * (NR_PI_F * 2.0f);
                float r = sqrtf(r2), h = sqrtf(1.f - r2);
                float sp, cp; sincosf(phi, &sp, &cp);
                return h * n + (r * cp) * ax1 + (r * sp) * ax2;
            }
            float r1 = s.next(), r2 = s.next();
            float cos_theta = powf(r1, 1.0f / (M.ns + 2.0f));
            float sin_theta = sqrtf(1.f - cos_theta);  // as written in the reference (matblinnphong.cpp:30)
            float phi = 2.0f * 3.14159f * r2;
            float sp, cp; sincosf(phi, &sp, &cp);
            f3 h = cos_theta * n + (sin_theta * cp) * ax1 + (sin_theta * sp) * ax2;
            return (2.0f * dot(h, wo)) * h - wo;
        }
        default:
            return mk(0.f);
    }
}

// Cache input encoding: nrc_encode.cuh.
__device__ __forceinline__ float nrc_roughness(const MatView& M) {
    if (M.type == NR_MAT_GGXR || M.type == NR_MAT_GGX) return M.alpha;
    if (M.type == NR_MAT_GLASS) return 0.f;
    return 1.f;
}
__device__ __forceinline__ bool nrc_diffuse(const MatView& M, float rough_min) {
    if (M.type == NR_MAT_LAMBERT || M.type == NR_MAT_BLINNPHONG) return true;
    if (M.type == NR_MAT_GGXR || M.type == NR_MAT_GGX) return M.alpha >= rough_min;
    return false;
}
// The cache's compact record of a vertex (nrc_encode.cuh): position in the
// scene box, outgoing direction and shading normal as (phi / 2pi + 0.5,
// theta / pi), roughness and albedo.
__device__ __forceinline__ void nrc_record(uint32_t rec[8], const float lo[3], const float inv_ext[3], f3 p, f3 wo, f3 n,
                                           float rough, f3 albedo) {
    rec[0] = __float_as_uint((p.x - lo[0]) * inv_ext[0]);
    rec[1] = __float_as_uint((p.y - lo[1]) * inv_ext[1]);
    rec[2] = __float_as_uint((p.z - lo[2]) * inv_ext[2]);
    auto sph = [](f3 d, float& u, float& v) {
        u = atan2f(d.z, d.x) * (0.5f / 3.14159265f) + 0.5f;
        v = acosf(fminf(1.f, fmaxf(-1.f, d.y))) * (1.f / 3.14159265f);
    };
    float u0, v0, u1, v1;
    sph(wo, u0, v0);
    sph(n, u1, v1);
    __nv_bfloat162 e0 = __floats2bfloat162_rn(u0, v0), e1 = __floats2bfloat162_rn(u1, v1);
    __nv_bfloat162 e2 = __floats2bfloat162_rn(rough, albedo.x), e3 = __floats2bfloat162_rn(albedo.y, albedo.z);
    rec[3] = *reinterpret_cast<uint32_t*>(&e0);
    rec[4] = *reinterpret_cast<uint32_t*>(&e1);
    rec[5] = *reinterpret_cast<uint32_t*>(&e2);
    rec[6] = *reinterpret_cast<uint32_t*>(&e3);
    rec[7] = 0u;
}
// The full 160-byte encoding of a vertex (a training record); dst 16-byte aligned.
__device__ __forceinline__ void nrc_encode(uint32_t* dst, const float lo[3], const float inv_ext[3], f3 p, f3 wo, f3 n,
                                           float rough, f3 albedo) {
    uint32_t rec[8], w[40];
    nrc_record(rec, lo, inv_ext, p, wo, n, rough, albedo);
    nrc_expand(rec, w);
    nrc_store_row(dst, w);
}

// Camera::generateRay (src/scene/camera.cpp:24-32); film_h precomputed as
// 2 tan(fov * 3.14159 / 360).
__device__ __forceinline__ f3 camera_ray(const nr_camera& C, float film_h, float img_x, float img_y, float w, float h) {
    float cx = img_x / w * 2.0f - 1.0f;
    float cy = img_y / h * 2.0f - 1.0f;
    f3 gaze = mk(C.gaze[0], C.gaze[1], C.gaze[2]), up = mk(C.up[0], C.up[1], C.up[2]);
    f3 hand = normalized(cross(gaze, up));
    float film_w = film_h * C.aspect;
    return normalized(gaze + hand * film_w * cx * 0.5f - up * film_h * cy * 0.5f);
}

}  // namespace nr
