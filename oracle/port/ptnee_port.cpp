// CPU restatement of the reference ptnee integrator. TEST INFRASTRUCTURE:
// see ptnee_port.h. Every function names the reference lines it restates.
// Expressions keep the reference's evaluation types: where the reference
// mixes a float with a double literal or calls a C libm function on a float,
// the value is computed in double and rounded back exactly as there.
// Build with -ffp-contract=off so no multiply-add is fused.
#include "ptnee_port.h"
#include "../philox.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

namespace {

struct V3 {
    float x, y, z;
    V3() : x(0.f), y(0.f), z(0.f) {}
    explicit V3(float s) : x(s), y(s), z(s) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return a * s; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float norm2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// vec3::norm: sqrt(float) binds to the C double sqrt (src/math/vec3.cpp:66-69)
inline float norm(V3 a) { return (float)std::sqrt((double)norm2(a)); }
// vec3::normalized divides by norm()+1e-8f (src/math/vec3.cpp:70-73)
inline V3 normalized(V3 a) { return a / (norm(a) + 1e-8f); }
// std::min / std::max component-wise (src/math/vec3.cpp:103-111)
inline float fmin_std(float a, float b) { return (b < a) ? b : a; }
inline float fmax_std(float a, float b) { return (a < b) ? b : a; }
inline V3 vmin(V3 a, V3 b) { return {fmin_std(a.x, b.x), fmin_std(a.y, b.y), fmin_std(a.z, b.z)}; }
inline V3 vmax(V3 a, V3 b) { return {fmax_std(a.x, b.x), fmax_std(a.y, b.y), fmax_std(a.z, b.z)}; }

const double PI_D = 3.14159;
const float PI_F = 3.14159f;

enum { MT_LAMBERT = 0, MT_GGXR = 1, MT_GGX = 2, MT_GLASS = 3, MT_BLINNPHONG = 4, MT_LIGHT = 5 };

struct Tex {
    int w = 0, h = 0;
    std::vector<V3> px;
    // Texture::pixel const: black outside (src/scene/texture.cpp:54-59)
    V3 at(int x, int y) const {
        if (x < 0 || y < 0 || x >= w || y >= h) return V3(0, 0, 0);
        return px[(size_t)y * w + x];
    }
    // Texture::pixelBi (src/scene/texture.cpp:61-67)
    V3 bilinear(float x, float y) const {
        int x0 = (int)std::floor((double)x), y0 = (int)std::floor((double)y);
        int x1 = x0 + 1, y1 = y0 + 1;
        return at(x1, y1) * (x - (float)x0) * (y - (float)y0) + at(x1, y0) * (x - (float)x0) * ((float)y1 - y) +
               at(x0, y1) * ((float)x1 - x) * (y - (float)y0) + at(x0, y0) * ((float)x1 - x) * ((float)y1 - y);
    }
    // Texture::pixelUV: wrap and flip v (src/scene/texture.cpp:69-72)
    V3 uv(float u, float v) const {
        double a = std::fmod(std::fmod((double)u, 1.0) + 1.0, 1.0) * w;
        double b = std::fmod(std::fmod((double)(1.0f - v), 1.0) + 1.0, 1.0) * h;
        return bilinear((float)a, (float)b);
    }
};

struct Mat {
    int type = MT_LAMBERT;
    V3 c0, c1;       // Kd / F0 / Ke, Ks
    float alpha = 0.5f, ior = 1.0f, ns = 10.0f;
    const Tex* t0 = nullptr;  // map_Kd (map_F0 for glass)
    const Tex* t1 = nullptr;  // map_Ks
};

struct Tri {
    V3 p[3], t[3], n[3];
    int mat;
    V3 pmin, pmax;
};

class Sampler {
public:
    virtual float random() = 0;
    virtual ~Sampler() {}
};
class PhiloxSampler : public Sampler {
public:
    nr_path_stream s;
    PhiloxSampler(uint64_t seed, uint32_t pixel, uint32_t sample) { nr_stream_init(&s, seed, pixel, sample, 0); }
    float random() override { return nr_stream_next(&s); }
};
class ListSampler : public Sampler {
public:
    const float* u; int n; int i = 0;
    ListSampler(const float* u_, int n_) : u(u_), n(n_) {}
    float random() override { return i < n ? u[i++] : 0.5f; }
};

// ---------------------------------------------------------------- geometry

// Triangle::intersection (src/scene/triangle.cpp:27-33): Moller-Trumbore with
// q = s1.e1 + 1e-6 evaluated in double and rounded to float.
inline void tri_intersect(const Tri& T, V3 o, V3 d, float& t, float& b1, float& b2) {
    V3 e1 = T.p[1] - T.p[0], e2 = T.p[2] - T.p[0];
    V3 s = o - T.p[0], s1 = cross(d, e2), s2 = cross(s, e1);
    float tt = dot(s2, e2), u = dot(s1, s), v = dot(s2, d);
    float q = (float)((double)dot(s1, e1) + 1e-6);
    t = tt / q; b1 = u / q; b2 = v / q;
}

// Triangle::getNormal / getTexCoords (src/scene/triangle.cpp:35-43)
inline V3 tri_normal(const Tri& T, float b1, float b2) {
    return normalized((1.0f - b1 - b2) * T.n[0] + b1 * T.n[1] + b2 * T.n[2]);
}
inline V3 tri_uv(const Tri& T, float b1, float b2) { return (1.0f - b1 - b2) * T.t[0] + b1 * T.t[1] + b2 * T.t[2]; }

// ---------------------------------------------------------------- BVH
struct Node {
    V3 pmin, pmax;
    int left = -1, right = -1;
    std::vector<int> prims;
};

struct BVH {
    std::vector<Node> nodes;   // nodes[0] is the root when non-empty
    const std::vector<Tri>* tris = nullptr;
    int root = -1;

    // BVHNode::intersect (src/hierarchy/bvhnode.cpp:35-48)
    static bool box_hit(const Node& n, V3 o, V3 d) {
        float t_in = -1e18f, t_out = 1e18f;
        for (int i = 0; i < 3; ++i) {
            float mn = n.pmin[i], mx = n.pmax[i];
            float t1 = (mn - o[i]) / (d[i] + 1e-9f), t2 = (mx - o[i]) / (d[i] + 1e-9f);
            if (t1 > t2) std::swap(t1, t2);
            t_in = fmax_std(t_in, t1);
            t_out = fmin_std(t_out, t2);
        }
        return t_in <= t_out && t_out >= 0;
    }

    struct Hit { float t, b1, b2; int tri; };

    // BVHNode::getIntersection (src/hierarchy/bvhnode.cpp:50-66)
    Hit leaf_hit(const Node& n, V3 o, V3 d) const {
        Hit h{1e18f, 0.f, 0.f, -1};
        for (int id : n.prims) {
            float t, b1, b2;
            tri_intersect((*tris)[id], o, d, t, b1, b2);
            if (t < h.t && t > 0 && b1 >= 0 && b2 >= 0 && b1 + b2 <= 1) h = {t, b1, b2, id};
        }
        return h;
    }

    // BVH::_traversal (src/hierarchy/bvh.cpp:99-127): exhaustive; left wins
    // only when strictly nearer.
    Hit traverse(int ni, V3 o, V3 d) const {
        if (ni < 0) return {1e18f, 0, 0, -1};
        const Node& n = nodes[ni];
        if (!box_hit(n, o, d)) return {1e18f, 0, 0, -1};
        if (n.left < 0 && n.right < 0) return leaf_hit(n, o, d);
        Hit l = traverse(n.left, o, d);
        Hit r = traverse(n.right, o, d);
        return (l.t > 0 && l.t < r.t) ? l : r;
    }
    Hit intersect(V3 o, V3 d) const { return traverse(root, o, d); }

    // BVH::_divide / _build (src/hierarchy/bvh.cpp:5-70): SAH over a sweep of
    // the primitives sorted by pMax on each axis; leaf at <= 5 primitives.
    struct Key { float k[3]; int id; };

    static float surface_area(V3 a, V3 b) {
        V3 d = b - a;
        return (d.x * d.y + d.y * d.z + d.z * d.x) * 2.0f;
    }

    void split(std::vector<Key>& prims, std::vector<Key>& L, std::vector<Key>& R) const {
        int ans_axis = 0, ans_mid = 0;
        float ans_cost = 1e38f;
        const size_t n = prims.size();
        std::vector<float> suffix(n);
        for (int axis = 0; axis < 3; ++axis) {
            std::sort(prims.begin(), prims.end(), [axis](const Key& a, const Key& b) { return a.k[axis] < b.k[axis]; });
            V3 lo(1e18f), hi(-1e18f);
            for (int i = (int)n - 1; i >= 0; --i) {
                const Tri& t = (*tris)[prims[i].id];
                lo = vmin(lo, t.pmin); hi = vmax(hi, t.pmax);
                suffix[i] = surface_area(lo, hi);
            }
            lo = V3(1e18f); hi = V3(-1e18f);
            for (size_t i = 0; i + 1 < n; ++i) {
                const Tri& t = (*tris)[prims[i].id];
                lo = vmin(lo, t.pmin); hi = vmax(hi, t.pmax);
                float pre = surface_area(lo, hi);
                float cost = pre * (float)(int)(i + 1) + suffix[i + 1] * (float)(n - i);
                if (cost < ans_cost) { ans_cost = cost; ans_mid = (int)i + 1; ans_axis = axis; }
            }
        }
        std::sort(prims.begin(), prims.end(), [ans_axis](const Key& a, const Key& b) { return a.k[ans_axis] < b.k[ans_axis]; });
        L.assign(prims.begin(), prims.begin() + ans_mid);
        R.assign(prims.begin() + ans_mid, prims.end());
    }

    int make_leaf(const std::vector<Key>& prims) {
        Node n;
        n.pmin = V3(1e18f); n.pmax = V3(-1e18f);
        for (const Key& k : prims) {
            const Tri& t = (*tris)[k.id];
            for (int i = 0; i < 3; ++i) { n.pmin = vmin(n.pmin, t.p[i]); n.pmax = vmax(n.pmax, t.p[i]); }
            n.prims.push_back(k.id);
        }
        nodes.push_back(std::move(n));
        return (int)nodes.size() - 1;
    }

    int build_rec(std::vector<Key>& prims) {
        if (prims.size() <= 5) return make_leaf(prims);
        std::vector<Key> L, R;
        split(prims, L, R);
        std::vector<Key>().swap(prims);
        int id = (int)nodes.size();
        nodes.emplace_back();
        int l = build_rec(L);
        int r = build_rec(R);
        Node& n = nodes[id];
        n.left = l; n.right = r;
        n.pmin = vmin(nodes[l].pmin, nodes[r].pmin);
        n.pmax = vmax(nodes[l].pmax, nodes[r].pmax);
        return id;
    }

    void build(const std::vector<Tri>& t) {
        tris = &t;
        std::vector<Key> prims(t.size());
        for (size_t i = 0; i < t.size(); ++i) {
            prims[i].id = (int)i;
            for (int a = 0; a < 3; ++a) prims[i].k[a] = t[i].pmax[a];
        }
        nodes.clear();
        nodes.reserve(t.size() / 2 + 16);
        root = build_rec(prims);
    }
};

// ---------------------------------------------------------------- lights
// LightSampler::setPrimitives / sampleLight / p (src/sampler/lightsampler.cpp:4-58,100-103)
struct Lights {
    std::vector<int> tris;
    std::vector<float> cdf;
    float sum_weight = 0.f;
    void build(const std::vector<Tri>& t, const std::vector<Mat>& mats) {
        std::vector<float> pdf;
        float sum = 0;
        for (size_t i = 0; i < t.size(); ++i) {
            if (mats[t[i].mat].type != MT_LIGHT) continue;
            float w = norm(cross(t[i].p[1] - t[i].p[0], t[i].p[2] - t[i].p[0]));  // Triangle::area (2x area)
            pdf.push_back(w);
            sum += w;
            tris.push_back((int)i);
        }
        sum = (float)((double)sum + 1e-8);
        for (auto& x : pdf) x /= sum;
        sum_weight = sum;
        float acc = 1e-6f;
        for (float x : pdf) { acc += x; cdf.push_back(acc); }
    }
    int pick(Sampler& s) const {
        if (tris.empty()) return -1;
        float r = s.random();
        size_t id = std::lower_bound(cdf.begin(), cdf.end(), r) - cdf.begin();
        if (id >= tris.size()) id = tris.size() - 1;  // the reference would read past its vector here
        return tris[id];
    }
    float p() const { return (float)(1.0 / ((double)sum_weight + 1e-8)); }
};

// ---------------------------------------------------------------- materials
inline void frame(V3 n, V3& ax1, V3& ax2) {
    V3 ax0 = ((double)std::fabs(n.x) < 0.8) ? V3(1, 0, 0) : V3(0, 1, 0);
    ax1 = normalized(cross(ax0, n));
    ax2 = normalized(cross(n, ax1));
}

inline V3 tex_or(const Tex* t, V3 c, V3 uv) { return t ? t->uv(uv.x, uv.y) : c; }

// MatGGX helpers (src/material/matggx.cpp:50-105)
inline V3 ggx_F(V3 v, V3 m, V3 Kd) {
    if (dot(v, m) < 0) return V3(0.f);
    return Kd + (V3(1.0f) - Kd) * (float)std::pow((double)(1 - dot(v, m)), 5.0);
}
inline float ggx_G1(const Mat& M, V3 v, V3 m, V3 n) {
    float vm = dot(v, m), vn = dot(v, n);
    if (vm * vn < 0) return 0.0f;
    float r2 = (float)(1.0f + std::pow((double)M.alpha * std::tan(std::acos((double)vn)), 2.0));
    return (float)(2.0f / (1.0f + std::sqrt((double)r2)));
}
inline float ggx_D(const Mat& M, V3 m, V3 n) {
    if (dot(n, m) < 0) return 0.0f;
    double a2 = std::pow((double)M.alpha, 2.0);
    return (float)(a2 / (double)PI_F / std::pow(std::pow((double)dot(n, m), 2.0) * (a2 - 1) + 1, 2.0));
}
inline V3 ggx_fr(const Mat& M, V3 i, V3 o, V3 n, V3 Kd) {
    if (dot(n, i) * dot(n, o) < 0) return V3(0.f);
    V3 h = normalized(i + o);
    V3 nn = dot(i, n) > 0 ? n : -n;
    V3 f = ggx_F(i, h, Kd);
    V3 g(ggx_G1(M, i, h, nn) * ggx_G1(M, o, h, nn));
    V3 d(ggx_D(M, h, nn));
    float denom = 4.0f * dot(i, nn) * dot(o, nn);
    return f * g * d / (denom + 1e-6f);
}
inline V3 ggx_ft(const Mat& M, V3 i, V3 o, V3 n, V3 Kd) {
    if (dot(n, i) * dot(n, o) > 0) return V3(0.f);
    float eta = dot(i, n) > 0 ? M.ior : 1.0f / M.ior;
    V3 h = -normalized(i + eta * o);
    float A = std::fabs(dot(i, h) * dot(o, h) / dot(i, n) / dot(o, n));
    V3 f = ggx_F(i, h, Kd);
    V3 g(ggx_G1(M, i, h, n) * ggx_G1(M, o, h, n));
    V3 d(ggx_D(M, h, n));
    V3 numer = (float)std::pow((double)eta, 2.0) * (V3(1.0f) - f) * g * d;
    float denom = (float)std::pow((double)(dot(i, h) + eta * dot(o, h)), 2.0);
    return A * numer / (denom + 1e-8f);
}

// Material::sampleBxdf
V3 mat_sample(const Mat& M, Sampler& s, V3 wo, V3 n) {
    switch (M.type) {
        case MT_LAMBERT: {  // src/material/matlambert.cpp:5-18
            float r2 = s.random() * 0.99f;
            float phi = (float)((double)s.random() * PI_D * 2);
            float r = (float)std::sqrt((double)r2), h = (float)std::sqrt((double)(1 - r2));
            V3 ax1, ax2; frame(n, ax1, ax2);
            return h * n + (float)(r * std::cos((double)phi)) * ax1 + (float)(r * std::sin((double)phi)) * ax2;
        }
        case MT_GGXR: {  // src/material/matggxrefl.cpp:5-33
            V3 ax1, ax2; frame(n, ax1, ax2);
            float r1 = s.random(), r2 = s.random();
            float theta = (float)(std::atan((double)M.alpha * std::sqrt((double)(r1 / (1 - r1)))) * 0.9999);
            float phi = 2.0f * 3.14159f * r2;
            V3 h = (float)std::cos((double)theta) * n +
                   (float)(std::sin((double)theta) * std::cos((double)phi)) * ax1 +
                   (float)(std::sin((double)theta) * std::sin((double)phi)) * ax2;
            return 2.0f * dot(h, wo) * h - wo;
        }
        case MT_GGX: {  // src/material/matggx.cpp:5-48
            V3 ax1, ax2; frame(n, ax1, ax2);
            float r1 = s.random(), r2 = s.random();
            float cos_theta = (float)std::sqrt((double)((1 - r1) / (1 + (M.alpha * M.alpha - 1) * r1)));
            float theta = (float)(std::acos((double)cos_theta) * 0.9999);
            float phi = 2.0f * 3.14159f * r2;
            V3 h = (float)std::cos((double)theta) * n +
                   (float)(std::sin((double)theta) * std::cos((double)phi)) * ax1 +
                   (float)(std::sin((double)theta) * std::sin((double)phi)) * ax2;
            V3 wi;
            if ((double)s.random() < 0.5) {
                wi = 2.0f * dot(h, wo) * h - wo;
            } else {
                float eta = 1.0f / M.ior;  // the reference tests the still-zero wi (matggx.cpp:43)
                float norm_h = std::fabs((eta + 1.0f) * dot(wo, h));
                wi = -eta * wo - h * norm_h;
            }
            return normalized(wi);
        }
        case MT_GLASS: {  // src/material/matglass.cpp:5-24
            if ((double)s.random() < 0.5) {
                float I = dot(wo, n) > 0 ? 1.0f / M.ior : M.ior;
                V3 nn = dot(wo, n) > 0 ? n : -n;
                V3 t = normalized(cross(cross(nn, wo), nn));
                float sin_o = dot(wo, t);
                float sin_i = sin_o * I;
                sin_i = fmin_std(sin_i, 1.0f);
                float cos_i = (float)std::sqrt((double)(1.0f - sin_i * sin_i));
                V3 i = cos_i * nn + sin_i * t;
                return -i;
            }
            V3 nn = dot(wo, n) > 0 ? n : -n;
            return (2.0f * dot(wo, nn)) * nn - wo;
        }
        case MT_BLINNPHONG: {  // src/material/matblinnphong.cpp:5-37
            float r0 = s.random();
            V3 ax1, ax2; frame(n, ax1, ax2);
            if (r0 < 0.5f) {
                float r2 = s.random() * 0.99f;
                float phi = (float)((double)s.random() * PI_D * 2);
                float r = (float)std::sqrt((double)r2), h = (float)std::sqrt((double)(1 - r2));
                return h * n + (float)(r * std::cos((double)phi)) * ax1 + (float)(r * std::sin((double)phi)) * ax2;
            }
            double r1 = s.random();
            double r2 = s.random();
            double cos_theta = std::pow(r1, (double)(1.0f / (M.ns + 2.0f)));
            double sin_theta = std::sqrt(1 - cos_theta);
            double phi = (double)(2.0f * 3.14159f) * r2;
            V3 h = (float)cos_theta * n + (float)(sin_theta * std::cos(phi)) * ax1 + (float)(sin_theta * std::sin(phi)) * ax2;
            return 2.0f * dot(h, wo) * h - wo;
        }
        default:
            return V3(0.f);
    }
}

// Material::bxdf
V3 mat_bxdf(const Mat& M, V3 wo, V3 n, V3 wi, V3 uv) {
    switch (M.type) {
        case MT_LAMBERT:  // src/material/matlambert.cpp:20-31
            if (dot(wi, n) * dot(wo, n) < 0) return V3(0.f);
            return tex_or(M.t0, M.c0, uv) / PI_F;
        case MT_GGXR: {  // src/material/matggxrefl.cpp:35-52
            if (dot(wi, n) * dot(wo, n) < 0) return V3(0.f);
            V3 Kd = tex_or(M.t0, M.c0, uv);
            V3 wh = normalized(wo + wi);
            double a2 = std::pow((double)M.alpha, 2.0);
            V3 D((float)(a2 / (double)PI_F / std::pow(std::pow((double)dot(n, wh), 2.0) * (a2 - 1) + 1, 2.0)));
            double k2 = std::pow((double)M.alpha * 0.5 + 0.5, 2.0);
            double ni = dot(n, wi), no = dot(n, wo);
            V3 Gl((float)(2 * ni / (ni + std::sqrt(k2 + (1 - k2 * std::pow(ni, 2.0))))));
            V3 Gv((float)(2 * no / (no + std::sqrt(k2 + (1 - k2 * std::pow(no, 2.0))))));
            V3 F = Kd + (V3(1.0f) - Kd) * (float)std::pow((double)(1.0f - dot(wh, wi)), 5.0);
            return D * Gl * Gv * F / 4.0f / (dot(n, wo) + 1e-6f) / (dot(n, wi) + 1e-6f);
        }
        case MT_GGX: {  // src/material/matggx.cpp:107-121
            V3 Kd = tex_or(M.t0, M.c0, uv);
            float bi = dot(wi, n), bo = dot(wo, n);
            if (bi * bo >= 0) return ggx_fr(M, wi, wo, n, Kd);
            return ggx_ft(M, wi, wo, n, Kd);
        }
        case MT_GLASS: {  // src/material/matglass.cpp:26-43
            if (std::fabs(dot(wi, n)) < 1e-3f) return V3(0.f);
            V3 f0 = tex_or(M.t0, M.c0, uv);
            V3 F = f0 + (V3(1.0f) - f0) * (float)std::pow((double)(1 - std::fabs(dot(n, wo))), 5.0);
            if (dot(wi, n) * dot(wo, n) > 0) return F;
            float I = dot(wo, n) > 0 ? 1.0f / M.ior : M.ior;
            return (V3(1.0f) - F) * (float)std::pow((double)I, 2.0);
        }
        case MT_BLINNPHONG: {  // src/material/matblinnphong.cpp:39-51
            if (dot(wi, n) * dot(wo, n) < 0) return V3(0.f);
            if ((double)dot(wi, n) <= 1e-4 || dot(wo, n) <= 1e-4f) return V3(0.f);
            V3 Rd = tex_or(M.t0, M.c0, uv);
            V3 Rs = tex_or(M.t1, M.c1, uv);
            V3 diffuse = Rd / PI_F;
            V3 h = normalized(wo + wi);
            V3 spec = (float)((double)(M.ns + 2) / PI_D / 8) * Rs * (float)std::pow((double)dot(n, h), (double)M.ns);
            return diffuse + spec;
        }
        default:
            return V3(0.f);
    }
}

// Material::pdf
float mat_pdf(const Mat& M, V3 wo, V3 n, V3 wi) {
    switch (M.type) {
        case MT_LAMBERT:  // src/material/matlambert.cpp:33-37
            return (float)(1.0 / PI_D * (double)(std::fabs(dot(wi, n)) + 1e-4f));
        case MT_GGXR: {  // src/material/matggxrefl.cpp:54-64
            if ((double)dot(wi, n) <= 1e-4 || dot(wo, n) <= 1e-4f) return 1e18f;
            V3 wh = normalized(wo + wi);
            double a2 = std::pow((double)M.alpha, 2.0);
            float D = (float)(a2 / (double)PI_F / std::pow(std::pow((double)dot(n, wh), 2.0) * (a2 - 1) + 1, 2.0));
            return D * dot(n, wh) / 4.0f + 1e-8f;
        }
        case MT_GGX: {  // src/material/matggx.cpp:123-148
            if (dot(wi, n) * dot(wo, n) > 0) {
                V3 wh = normalized(wo + wi);
                float d = ggx_D(M, wh, n);
                if (d < 1e-9f) return 1e18f;
                return d * dot(n, wh) / 4.0f;
            }
            float eta = dot(wi, n) > 0 ? M.ior : 1.0f / M.ior;
            V3 wh = -normalized(wi + eta * wo);
            if (dot(wh, n) < 0) wh = -wh;
            float d = ggx_D(M, wh, n);
            if (d < 1e-6f) return 1e18f;
            return fmax_std(d * dot(n, wh) / 4.0f, 1.0f);
        }
        case MT_GLASS:
            return 0.5f;
        case MT_BLINNPHONG: {  // src/material/matblinnphong.cpp:53-62
            if ((double)dot(wi, n) <= 1e-4 || dot(wo, n) <= 1e-4f) return 1e-18f;
            float pd = (float)(1.0 / PI_D * (double)(std::fabs(dot(wi, n)) + 1e-6f));
            V3 h = normalized(wo + wi);
            float ps = (float)((double)(M.ns + 2) / PI_D / 8 * std::pow((double)std::fabs(dot(n, h)), (double)(M.ns + 1)));
            return 0.5f * pd + (1.0f - 0.5f) * ps;
        }
        default:  // MatLight::pdf
            return (float)(1.0 / PI_D);
    }
}

inline bool mat_transmissive(const Mat& M) { return M.type == MT_GGX || M.type == MT_GLASS || M.type == MT_LIGHT; }
inline bool mat_nee(const Mat& M) { return M.type == MT_LAMBERT || M.type == MT_GGXR || M.type == MT_BLINNPHONG; }

// ---------------------------------------------------------------- config / camera
struct Config {
    std::map<std::string, std::string> mp;
    explicit Config(const char* s) {
        std::stringstream ss(s ? s : "");
        std::string kv;
        while (ss >> kv) {
            auto id = kv.find('=');
            mp[kv.substr(0, id)] = kv.substr(id + 1);
        }
    }
    int i(const char* k, int d) const {
        auto it = mp.find(k); if (it == mp.end()) return d;
        std::stringstream ss(it->second); int x; if (!(ss >> x)) return d; return x;
    }
    float f(const char* k, float d) const {
        auto it = mp.find(k); if (it == mp.end()) return d;
        std::stringstream ss(it->second); float x; if (!(ss >> x)) return d; return x;
    }
    V3 v(const char* k, V3 d) const {
        auto it = mp.find(k); if (it == mp.end()) return d;
        std::string s = it->second; for (auto& c : s) if (c == ',') c = ' ';
        std::stringstream ss(s); float x, y, z; if (!(ss >> x >> y >> z)) return d; return V3(x, y, z);
    }
};

struct Cam {
    V3 pos, gaze, up;
    float fov, asp;
    // Camera(fov, asp, pos, yaw, pitch, roll) + fromEuler (src/scene/camera.cpp:16-22, 88-105)
    Cam(const Config& c) {
        fov = c.f("camfov", 90.0f); asp = c.f("camasp", 1.0f);
        pos = c.v("campos", V3(0, 0, 0));
        V3 e = c.v("cameuler", V3(0, 0, 0));
        float c1 = (float)std::cos((double)(e.x / 180.0f) * PI_D), s1 = (float)std::sin((double)(e.x / 180.0f) * PI_D);
        float c2 = (float)std::cos((double)(e.y / 180.0f) * PI_D), s2 = (float)std::sin((double)(e.y / 180.0f) * PI_D);
        float c3 = (float)std::cos((double)(e.z / 180.0f) * PI_D), s3 = (float)std::sin((double)(e.z / 180.0f) * PI_D);
        float m12 = c3 * s1 * s2 - c1 * s3;
        float m13 = c2 * s1;
        float m22 = c2 * c3;
        float m23 = -s2;
        float m32 = s1 * s3 + c1 * c3 * s2;
        float m33 = c1 * c2;
        up = V3(m12, m22, m32);
        gaze = V3(-m13, -m23, -m33);
    }
    // Camera::generateRay (src/scene/camera.cpp:24-32)
    V3 ray(float x, float y, float w, float h) const {
        float cx = x / w * 2.0f - 1.0f;
        float cy = y / h * 2.0f - 1.0f;
        V3 hand = normalized(cross(gaze, up));
        float fh = (float)(2 * std::tan((double)fov * PI_D / 180 / 2));
        float fw = fh * asp;
        return normalized(gaze + hand * fw * cx * 0.5f - up * fh * cy * 0.5f);
    }
};

// ---------------------------------------------------------------- scene
// Environment sampling table of envis=1 (no counterpart in the reference):
// the construction the library documents in host_scene.h (EnvTable),
// restated. Cell (x, y) spans texels (x, y)..(x + 1, y + 1); weight = the
// largest r + g + b of its corners (black past the edges) times
// sin((y + 0.5) / h * 3.14159); cumulative sums in float, last entry 1.
struct EnvTable {
    int w = 0, h = 0;
    std::vector<float> weight, row_cdf, col_cdf;
    float total = 0.f;
    void build(const Tex& t) {
        w = t.w; h = t.h;
        weight.assign((size_t)w * h, 0.f);
        row_cdf.assign((size_t)h, 0.f);
        col_cdf.assign((size_t)w * h, 0.f);
        auto lum = [&](int x, int y) -> float {
            if (x >= w || y >= h) return 0.f;
            const V3& c = t.px[(size_t)y * w + x];
            return c.x + c.y + c.z;
        };
        std::vector<float> rows((size_t)h, 0.f);
        for (int y = 0; y < h; ++y) {
            const float sn = std::sin(((float)y + 0.5f) / (float)h * 3.14159f);
            float acc = 0.f;
            for (int x = 0; x < w; ++x) {
                float m = std::max(std::max(lum(x, y), lum(x + 1, y)), std::max(lum(x, y + 1), lum(x + 1, y + 1)));
                float wt = m > 0.f ? m * sn : 0.f;
                weight[(size_t)y * w + x] = wt;
                acc += wt;
                col_cdf[(size_t)y * w + x] = acc;
            }
            rows[y] = acc;
            for (int x = 0; x < w; ++x) {
                float& c = col_cdf[(size_t)y * w + x];
                c = acc > 0.f ? c / acc : (float)(x + 1) / (float)w;
            }
            col_cdf[(size_t)y * w + w - 1] = 1.f;
        }
        float acc = 0.f;
        for (int y = 0; y < h; ++y) { acc += rows[y]; row_cdf[y] = acc; }
        total = acc;
        for (int y = 0; y < h; ++y) row_cdf[y] = acc > 0.f ? row_cdf[y] / acc : (float)(y + 1) / (float)h;
        row_cdf[h - 1] = 1.f;
    }
    static int upper(const float* c, int n, float r) {
        int i = (int)(std::upper_bound(c, c + n, r) - c);
        return i < n ? i : n - 1;
    }
    // a cell by its row and column CDFs, a uniform point in it, the direction
    // the lookup maps it from, and the solid-angle density
    bool sample(float r1, float r2, V3& dir, float& pdf) const {
        const int y = upper(row_cdf.data(), h, r1);
        const float c0 = y ? row_cdf[y - 1] : 0.f, c1 = row_cdf[y];
        const float fy = std::min(std::max(c1 > c0 ? (r1 - c0) / (c1 - c0) : 0.5f, 0.f), 0.99999994f);
        const float* col = col_cdf.data() + (size_t)y * w;
        const int x = upper(col, w, r2);
        const float d0 = x ? col[x - 1] : 0.f, d1 = col[x];
        const float fx = std::min(std::max(d1 > d0 ? (r2 - d0) / (d1 - d0) : 0.5f, 0.f), 0.99999994f);
        const float wt = weight[(size_t)y * w + x];
        if (!(wt > 0.f) || !(total > 0.f)) return false;
        const float theta = ((float)y + fy) / (float)h * 3.14159f;
        const float phi = (((float)x + fx) / (float)w - 0.5f) * 2.0f * 3.14159f;
        const float st = std::sin(theta), ct = std::cos(theta), sp = std::sin(phi), cp = std::cos(phi);
        if (st < 1e-6f) return false;
        dir = V3(st * cp, ct, st * sp);
        pdf = wt / total * ((float)w * (float)h) / (2.0f * 3.14159f * 3.14159f * st);
        return true;
    }
    float pdf_of(V3 d) const {
        const float theta = std::acos(std::min(std::max(d.y, -1.f), 1.f));
        const float fv = theta / 3.14159f * (float)h;
        const float fu = (std::atan2(d.z, d.x) / 2.0f / 3.14159f + 0.5f) * (float)w;
        if (!(fv >= 0.f && fv < (float)h && fu >= 0.f && fu < (float)w)) return 0.f;
        const int y = (int)fv, x = (int)fu;
        const float st = std::sin(theta);
        if (st < 1e-6f || !(total > 0.f)) return 0.f;
        return weight[(size_t)y * w + x] / total * ((float)w * (float)h) / (2.0f * 3.14159f * 3.14159f * st);
    }
};

struct Scene {
    std::vector<Tri> tris;
    std::vector<Mat> mats;
    std::vector<Tex> texs;
    int env = -1;
    float env_gain = 1.0f;
    EnvTable env_table;
    BVH bvh;
    Lights lights;
};

struct Policy {
    bool nee = true;   // false: RendererPT (src/renderer/rendererpt.cpp:13-59), no light sampling
    float prr = 0.8f;
    bool mis = true;
    int rrdepth = 0;   // RR applies from this vertex index on (0: every vertex, as the reference)
    int maxdepth = 0;  // 0: unbounded (the reference); else vertices 0..maxdepth-1 only
    // renderer=nrc (RendererNRC::trace, src/renderer/renderernrc.cpp:13-185) with
    // the cache never reached (path_lim beyond every path): light samples
    // without MIS, an emitter hit counts only when the previous vertex took
    // no light sample, and a path continues while u < prr
    bool excl = false;
    // envis=1 (no counterpart in the reference): one environment light sample
    // more per light-sampling vertex, balance-heuristic MIS against BSDF misses
    bool envis = false;
};

struct Counters { uint64_t rays = 0, shadow = 0, verts = 0; };

// RendererPTLS::trace (src/renderer/rendererptls.cpp:13-94), recursive as there.
V3 trace(const Scene& S, const Policy& P, Sampler& smp, V3 orig, V3 dir, float light_fac, int depth, Counters& C,
         float env_pb = 0.f) {
    C.rays++;
    BVH::Hit hit = S.bvh.intersect(orig, dir);
    if (hit.tri < 0) {
        if (S.env < 0) return V3(0.f);
        // src/renderer/rendererptls.cpp:24-26, src/scene/envmap.cpp:17-24
        if (P.excl) {
            // renderernrc.cpp:24-25: renderernrc.h's `using namespace std` makes
            // acos / atan2 of a float the float overloads there
            float v = (float)(1 - (double)std::acos(dir.y) / PI_D);
            float u = (float)((double)(std::atan2(dir.z, dir.x) / 2) / PI_D + 0.5);
            return S.texs[S.env].uv(u, v) * S.env_gain;
        }
        float v = (float)(1 - std::acos((double)dir.y) / PI_D);
        float u = (float)(std::atan2((double)dir.z, (double)dir.x) / 2 / PI_D + 0.5);
        V3 e = S.texs[S.env].uv(u, v) * S.env_gain;
        if (env_pb > 0.f && S.env_table.w) e = e * (env_pb / (env_pb + S.env_table.pdf_of(dir)));
        return e;
    }
    const Tri& T = S.tris[hit.tri];
    const Mat& M = S.mats[T.mat];
    V3 wo = -dir;
    V3 normal = tri_normal(T, hit.b1, hit.b2);
    if (M.type == MT_LIGHT) return M.c0 * light_fac;
    V3 uv = tri_uv(T, hit.b1, hit.b2);
    if (dot(normal, dir) > 0 && !mat_transmissive(M)) return V3(0.f, 0.f, 0.f);
    C.verts++;
    V3 hit_pos = orig + dir * hit.t;
    V3 result;
    float fac = 1.0f;
    if (P.nee && mat_nee(M)) {
        if (P.excl) fac = 0.0f;  // is_light_sampled (renderernrc.cpp:139)
        int li = S.lights.pick(smp);
        if (li >= 0) {
            const Tri& LT = S.tris[li];
            // Triangle::sample (src/scene/triangle.cpp:45-55)
            float r1 = smp.random();
            float r2 = smp.random();
            if (r1 + r2 > 1) { r1 = 1 - r1; r2 = 1 - r2; }
            V3 light_pos = (1 - r1 - r2) * LT.p[0] + r1 * LT.p[1] + r2 * LT.p[2];
            V3 light_normal = tri_normal(LT, r1, r2);
            V3 light_vec = light_pos - hit_pos;
            V3 wl = normalized(light_vec);
            V3 light_int = S.mats[LT.mat].c0;
            float light_pdf = S.lights.p();
            float light_omega_pdf = light_pdf * dot(light_vec, light_vec) / fmax_std(1e-6f, dot(light_normal, -wl));
            float brdf_omega_pdf = mat_pdf(M, wo, normal, wl);
            float mis = light_omega_pdf / (light_omega_pdf + brdf_omega_pdf);
            if (!P.mis) mis = 0.5f;
            if (P.excl) mis = 1.0f;  // renderernrc.cpp:155: no MIS weight
            else fac = 1 - mis;
            C.shadow++;
            BVH::Hit sh = S.bvh.intersect(hit_pos + wl * 1e-3f, wl);
            if ((double)sh.t + 2e-3 > (double)norm(light_vec)) {
                V3 brdf = mat_bxdf(M, wo, normal, wl, uv);
                V3 Ll = light_int / norm2(light_vec) * fmax_std(0.0f, dot(light_normal, -wl)) / light_pdf;
                result = result + Ll * brdf * fmax_std(0.0f, dot(normal, normalized(light_pos - hit_pos))) * mis;
            }
        }
    }
    bool env_sampled = false;
    if (P.envis && P.nee && mat_nee(M) && S.env >= 0 && S.env_table.w) {
        env_sampled = true;
        const float r1 = smp.random(), r2 = smp.random();
        V3 we;
        float pe;
        if (S.env_table.sample(r1, r2, we, pe)) {
            const float cosn = dot(normal, we);
            if (cosn > 0.f) {
                const bool last = P.maxdepth > 0 && depth + 1 >= P.maxdepth;
                const float pb = last ? 0.f : mat_pdf(M, wo, normal, we);
                C.shadow++;
                BVH::Hit sh = S.bvh.intersect(hit_pos + we * 1e-3f, we);
                if (sh.tri < 0) {
                    float v = (float)(1 - std::acos((double)we.y) / PI_D);
                    float u = (float)(std::atan2((double)we.z, (double)we.x) / 2 / PI_D + 0.5);
                    V3 L = S.texs[S.env].uv(u, v) * S.env_gain;
                    result = result + mat_bxdf(M, wo, normal, we, uv) * L * (cosn / (pe + pb));
                }
            }
        }
    }
    if (P.maxdepth > 0 && depth + 1 >= P.maxdepth) return result;
    // Russian roulette (src/renderer/rendererptls.cpp:80-83)
    float prr = depth < P.rrdepth ? 1.0f : P.prr;
    float rr = smp.random();
    if (depth >= P.rrdepth && (P.excl ? !(rr < prr) : rr > prr)) return result;  // renderernrc.cpp:162: continue iff u < prr
    V3 wi = mat_sample(M, smp, wo, normal);
    float pdf = mat_pdf(M, wo, normal, wi);
    V3 brdf = mat_bxdf(M, wo, normal, wi, uv);
    V3 Li = trace(S, P, smp, hit_pos + wi * 1e-3f, wi, fac, depth + 1, C, env_sampled ? pdf : 0.f);
    V3 contri = Li * std::fabs(dot(wi, normal)) * brdf / pdf / prr;
    return result + contri;
}

template <class F>
void parallel_for(int n, int threads, F&& f) {
    if (threads <= 1 || n < 2) { for (int i = 0; i < n; ++i) f(i, 0); return; }
    std::atomic<int> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
        th.emplace_back([&, t]() { for (int i; (i = next.fetch_add(1)) < n;) f(i, t); });
    for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

void* port_scene_create(int ntri, const float* pos, const float* uv, const float* nrm, const int* tri_mat,
                        int nmat, const int* mat_i, const float* mat_f, int ntex, const int* tex_wh,
                        const float* tex_data, int env_tex, float env_gain, int build_threads) {
    (void)build_threads;
    auto* S = new Scene();
    S->texs.resize(ntex);
    size_t off = 0;
    for (int i = 0; i < ntex; ++i) {
        Tex& t = S->texs[i];
        t.w = tex_wh[2 * i]; t.h = tex_wh[2 * i + 1];
        t.px.resize((size_t)t.w * t.h);
        for (size_t k = 0; k < t.px.size(); ++k) t.px[k] = V3(tex_data[off + 3 * k], tex_data[off + 3 * k + 1], tex_data[off + 3 * k + 2]);
        off += t.px.size() * 3;
    }
    S->mats.resize(nmat);
    for (int m = 0; m < nmat; ++m) {
        Mat& M = S->mats[m];
        const int* I = mat_i + 4 * m; const float* F = mat_f + 12 * m;
        M.type = I[0];
        M.c0 = V3(F[0], F[1], F[2]); M.c1 = V3(F[3], F[4], F[5]);
        M.alpha = F[6]; M.ior = F[7]; M.ns = F[8];
        M.t0 = (I[1] >= 0 && I[1] < ntex) ? &S->texs[I[1]] : nullptr;
        M.t1 = (I[2] >= 0 && I[2] < ntex) ? &S->texs[I[2]] : nullptr;
    }
    S->tris.resize(ntri);
    for (int i = 0; i < ntri; ++i) {
        Tri& T = S->tris[i];
        for (int v = 0; v < 3; ++v) {
            T.p[v] = V3(pos[9 * i + 3 * v], pos[9 * i + 3 * v + 1], pos[9 * i + 3 * v + 2]);
            T.t[v] = V3(uv[6 * i + 2 * v], uv[6 * i + 2 * v + 1], 0.0f);
            T.n[v] = V3(nrm[9 * i + 3 * v], nrm[9 * i + 3 * v + 1], nrm[9 * i + 3 * v + 2]);
        }
        // Triangle constructor: face normal when n0 is (nearly) zero (src/scene/triangle.cpp:12-25)
        if ((double)norm2(T.n[0]) < 1e-4) {
            T.n[0] = normalized(cross(T.p[1] - T.p[0], T.p[2] - T.p[0]));
            T.n[1] = T.n[0]; T.n[2] = T.n[0];
        }
        T.mat = tri_mat[i];
        T.pmin = vmin(T.p[0], vmin(T.p[1], T.p[2]));
        T.pmax = vmax(T.p[0], vmax(T.p[1], T.p[2]));
    }
    S->env = env_tex; S->env_gain = env_gain;
    if (env_tex >= 0 && env_tex < ntex) S->env_table.build(S->texs[env_tex]);
    S->lights.build(S->tris, S->mats);
    S->bvh.build(S->tris);
    return S;
}

void port_scene_destroy(void* s) { delete static_cast<Scene*>(s); }

// Replaces the material parameters (same count, same types) without
// rebuilding the BVH; for finite differences over material parameters. The
// emitter table depends only on the geometry and the types (radiance is
// read from the materials where it is used), so it stays. Returns 0, or -1
// on a count or type change.
int port_scene_set_materials(void* s, int nmat, const int* mat_i, const float* mat_f) {
    auto* S = static_cast<Scene*>(s);
    if (nmat != (int)S->mats.size()) return -1;
    for (int m = 0; m < nmat; ++m)
        if (mat_i[4 * m] != S->mats[m].type) return -1;
    for (int m = 0; m < nmat; ++m) {
        Mat& M = S->mats[m];
        const float* F = mat_f + 12 * m;
        M.c0 = V3(F[0], F[1], F[2]); M.c1 = V3(F[3], F[4], F[5]);
        M.alpha = F[6]; M.ior = F[7]; M.ns = F[8];
    }
    return 0;
}

int port_bvh_export(void* s, float* box, int* kids, int* leaf_first, int* leaf_count, int* leaf_tris, int* n_leaf_tris) {
    auto* S = static_cast<Scene*>(s);
    int nn = 0, nt = 0;
    std::function<int(int)> walk = [&](int ni) -> int {
        const Node& n = S->bvh.nodes[ni];
        int id = nn++;
        if (box) for (int k = 0; k < 3; ++k) { box[6 * id + k] = n.pmin[k]; box[6 * id + 3 + k] = n.pmax[k]; }
        if (n.left < 0) {
            if (kids) { kids[2 * id] = -1; kids[2 * id + 1] = -1; }
            if (leaf_first) leaf_first[id] = nt;
            if (leaf_count) leaf_count[id] = (int)n.prims.size();
            for (int p : n.prims) { if (leaf_tris) leaf_tris[nt] = p; ++nt; }
        } else {
            int l = walk(n.left), r = walk(n.right);
            if (kids) { kids[2 * id] = l; kids[2 * id + 1] = r; }
            if (leaf_first) leaf_first[id] = -1;
            if (leaf_count) leaf_count[id] = 0;
        }
        return id;
    };
    if (S->bvh.root >= 0) walk(S->bvh.root);
    if (n_leaf_tris) *n_leaf_tris = nt;
    return nn;
}

void port_intersect(void* s, int n, const float* o, const float* d, int* tri, float* t, float* b1, float* b2, int threads) {
    auto* S = static_cast<Scene*>(s);
    parallel_for(n, threads, [&](int i, int) {
        BVH::Hit h = S->bvh.intersect(V3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), V3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
        tri[i] = h.tri; t[i] = h.t; b1[i] = h.b1; b2[i] = h.b2;
    });
}

void port_camera_rays(const char* params, int n, const float* fx, const float* fy, float* dir, float* origin) {
    Config c(params);
    Cam cam(c);
    int w = c.i("imgw", 1), h = c.i("imgh", 1);
    for (int i = 0; i < n; ++i) {
        V3 r = cam.ray(fx[i], fy[i], (float)w, (float)h);
        dir[3 * i] = r.x; dir[3 * i + 1] = r.y; dir[3 * i + 2] = r.z;
        origin[3 * i] = cam.pos.x; origin[3 * i + 1] = cam.pos.y; origin[3 * i + 2] = cam.pos.z;
    }
}

void port_render_samples(void* s, const char* params, int npix, const int* pix_xy, int sample0, int spp,
                         uint64_t seed, float* out, int threads, uint64_t* counters) {
    auto* S = static_cast<Scene*>(s);
    Config c(params);
    Cam cam(c);
    Policy P;
    P.prr = c.f("prr", 0.8f);
    P.mis = c.i("mis", 1) != 0;
    P.rrdepth = c.i("rrdepth", 0);
    P.maxdepth = c.i("maxdepth", 0);
    bool coin = false;
    {
        auto it = c.mp.find("renderer");
        P.nee = !(it != c.mp.end() && it->second == "pt");
        P.excl = it != c.mp.end() && it->second == "nrc";
        coin = P.excl;
    }
    P.envis = c.i("envis", 0) != 0;
    int w = c.i("imgw", 1), h = c.i("imgh", 1);
    int nth = threads < 1 ? 1 : threads;
    std::vector<Counters> C(nth);
    parallel_for(npix, nth, [&](int p, int tid) {
        int x = pix_xy[2 * p], y = pix_xy[2 * p + 1];
        for (int i = 0; i < spp; ++i) {
            PhiloxSampler smp(seed, (uint32_t)(y * w + x), (uint32_t)(sample0 + i));
            float jx = smp.random();
            float jy = smp.random();
            V3 dir = cam.ray((float)x + jx, (float)y + jy, (float)w, (float)h);
            if (coin) (void)smp.random();  // RendererNRC::render's training coin (renderernrc.cpp:255)
            V3 L = trace(*S, P, smp, cam.pos, dir, 1.0f, 0, C[tid]);
            L = vmax(V3(0.0f), L);  // max(0.0f, trace(...)) (rendererptls.cpp:173)
            float* o = out + ((size_t)p * spp + i) * 3;
            o[0] = L.x; o[1] = L.y; o[2] = L.z;
        }
    });
    if (counters) {
        counters[0] = counters[1] = counters[2] = 0;
        for (auto& c2 : C) { counters[0] += c2.rays; counters[1] += c2.shadow; counters[2] += c2.verts; }
    }
}

void port_material_probe(void* s, int mat, int n, const float* wo, const float* nrm, const float* wi, const float* uv,
                         const float* u, float* f, float* pdf, float* wi_s) {
    auto* S = static_cast<Scene*>(s);
    const Mat& M = S->mats[mat];
    for (int i = 0; i < n; ++i) {
        V3 a(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), nn(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        V3 b(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]), t(uv[3 * i], uv[3 * i + 1], uv[3 * i + 2]);
        V3 ff = mat_bxdf(M, a, nn, b, t);
        pdf[i] = mat_pdf(M, a, nn, b);
        ListSampler ls(u + 4 * i, 4);
        V3 ws = mat_sample(M, ls, a, nn);
        f[3 * i] = ff.x; f[3 * i + 1] = ff.y; f[3 * i + 2] = ff.z;
        wi_s[3 * i] = ws.x; wi_s[3 * i + 1] = ws.y; wi_s[3 * i + 2] = ws.z;
    }
}

float port_light_pick(void* s, int n, const float* u, int* tri) {
    auto* S = static_cast<Scene*>(s);
    for (int i = 0; i < n; ++i) { ListSampler ls(u + i, 1); tri[i] = S->lights.pick(ls); }
    return S->lights.p();
}

void port_texture_lookup(void* s, int mat, int kind, int n, const float* uvs, float* rgb) {
    auto* S = static_cast<Scene*>(s);
    const Tex* t = kind == 1 ? (S->env >= 0 ? &S->texs[S->env] : nullptr) : S->mats[mat].t0;
    for (int i = 0; i < n; ++i) {
        V3 c = t ? t->uv(uvs[2 * i], uvs[2 * i + 1]) : V3(0.f);
        rgb[3 * i] = c.x; rgb[3 * i + 1] = c.y; rgb[3 * i + 2] = c.z;
    }
}

}  // extern "C"
