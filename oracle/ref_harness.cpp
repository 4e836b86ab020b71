// Oracle harness around the reference's own ptnee sources.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled together with the
// unmodified reference sources (src/renderer/rendererptls.cpp,
// src/renderer/rendererpt.cpp, src/renderer/renderer.cpp, src/hierarchy/*.cpp, src/material/*.cpp,
// src/scene/*.cpp, src/sampler/*.cpp, src/math/vec3.cpp,
// src/utils/config.cpp) into oracle/_ref/libnuray_ref.so by oracle/Makefile.
// Only the tests and the golden-fixture script load it; nothing in the
// product links it.
//
// It exposes, through a C ABI:
//  * scene construction through the reference Loader (scene description +
//    OBJ/MTL) or from flat arrays (procedural scenes), followed by the
//    reference's Renderer::prepare (src/renderer/renderer.cpp:30-39);
//  * the reference BVH query Renderer::intersect (src/renderer/renderer.cpp:10-28);
//  * the reference estimators RendererPTLS::trace (src/renderer/rendererptls.cpp:13-94)
//    and, for renderer=pt, RendererPT::trace (src/renderer/rendererpt.cpp:13-59),
//    driven by the per-pixel sample loop of RendererPTLS::render
//    (src/renderer/rendererptls.cpp:165-175), with the glibc rand() sampler
//    replaced by a counter-based Philox stream keyed by (pixel, sample);
//  * the reference BVH tree, exported in depth-first order;
//  * the reference Material virtuals on caller-given directions.
#include "../renderer/rendererptls.h"
#include "../renderer/rendererpt.h"
#include "../renderer/renderernrc.h"
#include "../scene/loader.h"
#include "../material/matlambert.h"
#include "../material/matggxrefl.h"
#include "../material/matggx.h"
#include "../material/matglass.h"
#include "../material/matblinnphong.h"
#include "../material/matlight.h"
#include "philox.h"

#include <atomic>
#include <memory>
#include <thread>

namespace {

enum { MT_LAMBERT = 0, MT_GGXR = 1, MT_GGX = 2, MT_GLASS = 3, MT_BLINNPHONG = 4, MT_LIGHT = 5 };

class PhiloxSampler : public Sampler {
public:
    nr_path_stream s;
    PhiloxSampler(uint64_t seed, uint32_t pixel, uint32_t sample) { nr_stream_init(&s, seed, pixel, sample, 0); }
    float random() override { return nr_stream_next(&s); }
};

// Replays a caller-given sequence of uniforms (for per-material probes).
class ListSampler : public Sampler {
public:
    const float* u; int n; int i = 0;
    ListSampler(const float* u_, int n_) : u(u_), n(n_) {}
    float random() override { return i < n ? u[i++] : 0.5f; }
};

// RendererPT::trace (src/renderer/rendererpt.cpp:13-59), the plain path
// tracer, driven with the ptnee renderer's BVH and light sampler.
class OraclePT : public RendererPT {
public:
    using RendererPT::trace;
};

class OracleNRC : public RendererNRC {
public:
    using RendererNRC::trace;
};

class OracleRenderer : public RendererPTLS {
public:
    using RendererPTLS::trace;
    std::tuple<float, float, float, const Triangle*> query(const vec3& o, const vec3& d, const std::vector<Triangle>& tris) {
        return intersect(o, d, tris, bvh_);
    }
    BVH& bvh() { return bvh_; }
    LightSampler& lights() { return light_sampler_; }
};

struct RefScene {
    Loader loader;
    std::vector<Triangle> own_tris;
    std::vector<Material*> own_mats;
    std::vector<Texture*> own_tex;
    std::vector<Triangle>* tris = nullptr;
    std::vector<const Material*> mats;          // first-appearance order
    std::vector<int> tri_mat;                   // per triangle index into mats
    OracleRenderer renderer;
    OraclePT plain;
    OracleNRC nrc_renderer;
    std::unique_ptr<NeuralRadianceCache> nrc;  // RendererNRC::render's cache, shape [64, 64, 64, 64, 3]
    Texture* env_tex = nullptr;
    Envmap* env = nullptr;
    ~RefScene() {
        for (auto* m : own_mats) delete m;
        for (auto* t : own_tex) delete t;
        delete env;
        delete env_tex;
    }
    void finish() {
        std::map<const Material*, int> idx;
        tri_mat.resize(tris->size());
        for (size_t i = 0; i < tris->size(); ++i) {
            const Material* m = (*tris)[i].mat;
            auto it = idx.find(m);
            if (it == idx.end()) { it = idx.emplace(m, (int)mats.size()).first; mats.push_back(m); }
            tri_mat[i] = it->second;
        }
        renderer.prepare(*tris);
    }
};

BVHNode* bvh_root(BVH& b) {
    static_assert(sizeof(BVH) == sizeof(BVHNode*), "BVH holds only its root pointer");
    return *reinterpret_cast<BVHNode**>(&b);
}

Camera make_camera(Config& config) {
    // src/cmd/cmd.cpp:99-101
    vec3 e = config.getValueVec3("cameuler", {0, 0, 0});
    std::streambuf* old = std::cout.rdbuf(nullptr);  // Camera::fromEuler prints gaze/up
    Camera c(config.getValueFloat("camfov", 90.0f), config.getValueFloat("camasp", 1.0f),
             config.getValueVec3("campos", {0, 0, 0}), e[0], e[1], e[2]);
    std::cout.rdbuf(old);
    return c;
}

template <class F>
void parallel_for(int n, int threads, F&& f) {
    if (threads <= 1 || n < 2) { for (int i = 0; i < n; ++i) f(i); return; }
    std::atomic<int> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
        th.emplace_back([&]() { for (int i; (i = next.fetch_add(1)) < n;) f(i); });
    for (auto& x : th) x.join();
}

}  // namespace

extern "C" {

void* ref_scene_from_desc(const char* desc) {
    auto* s = new RefScene();
    std::streambuf* old = std::cerr.rdbuf(nullptr);
    s->loader.fromSceneDescription(desc);
    std::cerr.rdbuf(old);
    s->tris = &s->loader.getTriangles();
    s->finish();
    return s;
}

// Flat-array scene. pos/uv/nrm: 9/6/9 floats per triangle (vertex-major);
// mat_i: 4 ints per material (type, kd texture, ks texture, unused);
// mat_f: 12 floats per material (c0 rgb, c1 rgb, alpha, ior, Ns, ...);
// textures: tex_wh 2 ints each, tex_data concatenated rgb floats.
void* ref_scene_from_arrays(int ntri, const float* pos, const float* uv, const float* nrm, const int* tri_mat,
                            int nmat, const int* mat_i, const float* mat_f,
                            int ntex, const int* tex_wh, const float* tex_data,
                            int env_tex, float env_gain) {
    auto* s = new RefScene();
    std::vector<const float*> tex_ptr(ntex);
    size_t off = 0;
    for (int i = 0; i < ntex; ++i) { tex_ptr[i] = tex_data + off; off += (size_t)tex_wh[2 * i] * tex_wh[2 * i + 1] * 3; }
    auto fill = [&](Texture& t, int id) {
        int w = tex_wh[2 * id], h = tex_wh[2 * id + 1];
        t = Texture(w, h);
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const float* p = tex_ptr[id] + ((size_t)y * w + x) * 3;
                t.pixel(x, y) = vec3(p[0], p[1], p[2]);
            }
    };
    for (int m = 0; m < nmat; ++m) {
        const int* I = mat_i + 4 * m;
        const float* F = mat_f + 12 * m;
        vec3 c0(F[0], F[1], F[2]), c1(F[3], F[4], F[5]);
        Material* mat = nullptr;
        switch (I[0]) {
            case MT_LAMBERT: { auto* x = new MatLambert(c0); if (I[1] >= 0) { x->usetex_Kd_ = true; fill(x->map_Kd_, I[1]); } mat = x; break; }
            case MT_GGXR: { auto* x = new MatGGXRefl(c0, F[6]); if (I[1] >= 0) { x->usetex_Kd_ = true; fill(x->map_Kd_, I[1]); } mat = x; break; }
            case MT_GGX: { auto* x = new MatGGX(c0, F[6], F[7]); if (I[1] >= 0) { x->usetex_Kd_ = true; fill(x->map_Kd_, I[1]); } mat = x; break; }
            case MT_GLASS: { auto* x = new MatGlass(c0, F[7]); if (I[1] >= 0) { x->usetex_F0_ = true; fill(x->map_F0_, I[1]); } mat = x; break; }
            case MT_BLINNPHONG: {
                auto* x = new MatBlinnPhong(c0, c1, F[8]);
                if (I[1] >= 0) { x->usetex_Kd_ = true; fill(x->map_Kd_, I[1]); }
                if (I[2] >= 0) { x->usetex_Ks_ = true; fill(x->map_Ks_, I[2]); }
                mat = x; break;
            }
            default: mat = new MatLight(c0); break;
        }
        s->own_mats.push_back(mat);
    }
    s->own_tris.reserve(ntri);
    for (int i = 0; i < ntri; ++i) {
        const float* P = pos + 9 * i; const float* T = uv + 6 * i; const float* N = nrm + 9 * i;
        s->own_tris.push_back(Triangle(vec3(P[0], P[1], P[2]), vec3(P[3], P[4], P[5]), vec3(P[6], P[7], P[8]),
                                       vec3(T[0], T[1], 0.0f), vec3(T[2], T[3], 0.0f), vec3(T[4], T[5], 0.0f),
                                       vec3(N[0], N[1], N[2]), vec3(N[3], N[4], N[5]), vec3(N[6], N[7], N[8]),
                                       s->own_mats[tri_mat[i]]));
    }
    s->tris = &s->own_tris;
    if (env_tex >= 0) {
        s->env_tex = new Texture();
        fill(*s->env_tex, env_tex);
        s->env = new Envmap(s->env_tex, env_gain);
    }
    s->finish();
    // materials in first-appearance order may differ from the caller's table;
    // expose the caller's indices instead.
    s->mats.assign(s->own_mats.begin(), s->own_mats.end());
    for (int i = 0; i < ntri; ++i) s->tri_mat[i] = tri_mat[i];
    return s;
}

void ref_scene_destroy(void* h) { delete static_cast<RefScene*>(h); }

int ref_scene_num_tris(void* h) { return (int)static_cast<RefScene*>(h)->tris->size(); }
int ref_scene_num_mats(void* h) { return (int)static_cast<RefScene*>(h)->mats.size(); }

// Triangles in loader order: 9 pos, 6 uv, 9 normal floats and the material index.
void ref_scene_get_tris(void* h, float* pos, float* uv, float* nrm, int* mat) {
    auto* s = static_cast<RefScene*>(h);
    for (size_t i = 0; i < s->tris->size(); ++i) {
        const Triangle& t = (*s->tris)[i];
        for (int v = 0; v < 3; ++v)
            for (int k = 0; k < 3; ++k) { pos[9 * i + 3 * v + k] = t.p[v][k]; nrm[9 * i + 3 * v + k] = t.n[v][k]; }
        for (int v = 0; v < 3; ++v) { uv[6 * i + 2 * v] = t.t[v][0]; uv[6 * i + 2 * v + 1] = t.t[v][1]; }
        mat[i] = s->tri_mat[i];
    }
}

// Material table in the same 4-int/12-float layout as ref_scene_from_arrays.
void ref_scene_get_mats(void* h, int* mat_i, float* mat_f) {
    auto* s = static_cast<RefScene*>(h);
    for (size_t m = 0; m < s->mats.size(); ++m) {
        int* I = mat_i + 4 * m; float* F = mat_f + 12 * m;
        for (int k = 0; k < 4; ++k) I[k] = -1;
        for (int k = 0; k < 12; ++k) F[k] = 0.0f;
        const Material* p = s->mats[m];
        auto put = [&](const vec3& a, int o) { F[o] = a[0]; F[o + 1] = a[1]; F[o + 2] = a[2]; };
        if (auto* x = dynamic_cast<const MatLambert*>(p)) { I[0] = MT_LAMBERT; put(x->Kd_, 0); I[1] = x->usetex_Kd_ ? 0 : -1; }
        else if (auto* x = dynamic_cast<const MatGGXRefl*>(p)) { I[0] = MT_GGXR; put(x->Kd_, 0); F[6] = x->alpha_; I[1] = x->usetex_Kd_ ? 0 : -1; }
        else if (auto* x = dynamic_cast<const MatGGX*>(p)) { I[0] = MT_GGX; put(x->Kd_, 0); F[6] = x->alpha_; F[7] = x->ior_; I[1] = x->usetex_Kd_ ? 0 : -1; }
        else if (auto* x = dynamic_cast<const MatGlass*>(p)) { I[0] = MT_GLASS; put(x->F0_, 0); F[7] = x->Ior_; I[1] = x->usetex_F0_ ? 0 : -1; }
        else if (auto* x = dynamic_cast<const MatBlinnPhong*>(p)) { I[0] = MT_BLINNPHONG; put(x->Kd_, 0); put(x->Ks_, 3); F[8] = x->Ns_; I[1] = x->usetex_Kd_ ? 0 : -1; I[2] = x->usetex_Ks_ ? 0 : -1; }
        else if (auto* x = dynamic_cast<const MatLight*>(p)) { I[0] = MT_LIGHT; put(x->Ke_, 0); }
    }
}

// Depth-first (left child first) export of the reference BVH.
// Per node: box[6] (p_min, p_max), kids[2] (-1 for a leaf), leaf_first,
// leaf_count into leaf_tris (triangle indices in leaf order).
// Returns the node count; call with nulls to size the buffers.
int ref_bvh_export(void* h, float* box, int* kids, int* leaf_first, int* leaf_count, int* leaf_tris, int* n_leaf_tris) {
    auto* s = static_cast<RefScene*>(h);
    BVHNode* root = bvh_root(s->renderer.bvh());
    const Triangle* base = s->tris->data();
    int nn = 0, nt = 0;
    std::function<int(BVHNode*)> walk = [&](BVHNode* p) -> int {
        int id = nn++;
        if (box) for (int k = 0; k < 3; ++k) { box[6 * id + k] = p->p_min[k]; box[6 * id + 3 + k] = p->p_max[k]; }
        if (!p->left_child && !p->right_child) {
            if (kids) { kids[2 * id] = -1; kids[2 * id + 1] = -1; }
            if (leaf_first) leaf_first[id] = nt;
            if (leaf_count) leaf_count[id] = (int)p->primitives.size();
            for (auto* t : p->primitives) { if (leaf_tris) leaf_tris[nt] = (int)(t - base); ++nt; }
        } else {
            int l = walk(p->left_child);
            int r = walk(p->right_child);
            if (kids) { kids[2 * id] = l; kids[2 * id + 1] = r; }
            if (leaf_first) leaf_first[id] = -1;
            if (leaf_count) leaf_count[id] = 0;
        }
        return id;
    };
    if (root) walk(root);
    if (n_leaf_tris) *n_leaf_tris = nt;
    return nn;
}

// BVH::intersection for n rays (src/hierarchy/bvh.cpp:129-137). tri = -1 on a miss.
void ref_intersect(void* h, int n, const float* o, const float* d, int* tri, float* t, float* b1, float* b2, int threads) {
    auto* s = static_cast<RefScene*>(h);
    const Triangle* base = s->tris->data();
    parallel_for(n, threads, [&](int i) {
        auto [tt, u, v, obj] = s->renderer.query(vec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]),
                                                 vec3(d[3 * i], d[3 * i + 1], d[3 * i + 2]), *s->tris);
        tri[i] = obj ? (int)(obj - base) : -1;
        t[i] = tt; b1[i] = u; b2[i] = v;
    });
}

// Camera::generateRay for the given film coordinates (src/scene/camera.cpp:24-32).
void ref_camera_rays(const char* params, int n, const float* fx, const float* fy, float* dir, float* origin) {
    Config config(params);
    Camera cam = make_camera(config);
    int w = config.getValueInt("imgw", 1), hh = config.getValueInt("imgh", 1);
    for (int i = 0; i < n; ++i) {
        vec3 r = cam.generateRay(fx[i], fy[i], w, hh);
        for (int k = 0; k < 3; ++k) { dir[3 * i + k] = r[k]; origin[3 * i + k] = cam.pos[k]; }
    }
}

// Per-sample radiance of the reference estimator, after the per-sample
// max(0, .) of src/renderer/rendererptls.cpp:173. For each listed pixel and
// each sample in [sample0, sample0+spp): jitter x, jitter y, then trace().
// out: npix * spp * 3 floats, sample-major within a pixel.
void ref_render_samples(void* h, const char* params, int npix, const int* pix_xy, int sample0, int spp,
                        uint64_t seed, float* out, int threads) {
    auto* s = static_cast<RefScene*>(h);
    Config config(params);
    Camera cam = make_camera(config);
    int w = config.getValueInt("imgw", 1), hh = config.getValueInt("imgh", 1);
    std::streambuf* old = std::cerr.rdbuf(nullptr);  // getValueStr reports missing keys on stderr
    const std::string rname = config.getValueStr("renderer", "ptnee");
    const bool plain = rname == "pt", nrc_mode = rname == "nrc";
    std::cerr.rdbuf(old);
    if (nrc_mode && !s->nrc) s->nrc = std::make_unique<NeuralRadianceCache>(std::vector<int>{64, 64, 64, 64, 3});
    parallel_for(npix, threads, [&](int p) {
        int x = pix_xy[2 * p], y = pix_xy[2 * p + 1];
        Config local = config;  // getValue* builds stringstreams; keep threads apart
        for (int i = 0; i < spp; ++i) {
            PhiloxSampler smp(seed, (uint32_t)(y * w + x), (uint32_t)(sample0 + i));
            float jx = smp.random();
            float jy = smp.random();
            vec3 ray_dir = cam.generateRay(x + jx, y + jy, w, hh);
            vec3 L;
            if (nrc_mode) {
                // RendererNRC::render (src/renderer/renderernrc.cpp:250-255): the
                // training coin follows the jitter; no training here
                (void)smp.random();
                L = max(0.0f, s->nrc_renderer.trace(local, *s->nrc, 0, false, smp, cam.pos, ray_dir, *s->tris,
                                                    s->renderer.lights(), s->renderer.bvh(), true, s->env));
            } else {
                L = plain ? max(0.0f, s->plain.trace(local, smp, cam.pos, ray_dir, *s->tris, s->renderer.lights(),
                                                     s->renderer.bvh(), s->env))
                          : max(0.0f, s->renderer.trace(local, smp, cam.pos, ray_dir, *s->tris, s->renderer.lights(),
                                                        s->renderer.bvh(), true, s->env));
            }
            float* o = out + ((size_t)p * spp + i) * 3;
            o[0] = L[0]; o[1] = L[1]; o[2] = L[2];
        }
    });
}

// Material virtuals on caller-given inputs. For each of n queries:
// wo, normal, wi, uv (3 floats each). Writes f (3), pdf (1), and a sampled
// direction (3) drawn with the uniforms u[4*i .. 4*i+3].
void ref_material_probe(void* h, int mat, int n, const float* wo, const float* nrm, const float* wi, const float* uv,
                        const float* u, float* f, float* pdf, float* wi_s) {
    auto* s = static_cast<RefScene*>(h);
    const Material* m = s->mats[mat];
    for (int i = 0; i < n; ++i) {
        vec3 a(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), nn(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        vec3 b(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]), t(uv[3 * i], uv[3 * i + 1], uv[3 * i + 2]);
        vec3 ff = m->bxdf(a, nn, b, t);
        pdf[i] = m->pdf(a, nn, b);
        ListSampler ls(u + 4 * i, 4);
        vec3 ws = m->sampleBxdf(ls, a, nn);
        for (int k = 0; k < 3; ++k) { f[3 * i + k] = ff[k]; wi_s[3 * i + k] = ws[k]; }
    }
}

// LightSampler internals (src/sampler/lightsampler.cpp:4-58, 100-103):
// picks an emitter for each uniform and reports p().
float ref_light_pick(void* h, int n, const float* u, int* tri) {
    auto* s = static_cast<RefScene*>(h);
    const Triangle* base = s->tris->data();
    for (int i = 0; i < n; ++i) {
        ListSampler ls(u + i, 1);
        const Triangle* t = s->renderer.lights().sampleLight(ls);
        tri[i] = t ? (int)(t - base) : -1;
    }
    return s->renderer.lights().p();
}

// Texture::pixelUV on a scene texture-backed material (bilinear, wrap, v flip),
// src/scene/texture.cpp:61-72. kind 0: the material's Kd map; 1: the env map.
void ref_texture_lookup(void* h, int mat, int kind, int n, const float* uvs, float* rgb) {
    auto* s = static_cast<RefScene*>(h);
    const Texture* tex = nullptr;
    if (kind == 1) tex = s->env_tex;
    else {
        const Material* p = s->mats[mat];
        if (auto* x = dynamic_cast<const MatLambert*>(p)) tex = &x->map_Kd_;
        else if (auto* x = dynamic_cast<const MatGGXRefl*>(p)) tex = &x->map_Kd_;
        else if (auto* x = dynamic_cast<const MatGGX*>(p)) tex = &x->map_Kd_;
        else if (auto* x = dynamic_cast<const MatGlass*>(p)) tex = &x->map_F0_;
        else if (auto* x = dynamic_cast<const MatBlinnPhong*>(p)) tex = &x->map_Kd_;
    }
    for (int i = 0; i < n; ++i) {
        vec3 c = tex ? tex->pixelUV(uvs[2 * i], uvs[2 * i + 1]) : vec3(0.0f);
        rgb[3 * i] = c[0]; rgb[3 * i + 1] = c[1]; rgb[3 * i + 2] = c[2];
    }
}

}  // extern "C"
