// nuray_renderer.hpp — C++17 adapter with the shape of the reference's
// Renderer interface (src/renderer/renderer.h:15-35), implemented over the
// C ABI of libnuray_gpu.so (nuray.h). Header-only.
//
//   reference                                   this adapter
//   Renderer::prepare(const vector<Triangle>&)  RendererGPU::prepare(const vector<Triangle>&, materials, ...)
//   RendererPTLS::render(camera, triangles,     RendererGPU::render(camera, triangles, Image&, Config&,
//     QImage&, Config&, display_cb, con_flag,     display_cb, con_flag, progress_cb, mutex, env)
//     progress_cb, QMutex&, const Envmap*)
//   Renderer::intersect(o, d, triangles, bvh)   RendererGPU::intersect(o, d) -> (t, b1, b2, index)
//
// Differences forced by the boundary: triangles refer to materials by index
// (the reference holds Material pointers), the framebuffer is an 8-bit RGB
// Image instead of a QImage (Qt is not a dependency), and errors surface as
// nr::Error exceptions carrying the NR_ERR_* code instead of stderr prints.
#pragma once
#include <atomic>
#include <cstdint>
#include <functional>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "nuray.h"

namespace nr {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void check(int code) {
    if (code == NR_OK) return;
    char buf[1024];
    nr_last_error(buf, sizeof(buf));
    throw Error(code, buf);
}

// struct Triangle (src/scene/triangle.h:8-36) with a material index.
struct Triangle {
    float p[3][3];
    float t[3][2];
    float n[3][3];
    int32_t mat;
};

// 8-bit RGB framebuffer standing in for QImage::Format_RGB888.
struct Image {
    int width = 0, height = 0;
    std::vector<uint8_t> rgb;   // row-major, 3 bytes per pixel
    std::vector<float> hdr;     // linear per-pixel mean, 3 floats per pixel
};

// The reference's key=value parameter map (src/utils/config.h:7-22); only
// the string is handed to the library, which parses it with the same rules.
class ParamString {
public:
    ParamString() = default;
    explicit ParamString(std::string s) : s_(std::move(s)) {}
    void addItem(const std::string& kv) { s_ += (s_.empty() ? "" : " ") + kv; }
    const std::string& str() const { return s_; }

private:
    std::string s_;
};

class RendererGPU {
public:
    RendererGPU() = default;
    ~RendererGPU() { reset(); }
    RendererGPU(const RendererGPU&) = delete;
    RendererGPU& operator=(const RendererGPU&) = delete;

    // Renderer::prepare: flattens, builds the BVH and the emitter table and
    // uploads everything to the current CUDA device.
    void prepare(const std::vector<Triangle>& tris, const std::vector<nr_material>& mats,
                 const std::vector<int32_t>& tex_wh = {}, const std::vector<float>& tex_data = {},
                 int32_t env_tex = -1, float env_gain = 1.0f) {
        reset();
        std::vector<float> pos(9 * tris.size()), uv(6 * tris.size()), nrm(9 * tris.size());
        std::vector<int32_t> mat(tris.size());
        for (size_t i = 0; i < tris.size(); ++i) {
            for (int v = 0; v < 3; ++v)
                for (int k = 0; k < 3; ++k) { pos[9 * i + 3 * v + k] = tris[i].p[v][k]; nrm[9 * i + 3 * v + k] = tris[i].n[v][k]; }
            for (int v = 0; v < 3; ++v) { uv[6 * i + 2 * v] = tris[i].t[v][0]; uv[6 * i + 2 * v + 1] = tris[i].t[v][1]; }
            mat[i] = tris[i].mat;
        }
        nr_scene_desc d{};
        d.num_tris = (int32_t)tris.size();
        d.pos = pos.data(); d.uv = uv.data(); d.nrm = nrm.data(); d.mat = mat.data();
        d.num_mats = (int32_t)mats.size(); d.mats = mats.data();
        d.num_tex = (int32_t)(tex_wh.size() / 2);
        d.tex_wh = tex_wh.empty() ? nullptr : tex_wh.data();
        d.tex_data = tex_data.empty() ? nullptr : tex_data.data();
        d.env_tex = env_tex; d.env_gain = env_gain;
        check(nr_scene_create(&d, &scene_));
    }

    // Loads the reference's scene-description text (Loader::fromSceneDescription).
    void prepare(const std::string& scene_desc) {
        reset();
        check(nr_scene_load(scene_desc.c_str(), &scene_));
    }

    // RendererPTLS::render. Blocks until the image is done. con_flag is
    // polled between wavefront batches (set it to 0 to cancel, as in the
    // reference); progress is reported in percent. The image is written
    // under fb_mutex. Throws nr::Error(NR_ERR_CANCELLED) when cancelled.
    void render(const nr_camera& camera, Image& img, const ParamString& config,
                std::function<void(bool)> display_cb, std::atomic<int>& con_flag,
                std::function<void(float)> progress_cb, std::mutex& fb_mutex) {
        need_scene();
        int w = param_int(config.str(), "imgw", 1), h = param_int(config.str(), "imgh", 1);
        Image out;
        out.width = w; out.height = h;
        out.rgb.resize((size_t)w * h * 3);
        out.hdr.resize((size_t)w * h * 3);
        if (display_cb) display_cb(false);
        volatile int32_t cancel = 1;
        struct Ctx { std::function<void(float)>* cb; std::atomic<int>* flag; volatile int32_t* cancel; } ctx{&progress_cb, &con_flag, &cancel};
        auto prog = [](float pct, void* user) {
            Ctx* c = static_cast<Ctx*>(user);
            if (*c->cb) (*c->cb)(pct);
            if (c->flag->load() == 0) *c->cancel = 0;
        };
        check(nr_render(scene_, &camera, config.str().c_str(), out.hdr.data(), out.rgb.data(), &cancel, prog, &ctx));
        {
            std::lock_guard<std::mutex> lk(fb_mutex);
            img = std::move(out);
        }
        con_flag = 0;
        if (display_cb) display_cb(true);
    }

    // Renderer::intersect -> (t, b1, b2, triangle index or -1).
    std::tuple<float, float, float, int32_t> intersect(const float o[3], const float d[3]) {
        need_scene();
        int32_t tri;
        float t, b1, b2;
        check(nr_intersect(scene_, 1, o, d, &tri, &t, &b1, &b2, 0));
        return {t, b1, b2, tri};
    }

    nr_scene* scene() const { return scene_; }

    static nr_camera camera(const ParamString& config) {
        nr_camera c;
        check(nr_camera_from_params(config.str().c_str(), &c));
        return c;
    }

private:
    nr_scene* scene_ = nullptr;
    void reset() {
        if (scene_) nr_scene_destroy(scene_);
        scene_ = nullptr;
    }
    void need_scene() const {
        if (!scene_) throw Error(NR_ERR_INVALID, "prepare() has not been called");
    }
    static int param_int(const std::string& s, const std::string& key, int def) {
        size_t pos = 0;
        int val = def;
        while (pos < s.size()) {
            size_t end = s.find_first_of(" \t\n", pos);
            if (end == std::string::npos) end = s.size();
            std::string kv = s.substr(pos, end - pos);
            size_t eq = kv.find('=');
            if (eq != std::string::npos && kv.substr(0, eq) == key) {
                try { val = std::stoi(kv.substr(eq + 1)); } catch (...) { val = def; }
            }
            pos = end + 1;
        }
        return val;
    }
};

}  // namespace nr
