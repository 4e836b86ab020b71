// The reference's own frame loop, RendererPTLS::render
// (src/renderer/rendererptls.cpp:96-236), run end to end for an 8-bit image.
//
// TEST INFRASTRUCTURE ONLY, built by oracle/Makefile (`make ref-render`) into
// oracle/_ref/libnuray_ref_render.so together with the unmodified reference
// sources, with one substitution: src/sampler/samplerstd.cpp (glibc rand())
// is left out and SamplerStd is defined here on the project's Philox stream,
// the generator every other oracle path uses. render() creates its own
// SamplerStd and never says which pixel or sample it is drawing for, so the
// stream follows render()'s own order instead: with one worker
// (parallel=1) and one tile (blocksize >= imgw, imgh; random_shuffle of a
// single task does nothing), render() visits pixels row by row and samples
// in order, drawing the two jitter uniforms and then calling trace(). The
// renderer below overrides trace() (virtual in RendererPTLS) only to notice
// where a sample's top-level trace returns, and moves the stream on to the
// next (pixel, sample) there. Each sample therefore draws exactly the
// uniforms of the per-sample harness (ref_render_samples) and of the GPU.
#include "ref_harness.cpp"
#include "../sampler/samplerstd.h"

namespace {

// Which (pixel, sample) the single worker thread is drawing for.
struct RenderCursor {
    uint64_t seed = 0;
    int spp = 1, npix = 1;
    uint64_t index = 0;  // pixel * spp + sample, in render()'s order
    int depth = 0;       // nesting of trace() calls
    int calls = 0;       // SamplerStd::random calls of this sample
    nr_path_stream stream;
    void start() {
        const uint32_t pixel = (uint32_t)(index / (uint64_t)spp), sample = (uint32_t)(index % (uint64_t)spp);
        nr_stream_init(&stream, seed, pixel, sample, 0);
        calls = 0;
    }
};
RenderCursor g_cursor;
std::mutex g_render_mu;  // one render at a time: the cursor is global

class StreamRenderer : public RendererPTLS {
protected:
    vec3 trace(Config& config, Sampler& sampler, const vec3& orig, const vec3& dir, const std::vector<Triangle>& tris,
               LightSampler& ls, BVH& bvh, float light_fac_mis, const Envmap* env_map) override {
        ++g_cursor.depth;
        vec3 r = RendererPTLS::trace(config, sampler, orig, dir, tris, ls, bvh, light_fac_mis, env_map);
        if (--g_cursor.depth == 0) {  // the sample's path is done: the next draws are the next sample's jitter
            ++g_cursor.index;
            g_cursor.start();
        }
        return r;
    }
};

}  // namespace

SamplerStd::SamplerStd() {}

// render() passes `x + sampler.random(), y + sampler.random()` as two
// arguments of one call, whose evaluation order C++ leaves unspecified; g++
// evaluates them right to left, so in the reference's own build the first
// draw of a sample jitters y. The per-sample harness and the GPU jitter x
// with draw 0 and y with draw 1, so the first two calls of each sample get
// draws 1 and 0: the same uniforms reach the same axes.
float SamplerStd::random() {
    RenderCursor& c = g_cursor;
    const int k = c.calls++;
    if (k == 0) return nr_u01(c.stream.buf[1]);
    if (k == 1) {
        c.stream.n = 2;
        return nr_u01(c.stream.buf[0]);
    }
    return nr_stream_next(&c.stream);
}

extern "C" {

// The reference's render() of the whole image for params (imgw imgh spp
// campos cameuler camfov camasp and the estimator's keys; parallel and
// blocksize are set here as described above) on the Philox stream with
// this seed. rgb8: imgw * imgh * 3 bytes, row-major, from the stub QImage's
// RGB888 pixels. Returns 0, or -1 when the render did not finish.
int ref_render_image(void* h, const char* params, uint64_t seed, uint8_t* rgb8) {
    auto* s = static_cast<RefScene*>(h);
    std::lock_guard<std::mutex> lk(g_render_mu);
    std::string p(params);
    Config probe(params);
    const int w = probe.getValueInt("imgw", 1), hh = probe.getValueInt("imgh", 1);
    p += " parallel=1 blocksize=" + std::to_string(std::max(w, hh));
    Config config(p);
    Camera cam = make_camera(config);
    StreamRenderer r;
    r.prepare(*s->tris);
    g_cursor = RenderCursor();
    g_cursor.seed = seed;
    g_cursor.spp = config.getValueInt("spp", 1);
    g_cursor.npix = w * hh;
    g_cursor.start();
    QImage img;
    QMutex fb;
    std::atomic<int> con_flag{1};
    std::streambuf* old = std::cout.rdbuf(nullptr);  // render() reports progress on stdout
    r.render(cam, *s->tris, img, config, [](bool) {}, con_flag, [](float) {}, fb, s->env);
    std::cout.rdbuf(old);
    if (img.width() != w || img.height() != hh) return -1;
    if (g_cursor.index != (uint64_t)w * hh * (uint64_t)g_cursor.spp) return -1;
    for (int y = 0; y < hh; ++y)
        for (int x = 0; x < w; ++x) {
            const QRgb v = img.pixel(x, y);
            uint8_t* o = rgb8 + 3 * ((size_t)y * w + x);
            o[0] = (uint8_t)((v >> 16) & 0xff);
            o[1] = (uint8_t)((v >> 8) & 0xff);
            o[2] = (uint8_t)(v & 0xff);
        }
    return 0;
}

}  // extern "C"
