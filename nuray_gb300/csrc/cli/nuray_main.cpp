// nuray — command-line front end with the argv grammar of the reference's
// Cmd::main (src/cmd/cmd.cpp:9-114):
//
//   nuray <scene desc> --output <file> --params key=value ...
//
// e.g. nuray scenes/cornell/CornellBox-Original.obj -s 100 --output result.bmp
//            --params renderer=ptnee imgw=320 imgh=240 spp=16 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333
//
// renderer must be ptnee, pt or nrc (the reference also selects bdpt, pm and
// pssmlt; those are not implemented here and are rejected). For nrc a neural
// radiance cache is created (learning rate from lr=, default 1e-3 as the
// reference's SGD) and attached; path_lim= and path_lim_train= keep the
// reference's meaning. envmap= (PNG, PFM or binary PPM) and envmap_gain=
// attach an environment map as the reference CLI does.
// The output is written by extension as PNG (8-bit RGB), BMP (24-bit, what
// QImage::save produces for an RGB888 image), PPM (8-bit) or PFM (the linear
// HDR mean); other extensions get BMP.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <mutex>
#include <string>
#include <vector>

#include "../../../include/nuray_renderer.hpp"
#include "../host_scene.h"
#include "../image_io.h"

namespace {

bool ends_with(const std::string& s, const std::string& e) {
    return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}

void put_le(std::ofstream& f, uint32_t v, int bytes) {
    for (int i = 0; i < bytes; ++i) f.put((char)((v >> (8 * i)) & 0xff));
}

bool write_image(const std::string& path, const nr::Image& img) {
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    const int w = img.width, h = img.height;
    if (ends_with(path, ".png")) {
        std::vector<uint8_t> png = nr::png_encode_rgb8(img.rgb.data(), w, h);
        f.write(reinterpret_cast<const char*>(png.data()), (std::streamsize)png.size());
    } else if (ends_with(path, ".pfm")) {
        f << "PF\n" << w << " " << h << "\n-1.0\n";
        for (int y = h - 1; y >= 0; --y) f.write(reinterpret_cast<const char*>(&img.hdr[(size_t)y * w * 3]), (size_t)w * 12);
    } else if (ends_with(path, ".ppm")) {
        f << "P6\n" << w << " " << h << "\n255\n";
        f.write(reinterpret_cast<const char*>(img.rgb.data()), img.rgb.size());
    } else {  // BMP, bottom-up rows, BGR, rows padded to 4 bytes
        const int row = (3 * w + 3) & ~3;
        const uint32_t size = 54u + (uint32_t)row * h;
        f.put('B'); f.put('M');
        put_le(f, size, 4); put_le(f, 0, 4); put_le(f, 54, 4);
        put_le(f, 40, 4); put_le(f, (uint32_t)w, 4); put_le(f, (uint32_t)h, 4); put_le(f, 1, 2); put_le(f, 24, 2);
        put_le(f, 0, 4); put_le(f, (uint32_t)row * h, 4); put_le(f, 2835, 4); put_le(f, 2835, 4); put_le(f, 0, 4); put_le(f, 0, 4);
        std::vector<char> line(row, 0);
        for (int y = h - 1; y >= 0; --y) {
            for (int x = 0; x < w; ++x) {
                const uint8_t* p = &img.rgb[((size_t)y * w + x) * 3];
                line[3 * x] = (char)p[2]; line[3 * x + 1] = (char)p[1]; line[3 * x + 2] = (char)p[0];
            }
            f.write(line.data(), row);
        }
    }
    return (bool)f;
}

}  // namespace

int main(int argc, char** argv) {
    std::string scene_desc, output;
    nr::ParamString params;
    int stage = 0;
    for (int i = 1; i < argc; ++i) {  // src/cmd/cmd.cpp:21-48
        std::string s = argv[i];
        if (s == "--output") stage = 1;
        else if (s == "--params") stage = 2;
        if (stage == 0) { scene_desc += s; scene_desc += " "; }
        else if (stage == 1 && s != "--output") output = s;
        else if (stage == 2 && s != "--params") params.addItem(s);
    }
    if (argc < 2) {
        std::cerr << "usage: nuray <scene desc> --output <file> --params renderer=ptnee key=value ...\n";
        return 2;
    }
    nr::Config cfg(params.str().c_str());
    std::string renderer = cfg.get_str("renderer");  // Config::getValueStr returns "" when absent
    if (renderer != "ptnee" && renderer != "pt" && renderer != "nrc") {
        std::cerr << "renderer=" << renderer << " is not available (this library implements renderer=ptnee, pt and nrc)\n";
        return 2;
    }
    nr_nrc* cache = nullptr;
    try {
        nr::RendererGPU r;
        r.prepare(scene_desc);
        std::string env = cfg.get_str("envmap");
        if (!env.empty()) {
            int w = 0, h = 0;
            std::vector<float> rgb;
            std::string err = nr::read_image(env, w, h, rgb);
            if (!err.empty()) { std::cerr << err << "\n"; return 1; }
            nr::check(nr_scene_set_env(r.scene(), w, h, rgb.data(), cfg.get_float("envmap_gain", 1.0f)));
        }
        if (renderer == "nrc") {
            const std::string opts = "lr=" + std::to_string(cfg.get_float("lr", 0.001f));
            nr::check(nr_nrc_create(opts.c_str(), &cache));
            nr::check(nr_scene_attach_nrc(r.scene(), cache));
        }
        nr::Image img;
        std::mutex mu;
        std::atomic<int> con_flag{1};
        r.render(nr::RendererGPU::camera(params), img, params, nullptr, con_flag,
                 [](float pct) { std::cout << "Process: " << pct << "% \t" << std::flush; }, mu);
        nr_stats st;
        nr::check(nr_get_stats(r.scene(), &st));
        std::cout << "\nRendering... 100.00%   " << st.wall_ms * 1e-3 << " secs used" << std::endl;
        if (!output.empty() && !write_image(output, img)) {
            std::cerr << "cannot write " << output << "\n";
            return 1;
        }
        std::cout << "finish:)" << std::endl;
        if (cache) {
            nr::check(nr_scene_attach_nrc(r.scene(), nullptr));
            nr_nrc_destroy(cache);
        }
    } catch (const nr::Error& e) {
        std::cerr << "error " << e.code << ": " << e.what() << "\n";
        if (cache) nr_nrc_destroy(cache);
        return 1;
    }
    return 0;
}
