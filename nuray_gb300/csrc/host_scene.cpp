// Host side of libnuray_gpu.so: parameter grammar, scene loading and
// flattening, reference SAH BVH build. See host_scene.h.
#include "host_scene.h"
#include "image_io.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <future>
#include <memory>
#include <sstream>
#include <thread>

namespace nr {

// ------------------------------------------------------------------ Config
Config::Config(const char* text) {
    std::stringstream ss(text ? text : "");
    std::string kv;
    while (ss >> kv) add_item(kv);
}
void Config::add_item(const std::string& kv) {  // src/utils/config.cpp:90-97
    auto id = kv.find('=');
    mp_[kv.substr(0, id)] = id == std::string::npos ? kv : kv.substr(id + 1);
}
std::string Config::get_str(const std::string& key) const {
    auto it = mp_.find(key);
    return it == mp_.end() ? std::string() : it->second;
}
int Config::get_int(const std::string& key, int def) const {
    auto it = mp_.find(key);
    if (it == mp_.end()) return def;
    std::stringstream ss(it->second);
    int x;
    if (!(ss >> x)) return def;
    return x;
}
float Config::get_float(const std::string& key, float def) const {
    auto it = mp_.find(key);
    if (it == mp_.end()) return def;
    std::stringstream ss(it->second);
    float x;
    if (!(ss >> x)) return def;
    return x;
}
bool Config::get_vec3(const std::string& key, float out[3]) const {
    auto it = mp_.find(key);
    if (it == mp_.end()) return false;
    std::string s = it->second;
    for (auto& c : s) if (c == ',') c = ' ';
    std::stringstream ss(s);
    float x, y, z;
    if (!(ss >> x >> y >> z)) return false;
    out[0] = x; out[1] = y; out[2] = z;
    return true;
}

// ------------------------------------------------------------------ camera
nr_camera camera_from_config(const Config& c) {
    nr_camera cam;
    cam.fov = c.get_float("camfov", 90.0f);
    cam.aspect = c.get_float("camasp", 1.0f);
    float pos[3] = {0, 0, 0}, e[3] = {0, 0, 0};
    c.get_vec3("campos", pos);
    c.get_vec3("cameuler", e);
    for (int k = 0; k < 3; ++k) cam.pos[k] = pos[k];
    // Camera::fromEuler (src/scene/camera.cpp:88-105): angles in degrees,
    // the float / 180 product promoted to double by the literal 3.14159.
    const double PI = 3.14159;
    float c1 = (float)std::cos((double)(e[0] / 180.0f) * PI), s1 = (float)std::sin((double)(e[0] / 180.0f) * PI);
    float c2 = (float)std::cos((double)(e[1] / 180.0f) * PI), s2 = (float)std::sin((double)(e[1] / 180.0f) * PI);
    float c3 = (float)std::cos((double)(e[2] / 180.0f) * PI), s3 = (float)std::sin((double)(e[2] / 180.0f) * PI);
    float m12 = c3 * s1 * s2 - c1 * s3;
    float m13 = c2 * s1;
    float m22 = c2 * c3;
    float m23 = -s2;
    float m32 = s1 * s3 + c1 * c3 * s2;
    float m33 = c1 * c2;
    cam.up[0] = m12; cam.up[1] = m22; cam.up[2] = m32;
    cam.gaze[0] = -m13; cam.gaze[1] = -m23; cam.gaze[2] = -m33;
    return cam;
}
float film_height(const nr_camera& cam) { return (float)(2 * std::tan((double)cam.fov * 3.14159 / 180 / 2)); }

// ------------------------------------------------------------------ scene from arrays
static void face_normal_rule(HostScene& s, int i) {
    float* n = &s.nrm[9 * (size_t)i];
    double n2 = (double)(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(n2 < 1e-4)) return;
    const float* p = &s.pos[9 * (size_t)i];
    float e1[3] = {p[3] - p[0], p[4] - p[1], p[5] - p[2]};
    float e2[3] = {p[6] - p[0], p[7] - p[1], p[8] - p[2]};
    float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    float len = (float)std::sqrt((double)(c[0] * c[0] + c[1] * c[1] + c[2] * c[2])) + 1e-8f;
    for (int v = 0; v < 3; ++v)
        for (int k = 0; k < 3; ++k) n[3 * v + k] = c[k] / len;
}

std::string scene_from_desc(const nr_scene_desc& d, HostScene& s) {
    if (d.num_tris < 0 || d.num_mats < 0 || d.num_tex < 0) return "negative count";
    if (d.num_tris > 0 && (!d.pos || !d.mat)) return "pos and mat are required";
    if (d.num_tris > (1 << 27)) return "too many triangles (limit 2^27)";
    if (d.num_tris > 0 && (d.num_mats <= 0 || !d.mats)) return "materials are required";
    size_t n = (size_t)d.num_tris;
    s.pos.assign(d.pos, d.pos + 9 * n);
    s.uv.assign(6 * n, 0.0f);
    if (d.uv) s.uv.assign(d.uv, d.uv + 6 * n);
    s.nrm.assign(9 * n, 0.0f);
    if (d.nrm) s.nrm.assign(d.nrm, d.nrm + 9 * n);
    s.mat.assign(d.mat, d.mat + n);
    s.mats.assign(d.mats, d.mats + d.num_mats);
    // NaN or infinite inputs are refused: the reference would carry them
    // into every box and radiance they touch (it checks nothing)
    for (size_t i = 0; i < n; ++i) {
        if (s.mat[i] < 0 || s.mat[i] >= d.num_mats) return "triangle " + std::to_string(i) + ": material index out of range";
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(s.pos[9 * i + k])) return "triangle " + std::to_string(i) + ": non-finite position";
        for (int k = 0; k < 9; ++k)
            if (!std::isfinite(s.nrm[9 * i + k])) return "triangle " + std::to_string(i) + ": non-finite normal";
        for (int k = 0; k < 6; ++k)
            if (!std::isfinite(s.uv[6 * i + k])) return "triangle " + std::to_string(i) + ": non-finite texture coordinate";
    }
    size_t texels = 0;
    if (d.num_tex > 0) {
        if (!d.tex_wh || !d.tex_data) return "texture arrays missing";
        s.tex_wh.assign(d.tex_wh, d.tex_wh + 2 * (size_t)d.num_tex);
        for (int t = 0; t < d.num_tex; ++t) {
            if (s.tex_wh[2 * t] <= 0 || s.tex_wh[2 * t + 1] <= 0) return "texture " + std::to_string(t) + ": bad size";
            texels += (size_t)s.tex_wh[2 * t] * s.tex_wh[2 * t + 1];
        }
        s.tex_data.assign(d.tex_data, d.tex_data + 3 * texels);
        for (size_t i = 0; i < s.tex_data.size(); ++i)
            if (!std::isfinite(s.tex_data[i])) return "texel value " + std::to_string(i) + " is not finite";
    }
    for (int m = 0; m < d.num_mats; ++m) {
        const nr_material& M = s.mats[m];
        if (M.type < NR_MAT_LAMBERT || M.type > NR_MAT_LIGHT) return "material " + std::to_string(m) + ": bad type";
        if (M.tex0 >= d.num_tex || M.tex1 >= d.num_tex) return "material " + std::to_string(m) + ": texture index out of range";
        const float f[9] = {M.c0[0], M.c0[1], M.c0[2], M.c1[0], M.c1[1], M.c1[2], M.alpha, M.ior, M.ns};
        for (float x : f)
            if (!std::isfinite(x)) return "material " + std::to_string(m) + ": non-finite parameter";
    }
    if (d.env_tex >= d.num_tex) return "env_tex out of range";
    if (!std::isfinite(d.env_gain)) return "env_gain is not finite";
    s.env_tex = d.env_tex < 0 ? -1 : d.env_tex;
    s.env_gain = d.env_gain;
    for (size_t i = 0; i < n; ++i) face_normal_rule(s, (int)i);
    return "";
}

// ------------------------------------------------------------------ images
std::string read_image(const std::string& path, int& w, int& h, std::vector<float>& rgb) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return "cannot open " + path;
    {
        unsigned char sig[8] = {0};
        f.read(reinterpret_cast<char*>(sig), 8);
        if (f.gcount() >= 3 && sig[0] == 0xFF && sig[1] == 0xD8 && sig[2] == 0xFF) {
            f.seekg(0, std::ios::end);
            std::vector<uint8_t> bytes((size_t)f.tellg());
            f.seekg(0);
            f.read(reinterpret_cast<char*>(bytes.data()), (std::streamsize)bytes.size());
            if (!f) return "cannot read " + path;
            std::vector<uint8_t> px;
            std::string err = jpeg_decode(bytes, w, h, px);
            if (!err.empty()) return err + ": " + path;
            // the same 8-bit to linear mapping as for PNG below
            rgb.resize(px.size());
            for (size_t i = 0; i < px.size(); ++i) rgb[i] = (float)std::pow((double)(px[i] * 257) / 65535.0, (double)2.2f);
            return "";
        }
        if (f.gcount() == 8 && sig[0] == 0x89 && sig[1] == 'P' && sig[2] == 'N' && sig[3] == 'G') {
            f.seekg(0, std::ios::end);
            std::vector<uint8_t> bytes((size_t)f.tellg());
            f.seekg(0);
            f.read(reinterpret_cast<char*>(bytes.data()), (std::streamsize)bytes.size());
            if (!f) return "cannot read " + path;
            std::vector<uint8_t> rgba;
            std::string err = png_decode(bytes, w, h, rgba);
            if (!err.empty()) return err + ": " + path;
            // Texture::load: QColor::redF() = (8-bit value * 257) / 65535 as a
            // double, then pow(., 2.2f) (src/scene/texture.cpp:13-19)
            rgb.resize((size_t)w * h * 3);
            for (size_t i = 0; i < (size_t)w * h; ++i)
                for (int k = 0; k < 3; ++k)
                    rgb[3 * i + k] = (float)std::pow((double)(rgba[4 * i + k] * 257) / 65535.0, (double)2.2f);
            return "";
        }
        f.clear();
        f.seekg(0);
    }
    // bytes left after the header: the pixel data must fit in them before
    // anything is allocated for it
    auto left = [&f]() -> uint64_t {
        const std::streampos here = f.tellg();
        if (here < 0) return 0;
        f.seekg(0, std::ios::end);
        const std::streampos end = f.tellg();
        f.seekg(here);
        return end > here ? (uint64_t)(end - here) : 0;
    };
    std::string magic;
    f >> magic;
    if (magic == "PF" || magic == "Pf") {
        double scale;
        f >> w >> h >> scale;
        f.get();
        if (!f || w <= 0 || h <= 0) return "bad PFM header in " + path;
        int ch = magic == "PF" ? 3 : 1;
        if ((uint64_t)w * (uint64_t)h * (uint64_t)ch * 4u > left()) return "truncated PFM " + path;
        std::vector<float> raw((size_t)w * h * ch);
        f.read(reinterpret_cast<char*>(raw.data()), raw.size() * sizeof(float));
        if (!f) return "truncated PFM " + path;
        bool big = scale > 0;
        if (big) {
            for (auto& x : raw) {
                uint32_t u;
                std::memcpy(&u, &x, 4);
                u = (u >> 24) | ((u >> 8) & 0xff00u) | ((u << 8) & 0xff0000u) | (u << 24);
                std::memcpy(&x, &u, 4);
            }
        }
        rgb.resize((size_t)w * h * 3);
        for (int y = 0; y < h; ++y)  // PFM rows run bottom to top
            for (int x = 0; x < w; ++x)
                for (int k = 0; k < 3; ++k)
                    rgb[((size_t)(h - 1 - y) * w + x) * 3 + k] = raw[((size_t)y * w + x) * ch + (ch == 3 ? k : 0)];
        return "";
    }
    if (magic == "P6") {
        int maxv;
        f >> w >> h >> maxv;
        f.get();
        if (!f || w <= 0 || h <= 0 || maxv != 255) return "unsupported PPM " + path;
        if ((uint64_t)w * (uint64_t)h * 3u > left()) return "truncated PPM " + path;
        std::vector<unsigned char> raw((size_t)w * h * 3);
        f.read(reinterpret_cast<char*>(raw.data()), raw.size());
        if (!f) return "truncated PPM " + path;
        rgb.resize(raw.size());
        // Texture::load: channel^2.2 (src/scene/texture.cpp:16-19)
        for (size_t i = 0; i < raw.size(); ++i) rgb[i] = (float)std::pow(raw[i] / 255.0, (double)2.2f);
        return "";
    }
    return "unsupported image format (PNG, JPEG, PFM or binary PPM): " + path;
}

void build_env_table(const float* rgb, int w, int h, EnvTable& T) {
    T = EnvTable{};
    if (w <= 0 || h <= 0) return;
    T.w = w;
    T.h = h;
    T.weight.assign((size_t)w * h, 0.f);
    T.row_cdf.assign((size_t)h, 0.f);
    T.col_cdf.assign((size_t)w * h, 0.f);
    auto lum = [&](int x, int y) -> float {
        if (x >= w || y >= h) return 0.f;
        const float* c = rgb + 3 * ((size_t)y * w + x);
        return c[0] + c[1] + c[2];
    };
    std::vector<float> row_sum((size_t)h, 0.f);
    for (int y = 0; y < h; ++y) {
        const float th = ((float)y + 0.5f) / (float)h * 3.14159f;
        const float sn = std::sin(th);
        float acc = 0.f;
        for (int x = 0; x < w; ++x) {
            float m = std::max(std::max(lum(x, y), lum(x + 1, y)), std::max(lum(x, y + 1), lum(x + 1, y + 1)));
            float wt = m > 0.f ? m * sn : 0.f;
            T.weight[(size_t)y * w + x] = wt;
            acc += wt;
            T.col_cdf[(size_t)y * w + x] = acc;
        }
        row_sum[y] = acc;
        for (int x = 0; x < w; ++x) {
            float& c = T.col_cdf[(size_t)y * w + x];
            c = acc > 0.f ? c / acc : (float)(x + 1) / (float)w;
        }
        T.col_cdf[(size_t)y * w + w - 1] = 1.f;
    }
    float acc = 0.f;
    for (int y = 0; y < h; ++y) {
        acc += row_sum[y];
        T.row_cdf[y] = acc;
    }
    T.total = acc;
    for (int y = 0; y < h; ++y) T.row_cdf[y] = acc > 0.f ? T.row_cdf[y] / acc : (float)(y + 1) / (float)h;
    T.row_cdf[h - 1] = 1.f;
}

// ------------------------------------------------------------------ OBJ / MTL
namespace {

std::string path2dir(const std::string& path) {  // src/scene/loader.cpp:18-24
    std::size_t pos = path.find_last_of("/\\");
    if (pos == std::string::npos) return ".";
    return path.substr(0, pos);
}

struct LoaderState {
    HostScene& s;
    std::map<std::string, int> dict;  // "file:name" -> material index
    std::map<std::string, int> tex_cache;
    explicit LoaderState(HostScene& sc) : s(sc) {}

    int add_mat(const nr_material& m) {
        s.mats.push_back(m);
        return (int)s.mats.size() - 1;
    }
    std::string add_tex(const std::string& path, int& id) {
        auto it = tex_cache.find(path);
        if (it != tex_cache.end()) { id = it->second; return ""; }
        int w, h;
        std::vector<float> rgb;
        std::string err = read_image(path, w, h, rgb);
        if (!err.empty()) return err;
        id = (int)s.tex_wh.size() / 2;
        s.tex_wh.push_back(w); s.tex_wh.push_back(h);
        s.tex_data.insert(s.tex_data.end(), rgb.begin(), rgb.end());
        tex_cache[path] = id;
        return "";
    }

    // Loader::loadMtl (src/scene/loader.cpp:110-230)
    std::string load_mtl(const std::string& filename) {
        std::ifstream ifs(filename);
        if (!ifs) return "cannot open " + filename;
        float Ns = 10.0f;  // the reference leaves Ns uninitialised before the first newmtl commit
        float Kd[3] = {0, 0, 0}, Ks[3] = {0, 0, 0}, Ke[3] = {0, 0, 0};
        std::string map_Kd, map_Ks, name;
        auto vec = [](const std::vector<std::string>& b, float* o) {
            for (int k = 0; k < 3; ++k) o[k] = (float)std::atof(k + 1 < (int)b.size() ? b[k + 1].c_str() : "0");
        };
        std::string err;
        auto commit = [&]() {
            nr_material m;
            std::memset(&m, 0, sizeof(m));
            m.tex0 = -1; m.tex1 = -1; m.alpha = 0.5f; m.ior = 1.0f; m.ns = Ns;
            double ke2 = (double)(Ke[0] * Ke[0] + Ke[1] * Ke[1] + Ke[2] * Ke[2]);
            double ks2 = (double)(Ks[0] * Ks[0] + Ks[1] * Ks[1] + Ks[2] * Ks[2]);
            if (ke2 > 1e-6) {
                m.type = NR_MAT_LIGHT;
                std::memcpy(m.c0, Ke, sizeof(Ke));
            } else if (ks2 > 1e-6 || !map_Ks.empty()) {
                m.type = NR_MAT_BLINNPHONG;
                std::memcpy(m.c0, Kd, sizeof(Kd));
                std::memcpy(m.c1, Ks, sizeof(Ks));
                if (!map_Kd.empty() && err.empty()) err = add_tex(map_Kd, m.tex0);
                if (!map_Ks.empty() && err.empty()) err = add_tex(map_Ks, m.tex1);
            } else {
                m.type = NR_MAT_LAMBERT;
                std::memcpy(m.c0, Kd, sizeof(Kd));
                if (!map_Kd.empty() && err.empty()) err = add_tex(map_Kd, m.tex0);
            }
            dict[filename + ":" + name] = add_mat(m);
            Ns = 10.0f;
            for (int k = 0; k < 3; ++k) Kd[k] = Ks[k] = Ke[k] = 0.0f;
            map_Kd.clear(); map_Ks.clear();
        };
        std::string line;
        while (std::getline(ifs, line)) {
            if (!line.empty() && line[0] == '#') continue;
            std::stringstream ss(line);
            std::vector<std::string> b;
            std::string tok;
            while (ss >> tok) b.push_back(tok);
            if (b.empty()) continue;
            if (b[0] == "newmtl") {
                if (!name.empty()) commit();
                name = b.size() > 1 ? b[1] : "";
            } else if (b[0] == "Ns" && b.size() > 1) {
                Ns = (float)std::atof(b[1].c_str());
            } else if (b[0] == "Kd") {
                vec(b, Kd);
            } else if (b[0] == "Ks") {
                vec(b, Ks);
            } else if (b[0] == "Ke") {
                vec(b, Ke);
            } else if (b[0] == "map_Kd" && b.size() > 1) {
                map_Kd = path2dir(filename) + "/" + b[1];
            } else if (b[0] == "map_Ks" && b.size() > 1) {
                map_Ks = path2dir(filename) + "/" + b[1];
            }
            if (!err.empty()) return err;
        }
        if (!name.empty()) commit();
        return err;
    }

    // Loader::loadObj (src/scene/loader.cpp:232-361)
    std::string load_obj(const std::string& filename, const float position[3], float scale, int forcing) {
        std::ifstream ifs(filename);
        if (!ifs) return "cannot open " + filename;
        std::vector<float> V(3, 0.0f), N(3, 0.0f), T(3, 0.0f);  // index 0 is the zero entry
        std::string mtllib;
        int mtl = forcing;
        std::string line;
        int lineno = 0;
        while (std::getline(ifs, line)) {
            ++lineno;
            std::stringstream ss(line);
            std::vector<std::string> b;
            std::string tok;
            while (ss >> tok) b.push_back(tok);
            if (b.empty()) continue;
            if (b[0] == "mtllib" && b.size() > 1) {
                mtllib = path2dir(filename) + "/" + b[1];
                if (forcing < 0) {
                    std::string err = load_mtl(mtllib);
                    if (!err.empty()) return err;
                }
            } else if (b[0] == "usemtl" && b.size() > 1) {
                if (forcing < 0) {
                    auto it = dict.find(mtllib + ":" + b[1]);
                    if (it == dict.end()) return filename + ":" + std::to_string(lineno) + ": cannot find material " + mtllib + ":" + b[1];
                    mtl = it->second;
                }
            } else if (b[0] == "v") {
                if (b.size() < 4) return filename + ":" + std::to_string(lineno) + ": bad vertex";
                for (int k = 0; k < 3; ++k) V.push_back((float)std::atof(b[k + 1].c_str()) * scale + position[k]);
            } else if (b[0] == "vt") {
                if (b.size() < 3) return filename + ":" + std::to_string(lineno) + ": bad texcoord";
                T.push_back((float)std::atof(b[1].c_str()));
                T.push_back((float)std::atof(b[2].c_str()));
                T.push_back(0.0f);
            } else if (b[0] == "vn") {
                if (b.size() < 4) return filename + ":" + std::to_string(lineno) + ": bad normal";
                for (int k = 0; k < 3; ++k) N.push_back((float)std::atof(b[k + 1].c_str()));
            } else if (b[0] == "f") {
                int nv = (int)b.size() - 1;
                if (nv != 3 && nv != 4) continue;  // "Unsupported f type" in the reference
                if (mtl < 0) return filename + ":" + std::to_string(lineno) + ": face without material";
                int a[4][3];
                for (int i = 0; i < nv; ++i) {
                    const std::string& w = b[i + 1];
                    std::vector<size_t> sl;
                    for (size_t j = 0; j < w.size(); ++j) if (w[j] == '/') sl.push_back(j);
                    while (sl.size() < 3) sl.push_back(w.size());
                    size_t ptr = 0;
                    for (int j = 0; j < 3; ++j) {
                        size_t cur = sl[j];
                        a[i][j] = ptr < cur ? std::atoi(w.substr(ptr, cur - ptr).c_str()) : 0;
                        ptr = std::min(w.size(), cur + 1);
                    }
                    int nV = (int)V.size() / 3, nT = (int)T.size() / 3, nN = (int)N.size() / 3;
                    if (a[i][0] < 0) a[i][0] += nV;
                    if (a[i][1] < 0) a[i][1] += nT;
                    if (a[i][2] < 0) a[i][2] += nN;
                    if (a[i][0] <= 0 || a[i][0] >= nV) return filename + ":" + std::to_string(lineno) + ": vertex index out of range";
                    if (a[i][1] < 0 || a[i][1] >= nT) a[i][1] = 0;
                    if (a[i][2] < 0 || a[i][2] >= nN) a[i][2] = 0;
                }
                auto emit = [&](int i0, int i1, int i2) {
                    int ids[3] = {i0, i1, i2};
                    for (int v = 0; v < 3; ++v) {
                        for (int k = 0; k < 3; ++k) s.pos.push_back(V[3 * a[ids[v]][0] + k]);
                        s.uv.push_back(T[3 * a[ids[v]][1]]);
                        s.uv.push_back(T[3 * a[ids[v]][1] + 1]);
                        for (int k = 0; k < 3; ++k) s.nrm.push_back(N[3 * a[ids[v]][2] + k]);
                    }
                    s.mat.push_back(mtl);
                    face_normal_rule(s, s.num_tris() - 1);
                };
                emit(0, 1, 2);
                if (nv == 4) emit(2, 3, 0);
            }
        }
        return "";
    }
};

}  // namespace

std::string scene_from_text(const std::string& desc, HostScene& s) {
    s = HostScene();
    LoaderState L(s);
    std::stringstream all(desc);
    std::string line;
    while (std::getline(all, line)) {  // src/scene/loader.cpp:37-107
        std::stringstream ls(line);
        std::string filename;
        if (!(ls >> filename)) continue;
        float position[3] = {0, 0, 0}, scale = 1.0f, t_vec[3] = {0, 0, 0}, t_ps = 0, t_ps2 = 0;
        bool light = false, ggx = false, ggxr = false, glass = false;
        std::string op;
        while (ls >> op) {
            if (op == "-p") ls >> position[0] >> position[1] >> position[2];
            else if (op == "-s") ls >> scale;
            else if (op == "-m=light") { ls >> t_vec[0] >> t_vec[1] >> t_vec[2]; light = true; }
            else if (op == "-m=ggx") { ls >> t_vec[0] >> t_vec[1] >> t_vec[2] >> t_ps >> t_ps2; ggx = true; }
            else if (op == "-m=ggxr") { ls >> t_vec[0] >> t_vec[1] >> t_vec[2] >> t_ps; ggxr = true; }
            else if (op == "-m=glass") { ls >> t_vec[0] >> t_vec[1] >> t_vec[2] >> t_ps; glass = true; }
        }
        int forcing = -1;
        auto forced = [&](int type) {
            nr_material m;
            std::memset(&m, 0, sizeof(m));
            m.type = type; m.tex0 = -1; m.tex1 = -1; m.alpha = 0.5f; m.ior = 1.0f; m.ns = 10.0f;
            std::memcpy(m.c0, t_vec, sizeof(t_vec));
            if (type == NR_MAT_GGX) { m.alpha = t_ps; m.ior = t_ps2; }
            if (type == NR_MAT_GGXR) m.alpha = t_ps;
            if (type == NR_MAT_GLASS) m.ior = t_ps;
            forcing = L.add_mat(m);
        };
        // later flags replace earlier ones, in the reference's order
        if (light) forced(NR_MAT_LIGHT);
        if (ggx) forced(NR_MAT_GGX);
        if (ggxr) forced(NR_MAT_GGXR);
        if (glass) forced(NR_MAT_GLASS);
        std::string err = L.load_obj(filename, position, scale, forcing);
        if (!err.empty()) return err;
    }
    return "";
}

// ------------------------------------------------------------------ BVH
namespace {

struct Key {
    float k[3];
    int32_t id;
};

struct TmpNode {
    float lo[3], hi[3];
    std::unique_ptr<TmpNode> l, r;
    std::vector<int32_t> prims;
};

struct Builder {
    const std::vector<float>* pmin;  // 3 per triangle
    const std::vector<float>* pmax;
    const std::vector<float>* pos;
    std::atomic<int> spare_threads{0};
    int depth_limit = 0;
    std::atomic<bool> too_deep{false};

    static inline float fmn(float a, float b) { return (b < a) ? b : a; }  // std::min
    static inline float fmx(float a, float b) { return (a < b) ? b : a; }  // std::max
    static inline float area(const float lo[3], const float hi[3]) {
        float d0 = hi[0] - lo[0], d1 = hi[1] - lo[1], d2 = hi[2] - lo[2];
        return (d0 * d1 + d1 * d2 + d2 * d0) * 2.0f;
    }

    // BVH::_divide (src/hierarchy/bvh.cpp:5-58). std::sort over the same
    // comparisons as the reference's sort of Triangle pointers, so the same
    // permutation results.
    void split(std::vector<Key>& prims, std::vector<Key>& L, std::vector<Key>& R) {
        const size_t n = prims.size();
        int ans_axis = 0, ans_mid = 0;
        float ans_cost = 1e38f;
        std::vector<float> suffix(n);
        const float* PMIN = pmin->data();
        const float* PMAX = pmax->data();
        for (int axis = 0; axis < 3; ++axis) {
            std::sort(prims.begin(), prims.end(), [axis](const Key& a, const Key& b) { return a.k[axis] < b.k[axis]; });
            float lo[3] = {1e18f, 1e18f, 1e18f}, hi[3] = {-1e18f, -1e18f, -1e18f};
            for (int i = (int)n - 1; i >= 0; --i) {
                const float* a = PMIN + 3 * (size_t)prims[i].id;
                const float* b = PMAX + 3 * (size_t)prims[i].id;
                for (int k = 0; k < 3; ++k) { lo[k] = fmn(lo[k], a[k]); hi[k] = fmx(hi[k], b[k]); }
                suffix[i] = area(lo, hi);
            }
            for (int k = 0; k < 3; ++k) { lo[k] = 1e18f; hi[k] = -1e18f; }
            for (size_t i = 0; i + 1 < n; ++i) {
                const float* a = PMIN + 3 * (size_t)prims[i].id;
                const float* b = PMAX + 3 * (size_t)prims[i].id;
                for (int k = 0; k < 3; ++k) { lo[k] = fmn(lo[k], a[k]); hi[k] = fmx(hi[k], b[k]); }
                float cost = area(lo, hi) * (float)(int)(i + 1) + suffix[i + 1] * (float)(n - i);
                if (cost < ans_cost) { ans_cost = cost; ans_mid = (int)i + 1; ans_axis = axis; }
            }
        }
        // No cost below the start value (surface areas beyond the float range,
        // about 1e19 units of extent): the reference would keep every triangle
        // on one side and recurse until its stack overflows. A median split on
        // the first axis instead, as the device builder does.
        if (ans_mid == 0) {
            ans_axis = 0;
            ans_mid = (int)(n / 2);
        }
        std::sort(prims.begin(), prims.end(), [ans_axis](const Key& a, const Key& b) { return a.k[ans_axis] < b.k[ans_axis]; });
        L.assign(prims.begin(), prims.begin() + ans_mid);
        R.assign(prims.begin() + ans_mid, prims.end());
    }

    std::unique_ptr<TmpNode> build(std::vector<Key>& prims, int depth) {
        auto node = std::make_unique<TmpNode>();
        // past the depth limit the tree is refused whole; stop descending
        if (depth > depth_limit || too_deep.load(std::memory_order_relaxed)) {
            too_deep = true;
            return node;
        }
        if (prims.size() <= 5) {  // BVH::_build leaf rule (src/hierarchy/bvh.cpp:62-65)
            for (int k = 0; k < 3; ++k) { node->lo[k] = 1e18f; node->hi[k] = -1e18f; }
            const float* P = pos->data();
            for (const Key& key : prims) {
                for (int v = 0; v < 3; ++v)
                    for (int k = 0; k < 3; ++k) {
                        float x = P[9 * (size_t)key.id + 3 * v + k];
                        node->lo[k] = fmn(node->lo[k], x);
                        node->hi[k] = fmx(node->hi[k], x);
                    }
                node->prims.push_back(key.id);
            }
            return node;
        }
        std::vector<Key> L, R;
        split(prims, L, R);
        std::vector<Key>().swap(prims);
        if (L.size() + R.size() > 20000 && spare_threads.fetch_sub(1) > 0) {
            auto fut = std::async(std::launch::async, [&]() { return build(L, depth + 1); });
            node->r = build(R, depth + 1);
            node->l = fut.get();
            spare_threads.fetch_add(1);
        } else {
            node->l = build(L, depth + 1);
            node->r = build(R, depth + 1);
        }
        for (int k = 0; k < 3; ++k) {
            node->lo[k] = fmn(node->l->lo[k], node->r->lo[k]);
            node->hi[k] = fmx(node->l->hi[k], node->r->hi[k]);
        }
        return node;
    }
};

void flatten(const TmpNode* t, int depth, Bvh& out) {
    int id = (int)out.nodes.size();
    out.nodes.emplace_back();
    BvhNode n;
    for (int k = 0; k < 3; ++k) { n.lo[k] = t->lo[k]; n.hi[k] = t->hi[k]; }
    n.depth = depth;
    if (depth > out.max_depth) out.max_depth = depth;
    if (!t->l) {
        n.left = n.right = -1;
        n.first = (int)out.leaf_tris.size();
        n.count = (int)t->prims.size();
        out.leaf_tris.insert(out.leaf_tris.end(), t->prims.begin(), t->prims.end());
    } else {
        n.first = -1; n.count = 0;
        n.left = (int)out.nodes.size();
        flatten(t->l.get(), depth + 1, out);
        n.right = (int)out.nodes.size();
        flatten(t->r.get(), depth + 1, out);
    }
    out.nodes[id] = n;
}

}  // namespace

void build_bvh(const HostScene& s, Bvh& out, int threads, int depth_limit) {
    const int n = s.num_tris();
    std::vector<float> pmin(3 * (size_t)n), pmax(3 * (size_t)n);
    std::vector<Key> prims(n);
    for (int i = 0; i < n; ++i) {
        const float* p = &s.pos[9 * (size_t)i];
        for (int k = 0; k < 3; ++k) {
            // Triangle::pMin / pMax (src/scene/triangle.cpp:68-76)
            float a = p[k], b = p[3 + k], c = p[6 + k];
            float mx12 = (b < c) ? c : b, mn12 = (c < b) ? c : b;
            pmax[3 * (size_t)i + k] = (a < mx12) ? mx12 : a;
            pmin[3 * (size_t)i + k] = (mn12 < a) ? mn12 : a;
            prims[i].k[k] = pmax[3 * (size_t)i + k];
        }
        prims[i].id = i;
    }
    Builder b;
    b.pmin = &pmin; b.pmax = &pmax; b.pos = &s.pos;
    b.spare_threads = threads > 1 ? threads - 1 : 0;
    b.depth_limit = depth_limit;
    std::unique_ptr<TmpNode> root = b.build(prims, 0);
    out = Bvh();
    if (b.too_deep) {  // no tree; the depth says why
        out.max_depth = depth_limit + 1;
        return;
    }
    out.nodes.reserve(n > 0 ? (size_t)n : 1);
    flatten(root.get(), 0, out);
    // free the temporary tree iteratively-deep recursion is bounded by depth
    root.reset();
}

std::string bvh_from_arrays(const HostScene& s, int num_nodes, const float* box, const int32_t* kids,
                            const int32_t* leaf_first, const int32_t* leaf_count, const int32_t* leaf_tris,
                            int num_leaf_tris, int depth_limit, Bvh& out) {
    out = Bvh();
    const int n = s.num_tris();
    if (num_nodes < 0 || num_leaf_tris != n) return "the tree must order every triangle once (num_leaf_tris)";
    if (n == 0) return num_nodes == 0 ? "" : "a tree over no triangles must have no nodes";
    if (num_nodes < 1 || !box || !kids || !leaf_first || !leaf_count || !leaf_tris) return "tree arrays missing";
    std::vector<uint8_t> seen((size_t)n, 0);
    for (int i = 0; i < n; ++i) {
        const int32_t t = leaf_tris[i];
        if (t < 0 || t >= n || seen[t]++) return "leaf_tris is not a permutation of the triangles";
    }
    std::vector<int32_t> parent((size_t)num_nodes, -1);
    std::vector<uint8_t> covered((size_t)n, 0);
    out.nodes.resize((size_t)num_nodes);
    for (int i = 0; i < num_nodes; ++i) {
        BvhNode& nd = out.nodes[i];
        for (int k = 0; k < 3; ++k) {
            nd.lo[k] = box[6 * (size_t)i + k];
            nd.hi[k] = box[6 * (size_t)i + 3 + k];
            if (!std::isfinite(nd.lo[k]) || !std::isfinite(nd.hi[k]) || nd.lo[k] > nd.hi[k])
                return "node " + std::to_string(i) + ": bad box";
        }
        nd.left = kids[2 * (size_t)i];
        nd.right = kids[2 * (size_t)i + 1];
        nd.first = nd.count = 0;
        if (nd.left < 0 || nd.right < 0) {
            if (nd.left != -1 || nd.right != -1) return "node " + std::to_string(i) + ": a leaf has kids -1, -1";
            nd.first = leaf_first[i];
            nd.count = leaf_count[i];
            // the device encodes a leaf's count in 3 bits
            if (nd.count < 0 || nd.count > 7 || nd.first < 0 || (int64_t)nd.first + nd.count > n)
                return "node " + std::to_string(i) + ": leaf range outside the triangles (at most 7 per leaf)";
            for (int j = nd.first; j < nd.first + nd.count; ++j) {
                if (covered[j]++) return "leaves overlap at triangle position " + std::to_string(j);
                const float* p = &s.pos[9 * (size_t)leaf_tris[j]];
                for (int v = 0; v < 3; ++v)
                    for (int k = 0; k < 3; ++k)
                        if (!(p[3 * v + k] >= nd.lo[k] && p[3 * v + k] <= nd.hi[k]))
                            return "node " + std::to_string(i) + ": its box does not hold triangle " +
                                   std::to_string(leaf_tris[j]);
            }
        } else {
            for (int32_t c : {nd.left, nd.right}) {
                if (c <= i || c >= num_nodes) return "node " + std::to_string(i) + ": a child must follow its parent";
                if (parent[c] >= 0) return "node " + std::to_string(c) + " has two parents";
                parent[c] = i;
            }
        }
    }
    for (int j = 0; j < n; ++j)
        if (!covered[j]) return "triangle position " + std::to_string(j) + " is in no leaf";
    // a walk tests a child's box only inside its parent's: boxes must nest
    for (int i = 1; i < num_nodes; ++i) {
        const BvhNode &c = out.nodes[i], &p = out.nodes[parent[i] < 0 ? 0 : parent[i]];
        for (int k = 0; k < 3; ++k)
            if (parent[i] >= 0 && (c.lo[k] < p.lo[k] || c.hi[k] > p.hi[k]))
                return "node " + std::to_string(i) + ": its box is not inside its parent's";
    }
    // every node but the root has its parent before it: depths in one pass
    out.nodes[0].depth = 0;
    for (int i = 1; i < num_nodes; ++i) {
        if (parent[i] < 0) return "node " + std::to_string(i) + " is not reachable from the root";
        out.nodes[i].depth = out.nodes[parent[i]].depth + 1;
        out.max_depth = std::max(out.max_depth, out.nodes[i].depth);
        if (out.max_depth > depth_limit) {
            out = Bvh();
            out.max_depth = depth_limit + 1;
            return "";
        }
    }
    out.leaf_tris.assign(leaf_tris, leaf_tris + n);
    return "";
}

std::string check_tree_refs(const int32_t* refs, int num_inner, int num_tris) {
    std::vector<uint8_t> referenced((size_t)std::max(num_inner, 0), 0);
    for (int i = 0; i < num_inner; ++i)
        for (int side = 0; side < 2; ++side) {
            const int32_t r = refs[2 * (size_t)i + side];
            if (r >= 0) {
                if (r <= i || r >= num_inner) return "BVH is not a tree: node " + std::to_string(i) + " refers to " + std::to_string(r);
                if (referenced[r]++) return "BVH is not a tree: node " + std::to_string(r) + " has two parents";
            } else {
                const int32_t code = -1 - r, first = code >> 3, count = code & 7;
                if ((int64_t)first + count > num_tris)
                    return "BVH leaf outside the triangle array: node " + std::to_string(i);
            }
        }
    return "";
}

}  // namespace nr
