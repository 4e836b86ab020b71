// Test-only C shim over the product's host code (nuray_gb300/csrc/host_scene.cpp)
// so the CPU test suite can check the parameter grammar, the scene loader
// and the BVH builder without a GPU. Compiled by tests/test_host.py.
#include <cstring>
#include <string>

#include "host_scene.h"
#include "image_io.h"

extern "C" {

// BVH over n triangles (pos: 9 floats each). Returns the node count; arrays
// as nr_bvh_export. Call with null buffers to size them.
int shim_bvh(int n, const float* pos, float* box, int* kids, int* first, int* count, int* tris, int* n_tris,
             int* depth, int threads, int depth_limit) {
    nr::HostScene s;
    s.pos.assign(pos, pos + 9 * (size_t)n);
    s.mat.assign(n, 0);
    nr::Bvh b;
    nr::build_bvh(s, b, threads, depth_limit);
    for (size_t i = 0; i < b.nodes.size(); ++i) {
        const nr::BvhNode& x = b.nodes[i];
        if (box) for (int k = 0; k < 3; ++k) { box[6 * i + k] = x.lo[k]; box[6 * i + 3 + k] = x.hi[k]; }
        if (kids) { kids[2 * i] = x.left; kids[2 * i + 1] = x.right; }
        if (first) first[i] = x.first;
        if (count) count[i] = x.count;
    }
    if (tris) std::memcpy(tris, b.leaf_tris.data(), b.leaf_tris.size() * 4);
    if (n_tris) *n_tris = (int)b.leaf_tris.size();
    if (depth) *depth = b.max_depth;
    return (int)b.nodes.size();
}

// Loader: returns the triangle count (or -1 with the message in err) and
// fills the arrays when they are non-null.
int shim_load(const char* desc, float* pos, float* uv, float* nrm, int* mat, nr_material* mats, int* n_mats,
              char* err, int err_len) {
    nr::HostScene s;
    std::string e = nr::scene_from_text(desc, s);
    if (!e.empty()) {
        std::strncpy(err, e.c_str(), err_len - 1);
        err[err_len - 1] = 0;
        return -1;
    }
    if (pos) std::memcpy(pos, s.pos.data(), s.pos.size() * 4);
    if (uv) std::memcpy(uv, s.uv.data(), s.uv.size() * 4);
    if (nrm) std::memcpy(nrm, s.nrm.data(), s.nrm.size() * 4);
    if (mat) std::memcpy(mat, s.mat.data(), s.mat.size() * 4);
    if (mats) std::memcpy(mats, s.mats.data(), s.mats.size() * sizeof(nr_material));
    if (n_mats) *n_mats = (int)s.mats.size();
    return s.num_tris();
}

int shim_config_int(const char* params, const char* key, int def) { return nr::Config(params).get_int(key, def); }
float shim_config_float(const char* params, const char* key, float def) { return nr::Config(params).get_float(key, def); }
int shim_config_vec3(const char* params, const char* key, float* out) { return nr::Config(params).get_vec3(key, out) ? 1 : 0; }
void shim_camera(const char* params, nr_camera* cam, float* film_h) {
    *cam = nr::camera_from_config(nr::Config(params));
    *film_h = nr::film_height(*cam);
}

// PNG bytes -> RGBA8. Returns 0, or -1 with the message in err. rgba may be
// null to read the size only.
int shim_png_decode(const unsigned char* bytes, long n, int* w, int* h, unsigned char* rgba, char* err, int errlen) {
    std::vector<uint8_t> f(bytes, bytes + n), out;
    std::string e = nr::png_decode(f, *w, *h, out);
    if (!e.empty()) {
        std::strncpy(err, e.c_str(), (size_t)errlen - 1);
        err[errlen - 1] = 0;
        return -1;
    }
    if (rgba) std::memcpy(rgba, out.data(), out.size());
    return 0;
}

int shim_jpeg_decode(const unsigned char* bytes, long n, int* w, int* h, unsigned char* rgb, char* err, int errlen) {
    std::vector<uint8_t> f(bytes, bytes + n), out;
    std::string e = nr::jpeg_decode(f, *w, *h, out);
    if (!e.empty()) {
        std::strncpy(err, e.c_str(), (size_t)errlen - 1);
        err[errlen - 1] = 0;
        return -1;
    }
    if (rgb) std::memcpy(rgb, out.data(), out.size());
    return 0;
}

// RGB8 -> PNG bytes; returns the size (out may be null to size it).
long shim_png_encode(const unsigned char* rgb, int w, int h, unsigned char* out) {
    std::vector<uint8_t> png = nr::png_encode_rgb8(rgb, w, h);
    if (out) std::memcpy(out, png.data(), png.size());
    return (long)png.size();
}

// Texture file -> linear RGB floats as the scene loader reads it.
int shim_read_image(const char* path, int* w, int* h, float* rgb, char* err, int errlen) {
    std::vector<float> v;
    std::string e = nr::read_image(path, *w, *h, v);
    if (!e.empty()) {
        std::strncpy(err, e.c_str(), (size_t)errlen - 1);
        err[errlen - 1] = 0;
        return -1;
    }
    if (rgb) std::memcpy(rgb, v.data(), v.size() * sizeof(float));
    return 0;
}

// nr::bvh_from_arrays over n triangles: 0 (depth in *depth), or -1 with the message.
int shim_bvh_from_arrays(int n, const float* pos, int num_nodes, const float* box, const int32_t* kids,
                         const int32_t* first, const int32_t* count, const int32_t* tris, int depth_limit, int* depth,
                         char* err, int errlen) {
    nr::HostScene s;
    s.pos.assign(pos, pos + 9 * (size_t)n);
    s.mat.assign(n, 0);
    nr::Bvh b;
    std::string e = nr::bvh_from_arrays(s, num_nodes, box, kids, first, count, tris, n, depth_limit, b);
    if (depth) *depth = b.max_depth;
    if (e.empty()) return 0;
    std::strncpy(err, e.c_str(), (size_t)errlen - 1);
    err[errlen - 1] = 0;
    return -1;
}

// nr::check_tree_refs: 0 for a tree the traversal accepts, -1 with the message.
int shim_check_tree(const int32_t* refs, int num_inner, int num_tris, char* err, int errlen) {
    std::string e = nr::check_tree_refs(refs, num_inner, num_tris);
    if (e.empty()) return 0;
    std::strncpy(err, e.c_str(), (size_t)errlen - 1);
    err[errlen - 1] = 0;
    return -1;
}
}
