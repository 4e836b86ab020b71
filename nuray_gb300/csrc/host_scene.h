// Host side of libnuray_gpu.so: the reference's parameter grammar, scene
// loading and flattening, and the SAH BVH build.
#pragma once
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/nuray.h"

namespace nr {

// Config (src/utils/config.cpp): whitespace-separated key=value items split
// at the first '='; typed getters return the default when the key is absent
// or does not parse; vec3 values are comma-separated.
class Config {
public:
    explicit Config(const char* text = nullptr);
    void add_item(const std::string& kv);
    bool has(const std::string& key) const { return mp_.count(key) != 0; }
    std::string get_str(const std::string& key) const;  // "" when absent, as the reference
    int get_int(const std::string& key, int def) const;
    float get_float(const std::string& key, float def) const;
    bool get_vec3(const std::string& key, float out[3]) const;

private:
    std::map<std::string, std::string> mp_;
};

// Camera as Cmd::main builds it (src/cmd/cmd.cpp:99-101, src/scene/camera.cpp:88-105).
nr_camera camera_from_config(const Config& c);
// 2 tan(fov * 3.14159 / 180 / 2) evaluated in double as the reference, to float.
float film_height(const nr_camera& cam);

// Flattened scene in loader order.
struct HostScene {
    std::vector<float> pos;   // 9 per triangle
    std::vector<float> uv;    // 6 per triangle
    std::vector<float> nrm;   // 9 per triangle
    std::vector<int32_t> mat;
    std::vector<nr_material> mats;
    std::vector<int32_t> tex_wh;
    std::vector<float> tex_data;
    int32_t env_tex = -1;
    float env_gain = 1.0f;
    int num_tris() const { return (int)mat.size(); }
};

// Copies a caller description, applying the Triangle constructor's
// face-normal rule (src/scene/triangle.cpp:12-25). Returns "" or an error.
std::string scene_from_desc(const nr_scene_desc& d, HostScene& out);

// Loader::fromSceneDescription / loadObj / loadMtl (src/scene/loader.cpp).
// Texture maps referenced by MTL files may be PNG, PFM or binary PPM files
// (the reference decodes through Qt, which also reads JPG; JPG is not
// supported here). Returns "" or an error message.
std::string scene_from_text(const std::string& desc, HostScene& out);

// Reads a PNG or binary PPM (8-bit, decoded with c^2.2 as Texture::load
// does) or a PFM (float, used as is) image into linear RGB floats, row 0 at
// the top.
std::string read_image(const std::string& path, int& w, int& h, std::vector<float>& rgb);

// Sampling table of an environment map for envis=1 (no counterpart in the
// reference, whose ptnee only looks the map up on a miss). Cell (x, y) is
// the square between texels (x, y) and (x + 1, y + 1) over which the
// bilinear lookup interpolates (texels past the right / bottom edge are
// black, as Texture::pixel makes them). Its weight is the largest r + g + b
// of its four corners times sin(theta) at the cell's centre row, theta =
// (y + 0.5) / h * 3.14159; rows and columns are drawn from cumulative sums
// (float, in index order, the last entry forced to 1).
struct EnvTable {
    int w = 0, h = 0;
    std::vector<float> weight;   // w * h
    std::vector<float> row_cdf;  // h
    std::vector<float> col_cdf;  // w * h, per row
    float total = 0.f;
};
void build_env_table(const float* rgb, int w, int h, EnvTable& out);

// Binary BVH with the reference's SAH (BVH::_divide, src/hierarchy/bvh.cpp:5-58):
// primitives sorted by pMax along each axis, prefix/suffix surface-area sweep
// with cost SA_L * |L| + SA_R * (|R| + 1), leaves of at most 5 triangles.
// Nodes are stored depth-first, left child first.
struct BvhNode {
    float lo[3], hi[3];
    int32_t left, right;      // -1 for a leaf
    int32_t first, count;     // into leaf_tris for a leaf
    int32_t depth;
};
struct Bvh {
    std::vector<BvhNode> nodes;
    std::vector<int32_t> leaf_tris;  // triangle indices (loader order), leaves depth-first
    int32_t max_depth = 0;
};
// Stops past depth_limit (the tree would be refused by the traversal's
// stack) and returns no nodes with max_depth = depth_limit + 1, instead of
// recursing as deep as the scene asks (identical triangles make a chain).
void build_bvh(const HostScene& s, Bvh& out, int threads, int depth_limit = 2048);

// A tree given by the caller in the layout of nr_bvh_export (box[6] per
// node, kids[2] with -1, -1 for a leaf, leaf_first / leaf_count into
// leaf_tris, the triangle order in loader indices) over the triangles of s,
// checked and turned into out: node 0 is the root; every other node is the
// child of exactly one node, which precedes it; leaves partition leaf_tris,
// which is a permutation of the triangles; every triangle lies inside its
// leaf's box; the depth is at most depth_limit. Returns "" or what is wrong.
std::string bvh_from_arrays(const HostScene& s, int num_nodes, const float* box, const int32_t* kids,
                            const int32_t* leaf_first, const int32_t* leaf_count, const int32_t* leaf_tris,
                            int num_leaf_tris, int depth_limit, Bvh& out);

// The shape the device traversal relies on, checked on the child references
// of the GPU node array (two per inner node: >= 0 an inner node, < 0 a leaf
// -1 - ((first << 3) | count)): every inner node is the child of at most one
// inner node, which has a smaller index, and every leaf's triangles lie in
// [0, num_tris). A walk over such a tree visits each node at most once and
// ends. Returns "" or what is wrong.
std::string check_tree_refs(const int32_t* refs, int num_inner, int num_tris);

}  // namespace nr
