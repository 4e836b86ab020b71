// Device-side scene and wavefront layouts shared by the host code and the
// CUDA kernels of libnuray_gpu.so.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

#include "../../include/nuray.h"

// Entries of the per-thread traversal stack; scenes whose BVH is deeper are
// rejected at creation.
#define NR_STACK_LIMIT 96

// Default pruning margin of the closest-hit and shadow walks: a subtree is
// skipped when its entry distance exceeds the best hit by this relative
// amount (DeviceScene::prune_k = 1 + NR_PRUNE_MARGIN; prune=0 turns it off).
#define NR_PRUNE_MARGIN 1e-3f

namespace nr {

// BVH child reference: >= 0 is an internal node index, < 0 a leaf
// -1 - ((first << 3) | count) with `first` into the flattened triangle
// arrays (leaves laid out in depth-first order) and count <= 5.
__host__ __device__ inline int32_t leaf_ref(int32_t first, int32_t count) { return -1 - ((first << 3) | count); }
__host__ __device__ inline int32_t leaf_first(int32_t ref) { return (-1 - ref) >> 3; }
__host__ __device__ inline int32_t leaf_count(int32_t ref) { return (-1 - ref) & 7; }

// Internal BVH node, 64 bytes: both children's boxes and references.
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (ref0, ref1, depth, 0) as int bits
struct alignas(16) GpuNode {
    float4 a, b, c;
    int4 d;
};

// Per flattened triangle, traversal data, 48 bytes:
//   g0 = (p0.xyz, loader index bits), g1 = (e1.xyz, material bits), g2 = (e2.xyz, 0)
// with e1 = p1 - p0 and e2 = p2 - p0 rounded exactly as the reference does.
// Shading data, 64 bytes:
//   s0 = (n0.xyz, t0.x), s1 = (n1.xyz, t0.y), s2 = (n2.xyz, t1.x), s3 = (t1.y, t2.x, t2.y, material bits)
struct DeviceScene {
    const GpuNode* nodes;
    const float4* tri_geo;    // 3 per triangle
    const float4* tri_shade;  // 4 per triangle
    const nr_material* mats;
    const float4* tex_texels;
    const int4* tex_info;     // (w, h, texel offset, 0)
    const float4* lights;     // 6 per emitter: (p0, Ke.x) (p1, Ke.y) (p2, Ke.z) (n0,0) (n1,0) (n2,0)
    const float* light_cdf;
    const int32_t* light_guide;  // light_guide_k + 1 entries: lower_bound(light_cdf, b / light_guide_k)
    int32_t light_guide_k;       // a power of two
    const int32_t* light_mat;  // material index of each emitter
    int32_t num_lights;
    float light_p;            // LightSampler::p()
    int32_t root_ref;         // root as a child reference; INT32_MIN for an empty scene
    float root_lo[3], root_hi[3];
    int32_t num_tris;
    int32_t num_mats;
    int32_t env_tex;
    float env_gain;
    const float* env_weight;   // environment sampling table (envis=1), see EnvTable in host_scene.h
    const float* env_row_cdf;
    const float* env_col_cdf;
    float env_total;
    uint32_t cat_mask;        // shading categories that can occur: bit t for each material type present, and misses
    int32_t max_depth;        // deepest leaf (root = 0)
    int32_t num_nodes;        // internal nodes
    float prune_k;            // subtrees entered beyond prune_k x the best hit are skipped (infinity: none)
    const GpuNode* nodes_fast;  // the same nodes with every box widened for box_test_plain (traversal mode 2)
    float fast_origin_bound;    // mode 2 is conservative for ray origins with every |coordinate| <= this
};

// Render policy decoded from the parameter string.
struct Policy {
    float prr;        // survival probability (reference key prr, default 0.8)
    int32_t mis;      // reference key mis (default 1)
    int32_t rrdepth;  // RR applies at vertex index >= rrdepth (0 = reference)
    int32_t maxdepth; // 0 = unbounded (reference)
    uint32_t seed_lo, seed_hi;
    int32_t imgw, imgh;
    int32_t nee;      // 1: ptnee (RendererPTLS); 0: pt (RendererPT), no light sampling
    int32_t excl;     // 1: renderer=nrc's estimator (RendererNRC::trace): light samples without
                      // MIS, emitter hits dropped after a light sample, paths go on while u < prr
    int32_t coin;     // 1: a training coin is drawn after the jitter (RendererNRC::render)
    int32_t force_train;  // 1: every path is a training path (RendererNRC::render's first pass)
    int32_t envis;    // 1: one environment light sample per light-sampling vertex, MIS against BSDF misses
    int32_t trav;     // traversal tests: 0 exact arithmetic only, 1 fast path with exact fallback (same hits)
    int32_t adj;      // 1: a light sample is traced whenever its gradient can be nonzero, even where
                      // its contribution is zero (the adjoint's first pass); radiance unchanged
};

// One 16-byte field of every slot, stored beside another field that is read
// and written with it, so that a slot's pair fills one 32-byte sector: once
// the category sort has scattered the slots, each separate 16-byte field
// cost a whole sector. Pairs: (ray_o, ray_d) and (thr, meta). Measured
// against separate arrays: 1M-triangle frame 901.5 / 898.1 Mpaths/s, with
// textures, sky and dielectrics 698.0 / 693.8, adjoint 735.2 / 720.2.
template <class T>
struct SlotField {
    T* p;
    __host__ __device__ T& operator[](size_t i) const { return p[2 * i]; }
};

// Wavefront path state, structure of arrays, one slot per in-flight path.
struct PathState {
    SlotField<float4> ray_o;  // (origin, unused)
    SlotField<float4> ray_d;  // (direction, unused), beside ray_o
    float4* hit;     // (t, b1, b2, flattened triangle bits or -1)
    SlotField<float4> thr;    // (throughput, light_fac)
    float4* rad;     // (radiance, unused)
    SlotField<uint4> meta;    // (pixel, sample, draws taken, vertex depth), beside thr
    // queues of slot indices
    int32_t* queue_in;
    int32_t* queue_out;
    int32_t* sorted;      // slots bucketed by shading category
    // shadow rays
    float4* sh_o;    // (origin, t limit)
    float4* sh_d;    // (direction, slot bits)
    float4* sh_c;    // (contribution if unoccluded, training record)
    int32_t sh_cap;  // entries of the shadow-ray queue (1 or 2 per slot)
    uint8_t* vis;    // null, or per slot: 1 if its light sample of this bounce was unoccluded
    // device counters (see Counter)
    uint32_t* counters;
};

// Online neural radiance cache inside the wavefront (k_shade<true>): query
// and training records written during shading, consumed after the batch.
struct NrcCtx {
    uint4* q_rec;         // [cap][2] compact query records (nrc_encode.cuh)
    int32_t* q_slot;
    float4* q_thr;        // throughput at the query vertex
    void* t_x;            // __nv_bfloat16 [tcap][80] training encodings
    int32_t* t_slot;
    float4* t_thr;        // throughput on arrival at the vertex
    float4* t_before;     // path radiance before the vertex
    uint32_t* counters;   // [0] queries, [1] training records
    int32_t tcap;
    uint32_t train_stride;  // one path in train_stride is a training path
    int32_t query;          // 0: train only (every path runs to the end)
    int32_t min_depth;      // first vertex depth at which the cache may end a path
    float rough;            // GGX roughness from which a vertex counts as diffuse
    int32_t train_depth;    // > 0: training paths end in the cache from this vertex depth on
    int32_t direct;         // 1: the cache holds radiance after the vertex's own light sample
                            // (queries still sample a light); 0: all outgoing radiance
    int32_t first;          // 1: a path may end at its first diffuse vertex itself, not only after it
    float lo[3], inv_ext[3];  // scene box for the position encoding
};

// meta.w: vertex depth in the low 16 bits; this flag once a diffuse vertex
// has been passed (NRC mode).
#define NR_META_SEEN_DIFFUSE 0x80000000u
#define NR_META_TRAIN 0x40000000u  // training path by coin or forced (renderer=nrc)
#define NR_META_DEPTH_MASK 0xffffu

// Shading categories for the material sort: one per material type, then
// rays that left the scene.
enum { CAT_MISS = 6, NUM_CAT = 7 };

enum Counter {
    CNT_IN = 0,        // live paths in queue_in
    CNT_OUT = 1,       // continuing paths appended to queue_out
    CNT_SHADOW = 2,    // shadow rays appended
    CNT_WORK = 3,      // persistent-kernel work cursor (closest hit)
    CNT_WORK_SH = 4,   // persistent-kernel work cursor (shadow)
    CNT_CAT = 8,       // 8..14: per-category counts
    CNT_ERR = 16,      // internal error bits (NR_ERRBIT_*); 0 = fine
    CNT_RAYS = 18,     // 64-bit totals (lo, hi): extension rays,
    CNT_SHRAYS = 20,   // shadow rays,
    CNT_NODES = 22,    // BVH nodes visited by closest-hit rays (instrumented runs),
    CNT_TRIS = 24,     // triangles tested by closest-hit rays,
    CNT_SH_NODES = 26, // nodes visited by shadow rays,
    CNT_SH_TRIS = 28,  // triangles tested by shadow rays
    NUM_COUNTERS = 32
};

// Bits of counters[CNT_ERR], each set by a kernel that met the condition
// and returned instead of going on; the host turns them into NR_ERR_DEVICE.
enum ErrBit : uint32_t {
    NR_ERRBIT_STACK = 1u,       // traversal stack overflow
    NR_ERRBIT_STEPS = 2u,       // traversal step budget spent (corrupted tree)
    NR_ERRBIT_SHADOW_Q = 4u,    // shadow-ray queue full
    NR_ERRBIT_TC_WAIT = 8u,     // a tensor-core MMA wait timed out; the CTA waited again and stopped
    NR_ERRBIT_BOUNCES = 16u,    // the tail kernel's path still alive after NR_TAIL_MAX_BOUNCES bounces
    NR_ERRBIT_TC_LOST = 32u,    // the second MMA wait timed out too: tensor memory freed with MMAs possibly
                                // in flight; the library stops using the tensor-core kernels
};

// Text for the error bits set in `bits`.
inline const char* err_bits_text() {
    return "1 stack overflow, 2 traversal step cap, 4 shadow queue full, 8 tensor-core wait timed out, "
           "16 paths alive after 4096 bounces in the tail kernel, 32 tensor-core MMAs unfinished after a second wait";
}

}  // namespace nr
