// extern "C" boundary of libnuray_gpu.so (include/nuray.h): scene upload
// and the host loop of the ptnee wavefront.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/nuray.h"
#include "bvh_gpu.h"
#include "host_scene.h"
#include "integrator.h"
#include "nrc.h"
#include "adjoint.h"
#include "noalloc.h"
#include <random>

namespace {

thread_local std::string g_last_error;

struct NrError : std::runtime_error {
    int code;
    NrError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define NR_CUDA(call)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) {                                                                      \
            throw NrError(e_ == cudaErrorMemoryAllocation ? NR_ERR_OOM : NR_ERR_CUDA,                 \
                          std::string(#call) + ": " + cudaGetErrorString(e_));                        \
        }                                                                                             \
    } while (0)

template <class F>
int guarded(F&& f) {
    try {
        f();
        return NR_OK;
    } catch (const NrError& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return NR_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return NR_ERR_INVALID;
    }
}

// Device bytes a scene may hold (scene option max_device_bytes): every
// buffer of the scene draws on it, and an allocation past it fails with
// NR_ERR_OOM as a failed cudaMalloc does.
struct Budget {
    size_t cap = SIZE_MAX;
    size_t used = 0;
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    Budget* budget = nullptr;
    // Replaces the buffer by one of n bytes. Over the cap it throws before
    // touching the old buffer; if cudaMalloc fails the buffer is left empty,
    // so callers that cache sizes or pointers into it reset them first.
    void alloc(size_t n) {
        if (budget && n > budget->cap - (budget->used - bytes))
            throw NrError(NR_ERR_OOM, "device allocation of " + std::to_string(n) + " bytes exceeds the scene's cap of " +
                                          std::to_string(budget->cap) + " bytes (" +
                                          std::to_string(budget->used - bytes) + " in use)");
        release();
        if (n == 0) return;
        NR_CUDA(cudaMalloc(&p, n));
        bytes = n;
        if (budget) budget->used += n;
    }
    void release() {
        if (p) cudaFree(p);
        if (budget) budget->used -= bytes;
        p = nullptr;
        bytes = 0;
    }
    // keeps the current allocation when it is large enough
    void ensure(size_t n) {
        if (n > bytes) alloc(n);
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

// One neural radiance cache on one device.
struct nr_nrc {
    std::mutex mu;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    DevBuf pbuf;  // params | grad | m | v (FP32) then the BF16 copy
    nr::NrcDev dev{};
    float lr = 1e-3f, b1 = 0.9f, b2 = 0.99f, eps = 1e-8f, ema = 0.0f;
    int step = 0;
    // scratch for batches: x (BF16), y, out, acts, dz, loss
    DevBuf batch;
    int batch_cap = 0;
    __nv_bfloat16 *x = nullptr, *acts = nullptr, *dz = nullptr;
    float *y = nullptr, *out = nullptr, *loss = nullptr;
    float* xf = nullptr;  // FP32 staging of caller inputs
    float* loss_host = nullptr;  // pinned
    bool tc = true;              // inference on tcgen05 (nrc_tc.cu); false: mma.sync (nrc.cu)
    uint32_t tc_first_wait = NR_TC_FIRST_WAIT_LIMIT;  // bound of the first MMA wait of a layer
    // the tensor-core kernels, unless disabled here or, after an unfinished
    // MMA group (error bit 32), for the whole process
    bool use_tc() const { return tc && nr::nrc_tc_enabled(); }
    DevBuf errbuf;               // error word of the tensor-core kernels
    DevBuf wt_img;               // packed transposed weights of the tensor-core backward pass
    uint32_t* err_host = nullptr;  // pinned

    ~nr_nrc() {
        cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        pbuf.release();
        batch.release();
        if (loss_host) cudaFreeHost(loss_host);
        if (err_host) cudaFreeHost(err_host);
        errbuf.release();
        wt_img.release();
        if (stream) cudaStreamDestroy(stream);
    }
};

struct nr_scene {
    std::mutex mu;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    nr::HostScene host;
    nr::Bvh bvh;
    nr::DeviceScene dev{};
    DevBuf nodes, nodes_fast, tri_geo, tri_shade, mats, texels, tex_info, lights, light_cdf, light_guide, light_mat;
    DevBuf adj_L;  // per-path radiance for the adjoint replay
    DevBuf adj_wave;  // per-slot state of the wavefront adjoint replay
    DevBuf env_weight, env_row_cdf, env_col_cdf;  // environment sampling table (envis=1)
    int num_gpu_nodes = 0;
    // wavefront state
    DevBuf path_mem, film, out_hdr, out_rgb8, pix_list, scratch;
    int film_pixels = 0;
    uint64_t film_samples = 0;  // samples summed in film (accumulate=1 keeps adding)
    nr::PathState ps{};
    int capacity = 0;
    int sh_mult = 1;  // shadow-ray queue entries per path slot
    uint32_t* counters_host = nullptr;  // pinned
    nr_stats stats{};
    std::vector<cudaEvent_t> ev_pool;  // profile=1: events around every kernel group
    nr_nrc* nrc = nullptr;             // attached cache (not owned)
    DevBuf nrc_mem;                    // query / training records of the online cache
    int nrc_cap = 0, nrc_tcap = 0;
    nr::NrcCtx nrc_ctx{};
    float* nrc_pred = nullptr;
    __nv_bfloat16* nrc_qx = nullptr;  // expanded query rows, for a cache on the mma.sync kernels only
    float nrc_last_loss = 0.f;
    double bvh_wall_ms = 0.0, bvh_device_ms = 0.0;  // last BVH build
    Budget budget;

    nr_scene() {
        for (auto* b : all_bufs()) b->budget = &budget;
    }
    std::vector<DevBuf*> all_bufs() {
        return {&nodes, &nodes_fast, &tri_geo, &tri_shade, &mats, &texels, &tex_info, &lights, &light_cdf, &light_guide,
                &light_mat,
                &adj_L, &adj_wave, &env_weight, &env_row_cdf, &env_col_cdf, &path_mem, &film, &out_hdr, &out_rgb8,
                &pix_list, &scratch, &nrc_mem};
    }

    ~nr_scene() {
        if (device >= 0) cudaSetDevice(device);
        if (stream) cudaStreamSynchronize(stream);
        for (auto* b : all_bufs()) b->release();
        if (counters_host) cudaFreeHost(counters_host);
        for (auto& e : ev_pool) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

uint64_t device_bytes(const nr_scene* s) {
    uint64_t b = 0;
    for (auto* x : {&s->nodes, &s->nodes_fast, &s->tri_geo, &s->tri_shade, &s->mats, &s->texels, &s->tex_info, &s->lights,
                    &s->light_cdf, &s->light_guide, &s->light_mat})
        b += x->bytes;
    return b;
}

template <class T>
void upload(DevBuf& buf, const std::vector<T>& v, cudaStream_t st) {
    buf.alloc(v.size() * sizeof(T));
    if (!v.empty()) NR_CUDA(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

inline float bits_f(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }

// Flattens triangles in leaf order, converts the BVH into the two-box node
// layout and builds the emitter table (LightSampler::setPrimitives,
// src/sampler/lightsampler.cpp:4-39), then copies all of it to the device.
void upload_scene(nr_scene* s) {
    const nr::HostScene& H = s->host;
    const nr::Bvh& B = s->bvh;
    const int n = H.num_tris();
    cudaStream_t st = s->stream;

    std::vector<float4> geo(3 * (size_t)n), shade(4 * (size_t)n);
    for (int k = 0; k < n; ++k) {
        int i = B.leaf_tris[k];
        const float* p = &H.pos[9 * (size_t)i];
        const float* t = &H.uv[6 * (size_t)i];
        const float* nn = &H.nrm[9 * (size_t)i];
        geo[3 * k] = make_float4(p[0], p[1], p[2], bits_f(i));
        geo[3 * k + 1] = make_float4(p[3] - p[0], p[4] - p[1], p[5] - p[2], bits_f(H.mat[i]));
        geo[3 * k + 2] = make_float4(p[6] - p[0], p[7] - p[1], p[8] - p[2], 0.0f);
        shade[4 * k] = make_float4(nn[0], nn[1], nn[2], t[0]);
        shade[4 * k + 1] = make_float4(nn[3], nn[4], nn[5], t[1]);
        shade[4 * k + 2] = make_float4(nn[6], nn[7], nn[8], t[2]);
        shade[4 * k + 3] = make_float4(t[3], t[4], t[5], bits_f(H.mat[i]));
    }

    // internal nodes get consecutive GPU indices in depth-first order
    std::vector<int> gpu_index(B.nodes.size(), -1);
    int ng = 0;
    for (size_t i = 0; i < B.nodes.size(); ++i)
        if (B.nodes[i].left >= 0) gpu_index[i] = ng++;
    auto ref_of = [&](int i) {
        const nr::BvhNode& c = B.nodes[i];
        return c.left >= 0 ? gpu_index[i] : nr::leaf_ref(c.first, c.count);
    };
    std::vector<nr::GpuNode> gn(ng);
    for (size_t i = 0; i < B.nodes.size(); ++i) {
        const nr::BvhNode& N = B.nodes[i];
        if (N.left < 0) continue;
        const nr::BvhNode& L = B.nodes[N.left];
        const nr::BvhNode& R = B.nodes[N.right];
        nr::GpuNode& g = gn[gpu_index[i]];
        g.a = make_float4(L.lo[0], L.hi[0], L.lo[1], L.hi[1]);
        g.b = make_float4(R.lo[0], R.hi[0], R.lo[1], R.hi[1]);
        g.c = make_float4(L.lo[2], L.hi[2], R.lo[2], R.hi[2]);
        g.d = make_int4(ref_of(N.left), ref_of(N.right), N.depth, 0);
    }
    s->num_gpu_nodes = ng;
    // The traversal loops rely on this shape rather than counting steps:
    // every inner node is the child of at most one inner node, which has a
    // smaller index, and every leaf's triangles lie within the scene. A walk
    // then visits each node at most once and ends, and its stack holds at most
    // max_depth entries (checked against NR_STACK_LIMIT before the upload).
    {
        std::vector<int32_t> refs(2 * (size_t)ng);
        for (int i = 0; i < ng; ++i) {
            refs[2 * (size_t)i] = gn[i].d.x;
            refs[2 * (size_t)i + 1] = gn[i].d.y;
        }
        const std::string bad = nr::check_tree_refs(refs.data(), ng, n);
        if (!bad.empty()) throw NrError(NR_ERR_INVALID, bad);
    }

    // The same nodes with every child box widened by delta for the one-FMA
    // box test without margin (traversal mode 2). For a ray origin o with
    // |o_i| <= Bo and box bounds b with |b_i| <= A, the test's quotient
    // fma(b, 1/d, -o/d) and the reference's RN(RN(b - o) / d) each lie within
    // 2^-23 (|b| + |o|) / |d| of (b - o) / d, so widening by more than
    // 2.4e-7 (A + Bo) makes the test accept every box the reference's test
    // accepts. Origins are allowed out to Bo = 2 A + 4 E (E the largest half
    // extent of the scene box); delta = 4e-6 (A + E) covers that with more
    // than 2x to spare, and is a relative 1e-3 of a 1M-triangle scene's
    // smallest leaves at most.
    float A = 0.f, E = 0.f;
    if (!B.nodes.empty())
        for (int k = 0; k < 3; ++k) {
            A = std::max(A, std::max(std::fabs(B.nodes[0].lo[k]), std::fabs(B.nodes[0].hi[k])));
            E = std::max(E, 0.5f * (B.nodes[0].hi[k] - B.nodes[0].lo[k]));
        }
    const float delta = 4e-6f * (A + E) + 1e-30f;
    std::vector<nr::GpuNode> gf(gn);
    for (auto& g : gf) {
        g.a = make_float4(g.a.x - delta, g.a.y + delta, g.a.z - delta, g.a.w + delta);
        g.b = make_float4(g.b.x - delta, g.b.y + delta, g.b.z - delta, g.b.w + delta);
        g.c = make_float4(g.c.x - delta, g.c.y + delta, g.c.z - delta, g.c.w + delta);
    }

    // emitters in loader order, weight = Triangle::area (twice the area)
    std::vector<float4> lt;
    std::vector<float> pdf;
    std::vector<int32_t> lmat;
    float sum = 0.0f;
    for (int i = 0; i < n; ++i) {
        const nr_material& M = H.mats[H.mat[i]];
        if (M.type != NR_MAT_LIGHT) continue;
        const float* p = &H.pos[9 * (size_t)i];
        const float* nn = &H.nrm[9 * (size_t)i];
        float e1[3] = {p[3] - p[0], p[4] - p[1], p[5] - p[2]};
        float e2[3] = {p[6] - p[0], p[7] - p[1], p[8] - p[2]};
        float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        float w = (float)std::sqrt((double)(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
        pdf.push_back(w);
        lmat.push_back(H.mat[i]);
        sum += w;
        lt.push_back(make_float4(p[0], p[1], p[2], M.c0[0]));
        lt.push_back(make_float4(p[3], p[4], p[5], M.c0[1]));
        lt.push_back(make_float4(p[6], p[7], p[8], M.c0[2]));
        lt.push_back(make_float4(nn[0], nn[1], nn[2], 0.0f));
        lt.push_back(make_float4(nn[3], nn[4], nn[5], 0.0f));
        lt.push_back(make_float4(nn[6], nn[7], nn[8], 0.0f));
    }
    sum = (float)((double)sum + 1e-8);
    std::vector<float> cdf;
    float acc = 1e-6f;
    for (float& x : pdf) { x /= sum; acc += x; cdf.push_back(acc); }
    // Guide table of the CDF: entry b is lower_bound(cdf, b / K) for a power
    // of two K (twice the emitters, at most 2^16), so the device's lower_bound
    // of r searches only between entries floor(r K) and floor(r K) + 1 (r K
    // is exact in float) and returns the index the full search returns.
    int guide_k = 1;
    while (guide_k < 2 * (int)cdf.size() && guide_k < (1 << 16)) guide_k *= 2;
    std::vector<int32_t> guide(guide_k + 1);
    for (int b = 0; b <= guide_k; ++b) {
        const float u = (float)b / (float)guide_k;
        guide[b] = (int32_t)(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
    }

    std::vector<float4> texels;
    std::vector<int4> tinfo;
    size_t off = 0;
    nr::EnvTable env_table;
    for (size_t t = 0; t < H.tex_wh.size() / 2; ++t) {
        int w = H.tex_wh[2 * t], h = H.tex_wh[2 * t + 1];
        if ((int)t == H.env_tex) nr::build_env_table(&H.tex_data[3 * off], w, h, env_table);
        tinfo.push_back(make_int4(w, h, (int)(off / 1), 0));
        for (size_t k = 0; k < (size_t)w * h; ++k) {
            const float* c = &H.tex_data[3 * (off + k)];
            texels.push_back(make_float4(c[0], c[1], c[2], 0.0f));
        }
        off += (size_t)w * h;
    }
    if (off > (size_t)INT32_MAX) throw NrError(NR_ERR_INVALID, "textures exceed 2^31 texels");

    upload(s->tri_geo, geo, st);
    upload(s->tri_shade, shade, st);
    upload(s->nodes, gn, st);
    upload(s->nodes_fast, gf, st);
    upload(s->mats, H.mats, st);
    upload(s->texels, texels, st);
    upload(s->tex_info, tinfo, st);
    upload(s->lights, lt, st);
    upload(s->light_cdf, cdf, st);
    upload(s->light_guide, guide, st);
    upload(s->light_mat, lmat, st);
    upload(s->env_weight, env_table.weight, st);
    upload(s->env_row_cdf, env_table.row_cdf, st);
    upload(s->env_col_cdf, env_table.col_cdf, st);
    NR_CUDA(cudaStreamSynchronize(st));

    nr::DeviceScene& D = s->dev;
    D.nodes = s->nodes.as<nr::GpuNode>();
    D.nodes_fast = s->nodes_fast.as<nr::GpuNode>();
    D.fast_origin_bound = 2.0f * A + 4.0f * E;
    D.tri_geo = s->tri_geo.as<float4>();
    D.tri_shade = s->tri_shade.as<float4>();
    D.mats = s->mats.as<nr_material>();
    D.tex_texels = s->texels.as<float4>();
    D.tex_info = s->tex_info.as<int4>();
    D.lights = s->lights.as<float4>();
    D.light_cdf = s->light_cdf.as<float>();
    D.light_guide = s->light_guide.as<int32_t>();
    D.light_guide_k = guide_k;
    D.light_mat = s->light_mat.as<int32_t>();
    D.env_weight = env_table.w ? s->env_weight.as<float>() : nullptr;
    D.env_row_cdf = env_table.w ? s->env_row_cdf.as<float>() : nullptr;
    D.env_col_cdf = env_table.w ? s->env_col_cdf.as<float>() : nullptr;
    D.env_total = env_table.total;
    D.num_lights = (int)pdf.size();
    D.light_p = (float)(1.0 / ((double)sum + 1e-8));
    D.num_tris = n;
    D.num_mats = (int)H.mats.size();
    D.cat_mask = 1u << nr::CAT_MISS;
    for (const auto& m : H.mats)
        if (m.type >= 0 && m.type < nr::CAT_MISS) D.cat_mask |= 1u << m.type;
    D.env_tex = H.env_tex;
    D.env_gain = H.env_gain;
    D.max_depth = B.max_depth;
    D.num_nodes = ng;
    D.prune_k = 1.0f + NR_PRUNE_MARGIN;
    if (n == 0) {
        D.root_ref = INT32_MIN;
    } else {
        const nr::BvhNode& R = B.nodes[0];
        D.root_ref = R.left >= 0 ? 0 : nr::leaf_ref(R.first, R.count);
        for (int k = 0; k < 3; ++k) { D.root_lo[k] = R.lo[k]; D.root_hi[k] = R.hi[k]; }
    }
}

void finish_scene(nr_scene* s, const char* options, nr::Bvh* prebuilt = nullptr) {
    const nr::Config opt(options ? options : "");
    const std::string bvh = opt.get_str("bvh");
    if (!bvh.empty() && bvh != "host" && bvh != "gpu") throw NrError(NR_ERR_INVALID, "bvh must be host or gpu");
    const std::string cap = opt.get_str("max_device_bytes");
    if (!cap.empty()) {
        size_t used = 0;
        unsigned long long v = 0;
        try { v = std::stoull(cap, &used); } catch (const std::exception&) { used = 0; }
        if (used != cap.size() || cap[0] == '-') throw NrError(NR_ERR_INVALID, "max_device_bytes must be a byte count");
        s->budget.cap = (size_t)v;
    }
    NR_CUDA(cudaGetDevice(&s->device));
    NR_CUDA(cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->device));
    NR_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    NR_CUDA(cudaMallocHost(&s->counters_host, nr::NUM_COUNTERS * sizeof(uint32_t)));
    auto t0 = std::chrono::steady_clock::now();
    s->bvh_device_ms = 0.0;
    // the deepest tree the traversal stacks hold; the builders stop past it
    const int depth_limit = NR_STACK_LIMIT - 2;
    if (prebuilt) {
        s->bvh = std::move(*prebuilt);
    } else if (bvh == "gpu") {
        std::string err = nr::build_bvh_gpu(s->host.pos.data(), s->host.num_tris(), s->bvh, s->stream, &s->bvh_device_ms,
                                            depth_limit);
        if (!err.empty()) throw NrError(NR_ERR_CUDA, err);
    } else {
        int threads = (int)std::max(1u, std::thread::hardware_concurrency());
        nr::build_bvh(s->host, s->bvh, threads, depth_limit);
    }
    s->bvh_wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (s->bvh.max_depth > depth_limit)
        throw NrError(NR_ERR_INVALID, "BVH deeper than " + std::to_string(depth_limit) +
                                          " levels (the traversal stack's limit; many coincident triangles make "
                                          "the reference's SAH split them off one by one)");
    nr::launch_setup(s->num_sms);
    upload_scene(s);
    // the static scratch of nr_intersect_noalloc: reserved and located on
    // this device now, so that those calls load and allocate nothing (a
    // failure here is reported by the first such call, which tries again)
    (void)nr::noalloc_prepare(s->device);
}

// Drops every buffer a call grows for its own work (path state, films,
// staging, the adjoint's records and the cache's record tables), keeping the
// scene data: after an allocation failure the scene holds only what the next
// call needs to start from.
void release_work_buffers(nr_scene* s) {
    cudaStreamSynchronize(s->stream);
    for (auto* b : {&s->path_mem, &s->film, &s->out_hdr, &s->out_rgb8, &s->pix_list, &s->scratch, &s->adj_L,
                    &s->adj_wave, &s->nrc_mem})
        b->release();
    s->capacity = 0;
    s->sh_mult = 1;
    s->film_pixels = 0;
    s->film_samples = 0;
    s->nrc_cap = s->nrc_tcap = 0;
    s->nrc_qx = nullptr;
}

// Runs f, a call's work on scene s; an allocation failure inside frees the
// call's work buffers before it is reported.
template <class F>
void with_oom_release(nr_scene* s, F&& f) {
    try {
        f();
    } catch (const NrError& e) {
        if (e.code == NR_ERR_OOM) release_work_buffers(s);
        throw;
    }
}

// Sizes the path-state buffers for `cap` slots.
void ensure_paths(nr_scene* s, int cap, int sh_mult = 1) {
    if (cap <= s->capacity && sh_mult <= s->sh_mult) return;
    cap = std::max(cap, s->capacity);
    sh_mult = std::max(sh_mult, s->sh_mult);
    const size_t C = (size_t)cap, CS = C * (size_t)sh_mult;
    const size_t f4 = 16;
    size_t bytes = C * f4 * 5 + C * 16 + C * 4 * 2 + C * 4 * nr::NUM_CAT + CS * f4 * 3 + nr::NUM_COUNTERS * 4 + 256 * 16;
    const int old_cap = s->capacity;
    s->capacity = 0;  // no slots while the buffer is replaced (an allocation may fail)
    try {
        s->path_mem.alloc(bytes);
    } catch (...) {
        if (s->path_mem.p) s->capacity = old_cap;  // refused by the cap: the old buffer is intact
        throw;
    }
    char* p = s->path_mem.as<char>();
    auto take = [&](size_t n) { char* r = p; p += (n + 255) & ~size_t(255); return r; };
    nr::PathState& P = s->ps;
    float4* od = (float4*)take(2 * C * f4);  // (ray_o, ray_d) per slot
    P.ray_o.p = od;
    P.ray_d.p = od + 1;
    float4* tm = (float4*)take(2 * C * f4);  // (thr, meta) per slot
    P.thr.p = tm;
    P.meta.p = (uint4*)(tm + 1);
    P.hit = (float4*)take(C * f4);
    P.rad = (float4*)take(C * f4);
    P.queue_in = (int32_t*)take(C * 4);
    P.queue_out = (int32_t*)take(C * 4);
    P.sorted = (int32_t*)take(C * 4 * nr::NUM_CAT);
    P.sh_o = (float4*)take(CS * f4);
    P.sh_d = (float4*)take(CS * f4);
    P.sh_c = (float4*)take(CS * f4);
    P.sh_cap = (int32_t)std::min<size_t>(CS, (size_t)INT32_MAX);
    P.vis = nullptr;
    P.counters = (uint32_t*)take(nr::NUM_COUNTERS * 4);
    NR_CUDA(cudaMemsetAsync(P.counters, 0, nr::NUM_COUNTERS * 4, s->stream));
    s->capacity = cap;
    s->sh_mult = sh_mult;
}

// Sizes the batch scratch of a cache for m rows.
void nrc_ensure_batch(nr_nrc* c, int m) {
    if (m <= c->batch_cap) return;
    size_t M = (size_t)m;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    size_t bytes = al(M * NRC_IN * 2) + al(M * 12) + al(M * 12) + al(4 * M * NRC_H * 2) + al(5 * M * NRC_H * 2) + 256 +
                   al(M * NRC_IN * 4);
    c->batch.alloc(bytes);
    char* p = c->batch.as<char>();
    auto take = [&](size_t b) { char* r = p; p += al(b); return r; };
    c->x = (__nv_bfloat16*)take(M * NRC_IN * 2);
    c->y = (float*)take(M * 12);
    c->out = (float*)take(M * 12);
    c->acts = (__nv_bfloat16*)take(4 * M * NRC_H * 2);
    c->dz = (__nv_bfloat16*)take(5 * M * NRC_H * 2);
    c->loss = (float*)take(4);
    c->xf = (float*)take(M * NRC_IN * 4);
    c->batch_cap = m;
}

// Forward and backward of the rows R (gradients added to c->dev.grad, loss
// to c->loss): on the tensor cores (tcgen05: forward and data gradients;
// weight gradients by mma.sync) with tc, else all by mma.sync. err: the
// word that receives bit 8 if a tensor-core wait timed out.
void nrc_forward_backward(nr_nrc* c, const __nv_bfloat16* x, const float* y, const nr::NrcRows& R, uint32_t* err,
                          cudaStream_t st) {
    if (c->use_tc()) {
        nr::nrc_launch_forward_tc(c->dev.wb, c->dev.params, x, R, c->out, c->num_sms, err, st, c->acts,
                                  c->tc_first_wait);
        nr::nrc_launch_backward_data_tc(c->dev.wb, c->out, y, c->acts, c->dz, R, c->loss, c->num_sms, c->wt_img.p, err,
                                        st, c->tc_first_wait);
        nr::nrc_launch_backward_weight(c->dev, x, c->dz, c->acts, R, c->num_sms, st);
    } else {
        nr::nrc_launch_forward(c->dev, x, R, c->out, c->acts, c->num_sms, st);
        nr::nrc_launch_backward(c->dev, x, c->out, y, c->acts, c->dz, R, c->loss, c->num_sms, st);
    }
}

// Gradient (and, when `update`, one Adam step) on m rows already on the
// device: x BF16 [m][80], y [m][3]. Returns the summed loss asynchronously in c->loss.
void nrc_train_device(nr_nrc* c, const __nv_bfloat16* x, const float* y, int m, bool update, cudaStream_t st) {
    nrc_ensure_batch(c, m);
    NR_CUDA(cudaMemsetAsync(c->loss, 0, 4, st));
    const nr::NrcRows R = nr::nrc_rows(m);
    nrc_forward_backward(c, x, y, R, c->errbuf.as<uint32_t>(), st);
    if (update) {
        c->step++;
        nr::nrc_launch_adam(c->dev, c->lr, c->b1, c->b2, c->eps, c->step, c->ema, R, st, c->errbuf.as<uint32_t>());
    }
}

struct RenderArgs {
    nr::Policy pol;
    nr_camera cam;
    int spp;
    int wave;
    bool profile;
    bool count;
    int sample0;
    bool accumulate;
    // Wave layout: 0 scanline, 1 8x4 pixel tiles, 2 (default) a warp of
    // paths holds tile_samples consecutive samples of a pixel tile of
    // 32 / tile_samples pixels. Measured on the 1M-triangle frame at 64 spp
    // (Mpaths/s): 8x4 tiles 656.9; samples per warp 2: 668.1, 4: 679.0,
    // 8: 689.4, 16: 698.0, 32: 704.8. Paths of one pixel start together and
    // their first bounces stay close, so a warp walks much of the same tree.
    int tile;
    int tile_samples;     // 1, 2, 4, 8, 16 or 32
    // With maxdepth: the bounces after which the live count is read back, so
    // that later bounces size the shading grid to the paths left (0: never;
    // -1, the default: 5 for waves of more than 2^22 paths, else never).
    // 1M-triangle scene: 1080p x 64 spp 704.3 Mpaths/s with the readback
    // against 699.0 without; 960x540 frames of 1 spp 2.789 ms with it,
    // 2.735 without (the wait costs more than the grid saves).
    int live_sync;
    // Small waves (at most 2^22 paths): the wavefront bounces after which
    // k_tail takes every live path to its end in one launch (0: never).
    // 960x540 frames of 1 spp on the 1M-triangle scene: 2.557 ms without,
    // 2.305 / 1.805 / 1.821 / 2.046 ms after 1 / 2 / 3 / 4 bounces.
    int tail;
    bool nrc;
    int nrc_train;    // training paths per wavefront batch
    int nrc_steps;    // Adam steps per batch
    int nrc_query;    // 0: train only
    int nrc_mindepth; // first vertex at which a path may end in the cache
    float nrc_rough;  // roughness from which a GGX vertex is diffuse
    int nrc_direct;   // 1: light sample at the query vertex, cache for the rest
    int nrc_train_depth;  // > 0: training paths end in the cache from this depth on
    int nrc_first;        // 1: paths may end at their first diffuse vertex itself
    bool nrc_pre;         // renderer=nrc: one all-training pass before the samples (RendererNRC::render)
    bool adj_mega;        // adjoint replay as one thread per path (adj=mega) instead of the wavefront
    bool prune;           // 0: every node whose box a ray enters is visited, as the reference does
    int64_t adj_rec_bytes;  // the adjoint's per-bounce hit and visibility records: at most this many bytes
                            // (0: none; the replay traces every bounce again from the Philox keys)
};

// The traversal mode a render can use: the widened-box walk (trav=1)
// holds for ray origins inside the scene's origin bound, which every
// surface point meets; a camera outside it gets the exact walk (trav=0,
// the same hits).
void check_camera(const nr_scene* s, RenderArgs& A) {
    const float b = s->dev.fast_origin_bound;
    for (int k = 0; k < 3; ++k)
        if (!(std::fabs(A.cam.pos[k]) <= b)) A.pol.trav = 0;
}

// The scene as the kernels of one call see it: the pruning factor of the
// call's traversals.
nr::DeviceScene scene_for(const nr_scene* s, bool prune) {
    nr::DeviceScene D = s->dev;
    D.prune_k = prune ? 1.0f + NR_PRUNE_MARGIN : INFINITY;
    return D;
}

RenderArgs parse_args(const nr_camera* cam, const char* params) {
    nr::Config c(params);
    RenderArgs a;
    a.pol.prr = c.get_float("prr", 0.8f);
    a.pol.mis = c.get_int("mis", 1) != 0 ? 1 : 0;
    a.pol.rrdepth = c.get_int("rrdepth", 0);
    a.pol.maxdepth = c.get_int("maxdepth", 0);
    uint64_t seed = 0;
    std::string ss = c.get_str("seed");
    if (!ss.empty()) seed = std::stoull(ss);
    a.pol.seed_lo = (uint32_t)seed;
    a.pol.seed_hi = (uint32_t)(seed >> 32);
    a.pol.imgw = c.get_int("imgw", 1);
    a.pol.imgh = c.get_int("imgh", 1);
    a.spp = c.get_int("spp", 1);
    a.pol.trav = c.get_int("trav", 1);
    a.prune = c.get_int("prune", 1) != 0;
    {
        const std::string rec = c.get_str("adj_records");
        a.adj_rec_bytes = int64_t(32) << 30;
        if (!rec.empty()) {
            size_t used = 0;
            long long v = -1;
            try { v = std::stoll(rec, &used); } catch (const std::exception&) { used = 0; }
            if (used != rec.size() || v < 0) throw NrError(NR_ERR_INVALID, "adj_records must be a byte count >= 0");
            a.adj_rec_bytes = v;
        }
    }
    // renderer=ptnee (RendererPTLS), pt (RendererPT, the same estimator without
    // light sampling) or nrc (RendererNRC: light samples without MIS, the
    // cache asked from vertex path_lim on, path_lim_train on training paths)
    const std::string renderer = c.get_str("renderer");
    a.pol.excl = a.pol.coin = a.pol.force_train = a.pol.adj = 0;
    if (renderer.empty() || renderer == "ptnee") a.pol.nee = 1;
    else if (renderer == "pt") a.pol.nee = 0;
    else if (renderer == "nrc") { a.pol.nee = 1; a.pol.excl = 1; a.pol.coin = 1; }
    else throw NrError(NR_ERR_INVALID, "renderer=" + renderer + " is not implemented (ptnee, pt, nrc)");
    a.pol.envis = c.get_int("envis", 0) != 0 ? 1 : 0;
    if (a.pol.envis && (renderer == "pt" || renderer == "nrc"))
        throw NrError(NR_ERR_INVALID, "envis applies to renderer=ptnee");
    if (a.pol.trav < 0 || a.pol.trav > 1) throw NrError(NR_ERR_INVALID, "trav must be 0 or 1");
    a.wave = c.get_int("wave", 1 << 27);
    a.profile = c.get_int("profile", 0) != 0;
    a.count = c.get_int("count", 0) != 0;
    a.sample0 = c.get_int("sample0", 0);
    a.accumulate = c.get_int("accumulate", 0) != 0;
    a.tile = c.get_int("tile", 2);
    if (a.tile < 0 || a.tile > 2) throw NrError(NR_ERR_INVALID, "tile must be 0, 1 or 2");
    a.live_sync = c.get_int("live_sync", -1);
    a.tail = c.get_int("tail", 2);
    // 0: the largest power of two up to 32 that divides spp
    a.tile_samples = c.get_int("tile_samples", 0);
    if (a.tile_samples < 0 || a.tile_samples > 32 || (a.tile_samples & (a.tile_samples - 1)))
        throw NrError(NR_ERR_INVALID, "tile_samples must be 0 or a power of two up to 32");
    if (a.tile_samples == 0) {
        a.tile_samples = 1;
        while (a.tile_samples < 32 && a.spp % (2 * a.tile_samples) == 0) a.tile_samples *= 2;
    }
    {
        const std::string adj = c.get_str("adj");
        if (!adj.empty() && adj != "mega" && adj != "wave") throw NrError(NR_ERR_INVALID, "adj must be mega or wave");
        a.adj_mega = adj == "mega";
    }
    const bool nrc_mode = a.pol.excl != 0;
    a.nrc = c.get_int("nrc", nrc_mode ? 1 : 0) != 0;
    a.nrc_pre = nrc_mode && c.get_int("nrc_pre", 1) != 0;
    // Training work per wave. Waves of more than 2^22 paths (a 1080p frame
    // of 64 spp is one wave) train on 16384 paths in three Adam steps;
    // smaller waves (frames of one or a few samples per pixel, the real-time
    // regime, where the training's fixed cost weighs on every frame) on 4096
    // in one step. Time to relMSE 1e-3 against plain PT on the 1M-triangle
    // scene, interpolated to the crossing: 1080p at 64 spp per frame, three
    // steps 0.89x, two 0.90x; 960x540 at 1 spp per frame, one step on 16384
    // paths 0.94x, on 8192 0.92x (0.98x once the tail kernel had sped plain
    // PT up), on 4096 0.965x on that same run; two steps 0.97x, three 1.01x.
    {
        const int64_t wave_paths =
            std::min<int64_t>(std::max<int64_t>(0, (int64_t)a.pol.imgw * a.pol.imgh * a.spp), (int64_t)a.wave);
        const bool big_wave = wave_paths > nr::SHADE_SPLIT_MIN;
        a.nrc_train = c.get_int("nrc_train", big_wave ? 16384 : 4096);
        a.nrc_steps = c.get_int("nrc_steps", big_wave ? 3 : 1);
    }
    a.nrc_query = c.get_int("nrc_query", 1);
    a.nrc_first = nrc_mode ? 0 : (c.get_int("nrc_first", 0) != 0 ? 1 : 0);
    a.nrc_mindepth = nrc_mode ? c.get_int("path_lim", 2) : c.get_int("nrc_mindepth", a.nrc_first ? 0 : 1);
    // GGX vertices from this roughness on count as diffuse for ending paths
    // in the cache. Time to relMSE 1e-3 at 960x540, 64 spp per frame: 2.78 s
    // at 0.2, 2.72 at 0.1, 2.69 at 0.05 and at 0 (plain PT 2.89).
    a.nrc_rough = c.get_float("nrc_rough", 0.05f);
    a.nrc_direct = nrc_mode ? 0 : (c.get_int("nrc_direct", 1) != 0 ? 1 : 0);
    a.nrc_train_depth = nrc_mode ? c.get_int("path_lim_train", 4) : c.get_int("nrc_train_depth", 3);
    if (a.nrc_train_depth < 0) throw NrError(NR_ERR_INVALID, "nrc_train_depth must be >= 0");
    if (a.nrc && (a.nrc_train <= 0 || a.nrc_steps <= 0)) throw NrError(NR_ERR_INVALID, "nrc_train and nrc_steps must be positive");
    if (a.sample0 < 0) throw NrError(NR_ERR_INVALID, "sample0 must be >= 0");
    if (a.pol.imgw <= 0 || a.pol.imgh <= 0) throw NrError(NR_ERR_INVALID, "imgw and imgh must be positive");
    if ((int64_t)a.pol.imgw * a.pol.imgh > (1LL << 30)) throw NrError(NR_ERR_INVALID, "image too large");
    if (a.spp <= 0) throw NrError(NR_ERR_INVALID, "spp must be positive");
    if (a.wave <= 0) throw NrError(NR_ERR_INVALID, "wave must be positive");
    if (a.pol.maxdepth < 0 || a.pol.rrdepth < 0) throw NrError(NR_ERR_INVALID, "rrdepth and maxdepth must be >= 0");
    a.cam = cam ? *cam : nr::camera_from_config(c);
    // a camera the film cannot be built from: every ray would be NaN (the
    // reference checks nothing and renders black or garbage)
    {
        const nr_camera& k = a.cam;
        const float v[11] = {k.pos[0], k.pos[1], k.pos[2], k.gaze[0], k.gaze[1], k.gaze[2],
                             k.up[0], k.up[1], k.up[2], k.fov, k.aspect};
        for (float x : v)
            if (!std::isfinite(x)) throw NrError(NR_ERR_INVALID, "camera with a non-finite value");
        if (!(k.fov > 0.0f && k.fov < 180.0f)) throw NrError(NR_ERR_INVALID, "camera fov must lie in (0, 180) degrees");
        if (!(k.aspect > 0.0f)) throw NrError(NR_ERR_INVALID, "camera aspect must be positive");
    }
    return a;
}

// Traces all paths of [0, npix * spp) in waves. Per wave: ray generation,
// then trace/shade/shadow bounces until no path is live, then either the
// film accumulation (film != null) or the per-sample copy (out != null).
// The order of a wave's paths (RenderArgs::tile): tiles of tile_samples
// samples where they divide the frame and spp, else 8x4 pixel tiles, else
// scanline; a pixel list is always in list order.
void wave_layout(const RenderArgs& A, bool has_pix_list, nr::WaveDesc& W) {
    W.tiled = 0;
    W.g_s = A.tile_samples;
    W.g_w = W.g_s >= 16 ? 32 / W.g_s : (W.g_s >= 4 ? 16 / W.g_s : 4);  // 32 / g_s pixels, as square as fits
    W.g_h = 32 / (W.g_s * W.g_w);
    if (has_pix_list) return;
    if (A.tile == 2 && A.pol.imgw % W.g_w == 0 && A.pol.imgh % W.g_h == 0 && A.spp % W.g_s == 0) W.tiled = 2;
    else if (A.tile >= 1 && A.pol.imgw % 8 == 0 && A.pol.imgh % 4 == 0) W.tiled = 1;
}

// Bound on the bounces of a wave without a depth limit (the tail kernel's
// NR_TAIL_MAX_BOUNCES too): paths end by Russian roulette, misses and
// emitters, but prr = 1 in a closed scene would never end.
constexpr int kMaxBounces = 4096;

void run_waves(nr_scene* s, const RenderArgs& A, int npix, const int32_t* dev_pix, int sample0, float4* film,
               float* dev_out, volatile int32_t* cancel, void (*progress)(float, void*), void* user) {
    const uint64_t total = (uint64_t)npix * (uint64_t)A.spp;
    const int cap = (int)std::min<uint64_t>(total, (uint64_t)A.wave);
    ensure_paths(s, cap, A.pol.envis ? 2 : 1);
    cudaStream_t st = s->stream;
    // renderer=nrc without a cache attached renders its estimator alone (the
    // reference with path_lim beyond every path)
    const bool use_nrc = A.nrc && (s->nrc || !A.pol.excl);
    if (use_nrc) {
        if (!s->nrc) throw NrError(NR_ERR_INVALID, "nrc=1 needs a cache attached with nr_scene_attach_nrc");
        const int depth_cap = A.pol.maxdepth > 0 ? A.pol.maxdepth : 16;
        const int tcap = A.nrc_train * depth_cap;
        // the tensor-core forward reads compact query records; the mma.sync
        // one needs them expanded into rows of 80 first
        const bool need_qx = !s->nrc->use_tc();
        if (cap > s->nrc_cap || tcap > s->nrc_tcap || (need_qx && !s->nrc_qx)) {
            auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
            size_t C = (size_t)cap, T = (size_t)tcap;
            s->nrc_cap = s->nrc_tcap = 0;  // set again once the records are in place
            s->nrc_qx = nullptr;
            s->nrc_mem.alloc(al(C * 32) + al(C * 4) + al(C * 16) + al(T * NRC_IN * 2) + al(T * 4) + al(T * 16) * 2 +
                             256 + al(C * 12) + (need_qx ? al(C * NRC_IN * 2) : 0));
            char* p = s->nrc_mem.as<char>();
            auto take = [&](size_t b) { char* r = p; p += al(b); return r; };
            nr::NrcCtx& X = s->nrc_ctx;
            X.q_rec = (uint4*)take(C * 32);
            X.q_slot = (int32_t*)take(C * 4);
            X.q_thr = (float4*)take(C * 16);
            X.t_x = take(T * NRC_IN * 2);
            X.t_slot = (int32_t*)take(T * 4);
            X.t_thr = (float4*)take(T * 16);
            X.t_before = (float4*)take(T * 16);
            X.counters = (uint32_t*)take(16);
            s->nrc_pred = (float*)take(C * 12);
            if (need_qx) s->nrc_qx = (__nv_bfloat16*)take(C * NRC_IN * 2);
            s->nrc_cap = cap;
            s->nrc_tcap = tcap;
        }
        nr::NrcCtx& X = s->nrc_ctx;
        X.tcap = s->nrc_tcap;
        X.train_stride = (uint32_t)std::max<int64_t>(1, (int64_t)cap / A.nrc_train);
        X.query = A.nrc_query;
        X.min_depth = A.nrc_mindepth;
        X.rough = A.nrc_rough;
        X.direct = A.nrc_direct;
        X.train_depth = A.nrc_train_depth;
        X.first = A.nrc_first;
        for (int k = 0; k < 3; ++k) {
            float ext = s->dev.root_hi[k] - s->dev.root_lo[k];
            X.lo[k] = s->dev.root_lo[k];
            X.inv_ext[k] = ext > 0.f ? 1.0f / ext : 0.f;
        }
        nrc_ensure_batch(s->nrc, std::max(s->nrc_tcap, cap));
    }
    const float film_h = nr::film_height(A.cam);
    const nr::DeviceScene D = scene_for(s, A.prune);
    auto t0 = std::chrono::steady_clock::now();
    int nrc_loss_pending = 0;  // training steps behind the loss copied to the cache's pinned buffer
    nr_stats& S = s->stats;
    S = nr_stats{};
    // profile=1: events are recorded in sequence and read once at the end,
    // so the host never waits on them inside the loop.
    size_t nev = 0;
    std::vector<int> ev_kind;  // kernel group that ends at event i (0 trace, 1 shade, 2 shadow, 3 other)
    auto mark = [&](int kind) {
        if (!A.profile) return;
        if (nev == s->ev_pool.size()) {
            cudaEvent_t e;
            NR_CUDA(cudaEventCreate(&e));
            s->ev_pool.push_back(e);
        }
        NR_CUDA(cudaEventRecord(s->ev_pool[nev++], st));
        ev_kind.push_back(kind);
    };
    NR_CUDA(cudaMemsetAsync(s->ps.counters, 0, nr::NUM_COUNTERS * 4, st));
    S.kernel_launches = 0;
    const int live_sync = A.live_sync >= 0 ? A.live_sync : (cap > (1 << 22) ? 5 : 0);
    for (uint64_t base = 0; base < total; base += (uint64_t)cap) {
        if (cancel && *cancel == 0) throw NrError(NR_ERR_CANCELLED, "cancelled");
        nr::WaveDesc W;
        W.base = base;
        W.count = (int)std::min<uint64_t>((uint64_t)cap, total - base);
        W.npix = npix;
        W.sample0 = (uint32_t)sample0;
        W.pix_xy = dev_pix;
        wave_layout(A, dev_pix != nullptr, W);
        mark(-1);
        // queue_in / queue_out swap roles every bounce
        nr::PathState P = s->ps;
        nr::launch_reset_counters(P.counters, st);
        if (use_nrc) NR_CUDA(cudaMemsetAsync(s->nrc_ctx.counters, 0, 8, st));
        nr::launch_raygen(P, W, A.cam, film_h, A.pol, st);
        S.kernel_launches += 2;
        mark(3);
        int live = W.count;
        const bool tail = A.tail > 0 && cap <= nr::SHADE_SPLIT_MIN && !A.profile && !A.count;
        for (int bounce = 0;; ++bounce) {
            if (A.pol.maxdepth > 0 && bounce >= A.pol.maxdepth) break;
            if (bounce >= kMaxBounces) throw NrError(NR_ERR_DEVICE, "paths still alive after 4096 bounces (prr = 1?)");
            if (tail && bounce >= A.tail) {
                nr::launch_tail(P, D, A.pol, cap, use_nrc ? &s->nrc_ctx : nullptr, st);
                S.kernel_launches += 1;
                break;
            }
            cudaEvent_t evs[4];
            if (A.profile) {
                while (s->ev_pool.size() < nev + 4) {
                    cudaEvent_t e;
                    NR_CUDA(cudaEventCreate(&e));
                    s->ev_pool.push_back(e);
                }
                for (int k = 0; k < 4; ++k) evs[k] = s->ev_pool[nev + k];
                ev_kind.push_back(-1); ev_kind.push_back(0); ev_kind.push_back(1); ev_kind.push_back(2);
                nev += 4;
            }
            nr::launch_bounce(P, D, A.pol, cap, live, st, A.profile ? evs : nullptr, A.count,
                              use_nrc ? &s->nrc_ctx : nullptr);
            std::swap(P.queue_in, P.queue_out);
            S.bounces++;
            S.trace_launches++;
            S.kernel_launches += nr::bounce_launches(cap, A.pol.envis != 0, s->dev.cat_mask);
            // With a depth limit the loop runs exactly maxdepth bounces; without
            // one the live count is read back to find the end of the wave.
            if (A.pol.maxdepth == 0 || (live_sync > 0 && bounce + 1 >= live_sync)) {
                NR_CUDA(cudaMemcpyAsync(s->counters_host, s->ps.counters, nr::NUM_COUNTERS * 4, cudaMemcpyDeviceToHost, st));
                NR_CUDA(cudaStreamSynchronize(st));
                live = (int)s->counters_host[nr::CNT_IN];
                if (live == 0) break;
            }
        }
        if (use_nrc) {
            // Cache queries of this batch, then training on its training
            // paths. The query and record counts stay on the device: every
            // launch reads them there, so the host never waits here.
            nr_nrc* c = s->nrc;
            const nr::NrcCtx& X = s->nrc_ctx;
            const nr::NrcRows QR = nr::nrc_rows_counted(&X.counters[0], cap, 0, 1);
            if (c->use_tc()) {
                nr::nrc_launch_forward_tc_records(c->dev.wb_inf, c->dev.pinf, X.q_rec, QR, s->nrc_pred, c->num_sms,
                                                  s->ps.counters + nr::CNT_ERR, st, c->tc_first_wait);
            } else {
                if (!s->nrc_qx) throw NrError(NR_ERR_DEVICE, "cache left the tensor cores during a render");
                nr::nrc_launch_expand(X.q_rec, QR, s->nrc_qx, c->num_sms, st);
                nr::nrc_launch_forward_inf(c->dev, s->nrc_qx, QR, s->nrc_pred, c->num_sms, st);
                S.kernel_launches += 1;
            }
            nr::launch_nrc_apply(s->ps, X, s->nrc_pred, cap, st);
            nr::launch_nrc_targets(s->ps, X, c->y, 1e3f, st);
            NR_CUDA(cudaMemsetAsync(c->loss, 0, 4, st));
            const int steps = A.nrc_steps;
            for (int k = 0; k < steps; ++k) {
                const nr::NrcRows R = nr::nrc_rows_counted(&X.counters[1], s->nrc_tcap, k, steps);
                const __nv_bfloat16* x = (const __nv_bfloat16*)X.t_x;
                nrc_forward_backward(c, x, c->y, R, s->ps.counters + nr::CNT_ERR, st);
                c->step++;
                nr::nrc_launch_adam(c->dev, c->lr, c->b1, c->b2, c->eps, c->step, c->ema, R, st,
                                    s->ps.counters + nr::CNT_ERR);
            }
            NR_CUDA(cudaMemcpyAsync(c->loss_host, c->loss, 4, cudaMemcpyDeviceToHost, st));
            nrc_loss_pending = steps;
            S.kernel_launches += 3 + 4 * steps;
        }
        mark(-1);
        if (film) nr::launch_film(s->ps, W, film, A.pol.imgw, st);
        if (dev_out) nr::launch_collect(s->ps, W, dev_out, A.spp, A.pol.imgw, st);
        S.kernel_launches += 1;
        mark(3);
        S.waves++;
        if (progress) {
            NR_CUDA(cudaStreamSynchronize(st));
            progress((float)(100.0 * (double)(base + W.count) / (double)total), user);
        }
    }
    NR_CUDA(cudaMemcpyAsync(s->counters_host, s->ps.counters, nr::NUM_COUNTERS * 4, cudaMemcpyDeviceToHost, st));
    NR_CUDA(cudaStreamSynchronize(st));
    NR_CUDA(cudaGetLastError());
    if (nrc_loss_pending) s->nrc_last_loss = *s->nrc->loss_host / (float)nrc_loss_pending;
    uint32_t* c = s->counters_host;
    auto u64 = [&](int i) { return (uint64_t)c[i] | ((uint64_t)c[i + 1] << 32); };
    S.paths = total;
    S.rays = u64(nr::CNT_RAYS);
    S.shadow_rays = u64(nr::CNT_SHRAYS);
    S.nodes_visited = u64(nr::CNT_NODES);
    S.tris_tested = u64(nr::CNT_TRIS);
    S.shadow_nodes_visited = u64(nr::CNT_SH_NODES);
    S.shadow_tris_tested = u64(nr::CNT_SH_TRIS);
    for (size_t i = 1; i < nev; ++i) {
        if (ev_kind[i] < 0) continue;
        float ms = 0.0f;
        NR_CUDA(cudaEventElapsedTime(&ms, s->ev_pool[i - 1], s->ev_pool[i]));
        double* dst[4] = {&S.kernel_ms_trace, &S.kernel_ms_shade, &S.kernel_ms_shadow, &S.kernel_ms_other};
        *dst[ev_kind[i]] += ms;
    }
    S.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (c[nr::CNT_ERR] != 0) {
        if (c[nr::CNT_ERR] & nr::NR_ERRBIT_TC_LOST) nr::nrc_tc_disable();
        // the cache skipped the update of a failed step: drop its gradient too
        if (use_nrc) {
            NR_CUDA(cudaMemsetAsync(s->nrc->dev.grad, 0, NRC_NUM_PARAMS * 4, st));
            NR_CUDA(cudaStreamSynchronize(st));
        }
        throw NrError(NR_ERR_DEVICE, "device error bits " + std::to_string(c[nr::CNT_ERR]) + " (" + nr::err_bits_text() +
                                         ")");
    }
}

// Both passes of the adjoint on the wavefront, wave by wave. Pass 1 renders
// the wave (pol.adj: light samples traced wherever their gradient can be
// nonzero), recording every bounce's hits and light-sample visibility, and
// writes each path's radiance to adj_L. Pass 2 generates the same paths
// again, queues the ones with a nonzero gradient weight and replays them
// from the records: k_sort_recorded buckets the recorded hits by material,
// k_shade_adj shades them and adds the gradient terms. Bounces past the
// recorded depth (unbounded paths, or a record that would not fit) are traced
// again (k_trace, k_shadow_adj). Returns the kernel launches.
uint64_t adjoint_waves(nr_scene* s, const RenderArgs& A, int npix, const float* d_dldi, float* d_grad) {
    const uint64_t total = (uint64_t)npix * (uint64_t)A.spp;
    const int cap = (int)std::min<uint64_t>(total, (uint64_t)A.wave);
    ensure_paths(s, cap, 1);
    cudaStream_t st = s->stream;
    // slots, and shadow rays per bounce (one per path at most), of this wave size
    const size_t C = (size_t)std::max(cap, 1), CS = C;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    // recorded bounces: maxdepth, or 16 without one; at most adj_records bytes
    // of records (32 GiB by default; 0: none, every bounce traced again)
    int depth_rec = A.pol.maxdepth > 0 ? A.pol.maxdepth : 16;
    const size_t per_bounce = al(C * 16) + al(C);
    depth_rec = (int)std::min<size_t>((size_t)depth_rec, (size_t)A.adj_rec_bytes / per_bounce);
    s->adj_wave.ensure(al(C * 16) * 4 + al(CS * 16) * 2 + per_bounce * (size_t)depth_rec);
    char* p = s->adj_wave.as<char>();
    auto take = [&](size_t b) { char* r = p; p += al(b); return r; };
    nr::AdjWave J;
    J.L.p = (float4*)take(2 * C * 16);
    J.delta.p = J.L.p + 1;
    J.pk.p = (float4*)take(2 * C * 16);
    J.pa.p = J.pk.p + 1;
    J.sg0.p = (float4*)take(2 * CS * 16);
    J.sg1.p = J.sg0.p + 1;
    float4* rec_hit = (float4*)take(C * 16 * (size_t)depth_rec);
    uint8_t* rec_vis = (uint8_t*)take(C * (size_t)depth_rec);
    const float film_h = nr::film_height(A.cam);
    const nr::DeviceScene D = scene_for(s, A.prune);
    nr::Policy pol1 = A.pol;
    pol1.adj = 1;
    uint64_t launches = 0;
    NR_CUDA(cudaMemsetAsync(s->ps.counters, 0, nr::NUM_COUNTERS * 4, st));
    auto live_after = [&](int bounce, int& live) {
        // as in run_waves: the live count is read back once a wave may end early
        if (A.pol.maxdepth == 0 || bounce >= 4) {
            NR_CUDA(cudaMemcpyAsync(s->counters_host, s->ps.counters, nr::NUM_COUNTERS * 4, cudaMemcpyDeviceToHost, st));
            NR_CUDA(cudaStreamSynchronize(st));
            live = (int)s->counters_host[nr::CNT_IN];
        }
        return live > 0;
    };
    for (uint64_t base = 0; base < total; base += (uint64_t)cap) {
        nr::WaveDesc W;
        W.base = base;
        W.count = (int)std::min<uint64_t>((uint64_t)cap, total - base);
        W.npix = npix;
        W.sample0 = (uint32_t)A.sample0;
        W.pix_xy = nullptr;
        wave_layout(A, false, W);
        // pass 1
        nr::PathState P = s->ps;
        nr::launch_reset_counters(P.counters, st);
        nr::launch_raygen(P, W, A.cam, film_h, pol1, st);
        launches += 2;
        int live = W.count;
        for (int bounce = 0;; ++bounce) {
            if (A.pol.maxdepth > 0 && bounce >= A.pol.maxdepth) break;
            if (bounce >= kMaxBounces) throw NrError(NR_ERR_DEVICE, "paths still alive after 4096 bounces (prr = 1?)");
            const bool rec = bounce < depth_rec;
            P.hit = rec ? rec_hit + (size_t)bounce * C : s->ps.hit;
            P.vis = rec ? rec_vis + (size_t)bounce * C : nullptr;
            nr::launch_bounce(P, D, pol1, cap, live, st, nullptr, false, nullptr);
            std::swap(P.queue_in, P.queue_out);
            launches += nr::bounce_launches(cap, false, s->dev.cat_mask);
            if (!live_after(bounce, live)) break;
        }
        nr::launch_collect(s->ps, W, s->adj_L.as<float>(), A.spp, A.pol.imgw, st);
        // pass 2
        P = s->ps;
        nr::launch_reset_counters(P.counters, st);
        nr::launch_raygen(P, W, A.cam, film_h, A.pol, st);
        nr::launch_adj_init(P, J, W, A.pol.imgw, A.spp, s->adj_L.as<float>(), d_dldi, st);
        launches += 5;
        live = W.count;
        for (int bounce = 0;; ++bounce) {
            if (A.pol.maxdepth > 0 && bounce >= A.pol.maxdepth) break;
            if (bounce >= kMaxBounces) throw NrError(NR_ERR_DEVICE, "paths still alive after 4096 bounces (prr = 1?)");
            const bool rec = bounce < depth_rec;
            const uint8_t* vis = nullptr;
            if (rec) {
                P.hit = rec_hit + (size_t)bounce * C;
                vis = rec_vis + (size_t)bounce * C;
                nr::launch_sort_recorded(P, D, cap, st);
            } else {
                P.hit = s->ps.hit;
                nr::launch_trace(P, D, A.pol, cap, st);
            }
            launches += 2 + nr::launch_adj_bounce_shading(P, D, A.pol, cap, J, vis, d_grad, s->num_sms,
                                                          nr::shadow_grid(), st);
            nr::launch_advance(P.counters, st);
            std::swap(P.queue_in, P.queue_out);
            if (!live_after(bounce, live)) break;
        }
    }
    NR_CUDA(cudaMemcpyAsync(s->counters_host, s->ps.counters, nr::NUM_COUNTERS * 4, cudaMemcpyDeviceToHost, st));
    NR_CUDA(cudaStreamSynchronize(st));
    NR_CUDA(cudaGetLastError());
    if (s->counters_host[nr::CNT_ERR] != 0)
        throw NrError(NR_ERR_DEVICE, "device error bits " + std::to_string(s->counters_host[nr::CNT_ERR]) +
                                         " in the adjoint (" + nr::err_bits_text() + ")");
    return launches;
}

}  // namespace

extern "C" {

int nr_last_error(char* buf, size_t len) {
    if (!buf || len == 0) return NR_ERR_INVALID;
    std::strncpy(buf, g_last_error.c_str(), len - 1);
    buf[len - 1] = 0;
    return NR_OK;
}

int nr_scene_create_opts(const nr_scene_desc* desc, const char* options, nr_scene** out) {
    return guarded([&]() {
        if (!desc || !out) throw NrError(NR_ERR_INVALID, "null argument");
        *out = nullptr;
        auto s = std::make_unique<nr_scene>();
        std::string err = nr::scene_from_desc(*desc, s->host);
        if (!err.empty()) throw NrError(NR_ERR_INVALID, err);
        finish_scene(s.get(), options);
        *out = s.release();
    });
}

int nr_scene_create(const nr_scene_desc* desc, nr_scene** out) { return nr_scene_create_opts(desc, nullptr, out); }

int nr_scene_create_bvh(const nr_scene_desc* desc, const nr_bvh* bvh, const char* options, nr_scene** out) {
    return guarded([&]() {
        if (!desc || !bvh || !out) throw NrError(NR_ERR_INVALID, "null argument");
        *out = nullptr;
        auto s = std::make_unique<nr_scene>();
        std::string err = nr::scene_from_desc(*desc, s->host);
        if (!err.empty()) throw NrError(NR_ERR_INVALID, err);
        nr::Bvh tree;
        err = nr::bvh_from_arrays(s->host, bvh->num_nodes, bvh->box, bvh->kids, bvh->leaf_first, bvh->leaf_count,
                                  bvh->leaf_tris, s->host.num_tris(), NR_STACK_LIMIT - 2, tree);
        if (!err.empty()) throw NrError(NR_ERR_INVALID, "bvh: " + err);
        finish_scene(s.get(), options, &tree);
        *out = s.release();
    });
}

int nr_scene_load_opts(const char* text, const char* options, nr_scene** out) {
    return guarded([&]() {
        if (!text || !out) throw NrError(NR_ERR_INVALID, "null argument");
        *out = nullptr;
        auto s = std::make_unique<nr_scene>();
        std::string err = nr::scene_from_text(text, s->host);
        if (!err.empty()) throw NrError(err.rfind("cannot open", 0) == 0 ? NR_ERR_IO : NR_ERR_INVALID, err);
        finish_scene(s.get(), options);
        *out = s.release();
    });
}

int nr_scene_load(const char* text, nr_scene** out) { return nr_scene_load_opts(text, nullptr, out); }

int nr_scene_build_times(const nr_scene* s, double* bvh_wall_ms, double* bvh_device_ms) {
    return guarded([&]() {
        if (!s) throw NrError(NR_ERR_INVALID, "null scene");
        if (bvh_wall_ms) *bvh_wall_ms = s->bvh_wall_ms;
        if (bvh_device_ms) *bvh_device_ms = s->bvh_device_ms;
    });
}

int nr_scene_destroy(nr_scene* s) {
    return guarded([&]() { delete s; });
}

int nr_scene_set_env(nr_scene* s, int32_t width, int32_t height, const float* rgb, float gain) {
    return guarded([&]() {
        if (!s || width < 0 || height < 0 || (width > 0 && (height == 0 || !rgb))) throw NrError(NR_ERR_INVALID, "bad argument");
        if (!std::isfinite(gain)) throw NrError(NR_ERR_INVALID, "env gain is not finite");
        for (size_t i = 0; i < 3 * (size_t)width * height; ++i)
            if (!std::isfinite(rgb[i])) throw NrError(NR_ERR_INVALID, "environment texel value " + std::to_string(i) + " is not finite");
        std::lock_guard<std::mutex> lk(s->mu);
        NR_CUDA(cudaSetDevice(s->device));
        nr::HostScene& H = s->host;
        // drop a previously attached environment that no material uses
        if (H.env_tex >= 0 && H.env_tex == (int)H.tex_wh.size() / 2 - 1) {
            bool used = false;
            for (const auto& m : H.mats) used = used || m.tex0 == H.env_tex || m.tex1 == H.env_tex;
            if (!used) {
                size_t texels = (size_t)H.tex_wh[2 * H.env_tex] * H.tex_wh[2 * H.env_tex + 1];
                H.tex_data.resize(H.tex_data.size() - 3 * texels);
                H.tex_wh.resize(H.tex_wh.size() - 2);
            }
        }
        H.env_tex = -1;
        if (width > 0) {
            H.tex_wh.push_back(width);
            H.tex_wh.push_back(height);
            H.tex_data.insert(H.tex_data.end(), rgb, rgb + 3 * (size_t)width * height);
            H.env_tex = (int)H.tex_wh.size() / 2 - 1;
        }
        H.env_gain = gain;
        upload_scene(s);
    });
}

int nr_scene_set_materials(nr_scene* s, int32_t n, const nr_material* mats) {
    return guarded([&]() {
        if (!s || !mats || n != (int32_t)s->host.mats.size()) throw NrError(NR_ERR_INVALID, "material count differs from the scene's");
        for (int32_t m = 0; m < n; ++m) {
            const nr_material& a = mats[m];
            const nr_material& b = s->host.mats[m];
            if (a.type != b.type) throw NrError(NR_ERR_INVALID, "material " + std::to_string(m) + ": type changed");
            if ((a.type == NR_MAT_LIGHT) != (b.type == NR_MAT_LIGHT)) throw NrError(NR_ERR_INVALID, "emitters cannot change");
            if (a.tex0 >= (int)s->host.tex_wh.size() / 2 || a.tex1 >= (int)s->host.tex_wh.size() / 2)
                throw NrError(NR_ERR_INVALID, "material " + std::to_string(m) + ": texture index out of range");
            const float f[9] = {a.c0[0], a.c0[1], a.c0[2], a.c1[0], a.c1[1], a.c1[2], a.alpha, a.ior, a.ns};
            for (float x : f)
                if (!std::isfinite(x)) throw NrError(NR_ERR_INVALID, "material " + std::to_string(m) + ": non-finite parameter");
        }
        std::lock_guard<std::mutex> lk(s->mu);
        NR_CUDA(cudaSetDevice(s->device));
        s->host.mats.assign(mats, mats + n);
        // emitter colours live in the emitter table as well: rebuild it with the materials
        upload_scene(s);
    });
}

int nr_adjoint(nr_scene* s, const nr_camera* cam, const char* params, const float* dldi, float* grad, float* image) {
    return guarded([&]() {
        if (!s || !dldi || !grad) throw NrError(NR_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(s->mu);
        with_oom_release(s, [&]() {
            NR_CUDA(cudaSetDevice(s->device));
            RenderArgs A = parse_args(cam, params);
            check_camera(s, A);
            if (A.pol.excl) throw NrError(NR_ERR_INVALID, "the adjoint differentiates renderer=ptnee or pt");
            if (A.pol.envis) throw NrError(NR_ERR_INVALID, "the adjoint does not support envis");
            const int npix = A.pol.imgw * A.pol.imgh;
            const int nm = (int)s->host.mats.size();
            if ((size_t)nm * 7 * 4 > 200 * 1024) throw NrError(NR_ERR_INVALID, "too many materials for the adjoint (limit 7314)");
            cudaStream_t st = s->stream;
            size_t b_img = (size_t)npix * 12, b_grad = (size_t)nm * 7 * 4;
            s->scratch.ensure(2 * b_img + b_grad + 3 * 256);
            char* p = s->scratch.as<char>();
            auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };
            float* d_dldi = (float*)take(b_img);
            float* d_img = (float*)take(b_img);
            float* d_grad = (float*)take(b_grad);
            NR_CUDA(cudaMemcpyAsync(d_dldi, dldi, b_img, cudaMemcpyHostToDevice, st));
            NR_CUDA(cudaMemsetAsync(d_img, 0, b_img, st));
            NR_CUDA(cudaMemsetAsync(d_grad, 0, b_grad, st));
            nr::AdjArgs J;
            J.S = scene_for(s, A.prune);
            J.pol = A.pol;
            J.cam = A.cam;
            J.film_h = nr::film_height(A.cam);
            J.npix = npix;
            J.sample0 = (uint32_t)A.sample0;
            J.spp = A.spp;
            static bool attr = false;
            if (!attr) {
                nr::adjoint_setup();
                attr = true;
            }
            auto t0 = std::chrono::steady_clock::now();
            // every path's radiance (scanline pixel order, so the buffer index is
            // (y * imgw + x) * spp + sample), then the replay of every path
            s->adj_L.ensure((size_t)npix * A.spp * 12);
            uint64_t launches = 0;
            if (A.adj_mega) {
                RenderArgs P1 = A;
                P1.tile = 0;
                P1.tail = 0;  // the wavefront to the end, as the wavefront adjoint's first pass
                run_waves(s, P1, npix, nullptr, A.sample0, nullptr, s->adj_L.as<float>(), nullptr, nullptr, nullptr);
                nr::launch_adjoint(J, d_dldi, d_grad, s->adj_L.as<float>(), s->num_sms, st);
                launches = s->stats.kernel_launches + 1;
            } else {
                launches = adjoint_waves(s, A, npix, d_dldi, d_grad);
            }
            if (image) nr::launch_image_from_L(s->adj_L.as<float>(), npix, A.spp, d_img, st);
            NR_CUDA(cudaGetLastError());
            NR_CUDA(cudaMemcpyAsync(grad, d_grad, b_grad, cudaMemcpyDeviceToHost, st));
            if (image) NR_CUDA(cudaMemcpyAsync(image, d_img, b_img, cudaMemcpyDeviceToHost, st));
            NR_CUDA(cudaStreamSynchronize(st));
            if (image) for (size_t i = 0; i < (size_t)npix * 3; ++i) image[i] /= (float)A.spp;
            s->stats = nr_stats{};
            s->stats.paths = (uint64_t)npix * A.spp;
            s->stats.kernel_launches = launches + (image ? 1 : 0);
            s->stats.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        });
    });
}

int nr_scene_info(const nr_scene* s, int64_t info[6]) {
    return guarded([&]() {
        if (!s || !info) throw NrError(NR_ERR_INVALID, "null argument");
        info[0] = s->host.num_tris();
        info[1] = (int64_t)s->host.mats.size();
        info[2] = (int64_t)s->bvh.nodes.size();
        info[3] = s->bvh.max_depth;
        info[4] = s->dev.num_lights;
        info[5] = (int64_t)device_bytes(s);
    });
}

int nr_scene_export(const nr_scene* s, float* pos, float* uv, float* nrm, int32_t* mat, nr_material* mats) {
    return guarded([&]() {
        if (!s) throw NrError(NR_ERR_INVALID, "null scene");
        const nr::HostScene& H = s->host;
        if (pos) std::copy(H.pos.begin(), H.pos.end(), pos);
        if (uv) std::copy(H.uv.begin(), H.uv.end(), uv);
        if (nrm) std::copy(H.nrm.begin(), H.nrm.end(), nrm);
        if (mat) std::copy(H.mat.begin(), H.mat.end(), mat);
        if (mats) std::copy(H.mats.begin(), H.mats.end(), mats);
    });
}

int nr_bvh_export(const nr_scene* s, float* box, int32_t* kids, int32_t* leaf_first, int32_t* leaf_count,
                  int32_t* leaf_tris, int32_t* num_nodes, int32_t* num_leaf_tris) {
    return guarded([&]() {
        if (!s) throw NrError(NR_ERR_INVALID, "null scene");
        const nr::Bvh& B = s->bvh;
        for (size_t i = 0; i < B.nodes.size(); ++i) {
            const nr::BvhNode& n = B.nodes[i];
            if (box) for (int k = 0; k < 3; ++k) { box[6 * i + k] = n.lo[k]; box[6 * i + 3 + k] = n.hi[k]; }
            if (kids) { kids[2 * i] = n.left; kids[2 * i + 1] = n.right; }
            if (leaf_first) leaf_first[i] = n.first;
            if (leaf_count) leaf_count[i] = n.count;
        }
        if (leaf_tris) std::copy(B.leaf_tris.begin(), B.leaf_tris.end(), leaf_tris);
        if (num_nodes) *num_nodes = (int32_t)B.nodes.size();
        if (num_leaf_tris) *num_leaf_tris = (int32_t)B.leaf_tris.size();
    });
}

int nr_intersect(nr_scene* s, int32_t n, const float* o, const float* d, int32_t* tri, float* t, float* b1, float* b2,
                 int32_t flags) {
    return guarded([&]() {
        if (!s || n < 0 || (n > 0 && (!o || !d || !tri || !t || !b1 || !b2))) throw NrError(NR_ERR_INVALID, "bad argument");
        if (n == 0) return;
        std::lock_guard<std::mutex> lk(s->mu);
        with_oom_release(s, [&]() {
            NR_CUDA(cudaSetDevice(s->device));
            ensure_paths(s, 1);
            cudaStream_t st = s->stream;
            const float *dO = o, *dD = d;
            int32_t* dTri = tri;
            float *dT = t, *dB1 = b1, *dB2 = b2;
            if (!(flags & NR_PTR_DEVICE)) {
                size_t f3 = (size_t)n * 12, f1 = (size_t)n * 4;
                s->scratch.ensure(2 * f3 + 4 * f1 + 6 * 256);  // six 256-byte aligned pieces
                char* p = s->scratch.as<char>();
                auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };
                float* xo = (float*)take(f3);
                float* xd = (float*)take(f3);
                dTri = (int32_t*)take(f1); dT = (float*)take(f1); dB1 = (float*)take(f1); dB2 = (float*)take(f1);
                NR_CUDA(cudaMemcpyAsync(xo, o, f3, cudaMemcpyHostToDevice, st));
                NR_CUDA(cudaMemcpyAsync(xd, d, f3, cudaMemcpyHostToDevice, st));
                dO = xo; dD = xd;
            }
            NR_CUDA(cudaMemsetAsync(s->ps.counters + nr::CNT_ERR, 0, 4, st));
            nr::launch_intersect(scene_for(s, !(flags & NR_INTERSECT_EXHAUSTIVE)), n, dO, dD, dTri, dT, dB1, dB2,
                                 s->ps.counters + nr::CNT_ERR, st);
            NR_CUDA(cudaGetLastError());
            if (!(flags & NR_PTR_DEVICE)) {
                size_t f1 = (size_t)n * 4;
                NR_CUDA(cudaMemcpyAsync(tri, dTri, f1, cudaMemcpyDeviceToHost, st));
                NR_CUDA(cudaMemcpyAsync(t, dT, f1, cudaMemcpyDeviceToHost, st));
                NR_CUDA(cudaMemcpyAsync(b1, dB1, f1, cudaMemcpyDeviceToHost, st));
                NR_CUDA(cudaMemcpyAsync(b2, dB2, f1, cudaMemcpyDeviceToHost, st));
            }
            uint32_t err = 0;
            NR_CUDA(cudaMemcpyAsync(s->counters_host, s->ps.counters + nr::CNT_ERR, 4, cudaMemcpyDeviceToHost, st));
            NR_CUDA(cudaStreamSynchronize(st));
            err = s->counters_host[0];
            if (err) throw NrError(NR_ERR_DEVICE, "traversal error bits " + std::to_string(err) + " (" + nr::err_bits_text() + ")");
        });
    });
}

int nr_intersect_noalloc(nr_scene* s, int32_t n, const float* o, const float* d, int32_t* tri, float* t, float* b1,
                         float* b2) {
    return guarded([&]() {
        if (!s || n < 0 || (n > 0 && (!o || !d || !tri || !t || !b1 || !b2))) throw NrError(NR_ERR_INVALID, "bad argument");
        if (n > NR_NOALLOC_MAX_RAYS)
            throw NrError(NR_ERR_INVALID, "nr_intersect_noalloc takes at most " + std::to_string(NR_NOALLOC_MAX_RAYS) +
                                              " rays per call (got " + std::to_string(n) + "); split the batch");
        std::lock_guard<std::mutex> lk(s->mu);
        NR_CUDA(cudaSetDevice(s->device));
        std::string err = nr::noalloc_intersect(s->dev, s->device, s->stream, n, o, d, tri, t, b1, b2);
        if (!err.empty()) throw NrError(err.rfind("traversal", 0) == 0 ? NR_ERR_DEVICE : NR_ERR_CUDA, err);
    });
}

int nr_camera_from_params(const char* params, nr_camera* cam) {
    return guarded([&]() {
        if (!cam) throw NrError(NR_ERR_INVALID, "null camera");
        *cam = nr::camera_from_config(nr::Config(params));
    });
}

int nr_render(nr_scene* s, const nr_camera* cam, const char* params, float* hdr_rgb, uint8_t* rgb8,
              volatile int32_t* cancel, void (*progress)(float, void*), void* user) {
    return guarded([&]() {
        if (!s) throw NrError(NR_ERR_INVALID, "null scene");
        std::lock_guard<std::mutex> lk(s->mu);
        with_oom_release(s, [&]() {
            NR_CUDA(cudaSetDevice(s->device));
            RenderArgs A = parse_args(cam, params);
            check_camera(s, A);
            const int npix = A.pol.imgw * A.pol.imgh;
            cudaStream_t st = s->stream;
            if (s->film.bytes < (size_t)npix * sizeof(float4)) {
                s->film_pixels = 0;  // a new film holds nothing to accumulate onto
                s->film.ensure((size_t)npix * sizeof(float4));
            }
            bool fresh = false;
            if (!A.accumulate || s->film_pixels != npix) {
                NR_CUDA(cudaMemsetAsync(s->film.p, 0, (size_t)npix * sizeof(float4), st));
                s->film_samples = 0;
                s->film_pixels = npix;
                fresh = true;
            }
            int first = A.sample0;
            if (A.nrc_pre && fresh) {
                // RendererNRC::render (src/renderer/renderernrc.cpp:231-246): one
                // pass in which every path trains, added to the image like the
                // others, while the mean still divides by spp (:268)
                RenderArgs P = A;
                P.spp = 1;
                P.pol.coin = 0;
                P.pol.force_train = 1;
                run_waves(s, P, npix, nullptr, first, s->film.as<float4>(), nullptr, cancel, nullptr, nullptr);
                ++first;
            }
            run_waves(s, A, npix, nullptr, first, s->film.as<float4>(), nullptr, cancel, progress, user);
            s->film_samples += (uint64_t)A.spp;
            if (hdr_rgb || rgb8) {
                if (hdr_rgb) s->out_hdr.ensure((size_t)npix * 12);
                if (rgb8) s->out_rgb8.ensure((size_t)npix * 3);
                nr::launch_finish(s->film.as<float4>(), npix, 1.0f / (float)s->film_samples, hdr_rgb ? s->out_hdr.as<float>() : nullptr,
                                  rgb8 ? s->out_rgb8.as<uint8_t>() : nullptr, st);
                if (hdr_rgb) NR_CUDA(cudaMemcpyAsync(hdr_rgb, s->out_hdr.p, (size_t)npix * 12, cudaMemcpyDeviceToHost, st));
                if (rgb8) NR_CUDA(cudaMemcpyAsync(rgb8, s->out_rgb8.p, (size_t)npix * 3, cudaMemcpyDeviceToHost, st));
                NR_CUDA(cudaStreamSynchronize(st));
            }
            NR_CUDA(cudaGetLastError());
        });
    });
}

int nr_render_samples(nr_scene* s, const nr_camera* cam, const char* params, int32_t npix, const int32_t* pix_xy,
                      int32_t sample0, int32_t spp, float* out) {
    return guarded([&]() {
        if (!s || npix <= 0 || !pix_xy || spp <= 0 || !out || sample0 < 0) throw NrError(NR_ERR_INVALID, "bad argument");
        std::lock_guard<std::mutex> lk(s->mu);
        with_oom_release(s, [&]() {
            NR_CUDA(cudaSetDevice(s->device));
            RenderArgs A = parse_args(cam, params);
            check_camera(s, A);
            A.spp = spp;
            for (int32_t i = 0; i < npix; ++i)
                if (pix_xy[2 * i] < 0 || pix_xy[2 * i] >= A.pol.imgw || pix_xy[2 * i + 1] < 0 || pix_xy[2 * i + 1] >= A.pol.imgh)
                    throw NrError(NR_ERR_INVALID, "pixel outside the image");
            cudaStream_t st = s->stream;
            size_t nout = (size_t)npix * spp * 3;
            s->pix_list.ensure((size_t)npix * 8);
            s->out_hdr.ensure(nout * 4);
            NR_CUDA(cudaMemcpyAsync(s->pix_list.p, pix_xy, (size_t)npix * 8, cudaMemcpyHostToDevice, st));
            run_waves(s, A, npix, s->pix_list.as<int32_t>(), sample0, nullptr, s->out_hdr.as<float>(), nullptr, nullptr, nullptr);
            NR_CUDA(cudaMemcpyAsync(out, s->out_hdr.p, nout * 4, cudaMemcpyDeviceToHost, st));
            NR_CUDA(cudaStreamSynchronize(st));
        });
    });
}

int nr_get_stats(const nr_scene* s, nr_stats* st) {
    return guarded([&]() {
        if (!s || !st) throw NrError(NR_ERR_INVALID, "null argument");
        *st = s->stats;
    });
}

// ------------------------------------------------------------------ neural radiance cache
int nr_nrc_num_params(int64_t* n) {
    return guarded([&]() {
        if (!n) throw NrError(NR_ERR_INVALID, "null argument");
        *n = NRC_NUM_PARAMS;
    });
}

int nr_nrc_create(const char* params, nr_nrc** out) {
    return guarded([&]() {
        if (!out) throw NrError(NR_ERR_INVALID, "null argument");
        *out = nullptr;
        nr::Config c(params);
        auto n = std::make_unique<nr_nrc>();
        NR_CUDA(cudaGetDevice(&n->device));
        NR_CUDA(cudaDeviceGetAttribute(&n->num_sms, cudaDevAttrMultiProcessorCount, n->device));
        NR_CUDA(cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking));
        NR_CUDA(cudaMallocHost(&n->loss_host, 4));
        n->lr = c.get_float("lr", 1e-3f);
        n->b1 = c.get_float("beta1", 0.9f);
        n->b2 = c.get_float("beta2", 0.99f);
        n->eps = c.get_float("eps", 1e-8f);
        n->ema = c.get_float("ema", 0.99f);
        if (n->ema < 0.f || n->ema >= 1.f) throw NrError(NR_ERR_INVALID, "ema must be in [0, 1)");
        n->tc = c.get_int("tc", 1) != 0;
        // polls of the first bounded wait for a group of tensor-core MMAs;
        // 0 makes every such wait time out at once (the timeout path: error
        // bit 8, a second bounded wait for the MMAs in flight, tensor memory
        // freed, NR_ERR_DEVICE)
        {
            const long long fw = c.get_int("tc_first_wait", (int)NR_TC_FIRST_WAIT_LIMIT);
            if (fw < 0 || fw > (long long)NR_TC_FIRST_WAIT_LIMIT)
                throw NrError(NR_ERR_INVALID, "tc_first_wait must be in [0, " + std::to_string(NR_TC_FIRST_WAIT_LIMIT) + "]");
            n->tc_first_wait = (uint32_t)fw;
        }
        nr::nrc_setup();
        nr::nrc_tc_setup();
        n->errbuf.alloc(256);
        n->wt_img.alloc(nr::nrc_wt_image_bytes());
        NR_CUDA(cudaMemsetAsync(n->errbuf.p, 0, 4, n->stream));
        NR_CUDA(cudaMallocHost(&n->err_host, 4));
        const size_t P = NRC_NUM_PARAMS;
        n->pbuf.alloc(6 * P * 4 + 2 * P * 2 + 512);
        float* f = n->pbuf.as<float>();
        n->dev.params = f;
        n->dev.grad = f + P;
        n->dev.m = f + 2 * P;
        n->dev.v = f + 3 * P;
        n->dev.ema = f + 4 * P;
        n->dev.pinf = f + 5 * P;
        n->dev.wb = reinterpret_cast<__nv_bfloat16*>(f + 6 * P);
        n->dev.wb_inf = n->dev.wb + P + 64;
        // Glorot-uniform weights, zero biases; output rows 3..7 stay zero
        std::vector<float> init(P, 0.0f);
        std::mt19937_64 rng((uint64_t)c.get_int("seed", 0));
        auto fill = [&](int off, int rows, int cols, int used_rows) {
            float a = std::sqrt(6.0f / (float)(cols + used_rows));
            std::uniform_real_distribution<float> U(-a, a);
            for (int r = 0; r < used_rows; ++r)
                for (int k = 0; k < cols; ++k) init[off + r * cols + k] = U(rng);
            (void)rows;
        };
        fill(NRC_OFF_W0, NRC_H, NRC_IN, NRC_H);
        fill(NRC_OFF_W1, NRC_H, NRC_H, NRC_H);
        fill(NRC_OFF_W2, NRC_H, NRC_H, NRC_H);
        fill(NRC_OFF_W3, NRC_H, NRC_H, NRC_H);
        fill(NRC_OFF_W4, NRC_OUT_PAD, NRC_H, NRC_OUT);
        NR_CUDA(cudaMemcpyAsync(n->dev.params, init.data(), P * 4, cudaMemcpyHostToDevice, n->stream));
        NR_CUDA(cudaMemcpyAsync(n->dev.pinf, init.data(), P * 4, cudaMemcpyHostToDevice, n->stream));
        NR_CUDA(cudaMemsetAsync(n->dev.grad, 0, 4 * P * 4, n->stream));  // grad, m, v, ema
        nr::nrc_launch_to_bf16(n->dev.params, n->dev.wb, P, n->stream);
        nr::nrc_launch_to_bf16(n->dev.params, n->dev.wb_inf, P, n->stream);
        NR_CUDA(cudaStreamSynchronize(n->stream));
        *out = n.release();
    });
}

int nr_nrc_destroy(nr_nrc* n) {
    return guarded([&]() { delete n; });
}

int nr_nrc_get_params(nr_nrc* n, float* out) {
    return guarded([&]() {
        if (!n || !out) throw NrError(NR_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(n->mu);
        NR_CUDA(cudaSetDevice(n->device));
        NR_CUDA(cudaMemcpyAsync(out, n->dev.params, NRC_NUM_PARAMS * 4, cudaMemcpyDeviceToHost, n->stream));
        NR_CUDA(cudaStreamSynchronize(n->stream));
    });
}

int nr_nrc_set_params(nr_nrc* n, const float* in) {
    return guarded([&]() {
        if (!n || !in) throw NrError(NR_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(n->mu);
        NR_CUDA(cudaSetDevice(n->device));
        NR_CUDA(cudaMemcpyAsync(n->dev.params, in, NRC_NUM_PARAMS * 4, cudaMemcpyHostToDevice, n->stream));
        NR_CUDA(cudaMemcpyAsync(n->dev.pinf, in, NRC_NUM_PARAMS * 4, cudaMemcpyHostToDevice, n->stream));
        NR_CUDA(cudaMemsetAsync(n->dev.grad, 0, 4 * (size_t)NRC_NUM_PARAMS * 4, n->stream));
        nr::nrc_launch_to_bf16(n->dev.params, n->dev.wb, NRC_NUM_PARAMS, n->stream);
        nr::nrc_launch_to_bf16(n->dev.params, n->dev.wb_inf, NRC_NUM_PARAMS, n->stream);
        n->step = 0;
        NR_CUDA(cudaStreamSynchronize(n->stream));
    });
}

// Optimizer state of a cache, for checkpoints: which = NR_NRC_STATE_*.
int nr_nrc_get_state(nr_nrc* n, int32_t which, float* out) {
    return guarded([&]() {
        if (!n || !out) throw NrError(NR_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(n->mu);
        NR_CUDA(cudaSetDevice(n->device));
        const size_t P = NRC_NUM_PARAMS;
        if (which == NR_NRC_STATE_STEP) {
            out[0] = (float)n->step;
            return;
        }
        float* src = nullptr;
        const __nv_bfloat16* bsrc = nullptr;
        switch (which) {
            case NR_NRC_STATE_PARAMS: src = n->dev.params; break;
            case NR_NRC_STATE_GRAD: src = n->dev.grad; break;
            case NR_NRC_STATE_M: src = n->dev.m; break;
            case NR_NRC_STATE_V: src = n->dev.v; break;
            case NR_NRC_STATE_EMA: src = n->dev.ema; break;
            case NR_NRC_STATE_INFER: src = n->dev.pinf; break;
            case NR_NRC_STATE_PARAMS_BF16: bsrc = n->dev.wb; break;
            case NR_NRC_STATE_INFER_BF16: bsrc = n->dev.wb_inf; break;
            default: throw NrError(NR_ERR_INVALID, "unknown cache state " + std::to_string(which));
        }
        if (src) {
            NR_CUDA(cudaMemcpyAsync(out, src, P * 4, cudaMemcpyDeviceToHost, n->stream));
            NR_CUDA(cudaStreamSynchronize(n->stream));
        } else {
            std::vector<__nv_bfloat16> h(P);
            NR_CUDA(cudaMemcpyAsync(h.data(), bsrc, P * 2, cudaMemcpyDeviceToHost, n->stream));
            NR_CUDA(cudaStreamSynchronize(n->stream));
            for (size_t i = 0; i < P; ++i) {
                uint16_t b;
                std::memcpy(&b, &h[i], 2);
                const uint32_t u = (uint32_t)b << 16;
                std::memcpy(&out[i], &u, 4);
            }
        }
    });
}

int nr_nrc_set_state(nr_nrc* n, int32_t which, const float* in) {
    return guarded([&]() {
        if (!n || !in) throw NrError(NR_ERR_INVALID, "null argument");
        std::lock_guard<std::mutex> lk(n->mu);
        NR_CUDA(cudaSetDevice(n->device));
        const size_t P = NRC_NUM_PARAMS;
        if (which == NR_NRC_STATE_STEP) {
            if (!(in[0] >= 0.f) || in[0] > 1e9f || in[0] != std::floor(in[0]))
                throw NrError(NR_ERR_INVALID, "the step count must be a non-negative integer");
            n->step = (int)in[0];
            return;
        }
        float* dst = nullptr;
        switch (which) {
            case NR_NRC_STATE_PARAMS: dst = n->dev.params; break;
            case NR_NRC_STATE_GRAD: dst = n->dev.grad; break;
            case NR_NRC_STATE_M: dst = n->dev.m; break;
            case NR_NRC_STATE_V: dst = n->dev.v; break;
            case NR_NRC_STATE_EMA: dst = n->dev.ema; break;
            case NR_NRC_STATE_INFER: dst = n->dev.pinf; break;
            default: throw NrError(NR_ERR_INVALID, "cache state " + std::to_string(which) + " cannot be set");
        }
        NR_CUDA(cudaMemcpyAsync(dst, in, P * 4, cudaMemcpyHostToDevice, n->stream));
        // the BF16 copies the kernels read follow their FP32 sources
        if (which == NR_NRC_STATE_PARAMS) nr::nrc_launch_to_bf16(n->dev.params, n->dev.wb, P, n->stream);
        if (which == NR_NRC_STATE_INFER) nr::nrc_launch_to_bf16(n->dev.pinf, n->dev.wb_inf, P, n->stream);
        NR_CUDA(cudaStreamSynchronize(n->stream));
        NR_CUDA(cudaGetLastError());
    });
}

namespace {
// Reads the cache's error word (already copied to err_host): clears it on
// the device for the next call and turns a set bit into NR_ERR_DEVICE; bit
// 32 also stops the process's use of the tensor-core kernels.
void nrc_check_err(nr_nrc* c, const char* what) {
    const uint32_t e = *c->err_host;
    if (!e) return;
    if (e & nr::NR_ERRBIT_TC_LOST) nr::nrc_tc_disable();
    // the failed step's update was skipped; its partial gradient goes too
    NR_CUDA(cudaMemsetAsync(c->dev.grad, 0, NRC_NUM_PARAMS * 4, c->stream));
    NR_CUDA(cudaMemsetAsync(c->errbuf.p, 0, 4, c->stream));
    NR_CUDA(cudaStreamSynchronize(c->stream));
    throw NrError(NR_ERR_DEVICE, std::string("tensor-core ") + what + " wait timed out (error bits " + std::to_string(e) +
                                     ": " + nr::err_bits_text() + ")");
}

// Uploads n rows of FP32 inputs and converts them to BF16 in the batch scratch.
void nrc_upload_x(nr_nrc* c, int n, const float* x) {
    nrc_ensure_batch(c, n);
    NR_CUDA(cudaMemcpyAsync(c->xf, x, (size_t)n * NRC_IN * 4, cudaMemcpyHostToDevice, c->stream));
    nr::nrc_launch_to_bf16(c->xf, c->x, (size_t)n * NRC_IN, c->stream);
}
}  // namespace

int nr_nrc_infer(nr_nrc* c, int32_t n, const float* x, float* out) {
    return guarded([&]() {
        if (!c || n < 0 || (n > 0 && (!x || !out))) throw NrError(NR_ERR_INVALID, "bad argument");
        if (n == 0) return;
        std::lock_guard<std::mutex> lk(c->mu);
        NR_CUDA(cudaSetDevice(c->device));
        nrc_upload_x(c, n, x);
        if (c->use_tc())
            nr::nrc_launch_forward_tc(c->dev.wb, c->dev.params, c->x, nr::nrc_rows(n), c->out, c->num_sms,
                                      c->errbuf.as<uint32_t>(), c->stream, nullptr, c->tc_first_wait);
        else
            nr::nrc_launch_forward(c->dev, c->x, nr::nrc_rows(n), c->out, nullptr, c->num_sms, c->stream);
        NR_CUDA(cudaMemcpyAsync(out, c->out, (size_t)n * 12, cudaMemcpyDeviceToHost, c->stream));
        NR_CUDA(cudaMemcpyAsync(c->err_host, c->errbuf.p, 4, cudaMemcpyDeviceToHost, c->stream));
        NR_CUDA(cudaStreamSynchronize(c->stream));
        NR_CUDA(cudaGetLastError());
        nrc_check_err(c, "inference");
    });
}

static int nrc_grad_impl(nr_nrc* c, int32_t n, const float* x, const float* y, float* grad, float* loss, bool update) {
    return guarded([&]() {
        if (!c || n <= 0 || !x || !y) throw NrError(NR_ERR_INVALID, "bad argument");
        std::lock_guard<std::mutex> lk(c->mu);
        NR_CUDA(cudaSetDevice(c->device));
        nrc_upload_x(c, n, x);
        NR_CUDA(cudaMemcpyAsync(c->y, y, (size_t)n * 12, cudaMemcpyHostToDevice, c->stream));
        nrc_train_device(c, c->x, c->y, n, false, c->stream);
        if (grad) NR_CUDA(cudaMemcpyAsync(grad, c->dev.grad, NRC_NUM_PARAMS * 4, cudaMemcpyDeviceToHost, c->stream));
        if (update) {
            c->step++;
            nr::nrc_launch_adam(c->dev, c->lr, c->b1, c->b2, c->eps, c->step, c->ema, nr::nrc_rows(n), c->stream,
                                c->errbuf.as<uint32_t>());
        } else {
            NR_CUDA(cudaMemsetAsync(c->dev.grad, 0, NRC_NUM_PARAMS * 4, c->stream));
        }
        NR_CUDA(cudaMemcpyAsync(c->loss_host, c->loss, 4, cudaMemcpyDeviceToHost, c->stream));
        NR_CUDA(cudaMemcpyAsync(c->err_host, c->errbuf.p, 4, cudaMemcpyDeviceToHost, c->stream));
        NR_CUDA(cudaStreamSynchronize(c->stream));
        NR_CUDA(cudaGetLastError());
        nrc_check_err(c, "training");
        if (loss) *loss = *c->loss_host;
    });
}

int nr_nrc_gradient(nr_nrc* c, int32_t n, const float* x, const float* y, float* grad, float* loss) {
    return nrc_grad_impl(c, n, x, y, grad, loss, false);
}

int nr_nrc_train_step(nr_nrc* c, int32_t n, const float* x, const float* y, float* loss) {
    return nrc_grad_impl(c, n, x, y, nullptr, loss, true);
}

int nr_scene_attach_nrc(nr_scene* s, nr_nrc* c) {
    return guarded([&]() {
        if (!s) throw NrError(NR_ERR_INVALID, "null scene");
        if (c && c->device != s->device) throw NrError(NR_ERR_INVALID, "cache and scene live on different devices");
        std::lock_guard<std::mutex> lk(s->mu);
        s->nrc = c;
    });
}

int nr_scene_stream(const nr_scene* s, void** stream) {
    return guarded([&]() {
        if (!s || !stream) throw NrError(NR_ERR_INVALID, "null argument");
        *stream = (void*)s->stream;
    });
}

int nr_material_probe(nr_scene* s, int32_t mat, int32_t n, const float* wo, const float* nrm, const float* wi,
                      const float* uv, const float* u, float* f, float* pdf, float* wi_s) {
    return guarded([&]() {
        if (!s || n < 0 || mat < 0 || mat >= (int)s->host.mats.size()) throw NrError(NR_ERR_INVALID, "bad argument");
        if (n == 0) return;
        std::lock_guard<std::mutex> lk(s->mu);
        NR_CUDA(cudaSetDevice(s->device));
        cudaStream_t st = s->stream;
        size_t f3 = (size_t)n * 12, f1 = (size_t)n * 4, f4 = (size_t)n * 16;
        s->scratch.ensure(4 * f3 + f4 + 2 * f3 + f1 + 8 * 256);  // eight 256-byte aligned pieces
        char* p = s->scratch.as<char>();
        auto take = [&](size_t b) { char* r = p; p += (b + 255) & ~size_t(255); return r; };
        float *dwo = (float*)take(f3), *dn = (float*)take(f3), *dwi = (float*)take(f3), *duv = (float*)take(f3);
        float *du = (float*)take(f4), *df = (float*)take(f3), *dws = (float*)take(f3), *dp = (float*)take(f1);
        NR_CUDA(cudaMemcpyAsync(dwo, wo, f3, cudaMemcpyHostToDevice, st));
        NR_CUDA(cudaMemcpyAsync(dn, nrm, f3, cudaMemcpyHostToDevice, st));
        NR_CUDA(cudaMemcpyAsync(dwi, wi, f3, cudaMemcpyHostToDevice, st));
        NR_CUDA(cudaMemcpyAsync(duv, uv, f3, cudaMemcpyHostToDevice, st));
        NR_CUDA(cudaMemcpyAsync(du, u, f4, cudaMemcpyHostToDevice, st));
        nr::launch_material_probe(s->dev, mat, n, dwo, dn, dwi, duv, du, df, dp, dws, st);
        NR_CUDA(cudaGetLastError());
        NR_CUDA(cudaMemcpyAsync(f, df, f3, cudaMemcpyDeviceToHost, st));
        NR_CUDA(cudaMemcpyAsync(pdf, dp, f1, cudaMemcpyDeviceToHost, st));
        NR_CUDA(cudaMemcpyAsync(wi_s, dws, f3, cudaMemcpyDeviceToHost, st));
        NR_CUDA(cudaStreamSynchronize(st));
    });
}

}  // extern "C"
