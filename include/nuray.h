/* nuray.h — C ABI of libnuray_gpu.so, the GB300 (sm_103a) implementation of
 * nuRay's `ptnee` renderer (RendererPTLS, src/renderer/rendererptls.cpp).
 *
 * Every entry point returns an int status: NR_OK (0) or a negative NR_ERR_*
 * code. No C++ exception crosses this boundary. The message of the last
 * error on the calling thread is available from nr_last_error().
 *
 * Threading: calls on one scene are serialised by the library (one CUDA
 * stream and one lock per scene); distinct scenes may be used from
 * different threads. All pointers are host pointers unless a flag says
 * otherwise.
 *
 * Reference interfaces replaced (file:line in the reference project):
 *   nr_scene_load / nr_scene_create  Loader::fromSceneDescription (src/scene/loader.cpp:26-108)
 *                                    + Renderer::prepare (src/renderer/renderer.cpp:30-39)
 *   nr_scene_destroy                 Loader::~Loader / BVH::~BVH (src/scene/loader.cpp:10-16,
 *                                    src/hierarchy/bvh.cpp:76-79)
 *   nr_scene_set_env                 Renderer::setEnvmap + Envmap(texture, gain)
 *                                    (src/renderer/renderer.cpp:41-44, src/scene/envmap.cpp:5-24)
 *   nr_intersect                     Renderer::intersect -> BVH::intersection
 *                                    (src/renderer/renderer.cpp:10-28, src/hierarchy/bvh.cpp:129-137)
 *   nr_camera_from_params            Camera(fov, asp, pos, yaw, pitch, roll) as built by Cmd::main
 *                                    (src/cmd/cmd.cpp:99-101, src/scene/camera.cpp:16-22,88-105)
 *   nr_render                        RendererPTLS::render (src/renderer/rendererptls.cpp:96-236)
 *   nr_render_samples                the per-sample loop body of RendererPTLS::render
 *                                    (src/renderer/rendererptls.cpp:170-174) for listed pixels
 *   nr_material_probe                Material::bxdf/pdf/sampleBxdf (src/material/material.h:7-24)
 *   nr_nrc_*                         NNNodeMultiLayerPerceptron::eval / train (src/nn/nnnode.cpp:175-201)
 *   nr_scene_attach_nrc              RendererNRC's cache query (src/renderer/renderernrc.cpp:130-133)
 *   nr_adjoint, nr_scene_set_materials  no reference counterpart (differentiation)
 *   nr_get_stats / nr_scene_stream   no reference counterpart (the reference reports only a
 *                                    wall-clock "secs used", src/renderer/rendererptls.cpp:232-233)
 */
#ifndef NURAY_H
#define NURAY_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NR_OK 0
#define NR_ERR_INVALID (-1)    /* bad argument, malformed scene or parameter */
#define NR_ERR_CUDA (-2)       /* a CUDA call failed */
#define NR_ERR_OOM (-3)        /* device or host allocation failed */
#define NR_ERR_CANCELLED (-4)  /* *cancel became 0 during nr_render */
#define NR_ERR_IO (-5)         /* a scene file could not be read */
#define NR_ERR_DEVICE (-6)     /* a kernel reported an internal error (stack overflow, bad index),
                                  or paths still alive after 4096 bounces (prr=1, no maxdepth) */

/* Material types: the reference's Material subclasses (src/material/). */
#define NR_MAT_LAMBERT 0     /* MatLambert    (src/material/matlambert.cpp) */
#define NR_MAT_GGXR 1        /* MatGGXRefl    (src/material/matggxrefl.cpp), -m=ggxr */
#define NR_MAT_GGX 2         /* MatGGX        (src/material/matggx.cpp), -m=ggx dielectric */
#define NR_MAT_GLASS 3       /* MatGlass      (src/material/matglass.cpp), -m=glass */
#define NR_MAT_BLINNPHONG 4  /* MatBlinnPhong (src/material/matblinnphong.cpp), MTL Ks>0 */
#define NR_MAT_LIGHT 5       /* MatLight      (src/material/matlight.cpp), MTL Ke>0 or -m=light */

/* One material, 64 bytes.
 *   c0: Kd (Lambert, GGXR, GGX, BlinnPhong), F0 (Glass) or Ke (Light)
 *   c1: Ks (BlinnPhong)
 *   alpha: GGX roughness; ior: GGX / Glass index; ns: BlinnPhong exponent
 *   tex0: texture index replacing c0 (map_Kd, glass map_F0), -1 for none
 *   tex1: texture index replacing c1 (map_Ks), -1 for none */
typedef struct nr_material {
    int32_t type;
    int32_t tex0;
    int32_t tex1;
    int32_t reserved0;
    float c0[3];
    float c1[3];
    float alpha;
    float ior;
    float ns;
    float reserved1[3];
} nr_material;

/* A flattened scene, in the reference Loader's triangle order.
 *   pos: 9 floats per triangle (p0, p1, p2)
 *   uv:  6 floats per triangle (t0.xy, t1.xy, t2.xy), may be NULL (zeros)
 *   nrm: 9 floats per triangle (n0, n1, n2), may be NULL; as in the
 *        reference's Triangle constructor a face normal replaces them
 *        when |n0|^2 < 1e-4 (src/scene/triangle.cpp:12-25)
 *   mat: material index per triangle
 *   textures: tex_wh holds (width, height) per texture, tex_data the
 *        concatenated linear RGB floats, row-major, row 0 at v = 1
 *   env_tex: texture index of the environment map or -1; env_gain its gain
 * The library copies everything; the caller's buffers may be freed after
 * nr_scene_create returns. */
typedef struct nr_scene_desc {
    int32_t num_tris;
    const float* pos;
    const float* uv;
    const float* nrm;
    const int32_t* mat;
    int32_t num_mats;
    const nr_material* mats;
    int32_t num_tex;
    const int32_t* tex_wh;
    const float* tex_data;
    int32_t env_tex;
    float env_gain;
} nr_scene_desc;

/* Pinhole camera (struct Camera, src/scene/camera.h:6-31). fov is the
 * vertical field of view in degrees, aspect = film width / height. */
typedef struct nr_camera {
    float pos[3];
    float gaze[3];
    float up[3];
    float fov;
    float aspect;
} nr_camera;

typedef struct nr_scene nr_scene;

/* Render statistics of the last nr_render / nr_render_samples on a scene.
 * Kernel times are filled when the parameters contain profile=1 (CUDA events
 * around every kernel of the wavefront), traversal counts when they contain
 * count=1 (instrumented traversal kernels, slower). */
typedef struct nr_stats {
    uint64_t paths;            /* camera samples traced */
    uint64_t rays;             /* extension rays (camera + continuation) */
    uint64_t shadow_rays;      /* NEE shadow rays */
    uint64_t waves;            /* wavefront batches */
    uint64_t bounces;          /* trace/shade iterations over all waves */
    uint64_t kernel_launches;  /* kernels launched by the call */
    uint64_t trace_launches;   /* of which closest-hit traversal */
    uint64_t nodes_visited;    /* BVH nodes visited by extension rays (count=1) */
    uint64_t tris_tested;      /* triangles tested by extension rays (count=1) */
    uint64_t shadow_nodes_visited;
    uint64_t shadow_tris_tested;
    double kernel_ms_trace;    /* summed kernel time, closest-hit traversal + material sort */
    double kernel_ms_shadow;   /* summed kernel time, shadow traversal */
    double kernel_ms_shade;    /* summed kernel time, shading + NEE */
    double kernel_ms_other;    /* ray generation, film, counters */
    double wall_ms;            /* host wall time of the call */
} nr_stats;

/* Copies the message of the last failed call on this thread into buf. */
int nr_last_error(char* buf, size_t len);

/* Builds a scene from flat arrays: copies it, builds the reference SAH BVH
 * on the host, uploads triangles, BVH, materials, textures and the emitter
 * table to the current CUDA device. */
int nr_scene_create(const nr_scene_desc* desc, nr_scene** out);

/* Builds a scene from the reference's scene-description text: one OBJ path
 * per line with optional -p x y z, -s k, and forced materials
 * -m=light r g b | -m=ggx r g b alpha ior | -m=ggxr r g b alpha |
 * -m=glass r g b ior (src/scene/loader.cpp:26-108). MTL texture maps
 * (map_Kd, map_Ks) may be PNG, JPEG (baseline or progressive), PFM or
 * binary PPM; 8-bit images are linearised as Texture::load does
 * (src/scene/texture.cpp:13-19). */
int nr_scene_load(const char* scene_desc, nr_scene** out);

int nr_scene_destroy(nr_scene* scene);

/* Renderer::setEnvmap (src/renderer/renderer.cpp:41-44) together with the
 * Envmap the CLI builds from envmap= / envmap_gain= (src/cmd/cmd.cpp:59-65):
 * sets (or replaces) the environment looked up on a miss. rgb holds
 * width*height linear RGB floats, row 0 at v = 1. width = 0 removes it. */
int nr_scene_set_env(nr_scene* scene, int32_t width, int32_t height, const float* rgb, float gain);

/* info[0..5] = triangles, materials, BVH nodes, BVH depth, emitters, device bytes. */
int nr_scene_info(const nr_scene* scene, int64_t info[6]);

/* nr_scene_create / nr_scene_load with options ("key=value ..."; NULL or
 * "" for the defaults). bvh=host (default) builds the reference's SAH tree
 * (BVH::_build, src/hierarchy/bvh.cpp:60-70) on the host threads; bvh=gpu
 * builds it on the device, level by level: the same cost and split rule,
 * the same tree wherever no two triangles share a pMax coordinate, and a
 * stable (loader-index) order among equal keys where the reference's
 * std::sort order is unspecified. max_device_bytes=N caps the device memory
 * the scene's own buffers may hold (scene data, path state, films, staging;
 * not an attached cache): an allocation past it fails with NR_ERR_OOM, as a
 * failed cudaMalloc does, and the scene stays usable for calls that fit.
 * No reference counterpart for either option. Scenes whose positions,
 * normals, texture coordinates, material parameters, texels or environment
 * gain are not finite are refused with NR_ERR_INVALID. */
int nr_scene_create_opts(const nr_scene_desc* desc, const char* options, nr_scene** out);
int nr_scene_load_opts(const char* text, const char* options, nr_scene** out);

/* Wall-clock time of the scene's BVH build and, for bvh=gpu, the device
 * time of its kernels (0 for the host build). No reference counterpart. */
int nr_scene_build_times(const nr_scene* scene, double* bvh_wall_ms, double* bvh_device_ms);

/* Reads back the flattened scene in loader order (pos 9, uv 6, nrm 9 floats
 * and a material index per triangle; materials) for checks. Any pointer may
 * be NULL. */
int nr_scene_export(const nr_scene* scene, float* pos, float* uv, float* nrm, int32_t* mat, nr_material* mats);

/* A tree for nr_scene_create_bvh, in the layout nr_bvh_export writes:
 * num_nodes nodes, node 0 the root, every child after its parent (depth-first
 * order, as exported, is one such order); box[6] per node (min, max);
 * kids[2] per node, -1, -1 for a leaf; a leaf's leaf_first / leaf_count
 * (at most 7) into leaf_tris, the num_tris triangle indices (loader order)
 * in leaf order. Closest-hit ties between leaves go to the larger
 * leaf_first, which is the reference's "later leaf in depth-first order"
 * when the leaves are laid out depth-first, as the reference's are. */
typedef struct nr_bvh {
    int32_t num_nodes;
    const float* box;
    const int32_t* kids;
    const int32_t* leaf_first;
    const int32_t* leaf_count;
    const int32_t* leaf_tris;
} nr_bvh;

/* nr_scene_create_opts with the caller's tree instead of a build (the
 * reference's BVH built by BVH::build, src/hierarchy/bvh.cpp:60-70, handed
 * over, or a tree exported earlier). Refused with NR_ERR_INVALID unless
 * leaf_tris is a permutation of the triangles, the leaves partition it,
 * every node but the root has exactly one parent, which precedes it, every
 * box lies inside its parent's and every triangle inside its leaf's, and
 * the tree is at most 94 levels deep. */
int nr_scene_create_bvh(const nr_scene_desc* desc, const nr_bvh* bvh, const char* options, nr_scene** out);

/* BVH in depth-first order (left child first): box[6] per node (min, max),
 * kids[2] (-1, -1 for a leaf), leaf_first/leaf_count into leaf_tris
 * (triangle indices in loader order). Returns NR_OK and writes the node count
 * and leaf-triangle count into *num_nodes / *num_leaf_tris; buffers may be
 * NULL to query sizes. */
int nr_bvh_export(const nr_scene* scene, float* box, int32_t* kids, int32_t* leaf_first, int32_t* leaf_count,
                  int32_t* leaf_tris, int32_t* num_nodes, int32_t* num_leaf_tris);

#define NR_PTR_DEVICE 1          /* flag: the ray and hit arrays are device pointers */
#define NR_INTERSECT_EXHAUSTIVE 2 /* flag: visit every node whose box the ray enters, as the reference's
                                     BVH::_traversal does (src/hierarchy/bvh.cpp:99-127), instead of
                                     skipping subtrees entered beyond 1.001 x the best hit so far */

/* Closest hit for n rays (o, d: 3 floats each). tri receives the triangle
 * index in loader order or -1 for a miss (t = 1e18, b1 = b2 = 0), as
 * BVH::intersection does. The default walk skips subtrees that cannot hold
 * a nearer hit; it returns the reference's hit except where the ray crosses
 * a triangle at a grazing angle (|s1.e1| below about 1e-3, where the
 * reference's determinant bias 1e-6 lets the triangle report a t short of
 * its own box), which NR_INTERSECT_EXHAUSTIVE covers too. */
int nr_intersect(nr_scene* scene, int32_t n, const float* o, const float* d, int32_t* tri, float* t, float* b1,
                 float* b2, int32_t flags);

/* Camera from the reference parameter keys campos, cameuler, camfov, camasp
 * (defaults 0,0,0 / 0,0,0 / 90 / 1). */
int nr_camera_from_params(const char* params, nr_camera* cam);

/* nr_intersect for host arrays without any device allocation by the library
 * (no counterpart in the reference, which has no device memory at all).
 * For callers that cannot let a library allocate device memory while they
 * run: hosts that hand a plugin a fixed memory budget at start-up, or
 * real-time loops that cannot take cudaMalloc's implicit device
 * synchronisation mid-frame. Rays and results go through one static device
 * array of NR_NOALLOC_MAX_RAYS (65,536) rays, 2.6 MB. Under CUDA's lazy
 * module loading that array is reserved on a device when the first scene is
 * created there (nr_scene_create / nr_scene_load load its module and look up
 * its device address, with that device current), and it stays reserved until
 * the process exits; the calls themselves then load and allocate nothing.
 * Larger n is rejected with NR_ERR_INVALID (split the batch). All calls share
 * the array, which keeps the last call's contents; calls whose work overlapped
 * on the GPU would race on it, so the library serialises them under one
 * process-wide lock. Each call blocks until the results are on the host (it
 * synchronises the scene's stream and copies into pageable memory), so it must
 * not be called while the scene's stream, or any stream in a process-wide
 * capture, is being captured into a CUDA graph. */
#define NR_NOALLOC_MAX_RAYS 65536
int nr_intersect_noalloc(nr_scene* scene, int32_t n, const float* o, const float* d, int32_t* tri, float* t, float* b1,
                         float* b2);

/* Renders the image. params uses the reference grammar ("key=value ..."):
 * renderer (ptnee, the default; pt: RendererPT, src/renderer/rendererpt.cpp:13-59,
 * the same estimator without light sampling; nrc: RendererNRC,
 * src/renderer/renderernrc.cpp:13-281, light samples without MIS, a
 * training coin per sample, one all-training first pass added to the image
 * with the mean still divided by spp, and the attached cache asked from
 * vertex path_lim (default 2) on, path_lim_train (default 4) on training
 * paths; without an attached cache its estimator alone), imgw imgh spp prr mis
 * (reference keys and defaults) plus seed (Philox seed,
 * default 0), rrdepth (first vertex where Russian roulette applies, default 0
 * as in the reference), maxdepth (0 = unbounded as in the reference),
 * wave (paths per wavefront batch, default 2^27: a 1080p frame of 64 spp in
 * one batch, 24 GB of path state), trav (0: traversal with
 * the reference's exact arithmetic only, 1: fast tests with exact fallback,
 * default; both return the same hits), accumulate=1 (add to the film of
 * the previous call of the same size instead of clearing it; the outputs are
 * the mean over all samples added so far), sample0 (index of the first
 * sample, default 0: renders of disjoint sample ranges are independent and
 * their films sum), tile (the order of a wave's paths; the image is the same
 * for every choice. 2, the default: each warp's 32 paths are tile_samples
 * consecutive samples of a tile of 32 / tile_samples pixels, tile_samples
 * by default the largest power of two up to 32 dividing spp, when the tile
 * divides the image; else 1: 8x4 pixel tiles of one sample when imgw % 8 ==
 * 0 and imgh % 4 == 0; else or with 0: scanline order), live_sync (with
 * maxdepth: the bounce after which the live path count is read back each
 * bounce; -1, the default, 5 for waves of more than 2^22 paths and never
 * for smaller ones), tail (waves of at most 2^22 paths: after this many
 * wavefront bounces one launch takes every live path to its end, tracing
 * its light samples inline; default 2, 0 never; the image is the same),
 * prune (1, the default: a traversal skips subtrees entered beyond 1.001 x
 * its best hit so far or its shadow ray's length; 0: every node whose box a
 * ray enters is visited, as the reference's exhaustive BVH::_traversal, for
 * the reference's hits on grazing rays as well; see nr_intersect),
 * envis=1 (ptnee only, no reference counterpart: one environment light
 * sample per light-sampling vertex besides the area-light sample, weighted
 * against BSDF-sampled misses by the balance heuristic; the same expected
 * image where a material's pdf() is its sampling density, as for Lambert, but
 * not on GGX-reflect, whose pdf() omits the half-vector Jacobian),
 * profile=1 and count=1 (see nr_stats). cam may be NULL to take the camera from
 * params; a camera with a non-finite value, a fov outside (0, 180) degrees
 * or a non-positive aspect is refused (NR_ERR_INVALID). hdr_rgb (W*H*3 floats, the per-pixel mean of max(0, L)) and rgb8
 * (W*H*3 bytes: mean^(1/2.2)*255 clamped and truncated, as
 * src/renderer/rendererptls.cpp:175-180) may each be NULL. cancel, if not
 * NULL, is polled between waves; 0 cancels (the reference's con_flag).
 * progress, if not NULL, is called with the percentage done. */
int nr_render(nr_scene* scene, const nr_camera* cam, const char* params, float* hdr_rgb, uint8_t* rgb8,
              volatile int32_t* cancel, void (*progress)(float pct, void* user), void* user);

/* Per-sample radiance (after the per-sample max(0, .)) for npix listed pixels
 * (pix_xy: x, y pairs) and samples [sample0, sample0 + spp): out receives
 * npix * spp * 3 floats, sample-major within each pixel. Same parameters as
 * nr_render. */
int nr_render_samples(nr_scene* scene, const nr_camera* cam, const char* params, int32_t npix,
                      const int32_t* pix_xy, int32_t sample0, int32_t spp, float* out);

int nr_get_stats(const nr_scene* scene, nr_stats* stats);

/* The CUDA stream (cudaStream_t) on which the scene's kernels run, for
 * callers that time or order work against it. */
int nr_scene_stream(const nr_scene* scene, void** stream);

/* ------------------------------------------------------------------------
 * Neural radiance cache. Replaces the reference's nrc renderer network
 * (NNNodeMultiLayerPerceptron::eval / train, src/nn/nnnode.h:64-85,
 * src/nn/nnnode.cpp:175-201) with a fused 80-64-64-64-64-3 ReLU MLP on the
 * BF16 tensor cores with FP32 accumulation, FP32 master weights and Adam.
 * Loss: mean over rows and channels of (o - y)^2 / (o^2 + 0.01), the
 * reference's relative L2 (src/nn/nnnode.cpp:187-201) with o held constant
 * in the denominator.
 * ------------------------------------------------------------------------ */
#define NR_NRC_INPUTS 80

typedef struct nr_nrc nr_nrc;

/* params: lr (1e-3), beta1 (0.9), beta2 (0.99), eps (1e-8), seed (0, for the
 * Glorot-uniform initialisation), ema (0.99: renders query an exponential
 * moving average of the weights over Adam steps, 0 queries the current
 * weights), tc (1: the tcgen05 kernels for the forward and the data
 * gradients, the default; 0: mma.sync throughout), tc_first_wait (polls of
 * the first bounded wait for a group of tensor-core MMAs, default and maximum
 * 4194304; 0 makes every such wait time out at once, to exercise the
 * timeout path: the call then fails with NR_ERR_DEVICE, error bit 8, after
 * the kernel has waited again for its MMAs and freed its tensor memory).
 * Allocates on the current device. nr_nrc_infer and the gradient calls use
 * the current weights. */
int nr_nrc_create(const char* params, nr_nrc** out);
int nr_nrc_destroy(nr_nrc* nrc);
/* Number of FP32 parameters (weights and biases, layout in nrc.h). */
int nr_nrc_num_params(int64_t* n);
int nr_nrc_get_params(nr_nrc* nrc, float* params);
int nr_nrc_set_params(nr_nrc* nrc, const float* params);
/* The cache's whole training state, for checkpoint and resume (the
 * reference's network has no optimizer state to save). which selects one
 * array of nr_nrc_num_params floats: the FP32 parameters, the accumulated
 * gradient (zero between training calls), Adam's first and second moments,
 * the running sum of the moving average, the inference copy (that sum with
 * its start-up correction, what renders query), or, read only, the BF16
 * copies of the parameters and of the inference copy (widened to float); or
 * NR_NRC_STATE_STEP, one float holding the Adam step count, which sets the
 * bias corrections of the next step. Setting the parameters or the
 * inference copy refreshes its BF16 copy. */
#define NR_NRC_STATE_PARAMS 0
#define NR_NRC_STATE_GRAD 1
#define NR_NRC_STATE_M 2
#define NR_NRC_STATE_V 3
#define NR_NRC_STATE_EMA 4
#define NR_NRC_STATE_INFER 5
#define NR_NRC_STATE_PARAMS_BF16 6
#define NR_NRC_STATE_INFER_BF16 7
#define NR_NRC_STATE_STEP 8
int nr_nrc_get_state(nr_nrc* nrc, int32_t which, float* out);
int nr_nrc_set_state(nr_nrc* nrc, int32_t which, const float* in);
/* Forward pass for n rows of NR_NRC_INPUTS floats (rounded to BF16); out n*3. */
int nr_nrc_infer(nr_nrc* nrc, int32_t n, const float* x, float* out);
/* Gradient of the loss over n rows (no update): grad receives
 * nr_nrc_num_params floats; loss the mean loss. */
int nr_nrc_gradient(nr_nrc* nrc, int32_t n, const float* x, const float* y, float* grad, float* loss);
/* One Adam step on the loss over n rows; loss (may be NULL) receives the
 * mean loss before the step. */
int nr_nrc_train_step(nr_nrc* nrc, int32_t n, const float* x, const float* y, float* loss);
/* Attaches a cache to a scene: nr_render with nrc=1 then ends non-training
 * paths at the vertex after their first diffuse bounce (a Lambert or
 * BlinnPhong vertex, or GGX with roughness >= nrc_rough, default 0.05), at
 * vertex depth >= nrc_mindepth (default 1), with the cache's prediction, and
 * trains the cache online on the suffix radiance of nrc_train training paths
 * per wavefront batch in nrc_steps Adam steps (defaults: 16384 and 3 for
 * batches of more than 2^22 paths, 4096 and 1 for smaller ones). Training paths end in the cache too, from vertex depth
 * nrc_train_depth on (default 3; 0 lets them run to the end), as the
 * reference's path_lim_train does (src/renderer/renderernrc.cpp:130). The
 * counts stay on the device: a render with nrc=1 adds no host
 * synchronisation. nrc_query=0 only trains. With nrc_direct=1 (default) the
 * query vertex still takes its light sample (shadow ray) and the cache
 * stands in only for the radiance after it; nrc_direct=0 makes the cache
 * stand in for all of it. A cache trained one way must be queried the same
 * way. nrc_first=1 lets a path end at its first diffuse vertex itself
 * (nrc_mindepth then defaults to 0): a cheaper frame whose error stops at
 * the cache's own bias.
 * NULL detaches. The cache must not be used through nr_nrc_* while a render
 * of the scene runs. */
int nr_scene_attach_nrc(nr_scene* scene, nr_nrc* nrc);

/* ------------------------------------------------------------------------
 * Differentiation (no counterpart in the reference).
 * ------------------------------------------------------------------------ */

/* Replaces the material parameters of a scene (same count, same types,
 * emitters stay emitters) without rebuilding the BVH. */
int nr_scene_set_materials(nr_scene* scene, int32_t n, const nr_material* mats);

/* Path-replay adjoint of the ptnee estimator. Given dL_dimage = d loss /
 * d image (W*H*3 floats, the image being the per-pixel mean of max(0, L)
 * that nr_render returns for the same params), writes d loss / d params
 * into dL_dparams: 7 floats per material (albedo r, g, b; roughness;
 * emission r, g, b). Each wave of paths is rendered once, recording every
 * bounce's hits and light-sample visibility (17 bytes per path and bounce,
 * at most adj_records bytes, default 32 GiB), then replayed from its Philox
 * keys and those records; bounces past the records are traced again.
 * adj_records=0 keeps no records: every path is recomputed from its Philox
 * keys alone (the same gradients, more tracing, no memory beyond a wave's
 * path state). adj=mega replays each path in one thread, re-traced. image
 * (may be NULL) receives the primal image of the same samples. */
int nr_adjoint(nr_scene* scene, const nr_camera* cam, const char* params, const float* dL_dimage, float* dL_dparams,
               float* image);

/* Material::bxdf, ::pdf and ::sampleBxdf of scene material `mat` evaluated
 * on the device for n queries: wo, nrm, wi, uv (3 floats each) and 4
 * uniforms per query for sampling. Writes f (3), pdf (1), wi_s (3). */
int nr_material_probe(nr_scene* scene, int32_t mat, int32_t n, const float* wo, const float* nrm, const float* wi,
                      const float* uv, const float* u, float* f, float* pdf, float* wi_s);

#ifdef __cplusplus
}
#endif

#endif /* NURAY_H */
