// CPU restatement of the reference ptnee integrator (TEST INFRASTRUCTURE).
//
// A from-scratch C++ restatement of RendererPTLS (src/renderer/rendererptls.cpp:13-94)
// and everything it calls: the SAH BVH of src/hierarchy/bvh.cpp:5-137 and
// src/hierarchy/bvhnode.cpp:4-66, Triangle (src/scene/triangle.cpp), Camera
// (src/scene/camera.cpp), Texture/Envmap lookups (src/scene/texture.cpp:54-72,
// src/scene/envmap.cpp:17-24), LightSampler (src/sampler/lightsampler.cpp) and
// the six materials (src/material/*.cpp). It reproduces the reference's
// float/double promotions operation by operation, so on the same inputs and
// random stream it returns the reference's bits (pinned against the reference
// compiled from source by tests/test_oracle_pin.py and the fixtures in
// tests/golden/).
//
// Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
// The product (nuray_gb300/) never links it.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Scene from flat arrays (same layout as the product's nr_scene_desc):
// pos/uv/nrm 9/6/9 floats per triangle; mat_i 4 ints per material
// (type, kd/f0 texture, ks texture, unused); mat_f 12 floats per material
// (c0 rgb, c1 rgb, alpha, ior, Ns, 0, 0, 0); textures tex_wh (w,h) pairs and
// concatenated linear rgb floats; env_tex < 0 for no environment.
void* port_scene_create(int ntri, const float* pos, const float* uv, const float* nrm, const int* tri_mat,
                        int nmat, const int* mat_i, const float* mat_f, int ntex, const int* tex_wh,
                        const float* tex_data, int env_tex, float env_gain, int build_threads);
void port_scene_destroy(void* scene);
int port_scene_set_materials(void* scene, int nmat, const int* mat_i, const float* mat_f);

// Depth-first export of the BVH (same layout as the reference harness).
int port_bvh_export(void* scene, float* box, int* kids, int* leaf_first, int* leaf_count, int* leaf_tris,
                    int* n_leaf_tris);

// Closest hit for n rays with the reference's exhaustive traversal and tie rules.
void port_intersect(void* scene, int n, const float* o, const float* d, int* tri, float* t, float* b1, float* b2,
                    int threads);

// Camera::generateRay for given film coordinates.
void port_camera_rays(const char* params, int n, const float* fx, const float* fy, float* dir, float* origin);

// Per-sample radiance (after max(0,.)) for listed pixels; see the reference
// harness for the stream layout. counters (may be null) receives
// {extension rays, shadow rays, vertices} summed over all samples.
void port_render_samples(void* scene, const char* params, int npix, const int* pix_xy, int sample0, int spp,
                         uint64_t seed, float* out, int threads, uint64_t* counters);

// Material virtuals on given inputs (same contract as ref_material_probe).
void port_material_probe(void* scene, int mat, int n, const float* wo, const float* nrm, const float* wi,
                         const float* uv, const float* u, float* f, float* pdf, float* wi_s);

// Emitter pick for given uniforms; returns LightSampler::p().
float port_light_pick(void* scene, int n, const float* u, int* tri);

// Texture::pixelUV on material mat's first map (kind 0) or the env map (kind 1).
void port_texture_lookup(void* scene, int mat, int kind, int n, const float* uvs, float* rgb);

#ifdef __cplusplus
}
#endif
