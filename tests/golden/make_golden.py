"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout where the reference sources exist (it compiles them with
oracle/Makefile and calls them through oracle/_ref/libnuray_ref.so):

    python tests/golden/make_golden.py [/path/to/reference]

Fixtures (all small .npz files):
  cornell_scene.npz      the Cornell box (scenes/cornell/CornellBox-Original.obj -s 100)
                         as the reference Loader flattens it
  cornell_bvh.npz        the reference BVH of that scene, depth-first
  cornell_intersect.npz  BVH::intersection for 4096 seeded rays
  cornell_samples.npz    per-sample radiance (Philox stream, seed 0) for 96
                         pixels x 8 samples at 320x240
  small_*.npz            the same for the seeded mixed-material scene of
                         nuray_gb300.scenes.small_scene(), plus material,
                         light-pick and texture probes
  cornell_render_rgb8.npz  the 8-bit image of RendererPTLS::render itself
                         (oracle/ref_render.cpp: the reference's frame loop
                         on the Philox stream) for the Cornell workload,
                         320x240 at 16 spp

    python tests/golden/make_golden.py [/path/to/reference] [--only render]
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import bind  # noqa: E402
from nuray_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
CORNELL_PARAMS = ("renderer=ptnee imgw=320 imgh=240 spp=16 campos=0,120,200 cameuler=0,0,0 camfov=64 "
                  "camasp=1.333")


def ref_scene_arrays(R):
    import ctypes
    L = R.L
    for f in ("ref_scene_num_tris", "ref_scene_num_mats"):
        getattr(L, f).argtypes = [ctypes.c_void_p]
    L.ref_scene_get_tris.argtypes = [ctypes.c_void_p] * 5
    L.ref_scene_get_mats.argtypes = [ctypes.c_void_p] * 3
    n, m = L.ref_scene_num_tris(R.h), L.ref_scene_num_mats(R.h)
    pos, uv, nrm = (np.zeros((n, k), np.float32) for k in (9, 6, 9))
    mat = np.zeros(n, np.int32)
    L.ref_scene_get_tris(R.h, pos.ctypes.data, uv.ctypes.data, nrm.ctypes.data, mat.ctypes.data)
    mi = np.zeros((m, 4), np.int32)
    mf = np.zeros((m, 12), np.float32)
    L.ref_scene_get_mats(R.h, mi.ctypes.data, mf.ctypes.data)
    return dict(pos=pos, uv=uv, nrm=nrm, mat=mat, mat_i=mi, mat_f=mf)


def seeded_rays(scene_pos, n, seed):
    rng = np.random.Generator(np.random.Philox(key=[seed, 99]))
    lo, hi = scene_pos.reshape(-1, 3).min(0), scene_pos.reshape(-1, 3).max(0)
    o = rng.uniform(lo - 0.1 * (hi - lo), hi + 0.1 * (hi - lo), size=(n, 3)).astype(np.float32)
    tgt = rng.uniform(lo, hi, size=(n, 3))
    d = tgt - o
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    return o, d


def sample_pixels(w, h, n, seed):
    rng = np.random.Generator(np.random.Philox(key=[seed, 5]))
    return np.stack([rng.integers(0, w, n), rng.integers(0, h, n)], 1).astype(np.int32)


def probe_inputs(n, seed):
    rng = np.random.Generator(np.random.Philox(key=[seed, 17]))
    def unit(k):
        v = rng.normal(size=(k, 3))
        return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)
    nrm = unit(n)
    wo = unit(n)
    wo[: n // 2] *= np.sign(np.sum(wo[: n // 2] * nrm[: n // 2], 1))[:, None]  # half in the upper hemisphere
    wi = unit(n)
    uv = np.concatenate([rng.uniform(-1.5, 2.5, size=(n, 2)), np.zeros((n, 1))], 1).astype(np.float32)
    u = rng.uniform(0, 1, size=(n, 4)).astype(np.float32)
    return wo, nrm, wi, uv, u


def render_fixture():
    """RendererPTLS::render's 8-bit output (src/renderer/rendererptls.cpp:165-181:
    per-sample max(0, L), the mean, pow(1/2.2), x255, clamp, qRgb's
    truncation) for the Cornell workload, seed 0."""
    g = dict(np.load(os.path.join(OUT, "cornell_scene.npz")))
    mats = [dict(type=int(i[0]), c0=f[0:3].tolist(), c1=f[3:6].tolist(), alpha=float(f[6]), ior=float(f[7]),
                 ns=float(f[8])) for i, f in zip(g["mat_i"], g["mat_f"])]
    sc = dict(pos=g["pos"], uv=g["uv"], nrm=g["nrm"], mat=g["mat"], mats=mats)
    rgb8 = bind.ref_render_image(sc, CORNELL_PARAMS, seed=0)
    np.savez_compressed(os.path.join(OUT, "cornell_render_rgb8.npz"), rgb8=rgb8, params=np.array(CORNELL_PARAMS),
                        seed=np.uint64(0))


def main(ref_root, only=None):
    if bind.build_ref(ref_root) is None:
        sys.exit("reference sources not found at " + ref_root)
    if only == "render":
        render_fixture()
        print("fixture written to", OUT)
        return
    desc = os.path.join(ref_root, "scenes/cornell/CornellBox-Original.obj") + " -s 100\n"
    R = bind.Oracle("ref", desc=desc)
    sc = ref_scene_arrays(R)
    np.savez_compressed(os.path.join(OUT, "cornell_scene.npz"), **sc)
    box, kids, first, count, tris = R.bvh()
    np.savez_compressed(os.path.join(OUT, "cornell_bvh.npz"), box=box, kids=kids, first=first, count=count, tris=tris)
    o, d = seeded_rays(sc["pos"], 4096, 1)
    # add camera rays, which graze the box walls and corners
    fx = np.random.Generator(np.random.Philox(key=[2, 3])).uniform(0, 320, 1024).astype(np.float32)
    fy = np.random.Generator(np.random.Philox(key=[2, 4])).uniform(0, 240, 1024).astype(np.float32)
    co, cd = R.camera_rays(CORNELL_PARAMS, fx, fy)
    o, d = np.concatenate([o, co]), np.concatenate([d, cd])
    tri, t, b1, b2 = R.intersect(o, d)
    np.savez_compressed(os.path.join(OUT, "cornell_intersect.npz"), o=o, d=d, tri=tri, t=t, b1=b1, b2=b2,
                        fx=fx, fy=fy, cam_o=co, cam_d=cd)
    pix = sample_pixels(320, 240, 96, 7)
    rad = R.render_samples(CORNELL_PARAMS, pix, 8, seed=0)
    np.savez_compressed(os.path.join(OUT, "cornell_samples.npz"), pix=pix, rad=rad,
                        params=np.array(CORNELL_PARAMS))

    s = scenes.small_scene()
    R2 = bind.Oracle("ref", s)
    box, kids, first, count, tris = R2.bvh()
    o, d = seeded_rays(s["pos"], 4096, 3)
    tri, t, b1, b2 = R2.intersect(o, d)
    pix = sample_pixels(48, 32, 64, 9)
    rad = R2.render_samples(s["params"], pix, 8, seed=0)
    probes = {}
    wo, nrm, wi, uv, u = probe_inputs(512, 11)
    for m in range(len(s["mats"])):
        f, pdf, ws = R2.material_probe(m, wo, nrm, wi, uv, u)
        probes[f"f{m}"], probes[f"pdf{m}"], probes[f"ws{m}"] = f, pdf, ws
    ul = np.linspace(0, 1, 257, dtype=np.float32)[:-1]
    ltri, lp = R2.light_pick(ul)
    tex_mat = next(i for i, m in enumerate(s["mats"]) if m.get("tex0", -1) >= 0)
    tuv = np.random.Generator(np.random.Philox(key=[4, 4])).uniform(-2, 3, size=(512, 2)).astype(np.float32)
    tex = R2.texture_lookup(tex_mat, 0, tuv)
    env = R2.texture_lookup(0, 1, tuv)
    np.savez_compressed(os.path.join(OUT, "small_ref.npz"), box=box, kids=kids, first=first, count=count,
                        tris=tris, o=o, d=d, tri=tri, t=t, b1=b1, b2=b2, pix=pix, rad=rad,
                        params=np.array(s["params"]), wo=wo, nrm=nrm, wi=wi, uv=uv, u=u, light_u=ul,
                        light_tri=ltri, light_p=np.float32(lp), tex_mat=np.int32(tex_mat), tex_uv=tuv,
                        tex_rgb=tex, env_rgb=env, **probes)
    render_fixture()
    print("fixtures written to", OUT)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only:
        args = [a for a in args if a != only]
    main(args[0] if args else bind.REF_ROOT, only)
