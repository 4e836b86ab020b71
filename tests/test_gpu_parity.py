"""GPU parity: libnuray_gpu.so through its C ABI against the oracles.

Tolerances (stated per check):
* closest hits: triangle ids exact except t-ties (another triangle with t
  within 1e-6 relative of the reference hit); t within 1e-5 relative.
* material probes: FP32 device math against the reference's partly-double
  math: rtol 2e-3, atol 1e-5 on f / pdf / sampled directions, over at least
  99.5 % of the queries (the rest lie within float rounding of a branch).
* per-sample radiance with the same Philox stream: at least 97 % of samples
  within rtol 2e-3 / atol 1e-4 (a path may diverge from the CPU one when a
  rounded direction crosses a triangle edge).
* images: per-pixel 4-sigma z-test against an independent CPU render, at
  most 0.5 % of pixel channels outside (heavy-tailed estimator); relMSE
  against an FP64-accumulated CPU reference stated in the test output.
"""
import numpy as np
import pytest

from conftest import golden
from oracle.bind import Oracle, pixel_grid
from nuray_gb300 import scenes

pytestmark = pytest.mark.gpu

CORNELL = ("renderer=ptnee imgw=320 imgh=240 spp=16 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333")


def cornell_scene():
    g = golden("cornell_scene.npz")
    mats = [dict(type=int(i[0]), c0=f[0:3].tolist(), c1=f[3:6].tolist(), alpha=float(f[6]), ior=float(f[7]),
                 ns=float(f[8])) for i, f in zip(g["mat_i"], g["mat_f"])]
    return dict(pos=g["pos"], uv=g["uv"], nrm=g["nrm"], mat=g["mat"], mats=mats, textures=[], env_tex=-1,
                env_gain=1.0)


def gpu_scene(sc):
    from nuray_gb300 import Scene
    return Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc.get("uv"), nrm=sc.get("nrm"),
                             textures=sc.get("textures", []), env_tex=sc.get("env_tex", -1),
                             env_gain=sc.get("env_gain", 1.0))


def check_hits(oracle, o, d, tri_g, t_g, tri_r, t_r, b_g=None, b_r=None):
    """Exact ids except ties; returns the number of tie-excused mismatches."""
    hit = tri_r >= 0
    np.testing.assert_array_equal(tri_g >= 0, hit)
    np.testing.assert_allclose(t_g[hit], t_r[hit], rtol=1e-5)
    bad = np.nonzero(tri_g != tri_r)[0]
    for i in bad:
        # both candidates must lie at the same distance: a tie
        assert abs(t_g[i] - t_r[i]) <= 1e-6 * abs(t_r[i]), (i, tri_g[i], tri_r[i], t_g[i], t_r[i])
    return len(bad)


def test_intersect_cornell_golden(gpu_lib):
    g = golden("cornell_intersect.npz")
    S = gpu_scene(cornell_scene())
    tri, t, b1, b2 = S.intersect(g["o"], g["d"])
    ties = check_hits(None, g["o"], g["d"], tri, t, g["tri"], g["t"])
    assert ties == 0
    hit = g["tri"] >= 0
    # the reference's float arithmetic is reproduced, so hits agree to the bit
    assert np.mean(t[hit] == g["t"][hit]) > 0.999
    np.testing.assert_allclose(b1[hit], g["b1"][hit], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(b2[hit], g["b2"][hit], rtol=1e-5, atol=1e-6)


def test_intersect_mixed_golden(gpu_lib):
    g = golden("small_ref.npz")
    S = gpu_scene(scenes.small_scene())
    tri, t, b1, b2 = S.intersect(g["o"], g["d"])
    check_hits(None, g["o"], g["d"], tri, t, g["tri"], g["t"])
    assert np.mean(tri == g["tri"]) > 0.999


def test_intersect_million_triangles(gpu_lib, port_lib):
    sc = scenes.terrain_spheres(0)
    S = gpu_scene(sc)
    P = Oracle("port", sc)
    rng = np.random.default_rng(0)
    n = 30000
    fx, fy = rng.uniform(0, 1920, n).astype(np.float32), rng.uniform(0, 1080, n).astype(np.float32)
    o, d = P.camera_rays(sc["params"], fx, fy)
    # secondary-like rays: from hit points in random directions
    tri_r, t_r, _, _ = P.intersect(o, d)
    h = tri_r >= 0
    o2 = (o[h] + d[h] * t_r[h, None] * 0.999).astype(np.float32)
    d2 = rng.normal(size=o2.shape).astype(np.float32)
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    O, D = np.concatenate([o, o2]), np.concatenate([d, d2])
    tri_r, t_r, _, _ = P.intersect(O, D)
    tri_g, t_g, _, _ = S.intersect(O, D)
    ties = check_hits(P, O, D, tri_g, t_g, tri_r, t_r)
    assert ties <= 1e-3 * len(O)
    info = S.info()
    assert info["tris"] == sc["pos"].shape[0] and info["depth"] < 96


def test_samples_million_triangles_vs_port(gpu_lib, port_lib):
    """The benchmark frame's own scene and parameters (1M triangles, 32 quad
    lights, GGX-reflect materials, 1920x1080, maxdepth 8, RR from 3): the
    per-sample radiance of a spread of pixels on the shared Philox stream,
    GPU against the CPU restatement (a wave this small finishes its paths in
    the tail kernel after two bounces)."""
    sc = scenes.terrain_spheres(0)
    S = gpu_scene(sc)
    P = Oracle("port", sc)
    rng = np.random.default_rng(21)
    pix = np.stack([rng.integers(0, 1920, 400), rng.integers(0, 1080, 400)], 1).astype(np.int32)
    a = S.render_samples(sc["params"], pix, 4)
    b = P.render_samples(sc["params"], pix, 4)
    assert np.all(np.isfinite(a)) and a.mean() > 0
    assert _sample_match(a, b) >= 0.97


def test_material_probes(gpu_lib):
    g = golden("small_ref.npz")
    sc = scenes.small_scene()
    S = gpu_scene(sc)
    for m in range(len(sc["mats"])):
        f, pdf, ws = S.material_probe(m, g["wo"], g["nrm"], g["wi"], g["uv"], g["u"])
        for a, b in ((f, g[f"f{m}"]), (pdf[:, None], g[f"pdf{m}"][:, None]), (ws, g[f"ws{m}"])):
            ok = np.all(np.isclose(a, b, rtol=2e-3, atol=1e-5) | (np.isnan(a) & np.isnan(b)), axis=1)
            assert ok.mean() >= 0.995, (m, sc["mats"][m]["type"], ok.mean())


def _sample_match(gpu, ref):
    ok = np.all(np.isclose(gpu, ref, rtol=2e-3, atol=1e-4), axis=2)
    return ok.mean()


def test_samples_cornell_same_stream(gpu_lib):
    g = golden("cornell_samples.npz")
    S = gpu_scene(cornell_scene())
    rad = S.render_samples(str(g["params"]), g["pix"], 8)
    assert _sample_match(rad, g["rad"]) >= 0.97


def test_samples_mixed_same_stream(gpu_lib):
    g = golden("small_ref.npz")
    S = gpu_scene(scenes.small_scene())
    rad = S.render_samples(str(g["params"]), g["pix"], 8)
    assert _sample_match(rad, g["rad"]) >= 0.97


@pytest.mark.parametrize("extra", ["rrdepth=3 maxdepth=8", "mis=0 prr=0.6", "maxdepth=2", "seed=12345678901",
                                   "renderer=pt", "renderer=nrc path_lim=1000000"])
def test_samples_policies_vs_port(gpu_lib, port_lib, extra):
    sc = cornell_scene()
    S, P = gpu_scene(sc), Oracle("port", sc)
    params = CORNELL + " " + extra
    pix = pixel_grid(320, 240)[::97]
    seed = int(extra.split("seed=")[1]) if "seed=" in extra else 0
    a = S.render_samples(params, pix, 8)
    b = P.render_samples(params, pix, 8, seed=seed)
    assert _sample_match(a, b) >= 0.97


def _crop_stats(samples):
    x = samples.astype(np.float64)
    return x.mean(1), x.var(1, ddof=1) / x.shape[1]


def test_cornell_image_ztest_and_relmse(gpu_lib, port_lib):
    sc = cornell_scene()
    S, P = gpu_scene(sc), Oracle("port", sc)
    # a 40x30 crop around the box edge, light and shadows
    pix = np.array([(x, y) for y in range(60, 240, 6) for x in range(40, 280, 6)], np.int32)
    gpu = S.render_samples(CORNELL + " seed=1", pix, 256)
    ref = P.render_samples(CORNELL, pix, 1024, seed=2)
    mg, vg = _crop_stats(gpu)
    mr, vr = _crop_stats(ref)
    z = (mg - mr) / np.sqrt(vg + vr + 1e-12)
    frac_out = np.mean(np.abs(z) > 4)
    relmse = np.mean((mg - mr) ** 2 / (mr ** 2 + 1e-2))
    print(f"cornell crop: |z|>4 fraction {frac_out:.4f}, relMSE(GPU 256 spp vs CPU 1024 spp) {relmse:.3e}")
    assert frac_out <= 0.005
    assert relmse < 0.05


def test_render_api_consistency(gpu_lib):
    S = gpu_scene(cornell_scene())
    params = "renderer=ptnee imgw=64 imgh=48 spp=8 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333 wave=1000"
    hdr, rgb8 = S.render(params, want_rgb8=True)
    pix = pixel_grid(64, 48)
    smp = S.render_samples(params, pix, 8)
    np.testing.assert_allclose(hdr.reshape(-1, 3), smp.astype(np.float32).sum(1) / 8, rtol=1e-5, atol=1e-6)
    expect = np.clip(np.power(hdr, np.float32(1 / 2.2)) * 255, 0, 255).astype(np.int32)
    assert np.max(np.abs(expect - rgb8.astype(np.int32))) <= 1
    st = S.stats()
    assert st["paths"] == 64 * 48 * 8 and st["rays"] >= st["paths"] and st["waves"] == (64 * 48 * 8 + 999) // 1000
    # the same image whatever the wave size (per-path streams)
    hdr2 = S.render(params.replace("wave=1000", "wave=100000"))
    np.testing.assert_array_equal(hdr, hdr2)


def test_fast_traversal_tests_equal_exact_ones(gpu_lib):
    """trav=1 (approximate tests with exact fallback) must return the hits of
    trav=0 (the reference arithmetic throughout), so the images are identical."""
    for sc, params in ((cornell_scene(), CORNELL.replace("imgw=320 imgh=240", "imgw=96 imgh=72")),
                       (scenes.small_scene(3), scenes.small_scene(3)["params"])):
        S = gpu_scene(sc)
        a = S.render(params + " trav=0")
        b = S.render(params + " trav=1")
        np.testing.assert_array_equal(a, b)


def test_tiled_frame_order_gives_the_same_image(gpu_lib):
    S = gpu_scene(cornell_scene())
    params = "renderer=ptnee imgw=64 imgh=48 spp=4 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333"
    np.testing.assert_array_equal(S.render(params + " tile=1"), S.render(params + " tile=0"))


def test_accumulate_across_calls_equals_one_call(gpu_lib):
    S = gpu_scene(cornell_scene())
    params = "renderer=ptnee imgw=48 imgh=36 spp=4 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333"
    once = S.render(params)
    for k in range(4):
        img = S.render(params.replace("spp=4", "spp=1") + f" sample0={k}" + (" accumulate=1" if k else ""))
    np.testing.assert_allclose(img, once, rtol=1e-6, atol=1e-7)


def test_errors_and_cancel(gpu_lib):
    import ctypes
    from nuray_gb300 import NuRayError
    S = gpu_scene(cornell_scene())
    with pytest.raises(NuRayError, match="INVALID"):
        S.render("imgw=0 imgh=4")
    with pytest.raises(NuRayError, match="INVALID"):
        S.render_samples("imgw=4 imgh=4", np.array([[5, 0]]), 1)
    flag = ctypes.c_int32(0)
    with pytest.raises(NuRayError, match="CANCELLED"):
        S.render(CORNELL + " imgw=32 imgh=24 spp=2", cancel=flag)
    seen = []
    S.render(CORNELL + " imgw=32 imgh=24 spp=4 wave=512", progress=seen.append)
    assert seen and abs(seen[-1] - 100.0) < 1e-3 and seen == sorted(seen)
    with pytest.raises(NuRayError, match="INVALID"):
        gpu_scene(dict(cornell_scene(), mat=np.full(36, 99, np.int32)))


@pytest.mark.parametrize("renderer", ["ptnee", "nrc"])
def test_env_miss_and_textures_vs_port(gpu_lib, port_lib, renderer):
    sc = scenes.small_scene(5)
    S, P = gpu_scene(sc), Oracle("port", sc)
    pix = pixel_grid(48, 32)
    params = sc["params"].replace("renderer=ptnee", f"renderer={renderer}") + " path_lim=1000000"
    a = S.render_samples(params, pix, 4)
    b = P.render_samples(params, pix, 4)
    assert _sample_match(a, b) >= 0.97


def test_rgb8_vs_reference_render(gpu_lib, port_lib):
    """nr_render's 8-bit output against the reference's own RendererPTLS::render
    (src/renderer/rendererptls.cpp:165-181; fixture tests/golden/cornell_render_rgb8.npz,
    the reference's frame loop run whole on the Philox stream) for the
    Cornell workload, 320x240 at 16 spp. Where the GPU's per-pixel HDR mean
    agrees with the CPU restatement's mean of the same samples (every
    channel within the per-sample tolerance, rtol 2e-3 / atol 1e-4), the
    8-bit values may differ by one level only (a mean within that tolerance
    of a truncation boundary); at least 97 % of pixels agree that way, and
    most are identical."""
    g = golden("cornell_render_rgb8.npz")
    params = str(g["params"])
    S, P = gpu_scene(cornell_scene()), Oracle("port", cornell_scene())
    hdr, rgb8 = S.render(params + f" seed={int(g['seed'])}", want_rgb8=True)
    ref8 = g["rgb8"].astype(np.int32)
    mean = P.render_samples(params, pixel_grid(320, 240), 16, seed=int(g["seed"])).astype(np.float64).mean(1)
    agree = np.all(np.isclose(hdr.reshape(-1, 3).astype(np.float64), mean, rtol=2e-3, atol=1e-4), axis=1)
    diff = np.abs(rgb8.astype(np.int32) - ref8).reshape(-1, 3).max(1)
    print(f"8-bit vs the reference's render(): {np.mean(diff == 0) * 100:.2f}% identical, "
          f"{np.mean(diff <= 1) * 100:.2f}% within one level; HDR agrees on {agree.mean() * 100:.2f}%")
    assert np.all(diff[agree] <= 1)
    assert agree.mean() >= 0.97
    assert np.mean(diff == 0) >= 0.95
