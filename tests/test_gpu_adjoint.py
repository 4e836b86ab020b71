"""Path-replay adjoint against central finite differences with common random
numbers (the same Philox stream at theta +- h).

* albedo and emission: for fixed random numbers the estimator is a
  polynomial in them (sampling does not depend on either), so the adjoint
  must match the finite differences of the CPU restatement (oracle) to 5 %
  relative, per parameter;
* roughness: the adjoint holds sampled directions fixed while finite
  differences with common random numbers move them, so the two agree in
  expectation only: checked on a scene without occluders over ~1M paths,
  within 5 % relative.
"""
import numpy as np
import pytest

from oracle.bind import Oracle, pixel_grid

pytestmark = pytest.mark.gpu


def quad(x0, x1, y, z0, z1, down=False):
    a, b, c, d = [np.array(v, np.float32) for v in ((x0, y, z0), (x1, y, z0), (x1, y, z1), (x0, y, z1))]
    tris = [(a, b, c), (a, c, d)] if not down else [(a, c, b), (a, d, c)]
    n = np.array([0, -1 if down else 1, 0], np.float32)
    return [np.concatenate(t) for t in tris], np.tile(n, 3)


def box_scene():
    """Floor (GGX-reflect), back wall (Lambert), a small box (Lambert) and two area lights."""
    pos, nrm, mat = [], [], []
    def add(q, m):
        ts, n = q
        for t in ts:
            pos.append(t); nrm.append(n); mat.append(m)
    add(quad(-5, 5, 0, -5, 5), 0)                      # floor
    ts = [np.array([-5, 0, -5, 5, 0, -5, 5, 6, -5], np.float32), np.array([-5, 0, -5, 5, 6, -5, -5, 6, -5], np.float32)]
    for t in ts:
        pos.append(t); nrm.append(np.tile(np.array([0, 0, 1], np.float32), 3)); mat.append(1)
    add(quad(-1, 1, 1.5, -1, 1), 2)                      # top of a box
    add(quad(-3, -1.5, 5, -1, 0.5, down=True), 3)        # light 1
    add(quad(1.5, 3, 5.5, -2, -0.5, down=True), 4)       # light 2
    mats = [dict(type=1, c0=[0.6, 0.5, 0.4], alpha=0.35), dict(type=0, c0=[0.5, 0.7, 0.3]),
            dict(type=0, c0=[0.8, 0.2, 0.2]), dict(type=5, c0=[8.0, 7.0, 5.0]), dict(type=5, c0=[3.0, 4.0, 6.0])]
    return dict(pos=np.array(pos), nrm=np.array(nrm), uv=np.zeros((len(pos), 6), np.float32),
                mat=np.array(mat, np.int32), mats=mats, textures=[], env_tex=-1)


PARAMS = "renderer=ptnee imgw=40 imgh=30 spp=16 campos=0,3,9 cameuler=0,-15,0 camfov=60 camasp=1.333 rrdepth=2 maxdepth=5"


def gpu(sc):
    from nuray_gb300 import Scene
    return Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"])


def loss_weights(shape, seed=0):
    return np.random.default_rng(seed).uniform(0.5, 1.5, size=shape).astype(np.float32)


def cpu_image(sc, params, seed=0):
    w, h = 40, 30
    spp = int(params.split("spp=")[1].split()[0])
    rad = Oracle("port", sc).render_samples(params, pixel_grid(w, h), spp, seed=seed)
    return rad.astype(np.float64).mean(1).reshape(h, w, 3)


def perturbed(sc, m, key, k, h):
    s2 = dict(sc, mats=[dict(x) for x in sc["mats"]])
    if key == "alpha":
        s2["mats"][m]["alpha"] += h
    else:
        c = list(s2["mats"][m]["c0"])
        c[k] += h
        s2["mats"][m]["c0"] = c
    return s2


def test_albedo_and_emission_gradients_match_cpu_finite_differences(gpu_lib, port_lib):
    sc = box_scene()
    S = gpu(sc)
    W = loss_weights((30, 40, 3))
    g = S.adjoint(PARAMS, W)
    assert g.shape == (5, 7)
    checks = [(0, "c0", 0, 0), (0, "c0", 2, 2), (1, "c0", 1, 1), (2, "c0", 0, 0), (3, "c0", 0, 4), (4, "c0", 2, 6)]
    for m, key, k, col in checks:
        h = 1e-2 * max(1.0, abs(sc["mats"][m]["c0"][k]))
        fp = (W * cpu_image(perturbed(sc, m, key, k, h), PARAMS)).sum()
        fm = (W * cpu_image(perturbed(sc, m, key, k, -h), PARAMS)).sum()
        fd = (fp - fm) / (2 * h)
        print(f"material {m} param {col}: adjoint {g[m, col]:.5f}  FD {fd:.5f}")
        assert abs(g[m, col] - fd) <= 0.05 * abs(fd) + 1e-4, (m, col, g[m, col], fd)


def test_roughness_gradient_in_expectation(gpu_lib):
    sc = box_scene()
    del_occluder = [i for i, m in enumerate(sc["mat"]) if m != 2]
    sc = dict(sc, pos=sc["pos"][del_occluder], nrm=sc["nrm"][del_occluder], uv=sc["uv"][del_occluder],
              mat=sc["mat"][del_occluder])
    S = gpu(sc)
    params = PARAMS.replace("spp=16", "spp=1024").replace("imgw=40 imgh=30", "imgw=40 imgh=30")
    W = loss_weights((30, 40, 3), 1)
    g = S.adjoint(params, W)
    h = 0.02
    vals = []
    for sgn in (1, -1):
        mats = [dict(x) for x in sc["mats"]]
        mats[0]["alpha"] += sgn * h
        S.set_materials(mats)
        vals.append(float((W * S.render(params)).sum()))
    S.set_materials(sc["mats"])
    fd = (vals[0] - vals[1]) / (2 * h)
    print(f"roughness: adjoint {g[0, 3]:.5f}  FD (common random numbers) {fd:.5f}")
    assert abs(g[0, 3] - fd) <= 0.05 * abs(fd) + 1e-3


def test_adjoint_image_equals_render_and_gradient_is_linear_in_dl(gpu_lib):
    sc = box_scene()
    S = gpu(sc)
    W = loss_weights((30, 40, 3), 2)
    g1, img = S.adjoint(PARAMS, W, want_image=True)
    ref = S.render(PARAMS)
    np.testing.assert_allclose(img, ref, rtol=1e-3, atol=1e-4)
    g2 = S.adjoint(PARAMS, 2 * W)
    np.testing.assert_allclose(g2, 2 * g1, rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("case", ["box", "box_unbounded_small_waves", "textured_env"])
def test_wavefront_replay_equals_one_thread_per_path(gpu_lib, case):
    """The default replay runs on the wavefront (trace and sort, shade, shadow
    rays per bounce); adj=mega replays each path in one thread. Same paths and
    the same terms, summed in another order: equal to float rounding."""
    from nuray_gb300 import scenes
    if case == "textured_env":
        sc = scenes.small_scene(4, env=True, textures=True)
        from test_gpu_parity import gpu_scene
        S = gpu_scene(sc)
        params = sc["params"].replace("spp=1 ", "spp=4 ") + " rrdepth=3 maxdepth=6"
        w, h = (int(params.split(k)[1].split()[0]) for k in ("imgw=", "imgh="))
    else:
        sc = box_scene()
        S = gpu(sc)
        params = PARAMS
        if case == "box_unbounded_small_waves":
            params = PARAMS.replace("rrdepth=2 maxdepth=5", "rrdepth=3 maxdepth=0") + " wave=5000"
        w, h = 40, 30
    W = loss_weights((h, w, 3), 5)
    gw, img_w = S.adjoint(params, W, want_image=True)
    gm, img_m = S.adjoint(params + " adj=mega", W, want_image=True)
    np.testing.assert_array_equal(img_w, img_m)
    assert np.abs(gm).max() > 0
    np.testing.assert_allclose(gw, gm, rtol=1e-3, atol=1e-5 * np.abs(gm).max())


def test_large_wave_adjoint_equals_split_waves(gpu_lib):
    """A wave of more than 2^22 paths renders its first pass with one
    shading kernel per category; the same samples in waves of 2^22 use one
    kernel for all: same image, gradients equal to float rounding."""
    sc = box_scene()
    S = gpu(sc)
    params = PARAMS.replace("spp=16", "spp=4096")  # 40 x 30 x 4096 = 4.9 M paths
    W = loss_weights((30, 40, 3), 3)
    g1, img1 = S.adjoint(params, W, want_image=True)
    g2, img2 = S.adjoint(params + " wave=4194304", W, want_image=True)
    np.testing.assert_allclose(img1, img2, rtol=1e-5, atol=1e-6)
    assert np.abs(g1).max() > 0
    np.testing.assert_allclose(g1, g2, rtol=1e-3, atol=1e-5 * np.abs(g1).max())
