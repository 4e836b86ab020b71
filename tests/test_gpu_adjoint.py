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


def _c5_small():
    from nuray_gb300 import Scene, inverse
    sc = inverse.c5_scene_small(0)
    S = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"])
    return sc, S


def _set(mats, m, col, value):
    """mats with parameter `col` (albedo r g b 0-2, roughness 3, emission
    r g b 4-6, the adjoint's columns) of material m set to value."""
    out = [dict(x) for x in mats]
    if col == 3:
        out[m]["alpha"] = value
    else:
        c = list(out[m]["c0"])
        c[col % 4 if col < 3 else col - 4] = value
        out[m]["c0"] = c
    return out


def _get(mats, m, col):
    return mats[m]["alpha"] if col == 3 else mats[m]["c0"][col if col < 3 else col - 4]


def test_c5_reduced_gradients_vs_cpu_finite_differences(gpu_lib, port_lib):
    """The inverse-rendering workload reduced to what host cores can
    difference (inverse.c5_scene_small: the 200k-triangle scene, 8 surface
    materials, 2 emission materials, 128x128, depth 4, RR from 3): the
    adjoint's gradient of a weighted image sum for every albedo channel
    (all 8 materials), the emissions of both emitter materials, and the
    roughness of every GGX material, against central differences of the CPU
    restatement's renders (oracle/port) with h = 1e-3 and common random
    numbers.
    * albedo and emission: the estimator is polynomial in them for fixed
      random numbers, so the differences on the adjoint's own samples
      (16 spp, same seed) must agree within 5 %: one channel of every
      surface material, all three of the first emitter material, one of
      the second;
    * roughness: the differences move the sampled directions and cross
      visibility edges, the adjoint holds directions fixed; both estimate
      the same derivative of the expected image. The adjoint at 4096 spp
      against the restatement's differences over 4 independent seeds at
      32 spp each side: within 5 % plus three standard errors of the
      differences (their spread over the seeds). A far tighter check of the
      same quantity, with 16384 spp of differences from the GPU renderer
      (per-sample equal to the restatement), must agree within 5 %."""
    from nuray_gb300 import inverse
    from oracle.bind import Oracle
    sc, S = _c5_small()
    P = Oracle("port", sc)
    base = sc["params"]
    w = h = 128
    pix = pixel_grid(w, h)
    W = loss_weights((h, w, 3), 9)
    Wf = W.reshape(-1, 3).astype(np.float64)
    mats = sc["mats"]
    _, mask = inverse.param_table(mats)
    hstep = 1e-3

    def cpu_loss(m2, spp, seed):
        P.set_materials(m2)
        r = P.render_samples(base.replace("spp=64", f"spp={spp}"), pix, spp, seed=seed).astype(np.float64).mean(1)
        return float((Wf * r).sum())

    seed = 11
    g = S.adjoint(base.replace("spp=64", "spp=16") + f" seed={seed}", W)
    rows = []
    emitters = [m for m, mt in enumerate(mats) if mt["type"] == 5]
    for m, mt in enumerate(mats):
        if mt["type"] == 5:
            cols = [4, 5, 6] if m == emitters[0] else [5]
        else:
            cols = [m % 3]
        for col in cols:
            v = _get(mats, m, col)
            fd = (cpu_loss(_set(mats, m, col, v + hstep), 16, seed)
                  - cpu_loss(_set(mats, m, col, v - hstep), 16, seed)) / (2 * hstep)
            rows.append((m, col, g[m, col], fd))
            assert abs(g[m, col] - fd) <= 0.05 * abs(fd) + 1e-6 * np.abs(g).max(), (m, col, g[m, col], fd)
    P.set_materials(mats)
    print("albedo / emission (material, column, adjoint, FD):",
          ", ".join(f"({m},{c},{a:.4g},{f:.4g})" for m, c, a, f in rows))

    rough = [m for m, mt in enumerate(mats) if mask[m, 3]]
    assert len(rough) >= 4
    g_hi = S.adjoint(base.replace("spp=64", "spp=4096") + " seed=21", W)
    for m in rough:
        v = mats[m]["alpha"]
        fds = []
        for k in range(4):
            fds.append((cpu_loss(_set(mats, m, 3, v + hstep), 32, 100 + k)
                        - cpu_loss(_set(mats, m, 3, v - hstep), 32, 100 + k)) / (2 * hstep))
        fd_cpu, se_cpu = float(np.mean(fds)), float(np.std(fds, ddof=1) / 2)
        vals = []
        for sgn in (1, -1):
            S.set_materials(_set(mats, m, 3, v + sgn * hstep))
            vals.append(float((W * S.render(base.replace("spp=64", "spp=16384") + " seed=31")).sum()))
        S.set_materials(mats)
        fd_gpu = (vals[0] - vals[1]) / (2 * hstep)
        print(f"roughness of material {m} (alpha {v:.2f}): adjoint {g_hi[m, 3]:.4g}; CPU FD {fd_cpu:.4g} "
              f"(+-{se_cpu:.2g}); GPU-renderer FD {fd_gpu:.4g}")
        assert abs(g_hi[m, 3] - fd_cpu) <= 0.05 * abs(fd_cpu) + 3 * se_cpu, (m, g_hi[m, 3], fd_cpu, se_cpu)
        assert abs(g_hi[m, 3] - fd_gpu) <= 0.05 * abs(fd_gpu), (m, g_hi[m, 3], fd_gpu)
    P.set_materials(mats)


def test_autograd_function_vs_cpu_finite_differences(gpu_lib, port_lib):
    """nr_adjoint as the backward of a torch.autograd.Function
    (tests/adjoint_autograd.py): an L2 image loss against a target,
    loss.backward() gives d loss / d theta, checked against central
    differences (h = 1e-3, common random numbers) of the same loss on the CPU
    restatement's renders, for albedo and emission (exact estimators: within
    5 %); then torch.autograd.gradcheck on the albedo of two materials, its
    numerical side differencing the GPU forward."""
    import torch
    from adjoint_autograd import RenderImage
    from nuray_gb300 import inverse
    sc = box_scene()
    S = gpu(sc)
    P = Oracle("port", sc)
    mats = sc["mats"]
    params = PARAMS + " seed=3"
    P0, mask = inverse.param_table(mats)
    target = S.render(params.replace("seed=3", "seed=77"))
    theta = torch.tensor(P0 * 1.1, dtype=torch.float64, requires_grad=True)
    img = RenderImage.apply(theta, S, mats, params)
    loss = ((img - torch.from_numpy(target.astype(np.float64))) ** 2).mean()
    loss.backward()
    g = theta.grad.numpy()

    def cpu_loss(Pm):
        P.set_materials(inverse.apply(mats, Pm))
        r = P.render_samples(params, pixel_grid(40, 30), 16, seed=3).astype(np.float64).mean(1).reshape(30, 40, 3)
        return float(np.mean((r - target) ** 2))

    h = 1e-3
    for m, col in ((0, 0), (0, 2), (1, 1), (2, 0), (3, 4), (4, 6)):
        Pp, Pm = P0 * 1.1, P0 * 1.1
        Pp = Pp.copy(); Pm = Pm.copy()
        Pp[m, col] += h
        Pm[m, col] -= h
        fd = (cpu_loss(Pp) - cpu_loss(Pm)) / (2 * h)
        print(f"autograd material {m} column {col}: {g[m, col]:.6g}  CPU FD {fd:.6g}")
        assert abs(g[m, col] - fd) <= 0.05 * abs(fd) + 1e-9, (m, col, g[m, col], fd)
    assert np.all(g[~mask] == 0)

    # gradcheck on two albedo channels (the rest of theta held fixed)
    base = torch.tensor(P0 * 1.1, dtype=torch.float64)

    def f(x):
        t = base.clone()
        t[1, 1] = x[0]
        t[2, 0] = x[1]
        return ((RenderImage.apply(t, S, mats, params) - torch.from_numpy(target.astype(np.float64))) ** 2).mean()

    x0 = torch.tensor([float(base[1, 1]), float(base[2, 0])], dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(f, (x0,), eps=1e-3, atol=1e-7, rtol=0.05, nondet_tol=1e-7)
    S.set_materials(mats)


def test_pure_seed_replay_equals_recorded_replay(gpu_lib):
    """adj_records=0 keeps no per-bounce records: the replay traces every
    bounce again from the Philox keys (the checkpointing form of the
    adjoint). Same paths and terms as the default replay from records: equal
    gradients to float rounding, the same image."""
    sc = box_scene()
    S = gpu(sc)
    W = loss_weights((30, 40, 3), 8)
    for params in (PARAMS, PARAMS.replace("rrdepth=2 maxdepth=5", "rrdepth=3 maxdepth=0") + " wave=5000"):
        ga, ia = S.adjoint(params, W, want_image=True)
        gb, ib = S.adjoint(params + " adj_records=0", W, want_image=True)
        np.testing.assert_array_equal(ia, ib)
        assert np.abs(ga).max() > 0
        np.testing.assert_allclose(gb, ga, rtol=1e-3, atol=1e-5 * np.abs(ga).max())
