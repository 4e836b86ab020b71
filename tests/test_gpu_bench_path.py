"""The benchmarked frames themselves against the oracle restatement.

Every other per-sample comparison goes through nr_render_samples, whose
small pixel-list waves shade with the single all-category kernel and end in
the tail kernel. The frames that bench.py times take another route: one
wave of 2^27 paths (more than 2^22, so one shading kernel per material
category), the warp layout of 32 samples of a pixel (tile=2), the live
count read back from bounce 5 on, eight wavefront bounces and no tail
kernel. These tests render exactly those frames through nr_render with the
bench's own parameters and compare them with the CPU restatement
(oracle/port, bit-identical to the reference's RendererPTLS on x86):

* per-pixel means of the full 1920x1080x64 frame of the 1M-triangle scene
  on 2048 scattered pixels against the restatement's mean of the same 64
  Philox samples: a pixel agrees when every channel is within rtol 2e-3 /
  atol 1e-4 (the per-sample tolerance of test_gpu_parity.py; one path of
  64 that leaves a triangle edge differently fails its pixel), at least
  97 % of pixels;
* the same for the third workload's frame (HDR sky with its importance
  sampling, value-noise textures, 10 % GGX dielectrics, 256 spp: four
  waves of 2^27);
* a per-pixel 4-sigma z-test of a crop of the benchmark frame, with the
  GPU side taken from 32 independent bench-path frames (32 spp each, the
  variance from the spread of their means), against an independent
  1024-spp restatement render; relMSE printed;
* closest hits of 1.1 M rays aimed at grazing angles through the small
  sphere and terrain triangles (|s1.e1| < 2e-3), where the reference's
  biased determinant shortens t by q / (q + 1e-6), against the
  restatement's exhaustive traversal (src/hierarchy/bvh.cpp:99-127): the
  exhaustive GPU walk matches every id; the default pruned walk differs
  only on winners inside the band the bias opens;
* closest hits of 1.2 M rays of the frame's own distributions through the
  default pruned walk: every id, t-ties excepted.
"""
import numpy as np
import pytest

from oracle.bind import Oracle
from nuray_gb300 import scenes
from test_gpu_parity import check_hits, gpu_scene

pytestmark = pytest.mark.gpu

W, H = 1920, 1080


def _scatter(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, W, n), rng.integers(0, H, n)], 1).astype(np.int32)


def _pixel_agreement(img, pix, ref_mean):
    g = img[pix[:, 1], pix[:, 0]].astype(np.float64)
    ok = np.all(np.isclose(g, ref_mean, rtol=2e-3, atol=1e-4), axis=1)
    return ok.mean(), g


def _bench_path_stats(S, waves):
    st = S.stats()
    # one wave of 2^27 paths per 64 spp of 1080p, eight wavefront bounces
    # each, and no tail kernel (the tail kernel takes the place of the
    # bounces after the second)
    assert st["waves"] == waves, st
    assert st["bounces"] == 8 * waves, st
    return st


def test_bench_frame_pixel_means_vs_port(gpu_lib, port_lib):
    sc = scenes.terrain_spheres(0)
    S, P = gpu_scene(sc), Oracle("port", sc)
    params = sc["params"]
    img = S.render(params)
    _bench_path_stats(S, 1)
    pix = _scatter(2048, 31)
    ref = P.render_samples(params, pix, 64).astype(np.float64).mean(1)
    frac, g = _pixel_agreement(img, pix, ref)
    rel = np.abs(g - ref).sum() / ref.sum()
    print(f"1M-triangle bench frame: {frac * 100:.2f}% of 2048 pixel means within rtol 2e-3; "
          f"summed |diff| / summed mean {rel:.2e}")
    assert np.all(np.isfinite(img)) and img.mean() > 0
    assert frac >= 0.97
    assert rel < 2e-3


def test_c3_frame_pixel_means_vs_port(gpu_lib, port_lib):
    sc = scenes.with_env_textures(scenes.terrain_spheres(0), 0)
    S, P = gpu_scene(sc), Oracle("port", sc)
    params = sc["params"] + " envis=1"  # as bench.py --workload c3
    assert "spp=256" in params
    img = S.render(params)
    _bench_path_stats(S, 4)
    pix = _scatter(2048, 32)
    ref = P.render_samples(params, pix, 256).astype(np.float64).mean(1)
    frac, g = _pixel_agreement(img, pix, ref)
    rel = np.abs(g - ref).sum() / ref.sum()
    print(f"third-workload frame: {frac * 100:.2f}% of 2048 pixel means within rtol 2e-3; "
          f"summed |diff| / summed mean {rel:.2e}")
    assert frac >= 0.97
    assert rel < 2e-3


def test_bench_frame_crop_ztest(gpu_lib, port_lib):
    sc = scenes.terrain_spheres(0)
    S, P = gpu_scene(sc), Oracle("port", sc)
    # a 48x32 crop with terrain, spheres and their shadows in view
    xs, ys = np.meshgrid(np.arange(900, 900 + 48 * 4, 4), np.arange(500, 500 + 32 * 4, 4))
    pix = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
    frames = []
    for k in range(32):
        img = S.render(sc["params"].replace("spp=64", "spp=32").replace("seed=0", f"seed={k + 1}"))
        frames.append(img[pix[:, 1], pix[:, 0]].astype(np.float64))
    st = S.stats()
    assert st["waves"] == 1 and st["bounces"] == 8  # 66.4 M paths: still the per-category wavefront
    F = np.stack(frames)
    mg, vg = F.mean(0), F.var(0, ddof=1) / F.shape[0]
    ref = P.render_samples(sc["params"].replace("seed=0", "seed=999"), pix, 1024, seed=999).astype(np.float64)
    mr, vr = ref.mean(1), ref.var(1, ddof=1) / ref.shape[1]
    z = (mg - mr) / np.sqrt(vg + vr + 1e-12)
    frac_out = np.mean(np.abs(z) > 4)
    relmse = np.mean((mg - mr) ** 2 / (mr ** 2 + 1e-2))
    print(f"bench-frame crop ({len(pix)} pixels): |z|>4 fraction {frac_out:.4f}, relMSE(GPU 1024 spp in 32 "
          f"frames vs CPU 1024 spp) {relmse:.3e}")
    assert frac_out <= 0.005
    assert relmse < 0.05


def grazing_rays(sc, n, seed, first, last):
    """Rays through random points of random triangles in [first, last) whose
    direction makes q = s1.e1 = -d.(e1 x e2) fall in (1e-8, 2e-3), 80 %
    positive (the side where the biased t is shortened), arriving from a
    distance of 0.5 to 40 scene units."""
    pos = sc["pos"].astype(np.float64)
    rng = np.random.default_rng(seed)
    ti = rng.integers(first, last, n)
    p0, p1, p2 = pos[ti, 0:3], pos[ti, 3:6], pos[ti, 6:9]
    e1, e2 = p1 - p0, p2 - p0
    nn = np.cross(e1, e2)
    a2 = np.linalg.norm(nn, axis=1)
    keep = a2 > 1e-9
    ti, p0, e1, e2, nn, a2 = ti[keep], p0[keep], e1[keep], e2[keep], nn[keep], a2[keep]
    n = len(ti)
    nh = nn / a2[:, None]
    q = np.exp(rng.uniform(np.log(1e-8), np.log(2e-3), n)) * np.where(rng.uniform(size=n) < 0.8, 1.0, -1.0)
    c = np.clip(-q / a2, -1, 1)
    t1 = e1 / np.linalg.norm(e1, axis=1)[:, None]
    t2 = np.cross(nh, t1)
    ang = rng.uniform(0, 2 * np.pi, n)
    tan = t1 * np.cos(ang)[:, None] + t2 * np.sin(ang)[:, None]
    d = tan * np.sqrt(1 - c ** 2)[:, None] + nh * c[:, None]
    u, v = rng.uniform(size=n), rng.uniform(size=n)
    sw = u + v > 1
    u[sw], v[sw] = 1 - u[sw], 1 - v[sw]
    pt = p0 + e1 * u[:, None] + e2 * v[:, None]
    dist = np.exp(rng.uniform(np.log(0.5), np.log(40.0), n))
    o = pt - d * dist[:, None]
    return o.astype(np.float32), d.astype(np.float32), ti


def _q(sc, tri, d):
    """The reference's determinant s1.e1 (without its 1e-6) of triangle tri
    for direction d, in float64."""
    p = sc["pos"][tri].astype(np.float64)
    e1, e2 = p[:, 3:6] - p[:, 0:3], p[:, 6:9] - p[:, 0:3]
    return np.einsum("ij,ij->i", np.cross(d.astype(np.float64), e2), e1)


def _real_mismatches(tri_g, t_g, tri_r, t_r):
    bad = np.nonzero(tri_g != tri_r)[0]
    return np.array([i for i in bad if abs(t_g[i] - t_r[i]) > 1e-6 * abs(t_r[i])], np.int64), len(bad)


def test_grazing_rays_vs_exhaustive_traversal(gpu_lib, port_lib):
    """1.1 M rays aimed through sphere and terrain triangles at grazing
    angles. The exhaustive walk (NR_INTERSECT_EXHAUSTIVE, prune=0) returns
    the reference's hits for every one of them. The default walk, which
    skips subtrees entered beyond 1.001 x its best hit, may differ only
    where the reference's winner is a triangle whose determinant s1.e1 lies
    in the band where the 1e-6 bias shortens its t past the pruning margin
    (-1e-6 < q < 1e-3): each such difference is checked to be one."""
    sc = scenes.terrain_spheres(0)
    S, P = gpu_scene(sc), Oracle("port", sc)
    terrain = 64 * 64 * 8 * 8 * 2
    spheres = 512 * (24 * 18 * 2 + 2 * 24)
    batches = [grazing_rays(sc, 600000, 1, terrain, terrain + spheres),  # spheres, radius 0.5 to 3
               grazing_rays(sc, 500000, 2, 0, terrain)]                   # terrain cells
    total = 0
    for o, d, ti in batches:
        tri_r, t_r, _, _ = P.intersect(o, d)
        tri_x, t_x, _, _ = S.intersect(o, d, exhaustive=True)
        ties = check_hits(P, o, d, tri_x, t_x, tri_r, t_r)
        real_x, _ = _real_mismatches(tri_x, t_x, tri_r, t_r)
        tri_g, t_g, _, _ = S.intersect(o, d)
        real, nbad = _real_mismatches(tri_g, t_g, tri_r, t_r)
        q = _q(sc, tri_r[real], d[real]) if len(real) else np.zeros(0)
        print(f"grazing batch: {len(o)} rays, {np.mean(tri_r >= 0) * 100:.1f}% hit, "
              f"{np.mean(tri_r == ti) * 100:.1f}% hit the aimed triangle; exhaustive walk: {len(real_x)} id "
              f"mismatches, {ties} t-ties; default walk: {len(real)} mismatches (reference winner's q in "
              f"[{q.min() if len(q) else 0:.2e}, {q.max() if len(q) else 0:.2e}]), {nbad - len(real)} t-ties")
        assert len(real_x) == 0
        # every difference of the pruned walk is a winner in the biased band
        assert np.all((q > -1e-6) & (q < 1e-3)), q[(q <= -1e-6) | (q >= 1e-3)][:10]
        # and the pruned walk's own hit is the nearer one geometrically
        hit = tri_r[real] >= 0
        assert np.all(t_g[real][hit] > t_r[real][hit])
        total += len(o)
    assert total >= 1000000


def test_natural_rays_vs_exhaustive_reference(gpu_lib, port_lib):
    """1.2 M rays of the benchmark frame's own distributions (camera rays
    with the frame's jitter, and rays leaving their hit points in cosine-
    weighted and uniform directions). The exhaustive walk returns the
    reference's hits for all of them, t-ties excepted. The default pruned
    walk differs on a few in a million: rays whose reference winner has
    q = s1.e1 < 1e-3, where the bias shortens t by more than the pruning
    margin. That is not only grazing incidence: the pole triangles of the
    small spheres have |e1 x e2| down to 1.8e-3, so q < 1e-3 at most angles.
    Each difference is checked to be one of those."""
    sc = scenes.terrain_spheres(0)
    S, P = gpu_scene(sc), Oracle("port", sc)
    rng = np.random.default_rng(44)
    n = 400000
    fx, fy = rng.uniform(0, W, n).astype(np.float32), rng.uniform(0, H, n).astype(np.float32)
    o, d = P.camera_rays(sc["params"], fx, fy)
    tri, t, _, _ = P.intersect(o, d)
    h = tri >= 0
    p = sc["pos"][tri[h]].astype(np.float64)
    nn = np.cross(p[:, 3:6] - p[:, 0:3], p[:, 6:9] - p[:, 0:3])
    nn /= np.linalg.norm(nn, axis=1, keepdims=True) + 1e-30
    nn *= -np.sign(np.einsum("ij,ij->i", nn, d[h]))[:, None]  # facing the incoming ray
    x = o[h] + d[h] * t[h, None]
    rays_o, rays_d = [o], [d]
    for cosine in (True, False):
        v = rng.normal(size=nn.shape)
        v /= np.linalg.norm(v, axis=1, keepdims=True)
        v *= np.sign(np.einsum("ij,ij->i", v, nn))[:, None]
        if cosine:
            v = v + nn
            v /= np.linalg.norm(v, axis=1, keepdims=True)
        rays_o.append((x + 1e-3 * v).astype(np.float32))  # the renderer's offset along the new direction
        rays_d.append(v.astype(np.float32))
    O, D = np.concatenate(rays_o), np.concatenate(rays_d)
    tri_r, t_r, _, _ = P.intersect(O, D)
    tri_x, t_x, _, _ = S.intersect(O, D, exhaustive=True)
    ties = check_hits(P, O, D, tri_x, t_x, tri_r, t_r)
    tri_g, t_g, _, _ = S.intersect(O, D)
    real, nbad = _real_mismatches(tri_g, t_g, tri_r, t_r)
    q = _q(sc, tri_r[real], D[real]) if len(real) else np.zeros(0)
    print(f"natural rays: {len(O)}, {np.mean(tri_r >= 0) * 100:.1f}% hit; exhaustive walk: {ties} t-ties, no other "
          f"difference; default walk: {len(real)} differences (reference winner's q {np.round(q, 6).tolist()}), "
          f"{nbad - len(real)} t-ties")
    assert len(O) >= 1000000
    assert ties <= 1e-4 * len(O)
    assert np.all((q > -1e-6) & (q < 1e-3))
    assert len(real) <= 1e-5 * len(O)
