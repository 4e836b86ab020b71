"""Edge cases of the path against the oracle restatement (tolerances as in
test_gpu_parity.py): an empty scene, a scene without lights, a one-pixel
image, odd wavefront batch sizes, sample indices near 2^31, degenerate
(zero-area) triangles, and rays along the coordinate axes, where the
reference's slab test divides by d + 1e-9 (src/hierarchy/bvhnode.cpp:41)."""
import numpy as np
import pytest

from oracle.bind import Oracle, pixel_grid
from nuray_gb300 import scenes
from test_gpu_parity import _sample_match, cornell_scene, gpu_scene

pytestmark = pytest.mark.gpu

CORNELL = "renderer=ptnee imgw=64 imgh=48 spp=4 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333"


def test_empty_scene_renders_black_or_the_environment(gpu_lib):
    from nuray_gb300 import Scene
    S = Scene.from_arrays(np.zeros((0, 9), np.float32), np.zeros(0, np.int32), [dict(type=0, c0=[1, 1, 1])])
    img = S.render(CORNELL)
    assert img.shape == (48, 64, 3) and np.all(img == 0)
    tri, t, _, _ = S.intersect(np.zeros((4, 3), np.float32), np.tile(np.float32([0, 0, 1]), (4, 1)))
    assert np.all(tri == -1)
    sky = np.full((8, 16, 3), 0.5, np.float32)
    S.set_env(sky, 2.0)
    img = S.render(CORNELL)
    np.testing.assert_allclose(img, 1.0, rtol=1e-5)  # bilinear of a constant map (no edge texels reached)


def test_scene_without_lights_matches_port(gpu_lib, port_lib):
    sc = cornell_scene()
    mats = [dict(m, type=0) if m["type"] == 5 else m for m in sc["mats"]]
    sc = dict(sc, mats=mats)
    S, P = gpu_scene(sc), Oracle("port", sc)
    pix = pixel_grid(64, 48)[::7]
    a = S.render_samples(CORNELL, pix, 4)
    b = P.render_samples(CORNELL, pix, 4)
    assert np.all(a == 0) and np.all(b == 0)  # no emitter, no environment


def test_one_pixel_image_and_odd_waves(gpu_lib):
    S = gpu_scene(cornell_scene())
    one = S.render(CORNELL.replace("imgw=64 imgh=48", "imgw=1 imgh=1").replace("spp=4", "spp=257"))
    assert one.shape == (1, 1, 3) and np.all(np.isfinite(one))
    ref = S.render(CORNELL)
    for wave in (777, 4097):
        np.testing.assert_array_equal(S.render(CORNELL + f" wave={wave}"), ref)


def test_sample_indices_near_2_31(gpu_lib, port_lib):
    sc = cornell_scene()
    S, P = gpu_scene(sc), Oracle("port", sc)
    pix = pixel_grid(64, 48)[::11]
    s0 = 2 ** 31 - 3
    a = S.render_samples(CORNELL, pix, 2, sample0=s0)
    b = P.render_samples(CORNELL, pix, 2, sample0=s0)
    assert _sample_match(a, b) >= 0.97


def test_degenerate_triangles_match_port(gpu_lib, port_lib):
    sc = scenes.small_scene(7, env=False, textures=False)
    pos = sc["pos"].copy()
    rng = np.random.default_rng(3)
    bad = rng.choice(pos.shape[0], 200, replace=False)
    p = pos.reshape(-1, 3, 3)
    p[bad[:100], 2] = p[bad[:100], 1]                       # two equal vertices
    p[bad[100:], 2] = 0.5 * (p[bad[100:], 0] + p[bad[100:], 1])  # collinear
    sc = dict(sc, pos=p.reshape(-1, 9).astype(np.float32))
    S, P = gpu_scene(sc), Oracle("port", sc)
    pix = pixel_grid(48, 32)
    a = S.render_samples(sc["params"], pix, 4)
    b = P.render_samples(sc["params"], pix, 4)
    assert np.all(np.isfinite(a))
    assert _sample_match(a, b) >= 0.97


def test_axis_aligned_rays_match_port(gpu_lib, port_lib):
    sc = scenes.small_scene(2, env=False, textures=False)
    S, P = gpu_scene(sc), Oracle("port", sc)
    rng = np.random.default_rng(8)
    n = 6000
    o = rng.uniform(-20, 20, (n, 3)).astype(np.float32)
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                     [0.6, 0.8, 0], [0, -0.6, 0.8]], np.float32)
    d = axes[rng.integers(0, len(axes), n)]
    tri_g, t_g, _, _ = S.intersect(o, d)
    tri_r, t_r, _, _ = P.intersect(o, d)
    np.testing.assert_array_equal(tri_g >= 0, tri_r >= 0)
    h = tri_r >= 0
    assert h.mean() > 0.2
    np.testing.assert_allclose(t_g[h], t_r[h], rtol=1e-5)
    assert np.mean(tri_g[h] != tri_r[h]) < 1e-3


def test_wave_layouts_give_the_same_image(gpu_lib):
    """tile=0 (scanline), 1 (8x4 pixel tiles) and 2 (tile_samples samples of
    a tile of 32 / tile_samples pixels per warp; by default as many samples
    as divide spp, up to 32) order the paths differently in the wave; the
    film adds each pixel's samples in sample order in all of them, also
    across waves."""
    S = gpu_scene(cornell_scene())
    p = CORNELL.replace("spp=4", "spp=16")
    ref = S.render(p + " tile=0")
    for extra in (" tile=1", " tile=2", " tile=2 wave=777", " tile=2 wave=4096", " tile=2 wave=12289",
                  " tile=2 tile_samples=16", " tile=2 tile_samples=4 wave=3001", " tile=2 tile_samples=1",
                  " tile=2 tile_samples=2 wave=999"):
        np.testing.assert_array_equal(S.render(p + extra), ref, err_msg=extra)
    odd = CORNELL.replace("spp=4", "spp=12")
    for extra in (" tile=2", " tile=2 tile_samples=8"):  # 4 samples per warp; 8 do not divide 12: 8x4 tiles
        np.testing.assert_array_equal(S.render(odd + extra), S.render(odd + " tile=0"), err_msg=extra)


def test_many_emitters_light_pick_matches_port(gpu_lib, port_lib):
    """Half of the scene's triangles emitting, of unequal areas: the
    device's guided lower_bound over the emitter CDF picks the same light as
    the restatement's full search (LightSampler::sampleLight,
    src/sampler/lightsampler.cpp:56), so the per-sample radiance matches as
    for the other scenes."""
    sc = scenes.small_scene(5, env=False, textures=False)
    rng = np.random.default_rng(11)
    n = sc["pos"].shape[0]
    mats = [dict(m) for m in sc["mats"]] + [dict(type=5, c0=[2.0, 1.5, 1.0]), dict(type=5, c0=[0.5, 1.0, 2.5])]
    mat = sc["mat"].copy()
    pick = rng.choice(n, n // 2, replace=False)
    mat[pick] = len(mats) - 2 + (pick % 2)
    sc = dict(sc, mats=mats, mat=mat)
    S, P = gpu_scene(sc), Oracle("port", sc)
    assert S.info()["lights"] == int(sum(1 for m in sc["mat"] if sc["mats"][m]["type"] == 5))
    pix = pixel_grid(48, 32)
    a = S.render_samples(sc["params"], pix, 4)
    b = P.render_samples(sc["params"], pix, 4)
    assert np.all(np.isfinite(a)) and a.mean() > 0
    assert _sample_match(a, b) >= 0.97


def test_category_shading_kernels_equal_the_single_kernel(gpu_lib):
    """Waves of more than 2^22 paths shade with one kernel per shading
    category (material type fixed at compile time), smaller ones with one
    kernel for all categories: every material type, textures and an
    environment, rendered as one wave of 6.3 M paths and as waves of 2^22."""
    sc = scenes.small_scene(6, env=True, textures=True)
    S = gpu_scene(sc)
    p = sc["params"].replace("spp=4", "spp=4096")  # 48 x 32 x 4096 = 6.29 M paths
    one = S.render(p)
    split = S.render(p + " wave=4194304")
    assert np.all(np.isfinite(one)) and one.mean() > 0
    same = np.mean(one == split)
    np.testing.assert_allclose(one, split, rtol=1e-5, atol=1e-6)
    assert same >= 0.99, same


@pytest.mark.parametrize("envis", [0, 1])
def test_tail_kernel_gives_the_same_image(gpu_lib, envis):
    """tail=k: after k wavefront bounces one launch takes every live path
    to its end (light samples traced inline). The same functions in the same
    order: the same image, up to the compiler contracting a multiply-add
    differently where the shading code is inlined into the tail kernel
    (seen: one value in 4608 differing by one ulp)."""
    sc = scenes.small_scene(4, env=True, textures=True)
    S = gpu_scene(sc)
    p = sc["params"] + f" envis={envis}"
    ref = S.render(p)
    for k in (1, 2, 3, 5):
        img = S.render(p + f" tail={k}")
        np.testing.assert_allclose(img, ref, rtol=1e-6, atol=1e-7, err_msg=f"tail={k}")
        assert np.mean(img == ref) >= 0.999, k
    c = gpu_scene(cornell_scene())
    q = CORNELL.replace("spp=4", "spp=16") + " rrdepth=0 maxdepth=0"
    a, b = c.render(q + " tail=2"), c.render(q)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-7)
    assert np.mean(a == b) >= 0.999


def closed_cube(half=100.0):
    """Inward-facing cube of 12 triangles, white diffuse, no emitter."""
    v = np.array([[x, y, z] for x in (-half, half) for y in (-half, half) for z in (-half, half)], np.float32)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = [t for a, b, c, d in quads for t in ((a, c, b), (a, d, c))]  # quads wind outward: reversed
    pos = np.stack([v[list(t)].reshape(9) for t in tris]).astype(np.float32)
    return pos


@pytest.mark.parametrize("tail", [0, 2])
def test_endless_paths_stop_with_an_error(gpu_lib, tail):
    """prr=1 without a depth limit inside a closed white box: no path ever
    ends (the reference would loop forever). The render stops after 4096
    bounces with an error instead, and the scene stays usable."""
    from nuray_gb300 import NuRayError, Scene
    S = Scene.from_arrays(closed_cube(), np.zeros(12, np.int32), [dict(type=0, c0=[1, 1, 1])])
    p = "renderer=ptnee imgw=8 imgh=8 spp=16 campos=0,0,0 cameuler=0,0,0 camfov=64 camasp=1"
    # the host loop counts the bounces of the wavefront (tail=0); the tail
    # kernel counts its own and sets error bit 16
    with pytest.raises(NuRayError, match="error bits 16 " if tail else "4096 bounces"):
        S.render(p + f" prr=1 maxdepth=0 tail={tail}")
    img = S.render(p + f" tail={tail}")  # default prr: paths end, no light: black
    assert np.all(img == 0)


def test_camera_outside_the_widened_box_bound_takes_the_exact_walk(gpu_lib):
    """trav=1 walks boxes widened for ray origins inside the scene's origin
    bound (twice the largest coordinate plus four half extents); a camera
    outside it makes the render take the exact walk (trav=0), so both give
    the same image bit for bit."""
    S = gpu_scene(cornell_scene())
    far = CORNELL.replace("campos=0,120,200", "campos=0,120,40000").replace("camfov=64", "camfov=2")
    a = S.render(far)
    b = S.render(far + " trav=0")
    np.testing.assert_array_equal(a, b)
    assert a.mean() > 0
