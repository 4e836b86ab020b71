"""The device BVH build (bvh=gpu) against the host build of the reference's
SAH tree (bvh=host, itself equal to the reference's tree, test_host.py).

* Scenes whose triangles have distinct pMax coordinates have one SAH tree:
  the device build must return it node for node (boxes, children, leaf
  ranges, leaf triangle order).
* Where pMax coordinates repeat (the procedural terrain shares vertices) the
  order of equal keys is unspecified in the reference (std::sort) and
  stable here, so trees may differ; closest hits through either tree must
  agree except where two triangles give the same t.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def soup(n, seed):
    """Random triangles whose pMax coordinates are distinct on every axis."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-50, 50, (n, 1, 3))
    pos = (c + rng.normal(0, 1.5, (n, 3, 3))).astype(np.float32)
    while True:
        dup = np.zeros(n, bool)
        for a in range(3):
            key = pos[:, :, a].max(1)
            _, first, counts = np.unique(key, return_index=True, return_counts=True)
            rep = np.isin(key, key[first[counts > 1]])
            dup |= rep
        if not dup.any():
            break
        pos[dup] += rng.normal(0, 1e-2, (int(dup.sum()), 3, 3)).astype(np.float32)
    mats = [dict(type=0, c0=[0.7, 0.7, 0.7]), dict(type=5, c0=[5, 5, 5])]
    mat = (rng.uniform(size=n) < 0.01).astype(np.int32)
    return pos.reshape(n, 9), mat, mats


def tree(S):
    return S.bvh()


@pytest.mark.parametrize("n,seed", [(3, 0), (5, 1), (6, 2), (1000, 3), (60000, 4)])
def test_distinct_keys_give_the_reference_tree(gpu_lib, n, seed):
    from nuray_gb300 import Scene
    pos, mat, mats = soup(n, seed)
    H = Scene.from_arrays(pos, mat, mats)
    G = Scene.from_arrays(pos, mat, mats, options="bvh=gpu")
    for a, b in zip(tree(H), tree(G)):
        np.testing.assert_array_equal(a, b)
    wall, dev = G.build_times()
    print(f"{n} triangles: device build {dev:.2f} ms ({wall:.1f} ms wall); host build {H.build_times()[0]:.1f} ms")


def test_shared_keys_give_the_same_closest_hits(gpu_lib):
    from nuray_gb300 import Scene, scenes
    sc = scenes.terrain_spheres(2, tiles=24, cells_per_tile=8, spheres=64, slices=16, stacks=12, lights=16, n_mats=16,
                                extent=96.0)
    H = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"])
    G = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"], options="bvh=gpu")
    ih, ig = H.info(), G.info()
    print("nodes host / gpu:", ih, ig)
    rng = np.random.default_rng(5)
    n = 400000
    # camera-like rays from above and rays leaving surface points
    pos = sc["pos"].reshape(-1, 3, 3)
    ti = rng.integers(0, pos.shape[0], n // 2)
    w = rng.dirichlet((1, 1, 1), n // 2)
    p = np.einsum("nk,nkc->nc", w, pos[ti])
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.concatenate([rng.uniform(-50, 50, (n // 2, 3)) + [0, 60, 0], p + d[n // 2:] * 1e-3])
    o, d = o.astype(np.float32), d.astype(np.float32)
    th, tt, bh1, bh2 = H.intersect(o, d)
    tg, tt2, bg1, bg2 = G.intersect(o, d)
    np.testing.assert_array_equal(tt, tt2)  # the closest distance never depends on the tree
    diff = th != tg
    print(f"ids differing: {diff.sum()} of {n} (all at equal t)")
    assert diff.mean() < 1e-3


def test_render_through_either_tree(gpu_lib):
    from nuray_gb300 import Scene
    g = golden("cornell_scene.npz")
    mats = [dict(type=int(i[0]), c0=f[0:3].tolist()) for i, f in zip(g["mat_i"], g["mat_f"])]
    H = Scene.from_arrays(g["pos"], g["mat"], mats, uv=g["uv"], nrm=g["nrm"])
    G = Scene.from_arrays(g["pos"], g["mat"], mats, uv=g["uv"], nrm=g["nrm"], options="bvh=gpu")
    p = "renderer=ptnee imgw=64 imgh=48 spp=8 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333"
    a, b = H.render(p), G.render(p)
    # the Cornell box's axis-aligned walls share pMax values: trees may differ,
    # and only paths through exact ties can change
    assert np.mean(np.abs(a - b) > 1e-6) < 0.01


def test_bad_option_is_an_error(gpu_lib):
    from nuray_gb300 import Scene
    pos, mat, mats = soup(10, 0)
    with pytest.raises(Exception):
        Scene.from_arrays(pos, mat, mats, options="bvh=octree")


def test_overflowing_surface_areas_build_and_intersect(gpu_lib):
    """Nested triangles doubling in size up to 2^99 of extent: past about
    2^64 the SAH's surface areas overflow float and no split has a finite
    cost. Both builders split at the first axis's median there (the
    reference would recurse without end) and give the same tree (distinct
    keys); rays going up at (x, y) hit the smallest triangle that covers the
    point, index ceil(log2(x + y))."""
    from nuray_gb300 import Scene
    n = 100
    pos = np.array([[0, 0, 0.01 * k, 2.0 ** k, 0, 0.01 * k, 0, 2.0 ** k, 0.01 * k] for k in range(n)], np.float32)
    mat = np.zeros(n, np.int32)
    mats = [dict(type=0, c0=(0.5, 0.5, 0.5))]
    H = Scene.from_arrays(pos, mat, mats)
    G = Scene.from_arrays(pos, mat, mats, options="bvh=gpu")
    for a, b in zip(tree(H), tree(G)):
        np.testing.assert_array_equal(a, b)
    rng = np.random.default_rng(0)
    m = 4000
    u = rng.integers(0, 41, m) + rng.uniform(0.1, 0.9, m)  # log2(x + y), away from the triangles' edges
    f = rng.uniform(0.05, 0.95, m)
    s = 2.0 ** u
    o = np.stack([s * f, s * (1 - f), np.full(m, -1.0)], 1).astype(np.float32)
    d = np.tile(np.float32([0, 0, 1]), (m, 1))
    want = np.ceil(u).astype(np.int32)
    for S in (H, G):
        tri, t = S.intersect(o, d)[:2]
        np.testing.assert_array_equal(tri, want)
        np.testing.assert_allclose(t, 1.0 + 0.01 * want, rtol=1e-5)


def test_coincident_triangles_are_refused_at_the_depth_limit(gpu_lib):
    """20,000 coincident triangles: every split costs the same, the
    reference's SAH peels one off per level, and the chain is deeper than
    the traversal stack holds. Both builders stop at that limit and the
    scene is refused, instead of building (or recursing) 20,000 levels."""
    from nuray_gb300 import Scene
    from nuray_gb300._lib import NuRayError
    n = 20000
    pos = np.tile(np.float32([0, 0, 0, 1, 0, 0, 0, 1, 0]), (n, 1))
    for opts in ("", "bvh=gpu"):
        with pytest.raises(NuRayError, match="deeper than 94 levels"):
            Scene.from_arrays(pos, np.zeros(n, np.int32), [dict(type=0, c0=(0.5, 0.5, 0.5))], options=opts)
    # the device stays usable
    S = Scene.from_arrays(pos[:50], np.zeros(50, np.int32), [dict(type=0, c0=(0.5, 0.5, 0.5))], options="bvh=gpu")
    tri = S.intersect(np.float32([[0.2, 0.2, 1.0]]), np.float32([[0, 0, -1]]))[0]
    assert 0 <= tri[0] < 50


def test_given_tree_gives_the_same_hits_and_image(gpu_lib):
    """nr_scene_create_bvh: the tree exported from one scene, handed to a
    second scene over the same triangles, in depth-first and in
    breadth-first node order, gives the same closest hits and the same image
    bit for bit; broken trees are refused."""
    from nuray_gb300 import Scene, scenes
    from nuray_gb300._lib import NuRayError
    sc = scenes.terrain_spheres(2, tiles=16, cells_per_tile=8, spheres=32, slices=16, stacks=12, lights=8, n_mats=8,
                                extent=64.0)
    args = (sc["pos"], sc["mat"], sc["mats"])
    kw = dict(uv=sc["uv"], nrm=sc["nrm"])
    H = Scene.from_arrays(*args, **kw)
    box, kids, first, count, tris = H.bvh()
    order, q = [], [0]
    while q:
        v = q.pop(0)
        order.append(v)
        if kids[v, 0] >= 0:
            q += [int(kids[v, 0]), int(kids[v, 1])]
    new = {old: i for i, old in enumerate(order)}
    kb = np.array([[new[a], new[b]] if a >= 0 else [-1, -1] for a, b in kids[order]], np.int32)
    bfs = (box[order], kb, first[order], count[order], tris)
    rng = np.random.default_rng(3)
    o = rng.uniform(-30, 30, (100000, 3)).astype(np.float32)
    o[:, 1] = rng.uniform(5, 40, 100000)
    d = rng.normal(size=(100000, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    want = H.intersect(o, d)[:2]
    params = sc["params"].replace("imgw=1920", "imgw=96").replace("imgh=1080", "imgh=54").replace("spp=64", "spp=4")
    img = H.render(params)
    for tree in ((box, kids, first, count, tris), bfs):
        G = Scene.from_arrays(*args, **kw, bvh=tree)
        got = G.intersect(o, d)[:2]
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1], want[1])
        np.testing.assert_array_equal(G.render(params), img)
    bad = kids.copy()
    bad[int(np.flatnonzero(kids[:, 0] >= 0)[2]), 0] = 0
    with pytest.raises(NuRayError, match="NR_ERR_INVALID: bvh: .*follow its parent"):
        Scene.from_arrays(*args, **kw, bvh=(box, bad, first, count, tris))
    small = box.copy()
    small[int(np.flatnonzero(kids[:, 0] < 0)[0]), 3:] = small[int(np.flatnonzero(kids[:, 0] < 0)[0]), :3]
    with pytest.raises(NuRayError, match="does not hold"):
        Scene.from_arrays(*args, **kw, bvh=(small, kids, first, count, tris))
