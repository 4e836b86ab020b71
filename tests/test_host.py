"""Host-side logic without a GPU: the C ABI exports, the parameter grammar,
the loader and the reference-identical BVH builder (through tests/host_shim.cpp)."""
import ctypes
import os
import re

import numpy as np
import pytest

import shim
from conftest import REF_ROOT, ROOT, golden
from nuray_gb300 import scenes


@pytest.fixture(scope="module")
def host():
    return shim.load()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "nuray.h")).read()
    return sorted(set(re.findall(r"^int (nr_\w+)\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    from nuray_gb300 import build
    path = build.build()
    L = ctypes.CDLL(path)
    names = declared_functions()
    assert len(names) >= 13
    for n in names:
        assert hasattr(L, n), n
    from nuray_gb300._lib import SIGNATURES
    assert sorted(SIGNATURES) == names


def test_header_is_plain_c_and_links_from_c(tmp_path):
    """The boundary is a C ABI: include/nuray.h parses as pedantic C99, and a C
    program calling every declared entry point links against the library."""
    import subprocess
    from nuray_gb300 import build
    lib = build.build()
    names = declared_functions()
    src = tmp_path / "use.c"
    calls = "\n".join(f"    if (argc > 99) (void)(size_t)&{n};" for n in names)
    src.write_text('#include <stddef.h>\n#include "nuray.h"\nint main(int argc, char** argv) {\n    (void)argv;\n'
                   + calls + "\n    return nr_scene_destroy(NULL) == NR_OK ? 1 : 0;\n}\n")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-L", os.path.dirname(lib), "-lnuray_gpu", "-o", str(tmp_path / "use")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_library_without_gpu_reports_errors():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from nuray_gb300 import NuRayError, Scene
    with pytest.raises(NuRayError):
        Scene.from_arrays(np.zeros((1, 9), np.float32), np.zeros(1, np.int32), [dict(type=0, c0=(1, 1, 1))])


def test_config_grammar(host):
    p = b"renderer=ptnee imgw=320 spp=abc campos=0,120,200 bad=1,2 prr=0.5 k=v=w"
    assert host.shim_config_int(p, b"imgw", 1) == 320
    assert host.shim_config_int(p, b"spp", 7) == 7        # unparsable -> default
    assert host.shim_config_int(p, b"missing", 9) == 9
    assert abs(host.shim_config_float(p, b"prr", 0.8) - 0.5) < 1e-7
    v = np.zeros(3, np.float32)
    assert host.shim_config_vec3(p, b"campos", v.ctypes.data) == 1 and list(v) == [0, 120, 200]
    assert host.shim_config_vec3(p, b"bad", v.ctypes.data) == 0


def test_camera_matches_oracle(host, port_lib):
    from nuray_gb300._lib import Camera
    from oracle.bind import Oracle
    g = golden("cornell_intersect.npz")
    cam, fh = Camera(), ctypes.c_float()
    params = b"imgw=320 imgh=240 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333"
    host.shim_camera(params, ctypes.byref(cam), ctypes.byref(fh))
    assert list(cam.pos) == [0, 120, 200]
    np.testing.assert_allclose(list(cam.gaze), [0, 0, -1], atol=1e-6)
    np.testing.assert_allclose(fh.value, 2 * np.tan(64 * 3.14159 / 360), rtol=1e-6)
    cam2 = Camera()
    host.shim_camera(b"cameuler=30,-20,10", ctypes.byref(cam2), ctypes.byref(fh))
    assert abs(np.linalg.norm(list(cam2.gaze)) - 1) < 1e-5


def test_bvh_builder_matches_reference_tree(host):
    g = golden("cornell_bvh.npz")
    sc = golden("cornell_scene.npz")
    box, kids, first, count, tris, depth = shim.bvh(host, sc["pos"])
    for a, k in zip((box, kids, first, count, tris), ("box", "kids", "first", "count", "tris")):
        np.testing.assert_array_equal(a, g[k])
    s = golden("small_ref.npz")
    small = scenes.small_scene()
    res = shim.bvh(host, small["pos"])
    for a, k in zip(res[:5], ("box", "kids", "first", "count", "tris")):
        np.testing.assert_array_equal(a, s[k])


def _gpu_child_refs(kids, first, count):
    """The child references of the GPU node array (capi.cpp upload_scene):
    inner nodes numbered in depth-first order, leaves -1 - ((first << 3) | count)."""
    inner = np.flatnonzero(kids[:, 0] >= 0)
    index = -np.ones(len(kids), np.int64)
    index[inner] = np.arange(len(inner))
    ref = lambda c: int(index[c]) if kids[c, 0] >= 0 else -1 - ((int(first[c]) << 3) | int(count[c]))
    return np.array([[ref(kids[i, 0]), ref(kids[i, 1])] for i in inner], np.int32)


def _check_tree(host, refs, num_tris):
    refs = np.ascontiguousarray(refs, np.int32)
    err = ctypes.create_string_buffer(256)
    rc = host.shim_check_tree(refs.ctypes.data, len(refs), num_tris, err, 256)
    return rc, err.value.decode()


def test_tree_check_admits_built_trees_and_refuses_malformed_ones(host):
    """The closest-hit walk has no step budget: the upload refuses node arrays
    in which a node has two parents, a child does not follow its parent, or a
    leaf leaves the triangle array."""
    sc = scenes.terrain_spheres(3, tiles=8, cells_per_tile=8, spheres=16, slices=12, stacks=8, lights=4,
                                n_mats=4, extent=32.0)
    box, kids, first, count, tris, depth = shim.bvh(host, sc["pos"])
    n = len(sc["pos"])
    refs = _gpu_child_refs(kids, first, count)
    assert len(refs) > 100
    assert _check_tree(host, refs, n) == (0, "")
    inner = np.flatnonzero(refs[:, 0] >= 0)
    i = int(inner[len(inner) // 2])
    bad = refs.copy()
    bad[i, 0] = i  # a cycle: a node as its own child
    assert _check_tree(host, bad, n)[0] == -1
    bad = refs.copy()
    bad[i, 1] = bad[i, 0]  # one child referenced twice
    rc, msg = _check_tree(host, bad, n)
    assert rc == -1 and "two parents" in msg
    bad = refs.copy()
    bad[i + 1, 0] = i  # a child above its parent
    assert _check_tree(host, bad, n)[0] == -1
    bad = refs.copy()
    bad[len(bad) - 1, 1] = -1 - (((n - 1) << 3) | 5)  # a leaf reaching past the last triangle
    rc, msg = _check_tree(host, bad, n)
    assert rc == -1 and "leaf" in msg
    assert _check_tree(host, refs, n - 1)[0] == -1  # the same tree over fewer triangles


def test_bvh_builder_survives_overflowing_surface_areas(host):
    """Nested triangles doubling in size: past about 2^64 of extent the SAH's
    surface areas overflow float and no split has a finite cost. The
    reference's builder then keeps every triangle on one side and recurses
    until its stack overflows; this one splits at the median of the first
    axis, as the device builder does."""
    n = 100
    pos = np.array([[0, 0, 0.01 * k, 2.0 ** k, 0, 0.01 * k, 0, 2.0 ** k, 0.01 * k] for k in range(n)], np.float32)
    box, kids, first, count, tris, depth = shim.bvh(host, pos)
    assert sorted(tris.tolist()) == list(range(n))  # every triangle in exactly one leaf
    assert count.max() <= 5 and depth < 40
    assert _check_tree(host, _gpu_child_refs(kids, first, count), n) == (0, "")


def test_bvh_builder_stops_at_its_depth_limit(host):
    """Coincident triangles give every split the same cost, so the reference's
    SAH peels one off per level: a chain as deep as the triangle count. The
    builder stops past its depth limit (the traversal stack's, at scene
    creation) and returns no nodes with max_depth = limit + 1, instead of
    recursing until the host stack overflows (100,000 of them did)."""
    pos = np.tile(np.float32([0, 0, 0, 1, 0, 0, 0, 1, 0]), (100000, 1))
    box, kids, first, count, tris, depth = shim.bvh(host, pos, depth_limit=94)
    assert depth == 95 and len(kids) == 0
    box, kids, first, count, tris, depth = shim.bvh(host, pos[:300], depth_limit=94)
    assert depth == 95 and len(kids) == 0  # a chain of 295 levels is past the limit too
    box, kids, first, count, tris, depth = shim.bvh(host, pos[:60], depth_limit=94)
    assert depth == 55 and len(kids) == 2 * 55 + 1  # a chain within the limit is built whole


def test_given_trees_are_checked_before_use(host):
    """nr_scene_create_bvh's check (nr::bvh_from_arrays) on the builder's own
    tree, the same tree in breadth-first order (children still after their
    parents), and trees broken one way at a time."""
    sc = scenes.terrain_spheres(3, tiles=8, cells_per_tile=8, spheres=16, slices=12, stacks=8, lights=4,
                                n_mats=4, extent=32.0)
    pos = sc["pos"]
    box, kids, first, count, tris, depth = shim.bvh(host, pos)
    tree = (box, kids, first, count, tris)
    assert shim.bvh_from_arrays(host, pos, tree) == (0, depth)
    # breadth-first order of the same nodes
    order, q = [], [0]
    while q:
        v = q.pop(0)
        order.append(v)
        if kids[v, 0] >= 0:
            q += [int(kids[v, 0]), int(kids[v, 1])]
    new = {old: i for i, old in enumerate(order)}
    kb = np.array([[new[a], new[b]] if a >= 0 else [-1, -1] for a, b in kids[order]], np.int32)
    assert shim.bvh_from_arrays(host, pos, (box[order], kb, first[order], count[order], tris)) == (0, depth)
    assert shim.bvh_from_arrays(host, pos, tree, depth_limit=3) == (0, 4)  # too deep: no tree, depth past the limit

    def broken(edit):
        t = [a.copy() for a in tree]
        edit(t)
        return shim.bvh_from_arrays(host, pos, t)

    leaf = int(np.flatnonzero(kids[:, 0] < 0)[3])
    inner = int(np.flatnonzero(kids[:, 0] >= 0)[5])

    def dup_tri(t): t[4][1] = t[4][0]
    def child_first(t): t[1][inner, 0] = 0
    def two_parents(t): t[1][inner, 1] = t[1][inner, 0]
    def box_too_small(t): t[0][leaf, 3:] = t[0][leaf, :3]
    def overlap(t): t[2][leaf] = t[2][leaf] - 1 if t[2][leaf] > 0 else t[2][leaf] + 1
    def nan_box(t): t[0][inner, 0] = np.nan
    def big_leaf(t): t[3][leaf] = 8
    def outside_parent(t): t[0][int(t[1][inner, 0]), :3] -= 1.0  # a child box reaching out of its parent's
    for edit, msg in ((dup_tri, "permutation"), (child_first, "follow its parent"), (two_parents, "two parents"),
                      (box_too_small, "does not hold"), (overlap, "overlap"), (nan_box, "bad box"),
                      (big_leaf, "at most 7"), (outside_parent, "inside its parent")):
        rc, m = broken(edit)
        assert rc == -1 and msg in m, (edit.__name__, m)


def test_image_headers_promising_more_than_the_file_holds_are_refused(host, tmp_path):
    """Declared sizes are checked against the data before anything is
    allocated for the pixels: PPM and PFM against the bytes left in the
    file, PNG against the inflated rows (and the inflater stops past them),
    JPEG against a 2^28-pixel cap and one bit of scan data per coded block."""
    import struct
    import zlib
    import jpeg_enc

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xffffffff)

    def png(w, h, idat):
        return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
                + chunk(b"IDAT", idat) + chunk(b"IEND", b""))

    for name, data, msg in (("a.ppm", b"P6\n99999999 99999999\n255\n" + bytes(30), "truncated PPM"),
                            ("b.pfm", b"PF\n99999 99999\n-1.0\n" + bytes(30), "truncated PFM")):
        (tmp_path / name).write_bytes(data)
        with pytest.raises(ValueError, match=msg):
            shim.read_image(host, str(tmp_path / name))
    with pytest.raises(ValueError, match="truncated PNG image data"):
        shim.png_decode(host, png(30000, 30000, zlib.compress(b"\0" * 100)))
    with pytest.raises(ValueError, match="longer than expected"):  # 10 MB of rows for a 64 x 64 image
        shim.png_decode(host, png(64, 64, zlib.compress(b"\0" * 10_000_000, 9)))
    img = (np.random.default_rng(0).random((8, 8, 3)) * 255).astype(np.uint8)
    base = bytearray(jpeg_enc.encode(img)[0])
    i = base.find(b"\xff\xc0")
    for side, msg in ((65535, "larger than 2"), (16000, "too short for its frame size")):
        b = bytearray(base)
        b[i + 5:i + 7] = side.to_bytes(2, "big")
        b[i + 7:i + 9] = side.to_bytes(2, "big")
        with pytest.raises(ValueError, match=msg):
            shim.jpeg_decode(host, bytes(b))


def test_bvh_builder_parallel_is_deterministic(host, port_lib):
    from oracle.bind import Oracle
    sc = scenes.terrain_spheres(3, tiles=16, cells_per_tile=8, spheres=64, slices=16, stacks=12, lights=8,
                                n_mats=8, extent=64.0)
    one = shim.bvh(host, sc["pos"], threads=1)
    many = shim.bvh(host, sc["pos"], threads=8)
    port = Oracle("port", sc).bvh()
    for a, b, c in zip(one[:5], many[:5], port):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(a, c)
    assert one[2][one[1][:, 0] < 0].min() >= 0 and one[3].max() <= 5


def test_loader_matches_reference_loader_fixture(host):
    ref = os.path.join(REF_ROOT, "scenes/cornell/CornellBox-Original.obj")
    if not os.path.exists(ref):
        pytest.skip("reference scenes not present")
    pos, uv, nrm, mat, mats = shim.load_scene(host, ref + " -s 100\n")
    g = golden("cornell_scene.npz")
    np.testing.assert_array_equal(pos, g["pos"])
    np.testing.assert_array_equal(uv, g["uv"])
    np.testing.assert_array_equal(nrm, g["nrm"])
    # materials: compare contents per triangle (the indices follow creation order)
    for i in range(len(mat)):
        m = mats[mat[i]]
        gi, gf = g["mat_i"][g["mat"][i]], g["mat_f"][g["mat"][i]]
        assert m.type == gi[0]
        np.testing.assert_array_equal(list(m.c0), gf[0:3])


def test_loader_forced_materials_and_errors(host, tmp_path):
    obj = tmp_path / "q.obj"
    obj.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nf 1/1 2/2 3/3 4\nf -4 -3 -2\n")
    pos, uv, nrm, mat, mats = shim.load_scene(host, f"{obj} -p 1 2 3 -s 2 -m=ggxr 0.5 0.6 0.7 0.3\n"
                                                    f"{obj} -m=light 1 2 3\n{obj} -m=ggx 1 1 1 0.2 1.5 -m=glass 1 1 1 1.4\n")
    assert pos.shape[0] == 9  # quad -> 2 triangles + 1, three lines
    np.testing.assert_array_equal(pos[0, :3], [1, 2, 3])
    np.testing.assert_array_equal(pos[0, 3:6], [3, 2, 3])
    assert [m.type for m in mats] == [1, 5, 2, 3]  # later -m flags replace earlier ones, glass last
    assert abs(mats[0].alpha - 0.3) < 1e-7 and abs(mats[3].ior - 1.4) < 1e-6
    np.testing.assert_allclose(nrm[0, :3], [0, 0, 1], atol=1e-6)  # face normal when no vn
    np.testing.assert_array_equal(uv[1], [1, 1, 0, 0, 0, 0])      # second half of the quad: vt 3, (none), vt 1
    with pytest.raises(ValueError, match="cannot open"):
        shim.load_scene(host, str(tmp_path / "missing.obj") + "\n")
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError, match="out of range"):
        shim.load_scene(host, f"{bad} -m=light 1 1 1\n")


def _export_scene():
    return scenes.terrain_spheres(3, tiles=4, cells_per_tile=2, spheres=4, slices=8, stacks=6, lights=3, n_mats=6,
                                  extent=40.0, mixed_materials=True)


def test_scene_export_loads_back_identically(host, tmp_path):
    """scenes.write_scene: OBJ files and a scene description that the loader
    reads into the same triangles (grouped by material) and materials."""
    from nuray_gb300._lib import MAT_BLINNPHONG, MAT_GGX, MAT_GGXR, MAT_GLASS
    sc = _export_scene()
    assert len({m["type"] for m in sc["mats"]}) == 6  # every material type is written
    desc, order = scenes.write_scene(sc, tmp_path)
    assert (tmp_path / "scene.desc").read_text() == desc and (tmp_path / "scene.params").exists()
    pos, uv, nrm, mat, mats = shim.load_scene(host, desc)
    np.testing.assert_array_equal(pos, sc["pos"][order])
    np.testing.assert_array_equal(uv, sc["uv"][order])
    np.testing.assert_array_equal(nrm, sc["nrm"][order])
    for i in np.unique(mat, return_index=True)[1]:
        got, want = mats[mat[i]], sc["mats"][sc["mat"][order[i]]]
        assert got.type == want["type"]
        np.testing.assert_array_equal(list(got.c0), np.float32(want["c0"]))
        if got.type in (MAT_GGXR, MAT_GGX):
            assert got.alpha == np.float32(want["alpha"])
        if got.type in (MAT_GGX, MAT_GLASS):
            assert got.ior == np.float32(want["ior"])
        if got.type == MAT_BLINNPHONG:
            np.testing.assert_array_equal(list(got.c1), np.float32(want["c1"]))
            assert got.ns == np.float32(want["ns"])
    textured = scenes.with_env_textures(sc, 0, tex_size=8, env_size=(8, 4))
    with pytest.raises(ValueError, match="textured"):
        scenes.write_scene(textured, tmp_path / "t")


def test_scene_export_renders_identically_in_the_reference(port_lib, ref_lib, tmp_path):
    """The written files through the reference's own Loader
    (Loader::fromSceneDescription) give the samples of the arrays the
    export permuted: the reference reads the same scene."""
    from oracle.bind import Oracle, pixel_grid
    sc = _export_scene()
    desc, order = scenes.write_scene(sc, tmp_path)
    perm = dict(sc, pos=sc["pos"][order], uv=sc["uv"][order], nrm=sc["nrm"][order], mat=sc["mat"][order])
    R, P = Oracle("ref", desc=desc), Oracle("port", perm)
    params = "renderer=ptnee imgw=48 imgh=32 spp=4 campos=0,14,34 cameuler=0,-20,0 camfov=50 camasp=1.5"
    pix = pixel_grid(48, 32)
    a, b = P.render_samples(params, pix, 2, seed=1), R.render_samples(params, pix, 2, seed=1)
    assert a.mean() > 0
    np.testing.assert_array_equal(a, b)


def test_scene_export_command(tmp_path, capsys):
    scenes.main([str(tmp_path / "s"), "--small", "--seed", "2"])
    out = capsys.readouterr().out
    assert "triangles" in out
    desc = (tmp_path / "s" / "scene.desc").read_text().splitlines()
    assert desc and all(line.split()[0].endswith(".obj") for line in desc)
    assert "renderer=ptnee" in (tmp_path / "s" / "scene.params").read_text()
