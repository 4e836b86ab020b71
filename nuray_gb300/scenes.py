"""Seeded procedural scenes for the ptnee workloads.

The reference ships only the Cornell box; the larger workloads are
generated here from a seed with numpy's Philox generator, so the same
arrays come out on every machine:

* ``terrain_spheres(seed)`` with the defaults is the 1M-triangle scene:
  a 64x64-tile fBm heightfield (6 octaves, lacunarity 2, gain 0.5, 8x8
  quads per tile: 524,288 triangles), 512 UV spheres of radius U[0.5, 3]
  (24 slices x 20 stacks: 466,944 triangles), 32 emissive quads of
  radiance U[5, 20] (grey or tinted U[0.5, 1]^3), and 64 GGX-reflect
  materials with roughness U[0.05, 1] and albedo U[0.1, 0.9]^3:
  991,296 triangles in all.
* ``with_env_textures(scene, seed)`` adds a 2048x1024 HDR sky (gradient
  plus a Gaussian sun lobe of peak 5e3), 512x512 value-noise textures on
  half of the materials and turns 10 % of the materials into GGX
  dielectrics of IOR 1.5.
* Smaller variants (fewer cells and spheres, every material type) serve
  the parity tests.
* ``write_scene(scene, directory)`` writes a scene without textures as OBJ
  files and a scene description that the reference's Loader and
  ``nr_scene_load`` read into the same scene (``python -m
  nuray_gb300.scenes DIR`` for the 1M-triangle one: 79 MB, 12 s).

Each scene is a dict with pos (n,9), uv (n,6), nrm (n,9), mat (n,), mats
(list of material dicts), textures, env_tex, env_gain and the parameter
string of its camera.
"""
import numpy as np

from ._lib import MAT_BLINNPHONG, MAT_GGX, MAT_GGXR, MAT_GLASS, MAT_LAMBERT, MAT_LIGHT

C2_PARAMS = ("renderer=ptnee imgw=1920 imgh=1080 spp=64 campos=0,90,130 cameuler=0,-42,0 camfov=45 "
             "camasp=1.7778 maxdepth=8 rrdepth=3 seed=0")


def _rng(seed, stream):
    return np.random.Generator(np.random.Philox(key=[seed, stream]))


def _value_noise(x, z, lattice):
    """Smooth value noise on a periodic lattice (values in [-1, 1])."""
    n = lattice.shape[0]
    xi, zi = np.floor(x).astype(np.int64), np.floor(z).astype(np.int64)
    fx, fz = x - xi, z - zi
    sx, sz = fx * fx * (3 - 2 * fx), fz * fz * (3 - 2 * fz)
    a = lattice[xi % n, zi % n]
    b = lattice[(xi + 1) % n, zi % n]
    c = lattice[xi % n, (zi + 1) % n]
    d = lattice[(xi + 1) % n, (zi + 1) % n]
    return (a * (1 - sx) + b * sx) * (1 - sz) + (c * (1 - sx) + d * sx) * sz


def fbm(x, z, seed, octaves=6, lacunarity=2.0, gain=0.5):
    lattice = _rng(seed, 7).uniform(-1.0, 1.0, size=(256, 256))
    out = np.zeros_like(x)
    amp, freq = 1.0, 1.0
    for o in range(octaves):
        out += amp * _value_noise(x * freq + 17.0 * o, z * freq + 31.0 * o, lattice)
        amp *= gain
        freq *= lacunarity
    return out


def _terrain(seed, tiles, cells_per_tile, extent, height, scale, rng, n_mats):
    n = tiles * cells_per_tile
    xs = np.linspace(-extent / 2, extent / 2, n + 1)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    H = height * fbm(X / scale, Z / scale, seed)
    # normals from central differences of the height field
    dx = np.gradient(H, xs, axis=0)
    dz = np.gradient(H, xs, axis=1)
    N = np.stack([-dx, np.ones_like(H), -dz], -1)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    P = np.stack([X, H, Z], -1)
    U = np.stack([(X + extent / 2) / extent * tiles, (Z + extent / 2) / extent * tiles], -1)
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    i, j = i.ravel(), j.ravel()
    c00, c10, c01, c11 = (i, j), (i + 1, j), (i, j + 1), (i + 1, j + 1)
    tri_v = [(c00, c01, c11), (c00, c11, c10)]  # counter-clockwise seen from +y
    pos, nrm, uv = [], [], []
    for a, b, c in tri_v:
        pos.append(np.concatenate([P[a], P[b], P[c]], -1))
        nrm.append(np.concatenate([N[a], N[b], N[c]], -1))
        uv.append(np.concatenate([U[a], U[b], U[c]], -1))
    tile_mat = rng.integers(0, n_mats, size=(tiles, tiles))
    m = tile_mat[i // cells_per_tile, j // cells_per_tile]
    pos = np.stack(pos, 1).reshape(-1, 9)
    nrm = np.stack(nrm, 1).reshape(-1, 9)
    uv = np.stack(uv, 1).reshape(-1, 6)
    mat = np.repeat(m, 2)
    ground = lambda x, z: height * fbm(np.asarray(x) / scale, np.asarray(z) / scale, seed)
    return pos, nrm, uv, mat, ground


def _unit_sphere(slices, stacks):
    """UV sphere template: one triangle per cell at the poles, two elsewhere."""
    th = np.linspace(0, np.pi, stacks + 1)
    ph = np.linspace(0, 2 * np.pi, slices + 1)[:-1]
    T, F = np.meshgrid(th, ph, indexing="ij")
    N = np.stack([np.sin(T) * np.cos(F), np.cos(T), np.sin(T) * np.sin(F)], -1)
    U = np.stack([F / (2 * np.pi), 1 - T / np.pi], -1)
    tris = []
    for s in range(stacks):
        for k in range(slices):
            k1 = (k + 1) % slices
            a, b, c, d = (s, k), (s + 1, k), (s + 1, k1), (s, k1)
            if s == 0:
                tris.append((a, b, c))
            elif s == stacks - 1:
                tris.append((a, b, d))
            else:
                tris.append((a, b, c))
                tris.append((a, c, d))
    idx = np.array([[v[0] * slices + v[1] for v in t] for t in tris])
    Nf, Uf = N.reshape(-1, 3), U.reshape(-1, 2)
    return Nf[idx].reshape(-1, 9), Uf[idx].reshape(-1, 6)


def terrain_spheres(seed=0, tiles=64, cells_per_tile=8, spheres=512, slices=24, stacks=20, lights=32,
                    n_mats=64, extent=256.0, mixed_materials=False):
    rng = _rng(seed, 1)
    mats = []
    for k in range(n_mats):
        rough = float(rng.uniform(0.05, 1.0))
        alb = rng.uniform(0.1, 0.9, size=3).tolist()
        t = MAT_GGXR
        if mixed_materials:
            t = [MAT_GGXR, MAT_LAMBERT, MAT_GGX, MAT_GLASS, MAT_BLINNPHONG, MAT_GGXR][k % 6]
        m = dict(type=t, c0=alb, alpha=rough)
        if t == MAT_GGX:
            m.update(ior=1.5)
        if t == MAT_GLASS:
            m.update(ior=1.5, c0=[0.04, 0.04, 0.04])
        if t == MAT_BLINNPHONG:
            m.update(c1=[0.3, 0.3, 0.3], ns=float(rng.uniform(5, 80)))
        mats.append(m)
    pos, nrm, uv, mat, ground = _terrain(seed, tiles, cells_per_tile, extent, 12.0, 64.0, rng, n_mats)
    P, N, U, M = [pos], [nrm], [uv], [mat]
    lim = extent * 0.43
    unit_n, unit_uv = _unit_sphere(slices, stacks)
    for s in range(spheres):
        r = float(rng.uniform(0.5, 3.0))
        x, z = rng.uniform(-lim, lim, size=2)
        y = float(ground(x, z)) + 0.8 * r
        center = np.tile(np.array([x, y, z]), 3)
        P.append(center + r * unit_n), N.append(unit_n), U.append(unit_uv)
        M.append(np.full(unit_n.shape[0], rng.integers(0, n_mats)))
    for l in range(lights):
        size = float(rng.uniform(4.0, 10.0))
        x, z = rng.uniform(-lim, lim, size=2)
        y = float(rng.uniform(40.0, 60.0))
        radiance = float(rng.uniform(5.0, 20.0))
        tint = rng.uniform(0.5, 1.0, size=3) if rng.uniform() < 0.5 else np.ones(3)
        mats.append(dict(type=MAT_LIGHT, c0=(radiance * tint).tolist()))
        h = size / 2
        a, b, c, d = [np.array([x + sx, y, z + sz]) for sx, sz in ((-h, -h), (h, -h), (h, h), (-h, h))]
        down = np.array([0.0, -1.0, 0.0])
        for tri in ((a, b, c), (a, c, d)):  # normal (0,-1,0)
            P.append(np.concatenate(tri)[None])
            N.append(np.tile(down, 3)[None])
            U.append(np.zeros((1, 6)))
            M.append(np.array([len(mats) - 1]))
    return dict(pos=np.concatenate(P).astype(np.float32), nrm=np.concatenate(N).astype(np.float32),
                uv=np.concatenate(U).astype(np.float32), mat=np.concatenate(M).astype(np.int32), mats=mats,
                textures=[], env_tex=-1, env_gain=1.0, params=C2_PARAMS)


def sky(width=2048, height=1024, sun_dir=(0.3, 0.8, -0.5), peak=5e3, sharpness=2000.0):
    """HDR equirectangular sky in the layout of the reference's env lookup
    (u = atan2(z, x) / 2pi + 0.5, v = 1 - acos(y) / pi, row 0 at v = 1)."""
    v = 1.0 - (np.arange(height) + 0.5) / height
    u = (np.arange(width) + 0.5) / width
    V, Uu = np.meshgrid(v, u, indexing="ij")
    theta = (1.0 - V) * np.pi
    phi = (Uu - 0.5) * 2 * np.pi
    d = np.stack([np.sin(theta) * np.cos(phi), np.cos(theta), np.sin(theta) * np.sin(phi)], -1)
    s = np.array(sun_dir) / np.linalg.norm(sun_dir)
    grad = np.clip(d[..., 1], 0, 1)[..., None] * np.array([0.25, 0.45, 0.9]) + 0.05
    lobe = peak * np.exp(-sharpness * (1.0 - d @ s))[..., None] * np.array([1.0, 0.95, 0.85])
    return (grad + lobe).astype(np.float32)


def value_noise_texture(seed, size=512, cells=16):
    lattice = _rng(seed, 11).uniform(0.0, 1.0, size=(cells, cells, 3))
    x = (np.arange(size) + 0.5) / size * cells
    X, Z = np.meshgrid(x, x, indexing="ij")
    out = np.stack([_value_noise(X, Z, lattice[..., k]) for k in range(3)], -1)
    return (0.1 + 0.8 * out).astype(np.float32)


def with_env_textures(scene, seed=0, tex_size=512, env_size=(2048, 1024), dielectric_frac=0.1, spp=256):
    rng = _rng(seed, 3)
    s = dict(scene)
    mats = [dict(m) for m in scene["mats"]]
    textures = []
    surf = [i for i, m in enumerate(mats) if m["type"] != MAT_LIGHT]
    n_die = max(1, int(round(dielectric_frac * len(surf))))
    for i in rng.choice(surf, size=n_die, replace=False):
        mats[i].update(type=MAT_GGX, ior=1.5)
    for k, i in enumerate(surf[::2]):
        textures.append(value_noise_texture(seed * 1000 + k, tex_size))
        mats[i]["tex0"] = len(textures) - 1
    textures.append(sky(*env_size))
    s.update(mats=mats, textures=textures, env_tex=len(textures) - 1, env_gain=1.0,
             params=scene["params"].replace("spp=64", f"spp={spp}"))
    return s


def small_scene(seed=1, mixed=True, env=True, textures=True):
    """A few thousand triangles with every material type, for parity tests."""
    sc = terrain_spheres(seed, tiles=8, cells_per_tile=2, spheres=10, slices=10, stacks=7, lights=4, n_mats=12,
                         extent=40.0, mixed_materials=mixed)
    if env or textures:
        sc = with_env_textures(sc, seed, tex_size=32, env_size=(64, 32), dielectric_frac=0.0)
        if not env:
            sc["textures"] = sc["textures"][:-1]
            sc["env_tex"] = -1
        if not textures:
            for m in sc["mats"]:
                m.pop("tex0", None)
            sc["textures"] = sc["textures"][-1:]
            sc["env_tex"] = 0 if env else -1
    sc["params"] = "renderer=ptnee imgw=48 imgh=32 spp=4 campos=0,14,34 cameuler=0,-20,0 camfov=50 camasp=1.5"
    return sc


def _fmt_rows(tag, rows):
    # %.9g identifies a float32 exactly; the loaders parse through double
    # (atof) or float (operator>>) and both round back to the same value
    return "".join(f"{tag} {' '.join(format(float(x), '.9g') for x in r)}\n" for r in rows)


def _unique_rows(a):
    """Distinct rows by exact bit pattern (keeps -0.0 apart from 0.0), first
    occurrence order, and each input row's 1-based index among them."""
    bits = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)
    _, first, inv = np.unique(bits, axis=0, return_index=True, return_inverse=True)
    rank = np.empty(len(first), np.int64)
    order = np.argsort(first)
    rank[order] = np.arange(len(first))
    return a[first[order]], rank[inv.reshape(-1)] + 1


def write_scene(sc, directory, stem="scene"):
    """Writes a scene dict as files the reference Loader reads
    (Loader::fromSceneDescription, src/scene/loader.cpp:26-105): one OBJ
    per material (v / vt / vn and f v/vt/vn triplets, loader.cpp:270-330), a
    multi-line scene description forcing each file's material with the
    loader's flags (-m=light Ke, -m=ggxr Kd alpha, -m=ggx Kd alpha ior,
    -m=glass F0 ior) or, for Lambert and BlinnPhong, an MTL file
    (loader.cpp:108-229: Kd, Ks, Ns), and the camera parameters beside it.

    Returns (desc_text, order): the loader appends triangles file by file,
    so the loaded scene holds triangle order[i] of sc at position i, and
    its emitters, tree and hits are those of the arrays permuted by order.
    Textured materials and environment maps are not expressible in a scene
    description (the reference sets them through its classes' public
    fields and the envmap parameter) and are refused."""
    import os
    directory = os.path.abspath(directory)
    if any(c.isspace() for c in directory + stem):
        raise ValueError("the scene description grammar splits on whitespace: use a path without spaces")
    mats = sc["mats"]
    if any(m.get("tex0", -1) >= 0 for m in mats):
        raise ValueError("textured materials cannot be written as a scene description")
    os.makedirs(directory, exist_ok=True)
    mat = np.asarray(sc["mat"])
    n = mat.shape[0]
    pos = np.asarray(sc["pos"], np.float32).reshape(n, 3, 3)
    uv = np.asarray(sc.get("uv") if sc.get("uv") is not None else np.zeros((n, 6)), np.float32).reshape(n, 3, 2)
    nrm = np.asarray(sc.get("nrm") if sc.get("nrm") is not None else np.zeros((n, 9)), np.float32).reshape(n, 3, 3)
    order = np.argsort(mat, kind="stable")
    lines = []
    for k in np.unique(mat):
        idx = order[mat[order] == k]
        m = mats[int(k)]
        t = m["type"]
        name = f"{stem}_m{int(k)}"
        obj = os.path.join(directory, name + ".obj")
        v, vi = _unique_rows(pos[idx].reshape(-1, 3))
        vt, ti = _unique_rows(uv[idx].reshape(-1, 2))
        vn, ni = _unique_rows(nrm[idx].reshape(-1, 3))
        head = ""
        # material values as the float32 the arrays path would store
        f32 = lambda x: format(float(np.float32(x)), ".9g")  # noqa: E731
        c0 = " ".join(f32(x) for x in m.get("c0", (0, 0, 0)))
        fl = lambda key, d: f32(m.get(key, d))  # noqa: E731
        if t == MAT_LIGHT:
            desc = f"{obj} -m=light {c0}"
        elif t == MAT_GGXR:
            desc = f"{obj} -m=ggxr {c0} {fl('alpha', 0.5)}"
        elif t == MAT_GGX:
            desc = f"{obj} -m=ggx {c0} {fl('alpha', 0.5)} {fl('ior', 1.0)}"
        elif t == MAT_GLASS:
            desc = f"{obj} -m=glass {c0} {fl('ior', 0.0)}"
        elif t in (MAT_LAMBERT, MAT_BLINNPHONG):
            mtl = f"newmtl m\nNs {fl('ns', 10.0)}\nKd {c0}\n"
            if t == MAT_BLINNPHONG:
                ks = m.get("c1", (0, 0, 0))
                if float(np.dot(ks, ks)) <= 1e-6:
                    raise ValueError(f"material {int(k)}: BlinnPhong needs |Ks|^2 > 1e-6 to load as BlinnPhong")
                mtl += "Ks " + " ".join(f32(x) for x in ks) + "\n"
            with open(os.path.join(directory, name + ".mtl"), "w") as f:
                f.write(mtl)
            head = f"mtllib {name}.mtl\nusemtl m\n"
            desc = obj
        else:
            raise ValueError(f"material {int(k)}: unknown type {t}")
        face = np.stack([vi, ti, ni], -1).reshape(-1, 3, 3)
        body = "".join(f"f {a[0]}/{a[1]}/{a[2]} {b[0]}/{b[1]}/{b[2]} {c[0]}/{c[1]}/{c[2]}\n" for a, b, c in face)
        with open(obj, "w") as f:
            f.write(head + _fmt_rows("v", v) + _fmt_rows("vt", vt) + _fmt_rows("vn", vn) + body)
        lines.append(desc)
    text = "\n".join(lines) + "\n"
    with open(os.path.join(directory, stem + ".desc"), "w") as f:
        f.write(text)
    if sc.get("params"):
        with open(os.path.join(directory, stem + ".params"), "w") as f:
            f.write(sc["params"] + "\n")
    return text, order


def main(argv=None):
    """python -m nuray_gb300.scenes DIR [--seed S] [--small]: writes the
    1M-triangle scene (or the small parity scene without textures and
    environment) with write_scene, for the reference's Loader or nr_scene_load."""
    import argparse
    ap = argparse.ArgumentParser(prog="python -m nuray_gb300.scenes")
    ap.add_argument("directory")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--small", action="store_true")
    a = ap.parse_args(argv)
    sc = small_scene(a.seed, env=False, textures=False) if a.small else terrain_spheres(a.seed)
    text, _ = write_scene(sc, a.directory)
    print(f"{sc['pos'].shape[0]} triangles, {len(text.splitlines())} files; parameters in scene.params")


if __name__ == "__main__":
    main()
