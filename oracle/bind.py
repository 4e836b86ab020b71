"""ctypes access to the oracles. TEST INFRASTRUCTURE.

* Port: oracle/_build/libnuray_port.so, the project's CPU restatement of
  the reference ptnee (oracle/port/), built by `make -C oracle port`.
* Reference: oracle/_ref/libnuray_ref.so, the reference's own sources
  compiled with oracle/Makefile (only where the reference checkout exists).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libnuray_port.so")
REF_LIB = os.path.join(HERE, "_ref", "libnuray_ref.so")

_vp, _i32, _cp, _f32, _u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_float, ctypes.c_uint64
_SIG = {
    "scene_create": ([_i32, _vp, _vp, _vp, _vp, _i32, _vp, _vp, _i32, _vp, _vp, _i32, _f32, _i32], _vp),
    "scene_destroy": ([_vp], None),
    "bvh_export": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp], _i32),
    "intersect": ([_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _i32], None),
    "camera_rays": ([_cp, _i32, _vp, _vp, _vp, _vp], None),
    "render_samples": ([_vp, _cp, _i32, _vp, _i32, _i32, _u64, _vp, _i32, _vp], None),
    "material_probe": ([_vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], None),
    "light_pick": ([_vp, _i32, _vp, _vp], _f32),
    "texture_lookup": ([_vp, _i32, _i32, _i32, _vp, _vp], None),
}


def build_port():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


# Where the reference checkout lies (only the fixture script, the tests that
# pin the oracle and build() read it; the GPU host has none).
REF_ROOT = os.environ.get("NURAY_REF_ROOT", "/root/reference")
REF_RENDER_LIB = os.path.join(HERE, "_ref", "libnuray_ref_render.so")


def build_ref(ref_root=None):
    """Compiles the reference sources (both oracle libraries); returns the
    library path or None."""
    ref_root = ref_root or REF_ROOT
    if not os.path.isdir(os.path.join(ref_root, "src", "renderer")):
        return None
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", "ref-render", f"REF={ref_root}"], check=True)
    return REF_LIB


def ref_render_image(scene, params, seed=0):
    """The reference's RendererPTLS::render of the whole frame, 8-bit RGB
    (h, w, 3), on the Philox stream (oracle/ref_render.cpp)."""
    L = ctypes.CDLL(REF_RENDER_LIB)
    L.ref_scene_from_arrays.restype = _vp
    L.ref_scene_from_arrays.argtypes = _SIG["scene_create"][0][:13]
    L.ref_scene_destroy.argtypes = [_vp]
    L.ref_render_image.argtypes = [_vp, _cp, _u64, _vp]
    L.ref_render_image.restype = _i32
    pos = np.ascontiguousarray(scene["pos"], np.float32)
    n = pos.shape[0]
    uv = np.ascontiguousarray(scene.get("uv") if scene.get("uv") is not None else np.zeros((n, 6)), np.float32)
    nrm = np.ascontiguousarray(scene.get("nrm") if scene.get("nrm") is not None else np.zeros((n, 9)), np.float32)
    mat = np.ascontiguousarray(scene["mat"], np.int32)
    mi, mf = _mat_arrays(scene["mats"])
    h = L.ref_scene_from_arrays(n, _ptr(pos), _ptr(uv), _ptr(nrm), _ptr(mat), len(scene["mats"]), _ptr(mi), _ptr(mf),
                                0, None, None, -1, 1.0)
    cfg = dict(kv.split("=", 1) for kv in params.split() if "=" in kv)
    w, hh = int(cfg.get("imgw", 1)), int(cfg.get("imgh", 1))
    out = np.zeros((hh, w, 3), np.uint8)
    try:
        if L.ref_render_image(h, params.encode(), seed, _ptr(out)) != 0:
            raise RuntimeError("the reference's render() did not finish")
    finally:
        L.ref_scene_destroy(h)
    return out


def _ptr(a):
    return None if a is None else a.ctypes.data


def _mat_arrays(mats):
    mi = np.full((max(1, len(mats)), 4), -1, np.int32)
    mf = np.zeros((max(1, len(mats)), 12), np.float32)
    for i, m in enumerate(mats):
        mi[i, 0] = m["type"]
        mi[i, 1] = m.get("tex0", -1)
        mi[i, 2] = m.get("tex1", -1)
        mf[i, 0:3] = m.get("c0", (0, 0, 0))
        mf[i, 3:6] = m.get("c1", (0, 0, 0))
        mf[i, 6] = m.get("alpha", 0.5)
        mf[i, 7] = m.get("ior", 1.0)
        mf[i, 8] = m.get("ns", 10.0)
    return mi, mf


class Oracle:
    """One scene in one oracle library ('port' or 'ref')."""

    def __init__(self, kind, scene=None, desc=None):
        path = PORT_LIB if kind == "port" else REF_LIB
        if kind == "port" and not os.path.exists(path):
            build_port()
        self.L = ctypes.CDLL(path)
        self.pre = "port_" if kind == "port" else "ref_"
        for name, (args, res) in _SIG.items():
            if name == "scene_create":
                continue
            f = getattr(self.L, self.pre + name)
            f.argtypes, f.restype = args, res
        self.kind = kind
        if desc is not None:
            if kind != "ref":
                raise ValueError("scene descriptions load through the reference Loader only")
            self.L.ref_scene_from_desc.restype = _vp
            self.L.ref_scene_from_desc.argtypes = [_cp]
            self.h = self.L.ref_scene_from_desc(desc.encode())
        else:
            pos = np.ascontiguousarray(scene["pos"], np.float32)
            n = pos.shape[0]
            uv = np.ascontiguousarray(scene.get("uv") if scene.get("uv") is not None else np.zeros((n, 6)), np.float32)
            nrm = np.ascontiguousarray(scene.get("nrm") if scene.get("nrm") is not None else np.zeros((n, 9)), np.float32)
            mat = np.ascontiguousarray(scene["mat"], np.int32)
            mi, mf = _mat_arrays(scene["mats"])
            tex = scene.get("textures", [])
            wh = np.array([(t.shape[1], t.shape[0]) for t in tex], np.int32).reshape(-1) if tex else np.zeros(2, np.int32)
            td = np.concatenate([np.ascontiguousarray(t, np.float32).ravel() for t in tex]) if tex else np.zeros(3, np.float32)
            create = getattr(self.L, self.pre + ("scene_create" if kind == "port" else "scene_from_arrays"))
            create.argtypes, create.restype = _SIG["scene_create"][0][:13] + ([_i32] if kind == "port" else []), _vp
            args = [n, _ptr(pos), _ptr(uv), _ptr(nrm), _ptr(mat), len(scene["mats"]), _ptr(mi), _ptr(mf), len(tex),
                    _ptr(wh), _ptr(td), scene.get("env_tex", -1), scene.get("env_gain", 1.0)]
            if kind == "port":
                args.append(os.cpu_count() or 1)
            self.h = create(*args)
        if not self.h:
            raise RuntimeError("oracle scene creation failed")

    def close(self):
        if getattr(self, "h", None):
            getattr(self.L, self.pre + "scene_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_materials(self, mats):
        """Port only: new material parameters (same count and types), the
        BVH and the emitter table kept."""
        if self.kind != "port":
            raise ValueError("set_materials is a port entry point")
        mi, mf = _mat_arrays(mats)
        f = self.L.port_scene_set_materials
        f.argtypes, f.restype = [_vp, _i32, _vp, _vp], _i32
        if f(self.h, len(mats), _ptr(mi), _ptr(mf)) != 0:
            raise ValueError("material count or types differ from the scene's")

    def bvh(self):
        f = getattr(self.L, self.pre + "bvh_export")
        nt = ctypes.c_int()
        nn = f(self.h, None, None, None, None, None, ctypes.byref(nt))
        box = np.zeros((nn, 6), np.float32)
        kids = np.zeros((nn, 2), np.int32)
        first = np.zeros(nn, np.int32)
        count = np.zeros(nn, np.int32)
        tris = np.zeros(nt.value, np.int32)
        f(self.h, _ptr(box), _ptr(kids), _ptr(first), _ptr(count), _ptr(tris), ctypes.byref(nt))
        return box, kids, first, count, tris

    def intersect(self, o, d, threads=None):
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        n = o.shape[0]
        tri = np.zeros(n, np.int32)
        t, b1, b2 = (np.zeros(n, np.float32) for _ in range(3))
        getattr(self.L, self.pre + "intersect")(self.h, n, _ptr(o), _ptr(d), _ptr(tri), _ptr(t), _ptr(b1), _ptr(b2),
                                                threads or os.cpu_count() or 1)
        return tri, t, b1, b2

    def camera_rays(self, params, fx, fy):
        fx = np.ascontiguousarray(fx, np.float32)
        fy = np.ascontiguousarray(fy, np.float32)
        d = np.zeros((fx.size, 3), np.float32)
        o = np.zeros((fx.size, 3), np.float32)
        getattr(self.L, self.pre + "camera_rays")(params.encode(), fx.size, _ptr(fx), _ptr(fy), _ptr(d), _ptr(o))
        return o, d

    def render_samples(self, params, pix_xy, spp, sample0=0, seed=0, threads=None, counters=False):
        pix = np.ascontiguousarray(pix_xy, np.int32).reshape(-1, 2)
        out = np.zeros((pix.shape[0], spp, 3), np.float32)
        f = getattr(self.L, self.pre + "render_samples")
        args = [self.h, params.encode(), pix.shape[0], _ptr(pix), sample0, spp, seed, _ptr(out),
                threads or os.cpu_count() or 1]
        cnt = np.zeros(3, np.uint64)
        if self.kind == "port":
            args.append(_ptr(cnt) if counters else None)
        else:
            f.argtypes = f.argtypes[:9]
        f(*args)
        return (out, dict(rays=int(cnt[0]), shadow_rays=int(cnt[1]), vertices=int(cnt[2]))) if counters else out

    def material_probe(self, mat, wo, nrm, wi, uv, u):
        arrs = [np.ascontiguousarray(x, np.float32) for x in (wo, nrm, wi, uv, u)]
        n = arrs[0].shape[0]
        f = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        ws = np.zeros((n, 3), np.float32)
        getattr(self.L, self.pre + "material_probe")(self.h, mat, n, *[_ptr(a) for a in arrs], _ptr(f), _ptr(pdf),
                                                     _ptr(ws))
        return f, pdf, ws

    def light_pick(self, u):
        u = np.ascontiguousarray(u, np.float32)
        tri = np.zeros(u.size, np.int32)
        p = getattr(self.L, self.pre + "light_pick")(self.h, u.size, _ptr(u), _ptr(tri))
        return tri, p

    def texture_lookup(self, mat, kind, uvs):
        uvs = np.ascontiguousarray(uvs, np.float32).reshape(-1, 2)
        rgb = np.zeros((uvs.shape[0], 3), np.float32)
        getattr(self.L, self.pre + "texture_lookup")(self.h, mat, kind, uvs.shape[0], _ptr(uvs), _ptr(rgb))
        return rgb


def pixel_grid(w, h):
    ys, xs = np.mgrid[0:h, 0:w]
    return np.stack([xs.ravel(), ys.ravel()], 1).astype(np.int32)
