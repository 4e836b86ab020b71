"""ctypes binding of libnuray_gpu.so (include/nuray.h).

Loading fails loudly when the library has not been built: there is no
fallback implementation behind this module.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnuray_gpu.so")

NR_OK = 0
ERRORS = {-1: "NR_ERR_INVALID", -2: "NR_ERR_CUDA", -3: "NR_ERR_OOM", -4: "NR_ERR_CANCELLED", -5: "NR_ERR_IO",
          -6: "NR_ERR_DEVICE"}
NR_PTR_DEVICE = 1
NR_INTERSECT_EXHAUSTIVE = 2

MAT_LAMBERT, MAT_GGXR, MAT_GGX, MAT_GLASS, MAT_BLINNPHONG, MAT_LIGHT = range(6)


class NuRayError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Material(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("tex0", ctypes.c_int32), ("tex1", ctypes.c_int32),
                ("reserved0", ctypes.c_int32), ("c0", ctypes.c_float * 3), ("c1", ctypes.c_float * 3),
                ("alpha", ctypes.c_float), ("ior", ctypes.c_float), ("ns", ctypes.c_float),
                ("reserved1", ctypes.c_float * 3)]


class SceneDesc(ctypes.Structure):
    _fields_ = [("num_tris", ctypes.c_int32), ("pos", ctypes.c_void_p), ("uv", ctypes.c_void_p),
                ("nrm", ctypes.c_void_p), ("mat", ctypes.c_void_p), ("num_mats", ctypes.c_int32),
                ("mats", ctypes.c_void_p), ("num_tex", ctypes.c_int32), ("tex_wh", ctypes.c_void_p),
                ("tex_data", ctypes.c_void_p), ("env_tex", ctypes.c_int32), ("env_gain", ctypes.c_float)]


class Camera(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_float * 3), ("gaze", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov", ctypes.c_float), ("aspect", ctypes.c_float)]


class BvhDesc(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_int32), ("box", ctypes.c_void_p), ("kids", ctypes.c_void_p),
                ("leaf_first", ctypes.c_void_p), ("leaf_count", ctypes.c_void_p), ("leaf_tris", ctypes.c_void_p)]


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("paths", "rays", "shadow_rays", "waves", "bounces", "kernel_launches",
                                                "trace_launches", "nodes_visited", "tris_tested",
                                                "shadow_nodes_visited", "shadow_tris_tested")] + \
               [(k, ctypes.c_double) for k in ("kernel_ms_trace", "kernel_ms_shadow", "kernel_ms_shade",
                                                "kernel_ms_other", "wall_ms")]


# name -> argtypes, all returning int
_vp, _i32, _cp = ctypes.c_void_p, ctypes.c_int32, ctypes.c_char_p
SIGNATURES = {
    "nr_last_error": [_cp, ctypes.c_size_t],
    "nr_scene_create": [_vp, _vp],
    "nr_scene_load": [_cp, _vp],
    "nr_scene_create_opts": [_vp, _cp, _vp],
    "nr_scene_load_opts": [_cp, _cp, _vp],
    "nr_scene_build_times": [_vp, _vp, _vp],
    "nr_scene_destroy": [_vp],
    "nr_scene_set_env": [_vp, _i32, _i32, _vp, ctypes.c_float],
    "nr_scene_info": [_vp, _vp],
    "nr_scene_export": [_vp, _vp, _vp, _vp, _vp, _vp],
    "nr_bvh_export": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "nr_scene_create_bvh": [_vp, _vp, _cp, _vp],
    "nr_intersect": [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _i32],
    "nr_camera_from_params": [_cp, _vp],
    "nr_render": [_vp, _vp, _cp, _vp, _vp, _vp, _vp, _vp],
    "nr_render_samples": [_vp, _vp, _cp, _i32, _vp, _i32, _i32, _vp],
    "nr_get_stats": [_vp, _vp],
    "nr_material_probe": [_vp, _i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "nr_scene_stream": [_vp, _vp],
    "nr_nrc_create": [_cp, _vp],
    "nr_nrc_destroy": [_vp],
    "nr_nrc_num_params": [_vp],
    "nr_nrc_get_params": [_vp, _vp],
    "nr_nrc_set_params": [_vp, _vp],
    "nr_nrc_infer": [_vp, _i32, _vp, _vp],
    "nr_nrc_gradient": [_vp, _i32, _vp, _vp, _vp, _vp],
    "nr_nrc_train_step": [_vp, _i32, _vp, _vp, _vp],
    "nr_scene_attach_nrc": [_vp, _vp],
    "nr_scene_set_materials": [_vp, _i32, _vp],
    "nr_adjoint": [_vp, _vp, _cp, _vp, _vp, _vp],
    "nr_intersect_noalloc": [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp],
    "nr_nrc_get_state": [_vp, _i32, _vp],
    "nr_nrc_set_state": [_vp, _i32, _vp],
}

_lib = None


def lib():
    """Loads libnuray_gpu.so once; raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m nuray_gb300.build` "
                              "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = ctypes.c_int
        _lib = L
    return _lib


def check(code):
    if code != NR_OK:
        buf = ctypes.create_string_buffer(1024)
        lib().nr_last_error(buf, len(buf))
        raise NuRayError(code, buf.value.decode(errors="replace"))
    return code


def _ptr(a):
    return None if a is None else a.ctypes.data


class Scene:
    """A scene on the GPU (nr_scene)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)

    @classmethod
    def from_text(cls, desc, options=""):
        h = ctypes.c_void_p()
        check(lib().nr_scene_load_opts(desc.encode(), options.encode(), ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def from_arrays(cls, pos, mat, mats, uv=None, nrm=None, textures=(), env_tex=-1, env_gain=1.0, options="",
                    bvh=None):
        """pos (n,9) float32, mat (n,) int32, mats: list of dicts / Material,
        textures: list of (h, w, 3) float32 arrays (row 0 at v = 1); bvh: a
        tree (box, kids, first, count, tris) as Scene.bvh() returns it, used
        instead of a build (nr_scene_create_bvh)."""
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 9)
        n = pos.shape[0]
        mat = np.ascontiguousarray(mat, np.int32).reshape(n)
        uv = None if uv is None else np.ascontiguousarray(uv, np.float32).reshape(n, 6)
        nrm = None if nrm is None else np.ascontiguousarray(nrm, np.float32).reshape(n, 9)
        mt = (Material * max(1, len(mats)))()
        for i, m in enumerate(mats):
            mt[i] = m if isinstance(m, Material) else make_material(**m)
        wh = np.array([(t.shape[1], t.shape[0]) for t in textures], np.int32).reshape(-1)
        td = (np.concatenate([np.ascontiguousarray(t, np.float32).reshape(-1) for t in textures])
              if textures else np.zeros(1, np.float32))
        d = SceneDesc(n, _ptr(pos), _ptr(uv), _ptr(nrm), _ptr(mat), len(mats), ctypes.addressof(mt), len(textures),
                      _ptr(wh) if len(textures) else None, _ptr(td) if len(textures) else None, env_tex, env_gain)
        h = ctypes.c_void_p()
        if bvh is None:
            check(lib().nr_scene_create_opts(ctypes.byref(d), options.encode(), ctypes.byref(h)))
        else:
            box, kids, first, count, tris = (np.ascontiguousarray(a, t) for a, t in
                                             zip(bvh, (np.float32, np.int32, np.int32, np.int32, np.int32)))
            tree = BvhDesc(len(kids), _ptr(box), _ptr(kids), _ptr(first), _ptr(count), _ptr(tris))
            check(lib().nr_scene_create_bvh(ctypes.byref(d), ctypes.byref(tree), options.encode(), ctypes.byref(h)))
        return cls(h.value)

    def build_times(self):
        """(wall ms, device ms) of the scene's BVH build."""
        w, d = ctypes.c_double(), ctypes.c_double()
        check(lib().nr_scene_build_times(self._h, ctypes.byref(w), ctypes.byref(d)))
        return w.value, d.value

    def close(self):
        if self._h:
            check(lib().nr_scene_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_env(self, rgb, gain=1.0):
        """Attaches an environment map ((h, w, 3) float32, row 0 at v = 1); None removes it."""
        if rgb is None:
            check(lib().nr_scene_set_env(self._h, 0, 0, None, gain))
            return
        rgb = np.ascontiguousarray(rgb, np.float32)
        check(lib().nr_scene_set_env(self._h, rgb.shape[1], rgb.shape[0], _ptr(rgb), gain))

    def info(self):
        a = np.zeros(6, np.int64)
        check(lib().nr_scene_info(self._h, _ptr(a)))
        return dict(tris=int(a[0]), mats=int(a[1]), nodes=int(a[2]), depth=int(a[3]), lights=int(a[4]),
                    device_bytes=int(a[5]))

    def export(self):
        info = self.info()
        n, m = info["tris"], info["mats"]
        pos = np.zeros((n, 9), np.float32)
        uv = np.zeros((n, 6), np.float32)
        nrm = np.zeros((n, 9), np.float32)
        mat = np.zeros(n, np.int32)
        mats = (Material * max(1, m))()
        check(lib().nr_scene_export(self._h, _ptr(pos), _ptr(uv), _ptr(nrm), _ptr(mat), ctypes.addressof(mats)))
        return pos, uv, nrm, mat, [mats[i] for i in range(m)]

    def bvh(self):
        nn, nt = ctypes.c_int32(), ctypes.c_int32()
        check(lib().nr_bvh_export(self._h, None, None, None, None, None, ctypes.byref(nn), ctypes.byref(nt)))
        box = np.zeros((nn.value, 6), np.float32)
        kids = np.zeros((nn.value, 2), np.int32)
        first = np.zeros(nn.value, np.int32)
        count = np.zeros(nn.value, np.int32)
        tris = np.zeros(nt.value, np.int32)
        check(lib().nr_bvh_export(self._h, _ptr(box), _ptr(kids), _ptr(first), _ptr(count), _ptr(tris),
                                  ctypes.byref(nn), ctypes.byref(nt)))
        return box, kids, first, count, tris

    def intersect(self, o, d, exhaustive=False):
        """Closest hits (tri, t, b1, b2); exhaustive: visit every node whose
        box the ray enters, as the reference does (NR_INTERSECT_EXHAUSTIVE)."""
        o = np.ascontiguousarray(o, np.float32).reshape(-1, 3)
        d = np.ascontiguousarray(d, np.float32).reshape(-1, 3)
        n = o.shape[0]
        tri = np.zeros(n, np.int32)
        t, b1, b2 = (np.zeros(n, np.float32) for _ in range(3))
        check(lib().nr_intersect(self._h, n, _ptr(o), _ptr(d), _ptr(tri), _ptr(t), _ptr(b1), _ptr(b2),
                                 NR_INTERSECT_EXHAUSTIVE if exhaustive else 0))
        return tri, t, b1, b2

    def intersect_device(self, n, o_ptr, d_ptr, tri_ptr, t_ptr, b1_ptr, b2_ptr):
        check(lib().nr_intersect(self._h, n, o_ptr, d_ptr, tri_ptr, t_ptr, b1_ptr, b2_ptr, NR_PTR_DEVICE))

    def render(self, params, camera=None, want_rgb8=False, cancel=None, progress=None):
        cfg = parse_params(params)
        w, h = int(cfg.get("imgw", 1)), int(cfg.get("imgh", 1))
        hdr = np.zeros((h, w, 3), np.float32)
        rgb8 = np.zeros((h, w, 3), np.uint8) if want_rgb8 else None
        cam = ctypes.byref(camera) if camera is not None else None
        cb = None
        if progress is not None:
            CB = ctypes.CFUNCTYPE(None, ctypes.c_float, ctypes.c_void_p)
            cb = CB(lambda pct, user: progress(pct))
        check(lib().nr_render(self._h, cam, params.encode(), _ptr(hdr), _ptr(rgb8),
                              None if cancel is None else ctypes.addressof(cancel),
                              ctypes.cast(cb, ctypes.c_void_p) if cb is not None else None, None))
        return (hdr, rgb8) if want_rgb8 else hdr

    def render_device(self, params, camera=None):
        """Renders and keeps the image on the device (no host copy)."""
        cam = ctypes.byref(camera) if camera is not None else None
        check(lib().nr_render(self._h, cam, params.encode(), None, None, None, None, None))

    def render_samples(self, params, pix_xy, spp, sample0=0, camera=None):
        pix = np.ascontiguousarray(pix_xy, np.int32).reshape(-1, 2)
        out = np.zeros((pix.shape[0], spp, 3), np.float32)
        cam = ctypes.byref(camera) if camera is not None else None
        check(lib().nr_render_samples(self._h, cam, params.encode(), pix.shape[0], _ptr(pix), sample0, spp, _ptr(out)))
        return out

    def set_materials(self, mats):
        mt = (Material * len(mats))()
        for i, m in enumerate(mats):
            mt[i] = m if isinstance(m, Material) else make_material(**m)
        check(lib().nr_scene_set_materials(self._h, len(mats), ctypes.addressof(mt)))

    def adjoint(self, params, dl_dimage, camera=None, want_image=False):
        """d loss / d (albedo rgb, roughness, emission rgb) per material, shape (num_mats, 7)."""
        d = np.ascontiguousarray(dl_dimage, np.float32)
        n = self.info()["mats"]
        g = np.zeros((n, 7), np.float32)
        img = np.zeros(d.shape, np.float32) if want_image else None
        cam = ctypes.byref(camera) if camera is not None else None
        check(lib().nr_adjoint(self._h, cam, params.encode(), _ptr(d), _ptr(g), _ptr(img)))
        return (g, img) if want_image else g

    def stream(self):
        p = ctypes.c_void_p()
        check(lib().nr_scene_stream(self._h, ctypes.byref(p)))
        return p.value

    def stats(self):
        s = Stats()
        check(lib().nr_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def material_probe(self, mat, wo, nrm, wi, uv, u):
        arrs = [np.ascontiguousarray(x, np.float32) for x in (wo, nrm, wi, uv, u)]
        n = arrs[0].shape[0]
        f = np.zeros((n, 3), np.float32)
        pdf = np.zeros(n, np.float32)
        ws = np.zeros((n, 3), np.float32)
        check(lib().nr_material_probe(self._h, mat, n, *[_ptr(a) for a in arrs], _ptr(f), _ptr(pdf), _ptr(ws)))
        return f, pdf, ws


def make_material(type, c0=(0, 0, 0), c1=(0, 0, 0), alpha=0.5, ior=1.0, ns=10.0, tex0=-1, tex1=-1):
    m = Material()
    m.type, m.tex0, m.tex1 = type, tex0, tex1
    m.c0[:] = list(map(float, c0))
    m.c1[:] = list(map(float, c1))
    m.alpha, m.ior, m.ns = alpha, ior, ns
    return m


def camera_from_params(params):
    c = Camera()
    check(lib().nr_camera_from_params(params.encode(), ctypes.byref(c)))
    return c


def parse_params(params):
    """The reference's key=value grammar (src/utils/config.cpp:90-97)."""
    out = {}
    for kv in params.split():
        k, _, v = kv.partition("=")
        out[k] = v if _ else kv
    return out
