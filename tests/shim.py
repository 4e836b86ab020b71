"""Builds and binds tests/host_shim.cpp (product host code, no CUDA)."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "tests", "_build")
LIB = os.path.join(OUT, "libhost_shim.so")
CSRC = os.path.join(ROOT, "nuray_gb300", "csrc")


def load():
    srcs = [os.path.join(ROOT, "tests", "host_shim.cpp"), os.path.join(CSRC, "host_scene.cpp"),
            os.path.join(CSRC, "image_io.cpp"), os.path.join(CSRC, "jpeg.cpp")]
    deps = srcs + [os.path.join(CSRC, "host_scene.h"), os.path.join(CSRC, "image_io.h"),
                   os.path.join(ROOT, "include", "nuray.h")]
    if not os.path.exists(LIB) or any(os.path.getmtime(p) > os.path.getmtime(LIB) for p in deps):
        os.makedirs(OUT, exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared", "-I", CSRC, "-I",
                        os.path.join(ROOT, "include"), *srcs, "-o", LIB, "-lpthread"], check=True)
    L = ctypes.CDLL(LIB)
    vp = ctypes.c_void_p
    L.shim_bvh.argtypes = [ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int, ctypes.c_int]
    L.shim_load.argtypes = [ctypes.c_char_p, vp, vp, vp, vp, vp, vp, ctypes.c_char_p, ctypes.c_int]
    L.shim_config_int.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
    L.shim_config_float.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_float]
    L.shim_config_float.restype = ctypes.c_float
    L.shim_config_vec3.argtypes = [ctypes.c_char_p, ctypes.c_char_p, vp]
    L.shim_camera.argtypes = [ctypes.c_char_p, vp, vp]
    L.shim_png_decode.argtypes = [ctypes.c_char_p, ctypes.c_long, vp, vp, vp, ctypes.c_char_p, ctypes.c_int]
    L.shim_jpeg_decode.argtypes = [ctypes.c_char_p, ctypes.c_long, vp, vp, vp, ctypes.c_char_p, ctypes.c_int]
    L.shim_png_encode.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp]
    L.shim_png_encode.restype = ctypes.c_long
    L.shim_read_image.argtypes = [ctypes.c_char_p, vp, vp, vp, ctypes.c_char_p, ctypes.c_int]
    L.shim_check_tree.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
    L.shim_bvh_from_arrays.argtypes = [ctypes.c_int, vp, ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_int, vp,
                                       ctypes.c_char_p, ctypes.c_int]
    return L


def png_decode(L, data):
    """PNG bytes -> (h, w, 4) uint8 through the product decoder; raises ValueError."""
    w, h = ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    if L.shim_png_decode(data, len(data), ctypes.byref(w), ctypes.byref(h), None, err, 256) != 0:
        raise ValueError(err.value.decode())
    out = np.zeros((h.value, w.value, 4), np.uint8)
    L.shim_png_decode(data, len(data), ctypes.byref(w), ctypes.byref(h), out.ctypes.data, err, 256)
    return out


def jpeg_decode(L, data):
    """JPEG bytes -> (h, w, 3) uint8 through the product decoder; raises ValueError."""
    w, h = ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    if L.shim_jpeg_decode(data, len(data), ctypes.byref(w), ctypes.byref(h), None, err, 256) != 0:
        raise ValueError(err.value.decode())
    out = np.zeros((h.value, w.value, 3), np.uint8)
    L.shim_jpeg_decode(data, len(data), ctypes.byref(w), ctypes.byref(h), out.ctypes.data, err, 256)
    return out


def png_encode(L, rgb):
    rgb = np.ascontiguousarray(rgb, np.uint8)
    h, w = rgb.shape[:2]
    n = L.shim_png_encode(rgb.ctypes.data, w, h, None)
    out = np.zeros(n, np.uint8)
    L.shim_png_encode(rgb.ctypes.data, w, h, out.ctypes.data)
    return out.tobytes()


def read_image(L, path):
    w, h = ctypes.c_int(), ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    if L.shim_read_image(path.encode(), ctypes.byref(w), ctypes.byref(h), None, err, 256) != 0:
        raise ValueError(err.value.decode())
    out = np.zeros((h.value, w.value, 3), np.float32)
    L.shim_read_image(path.encode(), ctypes.byref(w), ctypes.byref(h), out.ctypes.data, err, 256)
    return out


def bvh(L, pos, threads=4, depth_limit=2048):
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 9)
    n = pos.shape[0]
    nt, dep = ctypes.c_int(), ctypes.c_int()
    nn = L.shim_bvh(n, pos.ctypes.data, None, None, None, None, None, ctypes.byref(nt), ctypes.byref(dep), threads,
                    depth_limit)
    box = np.zeros((nn, 6), np.float32)
    kids = np.zeros((nn, 2), np.int32)
    first = np.zeros(nn, np.int32)
    count = np.zeros(nn, np.int32)
    tris = np.zeros(nt.value, np.int32)
    L.shim_bvh(n, pos.ctypes.data, box.ctypes.data, kids.ctypes.data, first.ctypes.data, count.ctypes.data,
               tris.ctypes.data, ctypes.byref(nt), ctypes.byref(dep), threads, depth_limit)
    return box, kids, first, count, tris, dep.value


def load_scene(L, desc):
    from nuray_gb300._lib import Material
    err = ctypes.create_string_buffer(512)
    nm = ctypes.c_int()
    n = L.shim_load(desc.encode(), None, None, None, None, None, ctypes.byref(nm), err, 512)
    if n < 0:
        raise ValueError(err.value.decode())
    pos, uv, nrm = (np.zeros((n, k), np.float32) for k in (9, 6, 9))
    mat = np.zeros(n, np.int32)
    mats = (Material * max(1, nm.value))()
    L.shim_load(desc.encode(), pos.ctypes.data, uv.ctypes.data, nrm.ctypes.data, mat.ctypes.data,
                ctypes.addressof(mats), ctypes.byref(nm), err, 512)
    return pos, uv, nrm, mat, [mats[i] for i in range(nm.value)]


def bvh_from_arrays(L, pos, tree, depth_limit=94):
    """nr::bvh_from_arrays on (box, kids, first, count, tris): (0, depth) or (-1, message)."""
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 9)
    box, kids, first, count, tris = (np.ascontiguousarray(a, t) for a, t in
                                     zip(tree, (np.float32, np.int32, np.int32, np.int32, np.int32)))
    depth = ctypes.c_int()
    err = ctypes.create_string_buffer(256)
    rc = L.shim_bvh_from_arrays(len(pos), pos.ctypes.data, len(kids), box.ctypes.data, kids.ctypes.data,
                                first.ctypes.data, count.ctypes.data, tris.ctypes.data, depth_limit,
                                ctypes.byref(depth), err, 256)
    return (0, depth.value) if rc == 0 else (-1, err.value.decode())
