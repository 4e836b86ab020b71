"""Mutated inputs for the product's host-side parsers, run through the test
shim (tests/host_shim.cpp): PNG (with repaired chunk CRCs, so corrupted
deflate streams reach the inflater), JPEG (baseline, progressive, restart
intervals, subsampled, non-interleaved), OBJ/MTL scene descriptions and the
key=value parameter grammar, and trees handed to nr_scene_create_bvh. Each
input must decode or be refused; nothing may crash. Run as a child process
by tests/test_fuzz_host.py:

    python tests/fuzz_host.py KIND FIRST COUNT

prints "ok KIND COUNT" when every input of the range came back."""
import ctypes
import os
import struct
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

import jpeg_enc  # noqa: E402
import shim  # noqa: E402


def _chunk(t, d):
    return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xffffffff)


def _png_seeds():
    rng = np.random.default_rng(1)
    w, h = 19, 13
    seeds = []
    for ct, depth, rows, plte in (
            (2, 8, (rng.random((h, w * 3)) * 255).astype(np.uint8), None),
            (6, 8, (rng.random((h, w * 4)) * 255).astype(np.uint8), None),
            (0, 16, (rng.random((h, w * 2)) * 255).astype(np.uint8), None),
            (3, 4, (rng.random((h, (w + 1) // 2)) * 255).astype(np.uint8), bytes(range(48)))):
        head = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ct, 0, 0, 0))
        if plte:
            head += _chunk(b"PLTE", plte)
        raw = b"".join(b"\x00" + r.tobytes() for r in rows)
        seeds.append((head, raw))
    return seeds


def png_case(seeds, idx):
    rng = np.random.default_rng(idx)
    head, raw = seeds[idx % len(seeds)]
    comp = bytearray(zlib.compress(raw, 9))
    op = rng.integers(0, 4)
    if op == 0:
        for _ in range(rng.integers(1, 6)):
            comp[rng.integers(0, len(comp))] = rng.integers(0, 256)
    elif op == 1:
        comp = comp[:rng.integers(0, len(comp))]
    elif op == 2:
        comp[rng.integers(2, len(comp))] ^= 1 << int(rng.integers(0, 8))
    else:  # the filtered rows corrupted and compressed again (a valid stream)
        r = bytearray(raw)
        for _ in range(rng.integers(1, 6)):
            r[rng.integers(0, len(r))] = rng.integers(0, 256)
        comp = bytearray(zlib.compress(bytes(r[:rng.integers(len(r) // 2, len(r) + 1)]), 9))
    data = head + _chunk(b"IDAT", bytes(comp)) + _chunk(b"IEND", b"")
    if rng.random() < 0.2:  # header fields too (the CRC then refuses most)
        b = bytearray(data)
        b[rng.integers(8, 33)] = rng.integers(0, 256)
        data = bytes(b)
    return data


def _jpeg_seeds():
    rng = np.random.default_rng(0)
    img = (rng.random((23, 37, 3)) * 255).astype(np.uint8)
    return [jpeg_enc.encode(img, **kw)[0] for kw in (dict(), dict(progressive=True), dict(restart=2),
                                                      dict(sampling=[(2, 2), (1, 1), (1, 1)]), dict(interleave=False))]


def jpeg_case(seeds, idx):
    rng = np.random.default_rng(idx)
    b = bytearray(seeds[idx % len(seeds)])
    op = rng.integers(0, 4)
    if op == 0:
        for _ in range(rng.integers(1, 8)):
            b[rng.integers(0, len(b))] = rng.integers(0, 256)
    elif op == 1:
        b = b[:rng.integers(0, len(b))]
    elif op == 2:
        i = rng.integers(0, len(b))
        j = min(len(b), i + int(rng.integers(1, 64)))
        b = b[:j] + b[i:j] + b[j:]
    else:  # marker segments near the start (frame and scan headers, tables)
        for _ in range(rng.integers(1, 4)):
            b[rng.integers(0, min(len(b), 700))] = rng.integers(0, 256)
    return bytes(b)


OBJ = """mtllib box.mtl
v 0 0 0
v 1 0 0
v 0 1 0
v 1 1 0
v 0 0 1
vt 0 0
vt 1 0
vt 0 1
vn 0 0 1
vn 0 1 0
usemtl red
f 1/1/1 2/2/1 3/3/1
f 2/2/1 4/1/1 3/3/1
usemtl light
f 1//2 2//2 5//2
f 1 2 3 4 5
f -1 -2 -3
"""
MTL = """newmtl red
Kd 0.8 0.1 0.1
Ks 0.2 0.2 0.2
Ns 20
map_Kd tex.ppm
newmtl light
Ke 5 5 5
"""
TOKENS = ["", "0", "-1", "1e38", "-1e38", "nan", "inf", "1/", "/1", "//", "99999999999", "-99999999999", "f", "v",
          "vt", "vn", "usemtl", "newmtl", "mtllib", "Kd", "Ke", "Ns", "map_Kd", "1/2/3/4", "0/0/0", "\t", "#", "a b c",
          "-m=light", "-m=ggx", "-m=ggxr", "-s", "-p", "1 2", "2147483648", "-2147483649", "1.5e", "0x10", "\\"]


def _mutate_text(t, rng):
    lines = t.split("\n")
    for _ in range(rng.integers(1, 6)):
        op = rng.integers(0, 5)
        i = int(rng.integers(0, len(lines)))
        toks = lines[i].split(" ")
        if op == 0:
            toks[rng.integers(0, len(toks))] = TOKENS[rng.integers(0, len(TOKENS))]
        elif op == 1:
            toks.append(TOKENS[rng.integers(0, len(TOKENS))])
        elif op == 2 and len(toks) > 1:
            del toks[rng.integers(0, len(toks))]
        elif op == 3:
            lines.insert(i, " ".join(TOKENS[rng.integers(0, len(TOKENS))] for _ in range(rng.integers(0, 6))))
            continue
        else:
            toks = [lines[i][:rng.integers(0, len(lines[i]) + 1)]]
        lines[i] = " ".join(toks)
    return "\n".join(lines)


def obj_case(folder, idx):
    rng = np.random.default_rng(idx)
    with open(os.path.join(folder, "box.obj"), "w") as f:
        f.write(_mutate_text(OBJ, rng) if rng.random() < 0.8 else OBJ)
    with open(os.path.join(folder, "box.mtl"), "w") as f:
        f.write(_mutate_text(MTL, rng) if rng.random() < 0.5 else MTL)
    desc = os.path.join(folder, "box.obj")
    if rng.random() < 0.4:
        desc += " " + " ".join(TOKENS[rng.integers(0, len(TOKENS))] for _ in range(rng.integers(1, 6)))
    return desc + "\n"


def _tree_seed(L):
    rng = np.random.default_rng(5)
    pos = rng.uniform(-5, 5, (300, 9)).astype(np.float32)
    box, kids, first, count, tris, _ = shim.bvh(L, pos)
    return pos, (box, kids, first, count, tris)


def tree_case(tree, idx):
    """The builder's tree with a few entries of its arrays set to values in and
    out of range (the arrays keep their lengths, as the API requires)."""
    rng = np.random.default_rng(idx)
    t = [a.copy() for a in tree]
    n_nodes, n = len(t[1]), len(t[4])
    for _ in range(rng.integers(1, 4)):
        which = rng.integers(0, 5)
        a = t[which].reshape(-1)
        i = rng.integers(0, len(a))
        if which == 0:
            a[i] = [np.nan, np.inf, -np.inf, 0.0, 1e30, -1e30, a[i] * 0.5][rng.integers(0, 7)]
        else:
            a[i] = [-1, -2, 0, 1, n_nodes - 1, n_nodes, n - 1, n, 7, 8, 2 ** 31 - 1, -2 ** 31][rng.integers(0, 12)]
    return t


PARAM_TOKENS = ["imgw=", "spp=", "campos=", "cameuler=", "camfov=", "=", "==", "1", "-1", "1e40", "nan", "inf", ",",
                ",,", "1,2", "1,2,3,4", " ", "\t", "a=b=c", "x", "99999999999999999999", "-0", "0x1f", "1e-50"]


def main():
    kind, first, count = sys.argv[1], int(sys.argv[2]), int(sys.argv[3])
    L = shim.load()
    if kind == "png":
        seeds = _png_seeds()
        for i in range(first, first + count):
            try:
                shim.png_decode(L, png_case(seeds, i))
            except (ValueError, MemoryError):
                pass
    elif kind == "jpeg":
        seeds = _jpeg_seeds()
        for i in range(first, first + count):
            try:
                shim.jpeg_decode(L, jpeg_case(seeds, i))
            except (ValueError, MemoryError):
                pass
    elif kind == "obj":
        folder = tempfile.mkdtemp(prefix="nuray_fuzz_")
        with open(os.path.join(folder, "tex.ppm"), "wb") as f:
            f.write(b"P6\n2 2\n255\n" + bytes(range(12)))
        for i in range(first, first + count):
            try:
                shim.load_scene(L, obj_case(folder, i))
            except (ValueError, MemoryError):
                pass
    elif kind == "tree":
        pos, tree = _tree_seed(L)
        for i in range(first, first + count):
            shim.bvh_from_arrays(L, pos, tree_case(tree, i))
    elif kind == "params":
        out = (ctypes.c_float * 3)()
        cam = (ctypes.c_float * 11)()  # nr_camera
        film_h = (ctypes.c_float * 1)()
        for i in range(first, first + count):
            rng = np.random.default_rng(i)
            s = "".join(PARAM_TOKENS[rng.integers(0, len(PARAM_TOKENS))] for _ in range(rng.integers(0, 12))).encode()
            for k in (b"imgw", b"spp", b"campos", b"cameuler", b"camfov", b"x", b""):
                L.shim_config_int(s, k, 7)
                L.shim_config_float(s, k, 1.5)
                L.shim_config_vec3(s, k, out)
            L.shim_camera(s, cam, film_h)
    else:
        raise SystemExit(f"unknown kind {kind}")
    print("ok", kind, count)


if __name__ == "__main__":
    main()
