"""PNG decoding for textures and PNG output, on the CPU.

The product decoder (nuray_gb300/csrc/image_io.cpp: zlib, DEFLATE and PNG
written for this project) is checked against images this test encodes with
Python's zlib, over every colour type and bit depth, all five scanline
filters, Adam7 interlacing, stored / fixed-Huffman / dynamic-Huffman DEFLATE
blocks, palettes and tRNS. The encoder's output is checked by Python's zlib
(Adler-32) and CRC-32 and decoded back. The scene loader's texture values
follow Texture::load (src/scene/texture.cpp:13-19): pow(v * 257 / 65535,
2.2f) per 8-bit channel.
"""
import os
import struct
import zlib

import numpy as np
import pytest

import shim
from conftest import REF_ROOT

ADAM7 = [(0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2)]
CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}


@pytest.fixture(scope="module")
def L():
    return shim.load()


def chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xffffffff)


def pack_row(samples, depth):
    """Integer samples of one row -> bytes at the given bit depth."""
    if depth == 8:
        return bytes(np.asarray(samples, np.uint8))
    if depth == 16:
        return np.asarray(samples, ">u2").tobytes()
    out = bytearray((len(samples) * depth + 7) // 8)
    for i, v in enumerate(samples):
        bit = i * depth
        out[bit >> 3] |= int(v) << (8 - depth - (bit & 7))
    return bytes(out)


def paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def filter_row(cur, prev, bpp, ftype):
    out = bytearray(len(cur))
    for i in range(len(cur)):
        a = cur[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        pred = [0, a, b, (a + b) >> 1, paeth(a, b, c)][ftype]
        out[i] = (cur[i] - pred) & 0xff
    return bytes([ftype]) + bytes(out)


def encode(img, ctype, depth, interlace=False, filters=(0,), palette=None, trns=None, level=6, strategy=None,
           seed=0):
    """img: (h, w, channels) integer samples at `depth`."""
    h, w, ch = img.shape
    rng = np.random.default_rng(seed)
    bpp = max(1, ch * depth // 8)
    raw = bytearray()
    passes = ADAM7 if interlace else [(0, 0, 1, 1)]
    for x0, y0, dx, dy in passes:
        sub = img[y0::dy, x0::dx]
        if sub.size == 0:
            continue
        prev = bytes(len(pack_row(sub[0].ravel(), depth)))
        for row in sub:
            cur = pack_row(row.ravel(), depth)
            raw += filter_row(cur, prev, bpp, int(rng.choice(filters)))
            prev = cur
    if strategy is None:
        z = zlib.compress(bytes(raw), level)
    else:
        co = zlib.compressobj(level, zlib.DEFLATED, 15, 8, strategy)
        z = co.compress(bytes(raw)) + co.flush()
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, int(interlace)))
    if palette is not None:
        png += chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).ravel()))
    if trns is not None:
        png += chunk(b"tRNS", trns)
    half = len(z) // 2  # two IDAT chunks
    png += chunk(b"IDAT", z[:half]) + chunk(b"IDAT", z[half:]) + chunk(b"IEND", b"")
    return png


def expected_rgba(img, ctype, depth, palette=None, trns=None):
    h, w, _ = img.shape
    to8 = (lambda v: v >> 8) if depth == 16 else (lambda v: v * 255 // ((1 << depth) - 1))
    out = np.zeros((h, w, 4), np.int64)
    if ctype == 3:
        pal = np.asarray(palette)
        out[..., :3] = pal[img[..., 0]]
        alpha = np.full(len(pal), 255)
        if trns is not None:
            alpha[:len(trns)] = list(trns)
        out[..., 3] = alpha[img[..., 0]]
    elif ctype in (0, 4):
        out[..., :3] = to8(img[..., :1])
        out[..., 3] = to8(img[..., 1]) if ctype == 4 else 255
        if ctype == 0 and trns is not None:
            out[..., 3] = np.where(img[..., 0] == struct.unpack(">H", trns)[0], 0, 255)
    else:
        out[..., :3] = to8(img[..., :3])
        out[..., 3] = to8(img[..., 3]) if ctype == 6 else 255
        if ctype == 2 and trns is not None:
            key = struct.unpack(">HHH", trns)
            out[..., 3] = np.where(np.all(img[..., :3] == key, axis=2), 0, 255)
    return out.astype(np.uint8)


CASES = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8), (4, 8), (4, 16),
         (6, 8), (6, 16)]


@pytest.mark.parametrize("ctype,depth", CASES)
@pytest.mark.parametrize("interlace", [False, True])
def test_decode_matches_source(L, ctype, depth, interlace):
    rng = np.random.default_rng(ctype * 100 + depth + 7 * interlace)
    h, w = (13, 17) if interlace else (9, 23)
    top = (1 << depth) - 1
    palette = None
    if ctype == 3:
        n = min(top + 1, 40)
        palette = rng.integers(0, 256, (n, 3))
        img = rng.integers(0, n, (h, w, 1))
    else:
        img = rng.integers(0, top + 1, (h, w, CHANNELS[ctype]))
    png = encode(img, ctype, depth, interlace, filters=(0, 1, 2, 3, 4), palette=palette, seed=depth)
    np.testing.assert_array_equal(shim.png_decode(L, png), expected_rgba(img, ctype, depth, palette))


@pytest.mark.parametrize("level,strategy", [(0, None), (1, None), (9, None), (6, zlib.Z_FIXED),
                                            (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE)])
def test_deflate_block_kinds(L, level, strategy):
    rng = np.random.default_rng(level)
    # large enough for several stored blocks and long matches
    img = (np.arange(260 * 300 * 3).reshape(260, 300, 3) // 7 % 256 + rng.integers(0, 2, (260, 300, 3))) % 256
    png = encode(img, 2, 8, filters=(0, 1, 4), level=level, strategy=strategy)
    np.testing.assert_array_equal(shim.png_decode(L, png)[..., :3], img)


def test_trns_keys_and_palette_alpha(L):
    rng = np.random.default_rng(3)
    img = rng.integers(0, 4, (6, 7, 1))
    pal = rng.integers(0, 256, (4, 3))
    png = encode(img, 3, 2, palette=pal, trns=bytes([0, 128]))
    np.testing.assert_array_equal(shim.png_decode(L, png), expected_rgba(img, 3, 2, pal, bytes([0, 128])))
    g = rng.integers(0, 16, (5, 5, 1))
    png = encode(g, 0, 4, trns=struct.pack(">H", 3))
    np.testing.assert_array_equal(shim.png_decode(L, png), expected_rgba(g, 0, 4, trns=struct.pack(">H", 3)))
    c = rng.integers(0, 3, (5, 6, 3))
    key = struct.pack(">HHH", 1, 2, 0)
    np.testing.assert_array_equal(shim.png_decode(L, encode(c, 2, 8, trns=key)), expected_rgba(c, 2, 8, trns=key))


def test_corrupt_inputs_are_errors(L):
    img = np.random.default_rng(1).integers(0, 256, (8, 8, 3))
    good = encode(img, 2, 8)
    shim.png_decode(L, good)
    bad_crc = bytearray(good)
    bad_crc[40] ^= 0xff  # inside IHDR / first IDAT: CRC mismatch
    for data in (bytes(bad_crc), good[:60], b"not a png", good[:8] + good[33:]):
        with pytest.raises(ValueError):
            shim.png_decode(L, data)


def test_encoder_output_is_valid_png(L):
    rng = np.random.default_rng(5)
    for h, w in ((1, 1), (7, 5), (300, 251)):  # the last spans two stored blocks
        img = rng.integers(0, 256, (h, w, 3)).astype(np.uint8)
        png = shim.png_encode(L, img)
        assert png[:8] == b"\x89PNG\r\n\x1a\n"
        pos, idat = 8, b""
        while pos < len(png):
            n = struct.unpack(">I", png[pos:pos + 4])[0]
            t, data = png[pos + 4:pos + 8], png[pos + 8:pos + 8 + n]
            assert struct.unpack(">I", png[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(t + data) & 0xffffffff
            if t == b"IDAT":
                idat += data
            pos += 12 + n
        raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 3 * w + 1)  # checks Adler-32 too
        assert np.all(raw[:, 0] == 0)
        np.testing.assert_array_equal(raw[:, 1:].reshape(h, w, 3), img)
        np.testing.assert_array_equal(shim.png_decode(L, png)[..., :3], img)


def test_texture_values_follow_texture_load(L, tmp_path):
    rng = np.random.default_rng(9)
    img = rng.integers(0, 256, (6, 9, 3))
    p = tmp_path / "t.png"
    p.write_bytes(encode(img, 2, 8, filters=(2, 4)))
    got = shim.read_image(L, str(p))
    want = np.power((img * 257).astype(np.float64) / 65535.0, np.float64(np.float32(2.2))).astype(np.float32)
    np.testing.assert_array_equal(got, want)


def python_png_decode(data):
    """A second, independent decoder in numpy (8-bit RGB / RGBA / palette,
    non-interlaced) used to check the reference's shipped PNG assets."""
    pos, idat, hdr, pal = 8, b"", None, None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        t, d = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if t == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", d)
        elif t == b"PLTE":
            pal = np.frombuffer(d, np.uint8).reshape(-1, 3)
        elif t == b"IDAT":
            idat += d
        pos += 12 + n
    w, h, depth, ctype, _, _, interlace = hdr
    if depth != 8 or interlace or ctype not in (2, 3, 6, 0, 4):
        return None
    ch = CHANNELS[ctype]
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + w * ch)
    prev = np.zeros(w * ch, np.int64)
    rows = []
    for y in range(h):
        f, cur = raw[y, 0], raw[y, 1:].astype(np.int64)
        out = np.zeros_like(cur)
        for i in range(len(cur)):
            a = out[i - ch] if i >= ch else 0
            b = prev[i]
            c = prev[i - ch] if i >= ch else 0
            out[i] = (cur[i] + [0, a, b, (a + b) >> 1, paeth(a, b, c)][f]) & 0xff
        rows.append(out)
        prev = out
    img = np.array(rows).reshape(h, w, ch).astype(np.uint8)
    if ctype == 3:
        return pal[img[..., 0]]
    if ctype in (0, 4):
        return np.repeat(img[..., :1], 3, axis=2)
    return img[..., :3]


@pytest.mark.parametrize("name", ["default.png", "mitsuba-icon.png"])
def test_reference_scene_textures(L, name):
    path = os.path.join(REF_ROOT, "scenes/mitsuba", name)
    if not os.path.exists(path):
        pytest.skip("reference checkout not present")
    data = open(path, "rb").read()
    got = shim.png_decode(L, data)
    want = python_png_decode(data)
    if want is None:
        pytest.skip("asset uses a PNG form the numpy checker does not cover")
    np.testing.assert_array_equal(got[..., :3], want)


def test_loader_reads_reference_scene_with_png_texture(L, ref_lib):
    """scenes/mitsuba/mitsuba-back.obj: the backdrop's map_Kd default.png now
    loads; triangles match the reference Loader's, and the texture holds
    Texture::load's values of the decoded image."""
    import ctypes
    from oracle.bind import Oracle
    obj = os.path.join(REF_ROOT, "scenes/mitsuba/mitsuba-back.obj")
    pos, uv, nrm, mat, mats = shim.load_scene(L, obj + "\n")
    R = Oracle("ref", desc=obj + "\n")
    n = R.L.ref_scene_num_tris(ctypes.c_void_p(R.h))
    rp, ru, rn = (np.zeros((n, k), np.float32) for k in (9, 6, 9))
    rm = np.zeros(n, np.int32)
    R.L.ref_scene_get_tris.argtypes = [ctypes.c_void_p] * 5
    R.L.ref_scene_get_tris(R.h, rp.ctypes.data, ru.ctypes.data, rn.ctypes.data, rm.ctypes.data)
    np.testing.assert_array_equal(pos, rp)
    np.testing.assert_array_equal(uv, ru)
    np.testing.assert_array_equal(nrm, rn)
    textured = [m for m in mats if m.tex0 >= 0]
    assert len(textured) == 1 and textured[0].type == 4  # BlinnPhong (Ks 0.2) with map_Kd
    tex = shim.read_image(L, os.path.join(REF_ROOT, "scenes/mitsuba/default.png"))
    rgb = python_png_decode(open(os.path.join(REF_ROOT, "scenes/mitsuba/default.png"), "rb").read())
    want = np.power((rgb.astype(np.int64) * 257).astype(np.float64) / 65535.0,
                    np.float64(np.float32(2.2))).astype(np.float32)
    np.testing.assert_array_equal(tex, want)
