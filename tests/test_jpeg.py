"""JPEG texture decoding (the JPG branch of Texture::load through Qt,
src/scene/texture.cpp:5-31) against files written by tests/jpeg_enc.py.

Qt is not available, so the decoder is checked against properties of the
format rather than Qt's own output: the coded coefficients reconstructed
exactly (T.81 A.3.3 in double precision, centred linear upsampling, JFIF
colour equations) give the decoded pixels to within one level; baseline,
progressive, restart-interval and non-interleaved codings of the same
coefficients decode to the same pixels; fine quantisation reproduces the
source image closely; and unsupported or broken files are refused."""
import numpy as np
import pytest

import shim
from jpeg_enc import encode, reconstruct


@pytest.fixture(scope="module")
def L():
    return shim.load()


def image(h, w, seed=0, gray=False):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w]
    base = 128 + 80 * np.sin(x / 5.0 + seed) * np.cos(y / 7.0) + rng.normal(0, 12, (h, w))
    if gray:
        return np.clip(base, 0, 255).astype(np.uint8)
    rgb = np.stack([base, 255 - base * 0.7 + 20 * np.sin(y / 3.0), base * 0.5 + 60 + rng.normal(0, 20, (h, w))], -1)
    return np.clip(rgb, 0, 255).astype(np.uint8)


def check_exact(L, img, **kw):
    data, comps, hmax, vmax = encode(img, **kw)
    got = shim.jpeg_decode(L, data)
    want = reconstruct(comps, img.shape[1], img.shape[0], hmax, vmax, kw.get("ycc", True))
    assert got.shape == want.shape
    d = np.abs(got.astype(int) - want.astype(int))
    assert d.max() <= 1 and np.mean(d > 0) < 1e-3, (d.max(), np.mean(d > 0))
    return got, data


SAMPLINGS = {
    "444": [(1, 1), (1, 1), (1, 1)],
    "422": [(2, 1), (1, 1), (1, 1)],
    "420": [(2, 2), (1, 1), (1, 1)],
    "440": [(1, 2), (1, 1), (1, 1)],
    "411": [(4, 1), (1, 1), (1, 1)],
}


@pytest.mark.parametrize("name", list(SAMPLINGS))
@pytest.mark.parametrize("size", [(29, 37), (64, 48), (1, 1), (9, 130)])
def test_baseline_matches_exact_reconstruction(L, name, size):
    check_exact(L, image(*size, seed=len(name)), sampling=SAMPLINGS[name], qscale=3.0)


def test_grayscale_and_rgb_components(L):
    g = image(33, 21, seed=3, gray=True)
    got, _ = check_exact(L, g, qscale=2.0)
    assert np.all(got[..., 0] == got[..., 1]) and np.all(got[..., 1] == got[..., 2])
    rgb = image(24, 40, seed=4)
    check_exact(L, rgb, ycc=False, adobe=0)
    check_exact(L, rgb, ycc=False, ids=[ord("R"), ord("G"), ord("B")])


@pytest.mark.parametrize("name", ["444", "420", "422"])
def test_progressive_restart_and_scan_layout_decode_identically(L, name):
    img = image(45, 61, seed=7)
    kw = dict(sampling=SAMPLINGS[name], qscale=2.5)
    ref, _ = check_exact(L, img, **kw)
    for extra in (dict(progressive=True), dict(restart=3), dict(restart=1), dict(interleave=False),
                  dict(progressive=True, restart=2), dict(progressive=True, restart=5)):
        got = shim.jpeg_decode(L, encode(img, **kw, **extra)[0])
        np.testing.assert_array_equal(got, ref, err_msg=str(extra))


def test_progressive_long_eob_runs_and_zero_runs(L):
    # flat areas: long end-of-band runs; sparse high frequencies: ZRL symbols
    img = np.full((96, 160, 3), 120, np.uint8)
    img[40:44, 10:150] = 250
    img[::17, ::23] = 0
    kw = dict(sampling=SAMPLINGS["420"], qscale=0.5)
    ref = shim.jpeg_decode(L, encode(img, **kw)[0])
    script = [([0, 1, 2], 0, 0, 0, 2), ([0, 1, 2], 0, 0, 2, 1), ([0, 1, 2], 0, 0, 1, 0)]
    for c in range(3):
        script += [([c], 1, 2, 0, 3), ([c], 3, 63, 0, 3), ([c], 1, 63, 3, 2), ([c], 1, 63, 2, 1), ([c], 1, 63, 1, 0)]
    got = shim.jpeg_decode(L, encode(img, **kw, progressive=True, script=script)[0])
    np.testing.assert_array_equal(got, ref)


def test_fine_quantisation_reproduces_the_source(L):
    img = image(40, 56, seed=9)
    got = shim.jpeg_decode(L, encode(img, qscale=0.0)[0]).astype(float)  # every step 1
    err = got - img.astype(float)
    psnr = 10 * np.log10(255.0 ** 2 / np.mean(err ** 2))
    assert psnr > 40, psnr


def test_refusals(L):
    img = image(16, 16, seed=1)
    data = encode(img)[0]
    with pytest.raises(ValueError, match="not a JPEG"):
        shim.jpeg_decode(L, b"\x89PNG\r\n\x1a\n" + data)
    with pytest.raises(ValueError, match="truncated"):
        shim.jpeg_decode(L, data[: len(data) // 2])
    i = data.index(b"\xff\xc0")
    for marker, msg in ((0xC9, "arithmetic|not supported|unsupported"), (0xC3, "unsupported JPEG process")):
        bad = data[:i + 1] + bytes([marker]) + data[i + 2:]
        with pytest.raises(ValueError, match=msg):
            shim.jpeg_decode(L, bad)
    bad = bytearray(data)
    bad[i + 4] = 12  # sample precision
    with pytest.raises(ValueError, match="8-bit"):
        shim.jpeg_decode(L, bytes(bad))


def test_texture_loader_reads_jpeg(L, tmp_path):
    img = image(20, 28, seed=5)
    data, comps, hmax, vmax = encode(img, sampling=SAMPLINGS["420"], qscale=1.0)
    p = tmp_path / "t.jpg"
    p.write_bytes(data)
    px = shim.jpeg_decode(L, data)
    tex = shim.read_image(L, str(p))
    # Texture::load: QColor::redF() then pow(., 2.2f), as for PNG
    want = np.power(px.astype(np.float64) * 257 / 65535.0, np.float64(np.float32(2.2))).astype(np.float32)
    np.testing.assert_array_equal(tex, want)
