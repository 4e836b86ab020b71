"""renderer=nrc: RendererNRC's path semantics (src/renderer/renderernrc.cpp)
driven by this project's cache.

* Its estimator without the cache (path_lim beyond every path) matches the
  oracle restatement per sample (test_gpu_parity.py), which is pinned to the
  reference's RendererNRC::trace compiled from source (test_oracle_pin.py).
* With a cache attached but never asked, the image is unchanged while the
  cache trains.
* The first, all-training pass is added to the image and the mean divides
  by spp, as RendererNRC::render does (a frame of spp samples carries spp + 1).
* With the cache asked from vertex path_lim (2) on and path_lim_train (4) on
  training paths, the image stays close to the converged one.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

P = "renderer=nrc imgw=96 imgh=72 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333"


def cornell():
    from nuray_gb300 import Scene
    g = golden("cornell_scene.npz")
    mats = [dict(type=int(i[0]), c0=f[0:3].tolist()) for i, f in zip(g["mat_i"], g["mat_f"])]
    return Scene.from_arrays(g["pos"], g["mat"], mats, uv=g["uv"], nrm=g["nrm"])


def rel(a, ref):
    return float(np.mean((a.astype(np.float64) - ref) ** 2 / (ref.astype(np.float64) ** 2 + 1e-2)))


def test_unasked_cache_leaves_the_image_unchanged(gpu_lib):
    from nuray_gb300.nrc import Cache
    S = cornell()
    p = P + " spp=4 path_lim=1000000 path_lim_train=1000000"
    plain = S.render(p)
    c = Cache("seed=3")
    c.attach(S)
    w0 = c.get_params()
    img = S.render(p)
    np.testing.assert_array_equal(img, plain)
    assert not np.array_equal(w0, c.get_params())  # trained on the training paths


def test_first_pass_is_added_and_the_mean_divides_by_spp(gpu_lib):
    S = cornell()
    with_pre = S.render(P + " spp=1 path_lim=1000000 seed=5")
    without = S.render(P + " spp=1 path_lim=1000000 seed=5 nrc_pre=0")
    ratio = float(with_pre.mean() / without.mean())
    print(f"image mean with / without the first pass at spp=1: {ratio:.3f} (expected about 2)")
    assert 1.8 < ratio < 2.2


def test_cached_render_close_to_converged(gpu_lib):
    from nuray_gb300.nrc import Cache
    S = cornell()
    ref = S.render(P.replace("renderer=nrc", "renderer=ptnee") + " spp=4096 seed=9")
    c = Cache("lr=1e-3")
    c.attach(S)
    img = S.render(P + " spp=64 seed=2")
    scale = 64.0 / 65.0  # the first pass adds one sample per pixel to a mean over 64
    err = rel(img * scale, ref)
    print(f"renderer=nrc with the cache, 64 spp: relMSE {err:.4f}; image mean / converged {img.mean() * scale / ref.mean():.3f}")
    assert np.all(np.isfinite(img))
    assert err < 0.1
    assert abs(img.mean() * scale / ref.mean() - 1) < 0.1


def test_adjoint_rejects_nrc(gpu_lib):
    S = cornell()
    with pytest.raises(Exception):
        S.adjoint(P + " spp=1", np.zeros((72, 96, 3), np.float32))
