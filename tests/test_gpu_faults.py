"""Allocation failure without exhausting a shared GPU: the scene option
max_device_bytes caps the device memory of a scene's own buffers, and an
allocation past the cap fails with NR_ERR_OOM exactly where a failed
cudaMalloc would, leaving the scene usable for calls that fit."""
import numpy as np
import pytest

from test_host_faults import cornell

pytestmark = pytest.mark.gpu

SMALL = "renderer=ptnee imgw=64 imgh=48 spp=4 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333"


def _scene(options=""):
    from nuray_gb300 import Scene
    sc = cornell()
    return Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"], options=options)


def test_scene_over_the_cap_is_refused(gpu_lib):
    from nuray_gb300 import NuRayError
    need = _scene().info()["device_bytes"]
    with pytest.raises(NuRayError, match="NR_ERR_OOM: device allocation of .* exceeds the scene's cap"):
        _scene(f"max_device_bytes={need // 2}")
    with pytest.raises(NuRayError, match="NR_ERR_INVALID: max_device_bytes"):
        _scene("max_device_bytes=12x")


def test_render_over_the_cap_fails_and_the_scene_stays_usable(gpu_lib):
    from nuray_gb300 import NuRayError
    free = _scene()
    want = free.render(SMALL)
    S = _scene(f"max_device_bytes={free.info()['device_bytes'] + (32 << 20)}")
    # 1080p x 64 spp in one wave needs about 24 GB of path state
    with pytest.raises(NuRayError, match="NR_ERR_OOM"):
        S.render(SMALL.replace("imgw=64 imgh=48", "imgw=1920 imgh=1080").replace("spp=4", "spp=64"))
    np.testing.assert_array_equal(S.render(SMALL), want)
    # the same frame fits in waves small enough for the cap
    big = SMALL.replace("imgw=64 imgh=48", "imgw=320 imgh=240")
    np.testing.assert_array_equal(S.render(big + " wave=65536"), free.render(big))


def test_cameras_without_a_film_are_refused(gpu_lib):
    """A camera with a non-finite value, a field of view outside (0, 180)
    degrees or a non-positive aspect would make every ray NaN: the call is
    refused with NR_ERR_INVALID and the scene renders normally afterwards."""
    from nuray_gb300._lib import NuRayError, camera_from_params
    S = _scene()
    for bad in ("camfov=0", "camfov=180", "camfov=-5", "camasp=0", "camasp=-1"):
        with pytest.raises(NuRayError, match="NR_ERR_INVALID"):
            S.render(SMALL.replace("camfov=64", "").replace("camasp=1.333", "") + " " + bad)
    cam = camera_from_params(SMALL)
    cam.pos[1] = float("nan")
    with pytest.raises(NuRayError, match="non-finite"):
        S.render(SMALL, camera=cam)
    cam = camera_from_params(SMALL)
    cam.fov = float("inf")
    with pytest.raises(NuRayError, match="NR_ERR_INVALID"):
        S.render(SMALL, camera=cam)
    img = S.render(SMALL)
    assert np.all(np.isfinite(img)) and img.mean() > 0
