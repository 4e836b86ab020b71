"""Host-side faults that need no GPU: scenes with NaN or infinite inputs
are refused with NR_ERR_INVALID before anything reaches a device (the
reference checks nothing and would carry NaN into every box and sample its
triangles touch; its only failure path is a message on stderr,
src/sampler/lightsampler.cpp:35-38). The device byte cap that turns an
over-large allocation into NR_ERR_OOM is tested on the GPU
(test_gpu_faults.py)."""
import numpy as np
import pytest

from conftest import golden


def cornell():
    g = golden("cornell_scene.npz")
    mats = [dict(type=int(i[0]), c0=f[0:3].tolist(), c1=f[3:6].tolist(), alpha=float(f[6]), ior=float(f[7]),
                 ns=float(f[8])) for i, f in zip(g["mat_i"], g["mat_f"])]
    return dict(pos=g["pos"].copy(), uv=g["uv"].copy(), nrm=g["nrm"].copy(), mat=g["mat"].copy(), mats=mats)


def create(sc, textures=(), env_gain=1.0):
    from nuray_gb300 import Scene
    return Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"], textures=list(textures),
                             env_tex=len(textures) - 1 if textures else -1, env_gain=env_gain)


@pytest.mark.parametrize("field,row,col", [("pos", 3, 4), ("nrm", 7, 0), ("uv", 11, 5)])
@pytest.mark.parametrize("bad", [np.nan, np.inf, -np.inf])
def test_non_finite_geometry_is_refused(field, row, col, bad):
    from nuray_gb300 import NuRayError
    sc = cornell()
    sc[field][row, col] = bad
    with pytest.raises(NuRayError, match=r"NR_ERR_INVALID: triangle %d: non-finite" % row):
        create(sc)


@pytest.mark.parametrize("key", ["c0", "alpha", "ior"])
def test_non_finite_material_is_refused(key):
    from nuray_gb300 import NuRayError
    sc = cornell()
    m = dict(sc["mats"][1])
    m[key] = [1.0, np.nan, 0.5] if key == "c0" else np.inf
    sc["mats"][1] = m
    with pytest.raises(NuRayError, match="NR_ERR_INVALID: material 1: non-finite parameter"):
        create(sc)


def test_non_finite_texels_and_gain_are_refused():
    from nuray_gb300 import NuRayError
    sc = cornell()
    env = np.ones((4, 8, 3), np.float32)
    env[2, 3, 1] = np.nan
    with pytest.raises(NuRayError, match="NR_ERR_INVALID: texel value .* is not finite"):
        create(sc, textures=[env])
    with pytest.raises(NuRayError, match="NR_ERR_INVALID: env_gain is not finite"):
        create(sc, textures=[np.ones((4, 8, 3), np.float32)], env_gain=np.inf)
