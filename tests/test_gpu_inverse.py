"""Inverse rendering with the adjoint: from +-30 % perturbed materials,
Adam on the L2 image loss must bring the image and the parameters closer to
the hidden ones (small frame, few steps)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_inverse_rendering_recovers_materials(gpu_lib):
    from nuray_gb300 import Scene, inverse
    sc = inverse.c5_scene(0)
    S = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"])
    params = sc["params"].replace("imgw=512 imgh=512 spp=32", "imgw=96 imgh=96 spp=16")
    h = inverse.optimize(S, sc, params, steps=60, lr=0.02)
    print(f"image loss (same samples as the target) {h['eval_loss0']:.4g} -> {h['eval_loss']:.4g}; "
          f"error of the {h['params_constrained']} constrained parameters {h['param_err0']:.3f} -> {h['param_err'][-1]:.3f}")
    assert h["eval_loss"] < 0.5 * h["eval_loss0"]
    assert h["param_err"][-1] < h["param_err0"]
