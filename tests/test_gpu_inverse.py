"""Inverse rendering with the adjoint: from +-30 % perturbed materials,
Adam on the L2 image loss must bring the image closer to the target's
(loss evaluated with the target's own samples; small frame, few steps)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_inverse_rendering_recovers_materials(gpu_lib):
    from nuray_gb300 import Scene, inverse
    sc = inverse.c5_scene(0)
    S = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"])
    params = sc["params"].replace("imgw=512 imgh=512 spp=32", "imgw=160 imgh=160 spp=32")
    h = inverse.optimize(S, sc, params, steps=40, lr=0.02)
    print(f"image loss (same samples as the target) {h['eval_loss0']:.4g} -> {h['eval_loss']:.4g}; "
          f"error of the {h['params_constrained']} constrained parameters {h['param_err0']:.3f} -> {h['param_err'][-1]:.3f}")
    # the image is matched; individual parameters are not identifiable in
    # general (albedo against emission, barely visible materials)
    assert h["eval_loss"] < 0.6 * h["eval_loss0"]
