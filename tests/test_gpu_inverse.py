"""Inverse rendering with the adjoint on the inverse-rendering workload
(200k triangles, 64 surface materials, 16 emitters; a 160x160 frame of
32 spp, depth 4), from +-30 % perturbed materials, Adam on the L2 image
loss with the adjoint's gradients:

* everything free (albedo, roughness and emission of every material): the
  image must come closer to the target's (loss evaluated with the
  target's own samples);
* the identifiable part: emission fixed at its true value and only the
  materials that are the first hit of at least 1 % of the pixels free (a
  brighter light and darker surfaces give nearly the same image, and a
  material seen in a few pixels is barely constrained): the relative
  parameter error of the optimised albedos and roughnesses must fall to
  under a third of its start."""
import pytest

pytestmark = pytest.mark.gpu


def _scene():
    from nuray_gb300 import Scene, inverse
    sc = inverse.c5_scene(0)
    S = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"])
    params = sc["params"].replace("imgw=512 imgh=512 spp=32", "imgw=160 imgh=160 spp=32")
    return sc, S, params


def test_inverse_rendering_matches_the_image(gpu_lib):
    from nuray_gb300 import inverse
    sc, S, params = _scene()
    h = inverse.optimize(S, sc, params, steps=40, lr=0.02)
    print(f"all free: image loss (same samples as the target) {h['eval_loss0']:.4g} -> {h['eval_loss']:.4g}; "
          f"error of the {h['params_constrained']} constrained parameters {h['param_err0']:.3f} -> "
          f"{h['param_err'][-1]:.3f}")
    assert h["eval_loss"] < 0.6 * h["eval_loss0"]


def test_inverse_rendering_recovers_identifiable_materials(gpu_lib):
    from nuray_gb300 import inverse
    sc, S, params = _scene()
    h = inverse.optimize(S, sc, params, steps=60, lr=0.02, fix_emission=True, min_coverage=0.01)
    print(f"emission fixed, materials on >= 1 % of the pixels: {h['params_optimised']} parameters, relative error "
          f"{h['param_err0']:.3f} -> {h['param_err'][-1]:.3f}; image loss {h['eval_loss0']:.4g} -> {h['eval_loss']:.4g}")
    assert h["params_optimised"] >= 100
    assert h["param_err"][-1] < h["param_err0"] / 3
    assert h["eval_loss"] < 0.3 * h["eval_loss0"]
