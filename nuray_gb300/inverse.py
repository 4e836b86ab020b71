"""Inverse rendering with the path-replay adjoint: recover per-material
albedo, roughness and emission from a target image.

The target is rendered at hidden parameters; optimisation starts from a
seeded +-`perturb` multiplicative perturbation of them and runs Adam on the
L2 image loss mean((I - T)^2), with gradients from nr_adjoint (fresh Philox
seed every step). Albedo is kept in [0, 1], roughness in [0.05, 1] and
emission >= 0.

Which parameters an image determines: with the emitters' radiance free, a
brighter light and darker surfaces give nearly the same image, and a
material seen in a handful of pixels is barely constrained at all. So the
recovery can keep emission fixed (`fix_emission`) and optimise only the
materials whose surfaces are the first hit of at least `min_coverage` of
the pixels (`coverage`); the parameter error is measured over those.
"""
import time

import numpy as np

from ._lib import MAT_GGX, MAT_GGXR, MAT_LIGHT

ALBEDO, ROUGH, EMIT = slice(0, 3), 3, slice(4, 7)


def c5_scene(seed=0):
    """About 200k triangles and 64 surface materials (GGX reflect and Lambert)."""
    from .scenes import terrain_spheres
    sc = terrain_spheres(seed, tiles=32, cells_per_tile=8, spheres=128, slices=20, stacks=16, lights=16, n_mats=64,
                         extent=128.0)
    rng = np.random.Generator(np.random.Philox(key=[seed, 31]))
    for i, m in enumerate(sc["mats"]):
        if m["type"] != MAT_LIGHT and rng.uniform() < 0.3:
            m["type"] = 0  # Lambert
    sc["params"] = ("renderer=ptnee imgw=512 imgh=512 spp=32 campos=0,50,75 cameuler=0,-38,0 camfov=50 camasp=1 "
                    "maxdepth=4 rrdepth=3")
    return sc


def c5_scene_small(seed=0):
    """The inverse-rendering scene at the size its finite-difference check can
    afford on host cores: the same 200k-triangle terrain and spheres, 8
    surface materials (GGX reflect, about a third Lambert, each on 8-16 % of
    a 128x128 frame) and the 16 quad lights sharing 2 emission materials."""
    from .scenes import terrain_spheres
    sc = terrain_spheres(seed, tiles=32, cells_per_tile=8, spheres=128, slices=20, stacks=16, lights=16, n_mats=8,
                         extent=128.0)
    mats = sc["mats"]
    surf = [i for i, m in enumerate(mats) if m["type"] != MAT_LIGHT]
    for i in surf[1::3]:
        mats[i]["type"] = 0  # Lambert
    lights = [i for i, m in enumerate(mats) if m["type"] == MAT_LIGHT]
    keep = len(surf)
    # lights alternate between two emission materials with the first two lights' radiance
    remap = {i: i for i in surf}
    for k, i in enumerate(lights):
        remap[i] = keep + (k % 2)
    sc["mat"] = np.array([remap[int(m)] for m in sc["mat"]], np.int32)
    sc["mats"] = [mats[i] for i in surf] + [mats[lights[0]], mats[lights[1]]]
    sc["params"] = ("renderer=ptnee imgw=128 imgh=128 spp=64 campos=0,50,75 cameuler=0,-38,0 camfov=50 camasp=1 "
                    "maxdepth=4 rrdepth=3")
    return sc


def param_table(mats):
    """(num_mats, 7) parameter array and the mask of parameters that exist."""
    P = np.zeros((len(mats), 7), np.float64)
    mask = np.zeros((len(mats), 7), bool)
    for i, m in enumerate(mats):
        c0 = np.array(m.get("c0", (0, 0, 0)), np.float64)
        if m["type"] == MAT_LIGHT:
            P[i, EMIT] = c0
            mask[i, EMIT] = True
        else:
            if m.get("tex0", -1) < 0:
                P[i, ALBEDO] = c0
                mask[i, ALBEDO] = True
            if m["type"] in (MAT_GGXR, MAT_GGX):
                P[i, ROUGH] = m.get("alpha", 0.5)
                mask[i, ROUGH] = True
    return P, mask


def apply(mats, P):
    out = []
    for i, m in enumerate(mats):
        m = dict(m)
        if m["type"] == MAT_LIGHT:
            m["c0"] = [float(x) for x in P[i, EMIT]]
        else:
            if m.get("tex0", -1) < 0:
                m["c0"] = [float(x) for x in P[i, ALBEDO]]
            if m["type"] in (MAT_GGXR, MAT_GGX):
                m["alpha"] = float(P[i, ROUGH])
        out.append(m)
    return out


def clamp(P, mask):
    Q = P.copy()
    Q[:, ALBEDO] = np.clip(Q[:, ALBEDO], 0.0, 1.0)
    Q[:, ROUGH] = np.clip(Q[:, ROUGH], 0.05, 1.0)
    Q[:, EMIT] = np.maximum(Q[:, EMIT], 0.0)
    return np.where(mask, Q, P)


def coverage(scene, sc, params):
    """Fraction of the image's pixels whose centre ray first hits each
    material (nr_intersect on the camera's pixel-centre rays, the camera of
    Camera::generateRay, src/scene/camera.cpp:24-32)."""
    from ._lib import camera_from_params, parse_params
    cam = camera_from_params(params)
    cfg = parse_params(params)
    w, h = int(cfg["imgw"]), int(cfg["imgh"])
    xs, ys = np.meshgrid(np.arange(w) + 0.5, np.arange(h) + 0.5)
    cx, cy = xs.ravel() / w * 2 - 1, ys.ravel() / h * 2 - 1
    gaze, up = np.array(cam.gaze, np.float64), np.array(cam.up, np.float64)
    hand = np.cross(gaze, up)
    hand /= np.linalg.norm(hand) + 1e-8
    fh = 2 * np.tan(cam.fov * 3.14159 / 180 / 2)
    fw = fh * cam.aspect
    d = gaze[None] + hand[None] * (fw * cx * 0.5)[:, None] - up[None] * (fh * cy * 0.5)[:, None]
    d /= np.linalg.norm(d, axis=1, keepdims=True) + 1e-8
    o = np.tile(np.array(cam.pos, np.float64), (d.shape[0], 1))
    tri = scene.intersect(o.astype(np.float32), d.astype(np.float32))[0]
    m = np.where(tri >= 0, np.asarray(sc["mat"])[np.maximum(tri, 0)], -1)
    return np.bincount(m[m >= 0], minlength=len(sc["mats"])) / float(m.size)


TARGET_SEED = 1000003


def eval_loss(scene, mats, P, params, target):
    """Image loss at parameters P with the target's own samples (common random
    numbers), so it measures the parameter mismatch and not Monte Carlo noise."""
    scene.set_materials(apply(mats, P))
    img = scene.render(params + f" seed={TARGET_SEED}")
    return float(np.mean((img.astype(np.float64) - target) ** 2))


def optimize(scene, sc, params, steps=100, lr=0.02, perturb=0.3, seed=0, log_every=0, fix_emission=False,
             min_coverage=0.0):
    """Runs the recovery on a Scene built from `sc`; returns a history dict
    with the per-step loss, the relative parameter error over the parameters
    that receive gradient, and the common-random-number loss before / after.
    fix_emission keeps the emitters at their true radiance; min_coverage
    leaves materials seen in fewer pixels than that at their true values."""
    mats = sc["mats"]
    P_true, mask = param_table(mats)
    if fix_emission:
        mask[:, EMIT] = False
    if min_coverage > 0.0:
        cov = coverage(scene, sc, params)
        mask &= (cov >= min_coverage)[:, None]
    target = scene.render(params + f" seed={TARGET_SEED}")
    rng = np.random.default_rng(seed)
    # only the optimised parameters start perturbed; the rest stay at their true values
    P = np.where(mask, clamp(P_true * rng.uniform(1 - perturb, 1 + perturb, size=P_true.shape), mask), P_true)
    scale = np.where(mask, np.maximum(np.abs(P_true), 1e-3), 1.0)  # Adam in units of each parameter's size
    m = np.zeros_like(P)
    v = np.zeros_like(P)
    b1, b2, eps = 0.9, 0.999, 1e-8
    hist = {"loss": [], "param_err": [], "ms": []}
    npx = target.size
    P0 = P.copy()
    seen = np.zeros_like(mask)  # parameters the image constrains (nonzero gradient at some step)
    hist["eval_loss0"] = eval_loss(scene, mats, P, params, target)
    t0 = time.perf_counter()
    for k in range(steps):
        scene.set_materials(apply(mats, P))
        p = params + f" seed={k + 1}"
        img = scene.render(p)
        diff = img.astype(np.float64) - target
        loss = float(np.mean(diff ** 2))
        # the adjoint on samples independent of the image's, so that its
        # product with the image error is an unbiased gradient of the loss
        # of the expected image
        pa = params + f" seed={k + 1 + 1000}"
        g = scene.adjoint(pa, (2.0 * diff / npx).astype(np.float32)).astype(np.float64)
        g = np.where(mask, g * scale, 0.0)
        seen |= g != 0.0
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        step = lr * (m / (1 - b1 ** (k + 1))) / (np.sqrt(v / (1 - b2 ** (k + 1))) + eps)
        P = clamp(P - step * scale, mask)
        sel = mask & seen
        perr = float(np.sqrt(np.sum(((P - P_true) / scale)[sel] ** 2) / max(1, sel.sum())))
        hist["loss"].append(loss)
        hist["param_err"].append(perr)
        hist["ms"].append((time.perf_counter() - t0) * 1e3)
        if log_every and (k % log_every == 0 or k == steps - 1):
            print(f"step {k:3d} loss {loss:.6g} relative parameter error {perr:.4f}", flush=True)
    sel = mask & seen
    hist["param_err0"] = float(np.sqrt(np.sum(((P0 - P_true) / scale)[sel] ** 2) / max(1, sel.sum())))
    hist["eval_loss"] = eval_loss(scene, mats, P, params, target)
    hist["params_constrained"] = int(sel.sum())
    hist["params_optimised"] = int(mask.sum())
    hist["final_params"] = P
    scene.set_materials(mats)
    return hist
