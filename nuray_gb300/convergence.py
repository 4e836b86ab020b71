"""Time to a relMSE target: plain GPU path tracing against PT + the online
neural radiance cache, both progressive (one sample per pixel per frame)
on the same scene and GPU.

relMSE = mean over pixels and channels of (I - R)^2 / (R^2 + 1e-2) on linear
HDR with FP64 sums, R a high-sample plain render with an independent seed.
Wall time counts everything the method does per frame (for PT + NRC the
cache queries and its online training), measured with CUDA events on the
library's stream.
"""
import time

import numpy as np


def relmse(img, ref):
    a = img.astype(np.float64)
    r = ref.astype(np.float64)
    return float(np.mean((a - r) ** 2 / (r ** 2 + 1e-2)))


def progressive(scene, params, frames, ref, target, nrc=None, nrc_params="", time_limit_s=60.0):
    """Renders up to `frames` 1-spp frames; returns the relMSE curve as
    (elapsed_ms, spp, relmse) rows and the time at which `target` is met."""
    import torch
    stream = torch.cuda.ExternalStream(scene.stream())
    acc = None
    curve = []
    hit = None
    elapsed = 0.0
    t_wall = time.perf_counter()
    for k in range(frames):
        p = params.replace("spp=", "spp_unused=") + f" spp=1 sample0={k}"
        if nrc is not None:
            p += " nrc=1 " + nrc_params
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        img = scene.render(p)
        e1.record(stream)
        e1.synchronize()
        elapsed += e0.elapsed_time(e1)
        acc = img.astype(np.float64) if acc is None else acc + img
        err = relmse(acc / (k + 1), ref)
        curve.append((round(elapsed, 2), k + 1, err))
        if hit is None and err <= target:
            hit = elapsed
            break
        if time.perf_counter() - t_wall > time_limit_s:
            break
    return curve, hit


def compare(scene, params, target=1e-3, ref_spp=4096, frames=4096, nrc_params="nrc_train=16384", seed_ref=12345,
            time_limit_s=60.0):
    """Returns a dict with the reference, the plain curve and the NRC curve."""
    from .nrc import Cache
    ref = scene.render(params.replace("spp=", "spp_unused=") + f" spp={ref_spp} seed={seed_ref}")
    pt_curve, pt_t = progressive(scene, params, frames, ref, target, time_limit_s=time_limit_s)
    cache = Cache("lr=1e-3 beta1=0.9 beta2=0.99")
    cache.attach(scene)
    try:
        nrc_curve, nrc_t = progressive(scene, params, frames, ref, target, nrc=cache, nrc_params=nrc_params,
                                       time_limit_s=time_limit_s)
    finally:
        from ._lib import check, lib
        check(lib().nr_scene_attach_nrc(scene._h, None))
        cache.close()
    return {"target": target, "ref_spp": ref_spp,
            "pt": {"ms_to_target": None if pt_t is None else round(pt_t, 1), "frames": pt_curve[-1][1],
                   "final_relmse": pt_curve[-1][2]},
            "pt_nrc": {"ms_to_target": None if nrc_t is None else round(nrc_t, 1), "frames": nrc_curve[-1][1],
                       "final_relmse": nrc_curve[-1][2]},
            "pt_curve": pt_curve[:: max(1, len(pt_curve) // 32)], "nrc_curve": nrc_curve[:: max(1, len(nrc_curve) // 32)]}
