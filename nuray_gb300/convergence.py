"""Time to a relMSE target: plain GPU path tracing against PT + the online
neural radiance cache, both progressive (frames of `spf` samples per pixel,
accumulated) on the same scene and GPU.

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


def progressive(scene, params, frames, ref, target, nrc=None, nrc_params="", time_limit_s=60.0, growth=1.03,
                warmup=0, spf=1):
    """Renders up to `frames` frames of `spf` samples per pixel (default 1),
    accumulated on the device; the
    image is read back and compared at checkpoints spaced by `growth` in
    sample count. With a cache, the first `warmup` frames are plain path
    tracing that only trains it (unbiased samples that count towards the
    image); later frames end paths in the cache. Returns (elapsed_ms, spp,
    relmse) rows and the elapsed GPU time at the first checkpoint that meets
    `target`."""
    import torch
    stream = torch.cuda.ExternalStream(scene.stream())
    curve = []
    hit = None
    elapsed = 0.0
    next_check = 1.0
    t_wall = time.perf_counter()
    for k in range(frames):
        p = params.replace("spp=", "spp_unused=") + f" spp={spf} sample0={k * spf}" + (" accumulate=1" if k else "")
        if nrc is not None:
            p += " nrc=1 " + nrc_params + (" nrc_query=0" if k < warmup else "")
        check = k + 1 >= next_check or k == frames - 1
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        img = scene.render(p) if check else scene.render_device(p)
        e1.record(stream)
        e1.synchronize()
        elapsed += e0.elapsed_time(e1)
        if check:
            next_check = max(next_check * growth, k + 2)
            err = relmse(img, ref)
            curve.append((round(elapsed, 2), (k + 1) * spf, err))
            if err <= target:
                hit = elapsed
                break
        if time.perf_counter() - t_wall > time_limit_s:
            break
    return curve, hit


def reference(scene, params, ref_spp=8192, seed_ref=12345):
    return scene.render(params.replace("spp=", "spp_unused=") + f" spp={ref_spp} seed={seed_ref}")


def run_nrc(scene, params, ref, target, frames, nrc_params, time_limit_s, warmup=256, spf=1):
    from ._lib import check, lib
    from .nrc import Cache
    cache = Cache("lr=1e-3 beta1=0.9 beta2=0.99")
    cache.attach(scene)
    try:
        return progressive(scene, params, frames, ref, target, nrc=cache, nrc_params=nrc_params,
                           time_limit_s=time_limit_s, warmup=warmup, spf=spf)
    finally:
        check(lib().nr_scene_attach_nrc(scene._h, None))
        cache.close()


def crossing(curve, target):
    """GPU time at which relMSE reaches `target`, interpolated in log-log
    between the last checkpoint above it and the first at or below it (the
    checkpoints lie a few percent apart in sample count); None when the
    curve does not cross it."""
    import math
    for (t0, _, e0), (t1, _, e1) in zip(curve, curve[1:]):
        if e0 > target >= e1 and e0 > 0 and e1 > 0 and t0 > 0:
            if e0 == e1:
                return t1
            w = math.log(e0 / target) / math.log(e0 / e1)
            return math.exp(math.log(t0) + w * (math.log(t1) - math.log(t0)))
    return None


def summary(curve, t, target=1e-3):
    x = crossing(curve, target)
    return {"ms_to_target": None if t is None else round(t, 1), "spp": curve[-1][1], "final_relmse": curve[-1][2],
            "ms_to_target_interp": None if x is None else round(x, 1)}


def compare(scene, params, target=1e-3, ref_spp=8192, frames=50000, nrc_params="", time_limit_s=60.0):
    """Plain PT and PT + NRC against the same reference; returns both summaries and curves."""
    ref = reference(scene, params, ref_spp)
    pt_curve, pt_t = progressive(scene, params, frames, ref, target, time_limit_s=time_limit_s)
    nrc_curve, nrc_t = run_nrc(scene, params, ref, target, frames, nrc_params, time_limit_s)
    return {"target": target, "ref_spp": ref_spp, "pt": summary(pt_curve, pt_t), "pt_nrc": summary(nrc_curve, nrc_t),
            "pt_curve": pt_curve[:: max(1, len(pt_curve) // 32)], "nrc_curve": nrc_curve[:: max(1, len(nrc_curve) // 32)]}
