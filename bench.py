"""ptnee throughput benchmark (Mpaths/s) on the 1M-triangle procedural scene.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step renders one full frame of the workload: the seeded 1M-triangle
terrain + spheres scene, 1920x1080, 64 samples per pixel, max depth 8,
Russian roulette from depth 3, Philox seed 0 (132.7 M camera paths). The
scene (BVH, triangles, materials) and the path state live in HBM; both are
larger than the 129 MB L2 (about 150 MB of scene and 24 GB of path state:
the whole frame is one wavefront batch of up to 2^27 paths), so no L2
flush is inserted between steps.

value: paths / s with the scene resident and the image left on the device
(nr_render with no host output), timed with CUDA events on the library's
stream. e2e: the same render through nr_render with a pinned host output
image, so the 24.9 MB device-to-host copy is inside the timed region.
roofline: k_trace's algorithmic bytes (32 B per visited node, 36 B per
tested triangle) per second against the measured copy bandwidth; beside it
the issue roofline of k_trace and k_shadow (both issue-bound), and the whole
path's bytes. c3 / c5_adjoint (after the timed steps, own clocks): frames of
the third workload (sky with importance sampling, textures, dielectrics, 256
spp) and gradients of the inverse-rendering workload, timed the same way.
time_to_relmse (not part of `value`): the metric's second half, plain PT
against PT + the online neural radiance cache, at 1920x1080 and 64 spp per
frame (the fourth workload), and at 960x540 and 1 spp per frame.

Multi-GPU (torchrun): every rank renders its own 64-sample range of the
frame (sample0 = 64 * rank) with no collective on the data path (weak
scaling); timing takes the max over ranks.

--impl reference times the reference algorithm on the host cores: the CPU
restatement in oracle/ (bit-identical to the reference on x86; the
reference sources themselves are not present on the GPU host), all threads,
on a bounded pixel sample of the same workload per step.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MEASURED = os.path.join(ROOT, "MEASURED_PEAKS.json")
# Algorithmic bytes of the closest-hit walk: 32 B per visited node (one
# FP32 child box) and 36 B per tested triangle (three FP32 vertices), times
# the visits and tests counted by an instrumented frame of the workload.
BYTES_NODE = 32
BYTES_TRI = 36
# Figures that come from one ncu capture of the workload, not from this run:
# per bounce-0 closest-hit ray of k_trace, its DRAM bytes (read + write) and
# cache sector hit rates; per ray of k_trace and k_shadow, their warp
# instructions (smsp__inst_executed.sum over the launch's rays), which give
# the issue roofline: instructions / (SMs x 4 schedulers x clock x time).
NCU_CAPTURE = {
    "what": "ncu captures of a 480x270 x 32 spp frame of the same scene: DRAM bytes and hit rates of the bounce-0 "
            "k_trace launch; warp instructions of all of the frame's k_trace / k_shadow launches over its rays",
    "k_trace": {"dram_bytes_per_ray": 63.1, "l2_hit_rate": 0.661, "l1_hit_rate": 0.823,
                "warp_inst_per_ray": 248.8},
    "k_shadow": {"warp_inst_per_ray": 299.2},
}
SM_COUNT = 152


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--res", default="1920x1080")
    ap.add_argument("--wave", type=int, default=0, help="paths per wavefront batch (0: library default)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-tile-stride", type=int, default=4, help="CPU sample: every k-th 4x4 tile")
    ap.add_argument("--no-relmse", action="store_true", help="skip the time-to-relMSE comparison")
    ap.add_argument("--relmse-res", default="1920x1080",
                    help="frame of the time-to-relMSE comparison at 64 spp per frame (the 1-spp-per-frame leg "
                         "runs at 960x540)")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the third workload's frame and the adjoint leg of the default line")
    ap.add_argument("--nrc", default=None, metavar="PARAMS",
                    help="each step is a PT + NRC frame: a fresh cache is attached and the render gets "
                         "'nrc=1 nrc_train=16384 PARAMS' (measures the cache's per-frame cost)")
    ap.add_argument("--params", default="", metavar="KEY=VALUE ...",
                    help="extra renderer parameters appended to the workload's (e.g. 'tile=2')")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c5"],
                    help="c2: the 1M-triangle scene (default); c3: the same with an HDR sky, value-noise "
                         "textures on half the materials and 10%% GGX dielectrics, spp 256; c5: the path-replay "
                         "adjoint on the 200k-triangle, 64-material inverse-rendering scene (512x512, spp 32, "
                         "depth 4), one gradient per step")
    args = ap.parse_args()
    if args.nrc is not None:
        args.no_relmse = True  # the comparison attaches caches of its own
    return args


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    from nuray_gb300 import scenes
    sc = scenes.terrain_spheres(0)
    if args.workload == "c3":
        sc = scenes.with_env_textures(sc, 0)
        if args.spp == 64:
            args.spp = 256
    w, h = (int(x) for x in args.res.split("x"))
    params = sc["params"].replace("imgw=1920", f"imgw={w}").replace("imgh=1080", f"imgh={h}")
    params = params.replace("spp=64", f"spp={args.spp}").replace("spp=256", f"spp={args.spp}")
    if args.wave:
        params += f" wave={args.wave}"
    if args.workload == "c3":
        params += " envis=1"  # the environment map's importance sampling (IBL) the workload names
    if args.params:
        params += " " + args.params
    desc = (f"procedural terrain+spheres, {sc['pos'].shape[0]} triangles, {w}x{h}, spp={args.spp}, "
            "maxdepth 8, RR from depth 3, GGX-reflect materials, 32 quad lights, Philox seed 0")
    if args.workload == "c3":
        desc += (", 2048x1024 HDR sky (peak 5e3) with environment importance sampling (envis=1), 512x512 "
                 "value-noise textures on half the materials, 10% GGX dielectrics")
    return sc, params, desc, w, h


def peaks():
    try:
        return json.load(open(MEASURED)), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.rows.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_sample_pixels(w, h, stride):
    tiles = [(x, y) for y in range(0, h, 4) for x in range(0, w, 4)]
    pix = []
    for k, (x0, y0) in enumerate(tiles):
        if k % stride == 0:
            pix += [(x, y) for y in range(y0, min(h, y0 + 4)) for x in range(x0, min(w, x0 + 4))]
    return np.array(pix, np.int32)


def cpu_leg(sc, params, spp, w, h, stride, budget_s=20.0):
    """The oracle restatement on all host threads over a pixel sample; returns
    (Mpaths/s, description, threads)."""
    from oracle.bind import Oracle
    P = Oracle("port", sc)
    threads = os.cpu_count() or 1
    pix = cpu_sample_pixels(w, h, stride)
    # calibrate on a small slice, then size the timed sample to the time target
    probe = pix[:: max(1, len(pix) // 256)]
    t = time.perf_counter()
    P.render_samples(params, probe, spp, threads=threads)
    rate = len(probe) * spp / max(1e-6, time.perf_counter() - t)
    n = int(min(len(pix), max(64, budget_s * rate / spp)))
    pix = pix[:n]
    t = time.perf_counter()
    P.render_samples(params, pix, spp, threads=threads)
    dt = time.perf_counter() - t
    desc = (f"{n} pixels (every {stride}th 4x4 tile, first {n}) x {spp} spp of the same frame, "
            f"{n * spp} paths in {dt:.1f} s")
    return n * spp / dt / 1e6, desc, threads


def relmse_leg(S, params, res, target=1e-3, ref_spp=8192, limit_s=45.0, spf=64, res_1spp="960x540"):
    """Second half of the metric: wall time (CUDA events) to relMSE <= 1e-3
    against a converged render, plain PT against PT + the online neural
    radiance cache, both progressive with the same frame size: `spf`
    samples per pixel per frame (64: near the fastest frame size of either
    method on this scene) on the `res` frame (the fourth workload's
    1920x1080), and one sample per pixel per frame on a `res_1spp` frame
    (the real-time regime, where fixed per-frame costs weigh most)."""
    from nuray_gb300 import convergence as C
    out = {"target": target, "resolution": res, "reference_spp": ref_spp, "unit": "ms", "spp_per_frame": spf}
    refs = {}
    for k, r, label in ((spf, res, None), (1, res_1spp, "at_1_spp_per_frame")):
        w, h = r.split("x")
        p = params.replace("imgw=1920", f"imgw={w}").replace("imgh=1080", f"imgh={h}")
        if r not in refs:
            refs[r] = C.reference(S, p, ref_spp)
        ref = refs[r]
        pt_curve, pt_t = C.progressive(S, p, 100000, ref, target, time_limit_s=limit_s, spf=k)
        nrc_curve, nrc_t = C.run_nrc(S, p, ref, target, 100000, "", limit_s, warmup=max(1, 256 // k),
                                     spf=k)
        res_k = {"pt": C.summary(pt_curve, pt_t, target), "pt_nrc": C.summary(nrc_curve, nrc_t, target)}
        if label:
            res_k["resolution"] = r
            out[label] = res_k
        else:
            out.update(res_k)
    out["note"] = ("GPU time (CUDA events) of the frames up to the first checkpoint at or below the target; "
                   "'spp' is the samples per pixel at that checkpoint; None when not reached within the time limit; "
                   "'ms_to_target_interp' interpolates the time of the crossing in log-log between the checkpoints "
                   "on either side of it (checkpoints lie about 3 % apart in samples)")
    return out


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm on the host cores."""
    if rank != 0:
        return
    sc, params, desc, w, h = workload(args)
    from oracle.bind import Oracle
    P = Oracle("port", sc)
    threads = os.cpu_count() or 1
    pix = cpu_sample_pixels(w, h, 256)
    spp = args.spp
    for _ in range(args.warmup):
        P.render_samples(params, pix[:16], spp, threads=threads)
    t = time.perf_counter()
    for k in range(args.steps):
        P.render_samples(params, pix, spp, sample0=spp * k, threads=threads)
    dt = time.perf_counter() - t
    v = len(pix) * spp * args.steps / dt / 1e6
    sample = f"{len(pix)} pixels (every 256th 4x4 tile) x {spp} spp per step"
    out = {"impl": "reference", "metric": "Mpaths/s ptnee", "value": round(v, 4), "unit": "Mpaths/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(dt / args.steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
           "config": {"workload": desc, "host_threads": threads},
           "cpu_baseline": {"value": round(v, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": round(v, 4), "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def adjoint_leg(steps, warmup, extra_params="", clock_index=0):
    """One nr_adjoint call per step on the 200k-triangle, 64-material
    inverse-rendering workload (512x512, 32 spp, depth 4, RR from 3): a
    render pass that records every bounce's hits and light-sample visibility,
    then the adjoint replay of every path from those records, for a fixed
    seeded d loss / d image; the per-material gradient comes back to the
    host inside the timed region. Returns the measurements and the clocks."""
    import torch
    from nuray_gb300 import Scene, build, inverse
    build.build()
    sc = inverse.c5_scene(0)
    S = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"])
    params = sc["params"] + (" " + extra_params if extra_params else "")
    w = h = 512
    spp = 32
    rng = np.random.default_rng(7)
    dl = (rng.standard_normal((h, w, 3)) / (w * h * 3)).astype(np.float32)
    S.render_device(params.replace("spp=32", "spp=1") + " count=1")
    cnt = S.stats()
    stream = torch.cuda.ExternalStream(S.stream())
    for k in range(warmup):
        S.adjoint(params + f" seed={k + 1}", dl)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(clock_index) as clk:
        e0.record(stream)
        for k in range(steps):
            S.adjoint(params + f" seed={100 + k}", dl)
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    paths = w * h * spp * steps
    paths1 = max(1, cnt["paths"])
    b_path = ((32 * cnt["nodes_visited"] + 36 * cnt["tris_tested"] + 32 * cnt["shadow_nodes_visited"]
               + 36 * cnt["shadow_tris_tested"]) / paths1 + 240 * cnt["rays"] / paths1 + 12)
    # render pass: traversal and shading as in the ptnee frame, plus the hit
    # record and visibility byte written per ray; replay: per ray the record
    # read again, the shading reads (240 B) and the adjoint slot state (64 B)
    rays_pp = cnt["rays"] / paths1
    b_adj = b_path + rays_pp * (17 + 17 + 240 + 64) + 12
    out = {"value": paths / (ms / 1e3) / 1e6, "ms_per_step": ms / steps, "paths_per_step": w * h * spp,
           "bytes_per_path": b_adj, "gbs": b_adj * paths / (ms / 1e3) / 1e9,
           "launches": steps * S.stats()["kernel_launches"],
           "workload": f"path-replay adjoint, {sc['pos'].shape[0]} triangles, {len(sc['mats'])} materials, "
                       f"{w}x{h}, spp={spp}, maxdepth 4, RR from depth 3"}
    S.close()
    return out, clk.summary()


def run_adjoint(args, local):
    """--workload c5: the adjoint leg as the line's own metric."""
    r, clocks = adjoint_leg(args.steps, args.warmup, args.params, local)
    pk, pk_kind = peaks()
    peak = pk.get("hbm_gbs", 6800.0)
    out = {"metric": "Mpaths/s adjoint", "value": round(r["value"], 3), "unit": "Mpaths/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(r["ms_per_step"], 2),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded procedural scene, seeded d loss / d image)",
           "config": {"workload": r["workload"], "paths_per_step": r["paths_per_step"]},
           "roofline": {"kernel": "render pass with hit records + recorded replay", "bound": "hbm",
                        "achieved": round(r["gbs"], 1), "peak": peak, "unit": "GB/s",
                        "frac": round(r["gbs"] / peak, 3), "peak_source": pk_kind, "traffic": None,
                        "bytes_per_path": round(r["bytes_per_path"], 1),
                        "formula": "ptnee path bytes + rays x (17 record write + 17 read + 240 shading + 64 adjoint "
                                   "state) + 12"},
           "gpu_launches": r["launches"], "cpu_baseline": None, "e2e": None, "clocks": clocks}
    print(json.dumps(out), flush=True)


def c3_leg(steps, warmup, clock_index=0):
    """Frames of the third workload (the 1M-triangle scene with the HDR sky
    and its importance sampling, value-noise textures on half the materials,
    10 % GGX dielectrics; 1920x1080 at 256 spp: four waves of 2^27 paths),
    timed like the main frames."""
    import torch
    from nuray_gb300 import Scene, scenes
    sc = scenes.with_env_textures(scenes.terrain_spheres(0), 0)
    S = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"], textures=sc["textures"],
                          env_tex=sc["env_tex"], env_gain=sc["env_gain"])
    params = sc["params"] + " envis=1"
    stream = torch.cuda.ExternalStream(S.stream())
    for _ in range(warmup):
        S.render_device(params)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches = 0
    with ClockSampler(clock_index) as clk:
        e0.record(stream)
        for _ in range(steps):
            S.render_device(params)
            launches += S.stats()["kernel_launches"]
        e1.record(stream)
        e1.synchronize()
    ms = e0.elapsed_time(e1)
    paths = 1920 * 1080 * 256
    S.close()
    return {"value": round(paths * steps / (ms / 1e3) / 1e6, 3), "unit": "Mpaths/s", "steps": steps,
            "warmup": warmup, "ms_per_step": round(ms / steps, 2), "paths_per_step": paths, "gpu_launches": launches,
            "workload": "procedural terrain+spheres, 991296 triangles, 1920x1080, spp=256, maxdepth 8, RR from depth "
                        "3, 2048x1024 HDR sky (peak 5e3) with environment importance sampling (envis=1), 512x512 "
                        "value-noise textures on half the materials, 10% GGX dielectrics",
            "clocks": clk.summary()}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "c5":
        if rank == 0:
            run_adjoint(args, local)
        return
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from nuray_gb300 import Scene, build
    build.build()
    sc, params, desc, w, h = workload(args)
    t0 = time.perf_counter()
    S = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"], textures=sc["textures"],
                          env_tex=sc["env_tex"], env_gain=sc["env_gain"])
    build_s = time.perf_counter() - t0
    bvh_host_ms = S.build_times()[0]
    # the same tree built on the device (setup only; the timed steps use S)
    G = Scene.from_arrays(sc["pos"], sc["mat"], sc["mats"], uv=sc["uv"], nrm=sc["nrm"], textures=sc["textures"],
                          env_tex=sc["env_tex"], env_gain=sc["env_gain"], options="bvh=gpu")
    bvh_gpu_wall_ms, bvh_gpu_dev_ms = G.build_times()
    G.close()
    del G
    stream = torch.cuda.ExternalStream(S.stream())
    cache = None
    if args.nrc is not None:
        from nuray_gb300.nrc import Cache
        cache = Cache("lr=1e-3 beta1=0.9 beta2=0.99")
        cache.attach(S)
        params += " nrc=1 nrc_train=16384 " + args.nrc
    from nuray_gb300.shard import max_over_ranks, sample_range
    sample0, spp = sample_range(rank, world, args.spp, "weak")
    base = params + f" sample0={sample0}"

    # untimed instrumented frame: traversal work per ray for the roofline bytes
    S.render_device(base.replace(f"spp={spp}", "spp=1") + " count=1")
    cnt = S.stats()
    for _ in range(args.warmup):
        S.render_device(base + " profile=1")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    trace_ms, shadow_ms, trace_launches, rays, shadow_rays, launches = 0.0, 0.0, 0, 0, 0, 0
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for k in range(args.steps):
            S.render_device(base + " profile=1")
            st = S.stats()
            trace_ms += st["kernel_ms_trace"]
            shadow_ms += st["kernel_ms_shadow"]
            trace_launches += st["trace_launches"]
            rays += st["rays"]
            shadow_rays += st["shadow_rays"]
            launches += st["kernel_launches"]
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, "cuda")
    paths_total = float(w * h * spp * args.steps * world)
    value = paths_total / (ms / 1e3) / 1e6

    # end to end through the C ABI with a pinned host image
    e2e = None
    if not args.no_e2e:
        host = torch.empty((h, w, 3), dtype=torch.float32, pin_memory=True)
        hp = host.data_ptr()
        from nuray_gb300._lib import check, lib
        barrier()
        t = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            check(lib().nr_render(S._h, None, base.encode(), ctypes.c_void_p(hp), None, None, None, None))
        e1.record(stream)
        e1.synchronize()
        barrier()
        ems = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
        e2e = {"value": round(paths_total / (ems / 1e3) / 1e6, 3), "unit": "Mpaths/s",
               "h2d_bytes_per_step": len(base.encode()) + 44, "d2h_bytes_per_step": w * h * 3 * 4,
               "ms_per_step": round(ems / args.steps, 2)}
        launches_e2e = S.stats()["kernel_launches"] + 1

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    pk, pk_kind = peaks()
    clocks = clk.summary()
    # k_trace: the closest-hit walk's algorithmic bytes (32 B per visited
    # node, 36 B per tested triangle, counts of an instrumented frame) per
    # extension ray, x rays, / the summed CUDA-event time of its launches
    bytes_per_ray = (BYTES_NODE * cnt["nodes_visited"] + BYTES_TRI * cnt["tris_tested"]) / max(1, cnt["rays"])
    trace_bytes = bytes_per_ray * rays
    achieved = trace_bytes / (trace_ms / 1e3) / 1e9 if trace_ms > 0 else None
    peak = pk.get("hbm_gbs", 6800.0)
    roof = {"kernel": "k_trace (closest hit + material sort)", "bound": "hbm",
            "achieved": round(achieved, 1) if achieved else None, "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 3) if achieved else None, "peak_source": pk_kind,
            "traffic": None,
            "bytes_per_ray": round(bytes_per_ray, 1),
            "bytes_formula": "32 B x nodes visited + 36 B x triangles tested per extension ray",
            "nodes_per_ray": round(cnt["nodes_visited"] / max(1, cnt["rays"]), 2),
            "tris_per_ray": round(cnt["tris_tested"] / max(1, cnt["rays"]), 2),
            "avg_launch_ms": round(trace_ms / max(1, trace_launches), 4),
            "share_of_step": round(trace_ms / ms, 3)}
    tr = NCU_CAPTURE["k_trace"]
    roof["traffic"] = round(tr["dram_bytes_per_ray"] * rays / max(1, trace_launches))
    roof["ncu_capture"] = {"source": NCU_CAPTURE["what"] + " (constants, not measured in this run)",
                           "dram_bytes_per_ray": tr["dram_bytes_per_ray"], "l2_hit_rate": tr["l2_hit_rate"],
                           "l1_hit_rate": tr["l1_hit_rate"],
                           "traffic_formula": "dram_bytes_per_ray x extension rays per launch"}
    # issue roofline of the traversal kernels: warp instructions (per ray, from
    # the capture) x rays / (SMs x 4 issue slots per clock x the sampled SM
    # clock x the kernels' CUDA-event time)
    mhz = clocks.get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    issue = {"unit": "warp instructions / issue slot", "sm_mhz": mhz,
             "formula": "warp_inst_per_ray x rays / (152 SMs x 4 x SM clock x kernel time)"}
    for name, nrays, kms in (("k_trace", rays, trace_ms), ("k_shadow", shadow_rays, shadow_ms)):
        ipr = NCU_CAPTURE[name]["warp_inst_per_ray"]
        if ipr and kms > 0:
            slots = SM_COUNT * 4 * mhz * 1e6 * kms / 1e3
            issue[name] = {"warp_inst_per_ray": ipr, "frac": round(ipr * nrays / slots, 3),
                           "kernel_ms_per_step": round(kms / args.steps, 2)}
    roof["issue"] = issue
    # the whole path's algorithmic bytes, per path:
    # sum over rays (32 B per node, 36 B per triangle) + 240 B per shaded
    # vertex (hit attributes, material, path state, hit record) + 12 B film
    paths1 = max(1, cnt["paths"])
    b_path = ((32 * cnt["nodes_visited"] + 36 * cnt["tris_tested"] + 32 * cnt["shadow_nodes_visited"]
               + 36 * cnt["shadow_tris_tested"]) / paths1 + 240 * cnt["rays"] / paths1 + 12)
    path_gbs = value * 1e6 * b_path / 1e9
    roof["path"] = {"bytes_per_path": round(b_path, 1), "achieved": round(path_gbs, 1),
                    "frac": round(path_gbs / peak, 3),
                    "formula": "sum_rays(32 N_node + 36 N_tri) + 240 per shaded vertex + 12, counts of an "
                               "instrumented frame, x paths/s"}

    cpu = None
    if not args.no_cpu and world == 1:
        v, sample, threads = cpu_leg(sc, params, spp, w, h, args.cpu_tile_stride)
        cpu = {"value": round(v, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": sample}

    out = {"metric": "Mpaths/s ptnee" + ("+nrc" if cache else ""), "value": round(value, 3), "unit": "Mpaths/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 2),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded procedural scene; the reference publishes no benchmark scene)",
           "config": {"workload": desc, "triangles": int(sc["pos"].shape[0]), "paths_per_step": w * h * spp,
                      "l2": "inputs larger than L2 (scene ~150 MB, path state ~24 GB); no flush",
                      "parallelism": f"{world} rank(s), disjoint sample ranges, no collective on the data path",
                      "scene_build_s": round(build_s, 2),
                      "bvh_build_ms": {"host_threads": round(bvh_host_ms, 1), "gpu_wall": round(bvh_gpu_wall_ms, 1),
                                       "gpu_device": round(bvh_gpu_dev_ms, 1)}},
           "rays_per_s": round((rays + shadow_rays) / (ms / 1e3), 1), "extension_rays": rays,
           "shadow_rays": shadow_rays, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
           "e2e": e2e, "clocks": clocks}
    if e2e:
        out["gpu_launches_e2e"] = launches_e2e * args.steps
    if not args.no_extra and world == 1 and args.workload == "c2" and cache is None:
        # the other two GPU workloads, timed the same way (their own clocks)
        out["c3"] = c3_leg(max(2, args.steps // 4), 1, local)
        r, c5_clocks = adjoint_leg(max(5, args.steps), 2, "", local)
        out["c5_adjoint"] = {"value": round(r["value"], 3), "unit": "Mpaths/s of gradient",
                             "ms_per_step": round(r["ms_per_step"], 2), "paths_per_step": r["paths_per_step"],
                             "steps": max(5, args.steps), "warmup": 2, "gpu_launches": r["launches"],
                             "workload": r["workload"], "hbm_gbs": round(r["gbs"], 1),
                             "bytes_per_path": round(r["bytes_per_path"], 1), "clocks": c5_clocks}
    if not args.no_relmse and world == 1:
        out["time_to_relmse"] = relmse_leg(S, params, args.relmse_res)
    print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
