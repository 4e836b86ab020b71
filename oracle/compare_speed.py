"""Times the reference's own ptnee (oracle/_ref, compiled from its sources)
against the CPU restatement (oracle/_build) on the same samples of the
1M-triangle frame under the reference's own policy, same threads. TEST INFRASTRUCTURE: runs only where the
reference checkout exists (its objects do not travel to other machines).

    python oracle/compare_speed.py [threads] [pixels]
"""
import os
import platform
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import bind  # noqa: E402
from nuray_gb300 import scenes  # noqa: E402


def main(threads=None, npix=2048):
    threads = threads or os.cpu_count() or 1
    if bind.build_ref() is None:
        sys.exit("reference sources not found at " + bind.REF_ROOT)
    sc = scenes.terrain_spheres(0)
    # the reference's own policy (Russian roulette from the first vertex, no
    # depth limit): it does not read the rrdepth / maxdepth keys
    params = sc["params"].replace(" maxdepth=8", "").replace(" rrdepth=3", "")
    rng = np.random.default_rng(3)
    pix = np.stack([rng.integers(0, 1920, npix), rng.integers(0, 1080, npix)], 1).astype(np.int32)
    spp = 64
    out = {}
    for kind in ("port", "ref"):
        t = time.perf_counter()
        O = bind.Oracle(kind, sc)
        build_s = time.perf_counter() - t
        O.render_samples(params, pix[:16], spp, threads=threads)  # warm
        t = time.perf_counter()
        r = O.render_samples(params, pix, spp, threads=threads)
        dt = time.perf_counter() - t
        out[kind] = (r, dt, build_s)
        print(f"{kind:5s}: {npix * spp / dt / 1e6:.3f} Mpaths/s ({npix} pixels x {spp} spp in {dt:.2f} s, "
              f"{threads} threads); scene build incl. BVH {build_s:.1f} s", flush=True)
    same = np.mean(np.all(out["port"][0] == out["ref"][0], axis=2))
    print(f"machine: {platform.machine()}, {os.cpu_count()} cores; samples bit-identical: {same * 100:.2f}%; "
          f"restatement / reference speed: {out['ref'][1] / out['port'][1]:.2f}x")


if __name__ == "__main__":
    a = sys.argv[1:]
    main(int(a[0]) if a else None, int(a[1]) if len(a) > 1 else 2048)
