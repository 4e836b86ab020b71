"""nr_intersect_noalloc, the entry point for callers that cannot let the
library allocate device memory while they run (fixed memory budgets,
real-time loops that must not pay cudaMalloc's implicit synchronisation).
It stages rays through a static device array instead of cudaMalloc'd
scratch; its hits must equal nr_intersect's exactly (closest-hit ids are
integers and t, b1, b2 come from the same arithmetic), on two calls in a row
since the array keeps the previous call's contents.

Named to be collected last, so a run that stops at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden

pytestmark = pytest.mark.gpu


def _max_rays():
    """NR_NOALLOC_MAX_RAYS as the public header defines it (the library's
    limit and its array size come from the same definition)."""
    text = open(os.path.join(ROOT, "include", "nuray.h")).read()
    return int(re.search(r"#define NR_NOALLOC_MAX_RAYS (\d+)", text).group(1))


def _scene():
    from nuray_gb300 import Scene
    g = golden("cornell_scene.npz")
    mats = [dict(type=int(i[0]), c0=f[0:3].tolist()) for i, f in zip(g["mat_i"], g["mat_f"])]
    return Scene.from_arrays(g["pos"], g["mat"], mats, uv=g["uv"], nrm=g["nrm"])


def _noalloc(S, o, d):
    from nuray_gb300._lib import _ptr, check, lib
    n = o.shape[0]
    tri = np.full(n, -7, np.int32)
    t, b1, b2 = (np.full(n, -7.0, np.float32) for _ in range(3))
    check(lib().nr_intersect_noalloc(S._h, n, _ptr(o), _ptr(d), _ptr(tri), _ptr(t), _ptr(b1), _ptr(b2)))
    return tri, t, b1, b2


def test_noalloc_intersect_matches_intersect_twice(gpu_lib):
    S = _scene()
    g = golden("cornell_intersect.npz")
    rng = np.random.default_rng(11)
    batches = [(g["o"], g["d"])]
    o2 = rng.uniform(-60, 60, size=(3001, 3)).astype(np.float32) + np.array([0, 100, 0], np.float32)
    d2 = rng.normal(size=(3001, 3)).astype(np.float32)
    d2 /= np.linalg.norm(d2, axis=1, keepdims=True)
    batches.append((o2, d2))
    for o, d in batches:  # two calls in a row through the same static array
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        want = S.intersect(o, d)
        got = _noalloc(S, o, d)
        for a, b in zip(got, want):
            np.testing.assert_array_equal(a, b)
    assert (want[0] >= 0).any() and (want[0] < 0).any()


def test_noalloc_rejects_batches_over_the_limit(gpu_lib):
    from nuray_gb300 import NuRayError
    from nuray_gb300._lib import _ptr, check, lib
    S = _scene()
    limit = _max_rays()
    n = limit + 1
    o = np.zeros((n, 3), np.float32)
    d = np.tile(np.array([0, 0, -1], np.float32), (n, 1))
    out = [np.zeros(n, np.int32)] + [np.zeros(n, np.float32) for _ in range(3)]
    with pytest.raises(NuRayError, match=f"at most {limit} rays"):
        check(lib().nr_intersect_noalloc(S._h, n, _ptr(o), _ptr(d), *[_ptr(a) for a in out]))
    # the full limit is accepted
    tri, t, _, _ = _noalloc(S, o[:limit], d[:limit])
    assert tri.shape == (limit,)
