"""Multi-rank host logic on the CPU: two gloo ranks split the sample range
of a frame; the oracle stands in for the per-rank renderer (each rank traces
its own range of the Cornell scene). The gathered per-sample radiance must be
bit-identical to one process tracing every sample, the reduced film must
equal the single-process film sum, and the step time is the max over ranks."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import golden
from nuray_gb300.shard import max_over_ranks, reduce_film, sample_range

PARAMS = "renderer=ptnee imgw=12 imgh=10 campos=0,120,200 cameuler=0,0,0 camfov=64 camasp=1.333 rrdepth=3 maxdepth=8"
SPP = 6


def cornell():
    g = golden("cornell_scene.npz")
    mats = [dict(type=int(i[0]), c0=f[0:3].tolist()) for i, f in zip(g["mat_i"], g["mat_f"])]
    return dict(pos=g["pos"], mat=g["mat"], mats=mats, uv=g["uv"], nrm=g["nrm"])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, mode, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle.bind import Oracle, pixel_grid
        O = Oracle("port", cornell())
        s0, n = sample_range(rank, world, SPP, mode)
        pix = pixel_grid(12, 10)
        rad = O.render_samples(PARAMS, pix, n, sample0=s0, threads=1) if n else np.zeros((pix.shape[0], 0, 3),
                                                                                          np.float32)
        film = torch.from_numpy(np.maximum(rad, 0).sum(1).astype(np.float32))
        reduce_film(film, dist)
        parts = [None] * world
        dist.all_gather_object(parts, (s0, rad))
        slowest = max_over_ranks(float(rank + 1), dist)
        if rank == 0:
            np.savez(os.path.join(out_dir, f"{mode}.npz"), film=film.numpy(), slowest=slowest,
                     starts=np.array([p[0] for p in parts]),
                     rad=np.concatenate([p[1] for p in sorted(parts, key=lambda p: p[0])], 1))
    finally:
        dist.destroy_process_group()


def test_sample_ranges():
    for spp in (0, 1, 5, 64, 257):
        for world in (1, 2, 3, 8):
            got = sorted(sample_range(r, world, spp, "strong") for r in range(world))
            covered = [s for s0, n in got for s in range(s0, s0 + n)]
            assert covered == list(range(spp))
            assert max(n for _, n in got) - min(n for _, n in got) <= 1
            assert [sample_range(r, world, spp)[0] for r in range(world)] == [spp * r for r in range(world)]
    with pytest.raises(ValueError):
        sample_range(2, 2, 4)
    with pytest.raises(ValueError):
        sample_range(0, 1, 4, "diagonal")


@pytest.mark.parametrize("mode", ["strong", "weak"])
def test_two_rank_split_matches_one_process(tmp_path, port_lib, mode):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), mode, str(tmp_path)), nprocs=world, join=True)
    r = dict(np.load(tmp_path / f"{mode}.npz"))
    total = SPP if mode == "strong" else SPP * world
    from oracle.bind import Oracle, pixel_grid
    one = Oracle("port", cornell()).render_samples(PARAMS, pixel_grid(12, 10), total, threads=2)
    assert np.array_equal(r["rad"], one)  # same paths, bit for bit
    np.testing.assert_allclose(r["film"], np.maximum(one, 0).sum(1), rtol=1e-6, atol=1e-6)
    assert float(r["slowest"]) == world
