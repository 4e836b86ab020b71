"""Sharding one frame over ranks (one process per GPU).

Path (pixel, sample) draws every uniform from its own Philox4x32-10 stream
keyed by the pixel and the sample index, so the set of paths a frame
traces does not depend on how the sample range is split: rank r rendering
samples [s0, s0 + n) traces exactly the paths a single process traces for
those indices. The data path therefore needs no collective; the only
exchange, when one image is wanted, is one FP32 sum of the per-pixel
radiance sums (the films of disjoint sample ranges add).

The reference renders one frame in one process (`RendererPTLS::render`,
src/renderer/rendererptls.cpp:96-236, a thread pool over shuffled tiles);
this module is the multi-GPU form of that loop.
"""


def sample_range(rank, world, spp, mode="weak"):
    """(sample0, count) of `rank`.

    weak: every rank renders `spp` samples of its own, [spp*rank, spp*rank + spp)
    (the work per GPU is fixed as ranks are added).
    strong: the `spp` samples of one frame are split into contiguous ranges
    whose sizes differ by at most one (the total is fixed)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of size {world}")
    if spp < 0:
        raise ValueError("spp must be >= 0")
    if mode == "weak":
        return spp * rank, spp
    if mode == "strong":
        base, extra = divmod(spp, world)
        return rank * base + min(rank, extra), base + (1 if rank < extra else 0)
    raise ValueError(f"unknown sharding mode {mode!r}")


def max_over_ranks(value, dist=None, device="cpu"):
    """The maximum of a per-rank float over all ranks (the slowest rank
    sets a step's time). Without a process group it is the value itself."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_film(film_sum, dist=None):
    """Sums per-pixel radiance sums (a float32 tensor, modified in place)
    over all ranks; the image is the sum divided by the total sample count."""
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(film_sum, op=dist.ReduceOp.SUM)
    return film_sum
