"""Samples split over ranks: the reference's only parallel strategy (MPI
master/worker over samples, libcirc/innerprod.c:64-83 and
libcirc/probability.c:225-299), one process per GPU.

Each rank draws a contiguous block of the counter-based stream (state i of
stream `seed` is the same whoever draws it), evaluates its states on its own
GPU, and rank 0 gathers every state's value in index order.  The bin means and
the median are then computed exactly as on one GPU, so the sharded result is
bit-identical to the single-GPU one.  The only exchange is that gather of one
double per state: there is no data-path collective.

`backend` is anything with singleProjectorSample(P, L, exact, count, rng, seed)
and rng_position(seed, first) (circuitsimulator_gb300.backend.Backend on GPU
ranks; the CPU tests pass a stand-in).
"""
import numpy as np


def shard_bounds(total, rank, world):
    """[lo, hi) of the states rank `rank` draws out of `total`."""
    base, extra = divmod(int(total), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def median_of_means(values, samples, bins):
    """multiSampledProjector's reduction (innerprod.c:23-41): per-bin means in
    draw order, then the median as the reference's qsort computes it with its
    difference-truncating comparator."""
    import functools

    means = []
    for b in range(bins):
        tot = 0.0
        for v in values[b * samples:(b + 1) * samples]:
            tot += float(v)
        means.append(tot / samples)
    if bins == 1:
        return means[0]

    def cmp(a, b):
        return int(a - b)  # (int)(a - b), truncation toward zero

    s = sorted(means, key=functools.cmp_to_key(cmp))
    return s[(bins - 1) // 2] if bins % 2 == 1 else (s[bins // 2] + s[bins // 2 - 1]) / 2


def sharded_values(backend, P, L, exact, count, seed, rank, world, group=None):
    """Every state's singleProjectorSample value, gathered on rank 0 in draw order
    (None on the other ranks)."""
    import torch
    import torch.distributed as dist

    from .backend import RNG_PHILOX, SEED_CONTINUE

    lo, hi = shard_bounds(count, rank, world)
    backend.rng_position(seed, lo)
    mine = np.asarray(backend.singleProjectorSample(P, L, exact, hi - lo, RNG_PHILOX, SEED_CONTINUE), dtype=np.float64)
    if world == 1:
        return mine
    width = shard_bounds(count, 0, world)[1]  # the largest block
    buf = torch.zeros(width + 1, dtype=torch.float64)
    buf[0] = float(hi - lo)
    buf[1:1 + len(mine)] = torch.from_numpy(mine)
    out = [torch.zeros_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, out, dst=0, group=group)
    if rank != 0:
        return None
    vals = []
    for r in range(world):
        n = int(out[r][0].item())
        vals.append(out[r][1:1 + n].numpy())
    return np.concatenate(vals)


def sharded_multi_sampled_projector(backend, P, L, exact, norm, samples, bins, seed, rank, world, group=None):
    """multiSampledProjector over `world` ranks; the result on rank 0 (None elsewhere)."""
    nstabs = P.nstabs if hasattr(P, "nstabs") else None
    if nstabs == 0:
        return norm ** 2 if rank == 0 else None
    vals = sharded_values(backend, P, L, exact, samples * bins, seed, rank, world, group)
    if vals is None:
        return None
    return median_of_means(vals, samples, bins)
