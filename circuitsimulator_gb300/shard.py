"""The estimators split over ranks, one process per GPU.

Sampled mode follows the reference's parallel strategy (MPI master/worker over
samples, libcirc/innerprod.c:64-83 and libcirc/probability.c:225-299): each
rank draws a contiguous block of the counter-based stream (state i of stream
`seed` is the same whoever draws it), evaluates its states on its own GPU, and
rank 0 gathers every state's value in index order.  The bin means and the
median are then computed by the same native code as on one GPU
(csim_median_of_means), so the sharded result is bit-identical to the
single-GPU one.

Exact mode splits exactProjector's l-range (innerprod.c:169-195) by rows: rank
r takes a contiguous range of rows i (row i holds the chi - i pairs j >= i),
balanced by pair count.  Each row's sum is exact on the GPU; rank 0 gathers the
rows' values and adds them in row order, as csim_exact_projector does, so this
result too is bit-identical to one GPU.

The only exchange is one gather to rank 0 (one double per state, or two per
row); no collective touches the data path.  Under an NCCL group the gather
goes through CUDA tensors, under gloo through CPU tensors.

`backend` is anything with singleProjectorSample(P, L, exact, count, rng, seed),
rng_position(seed, first), exactProjector(P, L, exact, norm) and
exactProjectorRows(P, L, exact, i0, i1) (circuitsimulator_gb300.backend.Backend
on GPU ranks; the CPU tests pass a stand-in).
"""
import numpy as np


def shard_bounds(total, rank, world):
    """[lo, hi) of the states rank `rank` draws out of `total`."""
    base, extra = divmod(int(total), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def row_bounds(chi, rank, world):
    """[lo, hi) of exactProjector's rows for rank `rank`: row i holds chi - i
    pairs, and each rank gets rows up to its share of the chi(chi+1)/2 pairs."""
    chi, world = int(chi), int(world)
    total = chi * (chi + 1) // 2

    def first_row(r):
        # smallest i with pairs(rows < i) >= r * total / world
        target = (r * total + world - 1) // world
        lo, hi = 0, chi
        while lo < hi:
            mid = (lo + hi) // 2
            if mid * chi - mid * (mid - 1) // 2 >= target:
                hi = mid
            else:
                lo = mid + 1
        return lo

    return first_row(rank), (chi if rank == world - 1 else first_row(rank + 1))


def median_of_means(values, samples, bins):
    """multiSampledProjector's reduction (innerprod.c:23-41), by the native
    code csim_multi_sampled_projector itself uses."""
    from .backend import median_of_means as native

    return native(values, samples, bins)


def _gather_blocks(mine, rank, world, group=None):
    """Gathers each rank's 1-D float64 array on rank 0, in rank order (None
    elsewhere).  Blocks may differ in length."""
    import torch
    import torch.distributed as dist

    dev = "cpu"
    if dist.get_backend(group) == "nccl":
        dev = "cuda:%d" % torch.cuda.current_device()
    n = torch.tensor([len(mine)], dtype=torch.int64, device=dev)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    width = max(1, max(int(s.item()) for s in sizes))
    buf = torch.zeros(width, dtype=torch.float64, device=dev)
    buf[:len(mine)] = torch.from_numpy(np.ascontiguousarray(mine, dtype=np.float64)).to(dev)
    out = [torch.zeros_like(buf) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, out, dst=0, group=group)
    if rank != 0:
        return None
    return [out[r][:int(sizes[r].item())].cpu().numpy() for r in range(world)]


def sharded_values(backend, P, L, exact, count, seed, rank, world, group=None):
    """Every state's singleProjectorSample value, gathered on rank 0 in draw order
    (None on the other ranks)."""
    from .backend import RNG_PHILOX, SEED_CONTINUE

    lo, hi = shard_bounds(count, rank, world)
    backend.rng_position(seed, lo)
    mine = np.asarray(backend.singleProjectorSample(P, L, exact, hi - lo, RNG_PHILOX, SEED_CONTINUE), dtype=np.float64)
    if world == 1:
        return mine
    blocks = _gather_blocks(mine, rank, world, group)
    return None if blocks is None else np.concatenate(blocks)


def sharded_multi_sampled_projector(backend, P, L, exact, norm, samples, bins, seed, rank, world, group=None):
    """multiSampledProjector over `world` ranks; the result on rank 0 (None elsewhere)."""
    nstabs = P.nstabs if hasattr(P, "nstabs") else None
    if nstabs == 0:
        return norm ** 2 if rank == 0 else None
    vals = sharded_values(backend, P, L, exact, samples * bins, seed, rank, world, group)
    if vals is None:
        return None
    return median_of_means(vals, samples, bins)


def sharded_exact_projector(backend, P, L, exact, norm, rank, world, group=None):
    """exactProjector over `world` ranks, rows split by pair count; the result
    on rank 0 (None elsewhere), bit-identical to backend.exactProjector."""
    nstabs = P.nstabs if hasattr(P, "nstabs") else None
    t = P.nqubits if hasattr(P, "nqubits") else None
    if nstabs == 0 or t == 0:  # no rows: the reference's closed forms, on rank 0 alone
        return backend.exactProjector(P, L, exact, norm) if rank == 0 else None
    chi = (1 << ((t + 1) // 2)) if exact else (1 << len(L))
    lo, hi = row_bounds(chi, rank, world)
    re, im = backend.exactProjectorRows(P, L, exact, lo, hi)
    mine = np.concatenate([np.asarray(re, dtype=np.float64), np.asarray(im, dtype=np.float64)])
    if world == 1:
        blocks = [mine]
    else:
        blocks = _gather_blocks(mine, rank, world, group)
        if blocks is None:
            return None
    tr = ti = 0.0
    for b in blocks:  # rank order is row order
        half = len(b) // 2
        for x in b[:half]:
            tr += float(x)
        for y in b[half:]:
            ti += float(y)
    return float(np.sqrt(tr * tr + ti * ti))
