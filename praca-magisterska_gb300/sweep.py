"""Frequency sweeps across processes.

Every (geometry, frequency) solve is independent, so a sweep shards with no
collective in the data path: rank r of P takes frequencies r, r+P, r+2P, ... -- the
round-robin of the reference's MPI driver ("wersja gpu/Wire_MoM.cu":331,
``for (i = rank; i < nfreq; i += P)``) -- and the host gathers the results.  On one
GB300 the frequencies of a rank are batched on the device instead (Plan.solve).
"""
import numpy as np


def shard_frequencies(freqs, rank, world):
    """Indices and values of the frequencies rank `rank` of `world` solves."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    idx = np.arange(rank, len(freqs), world)
    return idx, np.asarray(freqs)[idx]


def gather_sweep(local_idx, local_results, nfreq, group=None):
    """All-gather per-rank (index, result) pairs into a list ordered by frequency.
    Uses torch.distributed's object collective (host side only)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, (list(map(int, local_idx)), list(local_results)), group=group)
    out = [None] * nfreq
    for idx, res in parts:
        for i, r in zip(idx, res):
            if out[i] is not None:
                raise RuntimeError(f"frequency {i} solved twice")
            out[i] = r
    missing = [i for i, r in enumerate(out) if r is None]
    if missing:
        raise RuntimeError(f"frequencies {missing} were not solved")
    return out


def solve_sharded(plan, freqs, ngap, rank, world, group=None, **kw):
    """Each rank solves its shard on its own GPU; returns (zin, currents) of the whole
    sweep on every rank."""
    idx, f = shard_frequencies(freqs, rank, world)
    if len(f):
        cur, zin, _ = plan.solve(f, ngap, **kw)
        local = [(complex(z), c) for z, c in zip(zin, cur)]
    else:
        local = []
    allr = gather_sweep(idx, local, len(freqs), group)
    return np.array([r[0] for r in allr]), np.array([r[1] for r in allr])
