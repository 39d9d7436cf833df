"""Multi-process sweep logic on CPU: world_size 2 over gloo.  Each rank solves its
round-robin shard of the frequencies (with the CPU oracle standing in for a GPU
solve, so no GPU is needed) and the gathered sweep must equal the single-process
sweep in order and value."""
import importlib
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


class _OraclePlan:
    """The Plan.solve interface, computed by the CPU oracle."""

    def __init__(self, topo):
        self.g = topo.arrays()

    def solve(self, freqs, ngap, **kw):
        from oracle import oracle as orc
        cur, zin = [], []
        for f in freqs:
            i, z, _ = orc.solve(self.g, float(f), ngap)
            cur.append(i)
            zin.append(z)
        return np.array(cur), np.array(zin), [{}] * len(freqs)


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w = importlib.import_module("praca-magisterska_gb300")
    from importlib import import_module
    sw = import_module("praca-magisterska_gb300.sweep")
    topo = w.Topology(w.geometry.dipole(1.0, 1e-3, 40))
    freqs = np.array([50.0, 100.0, 150.0, 200.0, 250.0], np.float32)
    zin, cur = sw.solve_sharded(_OraclePlan(topo), freqs, 20, rank, world)
    out[rank] = (zin, cur)
    dist.destroy_process_group()


def test_round_robin_shards_cover_sweep(wmom):
    sw = importlib.import_module("praca-magisterska_gb300.sweep")
    freqs = np.arange(11, dtype=np.float32)
    seen = np.concatenate([sw.shard_frequencies(freqs, r, 3)[0] for r in range(3)])
    assert sorted(seen.tolist()) == list(range(11))
    assert list(sw.shard_frequencies(freqs, 1, 3)[0]) == [1, 4, 7, 10]
    with pytest.raises(ValueError):
        sw.shard_frequencies(freqs, 3, 3)


def test_two_rank_gloo_sweep_matches_single_process(wmom, orc):
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    topo = wmom.Topology(wmom.geometry.dipole(1.0, 1e-3, 40))
    freqs = [50.0, 100.0, 150.0, 200.0, 250.0]
    ref = [orc.solve(topo.arrays(), f, 20)[1] for f in freqs]
    for r in range(world):
        zin, cur = out[r]
        assert np.array_equal(zin, np.array(ref))
