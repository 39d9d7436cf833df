"""Batched factorisation over geometries of uneven order (wmom_factor_geometries).

Each (geometry, frequency) pair is stored at the padded order of its size class with
an identity block, and pairs of one class are filled and factored together.  Tested:
* a pair's currents, input impedance and report are bit-identical whether it is
  factored alone or inside a batch of uneven geometries (the class depends on its
  order only), in both forms;
* they agree with the unpadded resident factor set (wmom_factor) to the forms'
  tolerances, and with the CPU oracle;
* the condition estimate of a padded set is that of the geometry's own matrix.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [300, 310, 700, 1000, 1020, 2500]  # 300 and 310 share a class, as do 1000 and 1020
FREQS = [0.02, 3.0, 7.5, 0.5, 12.0, 1.0]


def _plans(w):
    return [w.Plan(w.Topology(w.geometry.random_wires(n, seed=500 + i), listing=False)) for i, n in enumerate(SIZES)]


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_alone_and_in_batch_bit_identical(cuda, wmom, mode):
    w = wmom
    m = w.MODE_MIXED if mode == "mixed" else w.MODE_FP64
    plans = _plans(w)
    assert len({w.padded_order(n) for n in SIZES}) == 4
    batch = w.factor_geometries(plans, FREQS, mode=m)
    for i, p in enumerate(plans):
        alone = w.factor_geometries([p], [FREQS[i]], mode=m)[0]
        gap = SIZES[i] // 3
        ca, za, ra = alone.solve(gap, ampl=1.5, phas=10.0)
        cb, zb, rb = batch[i].solve(gap, ampl=1.5, phas=10.0)
        assert ca.shape == (1, SIZES[i])
        assert np.array_equal(ca, cb) and np.array_equal(za, zb), i
        assert ra == rb
        alone.close()
    for f in batch:
        f.close()
    for p in plans:
        p.close()


def test_padded_sets_match_unpadded_and_oracle(cuda, wmom, orc):
    w = wmom
    plans = _plans(w)
    sets = w.factor_geometries(plans, FREQS, mode=w.MODE_MIXED, condest=True)
    threads = os.cpu_count() or 1
    for i, p in enumerate(plans):
        gap = SIZES[i] // 2
        cur, zin, rep = sets[i].solve(gap)
        ref = w.Factors(p, [FREQS[i]], mode=w.MODE_MIXED, condest=True)
        cur0, zin0, rep0 = ref.solve(gap)
        assert rep[0]["status"] == 0 and rep[0]["rel_residual"] <= 1e-12
        rel = np.linalg.norm(cur[0] - cur0[0]) / np.linalg.norm(cur0[0])
        assert rel < 1e-11, (i, rel)
        # the estimate of the leading block, within the estimator's own spread
        assert 0.5 <= rep[0]["cond1"] / rep0[0]["cond1"] <= 2.0, (rep[0]["cond1"], rep0[0]["cond1"])
        g = orc.topology(w.geometry.random_wires(SIZES[i], seed=500 + i))
        i_ref, z_ref, _ = orc.solve(g, FREQS[i], gap, threads=threads)
        assert np.linalg.norm(cur[0] - i_ref) / np.linalg.norm(i_ref) < 1e-9
        assert abs(zin[0] - z_ref) / abs(z_ref) < 1e-9
        ref.close()
    for f in sets:
        f.close()
    for p in plans:
        p.close()
