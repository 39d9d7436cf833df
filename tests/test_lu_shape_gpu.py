"""Factorisation shapes of the precision form that the autotuner chooses between:
* the narrow tensor-core tile (128 x 128 real outputs) gives the same currents as the
  wide one (128 x 256): each output's K accumulation is the same sequence of MMAs;
* narrower FP32 panels (48 and 32 columns) change the blocking, and the refined
  currents still meet the precision form's 1e-9 against the plain FP64 form;
* a tuned sweep reports its shape (wmom_tuned_shape) within the candidates.
The shapes are forced with WMOM_LU_BATCH / WMOM_LU_SPAN / WMOM_TC_TILE / WMOM_PANEL_W,
which the library reads at every factorisation."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _solve(w, plan, freqs, env):
    keys = ("WMOM_LU_BATCH", "WMOM_LU_SPAN", "WMOM_TC_TILE", "WMOM_PANEL_W")
    old = {k: os.environ.get(k) for k in keys}
    try:
        for k in keys:
            os.environ.pop(k, None)
        os.environ.update(env)
        cur, _, rep = plan.solve(freqs, 300, mode=w.MODE_MIXED)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    assert all(r["status"] == 0 and r["tier"] == 1 for r in rep)
    return cur


def test_tile_and_panel_shapes(cuda, wmom):
    w = wmom
    plan = w.Plan(w.Topology(w.geometry.random_wires(2600, seed=77), listing=False))
    freqs = np.array([0.3, 3.0, 9.0], np.float32)
    ref, _, _ = plan.solve(freqs, 300, mode=w.MODE_FP64)
    base = {"WMOM_LU_BATCH": "3", "WMOM_LU_SPAN": "2"}
    wide = _solve(w, plan, freqs, dict(base, WMOM_TC_TILE="256"))
    narrow = _solve(w, plan, freqs, dict(base, WMOM_TC_TILE="128"))
    assert _rel(narrow, wide) <= 1e-13
    for pw in ("48", "32"):
        cur = _solve(w, plan, freqs, dict(base, WMOM_PANEL_W=pw))
        for k in range(len(freqs)):
            assert _rel(cur[k], ref[k]) <= 1e-9, (pw, k)
    for k in range(len(freqs)):
        assert _rel(wide[k], ref[k]) <= 1e-9
    plan.close()


def test_tuned_sweep_reports_its_shape(cuda, wmom):
    w = wmom
    n = 1800
    plan = w.Plan(w.Topology(w.geometry.random_wires(n, seed=78), listing=False))
    for k in ("WMOM_LU_BATCH", "WMOM_LU_SPAN", "WMOM_TC_TILE", "WMOM_PANEL_W"):
        assert k not in os.environ
    plan.solve(np.array([1.0, 2.0, 4.0, 8.0], np.float32), 100, mode=w.MODE_MIXED, currents=False)
    tile, pw = w.tuned_shape(n, w.MODE_MIXED)
    assert tile in (128, 256) and pw in (0, 48, 32)
    b, sp = w.tuned_config(n, w.MODE_MIXED)
    assert b >= 1 and sp in (1, 2, 4)
    plan.close()
