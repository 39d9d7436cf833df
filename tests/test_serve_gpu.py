"""Serving loop (praca-magisterska_gb300/serve.py): every result is the same alone and
inside a concurrent mix of requests (continuous batching, resident factors, repeat
excitations), admission by device-memory budget evicts idle factor sets, and the
resident-factor solves agree with the sweep solver and the oracle."""
import importlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# results in the mix equal results alone to this relative tolerance (the kernels are
# deterministic, so in practice they are bit-identical)
TOL_SAME = 1e-12


def _specs(g):
    geos = [g.random_wires(300, seed=1), g.dipole(1.0, 1e-3, 256), g.grid(5, 1.0, 1.0, 5e-3, None, 3)]
    return geos, [
        (0, [0.5, 3.0], 100, 1.0, 0.0),
        (1, [150.0], 128, 1.0, 0.0),
        (2, [10.0, 20.0, 30.0], 50, 2.0, 45.0),
        (0, [3.0], 7, 1.0, 0.0),          # repeat excitation of a resident pair
        (1, [150.0, 300.0], 10, 1.0, 90.0),
        (2, [20.0], 50, 2.0, 45.0),
    ]


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_results_same_alone_and_in_the_mix(cuda, wmom):
    serve = importlib.import_module("praca-magisterska_gb300.serve")
    geos, specs = _specs(wmom.geometry)
    alone = []
    for gi, fr, ngap, amp, ph in specs:
        srv = serve.Server(workers=1)
        alone.append(srv.submit(serve.Request(geos[gi], fr, ngap, amp, ph)).result(timeout=300))
        srv.close()
    srv = serve.Server(workers=2)
    futs = [srv.submit(serve.Request(geos[gi], fr, ngap, amp, ph)) for gi, fr, ngap, amp, ph in specs]
    mix = [f.result(timeout=600) for f in futs]
    st = srv.stats()
    srv.close()
    for a, m in zip(alone, mix):
        assert _rel(m["currents"], a["currents"]) <= TOL_SAME
        assert np.max(np.abs(m["zin"] - a["zin"]) / np.abs(a["zin"])) <= TOL_SAME
        assert all(r["status"] == 0 for r in m["reports"])
    assert st["requests"] == len(specs) and st["p50_ms"] is not None and st["p99_ms"] >= st["p50_ms"]


def test_resident_solves_match_sweep_and_oracle(cuda, wmom, orc):
    serve = importlib.import_module("praca-magisterska_gb300.serve")
    topo_text = wmom.geometry.dipole(1.0, 1e-3, 300)
    srv = serve.Server(workers=1)
    r1 = srv.submit(serve.Request(topo_text, [100.0, 200.0], 150)).result(timeout=300)
    r2 = srv.submit(serve.Request(topo_text, [100.0, 200.0], 20, 3.0, 30.0)).result(timeout=300)  # resident
    srv.close()
    plan = wmom.Plan(wmom.Topology(topo_text))
    c1, _, _ = plan.solve([100.0, 200.0], 150, mode=wmom.MODE_MIXED)
    c2, _, _ = plan.solve([100.0, 200.0], 20, ampl=3.0, phas=30.0, mode=wmom.MODE_MIXED)
    plan.close()
    assert _rel(r1["currents"], c1) <= TOL_SAME and _rel(r2["currents"], c2) <= TOL_SAME
    topo = wmom.Topology(topo_text)
    i_ref, _, _ = orc.solve(topo.arrays(), 200.0, 20, ampl=3.0, phas=30.0, threads=os.cpu_count() or 1)
    assert _rel(r2["currents"][1], i_ref) < 1e-9


def test_admission_by_memory_budget_evicts_idle_sets(cuda, wmom):
    serve = importlib.import_module("praca-magisterska_gb300.serve")
    g = wmom.geometry
    n = 299
    per = n * n * 24 + 4 * n
    srv = serve.Server(workers=1, hbm_budget_bytes=5 * per)
    texts = [g.random_wires(n, seed=s, n_wires=4) for s in (11, 12, 13)]
    outs = [srv.submit(serve.Request(t, [1.0, 5.0], 10)).result(timeout=300) for t in texts]
    st = srv.stats()
    srv.close()
    assert st["evictions"] >= 1 and st["resident_bytes"] <= 5 * per
    for t, o in zip(texts, outs):
        plan = wmom.Plan(wmom.Topology(t))
        c, _, _ = plan.solve([1.0, 5.0], 10, mode=wmom.MODE_MIXED)
        plan.close()
        assert _rel(o["currents"], c) <= TOL_SAME
    with pytest.raises(MemoryError):
        srv2 = serve.Server(workers=1, hbm_budget_bytes=per // 2)
        try:
            srv2.submit(serve.Request(texts[0], [1.0], 10)).result(timeout=60)
        finally:
            srv2.close()
