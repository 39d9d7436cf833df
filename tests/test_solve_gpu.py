"""End-to-end fill -> LU -> solve -> Z_in on the GPU against the oracle and the
reference fixtures.  Tolerances are the solver's contract: relative error 1e-10
on currents and input impedance for the plain FP64 form, 1e-9 for the refined
mixed-precision form."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_MIXED = 1e-9
EPS = 2.0 ** -53
KAPPA_FACTOR = 8  # two FP64-level solves of one system agree to about kappa * eps


def _bound(tol, kappa):
    """The tolerance of a form, or the conditioning's floor where that is larger."""
    return max(tol, KAPPA_FACTOR * kappa * EPS)


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def _fixture(name):
    d = np.load(os.path.join(GOLDEN, f"currents_{name}.npz"))
    geo = str(np.load(os.path.join(GOLDEN, f"topology_{name}.npz"))["geo"])
    return d, geo


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", ["dipole1m_512", "dipole25m_512", "mixed_junctions", "random_1024", "ground_monopole",
                                  "ground_frame", "ground_grid"])
def test_currents_match_reference_fixtures(cuda, wmom, name, mode):
    d, geo = _fixture(name)
    topo = wmom.Topology(geo, ienv=int(d["ienv"]))
    plan = wmom.Plan(topo)
    cur, zin, rep = plan.solve(d["freqs"], int(d["ngap"]), mode=mode, tol=1e-12)
    tol = TOL_FP64 if mode == 0 else TOL_MIXED
    for k in range(len(d["freqs"])):
        assert _rel(cur[k], d["currents"][k]) < tol, (k, _rel(cur[k], d["currents"][k]), rep[k])
        assert abs(zin[k] - d["zin"][k]) / abs(d["zin"][k]) < tol
        assert rep[k]["status"] == 0
    plan.close()


def test_grid_2048_against_reference(cuda, wmom):
    # junction grid: kappa_1 grows at low frequency (about 1e10 at 10 kHz), so the
    # bound is the form's tolerance or 8 kappa_1 eps, kappa_1 estimated per frequency
    d, geo = _fixture("grid21_2048")
    topo = wmom.Topology(geo)
    plan = wmom.Plan(topo)
    for mode in (0, 1):
        cur, zin, rep = plan.solve(d["freqs"], int(d["ngap"]), mode=mode, condest=True)
        for k in range(len(d["freqs"])):
            err = _rel(cur[k], d["currents"][k])
            bound = _bound(TOL_FP64 if mode == 0 else TOL_MIXED, rep[k]["cond1"])
            assert rep[k]["cond1"] > 1.0 and rep[k]["status"] == 0
            assert err < bound, (mode, k, err, bound, rep[k])
            assert abs(zin[k] - d["zin"][k]) / abs(d["zin"][k]) < bound
            assert rep[k]["rel_residual"] < bound
    plan.close()


def test_logged_zin_known_answers(cuda, wmom):
    with open(os.path.join(GOLDEN, "zin_logs.json")) as f:
        logs = json.load(f)
    for nsw in (512, 1024, 2048):
        rows = {}
        for r in logs:
            if r["nsw"] == nsw:
                rows.setdefault(r["freq"], r)
        freqs = sorted(rows)
        topo = wmom.Topology(wmom.geometry.dipole(25.0, 5e-4, nsw))
        plan = wmom.Plan(topo)
        for mode in (0, 1):
            _, zin, _ = plan.solve(freqs, 100, mode=mode, currents=False)
            for f, z in zip(freqs, zin):
                r = rows[f]
                for val, text in ((z.real, r["re_text"]), (z.imag, r["im_text"])):
                    v = abs(float(text))
                    half = 0.5 * 10.0 ** (math.floor(math.log10(v)) - 3) if v else 5e-5
                    assert abs(val - float(text)) <= 1.01 * half, (nsw, f, z, text)
        plan.close()


def test_batch_invariance_and_alone(cuda, wmom):
    # every frequency's result is the same alone and inside a batch
    topo = wmom.Topology(wmom.geometry.random_wires(700, seed=9))
    plan = wmom.Plan(topo)
    freqs = np.array([0.01, 0.3, 2.0, 9.0], np.float32)
    for mode in (0, 1):
        cb, zb, _ = plan.solve(freqs, 100, mode=mode)
        for k, f in enumerate(freqs):
            ca, za, _ = plan.solve([f], 100, mode=mode)
            assert np.array_equal(ca[0], cb[k])
    plan.close()


def test_mixed_reports_refinement(cuda, wmom, orc):
    topo = wmom.Topology(wmom.geometry.dipole(1.0, 1e-3, 512))
    plan = wmom.Plan(topo)
    cur, zin, rep = plan.solve([150.0], 256, mode=1, tol=1e-12)
    assert rep[0]["fell_back"] == 0 and rep[0]["iterations"] >= 1
    assert rep[0]["rel_residual"] <= 1e-12
    i_ref, zin_ref, _ = orc.solve(topo.arrays(), 150.0, 256, threads=os.cpu_count() or 1)
    assert _rel(cur[0], i_ref) < TOL_MIXED
    plan.close()


def test_dropin_zmatrix_symbol(cuda, wmom, orc):
    import ctypes
    lib = ctypes.CDLL(os.path.join(os.path.dirname(wmom.__file__), "libwmom.so"))
    f = getattr(lib, "_Z7zmatrixP7double2PfS1_S1_PiS2_S2_S1_idiiffff")
    fp, ip = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
    f.restype = None
    f.argtypes = [ctypes.c_void_p, fp, fp, fp, ip, ip, ip, fp, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                  ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    topo = wmom.Topology(wmom.geometry.grid(4, 1.0, 1.0, 5e-3, None, 3))
    n = topo.npls
    cz = np.zeros((n, n), np.complex128, order="F")
    p = lambda a, t: a.ctypes.data_as(t)
    f(cz.ctypes.data, p(topo.x, fp), p(topo.y, fp), p(topo.z, fp), p(topo.ipc, ip), p(topo.ips, ip),
      p(topo.ise, ip), p(topo.rad, fp), n, orc.ka(20.0), topo.nsmax, 1, 1.0, 1.0, 1.0, 1.0)
    zr = orc.fill(topo.arrays(), 20.0)
    assert np.max(np.abs(cz - zr) / np.max(np.abs(zr), axis=0)) < 1e-13


@pytest.mark.parametrize("ienv", [1, 2])
def test_dropin_zmatrix_gpu_symbol(cuda, wmom, orc, ienv):
    """The reference's GPU entry point (REF/Wire_MoM.h:49-51: host arrays in, host cz
    out, its own argument order) called through its mangled name; free space and the
    PEC-ground image terms."""
    import ctypes
    lib = ctypes.CDLL(os.path.join(os.path.dirname(wmom.__file__), "libwmom.so"))
    f = getattr(lib, "_Z11zmatrix_gpuP7double2PfS1_S1_S1_PiS2_S2_idiiffff")
    fp, ip = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)
    f.restype = None
    f.argtypes = [ctypes.c_void_p, fp, fp, fp, fp, ip, ip, ip, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                  ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]
    g = wmom.geometry
    text = g.grid(4, 1.0, 1.0, 5e-3, None, 3) if ienv == 1 else \
        g.geo_text([(0, 0, 0), (0, 0, 1.0), (1.0, 0, 1.0)], [(1, 2, 1e-3, 20), (2, 3, 1e-3, 20)])
    topo = wmom.Topology(text, ienv=ienv)
    n = topo.npls
    cz = np.zeros((n, n), np.complex128, order="F")
    p = lambda a, t: a.ctypes.data_as(t)
    sg = topo.sgn
    f(cz.ctypes.data, p(topo.x, fp), p(topo.y, fp), p(topo.z, fp), p(topo.rad, fp), p(topo.ipc, ip),
      p(topo.ips, ip), p(topo.ise, ip), topo.nsmax, orc.ka(20.0), n, ienv, sg[0], sg[1], sg[2], sg[3])
    zr = orc.fill(topo.arrays(), 20.0, ienv=ienv, sgn=sg)
    assert np.max(np.abs(cz - zr) / np.max(np.abs(zr), axis=0)) < 1e-13


def test_batch_width_does_not_change_results(cuda, wmom):
    # the same frequencies factored one matrix per launch and four per launch (without
    # the second-tier prediction, whose decisions follow the group boundaries)
    topo = wmom.Topology(wmom.geometry.precision_grid(2048))
    freqs = np.array([0.002, 0.05, 1.0, 7.0, 20.0], np.float32)
    out = {}
    for width in ("1", "4"):
        os.environ["WMOM_LU_BATCH"] = width
        os.environ["WMOM_TIER_PREDICT"] = "0"
        try:
            plan = wmom.Plan(topo)
            for mode in (0, 1):
                out[(width, mode)] = plan.solve(freqs, 1000, mode=mode)
            plan.close()
        finally:
            del os.environ["WMOM_LU_BATCH"]
            del os.environ["WMOM_TIER_PREDICT"]
    for mode in (0, 1):
        c1, z1, r1 = out[("1", mode)]
        c4, z4, r4 = out[("4", mode)]
        assert np.array_equal(c1, c4)
        assert [r["iterations"] for r in r1] == [r["iterations"] for r in r4]


def test_second_tier_serves_ill_conditioned_grid(cuda, wmom):
    # 21 x 21 junction grid at 10 and 30 kHz: kappa * u_fp32 >> 1, so the FP32 factors
    # stall.  The second tier (FP64 LU with digit-plane tensor-core trailing updates,
    # then FP64 refinement) must reach the plain FP64 solve's backward error, and
    # differ from that solve by about kappa * eps, as any two FP64 solves do (kappa is
    # near 1e10 here): within 8 kappa_1 eps, kappa_1 estimated per frequency.
    topo = wmom.Topology(wmom.geometry.precision_grid(2048))
    freqs = np.array([0.01, 0.03], np.float32)
    plan = wmom.Plan(topo)
    c64, z64, r64 = plan.solve(freqs, 1000, mode=0, condest=True)
    cm, zm, rm = plan.solve(freqs, 1000, mode=1)
    for k in range(len(freqs)):
        assert rm[k]["status"] == 0 and rm[k]["fell_back"] == 1 and rm[k]["tier"] == 2, rm[k]
        assert rm[k]["rel_residual"] <= 4 * r64[k]["rel_residual"] + 1e-15, (rm[k], r64[k])
        assert _rel(cm[k], c64[k]) < _bound(TOL_MIXED, r64[k]["cond1"]), (_rel(cm[k], c64[k]), r64[k])
        assert r64[k]["tier"] == 0
    # without the tensor-core tier the same matrices take the plain FP64 LU, whose
    # solution is the FP64 form's bit for bit
    os.environ["WMOM_NO_EMUL"] = "1"
    try:
        cp, zp, rp = plan.solve(freqs, 1000, mode=1)
    finally:
        del os.environ["WMOM_NO_EMUL"]
    for k in range(len(freqs)):
        assert rp[k]["tier"] == 3 and rp[k]["status"] == 0
        assert np.array_equal(cp[k], c64[k])
    plan.close()


def test_krylov_step_forced_on(cuda, wmom):
    # GMRES refinement with the FP32 factors runs by default only without the
    # tensor-core second tier; forced on, every result keeps the contract of the tier
    # that produced it (two FP64-level solves of these grid systems differ by up to
    # kappa * eps: within 8 kappa_1 eps, kappa_1 estimated per frequency).  Tier 1's
    # acceptance of backward-stable solutions at the residual floor is off here
    # (WMOM_T1_BERR=0): the matrices it keeps are the ones GMRES would refine.
    topo = wmom.Topology(wmom.geometry.precision_grid(2048))
    freqs = np.geomspace(0.05, 20.0, 8).astype(np.float32)
    plan = wmom.Plan(topo)
    c64, _, r64 = plan.solve(freqs, 1000, mode=0, condest=True)
    os.environ["WMOM_KRYLOV"] = "1"
    os.environ["WMOM_T1_BERR"] = "0"
    try:
        cm, _, rm = plan.solve(freqs, 1000, mode=1)
    finally:
        del os.environ["WMOM_KRYLOV"]
        del os.environ["WMOM_T1_BERR"]
    assert sum(r["krylov_steps"] for r in rm) > 0, rm
    for k in range(len(freqs)):
        assert rm[k]["status"] == 0 and rm[k]["tier"] in (1, 2, 3), rm[k]
        assert _rel(cm[k], c64[k]) < _bound(TOL_MIXED, r64[k]["cond1"]), (k, _rel(cm[k], c64[k]), rm[k], r64[k])
    plan.close()


def test_fp64_cluster_panel_lookahead_is_bit_identical(cuda, wmom):
    # the second tier's LU with complex128 storage and FP64 cluster panels
    # (WMOM_FF_TIER2=0, WMOM_FF_PANEL=0) with and without the panel's one-column
    # look-ahead: the same currents bit for bit
    topo = wmom.Topology(wmom.geometry.precision_grid(2048))
    freqs = np.array([0.01], np.float32)
    out = {}
    for la in ("1", "0"):
        os.environ["WMOM_PANEL_LOOKAHEAD"] = la
        os.environ["WMOM_FF_PANEL"] = "0"
        os.environ["WMOM_FF_TIER2"] = "0"
        try:
            plan = wmom.Plan(topo)
            out[la] = plan.solve(freqs, 1000, mode=1)
            plan.close()
        finally:
            del os.environ["WMOM_PANEL_LOOKAHEAD"]
            del os.environ["WMOM_FF_PANEL"]
            del os.environ["WMOM_FF_TIER2"]
    assert out["1"][2][0]["tier"] == 2
    assert np.array_equal(out["1"][0], out["0"][0])


@pytest.mark.parametrize("mode", [0, 1])
def test_pipelined_sweep_is_bit_identical(cuda, wmom, mode):
    """With the factorisation shape tuned, a sweep is split into groups whose fills run
    on a second stream while the previous group factors (WMOM_PIPELINE groups; by
    default only sweeps of two or more full-width groups); the currents, input
    impedances and reports must not depend on the number of groups."""
    topo = wmom.Topology(wmom.geometry.precision_grid(2048))
    plan = wmom.Plan(topo)
    freqs = np.array([0.003, 0.02, 0.2, 1.0, 3.0, 7.0, 12.0, 25.0], np.float32)
    out = {}
    os.environ["WMOM_TIER_PREDICT"] = "0"  # its decisions follow the group boundaries
    try:
        for groups in ("1", "1", "2", "3"):  # the first call tunes the shape
            os.environ["WMOM_PIPELINE"] = groups
            out[groups] = plan.solve(freqs, 1000, mode=mode)
    finally:
        os.environ.pop("WMOM_PIPELINE", None)
        os.environ.pop("WMOM_TIER_PREDICT", None)
    c1, z1, r1 = out["1"]
    for g in ("2", "3"):
        c, z, r = out[g]
        assert np.array_equal(c, c1) and np.array_equal(z, z1), g
        assert r == r1, g
    plan.close()


def test_second_tier_prediction(cuda, wmom):
    """A sweep runs its groups from the highest frequency down; once a whole group
    has fallen back to the second tier, the lower-frequency groups go there directly,
    without FP32 factors.  A predicted matrix must get the answer it gets after
    failing in tier 1, bit for bit; the sweep must factor fewer FP32 matrices; and
    the results come back in the caller's frequency order."""
    w = wmom
    topo = w.Topology(w.geometry.precision_grid(2048))
    plan = w.Plan(topo)
    freqs = np.array([0.003, 30.0, 0.001, 0.01, 10.0, 0.03, 1.0, 0.1], np.float32)  # not sorted
    out = {}
    os.environ["WMOM_LU_BATCH"] = "2"
    os.environ["WMOM_LU_SPAN"] = "2"
    try:
        for pred in ("0", "1"):
            os.environ["WMOM_TIER_PREDICT"] = pred
            w.stats_reset()
            out[pred] = plan.solve(freqs, 1000, mode=w.MODE_MIXED, condest=True) + (w.stats_read(),)
    finally:
        for k in ("WMOM_LU_BATCH", "WMOM_LU_SPAN", "WMOM_TIER_PREDICT"):
            os.environ.pop(k, None)
    c0, z0, r0, st0 = out["0"]
    c1, z1, r1, st1 = out["1"]
    cfp, _, _ = plan.solve(freqs, 1000, mode=w.MODE_FP64)
    plan.close()
    predicted = 0
    for k, f in enumerate(freqs):
        assert r1[k]["status"] == 0 and r0[k]["status"] == 0
        if r0[k]["tier"] >= 2 and r1[k]["tier"] >= 2:
            assert np.array_equal(c1[k], c0[k]) and z1[k] == z0[k], float(f)
            predicted += r1[k]["iterations"] < r0[k]["iterations"]
        bound = max(1e-9, 8 * r1[k]["cond1"] * 2.0 ** -53)
        assert _rel(c1[k], cfp[k]) <= bound, (float(f), r1[k])
    # the lowest frequencies sit in groups after a fully fallen-back one
    assert predicted >= 2, [(r["tier"], r["iterations"]) for r in r1]
    assert st1["tc_gemm"]["launches"] < st0["tc_gemm"]["launches"]


def test_float_float_second_tier(cuda, wmom):
    """The second tier's LU with complex128 storage and float-float panels and block
    solves (the default), with FP64 block solves (WMOM_FF_TRSM=0), with its matrix in
    float-float form (WMOM_FF_TIER2=1: panels, block solves and the digit-plane
    updates on the FP32 pipe), with FP64 panels (WMOM_FF_PANEL=0), and with the
    digit-plane update on 128 x 64 tiles (WMOM_EMUL_TILE=64): on the ill-conditioned
    junction grid each refines to solutions within 8 kappa_1 eps of the plain FP64
    solve, all in tier 2 (tier 1's acceptance at the residual floor, which keeps the
    0.3 MHz matrix there, is off: WMOM_T1_BERR=0)."""
    w = wmom
    topo = w.Topology(w.geometry.precision_grid(2048))
    freqs = np.array([0.003, 0.03, 0.3], np.float32)
    plan = w.Plan(topo)
    out = {}
    cases = {"ff_panels": {}, "fp64_trsm": {"WMOM_FF_TRSM": "0"}, "ff": {"WMOM_FF_TIER2": "1"},
             "fp64": {"WMOM_FF_TIER2": "0", "WMOM_FF_PANEL": "0"}, "wide_tile": {"WMOM_EMUL_TILE": "64"}}
    keys = ("WMOM_FF_TIER2", "WMOM_FF_PANEL", "WMOM_FF_TRSM", "WMOM_EMUL_TILE", "WMOM_T1_BERR")
    try:
        for name, env in cases.items():
            for k in keys:
                os.environ.pop(k, None)
            os.environ.update(env)
            os.environ["WMOM_T1_BERR"] = "0"
            out[name] = plan.solve(freqs, 1000, mode=w.MODE_MIXED, condest=True)
    finally:
        for k in keys:
            os.environ.pop(k, None)
    c64, _, _ = plan.solve(freqs, 1000, mode=w.MODE_FP64)
    plan.close()
    for ff in cases:
        cur, _, rep = out[ff]
        for k in range(len(freqs)):
            assert rep[k]["status"] == 0 and rep[k]["tier"] == 2, (ff, k, rep[k])
            bound = max(1e-9, 8 * rep[k]["cond1"] * 2.0 ** -53)
            assert _rel(cur[k], c64[k]) <= bound, (ff, float(freqs[k]), rep[k])


@pytest.mark.parametrize("name,loops", [("dipole1m_512", 0), ("random_1024", 0), ("mixed_junctions", 3),
                                        ("ground_monopole", 0), ("ground_frame", 1), ("ground_grid", 9)])
def test_plan_counts_wire_loops(cuda, wmom, name, loops):
    """Independent closed current paths: none for open wires and for a monopole
    standing on a PEC ground, one for a frame whose two legs stand on it (the current
    returns through the plane), one per cell of a grid."""
    _, geo = _fixture(name)
    d, _ = _fixture(name)
    plan = wmom.Plan(wmom.Topology(geo, ienv=int(d["ienv"])))
    if loops is None:
        assert plan.loops >= 0
    else:
        assert plan.loops == loops, (name, plan.loops)
    plan.close()
    g = wmom.geometry
    for geo, want in ((g.precision_grid(2048), 400),
                      (g.geo_text([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)],
                                  [(1, 2, 1e-3, 5), (2, 3, 1e-3, 5), (3, 4, 1e-3, 5), (4, 1, 1e-3, 5)]), 1)):
        plan = wmom.Plan(wmom.Topology(geo))
        assert plan.loops == want
        plan.close()


def test_second_tier_probe(cuda, wmom):
    """A one-group sweep of a structure with loops factors the upper half of its
    frequencies in FP32 first; the lowest of them needs the second tier here (10 kHz
    on the junction grid), so the lower half goes there without FP32 factors.  Each
    matrix must get the answer it gets without the prediction, bit for bit where both
    runs end in the same tier, and the predicted matrices skip their tier-1 steps."""
    w = wmom
    topo = w.Topology(w.geometry.precision_grid(2048))
    plan = w.Plan(topo)
    assert plan.loops > 0
    freqs = np.array([0.002, 20.0, 0.01, 0.001, 5.0, 0.005, 0.03, 0.003], np.float32)  # not sorted
    out = {}
    os.environ["WMOM_LU_BATCH"] = "8"  # the whole sweep is one group
    try:
        for pred in ("0", "1"):
            os.environ["WMOM_TIER_PREDICT"] = pred
            out[pred] = plan.solve(freqs, 1000, mode=w.MODE_MIXED, condest=True)
    finally:
        for k in ("WMOM_LU_BATCH", "WMOM_TIER_PREDICT"):
            os.environ.pop(k, None)
    c0, z0, r0 = out["0"]
    c1, z1, r1 = out["1"]
    cfp, _, _ = plan.solve(freqs, 1000, mode=w.MODE_FP64)
    plan.close()
    skipped = 0
    for k, f in enumerate(freqs):
        assert r1[k]["status"] == 0 and r0[k]["status"] == 0
        if (r0[k]["tier"] >= 2) == (r1[k]["tier"] >= 2):
            assert np.array_equal(c1[k], c0[k]) and z1[k] == z0[k], float(f)
        if f < 0.006:  # the lower half of the sorted sweep
            assert r1[k]["tier"] == 2, (float(f), r1[k])
            skipped += r1[k]["iterations"] < r0[k]["iterations"]
        bound = max(1e-9, 8 * r1[k]["cond1"] * 2.0 ** -53)
        assert _rel(c1[k], cfp[k]) <= bound, (float(f), r1[k])
    assert skipped == 4, [(r["tier"], r["iterations"]) for r in r1]


def test_fp32_solves_through_block_inverses(cuda, wmom):
    """Tier 1's FP32 solves multiply by the inverses of the factors' 64 x 64 diagonal
    blocks (the default) or substitute through each block (WMOM_TRSV_INV=0): both
    refine to the contract against the FP64 form, in the same tiers and about as many
    steps, on random wires and on the junction grid where it stays in tier 1."""
    w = wmom
    for geo, freqs in ((w.geometry.random_wires(1024), [0.01, 1.0, 10.0]),
                       (w.geometry.precision_grid(2048), [2.0, 10.0, 25.0])):
        plan = w.Plan(w.Topology(geo))
        ngap = plan.npls // 2
        freqs = np.array(freqs, np.float32)
        c64, _, r64 = plan.solve(freqs, ngap, mode=w.MODE_FP64, condest=True)
        out = {}
        for inv in ("1", "0"):
            os.environ["WMOM_TRSV_INV"] = inv
            try:
                out[inv] = plan.solve(freqs, ngap, mode=w.MODE_MIXED)
            finally:
                del os.environ["WMOM_TRSV_INV"]
        plan.close()
        for inv, (c, _, r) in out.items():
            for k in range(len(freqs)):
                assert r[k]["status"] == 0, (inv, r[k])
                assert _rel(c[k], c64[k]) < _bound(TOL_MIXED, r64[k]["cond1"]), (inv, float(freqs[k]), r[k])
        r1, r0 = out["1"][2], out["0"][2]
        assert [r["tier"] for r in r1] == [r["tier"] for r in r0]
        assert all(abs(a["iterations"] - b["iterations"]) <= 2 for a, b in zip(r1, r0)), (r1, r0)


def test_second_tier_probe_that_passes(cuda, wmom):
    """The probe's other branch: a one-group sweep of a structure with loops whose upper
    half all stays in tier 1 gives the lower half its FP32 factors afterwards (a second
    batched factorisation) and refines it in tier 1 too.  Every answer, tier and step
    count must equal the unprobed sweep's: factors and solves do not depend on the
    batch they run in."""
    w = wmom
    plan = w.Plan(w.Topology(w.geometry.precision_grid(2048)))
    assert plan.loops > 0
    freqs = np.array([3.0, 25.0, 4.0, 20.0, 6.0, 15.0, 8.0, 10.0], np.float32)
    out = {}
    os.environ["WMOM_LU_BATCH"] = "8"  # the whole sweep is one group
    try:
        for pred in ("0", "1"):
            os.environ["WMOM_TIER_PREDICT"] = pred
            out[pred] = plan.solve(freqs, 1000, mode=w.MODE_MIXED)
    finally:
        for k in ("WMOM_LU_BATCH", "WMOM_TIER_PREDICT"):
            os.environ.pop(k, None)
    plan.close()
    c0, z0, r0 = out["0"]
    c1, z1, r1 = out["1"]
    assert all(r["tier"] == 1 and r["status"] == 0 for r in r1), r1
    assert np.array_equal(c1, c0) and np.array_equal(z1, z0)
    assert [r["iterations"] for r in r1] == [r["iterations"] for r in r0]


def test_tier1_accepts_backward_stable_solutions(cuda, wmom):
    """A matrix whose FP32-factor refinement stops at the FP64 residual floor, above the
    requested tolerance, keeps its tier-1 solution when that solution is backward stable
    at FP64 level (componentwise backward error at most 4 sqrt(n) 2^-53); with the test
    turned off (WMOM_T1_BERR=0) the same matrix falls back to the second tier.  Both
    answers are within 8 kappa_1 eps of the plain FP64 solve (0.3 MHz on the N = 2048
    junction grid)."""
    w = wmom
    plan = w.Plan(w.Topology(w.geometry.precision_grid(2048)))
    freqs = np.array([0.3], np.float32)
    c64, _, r64 = plan.solve(freqs, 1000, mode=w.MODE_FP64, condest=True)
    ca, _, ra = plan.solve(freqs, 1000, mode=w.MODE_MIXED)
    os.environ["WMOM_T1_BERR"] = "0"
    try:
        cb, _, rb = plan.solve(freqs, 1000, mode=w.MODE_MIXED)
    finally:
        del os.environ["WMOM_T1_BERR"]
    plan.close()
    assert ra[0]["status"] == 0 and ra[0]["tier"] == 1 and ra[0]["fell_back"] == 0, ra[0]
    assert ra[0]["rel_residual"] > 1e-12  # stopped at the floor, not at the tolerance
    assert rb[0]["status"] == 0 and rb[0]["tier"] == 2, rb[0]
    bound = _bound(TOL_MIXED, r64[0]["cond1"])
    assert _rel(ca[0], c64[0]) < bound and _rel(cb[0], c64[0]) < bound
