"""Pins the CPU oracle before it is trusted as the checker:
* against the input impedances the reference printed in its own run logs
  (4 significant digits, 25 m dipole, a = 0.5 mm, gap 100, "Freq =" lines of
  results_P_F_N.txt in all four program variants);
* against the reference's own zmatrix() output and MKL currents (fixtures made by
  tests/golden/make_golden.py from the reference compiled unmodified);
* the C restatement of LAPACK's unblocked LU against scipy's zgetrf;
* the C restatement of the reference's geoinp + configwire (the topology of the CPU
  reference path) against the reference's own config() arrays.
"""
import glob
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _logs():
    with open(os.path.join(GOLDEN, "zin_logs.json")) as f:
        return json.load(f)


def _ulp4(text):
    """Half a unit in the last printed digit of a value printed with 4 significant
    digits (the reference's leaked setprecision(4), Wire_MoM.cu:24,394)."""
    v = abs(float(text))
    if v == 0.0:
        return 5e-5
    return 0.5 * 10.0 ** (math.floor(math.log10(v)) - 3)


def test_logs_agree_across_variants():
    by = {}
    for r in _logs():
        by.setdefault((r["nsw"], r["freq"]), set()).add((r["re_text"], r["im_text"]))
    assert len(by) >= 300
    conflicts = [k for k, v in by.items() if len(v) > 1]
    # one known artefact: interleaved stdout of 12 MPI ranks in one 512-segment log
    assert len(conflicts) <= 1, conflicts


@pytest.mark.parametrize("nsw", [512, 768, 1024])
def test_oracle_reproduces_logged_zin(orc, wmom, nsw):
    rows = {}
    for r in _logs():
        if r["nsw"] == nsw:
            rows.setdefault(r["freq"], r)
    assert rows, "no log lines for this size"
    topo = wmom.Topology(wmom.geometry.dipole(25.0, 5e-4, nsw))
    g = topo.arrays()
    nbad = 0
    for f, r in sorted(rows.items()):
        _, zin, _ = orc.solve(g, f, 100, threads=os.cpu_count() or 1)
        ok = abs(zin.real - r["re"]) <= 1.01 * _ulp4(r["re_text"]) and abs(zin.imag - r["im"]) <= 1.01 * _ulp4(
            r["im_text"])
        nbad += not ok
    assert nbad == 0


@pytest.mark.parametrize("name", ["dipole64", "grid5_ns3", "bent_ground", "mixed_junctions", "dipole25m_lowf",
                                  "ground_monopole", "ground_frame", "ground_grid"])
def test_oracle_fill_matches_reference_zmatrix(orc, wmom, name):
    d = np.load(os.path.join(GOLDEN, f"zfill_{name}.npz"))
    ienv = int(d["ienv"])
    topo = wmom.Topology(str(d["geo"]), ienv=ienv)
    z = orc.fill(topo.arrays(), float(d["freq"]), ienv=ienv, sgn=topo.sgn)
    zr = d["z"]
    scale = np.max(np.abs(zr), axis=0)
    assert np.max(np.abs(z - zr) / scale) < 1e-14


@pytest.mark.parametrize("name", ["dipole1m_512", "dipole25m_512", "mixed_junctions", "random_1024", "ground_monopole",
                                  "ground_frame", "ground_grid"])
def test_oracle_currents_match_reference_mkl(orc, wmom, name):
    d = np.load(os.path.join(GOLDEN, f"currents_{name}.npz"))
    ienv = int(d["ienv"])
    topo = wmom.Topology(str(np.load(os.path.join(GOLDEN, f"topology_{name}.npz"))["geo"]), ienv=ienv)
    g = topo.arrays()
    freqs = d["freqs"][:4]
    for k, f in enumerate(freqs):
        i, zin, _ = orc.solve(g, float(f), int(d["ngap"]), ienv=ienv, sgn=topo.sgn, threads=os.cpu_count() or 1)
        ir = d["currents"][k]
        assert np.linalg.norm(i - ir) / np.linalg.norm(ir) < 1e-10
        assert abs(zin - d["zin"][k]) / abs(d["zin"][k]) < 1e-10


def test_oracle_zgetf2_matches_lapack(orc):
    from scipy.linalg import lapack
    rng = np.random.default_rng(7)
    for n in (1, 2, 5, 17, 40):
        a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        lu, ipiv, info = orc.zgetf2(a)
        lu2, piv2, info2 = lapack.zgetrf(np.asfortranarray(a))
        assert info == info2 == 0
        assert np.array_equal(ipiv, piv2 + 1)
        assert np.allclose(lu, lu2, rtol=1e-12, atol=1e-12)
        b = rng.normal(size=n) + 1j * rng.normal(size=n)
        x = orc.zgetrs(lu, ipiv, b)
        assert np.allclose(a @ x, b, rtol=1e-10, atol=1e-10)


def test_oracle_zgetf2_ties_and_zero_pivot(orc):
    # |re|+|im| ties: the first row wins (izamax)
    a = np.array([[1 + 1j, 3, 0], [2 + 0j, 1, 1], [0 + 2j, 5, 2]], np.complex128)
    lu, ipiv, info = orc.zgetf2(a)
    assert ipiv[0] == 1  # |1+1j|_1 = 2 ties with rows 2 and 3: first occurrence
    s = np.zeros((3, 3), np.complex128)
    s[:, 0] = [1, 2, 3]
    s[:, 1] = [2, 4, 6]
    s[:, 2] = [0, 1, 1]
    _, _, info = orc.zgetf2(s)
    assert info == 2


def test_ka_matches_reference_formula(orc, wmom):
    for f in (0.001, 0.01, 1.0, 100.0, 150.0, 1200.0):
        c = 2.99792448e8
        lam = c / float(np.float32(f)) * 1e-6
        assert orc.ka(f) == (math.pi + math.pi) / lam
        assert wmom.ka(f) == orc.ka(f)


TOPO_NAMES = sorted(os.path.basename(p)[len("topology_"):-4]
                    for p in glob.glob(os.path.join(GOLDEN, "topology_*.npz")))


@pytest.mark.parametrize("name", TOPO_NAMES)
def test_oracle_topology_matches_reference(orc, name):
    """The oracle's topology equals the reference's config() output, bit for bit."""
    d = np.load(os.path.join(GOLDEN, f"topology_{name}.npz"))
    t = orc.topology(str(d["geo"]), ienv=int(d["ienv"]), nsmax=int(d["nsmax"]))
    assert (t["npls"], t["nseg"], t["npnt"]) == (int(d["npls"]), int(d["nseg"]), int(d["npnt"]))
    ns, npl, npnt, S = t["nseg"], t["npls"], t["npnt"], t["nsmax"]
    for k in ("x", "y", "z"):
        assert np.array_equal(t[k][:npnt], d[k]), k
    assert np.array_equal(t["rad"][:ns], d["rad"])
    assert np.array_equal(t["ipc"][:npl], d["ipc"])
    assert np.array_equal(t["ips"][:npl], d["ips1"]) and np.array_equal(t["ips"][S:S + npl], d["ips2"])
    assert np.array_equal(t["ise"][:ns], d["ise1"]) and np.array_equal(t["ise"][S:S + ns], d["ise2"])
    assert np.array_equal(t["isp"][:ns], d["isp1"]) and np.array_equal(t["isp"][S:S + ns], d["isp2"])


@pytest.mark.parametrize("kind", ["random_8192", "grid_8192", "random_14336", "ground"])
def test_oracle_topology_equals_product_whole_arrays(orc, wmom, kind):
    """Benchmark geometries: the oracle's arrays (the CPU reference path's) and the
    product's host builder agree on every slot, so both arms of the benchmark solve
    the same systems."""
    g = wmom.geometry
    text, ienv = {"random_8192": (g.random_wires(8192, seed=20261203), 1),
                  "grid_8192": (g.precision_grid(8192), 1),
                  "random_14336": (g.random_wires(14336, seed=20261203), 1),
                  "ground": (g.geo_text([(0, 0, 0), (0, 0, 1.0), (1.0, 0, 1.0)],
                                        [(1, 2, 1e-3, 20), (2, 3, 1e-3, 20)]), 2)}[kind]
    a = wmom.Topology(text, ienv=ienv, listing=False)
    b = orc.topology(text, ienv=ienv)
    assert (a.npls, a.nseg, a.npnt) == (b["npls"], b["nseg"], b["npnt"])
    for k in ("x", "y", "z", "rad", "ipc", "ips", "ise", "isp", "iwe"):
        assert np.array_equal(getattr(a, k), b[k]), k


@pytest.mark.parametrize("text", ["c\nc\n", "c\nc\n2\n0 0 0\n", "c\nc\n4000\n"])
def test_oracle_topology_rejects_bad_input(orc, text):
    with pytest.raises(ValueError):
        orc.topology(text)
