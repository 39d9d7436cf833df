"""GPU fill (libwmom, fill.cu) against the oracle fill and the reference's own
zmatrix() output (fixtures), entry by entry."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

# Per column, |Z_gpu - Z_ref| <= TOL * max|Z_ref column|: the two differ only in the
# last-bit rounding of the device sin/cos against the host libm.
TOL = 1e-13


def _gpu_fill(wmom, topo, freqs):
    plan = wmom.Plan(topo)
    z = plan.fill(freqs)
    out = [z[k].T.cpu().numpy() for k in range(len(freqs))]
    plan.close()
    return out


@pytest.mark.parametrize("name", ["dipole64", "grid5_ns3", "bent_ground", "mixed_junctions", "dipole25m_lowf",
                                  "ground_monopole", "ground_frame", "ground_grid"])
def test_fill_matches_reference_fixture(cuda, wmom, name):
    d = np.load(os.path.join(GOLDEN, f"zfill_{name}.npz"))
    topo = wmom.Topology(str(d["geo"]), ienv=int(d["ienv"]))
    (z,) = _gpu_fill(wmom, topo, [float(d["freq"])])
    zr = d["z"]
    err = np.max(np.abs(z - zr) / np.max(np.abs(zr), axis=0))
    assert err < TOL, err


@pytest.mark.parametrize("geo,freqs", [
    ("dipole", [0.01, 1.0, 150.0, 1200.0]),
    ("grid", [0.001, 0.1, 10.0, 30.0]),
    ("random", [0.01, 3.0, 10.0]),
])
def test_fill_matches_oracle_batched(cuda, wmom, orc, geo, freqs):
    g = wmom.geometry
    text = {"dipole": g.dipole(1.0, 1e-3, 300), "grid": g.grid(7, 1.0, 1.0, 5e-3, None, 3),
            "random": g.random_wires(600, seed=11)}[geo]
    topo = wmom.Topology(text)
    zs = _gpu_fill(wmom, topo, freqs)
    for f, z in zip(freqs, zs):
        zr = orc.fill(topo.arrays(), f, threads=os.cpu_count() or 1)
        err = np.max(np.abs(z - zr) / np.max(np.abs(zr), axis=0))
        assert err < TOL, (f, err)


def test_fill_batch_invariance(cuda, wmom):
    # a matrix is bit-identical whether filled alone or inside a batch
    topo = wmom.Topology(wmom.geometry.random_wires(400, seed=5))
    freqs = [0.01, 0.5, 7.0, 10.0]
    batch = _gpu_fill(wmom, topo, freqs)
    for f, zb in zip(freqs, batch):
        (za,) = _gpu_fill(wmom, topo, [f])
        assert np.array_equal(za, zb)


def test_fill_rejects_bad_arguments(cuda, wmom):
    topo = wmom.Topology(wmom.geometry.dipole(1.0, 1e-3, 32))
    plan = wmom.Plan(topo)
    import torch
    z = torch.empty((1, 31, 31), dtype=torch.complex128, device="cuda")
    with pytest.raises(wmom.WmomError):
        plan.fill_device(np.array([-1.0]), z.data_ptr(), 31, 31 * 31)
    with pytest.raises(wmom.WmomError):
        plan.fill_device(np.array([1.0]), z.data_ptr(), 30, 31 * 31)
    plan.close()


@pytest.mark.parametrize("geo", ["dipole", "grid", "random", "junctions"])
def test_pair_tiled_fill_equals_per_entry_fill(cuda, wmom, geo):
    # the pair-tiled kernel evaluates each distinct (observation, source) pair once and
    # assembles entries from them; it must reproduce the per-entry kernel exactly
    g = wmom.geometry
    text = {"dipole": g.dipole(1.0, 1e-3, 200), "grid": g.grid(6, 1.0, 1.0, 5e-3, None, 3),
            "random": g.random_wires(500, seed=2),
            "junctions": str(np.load(os.path.join(GOLDEN, "topology_mixed_junctions.npz"))["geo"])}[geo]
    topo = wmom.Topology(text)
    freqs = [0.01, 2.0, 30.0]
    plan = wmom.Plan(topo)
    assert plan.fill_variant == "pair"
    zp = plan.fill(freqs).cpu().numpy()
    os.environ["WMOM_FILL_ENTRY"] = "1"
    try:
        ze = plan.fill(freqs).cpu().numpy()
    finally:
        del os.environ["WMOM_FILL_ENTRY"]
    plan.close()
    assert np.array_equal(zp, ze)


def test_fill_of_uneven_geometries_in_one_call_equals_per_geometry_fill(cuda, wmom):
    """Geometries of uneven size (free space, and one over a ground plane), one
    frequency each, filled by one wmom_fill_geometries call: every matrix equals the
    per-geometry fill bit for bit (same tile arithmetic, one ragged launch)."""
    import torch
    g = wmom.geometry
    d = np.load(os.path.join(GOLDEN, "topology_bent_ground.npz"))
    topos = [wmom.Topology(g.random_wires(300, seed=3)), wmom.Topology(g.dipole(1.0, 1e-3, 64)),
             wmom.Topology(str(d["geo"]), ienv=2), wmom.Topology(g.grid(5, 1.0, 1.0, 5e-3, None, 3)),
             wmom.Topology(g.random_wires(1000, seed=4))]
    freqs = [3.0, 150.0, 30.0, 10.0, 0.5]
    plans = [wmom.Plan(t) for t in topos]
    try:
        assert [p.fill_variant for p in plans].count("entry") == 1
        zs = wmom.fill_geometries(plans, freqs)
        for p, f, z in zip(plans, freqs, zs):
            zr = p.fill([f])[0]
            assert z.shape == zr.shape and torch.equal(z, zr), (p.npls, f)
        with pytest.raises(ValueError):
            wmom.fill_geometries(plans, freqs[:2])
    finally:
        for p in plans:
            p.close()


def test_ground_plane_uses_per_entry_fill(cuda, wmom):
    d = np.load(os.path.join(GOLDEN, "topology_bent_ground.npz"))
    plan = wmom.Plan(wmom.Topology(str(d["geo"]), ienv=2))
    assert plan.fill_variant == "entry"
    plan.close()


def test_table_sincos_against_cuda_sincos(cuda, wmom):
    """The fill's table-driven sin/cos against CUDA's sincos() over the phase range
    the fill meets (k*R up to ~1e3 rad), the table nodes j*pi/128 and their
    half-way points, tiny and zero arguments, and the 1e6 hand-over to sincos()."""
    import torch
    rng = np.random.default_rng(7)
    h = np.pi / 128
    j = np.arange(-600, 60000, dtype=np.float64)
    x = np.concatenate([
        rng.uniform(0.0, 30.0, 200000), rng.uniform(0.0, 1e3, 200000), 10.0 ** rng.uniform(-12, 0, 20000),
        j * h, (j + 0.5) * h, np.nextafter((j + 0.5) * h, 0), -rng.uniform(0, 50, 1000),
        [0.0, -0.0, 5e-324, 999999.0, 1e6, 1e6 + 0.5, 3e7]])
    s, c, sr, cr = (t.cpu().numpy() for t in wmom.diag_sincos(torch.from_numpy(x).cuda()))
    err = max(np.max(np.abs(s - sr)), np.max(np.abs(c - cr)))
    # a few units in the last place of a number of magnitude <= 1
    assert err <= 4.5e-16, err
    small = np.abs(x) < 1e-3
    assert np.max(np.abs(s[small] - sr[small]) / np.maximum(np.abs(sr[small]), 1e-300)) <= 4.5e-16
    assert np.all(np.abs(s * s + c * c - 1.0) <= 1e-15)


@pytest.mark.parametrize("geo", ["random", "grid"])
def test_multi_frequency_fill_equals_per_frequency_fill(cuda, wmom, geo, monkeypatch):
    """The tile kernel that keeps each pair's geometry across a batch of frequencies
    gives bit-identical matrices to the one-frequency-per-CTA kernel."""
    topo = wmom.Topology(wmom.geometry.random_wires(700, seed=3) if geo == "random"
                         else wmom.geometry.grid(8, 1.0, 1.0, 5e-3, None, 4))
    freqs = [0.01, 0.7, 3.0, 10.0]
    plan = wmom.Plan(topo)
    z_multi = plan.fill(freqs).cpu().numpy()
    monkeypatch.setenv("WMOM_FILL_SINGLE", "1")
    z_single = plan.fill(freqs).cpu().numpy()
    plan.close()
    assert np.array_equal(z_multi, z_single)
