"""The host topology builder (geoinp + configwire restated in C++, libwmom) against
the reference's own configwire() output arrays and configwire.txt text
(fixtures from tests/golden/make_golden.py), bit for bit."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

NAMES = sorted(os.path.basename(p)[len("topology_"):-4] for p in glob.glob(os.path.join(GOLDEN, "topology_*.npz")))


@pytest.mark.parametrize("name", NAMES)
def test_topology_matches_reference(wmom, name):
    d = np.load(os.path.join(GOLDEN, f"topology_{name}.npz"))
    t = wmom.Topology(str(d["geo"]), ienv=int(d["ienv"]), nsmax=int(d["nsmax"]))
    assert (t.npls, t.nseg, t.npnt) == (int(d["npls"]), int(d["nseg"]), int(d["npnt"]))
    ns, npl, npnt, nsmax = t.nseg, t.npls, t.npnt, t.nsmax
    for k in ("x", "y", "z"):
        assert np.array_equal(getattr(t, k)[:npnt], d[k]), k
    assert np.array_equal(t.rad[:ns], d["rad"])
    assert np.array_equal(t.ipc[:npl], d["ipc"])
    assert np.array_equal(t.ips[:npl], d["ips1"]) and np.array_equal(t.ips[nsmax:nsmax + npl], d["ips2"])
    assert np.array_equal(t.ise[:ns], d["ise1"]) and np.array_equal(t.ise[nsmax:nsmax + ns], d["ise2"])
    assert np.array_equal(t.isp[:ns], d["isp1"]) and np.array_equal(t.isp[nsmax:nsmax + ns], d["isp2"])
    assert t.listing == str(d["listing"])


def test_unknown_counts_of_benchmark_geometries(wmom):
    g = wmom.geometry
    assert wmom.Topology(g.dipole(1.0, 1e-3, 512)).npls == 511
    for n in (2048, 8192):
        assert wmom.Topology(g.precision_grid(n)).npls == n
    for n in (1024, 4096):
        assert wmom.Topology(g.random_wires(n, seed=3)).npls == n


@pytest.mark.parametrize("text", [
    "c\nc\n",                                   # no node count
    "c\nc\n2\n0 0 0\n",                         # truncated nodes
    "c\nc\n2\n0 0 0\n0 0 1\n1\n1 3 0.001 4\n0\n",  # wire to a missing node
    "c\nc\n4000\n",                             # more nodes than nnmax
])
def test_bad_geometry_is_an_error(wmom, text):
    with pytest.raises(wmom.WmomError) as e:
        wmom.Topology(text)
    assert e.value.status == 7


def test_ground_rejects_negative_z(wmom):
    text = wmom.geometry.geo_text([(0, 0, -1.0), (0, 0, 1.0)], [(1, 2, 1e-3, 8)])
    with pytest.raises(wmom.WmomError):
        wmom.Topology(text, ienv=2)


def test_segment_limit(wmom):
    text = wmom.geometry.dipole(1.0, 1e-3, 200)
    with pytest.raises(wmom.WmomError):
        wmom.Topology(text, nsmax=150, nwmax=10)


def test_whole_arrays_match_the_reference_build(wmom, orc):
    """Every slot of the product's arrays, including the ones no basis function
    reaches (the reference's in-place shift leaves the second column's first entry in
    slot nsmax - 1), against the reference's own config() compiled here.  The last
    slot of each array is left out: the reference reads one entry past its array
    there."""
    if not orc.ref_available():
        pytest.skip("the reference's own build (oracle/_ref) exists only where the reference checkout is")
    g = wmom.geometry
    for text, ienv in ((g.precision_grid(2048), 1), (g.random_wires(1024, seed=20261203), 1),
                       (g.geo_text([(0, 0, 0), (0, 0, 1.0), (1.0, 0, 1.0)],
                                   [(1, 2, 1e-3, 20), (2, 3, 1e-3, 20)]), 2)):
        r = orc.ref_geometry(text, ienv=ienv)
        t = wmom.Topology(text, ienv=ienv, nsmax=r["nsmax"], listing=False)
        for k in ("x", "y", "z", "rad", "ipc", "ips", "ise", "isp", "iwe"):
            assert np.array_equal(getattr(t, k)[:-1], r[k][:-1]), k
