"""Host-side logic that needs no GPU: excitation, frequencies, argument checks."""
import numpy as np
import pytest


def test_excitation_matches_reference(wmom, orc):
    for ngap, ampl, phas in ((1, 1.0, 0.0), (100, 2.5, 30.0), (7, -1.0, 90.0)):
        v = wmom.excitation(128, ngap, ampl, phas)
        vr = orc.excitation(128, ngap, ampl, phas)
        assert np.array_equal(np.nonzero(v)[0], [ngap - 1])
        assert abs(v[ngap - 1] - vr[ngap - 1]) <= 1e-15 * abs(vr[ngap - 1])


def test_excitation_rejects_bad_gap(wmom):
    for ngap in (0, 129):
        with pytest.raises(wmom.WmomError):
            wmom.excitation(128, ngap)


def test_freq_file_parsing(wmom):
    text = "3\n1.00000000e+02\n2.5e2\n10.00000000e+02\n4.0e2\n"
    f = wmom.read_freq_file(text)
    assert f.dtype == np.float32 and list(f) == [100.0, 250.0, 1000.0]


def test_sweep_frequencies():
    import importlib
    g = importlib.import_module("praca-magisterska_gb300.geometry")
    f = g.sweep_freqs()
    assert len(f) == 12 and abs(f[0] - 0.01) < 1e-9 and abs(f[-1] - 10.0) < 1e-6
    assert np.all(np.diff(f) > 0)


def test_padded_order_classes(wmom):
    """Size classes of wmom_factor_geometries: at least n, at most 1.25 n above 256 (four
    classes per octave), a multiple of 64, and the class of the class is itself."""
    prev = 0
    for n in range(1, 20481, 7):
        p = wmom.padded_order(n)
        assert p >= n and p % 64 == 0 and p >= prev
        if n > 256:
            assert p <= 1.25 * n
        assert wmom.padded_order(p) == p
        prev = p
