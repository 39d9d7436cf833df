"""Pins the oracle's extended-precision truth and its condition estimate before they
are trusted as checkers (CPU only):
* on an exact Gaussian-integer system with kappa_1 = 1.4e13, where LAPACK's FP64
  solve is off by about 1e-7, iterative refinement with double-double residuals
  recovers the exact integer solution;
* the double-double residual of the exact solution is exactly zero;
* LAPACK zgecon's estimate (oracle.cond1) never exceeds the exact kappa_1 and is
  within a factor of 3 of it on random systems;
* the large fixtures (the reference's own fill + MKL at the benchmark sizes) are
  consistent: MKL lies within the conditioning bound of the truth, and the seeded
  geometry generators still produce the exact .geo text the fixtures were made from.
"""
import glob
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN

EPS = 2.0 ** -53
KAPPA_FACTOR = 8  # forward error <= max(tolerance, KAPPA_FACTOR * kappa_1 * eps)


def _integer_system(c=30, n=64, seed=7):
    """A = I + c u v^T with Gaussian-integer u, v and v^T u = 0, rows and columns
    permuted: A^-1 = I - c u v^T exactly, kappa_1 grows as c^2; x and b = A x are
    Gaussian integers held exactly in complex128."""
    rng = np.random.default_rng(seed)
    u = rng.integers(-9, 10, n) + 1j * rng.integers(-9, 10, n)
    u[-1] = 1
    v = rng.integers(-9, 10, n) + 1j * rng.integers(-9, 10, n)
    v[-1] = 0
    v[-1] = -(v @ u)
    assert v @ u == 0
    a = (np.eye(n) + c * np.outer(u, v)).astype(np.complex128)
    a = a[rng.permutation(n)][:, rng.permutation(n)]
    x = (rng.integers(-1000, 1000, n) + 1j * rng.integers(-1000, 1000, n)).astype(np.complex128)
    b = a @ x
    assert np.max(np.abs(b)) < 2.0 ** 52
    return a, x, b


def test_truth_recovers_exact_solution_of_ill_conditioned_system(orc):
    a, x, b = _integer_system()
    kappa = np.linalg.cond(a, 1)
    assert kappa > 1e13
    x0, info, f = orc.lu_solve(a, b, return_factors=True)
    err_lapack = np.linalg.norm(x0 - x) / np.linalg.norm(x)
    assert err_lapack > 1e-9  # FP64 LU alone is far from the exact solution here
    xt, hist = orc.refine_truth(a, b, x0, factors=f)
    assert np.array_equal(xt, x), (np.linalg.norm(xt - x) / np.linalg.norm(x), hist)
    assert hist[-1] <= 2.0 ** -100


def test_dd_residual_of_exact_solution_is_zero(orc):
    a, x, b = _integer_system(c=300)
    rh, rl = orc.residual_dd(a, b, x)
    assert not np.any(rh) and not np.any(rl)
    # and a perturbed solution gives the residual of the perturbation exactly
    d = np.zeros_like(x)
    d[3] = 2.0 ** -30
    rh, _ = orc.residual_dd(a, b, x + d)
    assert np.allclose(rh, -a[:, 3] * 2.0 ** -30, rtol=0, atol=0)


@pytest.mark.parametrize("seed", range(4))
def test_zgecon_estimate_is_a_tight_lower_bound(orc, seed):
    rng = np.random.default_rng(seed)
    n = 120
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    a[:, 5] = a[:, 6] + 1e-6 * a[:, 5]  # moderately ill-conditioned
    exact = np.linalg.cond(a, 1)
    est, anorm = orc.cond1(a)
    assert anorm == pytest.approx(np.linalg.norm(a, 1), rel=1e-12)
    assert est <= exact * (1 + 1e-8) and est >= exact / 3.0, (est, exact)


LARGE = sorted(glob.glob(os.path.join(GOLDEN, "large_*.npz")))


@pytest.mark.parametrize("path", LARGE, ids=[os.path.basename(p) for p in LARGE])
def test_large_fixture_consistent(wmom, path):
    d = np.load(path)
    name = os.path.basename(path)[len("large_"):-4]
    kind, n = name.rsplit("_", 1)
    g = wmom.geometry
    text = g.precision_grid(int(n)) if kind == "precision" else g.random_wires(int(n), seed=20261203)
    assert hashlib.sha256(text.encode()).hexdigest() == str(d["geo_sha256"])
    assert int(d["npls"]) == int(n) and d["currents_mkl"].shape == (len(d["freqs"]), int(n))
    for k, f in enumerate(d["freqs"]):
        kappa = float(d["kappa1"][k])
        err = np.linalg.norm(d["currents_mkl"][k] - d["truth"][k]) / np.linalg.norm(d["truth"][k])
        assert err == pytest.approx(float(d["mkl_vs_truth"][k]), rel=1e-6)
        assert err <= max(1e-13, KAPPA_FACTOR * kappa * EPS), (f, err, kappa)
