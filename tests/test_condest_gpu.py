"""Condition estimates on the device against LAPACK:
* wmom_zgecon on factors uploaded from scipy's zgetrf runs the estimator of LAPACK's
  zgecon (zlacn2: solves with A and with A^H) and must return scipy zgecon's rcond on
  the same factors -- the same sequence of steps, so the same estimate up to the
  rounding of the triangular solves;
* wmom_zlange1 is ||A||_1;
* the sweep's cond1 (WMOM_SOLVE_CONDEST) in both forms against zgecon on the
  oracle's matrix of the same system (different factors: within a factor of 2).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_factors(cuda, a):
    from scipy.linalg import lapack
    lu, piv, info = lapack.zgetrf(np.asfortranarray(a))
    assert info == 0
    d_lu = cuda.from_numpy(np.ascontiguousarray(lu.T)).to("cuda")  # column-major storage
    d_piv = cuda.from_numpy((piv + 1).astype(np.int32)).to("cuda")  # 1-based, as wmom_zgetrf's
    return lu, piv, d_lu, d_piv


def _cases():
    rng = np.random.default_rng(11)
    out = []
    for n in (300, 1000):
        a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
        out.append((f"random{n}", a))
    n = 640
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    a[:, 7] = a[:, 9] + 1e-9 * a[:, 7]
    out.append(("near_singular640", a))
    # exact Gaussian-integer system with kappa_1 = 1.4e13 (as in test_oracle_truth)
    n = 64
    r2 = np.random.default_rng(7)
    u = r2.integers(-9, 10, n) + 1j * r2.integers(-9, 10, n)
    u[-1] = 1
    v = r2.integers(-9, 10, n) + 1j * r2.integers(-9, 10, n)
    v[-1] = 0
    v[-1] = -(v @ u)
    a = (np.eye(n) + 30 * np.outer(u, v)).astype(np.complex128)
    out.append(("rank_one64", a[r2.permutation(n)][:, r2.permutation(n)]))
    # n not a multiple of the 64-row solve blocks
    n = 197
    out.append(("random197", rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))))
    return out


@pytest.mark.parametrize("name,a", _cases(), ids=[c[0] for c in _cases()])
def test_zgecon_matches_lapack_on_the_same_factors(cuda, wmom, name, a):
    from scipy.linalg import lapack
    n = a.shape[0]
    lu, piv, d_lu, d_piv = _device_factors(cuda, a)
    anorm = float(np.max(np.sum(np.abs(a), axis=0)))
    rc_ref, info = lapack.zgecon(lu, anorm, norm="1")
    rc = wmom.zgecon_device(d_lu.data_ptr(), n, n, d_piv.data_ptr(), anorm)
    assert rc == pytest.approx(rc_ref, rel=1e-6), (rc, rc_ref)
    # the estimate is a lower bound of the exact kappa_1, within the usual factor of 3
    exact = np.linalg.cond(a, 1)
    assert exact / 3.0 <= 1.0 / rc <= exact * (1 + 1e-6)


def test_zlange1(cuda, wmom):
    rng = np.random.default_rng(5)
    a = rng.normal(size=(777, 777)) + 1j * rng.normal(size=(777, 777))
    d = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
    v = wmom.zlange1_device(d.data_ptr(), 777, 777)
    assert v == pytest.approx(np.linalg.norm(a, 1), rel=1e-6)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_sweep_reports_condition_estimates(cuda, wmom, orc, mode):
    w = wmom
    topo = w.Topology(w.geometry.precision_grid(2048))
    plan = w.Plan(topo)
    freqs = np.array([0.01, 1.0, 10.0], np.float32)
    m = w.MODE_FP64 if mode == "fp64" else w.MODE_MIXED
    _, _, rep = plan.solve(freqs, 1000, mode=m, condest=True, currents=False)
    _, _, rep0 = plan.solve(freqs, 1000, mode=m, currents=False)
    g = orc.topology(w.geometry.precision_grid(2048))
    for k, f in enumerate(freqs):
        z = orc.fill(g, float(f), threads=8)
        kappa, _ = orc.cond1(z)
        assert rep0[k]["cond1"] == 0.0
        est = rep[k]["cond1"]
        assert kappa / 2.0 <= est <= 2.0 * kappa, (float(f), est, kappa, rep[k]["tier"])
    plan.close()
