"""FP64 LU with partial pivoting and the triangular solves (lu.cu) against LAPACK
semantics: the same pivot sequence as zgetf2 on matrices without ties, factors and
solutions within rounding, zero-pivot info, the host-buffer zgesv drop-in."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(n, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))


def _lu_device(cuda, wmom, a):
    n = a.shape[0]
    at = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")  # column-major storage of a
    ipiv = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    info = wmom.zgetrf_device(at.data_ptr(), n, n, ipiv.data_ptr())
    cuda.cuda.synchronize()
    return at, ipiv, info


@pytest.mark.parametrize("n", [1, 3, 63, 64, 65, 130, 257, 700])
def test_lu_pivots_and_factors_match_zgetf2(cuda, wmom, orc, n):
    a = _rand(n, n)
    at, ipiv, info = _lu_device(cuda, wmom, a)
    lu = at.cpu().numpy().T
    lu_r, ipiv_r, info_r = orc.zgetf2(a)
    assert info == info_r == 0
    assert np.array_equal(ipiv.cpu().numpy(), ipiv_r)
    assert np.max(np.abs(lu - lu_r)) <= 1e-11 * max(1.0, np.max(np.abs(lu_r)))


@pytest.mark.parametrize("n,nrhs", [(1, 1), (100, 1), (200, 3), (513, 2)])
def test_solve_matches_lapack(cuda, wmom, n, nrhs):
    from scipy.linalg import lapack
    a = _rand(n, 100 + n)
    b = np.random.default_rng(1).normal(size=(n, nrhs)) + 0j
    at, ipiv, info = _lu_device(cuda, wmom, a)
    bt = cuda.from_numpy(np.ascontiguousarray(b.T)).to("cuda")
    wmom.zgetrs_device(n, nrhs, at.data_ptr(), n, ipiv.data_ptr(), bt.data_ptr(), n)
    x = bt.cpu().numpy().T
    lu, piv, _ = lapack.zgetrf(np.asfortranarray(a))
    xr, _ = lapack.zgetrs(lu, piv, b)
    assert np.max(np.abs(x - xr)) <= 1e-10 * np.max(np.abs(xr))


def test_zero_pivot_reports_info(cuda, wmom, orc):
    a = np.zeros((80, 80), np.complex128)
    a[np.arange(80), np.arange(80)] = 1.0
    a[:, 40] = 0.0
    at, ipiv, info = _lu_device(cuda, wmom, a)
    _, _, info_r = orc.zgetf2(a)
    assert info == info_r == 41


def test_zgesv_like_dropin(cuda, wmom):
    n = 150
    a = _rand(n, 3)
    v = np.zeros(n, np.complex128)
    v[9] = 1.0
    i, lu, ipiv, info = wmom.zgesv_like(a, v)
    assert info == 0
    assert np.linalg.norm(a @ i - v) < 1e-11 * np.linalg.norm(a) * np.linalg.norm(i)
    from scipy.linalg import lapack
    lu_r, piv_r, _ = lapack.zgetrf(np.asfortranarray(a))
    assert np.array_equal(ipiv, piv_r + 1)


def test_large_lu_residual(cuda, wmom):
    n = 2000
    a = _rand(n, 77)
    at, ipiv, info = _lu_device(cuda, wmom, a)
    b = np.ones((n, 1), np.complex128)
    bt = cuda.from_numpy(np.ascontiguousarray(b.T)).to("cuda")
    wmom.zgetrs_device(n, 1, at.data_ptr(), n, ipiv.data_ptr(), bt.data_ptr(), n)
    x = bt.cpu().numpy().T
    r = np.linalg.norm(a @ x - b) / (np.linalg.norm(a, 1) * np.linalg.norm(x, 1))
    assert r < 1e-14


def _plu_backward_error(a, lu, ipiv):
    n = a.shape[0]
    L = np.tril(lu, -1) + np.eye(n)
    U = np.triu(lu)
    pa = a.copy()
    for i, p in enumerate(ipiv - 1):
        pa[[i, p]] = pa[[p, i]]
    return np.linalg.norm(pa - L @ U) / np.linalg.norm(a), np.max(np.abs(L))


# sizes: one row per thread of a single panel block, panel edges, several blocks per
# panel (the row-owner panel's grid barrier), several panels with tensor-core updates
@pytest.mark.parametrize("n", [1, 63, 65, 257, 700, 2000, 4100])
def test_fp32_lu_backward_error(cuda, wmom, n):
    """The precision form's LU (FP32 panels, 3xTF32 tensor-core updates): P A = L U to
    FP32 accuracy.  Bound: ||PA - LU||_F / ||A||_F at most 10x that of LAPACK cgetrf
    (FP32) on the same matrix: a 3xTF32 product hi*hi' + hi*lo' + lo*hi' keeps a
    relative error of about 3 * 2^-22 (TF32 tails, lo*lo' dropped) against FP32's
    2^-24 rounding; observed 2-5x.  And |l_ij| <= sqrt(2) (|re|+|im| pivoting)."""
    from scipy.linalg import lapack
    a = _rand(n, 1000 + n).astype(np.complex64)
    at = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
    ipiv = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    info = wmom.cgetrf_device(at.data_ptr(), n, n, ipiv.data_ptr())
    cuda.cuda.synchronize()
    assert info == 0
    lu = at.cpu().numpy().T.astype(np.complex128)
    err, lmax = _plu_backward_error(a.astype(np.complex128), lu, ipiv.cpu().numpy())
    lu_c, piv_c, info_c = lapack.cgetrf(a)
    err_c, _ = _plu_backward_error(a.astype(np.complex128), lu_c.astype(np.complex128), piv_c + 1)
    assert err <= 10.0 * err_c + 1e-7, (err, err_c)
    assert lmax <= np.sqrt(2.0) * (1 + 1e-5), lmax


@pytest.mark.parametrize("n", [7500, 9000])
def test_fp32_lu_large_panels(cuda, wmom, n):
    """Sizes whose first panels need the widest clusters and a panel narrower than 64
    columns (n = 7500), or two rows per thread (n = 9000): P A = L U checked on random
    probe vectors (a wrong update or interchange gives an O(1) residual; FP32 rounding
    gives ~1e-5)."""
    rng = np.random.default_rng(n)
    a = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
    at = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
    ipiv = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    info = wmom.cgetrf_device(at.data_ptr(), n, n, ipiv.data_ptr())
    cuda.cuda.synchronize()
    assert info == 0
    lu = at.cpu().numpy().T
    piv = ipiv.cpu().numpy() - 1
    perm = np.arange(n)
    for i, p in enumerate(piv):
        perm[[i, p]] = perm[[p, i]]
    x = (rng.normal(size=(n, 4)) + 1j * rng.normal(size=(n, 4))).astype(np.complex128)
    ux = np.triu(lu).astype(np.complex128) @ x
    lux = np.tril(lu, -1).astype(np.complex128) @ ux + ux
    pax = a.astype(np.complex128)[perm] @ x
    err = np.linalg.norm(pax - lux) / (np.linalg.norm(a.astype(np.complex128)) * np.linalg.norm(x) / np.sqrt(n))
    assert err <= 3e-4, err
    assert np.max(np.abs(np.tril(lu, -1))) <= np.sqrt(2.0) * (1 + 1e-5)


@pytest.mark.parametrize("n", [300, 4100, 9000])
def test_panel_lookahead_is_bit_identical(cuda, wmom, n):
    """The cluster panel with the one-column look-ahead publishes rows one update
    behind and each reader applies that update itself with the owner's arithmetic:
    its factors and pivots must equal the plain cluster panel's bit for bit (one
    cluster, 16-CTA clusters with 48-column panels, two rows per thread)."""
    import os
    rng = np.random.default_rng(77 + n)
    a = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
    out = {}
    for la in ("1", "0"):
        os.environ["WMOM_PANEL_LOOKAHEAD"] = la
        try:
            at = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
            ipiv = cuda.zeros(n, dtype=cuda.int32, device="cuda")
            assert wmom.cgetrf_device(at.data_ptr(), n, n, ipiv.data_ptr()) == 0
            cuda.cuda.synchronize()
            out[la] = (at.cpu().numpy(), ipiv.cpu().numpy())
        finally:
            del os.environ["WMOM_PANEL_LOOKAHEAD"]
    assert np.array_equal(out["1"][1], out["0"][1])
    assert np.array_equal(out["1"][0], out["0"][0])
