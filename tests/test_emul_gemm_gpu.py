"""The precision form's second-tier trailing update (lu_emul.cu: complex FP64 GEMM
from 8-bit digit planes on the bf16 tensor cores, tcgen05 kind::f16) against a
complex128 reference of the same operation.

* Operands whose entries have few significant bits are split without remainder and
  every kept digit product is summed exactly, so the result must equal the FP64
  reference bit for bit.
* Random operands with rows and columns of very different magnitude: the error of
  entry (m, n) is bounded by 2^-40 * k * max|A[m, :]| * max|B[:, n]| (written in
  the test; the method's own estimate is about 2^-45), far below the 3xTF32
  update's 4e-6.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _emul(wmom, cuda, a, b, c):
    m, k = a.shape
    n = b.shape[1]
    ad = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
    bd = cuda.from_numpy(np.ascontiguousarray(b.T)).to("cuda")
    cd = cuda.from_numpy(np.ascontiguousarray(c.T)).to("cuda")
    f = wmom._lib.wmom_zgemm_sub_emul
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_longlong] * 3 + [ctypes.c_void_p]
    st = f(m, n, k, ad.data_ptr(), m, bd.data_ptr(), k, cd.data_ptr(), m, None)
    assert st == 0
    return cd.cpu().numpy().T


@pytest.mark.parametrize("m,n,k", [(128, 64, 32), (300, 130, 96), (77, 500, 200)])
def test_emul_exact_on_short_operands(cuda, wmom, m, n, k):
    rng = np.random.default_rng(m + 3 * n + k)
    # integers below 2^7 times a power of two per row / column: two digits hold them
    a = (rng.integers(-127, 128, (m, k)) + 1j * rng.integers(-127, 128, (m, k))) * \
        np.exp2(rng.integers(-20, 20, (m, 1)))
    b = (rng.integers(-127, 128, (k, n)) + 1j * rng.integers(-127, 128, (k, n))) * \
        np.exp2(rng.integers(-20, 20, (1, n)))
    c = np.zeros((m, n), np.complex128)
    out = _emul(wmom, cuda, a, b, c)
    ref = -(a @ b)
    assert np.array_equal(out, ref)


# one tile; ragged edges; several tiles per CTA; K below one chunk; K split into
# launches of 96; a large square update
@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (130, 70, 64), (1000, 900, 64), (257, 33, 17), (64, 500, 5),
                                   (300, 200, 300), (1000, 3000, 96), (4096, 4096, 64)])
def test_emul_matches_complex128(cuda, wmom, m, n, k):
    rng = np.random.default_rng(m * 5 + n + 11 * k)
    rs = np.exp2(rng.uniform(-30, 30, (m, 1)))
    cs = np.exp2(rng.uniform(-30, 30, (1, n)))
    a = (rng.normal(size=(m, k)) + 1j * rng.normal(size=(m, k))) * rs
    b = (rng.normal(size=(k, n)) + 1j * rng.normal(size=(k, n))) * cs
    c = (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))) * rs * cs
    out = _emul(wmom, cuda, a, b, c)
    ref = c - a @ b
    amax = np.max(np.maximum(np.abs(a.real), np.abs(a.imag)), axis=1, keepdims=True)
    bmax = np.max(np.maximum(np.abs(b.real), np.abs(b.imag)), axis=0, keepdims=True)
    scale = k * amax * bmax
    err = np.abs(out - ref) / scale
    assert np.max(err) < 2.0 ** -40, np.max(err)


@pytest.mark.parametrize("tile", ["32", "64"])
def test_emul_tile_shapes(cuda, wmom, monkeypatch, tile):
    """Both tile shapes of the update (128 x 32 with one accumulator per level, the
    default; 128 x 64 with levels 3-5 sharing one) meet the same bound, on ragged
    edges and several tiles per CTA.  Each is within about 2^-45 of the scale of the
    exact product (dropped levels, digit remainder, FP32 rounding of levels 3-5), so
    the two agree to within twice that (measured 2^-44.1); the test allows 2^-43."""
    monkeypatch.setenv("WMOM_EMUL_TILE", tile)
    m, n, k = 700, 333, 96
    rng = np.random.default_rng(7)
    rs = np.exp2(rng.uniform(-20, 20, (m, 1)))
    cs = np.exp2(rng.uniform(-20, 20, (1, n)))
    a = (rng.normal(size=(m, k)) + 1j * rng.normal(size=(m, k))) * rs
    b = (rng.normal(size=(k, n)) + 1j * rng.normal(size=(k, n))) * cs
    c = (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))) * rs * cs
    out = _emul(wmom, cuda, a, b, c)
    ref = c - a @ b
    amax = np.max(np.maximum(np.abs(a.real), np.abs(a.imag)), axis=1, keepdims=True)
    bmax = np.max(np.maximum(np.abs(b.real), np.abs(b.imag)), axis=0, keepdims=True)
    scale = k * amax * bmax
    assert np.max(np.abs(out - ref) / scale) < 2.0 ** -40
    monkeypatch.setenv("WMOM_EMUL_TILE", "64" if tile == "32" else "32")
    other = _emul(wmom, cuda, a, b, c)
    assert np.max(np.abs(out - other) / scale) < 2.0 ** -43
