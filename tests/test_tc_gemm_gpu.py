"""The precision form's tensor-core trailing update (lu_tc.cu: tcgen05 kind::tf32,
3xTF32 split, complex embedded as real) against a complex128 reference of the
same operation.  The 3xTF32 product keeps close to FP32 accuracy: the error is
bounded by 4e-6 of |A| |B| per entry, written in the test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# shapes: one tile; ragged edges; a few tiles per CTA; K of one chunk; many tiles per
# CTA (both accumulators reused many times); long K (the stage ring wraps often)
@pytest.mark.parametrize("m,n,k", [(128, 64, 64), (130, 70, 64), (1000, 900, 64), (257, 33, 17), (64, 500, 5),
                                   (4096, 4096, 64), (300, 200, 300), (2000, 3000, 200)])
def test_cgemm_sub_tc_matches_complex128(cuda, wmom, m, n, k):
    rng = np.random.default_rng(m * 7 + n + k)
    a = (rng.normal(size=(m, k)) + 1j * rng.normal(size=(m, k))).astype(np.complex64)
    b = (rng.normal(size=(k, n)) + 1j * rng.normal(size=(k, n))).astype(np.complex64)
    c = (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))).astype(np.complex64)
    # column-major device copies (transposed C-order tensors)
    ad = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
    bd = cuda.from_numpy(np.ascontiguousarray(b.T)).to("cuda")
    cd = cuda.from_numpy(np.ascontiguousarray(c.T)).to("cuda")
    f = wmom._lib.wmom_cgemm_sub_tc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_longlong] * 3 + [ctypes.c_void_p]
    st = f(m, n, k, ad.data_ptr(), m, bd.data_ptr(), k, cd.data_ptr(), m, None)
    assert st == 0
    out = cd.cpu().numpy().T
    ref = c.astype(np.complex128) - a.astype(np.complex128) @ b.astype(np.complex128)
    bound = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64)
    err = np.abs(out - ref) / (bound + np.abs(c))
    assert np.max(err) < 4e-6, np.max(err)
