"""wmom_zgetrf_noalloc: the FP64 LU for callers that cannot call cudaMalloc (an
application that gives the library device buffers from its own pool and allows no
other device allocation, or a serving process that must not take cudaMalloc's
device-wide synchronisation once running).  Its scratch lives in a fixed __device__
array inside the library.  Called through the C ABI twice in a row, it must give
the same factors, pivots and info as wmom_zgetrf (the tolerance of the other LU
tests), allocate no device memory, and reject orders above WMOM_NOALLOC_MAX_N.
This file is collected last, and every test in it also passes alone in a fresh
process: the memory check brackets the no-alloc call only, after its operands are
on the device and the stream is idle."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 20480  # WMOM_NOALLOC_MAX_N in include/wmom.h


def _fn(wmom, name):
    f = getattr(wmom._lib, name)
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    return f


def _upload(cuda, a):
    """Column-major device copy of a and a device pivot array, both in place and the
    device idle before the call under test."""
    n = a.shape[0]
    at = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
    ipiv = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    cuda.cuda.synchronize()
    return at, ipiv


def _factor(cuda, f, a, check_no_alloc=False):
    n = a.shape[0]
    at, ipiv = _upload(cuda, a)
    info = ctypes.c_int(-1)
    if check_no_alloc:
        reserved = cuda.cuda.memory_reserved()
        free_before = cuda.cuda.mem_get_info()[0]
    st = f(n, at.data_ptr(), n, ipiv.data_ptr(), ctypes.byref(info), None)
    cuda.cuda.synchronize()
    if check_no_alloc:
        # nothing allocated on the device by the call: neither by the driver nor by
        # torch's caching allocator
        assert cuda.cuda.mem_get_info()[0] == free_before
        assert cuda.cuda.memory_reserved() == reserved
    return st, at.cpu().numpy().T, ipiv.cpu().numpy(), info.value


def test_noalloc_matches_zgetrf_on_two_calls_in_a_row(cuda, wmom):
    ref = _fn(wmom, "wmom_zgetrf")
    noalloc = _fn(wmom, "wmom_zgetrf_noalloc")
    rng = np.random.default_rng(4242)
    n = 1000
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    st_r, lu_r, piv_r, info_r = _factor(cuda, ref, a)
    assert st_r == 0 and info_r == 0
    # two calls in a row on fresh copies: the first loads the kernels it uses (module
    # loading may take device memory for code), the second must take none at all;
    # both must match wmom_zgetrf, so the array's contents left by the first call do
    # not leak into the second
    for call in range(2):
        st, lu, piv, info = _factor(cuda, noalloc, a, check_no_alloc=(call == 1))
        assert st == 0 and info == 0
        assert np.array_equal(piv, piv_r)
        assert np.max(np.abs(lu - lu_r)) <= 1e-11 * max(1.0, np.max(np.abs(lu_r)))


def test_noalloc_reports_zero_pivot_like_zgetrf(cuda, wmom):
    noalloc = _fn(wmom, "wmom_zgetrf_noalloc")
    a = np.eye(90, dtype=np.complex128)
    a[:, 70] = 0.0
    st, _, _, info = _factor(cuda, noalloc, a)
    assert st == 3 and info == 71


def test_noalloc_rejects_orders_above_its_maximum(cuda, wmom):
    noalloc = _fn(wmom, "wmom_zgetrf_noalloc")
    info = ctypes.c_int(0)
    # rejected on the host before any device work: the pointers are never touched
    st = noalloc(MAX_N + 1, ctypes.c_void_p(16), MAX_N + 1, ctypes.c_void_p(16), ctypes.byref(info), None)
    assert st == 1
