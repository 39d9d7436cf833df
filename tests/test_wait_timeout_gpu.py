"""A bounded device-side wait that runs out, on the GPU, without a fault.

The plain FP64 LU's cooperative panel kernel meets at a grid-wide counting barrier
once per column; every wait there gives up after 2 s, sets the workspace's error
word and returns.  The test hook wmom_debug_panel_missing_arrivals(1) makes every
barrier wait for one arrival more than the kernel's blocks send, so the first wait
runs out: wmom_zgetrf must return WMOM_ERR_TIMEOUT (4) and leave the context usable,
and the next factorisation with the hook off must succeed with LAPACK's pivots.
No kernel is made to fault, trap or hang: every wait is bounded and the kernel
returns.  (The reference has no device-side waits; it prints CUDA errors and goes
on, "wersja referencyjna/Wire_MoM.h":36-38.)
"""
import ctypes
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_panel_barrier_wait_runs_out_and_the_next_lu_succeeds(cuda, wmom):
    from scipy.linalg import lapack
    rng = np.random.default_rng(99)
    n = 700
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    f = wmom._lib.wmom_zgetrf
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]

    def factor():
        d = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")
        # pivots start out of range: the timed-out panel never writes its later ones
        piv = cuda.full((n,), -7, dtype=cuda.int32, device="cuda")
        info = ctypes.c_int(-1)
        cuda.cuda.synchronize()
        t0 = time.perf_counter()
        st = f(n, d.data_ptr(), n, piv.data_ptr(), ctypes.byref(info), None)
        cuda.cuda.synchronize()
        return st, time.perf_counter() - t0, d.cpu().numpy().T, piv.cpu().numpy(), info.value

    try:
        wmom.debug_panel_missing_arrivals(1)
        st, dt, _, _, _ = factor()
    finally:
        wmom.debug_panel_missing_arrivals(0)
    assert st == 4, wmom.STATUS_NAMES.get(st, st)
    assert 1.5 < dt < 60.0  # the 2 s limit of the first wait, then every block leaves
    # the context still works: a normal factorisation right after
    st, _, lu, piv, info = factor()
    assert st == 0 and info == 0
    lu_ref, piv_ref, _ = lapack.zgetrf(np.asfortranarray(a))
    assert np.array_equal(piv, piv_ref + 1)
    assert np.max(np.abs(lu - lu_ref)) <= 1e-10 * np.max(np.abs(lu_ref))
