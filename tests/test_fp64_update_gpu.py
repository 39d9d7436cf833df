"""The plain FP64 form's trailing update in its two forms: SIMT DFMA (the default)
and DMMA on the FP64 tensor pipe (mma.m8n8k4.f64, WMOM_FP64_UPDATE=dmma).  Both
must compute C - A B to FP64 accuracy on shapes that are not multiples of the tiles,
and the plain FP64 LU with the DMMA update must still meet the oracle at 1e-10."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def _fn(wmom):
    f = wmom._lib.wmom_zgemm_sub_fp64
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_longlong] * 3 + [ctypes.c_int, ctypes.c_void_p]
    return f


@pytest.mark.parametrize("variant", [0, 1], ids=["simt", "dmma"])
@pytest.mark.parametrize("m,n,k", [(64, 64, 8), (200, 130, 37), (1000, 900, 64), (77, 301, 3)])
def test_fp64_update_matches_numpy(cuda, wmom, variant, m, n, k):
    rng = np.random.default_rng(m * 7 + n + k)
    c = lambda *s: rng.normal(size=s) + 1j * rng.normal(size=s)
    a, b, cc = c(m, k), c(k, n), c(m, n)
    da = cuda.from_numpy(np.ascontiguousarray(a.T)).to("cuda")   # column-major storage
    db = cuda.from_numpy(np.ascontiguousarray(b.T)).to("cuda")
    dc = cuda.from_numpy(np.ascontiguousarray(cc.T)).to("cuda")
    st = _fn(wmom)(m, n, k, da.data_ptr(), m, db.data_ptr(), k, dc.data_ptr(), m, variant, None)
    assert st == 0
    got = dc.cpu().numpy().T
    ref = cc - a @ b
    bound = 1e-15 * k * np.max(np.abs(a)) * np.max(np.abs(b)) * 8
    assert np.max(np.abs(got - ref)) <= bound


def test_plain_lu_with_dmma_update_meets_oracle(cuda):
    """In a fresh process with WMOM_FP64_UPDATE=dmma (read once per process)."""
    code = r"""
import importlib, os, sys, numpy as np
sys.path.insert(0, %r)
w = importlib.import_module("praca-magisterska_gb300")
from oracle import build as ob; ob.build_port()
from oracle import oracle as orc
topo = w.Topology(w.geometry.precision_grid(2048))
plan = w.Plan(topo)
cur, zin, rep = plan.solve(np.array([10.0], np.float32), 1000, mode=w.MODE_FP64)
d = np.load(os.path.join(%r, "tests", "golden", "currents_grid21_2048.npz"))
k = list(d["freqs"]).index(np.float32(10.0))
ref = d["currents"][k]
err = np.linalg.norm(cur[0] - ref) / np.linalg.norm(ref)
print("ERR", err)
assert err < 1e-10, err
""" % (ROOT, ROOT)
    env = dict(os.environ, WMOM_FP64_UPDATE="dmma")
    p = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
