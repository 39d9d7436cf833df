"""The precision form's tensor-core update with FP16 operand planes
(WMOM_TC_PLANES=f16: each row of A' and column of B scaled by a power of two into
[2^14, 2^15), FP16 head and tail, tcgen05 kind::f16 with FP32 accumulation), run in a
fresh process since the switch is read once:
* the update against a complex128 reference at the 3xTF32 test's bound (4e-6 of
  |A| |B| per entry), also on operands whose rows and columns span 1e-6 .. 1e6;
* the FP32 LU (wmom_cgetrf) with that update: ||PA - LU|| / ||A|| <= 3e-5;
* the precision form's currents against the MKL fixtures at 1e-9, or 8 kappa_1 eps
  where the conditioning sets a larger floor (the junction grid at 10 kHz).
"""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import ctypes, importlib, json, os, sys
import numpy as np, torch
sys.path.insert(0, ROOT)
w = importlib.import_module("praca-magisterska_gb300")
out = {}
f = w._lib.wmom_cgemm_sub_tc
f.restype = ctypes.c_int
f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_longlong] * 3 + [ctypes.c_void_p]
worst = 0.0
for (m, n, k, scaled) in [(128, 64, 64, 0), (130, 70, 64, 0), (1000, 900, 64, 0), (257, 33, 17, 0),
                          (64, 500, 5, 0), (4096, 4096, 64, 0), (300, 200, 300, 0), (2000, 3000, 200, 0),
                          (700, 600, 96, 1)]:
    rng = np.random.default_rng(m * 7 + n + k)
    a = rng.normal(size=(m, k)) + 1j * rng.normal(size=(m, k))
    b = rng.normal(size=(k, n)) + 1j * rng.normal(size=(k, n))
    if scaled:  # rows of A and columns of B over twelve orders of magnitude
        a *= 10.0 ** rng.uniform(-6, 6, size=(m, 1))
        b *= 10.0 ** rng.uniform(-6, 6, size=(1, n))
    a, b = a.astype(np.complex64), b.astype(np.complex64)
    c = (rng.normal(size=(m, n)) + 1j * rng.normal(size=(m, n))).astype(np.complex64)
    ad = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    bd = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    cd = torch.from_numpy(np.ascontiguousarray(c.T)).cuda()
    assert f(m, n, k, ad.data_ptr(), m, bd.data_ptr(), k, cd.data_ptr(), m, None) == 0
    res = cd.cpu().numpy().T
    ref = c.astype(np.complex128) - a.astype(np.complex128) @ b.astype(np.complex128)
    bound = np.abs(a).astype(np.float64) @ np.abs(b).astype(np.float64)
    worst = max(worst, float(np.max(np.abs(res - ref) / (bound + np.abs(c)))))
out["gemm_worst"] = worst
# FP32 LU with the FP16-plane update
n = 1500
rng = np.random.default_rng(3)
a = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
d = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
piv = torch.zeros(n, dtype=torch.int32, device="cuda")
assert w.cgetrf_device(d.data_ptr(), n, n, piv.data_ptr()) == 0
lu = d.cpu().numpy().T.astype(np.complex128)
p = piv.cpu().numpy() - 1
L = np.tril(lu, -1) + np.eye(n)
U = np.triu(lu)
pa = a.astype(np.complex128).copy()
for i in range(n):
    if p[i] != i:
        pa[[i, p[i]]] = pa[[p[i], i]]
out["lu_backward"] = float(np.linalg.norm(pa - L @ U) / np.linalg.norm(a))
# the precision form against the MKL fixtures
errs = []
for name in ("grid21_2048", "random_1024", "dipole25m_512"):
    d = np.load(os.path.join(ROOT, "tests", "golden", f"currents_{name}.npz"))
    g = {"grid21_2048": lambda: w.geometry.precision_grid(2048),
         "random_1024": lambda: w.geometry.random_wires(1024, seed=20261203),
         "dipole25m_512": lambda: w.geometry.dipole(25.0, 5e-4, 512)}[name]()
    plan = w.Plan(w.Topology(g, listing=False))
    cur, zin, rep = plan.solve(d["freqs"], int(d["ngap"]), mode=w.MODE_MIXED, tol=1e-12, condest=True)
    for i in range(len(d["freqs"])):
        ref = d["currents"][i]
        errs.append((name, float(d["freqs"][i]), float(np.linalg.norm(cur[i] - ref) / np.linalg.norm(ref)),
                     int(rep[i]["tier"]), float(rep[i]["cond1"])))
    plan.close()
out["currents"] = errs
print("RESULT", json.dumps(out))
"""


def test_f16_planes(cuda):
    env = dict(os.environ, WMOM_TC_PLANES="f16")
    p = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + SCRIPT], env=env, capture_output=True,
                       text=True, timeout=900)
    assert p.returncode == 0, p.stdout[-3000:] + p.stderr[-3000:]
    res = json.loads([l for l in p.stdout.splitlines() if l.startswith("RESULT ")][-1][7:])
    assert res["gemm_worst"] < 4e-6, res["gemm_worst"]
    assert res["lu_backward"] <= 3e-5, res["lu_backward"]
    for name, f, err, tier, kappa in res["currents"]:
        assert err <= max(1e-9, 8 * kappa * 2.0 ** -53), (name, f, err, tier, kappa)
