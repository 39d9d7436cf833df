"""Generates the large parity fixtures in tests/golden/ from the reference itself:
the benchmark configurations' systems at their full sizes, filled by the reference's
own zmatrix() (compiled unmodified into oracle/_ref by oracle/build.py) and solved by
MKL zgetrf/zgetrs (the LAPACK the reference linked, reached through torch's MKL).

Run in a checkout that has the reference sources:

    WMOM_REFERENCE_DIR=<checkout>/"wersja referencyjna" python tests/golden/make_golden_large.py

For every (workload, frequency) it stores, in large_<workload>.npz:
  currents_mkl  the reference's currents: its fill + MKL zgetrf/zgetrs
  truth         the exact solution of the reference's FP64 matrix to about 2^-106,
                by iterative refinement with double-double residuals
                (oracle.refine_truth, the MKL factors as the preconditioner)
  kappa1        kappa_1 of the reference's matrix: ||Z||_1 times LAPACK zgecon's
                estimate from MKL's factors
  mkl_vs_truth  ||currents_mkl - truth|| / ||truth||
  zin_mkl       V[ngap-1] / I[ngap-1] of currents_mkl
and the geometry's .geo text digest, so a test can confirm it rebuilt the same input.
The matrices themselves (1 to 3.3 GB each) are not stored; the GPU tests refill them.
"""
import hashlib
import importlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SEED = 20261203


def cases(geo):
    return [
        ("precision_8192", geo.precision_grid(8192), [0.01, 10.0]),
        ("random_8192", geo.random_wires(8192, seed=SEED), [0.01, 10.0]),
        ("random_4096", geo.random_wires(4096, seed=SEED), [0.01, 10.0]),
        ("random_14336", geo.random_wires(14336, seed=SEED), [10.0]),
    ]


def mkl_factor_solve(z, v):
    """MKL zgetrf + zgetrs (torch's MKL) of the logical matrix z; returns the
    currents and the factors in LAPACK's column-major layout with 0-based pivots."""
    import torch
    zt = torch.from_numpy(np.ascontiguousarray(z))
    lu, piv = torch.linalg.lu_factor(zt)
    x = torch.linalg.lu_solve(lu, piv, torch.from_numpy(v.reshape(-1, 1))).numpy().ravel()
    return x, (np.asfortranarray(lu.numpy()), piv.numpy().astype(np.int32) - 1)


def main():
    from oracle import build as ob
    ob.build_port()
    if not ob.build_ref():
        raise SystemExit("the reference's own build (oracle/_ref) is needed: set WMOM_REFERENCE_DIR")
    from oracle import oracle as orc
    from scipy.linalg import lapack
    import torch
    geo = importlib.import_module("praca-magisterska_gb300.geometry")
    threads = os.cpu_count() or 1
    only = sys.argv[1:]
    for name, text, freqs in cases(geo):
        if only and name not in only:
            continue
        r = orc.ref_geometry(text)
        n = r["npls"]
        ngap = n // 2
        out = {k: [] for k in ("currents_mkl", "truth", "kappa1", "anorm", "mkl_vs_truth", "zin_mkl",
                               "truth_steps")}
        for f in freqs:
            t0 = time.time()
            z = orc.ref_fill(r, f)
            t1 = time.time()
            v = orc.excitation(n, ngap)
            x, (lu, piv) = mkl_factor_solve(z, v)
            t2 = time.time()
            anorm = float(np.max(np.sum(np.abs(z), axis=0)))
            rcond, _ = lapack.zgecon(lu, anorm, norm="1")
            truth, hist = orc.refine_truth(z, v, x, factors=(lu, piv), threads=threads)
            t3 = time.time()
            err = float(np.linalg.norm(x - truth) / np.linalg.norm(truth))
            out["currents_mkl"].append(x)
            out["truth"].append(truth)
            out["kappa1"].append(1.0 / rcond)
            out["anorm"].append(anorm)
            out["mkl_vs_truth"].append(err)
            out["zin_mkl"].append(v[ngap - 1] / x[ngap - 1])
            out["truth_steps"].append(len(hist))
            print(f"{name} f={f} N={n}: fill {t1 - t0:.0f} s, MKL {t2 - t1:.1f} s, truth {t3 - t2:.1f} s "
                  f"({len(hist)} steps), kappa1 {1.0 / rcond:.3g}, MKL vs truth {err:.3g}", flush=True)
            del z, lu
        np.savez_compressed(os.path.join(HERE, f"large_{name}.npz"), freqs=np.array(freqs, np.float32), ngap=ngap,
                            npls=n, geo_sha256=np.array(hashlib.sha256(text.encode()).hexdigest()),
                            lapack=np.array("MKL zgetrf/zgetrs via torch " + torch.__version__),
                            **{k: np.array(v) for k, v in out.items()})


if __name__ == "__main__":
    main()
