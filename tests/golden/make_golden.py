"""Generates the golden fixtures in tests/golden/ from the reference itself.

Run in a checkout that has the reference sources (the oracle's reference build,
oracle/_ref/libwmomref.so, compiled by oracle/build.py from the reference's own
Configuration.cpp / Zmatrix.cpp / Complex.cpp):

    python tests/golden/make_golden.py --reference-dir DIR

Writes:
  zin_logs.json     every "Freq = f <re> <im>" line of the reference's run logs
                    (results_P_F_N.txt of all four program variants), with N = nsw
                    taken from the file name; 25 m dipole, radius 0.5 mm, gap 100.
  topology_*.npz    configwire() output arrays of the reference for several
                    geometries (meaningful ranges only) and its configwire.txt text.
  zfill_*.npz       the reference's zmatrix() output for small cases.
  currents_*.npz    currents and input impedance from the reference's fill and the
                    MKL zgetrf/zgetrs that the reference linked (reached through
                    torch's CPU LAPACK, MKL 2024.2 in the generating container).
The fixtures are what the GPU machine checks against; it has no reference checkout.
"""
import argparse
import glob
import importlib
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

LINE = re.compile(r"Freq = ([\d.]+)\t([-\d.e+]+)\t([-\d.e+]+)")


def parse_logs(refroot):
    out = []
    for path in sorted(glob.glob(os.path.join(refroot, "*", "results_*_*_*.txt"))):
        m = re.search(r"results_(\d+)_(\d+)_(\d+)\.txt$", path)
        if not m:
            continue
        nsw = int(m.group(3))
        variant = os.path.basename(os.path.dirname(path))
        with open(path, encoding="latin-1") as f:
            for line in f:
                mm = LINE.search(line)
                if mm:
                    out.append(dict(variant=variant, file=os.path.basename(path), nsw=nsw,
                                    freq=float(mm.group(1)), re=float(mm.group(2)), im=float(mm.group(3)),
                                    re_text=mm.group(2), im_text=mm.group(3)))
    return out


def trimmed_topology(r):
    nsmax, ns, npl, npnt = r["nsmax"], r["nseg"], r["npls"], r["npnt"]
    return dict(nsmax=nsmax, nseg=ns, npls=npl, npnt=npnt, x=r["x"][:npnt], y=r["y"][:npnt], z=r["z"][:npnt],
                rad=r["rad"][:ns], ipc=r["ipc"][:npl], ips1=r["ips"][:npl], ips2=r["ips"][nsmax:nsmax + npl],
                ise1=r["ise"][:ns], ise2=r["ise"][nsmax:nsmax + ns], isp1=r["isp"][:ns],
                isp2=r["isp"][nsmax:nsmax + ns], listing=np.array(r["listing"]))


def mkl_solve(z, v):
    import torch
    zt = torch.from_numpy(np.ascontiguousarray(z))  # the same matrix, row-major storage
    lu, piv = torch.linalg.lu_factor(zt)
    x = torch.linalg.lu_solve(lu, piv, torch.from_numpy(v.reshape(-1, 1)))
    return x.numpy().ravel()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-dir", required=True,
                    help="root of the reference checkout (the directory holding 'wersja referencyjna')")
    ap.add_argument("--only", nargs="*", default=None,
                    help="write only the fixtures of these case names (default: all)")
    args = ap.parse_args()
    want = (lambda name: True) if not args.only else (lambda name: name in args.only)
    os.environ["WMOM_REFERENCE_DIR"] = os.path.join(args.reference_dir, "wersja referencyjna")
    from oracle import build as ob
    ob.REF_DIR = os.environ["WMOM_REFERENCE_DIR"]
    ob.build_port()
    if not ob.build_ref():
        raise SystemExit("reference sources not found")
    from oracle import oracle as orc
    geo = importlib.import_module("praca-magisterska_gb300.geometry")

    if want("zin_logs"):
        logs = parse_logs(args.reference_dir)
        with open(os.path.join(HERE, "zin_logs.json"), "w") as f:
            json.dump(logs, f, indent=0)
        print("log lines", len(logs))

    cases = {
        "dipole1m_512": (geo.dipole(1.0, 1e-3, 512), 1),
        "dipole25m_512": (geo.dipole(25.0, 5e-4, 512), 1),
        "grid5_ns3": (geo.grid(5, 1.0, 1.0, 5e-3, None, 3), 1),
        "grid21_2048": (geo.precision_grid(2048), 1),
        "random_1024": (geo.random_wires(1024, seed=20261203), 1),
        "bent_ground": (geo.geo_text([(0, 0, 0), (0, 0, 1.0), (1.0, 0, 1.0)],
                                     [(1, 2, 1e-3, 20), (2, 3, 1e-3, 20)]), 2),
        "mixed_junctions": (geo.geo_text([(0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1), (0.5, 0.5, 2)],
                                         [(1, 2, 2e-3, 4), (2, 3, 2e-3, 3), (4, 3, 2e-3, 4), (1, 4, 2e-3, 2),
                                          (5, 1, 1e-3, 5), (3, 5, 1e-3, 1), (2, 4, 1e-3, 6)]), 1),
        # PEC ground (ienv = 2): a monopole standing on the ground, a frame whose two
        # legs stand on it, and a grid held 0.5 m above it (no wire touching it)
        "ground_monopole": (geo.geo_text([(0, 0, 0), (0, 0, 1.0)], [(1, 2, 1e-3, 40)]), 2),
        "ground_frame": (geo.geo_text([(0, 0, 0), (0, 0, 0.5), (1.5, 0, 0.5), (1.5, 0, 0)],
                                      [(1, 2, 1e-3, 10), (2, 3, 1e-3, 30), (3, 4, 1e-3, 10)]), 2),
        "ground_grid": (geo.grid(4, 1.0, 0.5, 5e-3, None, 4), 2),
    }
    topos = {}
    for name, (text, ienv) in cases.items():
        r = orc.ref_geometry(text, ienv=ienv)
        topos[name] = r
        if not want(name):
            continue
        np.savez_compressed(os.path.join(HERE, f"topology_{name}.npz"), geo=np.array(text), ienv=ienv,
                            **trimmed_topology(r))
        print("topology", name, r["npls"])

    sg = {1: (1.0, 1.0, 1.0, 1.0), 2: (1.0, 1.0, -1.0, -1.0)}
    small = [("dipole64", geo.dipole(1.0, 1e-3, 64), 1, 150.0), ("grid5_ns3", cases["grid5_ns3"][0], 1, 30.0),
             ("bent_ground", cases["bent_ground"][0], 2, 100.0),
             ("mixed_junctions", cases["mixed_junctions"][0], 1, 60.0),
             ("dipole25m_lowf", geo.dipole(25.0, 5e-4, 96), 1, 0.01),
             ("ground_monopole", cases["ground_monopole"][0], 2, 75.0),
             ("ground_frame", cases["ground_frame"][0], 2, 40.0),
             ("ground_grid", cases["ground_grid"][0], 2, 20.0)]
    for name, text, ienv, f in small:
        if not want(name):
            continue
        r = orc.ref_geometry(text, ienv=ienv)
        z = orc.ref_fill(r, f, ienv=ienv, sgn=sg[ienv])
        np.savez_compressed(os.path.join(HERE, f"zfill_{name}.npz"), geo=np.array(text), ienv=ienv,
                            freq=np.float32(f), z=z)
        print("zfill", name, z.shape)

    cur_cases = [("dipole1m_512", [150.0], 256), ("dipole25m_512", [100., 200., 300., 400., 500., 600.], 100),
                 ("grid21_2048", [0.01, 1.0, 10.0], 1000), ("random_1024", list(geo.sweep_freqs()), 500),
                 ("mixed_junctions", [30.0, 60.0], 3),
                 ("ground_monopole", [37.5, 75.0, 150.0], 1), ("ground_frame", [20.0, 40.0, 80.0], 5),
                 ("ground_grid", [5.0, 20.0], 7)]
    for name, freqs, ngap in cur_cases:
        if not want(name):
            continue
        r = topos[name]
        ienv = cases[name][1]
        cur = []
        zin = []
        for f in freqs:
            z = orc.ref_fill(r, f, ienv=ienv, sgn=sg[ienv])
            v = orc.excitation(r["npls"], ngap)
            i = mkl_solve(z, v)
            cur.append(i)
            zin.append(v[ngap - 1] / i[ngap - 1])
        np.savez_compressed(os.path.join(HERE, f"currents_{name}.npz"), freqs=np.array(freqs, np.float32),
                            ngap=ngap, ienv=ienv, currents=np.array(cur), zin=np.array(zin),
                            lapack=np.array("MKL zgetrf/zgetrs via torch " + __import__("torch").__version__))
        print("currents", name, len(freqs))


if __name__ == "__main__":
    main()
