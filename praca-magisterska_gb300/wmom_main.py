"""Command-line driver with the reference program's inputs and outputs.

The reference's main() ("wersja referencyjna/Wire_MoM.cu":28-412) reads dipol.geo and
freq.txt from the working directory, writes configwire.txt, and for every frequency
prints one line

    Process - 0 Freq = <f>\t<Re Z_in>\t<Im Z_in>

with 4 significant digits (a std::setprecision(4) that leaks from its Timer,
Wire_MoM.cu:24).  This driver does the same on the GPU, keeps the reference's
defaults (free space, delta-gap source at basis function 100, 1 V, 0 degrees, no
loads), and additionally writes the full-precision results the reference never
saved: zin.csv (frequency, Re, Im) and currents.csv (frequency, basis function,
Re, Im), all at 17 significant digits.

    python praca-magisterska_gb300/wmom_main.py [--dir D] [--geo dipol.geo] [--freq freq.txt]
        [--ngap 100] [--ampl 1] [--phase 0] [--ienv 1|2] [--mode fp64|mixed]
        [--load INDEX:R_OHM:L_UH ...] [--no-currents]
"""
import argparse
import importlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--dir", default=".")
    ap.add_argument("--geo", default="dipol.geo")
    ap.add_argument("--freq", default="freq.txt")
    ap.add_argument("--ngap", type=int, default=100)
    ap.add_argument("--ampl", type=float, default=1.0)
    ap.add_argument("--phase", type=float, default=0.0)
    ap.add_argument("--ienv", type=int, default=1, choices=[1, 2])
    ap.add_argument("--mode", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--load", action="append", default=[],
                    help="lumped series load INDEX:R_OHM:L_UH on basis function INDEX (1-based)")
    ap.add_argument("--no-currents", action="store_true")
    args = ap.parse_args(argv)
    w = importlib.import_module("praca-magisterska_gb300")
    d = args.dir
    with open(os.path.join(d, args.geo)) as f:
        geo = f.read()
    with open(os.path.join(d, args.freq)) as f:
        freqs = w.read_freq_file(f.read())
    print()
    print(" -------------------------")
    print(" Implementacja MoM w C++ (GB300)")
    print(" -------------------------")
    print(f" Nazwa pliku geo: {args.geo}")
    topo = w.Topology(geo, ienv=args.ienv)
    with open(os.path.join(d, "configwire.txt"), "w") as f:
        f.write(topo.listing)
    if not 0 < args.ngap <= topo.npls:
        print("    ERROR (wrong number of source zone)")
        return 1
    print(f" Source (source zone on wire): {args.ngap}")
    print(f"  Number of frequency points: {len(freqs)}")
    plan = w.Plan(topo)
    loads = []
    for spec in args.load:
        k, r, l = spec.split(":")
        loads.append((int(k), float(r), float(l)))
    if loads:
        plan.set_loads(loads)
    mode = w.MODE_FP64 if args.mode == "fp64" else w.MODE_MIXED
    cur, zin, rep = plan.solve(freqs, args.ngap, ampl=args.ampl, phas=args.phase, mode=mode,
                               currents=not args.no_currents)
    for f, z in zip(freqs, zin):
        print()
        print(f" Process - 0 Freq = {float(f):.4g}\t{z.real:.4g}\t{z.imag:.4g}")
    with open(os.path.join(d, "zin.csv"), "w") as f:
        f.write("freq_mhz,re,im,rel_residual,refinement_steps,fp64_fallback\n")
        for fr, z, r in zip(freqs, zin, rep):
            f.write(f"{float(fr):.9g},{z.real:.17g},{z.imag:.17g},{r['rel_residual']:.3e},"
                    f"{r['iterations']},{r['fell_back']}\n")
    if cur is not None:
        with open(os.path.join(d, "currents.csv"), "w") as f:
            f.write("freq_mhz,basis,re,im\n")
            for fr, row in zip(freqs, cur):
                for k, c in enumerate(row):
                    f.write(f"{float(fr):.9g},{k + 1},{c.real:.17g},{c.imag:.17g}\n")
    plan.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
