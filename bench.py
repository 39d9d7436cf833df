#!/usr/bin/env python
"""Frequency-solves/s of the thin-wire MoM fill-and-solve path on GB300.

Workload (one "step"): the plain-FP64-sweep configuration at N = 8192 unknowns -- a
seeded random straight-wire structure (wires 0.5-5 m, radius 1-10 mm, endpoints in a
20 m cube, segments <= lambda/10 at 10 MHz) -- with its 12 frequencies log-spaced
10 kHz - 10 MHz: for every frequency the Z fill, the LU, the solve and Z_in.  Every
step solves all 12 (geometry, frequency) systems with the precision form (FP64 fill,
complex-FP32 tensor-core LU, FP64 iterative refinement to a relative residual of
1e-12; where that refinement stalls, an FP64 LU whose trailing updates run on the
bf16 tensor cores from digit planes, refined in FP64, and the plain FP64 LU last).
The plain FP64 form is timed on the same workload beside it (2 of the 12
frequencies) and both answers are compared.

    value  device throughput: geometry resident on the GPU before the timed region
    e2e    through the C ABI with host buffers: geometry tables uploaded (plan
           creation) and currents copied back inside the timed region

--impl reference times the reference's CPU path (its fill restated in C, threaded
over rows, plus LAPACK zgetrf/zgetrs) on the host cores instead, one frequency of the
same workload per step.

Multi-GPU: frequencies are independent, so N GPUs run N replicas of the step (weak
scaling, no collective in the data path); value = all ranks' solves / max time.
"""
import argparse
import importlib
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PKG = "praca-magisterska_gb300"
N_DEFAULT = 8192
SEED = 20261203
METRIC = "freq-solves/s and p50/p99 latency: mixed+refine vs FP64 LU at rel err <=1e-10"
UNIT = "freq-solves/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.path = tempfile.mktemp(prefix="wmom_clocks_", suffix=".csv")
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.f.close()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx = float(p[2])
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        except OSError:
            pass
        os.unlink(self.path) if os.path.exists(self.path) else None
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


WORKLOADS = {
    "sweep": "random-wire sweep, N={n}, {nf} frequencies 10 kHz-10 MHz",
    "precision": "20x20 m wire grid (1 m pitch, a = 5 mm), N={n}, {nf} frequencies 10 kHz-10 MHz",
    "batching": "20x20 m wire grid, N={n}, {nf} frequencies 1 kHz-30 MHz",
}


def _geometry():
    """The workload generators: seeded numpy draws written as .geo text (the
    reference's input format).  Loaded from their file on their own, so that the CPU
    reference arm reads the same inputs without importing the product package."""
    spec = importlib.util.spec_from_file_location("wmom_workload_geometry", os.path.join(ROOT, PKG, "geometry.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workload(n, kind="sweep", nfreq=None):
    """(.geo text, float32 MHz frequencies, gap index) of a workload."""
    import numpy as np
    g = _geometry()
    if kind == "sweep":
        geo, freqs = g.random_wires(n, seed=SEED), g.sweep_freqs()
    elif kind == "precision":
        geo, freqs = g.precision_grid(n), g.sweep_freqs()
    elif kind == "batching":
        geo, freqs = g.precision_grid(n), g.log_freqs(0.001, 30.0, 256)
    else:
        raise ValueError(kind)
    if nfreq and nfreq < len(freqs):
        # evenly spaced subset of the sweep (small cases for the profiler)
        freqs = freqs[np.unique(np.linspace(0, len(freqs) - 1, nfreq).round().astype(int))]
    return geo, freqs, n // 2


def config_dict(kind, n, nf, ngap):
    """The `config` object of both arms' lines: the same workload, the same keys."""
    return {"workload": WORKLOADS[kind].format(n=n, nf=nf), "unknowns": n, "frequencies": nf, "seed": SEED,
            "ngap": ngap, "refine_tol": 1e-12,
            "l2": "inputs larger than L2 (each Z is %.2f GB)" % (16 * n * n / 1e9)}


def oracle_topology(geo):
    """Topology arrays of the CPU reference path (the oracle's restatement of the
    reference's geoinp + configwire; no product library involved)."""
    from oracle import build as ob
    ob.build_port()
    from oracle import oracle as orc
    return orc.topology(geo)


def cpu_solve_once(topo, freq, ngap, threads):
    """One frequency of the reference's CPU path: oracle fill + LAPACK zgetrf/zgetrs."""
    from oracle import oracle as orc
    t0 = time.perf_counter()
    i, zin, _ = orc.solve(topo, float(freq), ngap, threads=threads)
    return time.perf_counter() - t0, i, zin


def run_reference(args):
    """The reference's CPU path (oracle port: fill threaded over rows + LAPACK), built
    from the oracle alone: this arm never loads the product library."""
    ws, rank, _ = _dist()
    if rank != 0:
        return
    geo, freqs, ngap = workload(args.n, args.workload, args.nfreq)
    topo = oracle_topology(geo)
    threads = os.cpu_count() or 1
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(threads))
    k = 0
    for _ in range(args.warmup):
        cpu_solve_once(topo, freqs[k % len(freqs)], ngap, threads)
        k += 1
    t = 0.0
    for _ in range(args.steps):
        dt, _, _ = cpu_solve_once(topo, freqs[k % len(freqs)], ngap, threads)
        t += dt
        k += 1
    value = args.steps / t
    n = topo["npls"]
    sample = (f"one frequency per step of the {len(freqs)}-frequency sweep (cycling), full N={n} "
              "fill + zgetrf + zgetrs")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "form": "FP64: oracle fill (reference zmatrix restated in C) + LAPACK zgetrf/zgetrs",
            "config": config_dict(args.workload, n, len(freqs), ngap),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _fixture(kind, n):
    """Full-size reference results of a workload (tests/golden/large_<kind>_<n>.npz:
    the reference's own fill + MKL currents, the extended-precision truth and
    kappa_1), or None."""
    import numpy as np
    name = {"sweep": "random", "precision": "precision"}.get(kind)
    p = os.path.join(ROOT, "tests", "golden", f"large_{name}_{n}.npz")
    return dict(np.load(p)) if name and os.path.exists(p) else None


def _rel(a, b):
    import numpy as np
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def accuracy_vs_reference(freqs, cur_mixed, cur_fp64_by_freq, reports, fx):
    """Per fixture frequency: both forms against the reference's fill + MKL currents
    and against the truth of the reference's FP64 system, with kappa_1 (LAPACK's on
    the reference's matrix and the device's estimate)."""
    import numpy as np
    out = {}
    if fx is None:
        return out
    for k, f in enumerate(fx["freqs"]):
        i = int(np.argmin(np.abs(freqs - f)))
        if abs(float(freqs[i]) - float(f)) > 1e-6 * float(f):
            continue
        mkl, truth = fx["currents_mkl"][k], fx["truth"][k]
        e = {"kappa1_lapack": float(fx["kappa1"][k]), "kappa1_device": reports[i].get("cond1"),
             "tier": reports[i].get("tier"), "refinement_steps": reports[i]["iterations"],
             "mixed_vs_mkl": _rel(cur_mixed[i], mkl), "mixed_vs_truth": _rel(cur_mixed[i], truth),
             "mkl_vs_truth": float(fx["mkl_vs_truth"][k])}
        c64 = cur_fp64_by_freq.get(float(f))
        if c64 is not None:
            e["fp64_vs_mkl"] = _rel(c64, mkl)
            e["fp64_vs_truth"] = _rel(c64, truth)
        out["%.6g MHz" % float(f)] = e
    return out


def time_sweep(w, plan, freqs, ngap, steps, warmup, mode, currents=False):
    """Device-timed sweeps (CUDA events on the current stream around `steps` calls
    after `warmup` untimed ones); returns (ms per step, reports of the last, host
    latencies of each call)."""
    import torch
    for _ in range(warmup):
        plan.solve(freqs, ngap, mode=mode, currents=False)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    lat, rep = [], None
    e0.record()
    for _ in range(steps):
        t0 = time.perf_counter()
        _, _, rep = plan.solve(freqs, ngap, mode=mode, currents=currents)
        lat.append(1e3 * (time.perf_counter() - t0))
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, rep, lat


def e2e_sweep(w, topo, freqs, ngap, steps):
    """End to end through the C ABI: a new plan (geometry tables uploaded), the sweep,
    currents to the host, per step.  Returns (freq-solves/s, h2d, d2h bytes per step,
    currents, reports of the last step)."""
    import torch
    n, nf = topo.npls, len(freqs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        p2 = w.Plan(topo)
        cur, _, rep = p2.solve(freqs, ngap, mode=w.MODE_MIXED, currents=True)
        up = p2.upload_bytes
        p2.close()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    iters = sum(r["iterations"] for r in rep)
    h2d = up + 4 * nf + 3 * 8 * nf + 16 * n          # tables, frequencies, k params, excitation
    d2h = 16 * n * nf + 32 * (iters + nf) + 16 * nf  # currents, residual norms, factor status
    return nf * steps / dt, h2d, d2h, cur, rep


def fp64_leg(w, plan, freqs, ngap):
    """The plain FP64 form on the lowest and highest frequency, warmed up once (batch
    width tuned), then timed once; returns (freq-solves/s, {freq: currents}, reports)."""
    import numpy as np
    import torch
    fsub = np.array([freqs[0], freqs[-1]], np.float32)
    plan.solve(fsub, ngap, mode=w.MODE_FP64, currents=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cur64, _, rep64 = plan.solve(fsub, ngap, mode=w.MODE_FP64, currents=True)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    return len(fsub) / dt, {float(f): cur64[j] for j, f in enumerate(fsub)}, rep64


def tier_counts(reports):
    return {str(t): sum(1 for r in reports if r.get("tier") == t) for t in (1, 2, 3)}


def fill_roofline(plan, nf, avg_ms, entries, fp64_peak, peaks, cap):
    """The fill kernel against the FP64 pipe: achieved = the FP64 flops the kernel
    executes (2 DFMA + DADD + DMUL thread instructions per launch, counted by ncu on a
    smaller case and scaled by this launch's (observation, source) pairs) / launch
    time; peak = the FMA-chain probe of this device."""
    pairs = plan.fill_pairs / float(plan.npls) ** 2
    flops_per_pair_freq = cap["fp64_flops"] / (cap["units"] * cap["pairs_per_entry"])
    flops = flops_per_pair_freq * pairs * entries
    achieved = flops / (avg_ms / 1e3) / 1e12
    alg = 16.0 * entries  # each complex128 entry written once
    return {"kernel": "fill_pair_multi_kernel" if plan.multi_frequency_fill and nf > 1 else "fill_pair_kernel",
            "bound": "fp64", "unit": "TFLOP/s", "achieved": achieved, "peak": fp64_peak,
            "frac": achieved / fp64_peak,
            "peak_source": "measured: FP64 FMA-chain probe on this device in this run (wmom_probe_fp64_tflops, "
                           "2 flop per DFMA); MEASURED_PEAKS.json has no FP64 figure",
            "work": "executed FP64 flops: %.1f per (pair, frequency) x %.4f pairs per entry x %d entries (2 DFMA "
                    "+ DADD + DMUL thread instructions from the ncu capture of profiles/dram_traffic.json)"
                    % (flops_per_pair_freq, pairs, entries),
            "fp64_pipe_busy_ncu": cap.get("fp64_pipe_busy"),
            "hbm_view": {"algorithmic_bytes": alg, "achieved_gbs": alg / (avg_ms / 1e3) / 1e9,
                         "frac_of_hbm": alg / (avg_ms / 1e3) / 1e9 / peaks["hbm_gbs"]}}


def precision_leg(w, args):
    """The precision configuration (20 x 20 m junction grid, N = 8192, 12 frequencies
    10 kHz - 10 MHz): device value, e2e, the FP64 form's rate, tiers, and per
    frequency kappa_1 (device estimate) plus, at the fixture frequencies, the errors
    against the reference's fill + MKL and against the truth."""
    import numpy as np
    n = 8192
    geo, freqs, ngap = workload(n, "precision")
    topo = w.Topology(geo, listing=False)
    plan = w.Plan(topo)
    steps = max(1, min(args.steps, 3))
    ms, rep, _ = time_sweep(w, plan, freqs, ngap, steps, 2, w.MODE_MIXED)
    value = len(freqs) / (ms / 1e3)
    e2e_value, h2d, d2h, _, _ = e2e_sweep(w, topo, freqs, ngap, 1)
    cur, _, repc = plan.solve(freqs, ngap, mode=w.MODE_MIXED, currents=True, condest=True)
    fp64_value, cur64, _ = fp64_leg(w, plan, freqs, ngap)
    plan.close()
    per_f = [{"freq_mhz": float(f), "kappa1_device": r["cond1"], "tier": r["tier"],
              "refinement_steps": r["iterations"], "rel_residual": r["rel_residual"]}
             for f, r in zip(freqs, repc)]
    if args.oracle_all_freqs:
        # every frequency against the CPU oracle (the reference's fill restated in C +
        # LAPACK) and against the truth of the oracle's FP64 system
        from oracle import oracle as orc
        topo_o = oracle_topology(geo)
        threads = os.cpu_count() or 1
        v = orc.excitation(n, ngap)
        for k, f in enumerate(freqs):
            z = orc.fill(topo_o, float(f), threads=threads)
            i_o, _, fac = orc.lu_solve(z, v, return_factors=True)
            truth, _ = orc.refine_truth(z, v, i_o, factors=fac, threads=threads)
            kap, _ = orc.cond1(z, fac)
            per_f[k].update(kappa1_lapack=kap, mixed_vs_oracle=_rel(cur[k], i_o), mixed_vs_truth=_rel(cur[k], truth),
                            oracle_vs_truth=_rel(i_o, truth))
            del z, fac
    return {"workload": WORKLOADS["precision"].format(n=n, nf=len(freqs)), "value": value, "unit": UNIT,
            "steps": steps, "warmup": 2, "ms_per_step": ms,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "fp64_path": {"value": fp64_value, "unit": UNIT, "frequencies": 2,
                          "speedup_mixed_over_fp64": value / fp64_value},
            "tiers": tier_counts(rep), "per_frequency": per_f,
            "vs_reference": accuracy_vs_reference(freqs, cur, cur64, repc, _fixture("precision", n))}


def serving_leg(args, rate, seconds, max_wait=None):
    """One offered rate of the serving configuration (Poisson requests over seeded
    random-wire geometries, N in [512, 6144], 1-16 frequencies in 1 kHz - 30 MHz, 30%
    repeat excitations): p50/p99 latency, throughput and goodput; max_wait: load
    shedding (requests that waited longer when a worker takes them are turned away)."""
    st = serve_rates(args, [rate], seconds, max_wait=max_wait)[0]
    return st


def run_wmom(args):
    import numpy as np
    import torch
    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w = importlib.import_module(PKG)
    geo, freqs, ngap = workload(args.n, args.workload, args.nfreq)
    topo = w.Topology(geo)
    n = topo.npls
    nf = len(freqs)
    plan = w.Plan(topo)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    def max_over_ranks(x):
        if ws == 1:
            return x
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    # warm-up
    for _ in range(args.warmup):
        plan.solve(freqs, ngap, mode=w.MODE_MIXED, currents=False)
    torch.cuda.synchronize()

    # timed region: K steps of the mixed + refinement sweep, device-resident geometry,
    # nothing instrumented
    w.stats_reset()
    reports = []
    step_ms = []
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            t0 = time.perf_counter()
            _, zin, rep = plan.solve(freqs, ngap, mode=w.MODE_MIXED, currents=False)
            step_ms.append(1e3 * (time.perf_counter() - t0))
            reports.extend(rep)
        e1.record()
        torch.cuda.synchronize()
        barrier()
    launches = w.stats_read()
    clocks = clk.summary()
    ms = max_over_ranks(e0.elapsed_time(e1))
    value = ws * nf * args.steps / (ms / 1e3)

    # instrumented pass of one step: every library launch bracketed by CUDA events on
    # its stream (factorisations launched directly, not as a replayed graph, so each
    # kernel is timed); the roofline below comes from these per-launch times
    os.environ["WMOM_NO_GRAPHS"] = "1"
    w.stats_reset()
    w.stats_enable(True)
    plan.solve(freqs, ngap, mode=w.MODE_MIXED, currents=False)
    torch.cuda.synchronize()
    w.stats_enable(False)
    st = w.stats_read()
    del os.environ["WMOM_NO_GRAPHS"]

    # end to end through the C ABI: geometry upload + solves + currents to host
    barrier()
    e2e_value, h2d, d2h, cur, rep_e2e = e2e_sweep(w, topo, freqs, ngap, max(1, min(args.steps, 3)))
    e2e_value = ws * max_over_ranks(1.0 / e2e_value) ** -1

    # plain FP64 form on the same systems (lowest and highest frequency) + agreement,
    # and one more mixed sweep with condition estimates for the accuracy record
    fp64_value, cur64, rep64 = fp64_leg(w, plan, freqs, ngap)
    cur_c, _, rep_c = plan.solve(freqs, ngap, mode=w.MODE_MIXED, currents=True, condest=True)
    idx = {float(f): int(np.argmin(np.abs(freqs - f))) for f in cur64}
    rel = [_rel(cur[idx[f]], c) for f, c in cur64.items()]

    # roofline of the dominant kernel class (per-launch device time from the instrumented step)
    peaks, peak_src = _peaks()
    fp64_peak = w.probe_fp64_tflops()
    dom = max(st, key=lambda c: st[c]["ms"])
    d = st[dom]
    avg_ms = d["ms"] / max(d["timed"], 1)
    work_per_launch = d["work"] / max(d["timed"], 1)
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            caps = json.load(f)
    except (OSError, ValueError):
        caps = {}
    if dom == "fill":
        entries = work_per_launch / 384.0  # the library counts the fill's launches in 384 flop-eq per entry
        roof = fill_roofline(plan, nf, avg_ms, entries, fp64_peak, peaks, caps.get("fill_pair_multi_kernel"))
        units = entries
    else:
        if dom == "tc_gemm":
            achieved = work_per_launch / (avg_ms / 1e3) / 1e12
            roof = {"kernel": "cgemm_sub_tc_kernel", "bound": "tensor", "unit": "TFLOP/s",
                    "peak": peaks["bf16_tflops"], "peak_source": f"{peak_src} bf16 (TF32 nominal is half of it)"}
        elif dom == "emul_gemm":
            # 21 bf16 digit-plane products per complex FP64 product: issued tensor flops
            achieved = 21.0 * work_per_launch / (avg_ms / 1e3) / 1e12
            roof = {"kernel": "zgemm_sub_emul_kernel", "bound": "tensor", "unit": "TFLOP/s",
                    "peak": peaks["bf16_tflops"], "peak_source": f"{peak_src} bf16",
                    "note": "achieved counts the 21 bf16 plane products issued per FP64-grade product; the "
                            "FP64-equivalent rate is achieved / 21"}
        elif dom == "residual":
            achieved = work_per_launch / (avg_ms / 1e3) / 1e9
            roof = {"kernel": "gemv_partial_kernel", "bound": "hbm", "unit": "GB/s", "peak": peaks["hbm_gbs"],
                    "peak_source": peak_src}
        else:
            achieved = work_per_launch / (avg_ms / 1e3) / 1e12
            roof = {"kernel": {"panel": "panel_cluster_la_kernel"}.get(dom, dom), "bound": "fp64",
                    "unit": "TFLOP/s", "peak": fp64_peak,
                    "peak_source": "FP64 FMA pipe, measured in this run by wmom_probe_fp64_tflops"}
        roof.update({"achieved": achieved, "frac": achieved / roof["peak"]})
        units = {"tc_gemm": work_per_launch / (8.0 * 96),     # complex entries of C (K = 96)
                 "emul_gemm": work_per_launch / (8.0 * 96)}.get(dom)
    roof.update({"traffic": None, "avg_launch_ms": avg_ms, "launches": d["timed"],
                 "share_of_device_time": d["ms"] / max(sum(v["ms"] for v in st.values()), 1e-9)})
    # DRAM traffic per launch: bytes per unit from one ncu capture of a smaller case,
    # scaled by the units this launch processed (traffic grows in proportion)
    cap = caps.get(roof["kernel"].split("::")[-1])
    if cap and units:
        roof["traffic"] = cap["dram_bytes"] / cap["units"] * units
        roof["traffic_source"] = "ncu capture of a smaller case (%s), scaled by units" % cap["unit"]

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c128 fill/residual, c64 tensor-core LU", "data": "synthetic (seeded random wires)",
        "form": "mixed+refine (precision form)",
        "config": config_dict(args.workload, n, nf, ngap),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(sum(v["launches"] for v in launches.values())),
        "roofline": roof,
        "fp64_path": {"value": fp64_value, "unit": UNIT, "frequencies": len(cur64),
                      "speedup_mixed_over_fp64": value / ws / fp64_value,
                      "timing": "one warm-up call, then one timed call of both frequencies"},
        "accuracy": {"max_rel_err_mixed_vs_fp64": max(rel),
                     "max_rel_residual": max(r["rel_residual"] for r in reports),
                     "tiers": tier_counts(reports),
                     "krylov_refined": sum(1 for r in reports if r.get("krylov_steps", 0) > 0),
                     "max_refinement_steps": max(r["iterations"] for r in reports),
                     "kappa1_device": [r["cond1"] for r in rep_c],
                     "vs_reference": accuracy_vs_reference(freqs, cur_c, cur64, rep_c,
                                                           _fixture(args.workload, n) if not args.nfreq else None)},
        "latency_ms": {"p50_sweep": statistics.median(step_ms), "p99_sweep": sorted(step_ms)[-1]},
        "kernel_ms_one_instrumented_step": {k: round(v["ms"], 3) for k, v in st.items()},
        "fill_pairs_per_entry": plan.fill_pairs / float(n * n),
        "lu_config": dict(zip(("batch", "span", "tile_n", "panel_w"),
                              (w.tuned_config(n, w.MODE_MIXED) or (None, None)) +
                              (w.tuned_shape(n, w.MODE_MIXED) or (None, None)))),
        "clocks": clocks,
    }
    plan.close()
    if rank == 0 and not args.no_cpu_baseline:
        topo_o = oracle_topology(geo)  # the CPU path builds its own topology
        threads = os.cpu_count() or 1
        dt, i_cpu, _ = cpu_solve_once(topo_o, freqs[-1], ngap, threads)
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"1 of the {nf} frequencies ({freqs[-1]:.4g} MHz), full N={n} fill + "
                                          "zgetrf + zgetrs"}
        line["accuracy"]["cpu_oracle_%.6g_MHz" % freqs[-1]] = {
            "mixed_vs_cpu_oracle": _rel(cur_c[nf - 1], i_cpu),
            "fp64_vs_cpu_oracle": _rel(cur64[float(freqs[-1])], i_cpu)}
    if rank == 0 and args.workload == "sweep" and not args.nfreq and not args.no_extra_legs:
        line["precision_grid"] = precision_leg(w, args)
        line["serving"] = serving_leg(args, args.serve_default_rate, args.serve_default_seconds)
        # the configuration's own rate, 200 req/s, is beyond one GB300's capacity for
        # these requests (about 58 req/s): a server that sheds requests which waited over
        # 1 s keeps the served requests' latency bounded; shed count and goodput say
        # what that costs
        line["serving_200"] = serving_leg(args, 200.0, 4.0, max_wait=1.0)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def serve_rates(args, rates, seconds, max_wait=None):
    """Poisson request streams over a pool of seeded random-wire geometries (N uniform
    in [nmin, nmax]), 1-16 frequencies per request drawn log-uniformly from 64 values
    in 1 kHz - 30 MHz, 30% of the requests repeating an earlier (geometry,
    frequencies) with a new gap/amplitude (resident factors): one server per offered
    rate, `seconds` of arrivals, then drained.  Returns the server's stats per rate
    (p50/p99 latency, throughput, goodput within a 1 s objective)."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    w = importlib.import_module(PKG)
    serve = importlib.import_module(PKG + ".serve")
    if max_wait is None:
        max_wait = args.serve_max_wait
    rng = np.random.default_rng(SEED)
    pool = [w.geometry.random_wires(int(rng.integers(args.serve_nmin, args.serve_nmax + 1)), seed=SEED + i)
            for i in range(args.serve_geometries)]
    grid = w.geometry.log_freqs(0.001, 30.0, 64)
    results = []
    for rate in rates:
        warm = serve.Server(workers=1)  # warm-up: CUDA context, kernels, batch-width tuner
        warm.submit(serve.Request(pool[0], grid[:2], 1, currents=False)).result()
        warm.close()
        srv = serve.Server(workers=args.serve_workers, coalesce_freqs=args.serve_coalesce, max_wait_s=max_wait)
        t_end = time.perf_counter() + seconds
        history, futs = [], []
        t = time.perf_counter()
        while t < t_end:
            if history and rng.random() < 0.3:
                gi, fr = history[int(rng.integers(len(history)))]
            else:
                gi = int(rng.integers(len(pool)))
                fr = np.sort(rng.choice(grid, size=int(rng.integers(1, 17)), replace=False))
                history.append((gi, fr))
            ngap = int(rng.integers(1, 200))
            futs.append(srv.submit(serve.Request(pool[gi], fr, ngap, float(rng.uniform(0.5, 2.0)), currents=False)))
            t += rng.exponential(1.0 / rate)
            time.sleep(max(0.0, t - time.perf_counter()))
        for f in futs:
            try:
                f.result()
            except serve.Shed:
                pass  # counted by the server (shed_requests)
        st = srv.stats()
        srv.close()
        st.update(offered_req_per_s=rate, submitted=len(futs), seconds=seconds,
                  workload=f"Poisson requests, N in [{args.serve_nmin}, {args.serve_nmax}] over "
                           f"{args.serve_geometries} geometries, 1-16 frequencies in 1 kHz-30 MHz, 30% repeat "
                           f"excitations, {args.serve_workers} worker streams, waiting requests of one "
                           f"geometry factored together up to {args.serve_coalesce} frequencies"
                           + (f", requests that waited over {max_wait} s shed" if max_wait is not None else ""))
        results.append(st)
    return results


def run_serving(args):
    """Serving configuration at each offered rate of --serve-rates."""
    results = serve_rates(args, args.serve_rates, args.serve_seconds)
    line = {"metric": "serving: p50/p99 latency and freq-solves/s under a Poisson request stream",
            "unit": "freq-solves/s", "value": max(r["solves_per_s"] for r in results), "higher_is_better": True,
            "n_gpus": 1, "data": "synthetic (seeded random wires)",
            "config": {"workload": f"Poisson requests, N in [{args.serve_nmin}, {args.serve_nmax}], 1-16 "
                                   "frequencies in 1 kHz-30 MHz, 30% repeat excitations",
                       "geometries": args.serve_geometries, "seconds_per_rate": args.serve_seconds,
                       "workers": args.serve_workers, "coalesce_freqs": args.serve_coalesce,
                       "max_wait_s": args.serve_max_wait},
            "rates": results}
    print(json.dumps(line), flush=True)


def geometries_batched(w, pool, freqs, workers):
    """The set solved through wmom_factor_geometries: plans built on `workers` host
    threads (geometry tables are host work; ctypes releases the interpreter lock),
    one batched fill + factorisation per size class for all pairs, then every pair's
    solve (precision form, refinement to 1e-12) spread over `workers` streams.
    Returns (seconds, {phase: ms}, reports)."""
    import concurrent.futures as cf
    import torch
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(workers) as ex:
        plans = list(ex.map(lambda g: w.Plan(w.Topology(g, listing=False)), pool))
    t1 = time.perf_counter()
    sets = w.factor_geometries(plans, freqs, mode=w.MODE_MIXED)
    t2 = time.perf_counter()
    streams = [torch.cuda.Stream() for _ in range(workers)]

    def solve(i):
        st = streams[i % workers]
        return sets[i].solve(1, currents=False, stream=st.cuda_stream)[2][0]

    with cf.ThreadPoolExecutor(workers) as ex:
        reps = list(ex.map(solve, range(len(sets))))
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    for f in sets:
        f.close()
    for p in plans:
        p.close()
    return t3 - t0, {"plans": 1e3 * (t1 - t0), "fill_and_factor": 1e3 * (t2 - t1), "solves": 1e3 * (t3 - t2)}, reps


def run_geometries(args):
    """Batching over geometries: 64 seeded random-wire geometries with N uniform in
    [256, 4096] and one frequency each (log-uniform in 1 kHz - 30 MHz).  `value`: the
    whole set through wmom_factor_geometries (batched fill + factorisation per size
    class); beside it the same set submitted at once to the serving engine (one
    factorisation per request on its worker streams).  Reports freq-solves/s over the
    whole set, wall-clock from the geometry text to every pair's solution."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    w = importlib.import_module("praca-magisterska_gb300")
    serve = importlib.import_module("praca-magisterska_gb300.serve")
    rng = np.random.default_rng(SEED + 64)
    sizes = rng.integers(256, 4097, size=args.geometries)
    pool = [w.geometry.random_wires(int(nv), seed=SEED + 1000 + i) for i, nv in enumerate(sizes)]
    freqs = 10.0 ** rng.uniform(-3.0, np.log10(30.0), size=args.geometries)
    warm = serve.Server(workers=1)  # CUDA context and kernels
    warm.submit(serve.Request(pool[0], [float(freqs[0])], 1, currents=False)).result()
    warm.close()
    runs = []
    for _ in range(max(1, args.steps)):
        srv = serve.Server(workers=args.workers)
        t0 = time.perf_counter()
        futs = [srv.submit(serve.Request(g, [float(f)], 1, currents=False)) for g, f in zip(pool, freqs)]
        done = [f.result() for f in futs]
        dt = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        runs.append((dt, st, done))
    dt, st, done = min(runs, key=lambda r: r[0])
    fill_ms = _fill_all_geometries(w, pool, freqs)
    geometries_batched(w, pool, freqs, args.batch_workers)  # warm-up (kernels of every class)
    bruns = [geometries_batched(w, pool, freqs, args.batch_workers) for _ in range(max(1, args.steps))]
    bdt, phases, breps = min(bruns, key=lambda r: r[0])
    line = {"metric": "freq-solves/s over a set of geometries of uneven size (one frequency each)",
            "unit": "freq-solves/s", "value": args.geometries / bdt, "higher_is_better": True, "n_gpus": 1,
            "ms_per_step": 1e3 * bdt, "steps": len(bruns), "data": "synthetic (seeded random wires)",
            "config": {"workload": f"{args.geometries} random-wire geometries, N uniform in [256, 4096], one "
                                   "frequency each in 1 kHz-30 MHz, precision form", "workers": args.workers,
                       "batch_workers": args.batch_workers,
                       "unknowns_total": int(sizes.sum()),
                       "classes": len({w.padded_order(int(n)) for n in sizes})},
            "batched": {"phases_ms": phases, "tiers": tier_counts(breps),
                        "max_rel_residual": max(r["rel_residual"] for r in breps)},
            "serving_engine": {"value": args.geometries / dt, "ms": 1e3 * dt,
                               "latency_ms": {"p50": st.get("p50_ms"), "p99": st.get("p99_ms")}},
            "fill_ms_all_geometries": fill_ms,
            "fallbacks": int(sum(r["fell_back"] for d in done for r in d["reports"])) if done and
            isinstance(done[0], dict) and "reports" in done[0] else None}
    print(json.dumps(line), flush=True)


def _fill_all_geometries(w, pool, freqs, reps=3):
    """Device time to fill the Z of every geometry of the set at its frequency: one
    launch per geometry (Plan.fill) against one ragged launch for all of them
    (fill_geometries); best of `reps`, CUDA events on the current stream."""
    import torch
    plans = [w.Plan(w.Topology(g, listing=False)) for g in pool]
    fl = [float(f) for f in freqs]

    def timed(fn):
        best = None
        for _ in range(reps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn()
            e1.record()
            torch.cuda.synchronize()
            best = e0.elapsed_time(e1) if best is None else min(best, e0.elapsed_time(e1))
            del out
        return best

    try:
        per = timed(lambda: [p.fill([f]) for p, f in zip(plans, fl)])
        one = timed(lambda: w.fill_geometries(plans, fl))
    finally:
        for p in plans:
            p.close()
    return {"one_launch_per_geometry": per, "one_launch_for_all": one}


def run_gemm(args):
    """One trailing-update kernel alone (profiling cases): C -= A B for complex operands,
    m = n = --n, k = --k, through the C ABI on device-resident operands; W untimed then K
    timed calls, each bracketed by CUDA events.  gemm_emul: the FP64-grade digit-plane
    update (complex128); gemm_tc: the 3xTF32 update of the FP32 factorisation
    (complex64); gemm_simt / gemm_dmma: the plain FP64 form's update as SIMT DFMA or as
    DMMA on the FP64 tensor pipe (complex128)."""
    import ctypes
    import torch
    torch.cuda.set_device(0)
    w = importlib.import_module("praca-magisterska_gb300")
    m = nn = args.n
    k = args.k
    fp64 = args.workload in ("gemm_emul", "gemm_dmma", "gemm_simt")
    dt = torch.complex128 if fp64 else torch.complex64
    g = torch.Generator(device="cuda").manual_seed(SEED)
    a = torch.randn(k, m, dtype=dt, device="cuda", generator=g)   # column-major m x k
    b = torch.randn(nn, k, dtype=dt, device="cuda", generator=g)  # column-major k x n
    c = torch.randn(nn, m, dtype=dt, device="cuda", generator=g)  # column-major m x n
    if args.workload in ("gemm_dmma", "gemm_simt"):
        f = w._lib.wmom_zgemm_sub_fp64
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_longlong] * 3 + [ctypes.c_int, ctypes.c_void_p]
        variant = 1 if args.workload == "gemm_dmma" else 0
        call = lambda: f(m, nn, k, a.data_ptr(), m, b.data_ptr(), k, c.data_ptr(), m, variant, None)
    else:
        f = w._lib.wmom_zgemm_sub_emul if args.workload == "gemm_emul" else w._lib.wmom_cgemm_sub_tc
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_longlong] * 3 + [ctypes.c_void_p]
        call = lambda: f(m, nn, k, a.data_ptr(), m, b.data_ptr(), k, c.data_ptr(), m, None)
    for _ in range(args.warmup):
        assert call() == 0
    ms = []
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        assert call() == 0
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    med = statistics.median(ms)
    kernel = {"gemm_emul": "zgemm_sub_emul_kernel", "gemm_tc": "cgemm_sub_tc_kernel",
              "gemm_dmma": "zgemm_sub_dmma_kernel", "gemm_simt": "gemm_sub_kernel<double2>"}[args.workload]
    print(json.dumps({"metric": "trailing-update GEMM, algorithmic complex TFLOP/s (8 m n k)",
                      "kernel": kernel,
                      "value": 8.0 * m * nn * k / (med / 1e3) / 1e12, "unit": "TFLOP/s", "ms_per_call": med,
                      "steps": args.steps, "warmup": args.warmup, "config": {"m": m, "n": nn, "k": k}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="wmom", choices=["wmom", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--workload", default="sweep",
                    choices=sorted(WORKLOADS) + ["serving", "geometries", "gemm_emul", "gemm_tc", "gemm_dmma",
                                                 "gemm_simt"])
    ap.add_argument("--k", type=int, default=96, help="inner dimension of the gemm_* workloads")
    ap.add_argument("--geometries", type=int, default=64)
    ap.add_argument("--workers", type=int, default=6)  # best of 4/6/8/10 on the 64-geometry set
    ap.add_argument("--batch-workers", type=int, default=6,
                    help="host threads and streams of the geometry batch's plan builds and solves")
    ap.add_argument("--fp64-freqs", type=int, default=2)
    ap.add_argument("--nfreq", type=int, default=None,
                    help="use an evenly spaced subset of the workload's frequencies (profiling cases)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra-legs", action="store_true",
                    help="skip the precision-grid and serving sub-objects of the default run")
    ap.add_argument("--oracle-all-freqs", action="store_true",
                    help="precision-grid leg: compare every frequency with the CPU oracle and the truth")
    ap.add_argument("--serve-default-rate", type=float, default=40.0)
    ap.add_argument("--serve-default-seconds", type=float, default=8.0)
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[2.0, 5.0, 10.0])
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-nmin", type=int, default=512)
    ap.add_argument("--serve-nmax", type=int, default=6144)
    ap.add_argument("--serve-geometries", type=int, default=8)
    ap.add_argument("--serve-workers", type=int, default=4)  # 4 beat 2 at the saturated rates
    ap.add_argument("--serve-max-wait", type=float, default=None,
                    help="load shedding: requests that waited longer (s) when a worker takes them are turned away")
    ap.add_argument("--serve-coalesce", type=int, default=32,
                    help="distinct frequencies of one geometry factored together (0: one request at a time)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload in ("gemm_emul", "gemm_tc", "gemm_dmma", "gemm_simt"):
        run_gemm(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "geometries":
        run_geometries(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_wmom(args)


if __name__ == "__main__":
    main()
