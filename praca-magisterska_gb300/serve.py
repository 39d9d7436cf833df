"""Serving: a continuous-batching request loop for (geometry, frequency list) solves.

A request names a geometry (.geo text), a list of frequencies and an excitation
(gap, amplitude, phase).  Worker threads, each with its own CUDA stream, take
requests as they arrive:

* the geometry's plan (device-resident tables) is created once and reused;
* Z and its LU factors of every (geometry, frequency) are kept resident on the
  device (libwmom wmom_factor), so a repeat excitation of a resident pair runs only
  the solves and refinement (wmom_factors_solve);
* the frequencies a request still needs are filled and factored together, i.e.
  batched on the device;
* admission is by device-memory footprint: the bytes of the factor sets a request
  must create (Z + factors, nf * (16 + 8) * N^2 bytes in the precision form) are
  reserved against a budget; idle resident sets are evicted least-recently-used
  first, and a request that still does not fit waits until running requests free
  memory;
* requests that arrive while others run are admitted as soon as a worker and
  memory are free, and their GPU work overlaps with the running ones (separate
  streams).

Each completed request records its latency (arrival to completion); Server.stats()
reports p50/p99 latency, throughput and goodput.  The reference has no serving
path; its driver solved one fixed deck per run ("wersja referencyjna/Wire_MoM.cu":28-412).
"""
import collections
import hashlib
import importlib
import threading
import time
from concurrent.futures import Future

import numpy as np


class Request:
    def __init__(self, geo_text, freqs_mhz, ngap, ampl=1.0, phas=0.0, ienv=1, currents=True):
        self.geo_text = geo_text
        self.freqs = np.ascontiguousarray(np.atleast_1d(freqs_mhz), np.float32)
        self.ngap = int(ngap)
        self.ampl = float(ampl)
        self.phas = float(phas)
        self.ienv = int(ienv)
        self.currents = currents
        self.geo_key = hashlib.sha1(f"{ienv}\n{geo_text}".encode()).hexdigest()
        self.arrival = None
        self.future = Future()


_BUILDING = object()  # placeholder of a plan under construction


class _Resident:
    """One factor set: some frequencies of one geometry."""

    def __init__(self, factors, key, freqs):
        self.factors = factors
        self.key = key
        self.index = {float(f): i for i, f in enumerate(freqs)}
        self.bytes = factors.device_bytes
        self.pins = 0


def _cuda_stream():
    """A CUDA stream for one worker: (owner kept alive by the worker, raw handle)."""
    import torch
    s = torch.cuda.Stream()
    return s, s.cuda_stream


class Server:
    """`lib` and `stream_factory` stand in for the solver package and the worker
    streams (the host-logic tests run the loop on the CPU against a fake library)."""

    def __init__(self, mode=None, hbm_budget_bytes=None, workers=2, tol=1e-12, lib=None, stream_factory=None):
        self._w = lib if lib is not None else importlib.import_module("praca-magisterska_gb300")
        self._new_stream = stream_factory or _cuda_stream
        self.mode = self._w.MODE_MIXED if mode is None else mode
        if hbm_budget_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            hbm_budget_bytes = int(free * 0.6)
        self.budget = int(hbm_budget_bytes)
        self.tol = tol
        self._lock = threading.Condition()
        self._queue = collections.deque()
        self._plans = {}          # geo key -> (Topology, Plan)
        self._sets = collections.OrderedDict()  # id -> _Resident, LRU order
        self._lookup = {}         # (geo key, freq) -> _Resident
        self._used = 0            # resident bytes
        self._reserved = 0        # bytes reserved by admitted requests still factoring
        self._stop = False
        self._latency = []
        self._done_sizes = []     # frequencies of each completed request, in completion order
        self._solves = 0
        self._t0 = None
        self._t1 = None
        self.evictions = 0
        self._workers = [threading.Thread(target=self._run, args=(i,), daemon=True) for i in range(workers)]
        for t in self._workers:
            t.start()

    # ---------------------------------------------------------------- api ----
    def submit(self, req):
        req.arrival = time.perf_counter()
        with self._lock:
            if self._t0 is None:
                self._t0 = req.arrival
            self._queue.append(req)
            self._lock.notify_all()
        return req.future

    def close(self):
        with self._lock:
            self._stop = True
            self._lock.notify_all()
        for t in self._workers:
            t.join()
        with self._lock:
            for r in self._sets.values():
                r.factors.close()
            self._sets.clear()
            self._lookup.clear()
            for _, plan in self._plans.values():
                plan.close()
            self._plans.clear()

    def stats(self, slo_ms=1000.0):
        """Completed requests, frequency-solves, throughput, p50/p99 latency, and
        goodput: the frequency-solves per second of the requests that completed within
        slo_ms of their arrival."""
        with self._lock:
            lat = sorted(self._latency)
            span = (self._t1 - self._t0) if self._t0 and self._t1 else 0.0
            good = sum(nf for t, nf in zip(self._latency, self._done_sizes) if 1e3 * t <= slo_ms)
            out = {"requests": len(lat), "freq_solves": self._solves,
                   "solves_per_s": self._solves / span if span > 0 else 0.0,
                   "p50_ms": 1e3 * lat[len(lat) // 2] if lat else None,
                   "p99_ms": 1e3 * lat[min(len(lat) - 1, int(0.99 * len(lat)))] if lat else None,
                   "slo_ms": slo_ms, "goodput_solves_per_s": good / span if span > 0 else 0.0,
                   "resident_bytes": self._used, "budget_bytes": self.budget, "evictions": self.evictions}
        return out

    # ------------------------------------------------------------ internals ----
    def _plan(self, req):
        """The geometry's (Topology, Plan), built once.  Builds of different geometries
        run in parallel outside the server lock (parsing and table building are host
        work of tens of ms); a request for a geometry being built waits for it."""
        with self._lock:
            while True:
                ent = self._plans.get(req.geo_key)
                if ent is None:
                    self._plans[req.geo_key] = _BUILDING
                    break
                if ent is not _BUILDING:
                    return ent
                self._lock.wait(timeout=0.05)
        try:
            topo = self._w.Topology(req.geo_text, ienv=req.ienv, listing=False)
            ent = (topo, self._w.Plan(topo))
        except BaseException:
            with self._lock:
                del self._plans[req.geo_key]
                self._lock.notify_all()
            raise
        with self._lock:
            self._plans[req.geo_key] = ent
            self._lock.notify_all()
        return ent

    def _per_matrix_bytes(self, n):
        return n * n * (16 + (8 if self.mode == self._w.MODE_MIXED else 16)) + 4 * n

    def _admit(self, need):
        """Reserve `need` bytes, evicting idle sets LRU-first; caller holds the lock.
        Returns False when it does not fit yet."""
        while self._used + self._reserved + need > self.budget:
            victim = next((k for k, r in self._sets.items() if r.pins == 0), None)
            if victim is None:
                return False
            r = self._sets.pop(victim)
            for f in list(r.index):
                if self._lookup.get((r.key, f)) is r:
                    del self._lookup[(r.key, f)]
            self._used -= r.bytes
            r.factors.close()
            self.evictions += 1
        self._reserved += need
        return True

    def _run(self, wid):
        owner, sp = self._new_stream()  # noqa: F841  (owner keeps the stream alive)
        while True:
            with self._lock:
                while not self._queue and not self._stop:
                    self._lock.wait()
                if self._stop and not self._queue:
                    return
                req = self._queue.popleft()
            try:
                self._serve(req, sp)
            except Exception as e:  # the request fails, the loop goes on
                req.future.set_exception(e)

    def _serve(self, req, sp):
        topo, plan = self._plan(req)
        n = topo.npls
        if not 0 < req.ngap <= n:
            raise ValueError("gap outside the geometry")
        freqs = [float(f) for f in req.freqs]
        with self._lock:
            while True:
                # pin what is resident, reserve what must be factored
                have = {f: self._lookup.get((req.geo_key, f)) for f in freqs}
                missing = sorted({f for f, r in have.items() if r is None})
                pinned = {id(r): r for r in have.values() if r is not None}
                need = len(missing) * self._per_matrix_bytes(n)
                if need > self.budget:
                    raise MemoryError("request needs more device memory than the serving budget")
                for r in pinned.values():
                    r.pins += 1
                    self._sets.move_to_end(id(r))
                if not missing or self._admit(need):
                    break
                # a waiting request holds no pins: two waiters pinning the sets the
                # other must evict would wait for each other forever
                for r in pinned.values():
                    r.pins -= 1
                self._lock.wait(timeout=0.05)
        reserved = need
        try:
            if missing:
                fac = self._w.Factors(plan, np.array(missing, np.float32), mode=self.mode, stream=sp)
                res = _Resident(fac, req.geo_key, missing)
                res.pins = 1
                with self._lock:
                    self._reserved -= need
                    reserved = 0
                    self._used += res.bytes
                    self._sets[id(res)] = res
                    for f in missing:
                        self._lookup[(req.geo_key, f)] = res
                        have[f] = res
                    self._lock.notify_all()
                pinned[id(res)] = res
            # solve every frequency from its resident set
            cur = np.zeros((len(freqs), n), np.complex128) if req.currents else None
            zin = np.zeros(len(freqs), np.complex128)
            reports = [None] * len(freqs)
            by_set = collections.defaultdict(list)
            for k, f in enumerate(freqs):
                by_set[id(have[f])].append((have[f].index[f], k))
            for sid, items in by_set.items():
                res = pinned[sid]
                items.sort()
                # contiguous runs of set indices solve in one call
                run = [items[0]]
                for it in items[1:] + [None]:
                    if it is not None and it[0] == run[-1][0] + 1:
                        run.append(it)
                        continue
                    c, z, rp = res.factors.solve(req.ngap, req.ampl, req.phas, first=run[0][0], count=len(run),
                                                 tol=self.tol, currents=req.currents, stream=sp)
                    for j, (_, k) in enumerate(run):
                        zin[k] = z[j]
                        reports[k] = rp[j]
                        if cur is not None:
                            cur[k] = c[j]
                    run = [it] if it is not None else []
            done = time.perf_counter()
            with self._lock:
                self._latency.append(done - req.arrival)
                self._done_sizes.append(len(freqs))
                self._solves += len(freqs)
                self._t1 = done
            req.future.set_result({"zin": zin, "currents": cur, "reports": reports,
                                   "latency_s": done - req.arrival})
        finally:
            with self._lock:
                self._reserved -= reserved  # a factorisation that failed returns its reservation
                for r in pinned.values():
                    r.pins -= 1
                self._lock.notify_all()
