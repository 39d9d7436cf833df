"""Serving: a continuous-batching request loop for (geometry, frequency list) solves.

A request names a geometry (.geo text), a list of frequencies and an excitation
(gap, amplitude, phase).  Worker threads, each with its own CUDA stream, take
requests as they arrive:

* the geometry's plan (device-resident tables) is created once and reused;
* Z and its LU factors of every (geometry, frequency) are kept resident on the
  device (libwmom wmom_factor), so a repeat excitation of a resident pair runs only
  the solves and refinement (wmom_factors_solve);
* the frequencies a request still needs are filled and factored together, i.e.
  batched on the device, with those of the requests for the same geometry that are
  waiting in the queue when a worker takes it (a frequency batch of one geometry:
  its results do not depend on the batch's composition);
* admission is by device-memory footprint: the bytes of the factor sets a request
  must create (Z + factors, nf * (16 + 8) * N^2 bytes in the precision form) are
  reserved against a budget; idle resident sets are evicted least-recently-used
  first, and a request that still does not fit waits until running requests free
  memory;
* requests that arrive while others run are admitted as soon as a worker and
  memory are free, and their GPU work overlaps with the running ones (separate
  streams);
* optional load shedding (max_wait_s): a request that has already waited longer
  when a worker takes it fails with Shed, so that under overload the served
  requests keep a bounded latency.

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


class Shed(Exception):
    """The request waited in the queue longer than the server's max_wait_s and was
    turned away without being served."""


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

    def __init__(self, mode=None, hbm_budget_bytes=None, workers=2, tol=1e-12, lib=None, stream_factory=None,
                 coalesce_freqs=32, max_wait_s=None):
        self._w = lib if lib is not None else importlib.import_module("praca-magisterska_gb300")
        self._new_stream = stream_factory or _cuda_stream
        self.mode = self._w.MODE_MIXED if mode is None else mode
        if hbm_budget_bytes is None:
            import torch
            free, _ = torch.cuda.mem_get_info()
            hbm_budget_bytes = int(free * 0.6)
        self.budget = int(hbm_budget_bytes)
        self.tol = tol
        # a worker serves, with the request it takes, the queued requests of the same
        # geometry, up to this many distinct frequencies together (0: one at a time)
        self.coalesce_freqs = int(coalesce_freqs)
        # load shedding: a request that has waited longer than this when a worker
        # takes it fails with Shed instead of being served (None: never)
        self.max_wait_s = max_wait_s
        self.shed = 0
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
        self.coalesced = 0        # requests served in a group of two or more
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
                   "resident_bytes": self._used, "budget_bytes": self.budget, "evictions": self.evictions,
                   "coalesced_requests": self.coalesced, "shed_requests": self.shed}
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

    def _admit(self, need, evicted):
        """Reserve `need` bytes, evicting idle sets LRU-first; caller holds the lock.
        Evicted sets leave the books here and are appended to `evicted`, which the
        caller closes after releasing the lock (freeing device memory must not hold up
        the other workers).  Returns False when it does not fit yet."""
        while self._used + self._reserved + need > self.budget:
            victim = next((k for k, r in self._sets.items() if r.pins == 0), None)
            if victim is None:
                return False
            r = self._sets.pop(victim)
            for f in list(r.index):
                if self._lookup.get((r.key, f)) is r:
                    del self._lookup[(r.key, f)]
            self._used -= r.bytes
            evicted.append(r)
            self.evictions += 1
        self._reserved += need
        return True

    def _take_group(self, req):
        """Queued requests for req's geometry that join it (caller holds the lock):
        taken in arrival order while their frequencies together stay within
        coalesce_freqs; the others keep their places in the queue."""
        group = [req]
        if self.coalesce_freqs <= 0:
            return group
        freqs = set(float(f) for f in req.freqs)
        keep = collections.deque()
        while self._queue:
            r = self._queue.popleft()
            if r.geo_key == req.geo_key:
                more = freqs | set(float(f) for f in r.freqs)
                if len(more) <= self.coalesce_freqs:
                    group.append(r)
                    freqs = more
                    continue
            keep.append(r)
        self._queue = keep
        return group

    def _run(self, wid):
        owner, sp = self._new_stream()  # noqa: F841  (owner keeps the stream alive)
        while True:
            with self._lock:
                while not self._queue and not self._stop:
                    self._lock.wait()
                if self._stop and not self._queue:
                    return
                group = self._take_group(self._queue.popleft())
                if self.max_wait_s is not None:
                    now = time.perf_counter()
                    late = [r for r in group if now - r.arrival > self.max_wait_s]
                    group = [r for r in group if now - r.arrival <= self.max_wait_s]
                    self.shed += len(late)
                else:
                    late = []
                if len(group) > 1:
                    self.coalesced += len(group)
            for r in late:
                r.future.set_exception(Shed(f"waited more than {self.max_wait_s} s in the queue"))
            if not group:
                continue
            try:
                self._serve(group, sp)
            except Exception as e:  # the group's requests fail, the loop goes on
                if len(group) == 1:
                    group[0].future.set_exception(e)
                    continue
                # one request may have caused it: each is retried alone, so that only
                # that request fails
                for r in group:
                    if r.future.done():
                        continue
                    try:
                        self._serve([r], sp)
                    except Exception as e1:
                        r.future.set_exception(e1)

    def _serve(self, group, sp):
        """Serves requests of one geometry: one admission and one factorisation of the
        frequencies they need that are not resident (a frequency batch of the
        geometry, whose results do not depend on its composition), then each
        request's solves."""
        topo, plan = self._plan(group[0])
        n = topo.npls
        key = group[0].geo_key
        ok = []
        for r in group:
            if 0 < r.ngap <= n:
                ok.append(r)
            else:
                r.future.set_exception(ValueError("gap outside the geometry"))
        if not ok:
            return
        group = ok
        freqs = sorted(set(float(f) for r in group for f in r.freqs))
        while True:
            evicted = []
            with self._lock:
                # pin what is resident, reserve what must be factored
                have = {f: self._lookup.get((key, f)) for f in freqs}
                missing = sorted(f for f, r in have.items() if r is None)
                pinned = {id(r): r for r in have.values() if r is not None}
                need = len(missing) * self._per_matrix_bytes(n)
                if need > self.budget:
                    raise MemoryError("request needs more device memory than the serving budget")
                for r in pinned.values():
                    r.pins += 1
                    self._sets.move_to_end(id(r))
                admitted = not missing or self._admit(need, evicted)
                if not admitted:
                    # a waiting request holds no pins: two waiters pinning the sets the
                    # other must evict would wait for each other forever
                    for r in pinned.values():
                        r.pins -= 1
            for r in evicted:  # unpinned and off the books: no request can reach them
                r.factors.close()
            if admitted:
                break
            with self._lock:
                self._lock.wait(timeout=0.05)
        reserved = need
        try:
            if missing:
                fac = self._w.Factors(plan, np.array(missing, np.float32), mode=self.mode, stream=sp)
                res = _Resident(fac, key, missing)
                res.pins = 1
                with self._lock:
                    self._reserved -= need
                    reserved = 0
                    self._used += res.bytes
                    self._sets[id(res)] = res
                    for f in missing:
                        self._lookup[(key, f)] = res
                        have[f] = res
                    self._lock.notify_all()
                pinned[id(res)] = res
            for req in group:
                self._solve_request(req, n, have, pinned, sp)
        finally:
            with self._lock:
                self._reserved -= reserved  # a factorisation that failed returns its reservation
                for r in pinned.values():
                    r.pins -= 1
                self._lock.notify_all()

    def _solve_request(self, req, n, have, pinned, sp):
        """Solves every frequency of req from its resident set (contiguous runs of a
        set's frequencies in one call) and completes its future."""
        freqs = [float(f) for f in req.freqs]
        cur = np.zeros((len(freqs), n), np.complex128) if req.currents else None
        zin = np.zeros(len(freqs), np.complex128)
        reports = [None] * len(freqs)
        by_set = collections.defaultdict(list)
        for k, f in enumerate(freqs):
            by_set[id(have[f])].append((have[f].index[f], k))
        for sid, items in by_set.items():
            res = pinned[sid]
            items.sort()
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
