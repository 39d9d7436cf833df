"""Host logic of the serving loop (praca-magisterska_gb300/serve.py) on the CPU, against a
fake solver library: resident factor sets are reused by repeat excitations, admission
evicts idle sets least-recently-used first and never a pinned one, an oversized or a
failing request fails alone and returns its memory reservation, and requests waiting
for memory do not block each other, and waiting requests of one geometry are
factored together, a failing one failing alone.  The device path of the same loop is
covered by test_serve_gpu.py."""
import importlib
import threading
import time

import numpy as np
import pytest

serve = importlib.import_module("praca-magisterska_gb300.serve")

MODE_MIXED = 1


def _per_set(n, nf=1):
    """Bytes the server charges for nf matrices of order n in the precision form."""
    return nf * (n * n * (16 + 8) + 4 * n)


class FakeLib:
    """Topology/Plan/Factors with the package's call signatures.  A geometry text is
    "<name> <n>"; the solution of frequency f has Z_in = f + j*ampl and currents
    filled with f."""

    MODE_MIXED = MODE_MIXED

    def __init__(self):
        self.created = []     # (geometry name, tuple of frequencies) per Factors
        self.closed = []
        self.fail_freq = None
        self.hold = {}        # ampl -> (entered Event, release Event): solve() waits there
        self.mu = threading.Lock()
        self.topologies = []  # geometry name per Topology built
        self.parse_s = 0.0    # host time of one Topology build
        self.bad_geometries = set()
        lib = self

        class Topology:
            def __init__(self, text, ienv=1, listing=True):
                self.name, n = text.split()
                self.npls = int(n)
                with lib.mu:
                    lib.topologies.append(self.name)
                time.sleep(lib.parse_s)
                if self.name in lib.bad_geometries:
                    raise RuntimeError("bad geometry")

        class Plan:
            def __init__(self, topo):
                self.topo = topo

            def close(self):
                pass

        class Factors:
            def __init__(self, plan, freqs, mode, stream):
                assert mode == MODE_MIXED and stream == "stream"
                if lib.fail_freq is not None and lib.fail_freq in [float(f) for f in freqs]:
                    raise RuntimeError("factorisation failed")
                self.n = plan.topo.npls
                self.freqs = [float(f) for f in freqs]
                self.device_bytes = _per_set(self.n, len(self.freqs))
                with lib.mu:
                    lib.created.append((plan.topo.name, tuple(self.freqs)))

            def solve(self, ngap, ampl, phas, first, count, tol, currents, stream):
                if ampl in lib.hold:
                    entered, release = lib.hold[ampl]
                    entered.set()
                    assert release.wait(10)
                fs = self.freqs[first:first + count]
                c = np.array([np.full(self.n, f, np.complex128) for f in fs])
                z = np.array([f + 1j * ampl for f in fs])
                return c, z, [{"status": 0}] * count

            def close(self):
                with lib.mu:
                    lib.closed.append(tuple(self.freqs))

        self.Topology, self.Plan, self.Factors = Topology, Plan, Factors


def _server(lib, budget, workers=1):
    return serve.Server(hbm_budget_bytes=budget, workers=workers, lib=lib,
                        stream_factory=lambda: (None, "stream"))


def _check(res, freqs, ampl):
    np.testing.assert_array_equal(res["zin"], np.array([f + 1j * ampl for f in freqs]))
    for row, f in zip(res["currents"], freqs):
        assert np.all(row == f)


def test_repeat_excitation_reuses_resident_factors():
    lib = FakeLib()
    srv = _server(lib, budget=_per_set(64, 8))
    try:
        r1 = srv.submit(serve.Request("a 64", [1.0, 2.0], 5)).result(timeout=10)
        r2 = srv.submit(serve.Request("a 64", [3.0, 2.0, 1.0], 9, ampl=2.0)).result(timeout=10)
        _check(r1, [1.0, 2.0], 1.0)
        _check(r2, [3.0, 2.0, 1.0], 2.0)
        # the second request factors only the frequency that was not resident
        assert lib.created == [("a", (1.0, 2.0)), ("a", (3.0,))]
        st = srv.stats()
        assert st["requests"] == 2 and st["freq_solves"] == 5 and st["evictions"] == 0
        assert st["resident_bytes"] == _per_set(64, 3)
    finally:
        srv.close()
    assert sorted(lib.closed) == [(1.0, 2.0), (3.0,)]


def test_admission_evicts_least_recently_used_set():
    lib = FakeLib()
    srv = _server(lib, budget=_per_set(64, 2))
    try:
        for f in (1.0, 2.0):
            srv.submit(serve.Request("a 64", [f], 1)).result(timeout=10)
        srv.submit(serve.Request("a 64", [1.0], 2)).result(timeout=10)   # 1.0 is now the most recent
        srv.submit(serve.Request("a 64", [3.0], 1)).result(timeout=10)   # evicts 2.0
        assert lib.closed == [(2.0,)] and srv.stats()["evictions"] == 1
        srv.submit(serve.Request("a 64", [1.0, 3.0], 4)).result(timeout=10)
        assert len(lib.created) == 3   # both still resident
    finally:
        srv.close()


def test_oversized_request_fails_alone():
    lib = FakeLib()
    srv = _server(lib, budget=_per_set(64, 2))
    try:
        with pytest.raises(MemoryError):
            srv.submit(serve.Request("a 64", [1.0, 2.0, 3.0], 1)).result(timeout=10)
        with pytest.raises(ValueError):
            srv.submit(serve.Request("a 64", [1.0], 65)).result(timeout=10)   # gap outside the geometry
        _check(srv.submit(serve.Request("a 64", [1.0, 2.0], 1)).result(timeout=10), [1.0, 2.0], 1.0)
    finally:
        srv.close()


def test_failed_factorisation_returns_its_reservation():
    lib = FakeLib()
    srv = _server(lib, budget=_per_set(64, 2))
    try:
        lib.fail_freq = 7.0
        with pytest.raises(RuntimeError):
            srv.submit(serve.Request("a 64", [7.0, 8.0], 1)).result(timeout=10)
        lib.fail_freq = None
        # the whole budget is free again: a request needing all of it is admitted
        _check(srv.submit(serve.Request("a 64", [1.0, 2.0], 1)).result(timeout=10), [1.0, 2.0], 1.0)
        assert srv.stats()["resident_bytes"] == _per_set(64, 2)
    finally:
        srv.close()


@pytest.mark.timeout(60)   # the failure this guards against is a hang
def test_waiting_requests_do_not_pin_each_others_sets():
    """Two resident sets fill the budget.  While a repeat excitation solves from set A,
    request D (B + one new frequency) and request C (A + one new frequency) both wait
    for memory.  A waiter that kept its pins would hold the set the other must evict,
    and neither would ever be admitted."""
    lib = FakeLib()
    srv = _server(lib, budget=_per_set(64, 2), workers=3)
    try:
        srv.submit(serve.Request("a 64", [1.0], 1)).result(timeout=10)
        srv.submit(serve.Request("b 64", [1.0], 1)).result(timeout=10)
        entered, release = threading.Event(), threading.Event()
        lib.hold[7.0] = (entered, release)
        f_hold = srv.submit(serve.Request("a 64", [1.0], 3, ampl=7.0))   # pins A while it solves
        assert entered.wait(10)
        f_d = srv.submit(serve.Request("b 64", [1.0, 2.0], 2))
        time.sleep(0.2)
        f_c = srv.submit(serve.Request("a 64", [1.0, 2.0], 2))
        time.sleep(0.2)
        release.set()
        _check(f_hold.result(timeout=10), [1.0], 7.0)
        _check(f_c.result(timeout=10), [1.0, 2.0], 1.0)
        _check(f_d.result(timeout=10), [1.0, 2.0], 1.0)
        st = srv.stats()
        assert st["resident_bytes"] <= st["budget_bytes"] and st["evictions"] >= 1
    finally:
        srv.close()


def test_plans_build_in_parallel_and_once_per_geometry():
    """Plans of different geometries build concurrently, outside the server lock; two
    requests for one geometry share one build."""
    lib = FakeLib()
    lib.parse_s = 0.5
    srv = _server(lib, budget=_per_set(64, 16), workers=4)
    try:
        t0 = time.perf_counter()
        futs = [srv.submit(serve.Request(f"{g} 64", [1.0], 1)) for g in ("a", "b", "c", "a")]
        for f in futs:
            _check(f.result(timeout=10), [1.0], 1.0)
        dt = time.perf_counter() - t0
        assert sorted(lib.topologies) == ["a", "b", "c"]
        assert dt < 2 * lib.parse_s, dt   # serial builds would take 3 x 0.5 s
    finally:
        srv.close()


def test_failed_plan_build_fails_alone_and_is_retried():
    """A geometry whose plan build raises fails its request; the next request for it
    builds again (no placeholder is left behind), and other geometries are served."""
    lib = FakeLib()
    lib.bad_geometries.add("x")
    srv = _server(lib, budget=_per_set(64, 4), workers=2)
    try:
        with pytest.raises(RuntimeError):
            srv.submit(serve.Request("x 64", [1.0], 1)).result(timeout=10)
        _check(srv.submit(serve.Request("a 64", [1.0], 1)).result(timeout=10), [1.0], 1.0)
        lib.bad_geometries.clear()
        _check(srv.submit(serve.Request("x 64", [2.0], 1)).result(timeout=10), [2.0], 1.0)
        assert lib.topologies == ["x", "a", "x"]
    finally:
        srv.close()


def test_waiting_requests_of_one_geometry_are_factored_together():
    """While the only worker is busy, three requests for geometry a and one for b
    queue up.  The worker then takes the a requests together: one factorisation of
    the union of their missing frequencies (a frequency that is resident or shared is
    factored once), and b on its own.  Every request gets its own answers."""
    lib = FakeLib()
    srv = _server(lib, budget=_per_set(64, 16), workers=1)
    try:
        srv.submit(serve.Request("a 64", [1.0], 1)).result(timeout=10)
        entered, release = threading.Event(), threading.Event()
        lib.hold[9.0] = (entered, release)
        f_hold = srv.submit(serve.Request("a 64", [1.0], 2, ampl=9.0))
        assert entered.wait(10)
        f1 = srv.submit(serve.Request("a 64", [2.0, 3.0], 1, ampl=2.0))
        f2 = srv.submit(serve.Request("b 64", [2.0], 1, ampl=3.0))
        f3 = srv.submit(serve.Request("a 64", [3.0, 1.0, 4.0], 5, ampl=4.0))
        f4 = srv.submit(serve.Request("a 64", [5.0], 5, ampl=5.0))
        release.set()
        _check(f_hold.result(timeout=10), [1.0], 9.0)
        _check(f1.result(timeout=10), [2.0, 3.0], 2.0)
        _check(f2.result(timeout=10), [2.0], 3.0)
        _check(f3.result(timeout=10), [3.0, 1.0, 4.0], 4.0)
        _check(f4.result(timeout=10), [5.0], 5.0)
        assert lib.created == [("a", (1.0,)), ("a", (2.0, 3.0, 4.0, 5.0)), ("b", (2.0,))]
        st = srv.stats()
        assert st["requests"] == 6 and st["coalesced_requests"] == 3
    finally:
        srv.close()


def test_coalescing_respects_its_frequency_limit():
    lib = FakeLib()
    srv = serve.Server(hbm_budget_bytes=_per_set(64, 16), workers=1, lib=lib,
                       stream_factory=lambda: (None, "stream"), coalesce_freqs=3)
    try:
        entered, release = threading.Event(), threading.Event()
        lib.hold[9.0] = (entered, release)
        f_hold = srv.submit(serve.Request("a 64", [1.0], 2, ampl=9.0))
        assert entered.wait(10)
        futs = [srv.submit(serve.Request("a 64", fs, 1)) for fs in ([2.0, 3.0], [4.0, 5.0], [3.0])]
        release.set()
        f_hold.result(timeout=10)
        for f, fs in zip(futs, ([2.0, 3.0], [4.0, 5.0], [3.0])):
            _check(f.result(timeout=10), fs, 1.0)
        # [2, 3] + [4, 5] would be 4 frequencies: the second request waits for the
        # next round, the third (frequency 3) joins the first
        assert lib.created == [("a", (1.0,)), ("a", (2.0, 3.0)), ("a", (4.0, 5.0))]
    finally:
        srv.close()


def test_failing_request_in_a_group_fails_alone():
    """A group's factorisation fails because of one request's frequency: the
    requests are retried one by one, and only that request fails."""
    lib = FakeLib()
    srv = _server(lib, budget=_per_set(64, 16), workers=1)
    try:
        entered, release = threading.Event(), threading.Event()
        lib.hold[9.0] = (entered, release)
        f_hold = srv.submit(serve.Request("a 64", [1.0], 2, ampl=9.0))
        assert entered.wait(10)
        lib.fail_freq = 7.0
        f_ok1 = srv.submit(serve.Request("a 64", [2.0], 1))
        f_bad = srv.submit(serve.Request("a 64", [7.0, 3.0], 1))
        f_ok2 = srv.submit(serve.Request("a 64", [3.0], 1))
        release.set()
        f_hold.result(timeout=10)
        _check(f_ok1.result(timeout=10), [2.0], 1.0)
        _check(f_ok2.result(timeout=10), [3.0], 1.0)
        with pytest.raises(RuntimeError):
            f_bad.result(timeout=10)
        st = srv.stats()
        assert st["requests"] == 3 and st["resident_bytes"] <= st["budget_bytes"]
    finally:
        srv.close()


def test_load_shedding_turns_away_requests_that_waited_too_long():
    """With max_wait_s set, a request that has waited longer than that when a worker
    takes it fails with Shed and is counted; the others are served."""
    lib = FakeLib()
    srv = serve.Server(hbm_budget_bytes=_per_set(64, 16), workers=1, lib=lib,
                       stream_factory=lambda: (None, "stream"), max_wait_s=0.2)
    try:
        entered, release = threading.Event(), threading.Event()
        lib.hold[9.0] = (entered, release)
        f_hold = srv.submit(serve.Request("a 64", [1.0], 2, ampl=9.0))
        assert entered.wait(10)
        f_late = srv.submit(serve.Request("b 64", [1.0], 1))
        time.sleep(0.4)
        release.set()
        _check(f_hold.result(timeout=10), [1.0], 9.0)
        with pytest.raises(serve.Shed):
            f_late.result(timeout=10)
        _check(srv.submit(serve.Request("b 64", [2.0], 1)).result(timeout=10), [2.0], 1.0)
        st = srv.stats()
        assert st["shed_requests"] == 1 and st["requests"] == 2
    finally:
        srv.close()
