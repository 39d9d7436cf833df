"""wmom -- GB300-native thin-wire Method-of-Moments fill-and-solve.

Host-side Python mirror of the reference's fill-and-solve path ("Praca magisterska",
``wersja referencyjna``): the same ``.geo`` / ``freq.txt`` inputs, the same
``configwire`` topology arrays, the same ``zmatrix`` fill and LAPACK-style LU
semantics, and the per-frequency input impedance and currents.  Every numeric
step runs in libwmom.so (hand-written sm_103a CUDA behind a C ABI, include/wmom.h);
this module only marshals arguments.  There is no CPU fallback: if the library is
missing, importing this package raises.

The package directory name contains a hyphen, so import it with
``importlib.import_module("praca-magisterska_gb300")``.
"""
import ctypes
import os

import numpy as np

from . import geometry  # noqa: F401  (workload generators)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libwmom.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        "libwmom.so is not built; run praca-magisterska_gb300/build.py (or __graft_entry__.build()) first")

_lib = ctypes.CDLL(LIB_PATH)

WMOM_OK = 0
STATUS_NAMES = {
    0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "singular matrix (zero pivot)",
    4: "device-side wait timed out", 5: "out of device memory",
    6: "iterative refinement did not converge", 7: "invalid geometry", 8: "unsupported device",
}
MODE_FP64 = 0
MODE_MIXED = 1
SOLVE_CONDEST = 0x100  # OR'd into a mode: estimate kappa_1 of every matrix (report "cond1")
NSMAX = 30480   # array capacity of the reference driver (Wire_MoM.cu:44)
NWMAX = 10000


class WmomError(RuntimeError):
    def __init__(self, status, what="", detail=""):
        self.status = status
        self.detail = detail
        msg = f"{what}: {STATUS_NAMES.get(status, status)} (status {status})"
        super().__init__(msg + (f" [{detail}]" if detail else ""))


_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class _Topology(ctypes.Structure):
    _fields_ = [("nsmax", ctypes.c_int), ("npnt", ctypes.c_int), ("npls", ctypes.c_int),
                ("nseg", ctypes.c_int), ("nw", ctypes.c_int),
                ("x", _fp), ("y", _fp), ("z", _fp), ("rad", _fp),
                ("ipc", _ip), ("ips", _ip), ("ise", _ip), ("isp", _ip), ("iwe", _ip)]


class _Report(ctypes.Structure):
    _fields_ = [("rel_residual", ctypes.c_double), ("iterations", ctypes.c_int),
                ("fell_back", ctypes.c_int), ("info", ctypes.c_int), ("status", ctypes.c_int),
                ("krylov_steps", ctypes.c_int), ("tier", ctypes.c_int), ("cond1", ctypes.c_double)]


def _sig(name, res, args):
    f = getattr(_lib, name)
    f.restype = res
    f.argtypes = args
    return f


_topology_from_geo = _sig("wmom_topology_from_geo", ctypes.c_int,
                          [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Topology),
                           ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t])
_ka = _sig("wmom_ka", ctypes.c_double, [ctypes.c_float])
_plan_create = _sig("wmom_plan_create", ctypes.c_int,
                    [_fp, _fp, _fp, _fp, _ip, _ip, _ip, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                     ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.POINTER(_vp)])
_plan_destroy = _sig("wmom_plan_destroy", ctypes.c_int, [_vp])
_plan_npls = _sig("wmom_plan_npls", ctypes.c_int, [_vp])
_plan_upload_bytes = _sig("wmom_plan_upload_bytes", ctypes.c_longlong, [_vp])
_plan_fill_variant = _sig("wmom_plan_fill_variant", ctypes.c_int, [_vp])
_plan_fill_pairs = _sig("wmom_plan_fill_pairs", ctypes.c_longlong, [_vp])
_plan_loops = _sig("wmom_plan_loops", ctypes.c_int, [_vp])
_plan_set_loads = _sig("wmom_plan_set_loads", ctypes.c_int, [_vp, ctypes.c_int, _ip, _dp, _dp])
_fill = _sig("wmom_fill", ctypes.c_int, [_vp, _dp, ctypes.c_int, _vp, ctypes.c_longlong, ctypes.c_longlong, _vp])
_fill_geometries = _sig("wmom_fill_geometries", ctypes.c_int,
                        [ctypes.POINTER(_vp), ctypes.c_int, _dp, ctypes.POINTER(_vp),
                         ctypes.POINTER(ctypes.c_longlong), _vp])
_zgetrf = _sig("wmom_zgetrf", ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_longlong, _vp, _ip, _vp])
_cgetrf = _sig("wmom_cgetrf", ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_longlong, _vp, _ip, _vp])
_zgetrs = _sig("wmom_zgetrs", ctypes.c_int,
               [ctypes.c_int, ctypes.c_int, _vp, ctypes.c_longlong, _vp, _vp, ctypes.c_longlong, _vp])
_zgesv_like = _sig("wmom_zgesv_like", ctypes.c_int, [ctypes.c_int, _dp, _dp, _dp, _ip, _ip])
_zlange1 = _sig("wmom_zlange1", ctypes.c_int, [ctypes.c_int, _vp, ctypes.c_longlong, _dp, _vp])
_zgecon = _sig("wmom_zgecon", ctypes.c_int,
               [ctypes.c_int, _vp, ctypes.c_longlong, _vp, ctypes.c_double, _dp, _vp])
_debug_missing = _sig("wmom_debug_panel_missing_arrivals", None, [ctypes.c_int])
_excitation = _sig("wmom_excitation", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, _dp])
_solve_sweep = _sig("wmom_solve_sweep", ctypes.c_int,
                    [_vp, _fp, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                     ctypes.c_double, _dp, _dp, ctypes.POINTER(_Report), _vp])
_status_string = _sig("wmom_status_string", ctypes.c_char_p, [ctypes.c_int])
_last_error = _sig("wmom_last_error", ctypes.c_char_p, [])
_factor = _sig("wmom_factor", ctypes.c_int, [_vp, _fp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp), _vp])
_factors_solve = _sig("wmom_factors_solve", ctypes.c_int,
                      [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_double,
                       _dp, _dp, ctypes.POINTER(_Report), _vp])
_factors_bytes = _sig("wmom_factors_device_bytes", ctypes.c_longlong, [_vp])
_factor_geometries = _sig("wmom_factor_geometries", ctypes.c_int,
                          [ctypes.POINTER(_vp), ctypes.c_int, _fp, ctypes.c_int, ctypes.POINTER(_vp), _vp])
_padded_order = _sig("wmom_padded_order", ctypes.c_int, [ctypes.c_int])
_factors_destroy = _sig("wmom_factors_destroy", ctypes.c_int, [_vp])
_stats_enable = _sig("wmom_stats_enable", None, [ctypes.c_int])
_stats_reset = _sig("wmom_stats_reset", None, [])
_stats_read = _sig("wmom_stats_read", ctypes.c_int,
                   [_dp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong), _dp, ctypes.c_int])

_probe_fp64 = _sig("wmom_probe_fp64_tflops", ctypes.c_int, [_dp])
_diag_sincos = _sig("wmom_diag_sincos", ctypes.c_int, [_vp, ctypes.c_longlong, _vp, _vp])
_tuned_config = _sig("wmom_tuned_config", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _ip, _ip])
_tuned_shape = _sig("wmom_tuned_shape", ctypes.c_int, [ctypes.c_int, ctypes.c_int, _ip, _ip])

STAT_CLASSES = ["fill", "panel", "tc_gemm", "gemm", "trsm", "laswp", "residual", "misc", "emul_gemm", "trsv"]


def stats_enable(on=True):
    """Bracket every library kernel launch with CUDA events on its stream."""
    _stats_enable(1 if on else 0)


def stats_reset():
    _stats_reset()


def stats_read():
    """{class: dict(ms, launches, timed, work)} since the last reset."""
    n = len(STAT_CLASSES)
    ms = (ctypes.c_double * n)()
    la = (ctypes.c_longlong * n)()
    ti = (ctypes.c_longlong * n)()
    wk = (ctypes.c_double * n)()
    _stats_read(ms, la, ti, wk, n)
    return {c: dict(ms=ms[i], launches=la[i], timed=ti[i], work=wk[i]) for i, c in enumerate(STAT_CLASSES)}


def probe_fp64_tflops():
    """FP64 FMA throughput of the current device in TFLOP/s (short bounded kernel)."""
    v = ctypes.c_double(0.0)
    _check(_probe_fp64(ctypes.byref(v)), "wmom_probe_fp64_tflops")
    return v.value


def diag_sincos(x):
    """(sin, cos, sin_ref, cos_ref) of a CUDA float64 tensor: the fill's table-driven
    sin/cos and CUDA's sincos() of the same arguments."""
    import torch
    x = x.contiguous()
    out = torch.empty((x.numel(), 4), dtype=torch.float64, device=x.device)
    _check(_diag_sincos(x.data_ptr(), x.numel(), out.data_ptr(), torch.cuda.current_stream().cuda_stream),
           "wmom_diag_sincos")
    return out[:, 0], out[:, 1], out[:, 2], out[:, 3]


def tuned_config(n, mode):
    """(batch, span) the autotuner chose for order n in this process, or None."""
    b, sp = ctypes.c_int(0), ctypes.c_int(0)
    if _tuned_config(n, mode, ctypes.byref(b), ctypes.byref(sp)) != WMOM_OK:
        return None
    return b.value, sp.value


def tuned_shape(n, mode):
    """(tile columns, widest panel) the autotuner chose for order n in this process:
    FP32 columns of a tensor-core update tile (256 or 128) and the widest FP32 panel
    (0 = as wide as shared memory allows); None before order n was tuned."""
    t, pw = ctypes.c_int(0), ctypes.c_int(0)
    if _tuned_shape(n, mode, ctypes.byref(t), ctypes.byref(pw)) != WMOM_OK:
        return None
    return t.value, pw.value


def _check(st, what):
    if st != WMOM_OK:
        detail = _last_error().decode(errors="replace") if st == 2 else ""  # WMOM_ERR_CUDA
        raise WmomError(st, what, detail)


def _ptr(a, t):
    return a.ctypes.data_as(t)


def library_symbols():
    """Names of the C-ABI entry points this module binds."""
    return ["wmom_topology_from_geo", "wmom_ka", "wmom_plan_create", "wmom_plan_destroy", "wmom_plan_npls",
            "wmom_fill", "wmom_zgetrf", "wmom_zgetrs", "wmom_zgesv_like", "wmom_excitation",
            "wmom_solve_sweep", "wmom_status_string", "wmom_stats_enable", "wmom_stats_reset", "wmom_stats_read"]


# ----------------------------------------------------------------- geometry ----
class Topology:
    """Reference topology arrays (configwire layout: 0-based storage, 1-based values,
    second columns at offset nsmax) built from the text of a .geo file."""

    def __init__(self, geo_text, ienv=1, nsmax=NSMAX, nwmax=NWMAX, listing=True):
        """listing=False skips the configwire.txt text (self.listing is then None)."""
        self.nsmax = nsmax
        self.ienv = ienv
        self.x = np.zeros(nsmax, np.float32)
        self.y = np.zeros(nsmax, np.float32)
        self.z = np.zeros(nsmax, np.float32)
        self.rad = np.zeros(nsmax, np.float32)
        self.ipc = np.zeros(nsmax, np.int32)
        self.ips = np.zeros(2 * nsmax, np.int32)
        self.ise = np.zeros(2 * nsmax, np.int32)
        self.isp = np.zeros(2 * nsmax, np.int32)
        self.iwe = np.zeros(2 * nsmax, np.int32)
        t = _Topology(nsmax, 0, 0, 0, 0, _ptr(self.x, _fp), _ptr(self.y, _fp), _ptr(self.z, _fp),
                      _ptr(self.rad, _fp), _ptr(self.ipc, _ip), _ptr(self.ips, _ip), _ptr(self.ise, _ip),
                      _ptr(self.isp, _ip), _ptr(self.iwe, _ip))
        cap = (1 << 24) if listing else 0
        buf = ctypes.create_string_buffer(cap) if listing else None
        err = ctypes.create_string_buffer(512)
        st = _topology_from_geo(geo_text.encode(), ienv, nsmax, nwmax, ctypes.byref(t), buf, cap, err, 512)
        if st != WMOM_OK:
            raise WmomError(st, "wmom_topology_from_geo: " + err.value.decode(errors="replace"))
        self.npnt, self.npls, self.nseg, self.nw = t.npnt, t.npls, t.nseg, t.nw
        self.listing = buf.value.decode() if listing else None
        if ienv == 1:
            self.sgn = (1.0, 1.0, 1.0, 1.0)
        else:  # PEC ground at z = 0 (Wire_MoM.cu:107-122)
            self.sgn = (1.0, 1.0, -1.0, -1.0)

    @classmethod
    def from_file(cls, path, **kw):
        with open(path) as f:
            return cls(f.read(), **kw)

    def arrays(self):
        return dict(x=self.x, y=self.y, z=self.z, rad=self.rad, ipc=self.ipc, ips=self.ips, ise=self.ise,
                    nsmax=self.nsmax, npls=self.npls)


def ka(freq_mhz):
    """Wave number of a float32 MHz frequency (Wire_MoM.cu:338-340)."""
    return _ka(float(np.float32(freq_mhz)))


def read_freq_file(text):
    """freq.txt: a count, then that many frequencies in MHz, read as float32
    (Wire_MoM.cu:254-265)."""
    tok = text.split()
    n = int(tok[0])
    return np.array([np.float32(t) for t in tok[1:1 + n]], np.float32)


def excitation(npls, ngap, ampl=1.0, phas=0.0):
    v = np.zeros(npls, np.complex128)
    _check(_excitation(npls, ngap, ampl, phas, _ptr(v.view(np.float64), _dp)), "wmom_excitation")
    return v


# --------------------------------------------------------------------- plan ----
class Plan:
    """One geometry resident on the current CUDA device."""

    def __init__(self, topo):
        self.topo = topo
        h = _vp()
        sg = topo.sgn
        st = _plan_create(_ptr(topo.x, _fp), _ptr(topo.y, _fp), _ptr(topo.z, _fp), _ptr(topo.rad, _fp),
                          _ptr(topo.ipc, _ip), _ptr(topo.ips, _ip), _ptr(topo.ise, _ip), topo.nsmax, topo.npls,
                          topo.ienv, sg[0], sg[1], sg[2], sg[3], ctypes.byref(h))
        _check(st, "wmom_plan_create")
        self._h = h
        self.npls = topo.npls
        self.upload_bytes = int(_plan_upload_bytes(h))
        fv = _plan_fill_variant(h)
        self.fill_variant = "pair" if fv >= 1 else "entry"
        self.multi_frequency_fill = fv == 2
        # pairs the pair-tiled fill evaluates per frequency (0 for the per-entry fill)
        self.fill_pairs = int(_plan_fill_pairs(h))
        # independent closed current paths (0 for open wires and trees)
        self.loops = int(_plan_loops(h))

    def close(self):
        if self._h:
            _plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_loads(self, loads):
        """Lumped series loads [(basis index 1-based, R ohm, L uH), ...] added to the
        diagonal of Z in every sweep of this plan (empty list clears)."""
        n = len(loads)
        idx = np.array([l[0] for l in loads], np.int32)
        r = np.array([l[1] for l in loads], np.float64)
        lh = np.array([l[2] for l in loads], np.float64)
        _check(_plan_set_loads(self._h, n, _ptr(idx, _ip), _ptr(r, _dp), _ptr(lh, _dp)), "wmom_plan_set_loads")

    def fill_device(self, kas, z_ptr, ldz, zstride, stream=0):
        kas = np.ascontiguousarray(kas, np.float64)
        _check(_fill(self._h, _ptr(kas, _dp), len(kas), z_ptr, ldz, zstride, stream), "wmom_fill")

    def fill(self, freqs_mhz):
        """Impedance matrices for float32 MHz frequencies, as a complex128 torch tensor
        on the device of shape (nfreq, npls, npls) whose [k].T is the reference's
        column-major cz (element [k, n, m] = Z[m, n])."""
        import torch
        freqs = np.atleast_1d(np.asarray(freqs_mhz, np.float32))
        n = self.npls
        z = torch.empty((len(freqs), n, n), dtype=torch.complex128, device="cuda")
        kas = np.array([ka(f) for f in freqs], np.float64)
        self.fill_device(kas, z.data_ptr(), n, n * n, torch.cuda.current_stream().cuda_stream)
        return z

    def solve(self, freqs_mhz, ngap, ampl=1.0, phas=0.0, mode=MODE_FP64, tol=1e-12, currents=True, stream=0,
              condest=False):
        """Fill, factor and solve per frequency.  Returns (currents (nfreq, npls) complex128
        or None, zin (nfreq,) complex128, reports list of dicts).  condest=True adds the
        estimated 1-norm condition number of every matrix to its report ("cond1")."""
        if condest:
            mode |= SOLVE_CONDEST
        freqs = np.ascontiguousarray(np.atleast_1d(freqs_mhz), np.float32)
        nf = len(freqs)
        cur = np.zeros((nf, self.npls), np.complex128) if currents else None
        zin = np.zeros(nf, np.complex128)
        reps = (_Report * nf)()
        st = _solve_sweep(self._h, _ptr(freqs, _fp), nf, ngap, ampl, phas, mode, tol,
                          _ptr(cur.view(np.float64), _dp) if cur is not None else None,
                          _ptr(zin.view(np.float64), _dp), reps, stream)
        if st not in (WMOM_OK, 3):
            raise WmomError(st, "wmom_solve_sweep")
        return cur, zin, _reports(reps)


def _reports(reps):
    return [dict(rel_residual=r.rel_residual, iterations=r.iterations, fell_back=r.fell_back, info=r.info,
                 status=r.status, krylov_steps=r.krylov_steps, tier=r.tier, cond1=r.cond1) for r in reps]


def fill_geometries(plans, freqs_mhz):
    """Impedance matrices of several geometries (plans) of any sizes, one float32 MHz
    frequency each, filled in one launch: a list of complex128 device tensors, the
    i-th of shape (npls_i, npls_i) laid out as Plan.fill's [k] (its .T is cz)."""
    import torch
    freqs = np.atleast_1d(np.asarray(freqs_mhz, np.float32))
    if len(freqs) != len(plans) or not plans:
        raise ValueError("one frequency per plan")
    zs = [torch.empty((p.npls, p.npls), dtype=torch.complex128, device="cuda") for p in plans]
    count = len(plans)
    hs = (_vp * count)(*[p._h for p in plans])
    kas = np.array([ka(f) for f in freqs], np.float64)
    ptrs = (_vp * count)(*[z.data_ptr() for z in zs])
    lds = (ctypes.c_longlong * count)(*[p.npls for p in plans])
    _check(_fill_geometries(hs, count, _ptr(kas, _dp), ptrs, lds, torch.cuda.current_stream().cuda_stream),
           "wmom_fill_geometries")
    return zs


class Factors:
    """Z and its LU factors for a list of frequencies of one plan, resident on the
    device: new excitations of those (geometry, frequency) pairs only run solves."""

    def __init__(self, plan, freqs_mhz, mode=MODE_MIXED, stream=0, condest=False):
        self.plan = plan  # keeps the plan alive
        self.freqs = np.ascontiguousarray(np.atleast_1d(freqs_mhz), np.float32)
        self.mode = mode
        h = _vp()
        _check(_factor(plan._h, _ptr(self.freqs, _fp), len(self.freqs), mode | (SOLVE_CONDEST if condest else 0),
                       ctypes.byref(h), stream), "wmom_factor")
        self._h = h
        self.device_bytes = int(_factors_bytes(h))

    @classmethod
    def _adopt(cls, plan, freqs_mhz, mode, handle):
        """Wraps a factor set the library made (factor_geometries)."""
        self = cls.__new__(cls)
        self.plan = plan
        self.freqs = np.ascontiguousarray(np.atleast_1d(freqs_mhz), np.float32)
        self.mode = mode
        self._h = _vp(handle)
        self.device_bytes = int(_factors_bytes(self._h))
        return self

    def solve(self, ngap, ampl=1.0, phas=0.0, first=0, count=None, tol=1e-12, currents=True, stream=0):
        count = len(self.freqs) - first if count is None else count
        n = self.plan.npls
        cur = np.zeros((count, n), np.complex128) if currents else None
        zin = np.zeros(count, np.complex128)
        reps = (_Report * count)()
        st = _factors_solve(self._h, first, count, ngap, ampl, phas, tol,
                            _ptr(cur.view(np.float64), _dp) if cur is not None else None,
                            _ptr(zin.view(np.float64), _dp), reps, stream)
        if st not in (WMOM_OK, 3):
            raise WmomError(st, "wmom_factors_solve")
        return cur, zin, _reports(reps)

    def close(self):
        if self._h:
            _factors_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def padded_order(npls):
    """The order at which factor_geometries stores a geometry of npls unknowns (its
    size class: four per octave, at most 1.25 npls)."""
    return int(_padded_order(int(npls)))


def factor_geometries(plans, freqs_mhz, mode=MODE_MIXED, condest=False, stream=0):
    """Factor sets for (plans[i], freqs_mhz[i]) pairs of uneven orders, filled and
    factored in batched launches per size class (wmom_factor_geometries): a list of
    one-frequency Factors, each used like Factors(plan, [f]).  A pair's results do not
    depend on the other pairs of the call."""
    freqs = np.ascontiguousarray(np.atleast_1d(freqs_mhz), np.float32)
    if len(freqs) != len(plans) or not plans:
        raise ValueError("one frequency per plan")
    count = len(plans)
    hs = (_vp * count)(*[p._h for p in plans])
    outs = (_vp * count)()
    _check(_factor_geometries(hs, count, _ptr(freqs, _fp), mode | (SOLVE_CONDEST if condest else 0), outs, stream),
           "wmom_factor_geometries")
    return [Factors._adopt(p, [f], mode, outs[i]) for i, (p, f) in enumerate(zip(plans, freqs))]


# ----------------------------------------------------------------- LAPACK-ish ----
def zgetrf_device(a_ptr, n, lda, ipiv_ptr, stream=0):
    info = ctypes.c_int(0)
    st = _zgetrf(n, a_ptr, lda, ipiv_ptr, ctypes.byref(info), stream)
    if st not in (WMOM_OK, 3):
        raise WmomError(st, "wmom_zgetrf")
    return info.value


def cgetrf_device(a_ptr, n, lda, ipiv_ptr, stream=0):
    """FP32 (complex64) LU of the precision form on a device matrix; returns info."""
    info = ctypes.c_int(0)
    st = _cgetrf(n, a_ptr, lda, ipiv_ptr, ctypes.byref(info), stream)
    if st not in (WMOM_OK, 3):
        raise WmomError(st, "wmom_cgetrf")
    return info.value


def zlange1_device(a_ptr, n, lda, stream=0):
    """||A||_1 of an n x n complex128 device matrix (LAPACK zlange '1')."""
    v = ctypes.c_double(0.0)
    _check(_zlange1(n, a_ptr, lda, ctypes.byref(v), stream), "wmom_zlange1")
    return v.value


def zgecon_device(a_ptr, n, lda, ipiv_ptr, anorm, stream=0):
    """LAPACK zgecon ('1' norm) on device factors from zgetrf_device: the reciprocal
    condition estimate 1 / (anorm * est ||A^-1||_1)."""
    v = ctypes.c_double(0.0)
    _check(_zgecon(n, a_ptr, lda, ipiv_ptr, anorm, ctypes.byref(v), stream), "wmom_zgecon")
    return v.value


def debug_panel_missing_arrivals(count):
    """Test hook: the plain FP64 LU's cooperative panel barriers wait for `count`
    arrivals that never come (their bounded waits run out); 0 restores normal use."""
    _debug_missing(int(count))


def zgetrs_device(n, nrhs, a_ptr, lda, ipiv_ptr, b_ptr, ldb, stream=0):
    _check(_zgetrs(n, nrhs, a_ptr, lda, ipiv_ptr, b_ptr, ldb, stream), "wmom_zgetrs")


def zgesv_like(Z, V):
    """Host-buffer drop-in for LAPACKE_zgetrf + zgetrs: Z (n, n) complex128 in the
    reference's column-major layout (a Fortran-ordered array), V (n,).  Returns
    (I, LU, ipiv, info)."""
    n = Z.shape[0]
    lu = np.array(Z, dtype=np.complex128, order="F", copy=True)
    v = np.ascontiguousarray(V, np.complex128)
    i_out = np.zeros(n, np.complex128)
    ipiv = np.zeros(n, np.int32)
    info = ctypes.c_int(0)
    st = _zgesv_like(n, lu.ctypes.data_as(_dp), _ptr(v.view(np.float64), _dp), _ptr(i_out.view(np.float64), _dp),
                     _ptr(ipiv, _ip), ctypes.byref(info))
    if st not in (WMOM_OK, 3):
        raise WmomError(st, "wmom_zgesv_like")
    return i_out, lu, ipiv, info.value
