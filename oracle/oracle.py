"""CPU oracle of the thin-wire MoM fill-and-solve path -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs
as the checker; never by the product library.

* fill(): the C restatement of the reference's zmatrix() (oracle/wmom_oracle.c,
  after "wersja referencyjna/Zmatrix.cpp":27-770), optionally threaded over rows
  (entries are independent, so the result does not depend on the thread count).
* lu_solve(): LAPACK zgetrf + zgetrs, the routines the reference calls through
  LAPACKE ("wersja referencyjna/Wire_MoM.cu":372,382).  The reference linked Intel
  MKL (unversioned); here the system LAPACK that scipy ships is used (OpenBLAS on
  aarch64; in the build container torch's MKL 2024.2 is used instead when
  available, see lapack_backend()).  zgetf2()/zgetrs() restate the unblocked
  algorithm in C for small pinning cases.
* topology(): the reference's geoinp() + configwire() restated in C
  (oracle/topology_oracle.c), so that the CPU reference path builds its topology
  arrays without the product library.
* residual_dd() / refine_truth(): residuals in about twice double precision
  (oracle/refine_oracle.c) and iterative refinement with them, an extended-precision
  "truth" of the solution of a given FP64 system, which separates a solver's own
  error from the error the system's conditioning imposes on every FP64 solver.
* ref_*(): the reference's own Configuration.cpp/Zmatrix.cpp compiled unmodified
  (oracle/_ref/libwmomref.so), present only where the reference checkout exists.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libwmomref.so")

_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)

_port = None
_ref = None


def _load_port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            from . import build as _b
            _b.build_port()
        _port = ctypes.CDLL(PORT_SO)
        _port.oracle_zmatrix.restype = None
        _port.oracle_zmatrix.argtypes = [_dp, _fp, _fp, _fp, _ip, _ip, _ip, _fp, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_float, ctypes.c_int]
        _port.oracle_ka.restype = ctypes.c_double
        _port.oracle_ka.argtypes = [ctypes.c_float]
        _port.oracle_zgetf2.restype = ctypes.c_int
        _port.oracle_zgetf2.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip]
        _port.oracle_zgetrs.restype = None
        _port.oracle_zgetrs.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _dp]
        _port.oracle_residual_dd.restype = None
        _port.oracle_residual_dd.argtypes = [ctypes.c_int] + [_dp] * 6 + [ctypes.c_int]
        _port.oracle_topology.restype = ctypes.c_int
        _port.oracle_topology.argtypes = [ctypes.c_char_p] + [ctypes.c_int] * 5 + [_fp] * 4 + [_ip] * 6
    return _port


def ref_available():
    return os.path.exists(REF_SO)


def _load_ref():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_SO)
        _ref.ref_nsmax.restype = ctypes.c_int
        _ref.ref_load_geometry.restype = ctypes.c_int
        _ref.ref_load_geometry.argtypes = [ctypes.c_char_p, ctypes.c_int, _ip, _fp, _fp, _fp, _fp, _ip, _ip, _ip,
                                           _ip, _ip]
        _ref.ref_zmatrix.restype = None
        _ref.ref_zmatrix.argtypes = [_dp, _fp, _fp, _fp, _ip, _ip, _ip, _fp, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float]
    return _ref


def _p(a, t):
    return a.ctypes.data_as(t)


# array capacities of the reference driver ("wersja referencyjna/Wire_MoM.cu":43-44)
NNMAX, NTMAX, NWMAX, NSMAX = 3000, 5000, 10000, 30480
TOPOLOGY_ERRORS = {1: "parse error", 2: "too many nodes", 3: "too many wires", 4: "too many patches",
                   5: "node below a PEC ground", 6: "too many segments", 7: "too many basis functions",
                   8: "out of memory"}


def topology(geo_text, ienv=1, nsmax=NSMAX, nwmax=NWMAX):
    """The reference's geoinp() + configwire() on the text of a .geo file: a dict with
    x, y, z, rad, ipc (nsmax entries), ips, ise, isp, iwe (2*nsmax) in the reference
    layout, npnt, npls, nseg, nw, nsmax and the sign quadruple of its environment."""
    lib = _load_port()
    out = dict(x=np.zeros(nsmax, np.float32), y=np.zeros(nsmax, np.float32), z=np.zeros(nsmax, np.float32),
               rad=np.zeros(nsmax, np.float32), ipc=np.zeros(nsmax, np.int32), ips=np.zeros(2 * nsmax, np.int32),
               ise=np.zeros(2 * nsmax, np.int32), isp=np.zeros(2 * nsmax, np.int32),
               iwe=np.zeros(2 * nsmax, np.int32))
    counts = np.zeros(4, np.int32)
    rc = lib.oracle_topology(geo_text.encode(), ienv, nsmax, nwmax, NNMAX, NTMAX, _p(out["x"], _fp),
                             _p(out["y"], _fp), _p(out["z"], _fp), _p(out["rad"], _fp), _p(out["ipc"], _ip),
                             _p(out["ips"], _ip), _p(out["ise"], _ip), _p(out["isp"], _ip), _p(out["iwe"], _ip),
                             _p(counts, _ip))
    if rc != 0:
        raise ValueError("oracle topology: " + TOPOLOGY_ERRORS.get(rc, str(rc)))
    out.update(npnt=int(counts[0]), npls=int(counts[1]), nseg=int(counts[2]), nw=int(counts[3]), nsmax=nsmax,
               ienv=ienv, sgn=(1.0, 1.0, 1.0, 1.0) if ienv == 1 else (1.0, 1.0, -1.0, -1.0))
    return out


def ka(freq_mhz):
    return _load_port().oracle_ka(float(np.float32(freq_mhz)))


def fill(g, freq_mhz, ienv=1, sgn=(1.0, 1.0, 1.0, 1.0), threads=1):
    """Z (npls x npls complex128, Fortran order = the reference's column-major cz).
    g: mapping with x, y, z, rad, ipc, ips, ise (reference layout), nsmax, npls."""
    lib = _load_port()
    n = int(g["npls"])
    z = np.zeros((n, n), np.complex128, order="F")
    lib.oracle_zmatrix(z.ctypes.data_as(_dp), _p(g["x"], _fp), _p(g["y"], _fp), _p(g["z"], _fp),
                       _p(g["ipc"], _ip), _p(g["ips"], _ip), _p(g["ise"], _ip), _p(g["rad"], _fp), n,
                       ka(freq_mhz), int(g["nsmax"]), ienv, sgn[0], sgn[1], sgn[2], sgn[3], threads)
    return z


def zgetf2(a):
    """Unblocked LU (zgetf2 semantics) of a copy of a; returns (lu, ipiv 1-based, info)."""
    lib = _load_port()
    lu = np.array(a, np.complex128, order="F", copy=True)
    n = lu.shape[0]
    ipiv = np.zeros(n, np.int32)
    info = lib.oracle_zgetf2(n, lu.ctypes.data_as(_dp), n, _p(ipiv, _ip))
    return lu, ipiv, info


def zgetrs(lu, ipiv, b):
    lib = _load_port()
    x = np.array(b, np.complex128, copy=True)
    n = lu.shape[0]
    lu = np.asfortranarray(lu)
    lib.oracle_zgetrs(n, lu.ctypes.data_as(_dp), n, _p(np.ascontiguousarray(ipiv, np.int32), _ip),
                      x.ctypes.data_as(_dp))
    return x


def lapack_backend():
    return "scipy"


def lu_solve(z, v, return_factors=False):
    """I = Z^-1 V with LAPACK zgetrf + zgetrs (partial pivoting).  Returns (I, info),
    or (I, info, (lu, piv)) with return_factors."""
    from scipy.linalg import lapack
    lu, piv, info = lapack.zgetrf(np.asfortranarray(z), overwrite_a=0)
    if info < 0:
        raise ValueError("zgetrf argument error")
    x, info2 = lapack.zgetrs(lu, piv, np.asarray(v, np.complex128))
    if return_factors:
        return x, info, (lu, piv)
    return x, info


def cond1(z, factors=None):
    """kappa_1 of Z estimated by LAPACK zgecon from (lu, piv) of scipy's zgetrf, and
    ||Z||_1 (zlange '1')."""
    from scipy.linalg import lapack
    zf = np.asfortranarray(z, np.complex128)
    anorm = float(np.max(np.sum(np.abs(zf), axis=0)))
    if factors is None:
        lu, piv, _ = lapack.zgetrf(zf, overwrite_a=0)
    else:
        lu, piv = factors
    rcond, info = lapack.zgecon(lu, anorm, norm="1")
    return (1.0 / rcond if rcond > 0 else float("inf")), anorm


def residual_dd(z, v, xh, xl=None, threads=1):
    """(r_hi, r_lo): b - Z (xh + xl) in about twice double precision; Z (n, n)
    complex128 (any memory order), v, xh, xl complex n-vectors."""
    lib = _load_port()
    zf = np.asfortranarray(z, np.complex128)
    n = zf.shape[0]
    v = np.ascontiguousarray(v, np.complex128)
    xh = np.ascontiguousarray(xh, np.complex128)
    xl = np.zeros(n, np.complex128) if xl is None else np.ascontiguousarray(xl, np.complex128)
    rh = np.zeros(n, np.complex128)
    rl = np.zeros(n, np.complex128)
    lib.oracle_residual_dd(n, zf.ctypes.data_as(_dp), v.ctypes.data_as(_dp), xh.ctypes.data_as(_dp),
                           xl.ctypes.data_as(_dp), rh.ctypes.data_as(_dp), rl.ctypes.data_as(_dp), threads)
    return rh, rl


def refine_truth(z, v, x0, factors=None, max_steps=30, threads=1):
    """Solution of the FP64 system Z x = v to about 2^-106 relative: iterative
    refinement from x0 with residuals in twice double precision (residual_dd), the
    corrections solved with an FP64 LU (`factors` = scipy zgetrf (lu, piv) of Z or of
    a matrix close to Z; computed here when None), x carried as a double-double.
    Returns (x rounded to complex128, list of ||d|| / ||x|| per step)."""
    from scipy.linalg import lapack
    zf = np.asfortranarray(z, np.complex128)
    if factors is None:
        lu, piv, info = lapack.zgetrf(zf, overwrite_a=0)
        if info != 0:
            raise ValueError("zgetrf info %d" % info)
    else:
        lu, piv = factors
    xh = np.array(x0, np.complex128, copy=True)
    xl = np.zeros_like(xh)
    hist = []
    for _ in range(max_steps):
        rh, _ = residual_dd(zf, v, xh, xl, threads)
        d, info = lapack.zgetrs(lu, piv, rh)
        # (xh, xl) += d, componentwise two-sum then renormalisation
        s = xh + d
        bb = s - xh
        e = (xh - (s - bb)) + (d - bb)
        lo = xl + e
        hi = s + lo
        xl = lo - (hi - s)
        xh = hi
        rel = float(np.linalg.norm(d) / max(np.linalg.norm(xh), 1e-300))
        hist.append(rel)
        # done: the correction is far below double precision, or it no longer
        # shrinks at the level set by the double-double residual's own rounding
        # (about kappa * 2^-106)
        if rel <= 2.0 ** -80 or (len(hist) > 2 and rel > 0.5 * hist[-2] and rel < 2.0 ** -60):
            break
    return xh, hist


def zin(v, i, ngap):
    return complex(v[ngap - 1]) / complex(i[ngap - 1])


def excitation(npls, ngap, ampl=1.0, phas=0.0):
    v = np.zeros(npls, np.complex128)
    arg = np.pi * float(np.float32(phas)) / 180.0
    a = abs(float(np.float32(ampl)))
    v[ngap - 1] = complex(a * np.cos(arg), a * np.sin(arg))
    return v


def solve(g, freq_mhz, ngap, ampl=1.0, phas=0.0, ienv=1, sgn=(1.0, 1.0, 1.0, 1.0), threads=1):
    """One frequency of the reference driver: fill, LU, solve, Z_in.  Returns (I, zin, Z)."""
    z = fill(g, freq_mhz, ienv, sgn, threads)
    v = excitation(int(g["npls"]), ngap, ampl, phas)
    i, _ = lu_solve(z, v)
    return i, zin(v, i, ngap), z


# ------------------------------------------------------------ reference ----
def ref_geometry(geo_text, ienv=1, workdir=None):
    """Runs the reference's geoinp()+config() on geo_text; returns the topology arrays
    and the configwire.txt text it wrote."""
    import tempfile
    lib = _load_ref()
    nsmax = lib.ref_nsmax()
    d = workdir or tempfile.mkdtemp(prefix="wmomref_")
    with open(os.path.join(d, "dipol.geo"), "w") as f:
        f.write(geo_text)
    counts = np.zeros(3, np.int32)
    out = dict(x=np.zeros(nsmax, np.float32), y=np.zeros(nsmax, np.float32), z=np.zeros(nsmax, np.float32),
               rad=np.zeros(nsmax, np.float32), ipc=np.zeros(nsmax, np.int32), ips=np.zeros(2 * nsmax, np.int32),
               ise=np.zeros(2 * nsmax, np.int32), isp=np.zeros(2 * nsmax, np.int32),
               iwe=np.zeros(2 * nsmax, np.int32))
    rc = lib.ref_load_geometry(d.encode(), ienv, _p(counts, _ip), _p(out["x"], _fp), _p(out["y"], _fp),
                               _p(out["z"], _fp), _p(out["rad"], _fp), _p(out["ipc"], _ip), _p(out["ips"], _ip),
                               _p(out["ise"], _ip), _p(out["isp"], _ip), _p(out["iwe"], _ip))
    if rc != 0:
        raise RuntimeError(f"ref_load_geometry failed ({rc})")
    out.update(npnt=int(counts[0]), npls=int(counts[1]), nseg=int(counts[2]), nsmax=nsmax)
    with open(os.path.join(d, "configwire.txt")) as f:
        out["listing"] = f.read()
    return out


def ref_fill(g, freq_mhz, ienv=1, sgn=(1.0, 1.0, 1.0, 1.0)):
    lib = _load_ref()
    n = int(g["npls"])
    z = np.zeros((n, n), np.complex128, order="F")
    lib.ref_zmatrix(z.ctypes.data_as(_dp), _p(g["x"], _fp), _p(g["y"], _fp), _p(g["z"], _fp), _p(g["ipc"], _ip),
                    _p(g["ips"], _ip), _p(g["ise"], _ip), _p(g["rad"], _fp), n, ka(freq_mhz), int(g["nsmax"]),
                    ienv, sgn[0], sgn[1], sgn[2], sgn[3])
    return z
