"""The C-ABI library loads without a GPU and exports every entry point the public
headers declare (no compute call is made here)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HDR = os.path.join(ROOT, "include", "wmom.h")
LIB = os.path.join(ROOT, "praca-magisterska_gb300", "libwmom.so")


def _declared():
    text = open(HDR).read()
    return sorted(set(re.findall(r"\b(wmom_[a-z0-9_]+)\s*\(", text)))


def _exports():
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_header_declares_entry_points():
    names = _declared()
    for must in ("wmom_plan_create", "wmom_fill", "wmom_zgetrf", "wmom_zgetrs", "wmom_zgesv_like",
                 "wmom_solve_sweep", "wmom_topology_from_geo"):
        assert must in names


def test_library_exports_every_declared_symbol(wmom):
    exp = _exports()
    missing = [n for n in _declared() if n not in exp]
    assert not missing, missing
    lib = ctypes.CDLL(LIB)
    for n in _declared():
        getattr(lib, n)


def _prototypes():
    """name -> number of parameters of every function prototype in wmom.h."""
    text = re.sub(r"/\*.*?\*/", " ", open(HDR).read(), flags=re.S)
    out = {}
    for name, params in re.findall(r"\b(wmom_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        params = params.strip()
        out[name] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_python_bindings_match_header_arity(wmom):
    """Every ctypes binding of the Python package declares as many arguments as the
    header's prototype of the same entry point."""
    protos = _prototypes()
    bound = {}
    for v in vars(wmom).values():
        if isinstance(v, ctypes._CFuncPtr) and v.__name__.startswith("wmom_") and v.argtypes is not None:
            bound[v.__name__] = len(v.argtypes)
    assert len(bound) >= 20
    wrong = {n: (k, protos.get(n)) for n, k in bound.items() if protos.get(n) != k}
    assert not wrong, wrong


def test_dropin_cxx_symbols_have_reference_mangling(wmom):
    # the reference's own declarations mangle to these names (g++ Itanium ABI)
    exp = _exports()
    for sym in ("_Z7zmatrixP7double2PfS1_S1_PiS2_S2_S1_idiiffff",
                "_Z11zmatrix_gpuP7double2PfS1_S1_S1_PiS2_S2_idiiffff",
                "_Z6geoinpiiiRiPfS0_S0_S_PiS0_S1_S_S1_"):
        assert sym in exp, sym
    assert any(s.startswith("_Z6configRi") for s in exp)
    assert any(s.startswith("_Z10configwireRi") for s in exp)


def test_status_strings(wmom):
    for code, name in wmom.STATUS_NAMES.items():
        assert wmom._status_string(code).decode() == name


def test_no_device_calls_fail_cleanly_without_gpu(wmom):
    import torch
    if torch.cuda.is_available():
        pytest.skip("has a GPU")
    topo = wmom.Topology(wmom.geometry.dipole(1.0, 1e-3, 16))
    with pytest.raises(wmom.WmomError) as e:
        wmom.Plan(topo)
    assert e.value.status in (2, 8)


def test_fill_geometries_rejects_bad_arguments(wmom):
    """Argument checks of wmom_fill_geometries come before any device call."""
    import ctypes
    f = wmom._fill_geometries
    ka = (ctypes.c_double * 1)(1.0)
    ptr = (ctypes.c_void_p * 1)(1)
    ld = (ctypes.c_longlong * 1)(4)
    plans = (ctypes.c_void_p * 1)(None)
    assert f(plans, 0, ka, ptr, ld, None) == 1          # count 0
    assert f(None, 1, ka, ptr, ld, None) == 1           # no plan array
    assert f(plans, 1, ka, ptr, ld, None) == 1          # null plan


def test_geometry_batch_and_tuner_queries_reject_bad_arguments(wmom):
    """wmom_factor_geometries checks its arguments before any device call;
    wmom_tuned_config / wmom_tuned_shape report an order that was never tuned (or a
    bad one) as WMOM_ERR_ARG; wmom_padded_order is the size-class ladder."""
    import ctypes
    f = wmom._factor_geometries
    freqs = (ctypes.c_float * 1)(10.0)
    outs = (ctypes.c_void_p * 1)()
    plans = (ctypes.c_void_p * 1)(None)
    assert f(plans, 0, freqs, wmom.MODE_MIXED, outs, None) == 1   # count 0
    assert f(plans, 1, freqs, wmom.MODE_MIXED, None, None) == 1   # no output array
    assert f(plans, 1, freqs, wmom.MODE_MIXED, outs, None) == 1   # null plan
    assert f(plans, 1, freqs, 7, outs, None) == 1                  # unknown mode
    assert wmom.tuned_config(4096, wmom.MODE_MIXED) is None
    assert wmom.tuned_shape(4096, wmom.MODE_MIXED) is None
    assert wmom._tuned_shape(0, wmom.MODE_MIXED, None, None) == 1
    assert wmom._tuned_shape(4096, 5, None, None) == 1
    assert [wmom.padded_order(n) for n in (1, 64, 65, 256, 257, 320, 321, 1000, 4096, 4097)] == \
        [64, 64, 128, 256, 320, 320, 384, 1024, 4096, 5120]


def test_stats_classes_match_library(wmom):
    """The Python names of the stats classes and the library's class count agree
    (wmom_stats_read returns the number of classes and needs no GPU)."""
    import ctypes
    f = wmom._lib.wmom_stats_read
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_int]
    assert f(None, None, None, None, 0) == len(wmom.STAT_CLASSES)
    assert wmom.STAT_CLASSES[8:] == ["emul_gemm", "trsv"]


def test_report_layout_matches_header(wmom):
    """wmom_report: a double, six ints (rel_residual, iterations, fell_back, info,
    status, krylov_steps, tier) and a double (cond1), 40 bytes; the ctypes mirror has
    the same layout."""
    import ctypes
    import re
    from conftest import ROOT
    hdr = open(f"{ROOT}/include/wmom.h").read()
    body = re.search(r"typedef struct wmom_report \{(.*?)\} wmom_report;", hdr, re.S).group(1)
    fields = re.findall(r"^\s*(double|int)\s+(\w+);", body, re.M)
    assert [n for _, n in fields] == [n for n, _ in wmom._Report._fields_]
    assert ctypes.sizeof(wmom._Report) == 40
    assert wmom._Report.cond1.offset == 32
