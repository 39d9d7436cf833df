"""Seeded synthetic wire geometries written as .geo text (the reference's input
format, read by geoinp(), "wersja referencyjna/Configuration.cpp":5-75):

    <comment line>
    <comment line>
    nnod
    x y z                  (nnod lines, metres)
    nw
    n1 n2 radius nsegments (nw lines, 1-based node numbers)
    nt                     (patch count, 0)

Values are written with 9 significant digits so that parsing them back as float32
is exact.  None of these geometries comes from a dataset: they are the synthetic
workloads of the solver's benchmark configurations.
"""
import math

import numpy as np


def _f(v):
    return "%.9g" % float(np.float32(v))


def geo_text(nodes, wires, comment="wmom synthetic geometry"):
    lines = [comment, "", str(len(nodes))]
    for x, y, z in nodes:
        lines.append(f"{_f(x)}\t{_f(y)}\t{_f(z)}")
    lines.append(str(len(wires)))
    for n1, n2, a, ns in wires:
        lines.append(f"{int(n1)}\t{int(n2)}\t{_f(a)}\t{int(ns)}")
    lines.append("0")
    return "\n".join(lines) + "\n"


def dipole(length=1.0, radius=1e-3, nsw=512, z0=None):
    """Straight dipole along z centred at the origin (npls = nsw - 1 unknowns).  The
    reference's own test deck is dipole(25.0, 5e-4, nsw) (dipol.geo)."""
    h = length / 2.0
    zs = -h if z0 is None else z0
    nodes = [(0.0, 0.0, zs), (0.0, 0.0, zs + length)]
    return geo_text(nodes, [(1, 2, radius, nsw)], "Dipole")


def grid(n_per_side=21, pitch=1.0, height=1.0, radius=5e-3, segments=None, ns_default=1):
    """Rectangular wire grid (n_per_side x n_per_side nodes at height z), horizontal
    wires row by row, then vertical wires.  `segments` is the per-wire segment count
    list (length 2*n*(n-1)); with the reference's junction rule the unknown count is
    sum(ns - 1) + (2*n_wires - n_nodes)."""
    n = n_per_side
    nodes = []
    for j in range(n):
        for i in range(n):
            nodes.append((i * pitch, j * pitch, height))
    wires = []
    for j in range(n):
        for i in range(n - 1):
            wires.append([j * n + i + 1, j * n + i + 2])
    for i in range(n):
        for j in range(n - 1):
            wires.append([j * n + i + 1, (j + 1) * n + i + 1])
    if segments is None:
        segments = [ns_default] * len(wires)
    assert len(segments) == len(wires)
    return geo_text(nodes, [(a, b, radius, ns) for (a, b), ns in zip(wires, segments)], "Grid")


def grid_segments_for(n_unknowns, n_per_side=21):
    """Per-wire segment counts giving exactly n_unknowns on the grid: the first k
    wires get s+1 segments and the rest s (s, k chosen so the total matches)."""
    n = n_per_side
    nwires = 2 * n * (n - 1)
    junction = 2 * nwires - n * n
    interior = n_unknowns - junction
    if interior < 0:
        raise ValueError("too few unknowns for this grid")
    s = interior // nwires      # every wire has s interior functions -> s+1 segments
    k = interior - s * nwires   # the first k wires get one more
    return [s + 2 if w < k else s + 1 for w in range(nwires)]


def precision_grid(n_unknowns=8192):
    """20 x 20 m grid, 1 m pitch, radius 5 mm, at z = 1 m, with n_unknowns unknowns."""
    return grid(21, 1.0, 1.0, 5e-3, grid_segments_for(n_unknowns, 21))


def random_wires(n_unknowns, seed=20261203, fmax_mhz=10.0, n_wires=None, cube=20.0):
    """Seeded random straight wires: first endpoint uniform in a `cube`-metre cube,
    direction uniform on the sphere, length U(0.5, 5) m (redrawn if the wire leaves
    the cube), radius U(1, 10) mm; segment counts proportional to length, at least
    ceil(L / (lambda_min / 10)), summing to exactly n_unknowns unknowns (wires do not
    touch, so each wire contributes nsw - 1)."""
    rng = np.random.default_rng(seed)
    if n_wires is None:
        n_wires = int(min(1500, max(4, n_unknowns // 64)))
    lam_min = 2.99792458e8 / (fmax_mhz * 1e6)
    ends = []
    lengths = []
    for _ in range(n_wires):
        while True:
            p0 = rng.uniform(0.0, cube, 3)
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            L = rng.uniform(0.5, 5.0)
            p1 = p0 + L * d
            if np.all(p1 >= 0.0) and np.all(p1 <= cube):
                break
        ends.append((p0, p1))
        lengths.append(L)
    radii = rng.uniform(1e-3, 10e-3, n_wires)
    lengths = np.array(lengths)
    nmin = np.maximum(2, np.ceil(lengths / (lam_min / 10.0)).astype(int))  # segments
    need = n_unknowns + n_wires  # sum of segment counts
    if nmin.sum() > need:
        raise ValueError("too many wires for this unknown count")
    share = lengths / lengths.sum() * need
    ns = np.maximum(nmin, np.floor(share).astype(int))
    # largest remainders first until the total is exact
    while ns.sum() < need:
        rem = share - ns
        ns[int(np.argmax(rem))] += 1
    while ns.sum() > need:
        cand = np.where(ns > nmin)[0]
        ns[cand[int(np.argmax(ns[cand] - share[cand]))]] -= 1
    nodes = []
    wires = []
    for w, ((p0, p1), a) in enumerate(zip(ends, radii)):
        nodes.append(tuple(p0))
        nodes.append(tuple(p1))
        wires.append((2 * w + 1, 2 * w + 2, a, int(ns[w])))
    return geo_text(nodes, wires, "Random wires")


def log_freqs(fmin_mhz, fmax_mhz, n):
    """n log-spaced float32 frequencies in MHz."""
    if n == 1:
        return np.array([fmin_mhz], np.float32)
    k = np.arange(n)
    return (10.0 ** (math.log10(fmin_mhz) + (math.log10(fmax_mhz) - math.log10(fmin_mhz)) * k / (n - 1))).astype(
        np.float32)


def sweep_freqs():
    """12 frequencies log-spaced 10 kHz - 10 MHz: f_k = 10^(-2 + 3k/11) MHz."""
    return log_freqs(0.01, 10.0, 12)
