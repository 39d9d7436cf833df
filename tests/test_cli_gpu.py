"""The command-line driver (the reference program's inputs and outputs) and lumped
loads, on the GPU."""
import importlib
import io
import json
import math
import os
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


def test_driver_reproduces_reference_run(cuda, wmom, tmp_path):
    # the reference's own deck: 25 m dipole, 512 segments, gap 100, six frequencies
    (tmp_path / "dipol.geo").write_text(wmom.geometry.dipole(25.0, 5e-4, 512))
    (tmp_path / "freq.txt").write_text("6\n" + "\n".join("%.8e" % f for f in (100, 200, 300, 400, 500, 600)) + "\n")
    main = importlib.import_module("praca-magisterska_gb300.wmom_main")
    out = io.StringIO()
    with redirect_stdout(out):
        assert main.main(["--dir", str(tmp_path)]) == 0
    lines = [l for l in out.getvalue().splitlines() if "Freq =" in l]
    with open(os.path.join(GOLDEN, "zin_logs.json")) as f:
        logs = {r["freq"]: r for r in json.load(f) if r["nsw"] == 512 and r["file"] == "results_1_6_512.txt"}
    assert len(lines) == 6
    for line in lines:
        f, re_, im = line.split("Freq = ")[1].split("\t")
        r = logs[float(f)]
        assert (re_, im) == (r["re_text"], r["im_text"]), (line, r)
    assert (tmp_path / "configwire.txt").read_text() == wmom.Topology(wmom.geometry.dipole(25.0, 5e-4, 512)).listing
    d = np.load(os.path.join(GOLDEN, "currents_dipole25m_512.npz"))
    rows = np.loadtxt(tmp_path / "currents.csv", delimiter=",", skiprows=1)
    for k in range(6):
        sel = rows[rows[:, 0] == d["freqs"][k]]
        cur = sel[:, 2] + 1j * sel[:, 3]
        assert np.linalg.norm(cur - d["currents"][k]) / np.linalg.norm(d["currents"][k]) < 1e-10


def test_lumped_loads_match_oracle(cuda, wmom, orc):
    topo = wmom.Topology(wmom.geometry.dipole(2.0, 1e-3, 200))
    loads = [(50, 30.0, 0.0), (120, 1.0, 4.5), (120, 0.5, 0.1)]
    plan = wmom.Plan(topo)
    plan.set_loads(loads)
    freqs = [10.0, 75.0]
    cur, zin, _ = plan.solve(freqs, 100)
    for k, f in enumerate(freqs):
        z = orc.fill(topo.arrays(), f)
        for i, r, l in loads:
            z[i - 1, i - 1] += complex(r, 2 * math.pi * float(np.float32(f)) * l)
        v = orc.excitation(topo.npls, 100)
        i_ref, _ = orc.lu_solve(z, v)
        assert np.linalg.norm(cur[k] - i_ref) / np.linalg.norm(i_ref) < 1e-10
    plan.set_loads([])
    cur0, _, _ = plan.solve(freqs[:1], 100)
    i0, _, _ = orc.solve(topo.arrays(), freqs[0], 100)
    assert np.linalg.norm(cur0[0] - i0) / np.linalg.norm(i0) < 1e-10
    with pytest.raises(wmom.WmomError):
        plan.set_loads([(0, 1.0, 1.0)])
    plan.close()
