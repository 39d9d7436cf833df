"""The JSON line of bench.py's reference arm (the reference's CPU path: oracle fill +
LAPACK) on a small random-wire sweep, run here on the CPU: the keys and values the
bench line promises, warm-up raised to at least 3 steps, and a rank other than 0 of
a multi-rank launch exiting 0 without output."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def _bench(args, env_extra=None):
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    env.update(env_extra or {})
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return [json.loads(l) for l in p.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line():
    (line,) = _bench(["--impl", "reference", "--n", "1024", "--steps", "2", "--warmup", "1"])
    assert line["impl"] == "reference"
    assert line["unit"] == "freq-solves/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 3 and line["n_gpus"] == 1
    assert abs(line["ms_per_step"] - 1e3 / line["value"]) <= 1e-6 * line["ms_per_step"]
    assert line["config"]["unknowns"] == 1024 and line["config"]["frequencies"] == 12
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["unit"] == line["unit"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["vs_baseline"] is None


def test_reference_arm_other_ranks_print_nothing():
    out = _bench(["--impl", "reference", "--n", "1024", "--steps", "1", "--gpus", "2"],
                 {"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert out == []
