"""bench.py end to end on a small workload: the process exits 0 and prints
one JSON line with every key the measurement contract needs."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def _run(*args, timeout=600):
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                         timeout=timeout, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-4000:]
    lines = [l for l in res.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, res.stdout[-2000:]
    return json.loads(lines[0])


def test_bench_line_has_the_contract_keys():
    line = _run("--workload", "poisson2d_p1_256", "--steps", "3", "--warmup", "3")
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "clocks",
                "gpu_launches", "p50_ms", "p99_ms"):
        assert key in line, key
    assert line["value"] > 0 and line["n_gpus"] == 1 and line["steps"] == 3
    assert line["gpu_launches"] > 0
    for key in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert key in line["e2e"]
    assert line["e2e"]["h2d_bytes_per_step"] > 0 and line["e2e"]["d2h_bytes_per_step"] > 0
    for key in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert key in line["roofline"]
    assert 0 < line["roofline"]["frac"] < 2
    for key in ("value", "unit", "cores", "kind", "sample"):
        assert key in line["cpu_baseline"]
    assert line["rel_err_vs_fp64"] <= 1e-8
