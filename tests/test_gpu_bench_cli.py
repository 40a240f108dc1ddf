"""bench.py's workloads end to end on the GPU at reduced sizes: each prints
one JSON line with the contract's keys (the full-size runs take minutes)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "clocks", "roofline"}


def _run(args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_fullband_reduced():
    d = _run(["--workload", "fullband", "--steps", "2", "--warmup", "3", "--no-cpu", "--nsub", "8",
              "--tdms", "64", "--chunk", "4096"])
    assert KEYS <= set(d) and d["value"] > 0 and d["e2e"]["value"] > 0
    assert "reduced" in d["config"]["workload"]


def test_batch_reduced_with_parity():
    d = _run(["--beams", "3", "--chunk", "1024", "--steps", "2", "--warmup", "3", "--no-cpu", "--no-serve",
              "--variant", "7"])
    assert KEYS <= set(d) and d["value"] > 0 and d["e2e"]["value"] > 0
    assert d["parity"]["identical"] == d["parity"]["windows_compared"] > 0
    assert d["roofline"]["kernel"] == "dedisperse_pair_kernel"
