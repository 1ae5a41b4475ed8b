"""The benchmark's default path end to end, on a small flux grid.

Runs `bench.py` with every part of its default line enabled (the plain FP64
drop-in sample, the FP64 batch, the large-sector kernels of the 4x6
checkerboard and 4x4 Hubbard sectors, and a short served stream) and checks
that it prints one JSON line with the keys of the benchmark contract.  Only the
twist grid, the step counts and the served stream's length are reduced.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_default_line_has_every_key():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--twist-grid", "2", "--steps", "1", "--warmup", "3",
           "--plain-sample", "2", "--cpu-sample", "1", "--extras-served-n", "24"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-3000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "e2e", "roofline", "cpu_baseline", "gpu_launches", "clocks",
              "launch_shape", "fp64_batched", "plain_fp64_dropin", "kernels", "served"):
        assert k in d, k
    assert d["value"] > 0 and d["e2e"]["value"] > 0 and d["gpu_launches"] >= 1
    assert d["fp64_batched"]["launch_shape"]["krylovdim"] > 0
    assert d["roofline"]["frac"] > 0 and d["cpu_baseline"]["value"] > 0
    assert d["max_rel_dE_mixed_vs_fp64"] <= 1e-9
    assert set(d["kernels"]) and all(v for v in d["kernels"].values())
    served = d["served"]
    assert served["served"]["n"] == 24 and not served["unconverged"] and not served["errors"]
    assert served["max_rel_dE_vs_plain_fp64"] <= 1e-9
