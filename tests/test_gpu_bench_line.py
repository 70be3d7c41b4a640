"""bench.py's own line on the GPU: one short run of the default workload prints one JSON
line with the keys of the bench contract, both arms (FP32 value and the tensor-core `tc`
object with its ratio), their FP64 errors within bounds, the e2e and drop-in legs with
their copied bytes, the roofline of the dominant kernel and the clock record."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_default_bench_line(built_lib):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "3", "--warmup", "3",
                        "--no-cpu-baseline"], capture_output=True, text=True, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "roofline", "e2e", "gpu_launches", "clocks",
              "tc", "accuracy", "e2e_dropin"):
        assert k in d, k
    assert d["value"] > 0 and d["unit"] == "conv/s" and d["steps"] == 3 and d["gpu_launches"] > 0
    assert d["roofline"]["bound"] == "hbm" and d["roofline"]["achieved"] > 0 and d["roofline"]["peak"] > 0
    tc = d["tc"]
    assert tc["value"] > 0 and abs(tc["tc_over_fp32"] - tc["value"] / d["value"]) < 1e-3
    assert d["accuracy"]["fp32"]["rel_l2"] < 1e-6 and d["accuracy"]["tc"]["rel_l2"] <= 1e-5
    for e in (d["e2e"], tc["e2e"], d["e2e_dropin"]):
        assert e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    assert d["e2e_dropin"]["pinned_value"] > 0
    assert d["tc"]["device_status"] == 0
