"""bench.py's reference arm (the CPU implementation of the path, timed on the host cores):
one short run on CPU, and the JSON line it prints carries the keys of the bench contract."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["unit"] == "conv/s" and line["higher_is_better"] is True
    assert line["n_gpus"] == 1 and line["steps"] == 1
    assert line["warmup"] == 3  # fewer warm-up steps than 3 are raised to 3
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "sample" in cb and cb["cpu_model"]
    assert line["e2e"] == {"value": line["value"], "unit": "conv/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "workload" in line["config"]


def test_cpu_baselines_of_the_other_workloads():
    """The CPU rates that `--workload configs` and `--workload uneven96` report beside their
    GPU numbers: the same pipeline over the same job list (small sizes here)."""
    sys.path.insert(0, ROOT)
    import bench

    t = bench._cpu_jobs_seconds([(16, 2, False), (32, 1, True)], 2)
    assert t > 0
    r = bench.cpu_configs_baseline(["c64x1"], budget_s=0.5)
    c = r["configs"]["c64x1"]
    assert r["cpu_model"] and c["value"] > 0 and c["unit"] == "conv/s" and c["kind"] == "port"
    assert c["cores"] >= 1 and "pocketfft" in c["sample"]
