"""The `convolution` sample application (flags and flow of the reference's
src/main.cpp + src/helper.cpp) run as a subprocess."""
import os
import subprocess

import pytest

import convfpga_gb300 as cg
from convfpga_gb300 import build

APP = build.APP


@pytest.fixture(scope="module")
def app(built_lib):
    build.build_app()
    assert os.path.exists(APP)
    return APP


def _run(app, *args, timeout=300):
    return subprocess.run([app, *args], capture_output=True, text=True, timeout=timeout)


def test_help(app):
    r = _run(app, "--help")
    assert r.returncode == 0 and "--cpu-only" in r.stdout


def test_cpu_only(app):
    r = _run(app, "-c", "-n", "16", "-i", "2", "-t", "2")
    assert r.returncode == 0, r.stderr
    assert "Conv3D Runtime" in r.stdout


def test_bitstream_path_required(app):
    r = _run(app, "-n", "16")
    assert r.returncode == 1 and "path" in r.stdout


def test_bad_option(app):
    assert _run(app, "--bogus").returncode == 1


@pytest.mark.gpu
@pytest.mark.parametrize("args", [
    ["-n", "32", "-i", "3"],                    # fpgaf_conv3D
    ["-n", "64", "-s"],                         # fpgaf_conv3D_svm
    ["-n", "32", "-s", "-b", "3", "-i", "2"],   # fpgaf_conv3D_svm_batch, odd batch
    ["-n", "16", "-b", "2", "-t", "4"],         # non-SVM batch through convgpu_conv3d_host
])
def test_gpu_runs_verify(app, args):
    r = _run(app, "-p", "convgpu_plans.json", *args)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "verified" in r.stdout and "Measurements in ms" in r.stdout


@pytest.mark.gpu
def test_gpu_autotune_writes_the_plan_cache(app, tmp_path):
    """-a tunes the plan for N and writes it to the -p file (the wisdom-file analogue); a
    second run reads it back."""
    import json

    path = str(tmp_path / "plans.json")
    r = _run(app, "-p", path, "-n", "32", "-a")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "tuned and written" in r.stdout and "verified" in r.stdout
    plans = json.load(open(path))
    assert "32" in plans["sizes"]
    r = _run(app, "-p", path, "-n", "32")
    assert r.returncode == 0, r.stdout + r.stderr
