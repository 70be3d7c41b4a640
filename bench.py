#!/usr/bin/env python
"""Benchmark: FFT-based 3D convolutions per second on GB300 (one JSON line on rank 0).

Workload (the size the headline metric is quoted on): 4 convolutions of 256^3 complex64
signals (re/im i.i.d. N(0,1)) with per-signal complex64 filters (re/im U[-1,1]), seeded
synthetic data. One step = one batch of 4 convolutions through the library's C ABI.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--path both|fp32|tc]

value      : convolutions/s of the plain FP32 path with inputs resident in HBM
             (convgpu_conv3d_device), all ranks.
tc         : the same K steps on the same inputs through the tensor-core split path
             (CONVGPU_TENSOR_SPLIT, TF32x3 on tcgen05): conv/s, its own roofline and pass
             times, and tc_over_fp32 = its conv/s / the FP32 path's (default --path both).
accuracy   : relative L2 and max-abs error of both paths against an FP64 FFT convolution
             (numpy complex128) of one cube, checked after the timed region.
e2e        : convolutions/s through convgpu_conv3d_host with pinned host buffers; every step
             copies its inputs host->device and its outputs device->host (tc.e2e: the same
             with CONVGPU_TENSOR_SPLIT).
e2e_dropin : a reference caller's call: fpgaf_conv3D_svm_batch on buffers from
             fpgaf_complex_malloc (pageable), 128^3 x 8 with one shared real Gaussian filter.
roofline   : the dominant pass kernel: algorithmic bytes per launch / mean launch time, timed
             with CUDA events on its stream during the timed region, against the measured HBM
             copy bandwidth of MEASURED_PEAKS.json.
cpu_baseline: the CPU FFT convolution (pocketfft complex64, all host threads; FFTW3 is not
             installed) on a bounded sample, rank 0 at N=1 only.
--impl reference: times that CPU implementation alone as the reference arm.
--workload configs / uneven96: the other single-GPU workloads; each line carries a
             cpu_baseline of its own (the same pipeline over the same jobs on the host cores).

Multi-GPU (torchrun, one rank per GPU): every rank convolves its own batch of 4 (independent
convolutions, no collective on the data path); value = all ranks' convolutions / max time.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "3D FFT-conv/s + HBM GB/s at 256^3 c64: TC split vs plain FP32, rel-L2≤1e-5"
N, BATCH = 256, 4
WORKLOAD = "256^3 complex64 x4 convolutions, per-signal filters"


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--path", choices=["both", "fp32", "tc"], default="both",
                   help="both: the FP32 path (value) and the tensor-core split path (tc) on the same inputs")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    p.add_argument("--batch", type=int, default=BATCH, help="cubes per step (profiling runs use 1)")
    p.add_argument("--plan-cache", default=None,
                   help="plan-cache file: loaded instead of autotuning when it exists, written by the "
                        "autotuner otherwise (profiling runs replay the plan of the plain run)")
    p.add_argument("--workload", choices=["c256x4", "uneven96", "configs"], default="c256x4",
                   help="configs: the 64^3 x1, 128^3 x8 and 512^3 x1 workloads on device buffers; "
                        "c256x4: the headline 256^3 x4 workload; uneven96: 96 convolutions of sizes "
                        "32..256 (work-queue launch vs one job at a time)")
    a = p.parse_args()
    a.warmup = max(a.warmup, 3)
    return a


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


PATHS = {"fp32": "plain FP32 passes (autotuned plan)", "tc": "tcgen05 split-TF32 (TF32x3) passes",
         "both": "plain FP32 passes (value) and tcgen05 split-TF32 passes (tc), same inputs"}


def _config(path: str) -> dict:
    return {
        "workload": WORKLOAD,
        "n": N,
        "batch": BATCH,
        "filters": "per-signal",
        "path": PATHS[path],
        "normalised": False,
        "l2": "no flush: each step reads 1 GiB of inputs (> 129 MB L2)",
    }


def _cpu_model() -> str:
    """CPU model name of this host (lscpu), for the CPU baseline's record."""
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.split(":")[0].strip() == "Model name":
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.processor() or platform.machine()


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile

            fd, self.path = tempfile.mkstemp(prefix=f"convgpu_clocks_{self.device}_", suffix=".csv")
            self.fh = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.device)], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        try:
            os.unlink(self.path)
        except OSError:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# --------------------------------------------------------------------------- CPU side
def _cpu_conv_sample(frac: float, sig, filt, workers: int) -> float:
    """Seconds for `frac` of one FFT convolution (filter FFT, signal FFT, multiply,
    inverse FFT) with pocketfft complex64 — the reference CPU path's operations
    (src/fft_conv3D.cpp:137-160) on a slab of planes / columns."""
    import numpy as np
    import scipy.fft as sfft

    from oracle import comp_mult

    n = sig.shape[-1]
    m = max(1, int(round(frac * n)))
    t0 = time.perf_counter()
    if m >= n:
        fs = sfft.fftn(filt, workers=workers)
        ss = sfft.fftn(sig, workers=workers)
        prod = comp_mult(ss, fs)
        sfft.ifftn(prod, norm="forward", workers=workers)
    else:
        for a in (filt, sig):  # same operation count as the full transforms, on m/n of the lines
            b = sfft.fftn(a[:m], axes=(1, 2), workers=workers)
            sfft.fft(a[:, :m, :], axis=0, workers=workers)
        prod = comp_mult(b, b)
        sfft.fftn(prod, axes=(1, 2), workers=workers)
        sfft.fft(sig[:, :m, :], axis=0, workers=workers)
    return time.perf_counter() - t0


def _cpu_inputs():
    import numpy as np

    rng = np.random.default_rng(3)
    sig = np.empty((N, N, N), np.complex64)
    sig.real = rng.standard_normal((N, N, N), dtype=np.float32)
    sig.imag = rng.standard_normal((N, N, N), dtype=np.float32)
    filt = np.empty((N, N, N), np.complex64)
    filt.real = rng.uniform(-1, 1, (N, N, N)).astype(np.float32)
    filt.imag = rng.uniform(-1, 1, (N, N, N)).astype(np.float32)
    return sig, filt


def cpu_baseline(budget_s: float = 20.0) -> dict:
    workers = os.cpu_count() or 1
    sig, filt = _cpu_inputs()
    _cpu_conv_sample(0.25, sig, filt, workers)  # warm-up (plans, page faults)
    t1 = _cpu_conv_sample(1.0, sig, filt, workers)
    reps = max(2, min(5, int(budget_s / max(t1, 1e-3))))
    ts = [t1] + [_cpu_conv_sample(1.0, sig, filt, workers) for _ in range(reps - 1)]
    med = statistics.median(ts)
    return {"value": 1.0 / med, "unit": "conv/s", "cores": workers, "kind": "port", "cpu_model": _cpu_model(),
            "sample": f"median of {len(ts)} single 256^3 convolutions (filter FFT + signal FFT + multiply + "
                      f"inverse FFT, pocketfft complex64, {workers} threads; FFTW3 unavailable - pocketfft "
                      f"stand-in), one of the 4 per step"}


def _cpu_jobs_seconds(jobs, workers: int) -> float:
    """Seconds for the CPU path over `jobs` = [(n, signals, filter per signal)]: one
    forward FFT per distinct filter, then per signal its FFT, the product and the inverse
    FFT (src/fft_conv3D.cpp:50-177), pocketfft complex64. Inputs are U[-1,1] complex64: the
    timing of an FFT does not depend on the values."""
    import numpy as np
    import scipy.fft as sfft

    from oracle import comp_mult

    rng = np.random.default_rng(11)
    tot = 0.0
    for n, count, per_signal in jobs:
        a = rng.uniform(-1, 1, (2, n, n, n)).astype(np.float32)
        x = (a[0] + 1j * a[1]).astype(np.complex64)
        del a
        t0 = time.perf_counter()
        fs = None
        for _ in range(count):
            if fs is None or per_signal:
                fs = sfft.fftn(x, workers=workers)
            ss = sfft.fftn(x, workers=workers)
            sfft.ifftn(comp_mult(ss, fs), norm="forward", workers=workers)
        tot += time.perf_counter() - t0
    return tot


def cpu_configs_baseline(names, budget_s: float = 8.0) -> dict:
    """CPU conv/s of each single-GPU workload on all host threads: 64^3 x1 and 128^3 x8 as
    whole steps (median of up to 5), 512^3 x1 as a slice of one convolution (the same
    transforms on m/512 of the planes and columns, about three seconds) scaled up."""
    workers = os.cpu_count() or 1
    out = {}
    for name in names:
        n, b = {"c64x1": (64, 1), "c128x8": (128, 8), "c512x1": (512, 1)}[name]
        if n <= 256:
            _cpu_jobs_seconds([(n, 1, False)], workers)  # warm-up (plans, page faults)
            t1 = _cpu_jobs_seconds([(n, b, False)], workers)
            reps = max(1, min(5, int(budget_s / max(t1, 1e-3))))
            ts = [t1] + [_cpu_jobs_seconds([(n, b, False)], workers) for _ in range(reps - 1)]
            value = b / statistics.median(ts)
            sample = f"median of {len(ts)} steps of {b} {n}^3 convolution(s) with one shared filter"
        else:
            import numpy as np

            rng = np.random.default_rng(12)
            sig = np.empty((n, n, n), np.complex64)
            sig.real = rng.uniform(-1, 1, (n, n, n)).astype(np.float32)
            sig.imag = 0.0
            filt = sig.copy()
            t = _cpu_conv_sample(1.0 / 64, sig, filt, workers)  # 1/64 of a convolution
            m = max(1, min(n, int(round(n * 3.0 / max(64 * t, 1e-3)))))  # a slice of about 3 s
            t = _cpu_conv_sample(m / n, sig, filt, workers)
            value = (m / n) / t
            sample = f"{m}/{n} of one {n}^3 convolution (filter FFT + signal FFT + multiply + inverse FFT), scaled"
            del sig, filt
        out[name] = {"value": round(value, 3), "unit": "conv/s", "cores": workers, "kind": "port",
                     "sample": sample + f", pocketfft complex64, {workers} threads (FFTW3 unavailable - "
                                        "pocketfft stand-in)"}
    return {"cpu_model": _cpu_model(), "configs": out}


def run_reference(a) -> None:
    rank, world, _ = _dist()
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    sig, filt = _cpu_inputs()
    _cpu_conv_sample(0.25, sig, filt, workers)
    t1 = _cpu_conv_sample(1.0, sig, filt, workers)
    # Each step is one convolution, or a fixed fraction of one when K+W full convolutions
    # would take longer than about three minutes.
    frac = min(1.0, 170.0 / ((a.steps + a.warmup) * t1))
    m = max(1, int(round(frac * N)))
    frac = m / N
    for _ in range(a.warmup):
        _cpu_conv_sample(frac, sig, filt, workers)
    tot = 0.0
    for _ in range(a.steps):
        tot += _cpu_conv_sample(frac, sig, filt, workers)
    conv_s = a.steps * frac / tot
    sample = (f"each step: {'one' if frac >= 1 else f'{m}/{N} of one'} 256^3 convolution with its own filter "
              f"(filter FFT + signal FFT + multiply + inverse FFT), pocketfft complex64, {workers} threads "
              f"(FFTW3 unavailable - pocketfft stand-in for src/fft_conv3D.cpp:50-177)")
    line = {
        "impl": "reference", "metric": METRIC, "value": conv_s, "unit": "conv/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * tot / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": _config("fp32"),
        "cpu_baseline": {"value": conv_s, "unit": "conv/s", "cores": workers, "kind": "port",
                         "cpu_model": _cpu_model(), "sample": sample},
        "e2e": {"value": conv_s, "unit": "conv/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- GPU side
def _roofline(passes: dict, peak: float, peak_kind: str, arm: str = "fp32") -> dict:
    """The dominant pass kernel's algorithmic bytes per launch over its mean launch time."""
    dom_name, dom = max(passes.items(), key=lambda kv: kv[1]["ms"])
    per_launch_bytes = dom["bytes"] / dom["launches"]
    per_launch_s = dom["ms"] / dom["launches"] / 1e3
    achieved = per_launch_bytes / per_launch_s / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": _read_traffic(dom_name if arm == "fp32" else f"{arm}/{dom_name}"),
            "kernel": dom_name if arm == "fp32" else f"{arm}/{dom_name}",
            "bytes_per_launch": per_launch_bytes,
            "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s",
            "share_of_step": round(dom["ms"] / sum(p["ms"] for p in passes.values()), 3)}


def _passes_summary(passes: dict) -> dict:
    return {k: {"ms_per_launch": round(v["ms"] / v["launches"], 4), "launches": v["launches"],
                "gbs": round(v["bytes"] / (v["ms"] / 1e3) / 1e9, 1)} for k, v in passes.items()}


def _time_arm(a, cg, flags, sig, filt, out, stream, world, barrier) -> dict:
    """W warm-up steps, then K timed steps (CUDA events on the launching stream, barrier
    and synchronize on both sides, max over ranks) with per-pass events recorded."""
    import torch

    def step():
        cg.conv3d_device(N, sig, filt, out, BATCH, flags, stream)

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    launches0 = cg.launch_count()
    cg.pass_timing_start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(a.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    launches = cg.launch_count() - launches0
    passes = cg.pass_timing_read()
    cg.pass_timing_stop()
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return {"ms": ms, "passes": passes, "gpu_launches": launches, "status": cg.device_status()}


def _fp64_errors(sig0, filt0, outs: dict) -> dict:
    """Relative L2 and max-abs error of each path's output cube against the same
    convolution in FP64: forward 3D FFTs of signal and filter in complex128, product,
    unnormalised backward 3D FFT (numpy / scipy pocketfft, all host threads)."""
    import numpy as np

    try:
        import scipy.fft as sfft

        kw = {"workers": os.cpu_count() or 1}
    except Exception:  # numpy alone
        sfft, kw = np.fft, {}
    s64 = sfft.fftn(sig0.astype(np.complex128), **kw)
    s64 *= sfft.fftn(filt0.astype(np.complex128), **kw)
    ref = sfft.ifftn(s64, norm="forward", **kw)
    den = float(np.linalg.norm(ref.ravel()))
    res = {}
    for k, o in outs.items():
        d = o.astype(np.complex128) - ref
        res[k] = {"rel_l2": float(np.linalg.norm(d.ravel())) / den, "max_abs": float(np.abs(d).max()),
                  "max_abs_ref": float(np.abs(ref).max())}
    return res


def run_ours(a) -> None:
    import torch

    import convfpga_gb300 as cg

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if not os.path.exists(cg.LIB_PATH):
        from convfpga_gb300 import build

        build.build()
    replay = bool(a.plan_cache) and os.path.exists(a.plan_cache)
    rc = cg.fpga_initialize(f"cuda:{local}", a.plan_cache or "convgpu_plans.json", False)
    if rc != 0:
        raise SystemExit(f"fpga_initialize failed: {rc} {cg.last_error()}")

    global BATCH
    BATCH = a.batch
    # The library's autotuner picks the plan for this size (shape variants, fused x+y
    # pass or not, tensor-core kernel family) on this GPU before anything is timed.
    if not replay:
        cg.autotune([N], write_cache=bool(a.plan_cache))
    plan = {k: cg.plan_variant(N, i) for i, k in enumerate(cg.PLAN_KINDS)}
    g = torch.Generator(device="cuda").manual_seed(1234 + rank)
    shape = (BATCH, N, N, N)
    sig = torch.complex(torch.randn(shape, device="cuda", generator=g),
                        torch.randn(shape, device="cuda", generator=g))
    filt = torch.complex(torch.rand(shape, device="cuda", generator=g) * 2 - 1,
                         torch.rand(shape, device="cuda", generator=g) * 2 - 1)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    arms = ["fp32", "tc"] if a.path == "both" else [a.path]
    flags = {"fp32": cg.FILTER_PER_SIGNAL, "tc": cg.FILTER_PER_SIGNAL | cg.TENSOR_SPLIT}
    outs = {k: torch.empty_like(sig) for k in arms}
    sampler = ClockSampler(local)
    sampler.start()
    res = {k: _time_arm(a, cg, flags[k], sig, filt, outs[k], stream, world, barrier) for k in arms}
    clocks = sampler.stop()

    peak, peak_kind = _peaks()
    model_bytes = BATCH * 136 * N ** 3  # per step: 48 N^3 per filter + 88 N^3 per signal

    def arm_line(k):
        r = res[k]
        ms_step = r["ms"] / a.steps
        return {"value": world * BATCH * a.steps / (r["ms"] / 1e3), "ms_per_step": ms_step,
                "hbm_gbs_model": round(model_bytes / (ms_step / 1e3) / 1e9, 1),
                "roofline": _roofline(r["passes"], peak, peak_kind, k), "passes": _passes_summary(r["passes"]),
                "gpu_launches": r["gpu_launches"], "device_status": r["status"]}

    lines = {k: arm_line(k) for k in arms}
    # cube 0 of each path's last timed step, kept for the accuracy check below
    torch.cuda.synchronize()
    cube0 = {k: outs[k][0].cpu().numpy() for k in arms}
    del outs

    # e2e through the host-buffer C ABI entry point with pinned buffers, per arm; before the
    # accuracy check, whose FP64 transforms keep every host core busy for seconds.
    e2e = {k: (_e2e(a, cg, sig, filt, shape, world, barrier, flags[k]) if not a.no_e2e else None) for k in arms}
    dropin = _e2e_dropin(a, cg, world, barrier) if not a.no_e2e else None

    # Accuracy of both paths on cube 0 of the last timed step, after the timed regions.
    accuracy = None
    if rank == 0:
        accuracy = _fp64_errors(sig[0].cpu().numpy(), filt[0].cpu().numpy(), cube0)
        accuracy["cube"] = "cube 0 of the batch, FP64 reference: numpy/scipy complex128 FFT convolution"

    if rank != 0:
        return
    main = arms[0]
    line = {
        "metric": METRIC, "value": lines[main]["value"], "unit": "conv/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": lines[main]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3" if main == "tc" else "f32",
        "data": "synthetic (seeded torch generator; signals N(0,1), filters U[-1,1])",
        "config": _config(a.path),
        "hbm_gbs_model": lines[main]["hbm_gbs_model"],
        "plan": plan,
        "roofline": lines[main]["roofline"],
        "passes": lines[main]["passes"],
        "e2e": e2e[main],
        "gpu_launches": lines[main]["gpu_launches"],
        "clocks": clocks,
        "accuracy": accuracy,
        "e2e_dropin": dropin,
    }
    if "tc" in arms and main != "tc":
        tc = dict(lines["tc"])
        tc["dtype"] = "tf32x3"
        tc["e2e"] = e2e["tc"]
        tc["tc_over_fp32"] = round(tc["value"] / lines[main]["value"], 4)
        line["tc"] = tc
    if world == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line), flush=True)


def _e2e(a, cg, sig, filt, shape, world, barrier, e2e_flags):
    import torch

    vol = BATCH * N ** 3
    hs = cg.PinnedBuffer.alloc(vol * 8)
    hf = cg.PinnedBuffer.alloc(vol * 8)
    ho = cg.PinnedBuffer.alloc(vol * 8)
    sig_h, filt_h, out_h = hs.array(shape), hf.array(shape), ho.array(shape)
    sig_h[...] = sig.cpu().numpy()
    filt_h[...] = filt.cpu().numpy()
    for _ in range(3):
        t = cg.conv3d_host(N, hs.ptr, hf.ptr, ho.ptr, BATCH, e2e_flags)
        assert t.valid, cg.last_error()
    # 60 calls (~0.4 s at 256^3 x 4), or K when K is larger: long enough that a brief
    # stall of the shared host link weighs little in the total
    e2e_steps = max(60, a.steps)
    barrier()
    # Python's collector stays off while the calls are timed: a collection pass between two
    # calls is host work of this script, not of the library.
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    ok = True
    call_s = []
    slowest = None
    for _ in range(e2e_steps):
        tc0 = time.perf_counter()
        t = cg.conv3d_host(N, hs.ptr, hf.ptr, ho.ptr, BATCH, e2e_flags)
        call_s.append(time.perf_counter() - tc0)
        ok = ok and t.valid
        if call_s[-1] == max(call_s):
            slowest = t.as_dict()
    e2e_s = time.perf_counter() - t0
    gc.enable()
    assert ok, cg.last_error()
    if world > 1:
        import torch.distributed as dist

        tt = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e = {"value": world * BATCH * e2e_steps / e2e_s, "unit": "conv/s",
           "h2d_bytes_per_step": 2 * vol * 8, "d2h_bytes_per_step": vol * 8,
           "api": "convgpu_conv3d_host (pinned host buffers)"
                  + (", CONVGPU_TENSOR_SPLIT" if e2e_flags & cg.TENSOR_SPLIT else ""),
           # the spread of the timed calls (the value above is their total): on a shared
           # machine a few calls can wait on the host link
           "call_ms": {"min": round(1e3 * min(call_s), 3), "median": round(1e3 * statistics.median(call_s), 3),
                       "max": round(1e3 * max(call_s), 3), "slowest_call": call_s.index(max(call_s))},
           # the library's own event timings of the slowest call (copies, compute): a stall
           # outside them was on the host side of the call
           "slowest_call_ms": {k: round(v, 3) for k, v in slowest.items() if k != "valid"},
           "last_call_ms": {k: round(v, 3) for k, v in t.as_dict().items() if k != "valid"}}
    for b in (hs, hf, ho):
        b.free()
    return e2e


def _e2e_dropin(a, cg, world, barrier) -> dict:
    """What a reference caller gets: src/main.cpp:64-74 of pc2/ConvFPGA allocates its
    buffers with fpgaf_complex_malloc (pageable host memory) and calls
    fpgaf_conv3D_svm_batch. Workload: 128^3 x 8 signals (U[-1,1]) with one shared real
    periodic Gaussian filter (sigma 4) stored as complex with zero imaginary parts, as the
    reference's API takes it. Each call copies 8 signals and the filter up and 8 outputs
    down; the library transforms the filter on every call, as the reference does."""
    import numpy as np
    import torch

    n, b = 128, 8
    vol = n ** 3
    hs, hf, ho = (cg.ComplexMalloc.alloc(c * vol * 8) for c in (b, 1, b))
    rng = np.random.default_rng(7)
    sa, fa = hs.array((b, n, n, n)), hf.array((n, n, n))
    sa.real = rng.uniform(-1, 1, (b, n, n, n)).astype(np.float32)
    sa.imag = rng.uniform(-1, 1, (b, n, n, n)).astype(np.float32)
    d = np.minimum(np.arange(n), n - np.arange(n)).astype(np.float64) ** 2
    fa[...] = np.exp(-(d[:, None, None] + d[None, :, None] + d[None, None, :]) / (2 * 16.0)).astype(np.complex64)
    ho.array((b, n, n, n))[...] = 0
    for _ in range(2):
        t = cg.fpgaf_conv3D_svm_batch(n, hs.ptr, hf.ptr, ho.ptr, b)
        assert t.valid, cg.last_error()
    calls = max(30, a.steps)
    barrier()
    call_s = []
    ok = True
    gc.collect()
    gc.disable()
    t0 = time.perf_counter()
    for _ in range(calls):
        tc0 = time.perf_counter()
        t = cg.fpgaf_conv3D_svm_batch(n, hs.ptr, hf.ptr, ho.ptr, b)
        call_s.append(time.perf_counter() - tc0)
        ok = ok and t.valid
    tot = time.perf_counter() - t0
    gc.enable()
    assert ok, cg.last_error()
    if world > 1:
        import torch.distributed as dist

        tt = torch.tensor([tot], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tot = float(tt.item())
    res = {"value": world * b * calls / tot, "unit": "conv/s", "h2d_bytes_per_step": (b + 1) * vol * 8,
           "d2h_bytes_per_step": b * vol * 8,
           "api": "fpgaf_conv3D_svm_batch on fpgaf_complex_malloc buffers (pageable)",
           "workload": "128^3 complex64 x8, one shared real Gaussian filter (sigma 4) as complex",
           "call_ms": {"min": round(1e3 * min(call_s), 3), "median": round(1e3 * statistics.median(call_s), 3),
                       "max": round(1e3 * max(call_s), 3)},
           "last_call_ms": {k: round(v, 3) for k, v in t.as_dict().items() if k != "valid"}}
    # the same call on pinned copies of the buffers (convgpu_host_alloc), for comparison
    ps, pf, po = (cg.PinnedBuffer.alloc(c * vol * 8) for c in (b, 1, b))
    ps.array((b, n, n, n))[...] = sa
    pf.array((n, n, n))[...] = fa
    for _ in range(2):
        assert cg.fpgaf_conv3D_svm_batch(n, ps.ptr, pf.ptr, po.ptr, b).valid, cg.last_error()
    t0 = time.perf_counter()
    for _ in range(calls):
        assert cg.fpgaf_conv3D_svm_batch(n, ps.ptr, pf.ptr, po.ptr, b).valid, cg.last_error()
    res["pinned_value"] = b * calls / (time.perf_counter() - t0)
    for h in (hs, hf, ho, ps, pf, po):
        h.free()
    return res


def run_uneven(a) -> None:
    """96 convolutions with sizes drawn (seed 4) from {32,64,128,256} with p = {.4,.3,.2,.1},
    complex64 signals U[-1,1] and real Gaussian filters (sigma U[1,8]) - the same draw as the
    oracle's generator. One step = all 96 convolutions."""
    import numpy as np
    import torch

    import convfpga_gb300 as cg

    torch.cuda.set_device(0)
    if not os.path.exists(cg.LIB_PATH):
        from convfpga_gb300 import build

        build.build()
    rc = cg.fpga_initialize("cuda:0", "convgpu_plans.json", False)
    if rc != 0:
        raise SystemExit(f"fpga_initialize failed: {rc} {cg.last_error()}")
    sizes = [int(v) for v in np.random.default_rng(4).choice([32, 64, 128, 256], size=96, p=[.4, .3, .2, .1])]
    # autotuned plan per size (shape variants; fused x+y for the 256^3 jobs), outside the timing
    cg.autotune(sorted(set(sizes)), write_cache=False)
    offs = np.cumsum([0] + [n ** 3 for n in sizes])
    total = int(offs[-1])
    g = torch.Generator(device="cuda").manual_seed(99)
    sig = torch.complex(torch.rand(total, device="cuda", generator=g) * 2 - 1,
                        torch.rand(total, device="cuda", generator=g) * 2 - 1)
    filt = torch.empty(total, dtype=torch.complex64, device="cuda")
    sigmas = np.random.default_rng(5).uniform(1.0, 8.0, size=len(sizes))
    for i, n in enumerate(sizes):
        d = torch.arange(n, device="cuda", dtype=torch.float64)
        d = torch.minimum(d, n - d)
        g1 = torch.exp(-0.5 * (d / sigmas[i]) ** 2)
        gg = (g1[:, None, None] * g1[None, :, None] * g1[None, None, :]).to(torch.float32)
        filt[offs[i]:offs[i + 1]] = torch.complex(gg, torch.zeros_like(gg)).reshape(-1)
    out = torch.empty_like(sig)
    jobs = [(n, int(offs[i]), int(offs[i]), int(offs[i])) for i, n in enumerate(sizes)]
    stream = torch.cuda.current_stream()

    def timed(flags):
        for _ in range(a.warmup):
            cg.conv3d_uneven_device(jobs, sig, filt, out, flags, stream)
        torch.cuda.synchronize()
        l0 = cg.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            cg.conv3d_uneven_device(jobs, sig, filt, out, flags, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / a.steps, cg.launch_count() - l0

    sampler = ClockSampler(0)
    sampler.start()
    ms_g, launches_g = timed(0)
    clocks = sampler.stop()
    ms_q, launches_q = timed(cg.UNEVEN_QUEUE)
    ms_j, launches_j = timed(cg.UNEVEN_PER_JOB)
    status = cg.device_status()
    model = sum(136 * n ** 3 for n in sizes)
    line = {
        "metric": "3D FFT-conv/s, uneven batch of 96 (sizes 32..256), per-size launches in one CUDA graph",
        "value": len(sizes) / (ms_g / 1e3), "unit": "conv/s", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_g, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": "uneven96: 96 convolutions, sizes from {32,64,128,256} p={.4,.3,.2,.1} (seed 4), "
                               "real Gaussian filters sigma U[1,8]",
                   "size_counts": {str(n): sizes.count(n) for n in (32, 64, 128, 256)},
                   "l2": f"no flush: each step reads {2 * total * 8 / 2**30:.2f} GiB of inputs (> 129 MB L2)"},
        "hbm_gbs_model": round(model / (ms_g / 1e3) / 1e9, 1),
        "work_queue": {"value": len(sizes) / (ms_q / 1e3), "ms_per_step": ms_q,
                       "gpu_launches_per_step": launches_q / a.steps},
        "per_job": {"value": len(sizes) / (ms_j / 1e3), "ms_per_step": ms_j, "gpu_launches_per_step": launches_j / a.steps},
        "speedup_vs_per_job": ms_j / ms_g,
        "plan": {str(n): {k: cg.plan_variant(n, i) for i, k in enumerate(cg.PLAN_KINDS)} for n in sorted(set(sizes))},
        "gpu_launches": launches_g, "device_status": status, "clocks": clocks,
    }
    if not a.no_cpu_baseline:  # the same 96 convolutions on the host cores
        workers = os.cpu_count() or 1
        _cpu_jobs_seconds([(n, 1, True) for n in sorted(set(sizes))], workers)  # warm-up
        t = _cpu_jobs_seconds([(n, 1, True) for n in sizes], workers)
        line["cpu_baseline"] = {"value": round(len(sizes) / t, 3), "unit": "conv/s", "cores": workers, "kind": "port",
                                "cpu_model": _cpu_model(),
                                "sample": f"one pass over the 96 convolutions, each with its own filter "
                                          f"(filter FFT + signal FFT + multiply + inverse FFT), pocketfft "
                                          f"complex64, {workers} threads (FFTW3 unavailable - pocketfft stand-in)"}
    print(json.dumps(line), flush=True)


def run_configs(a) -> None:
    """The other single-GPU workloads, timed on device buffers (K steps after W warm-up
    steps, CUDA events): 64^3 x1 (signal and filter U[-1,1], normalised), 128^3 x8 (shared
    real periodic Gaussian filter, sigma 4) and 512^3 x1 (shared real periodic Gaussian
    filter, sigma 6), the last on both the FP32 and the tensor-core split path. The real
    filters are passed as floats (CONVGPU_FILTER_REAL). Inputs are generated on the device
    with the workloads' shapes; for timing, the 512^3 signal is U[-1,1] noise instead of
    the workload's sum of Gaussian blobs."""
    import torch

    import convfpga_gb300 as cg

    torch.cuda.set_device(0)
    if not os.path.exists(cg.LIB_PATH):
        from convfpga_gb300 import build

        build.build()
    replay = bool(a.plan_cache) and os.path.exists(a.plan_cache)
    rc = cg.fpga_initialize("cuda:0", a.plan_cache or "convgpu_plans.json", False)
    if rc != 0:
        raise SystemExit(f"fpga_initialize failed: {rc} {cg.last_error()}")
    if not replay:  # the plans of all three sizes, before anything is timed
        cg.autotune([64, 128, 512], write_cache=bool(a.plan_cache))
    g = torch.Generator(device="cuda").manual_seed(99)

    def uni(shape):
        return torch.complex(torch.rand(shape, device="cuda", generator=g) * 2 - 1,
                             torch.rand(shape, device="cuda", generator=g) * 2 - 1)

    def gauss(n, sigma):
        i = torch.arange(n, device="cuda", dtype=torch.float32)
        d = torch.minimum(i, n - i) ** 2
        r2 = d[:, None, None] + d[None, :, None] + d[None, None, :]
        return torch.exp(-r2 / (2.0 * sigma * sigma)).contiguous()

    results = {}
    for name, n, b in (("c64x1", 64, 1), ("c128x8", 128, 8), ("c512x1", 512, 1), ("c512x1_tc", 512, 1)):
        sig = uni((b, n, n, n))
        if name == "c64x1":
            filt, flags = uni((n, n, n)), cg.NORMALIZE
        else:
            filt, flags = gauss(n, 4.0 if n == 128 else 6.0), cg.FILTER_REAL | cg.NORMALIZE
        if name == "c512x1_tc":
            flags |= cg.TENSOR_SPLIT  # the tcgen05 split-TF32 kernels of N = 512
        out = torch.empty_like(sig)
        steps = max(3, a.steps if n < 512 else min(a.steps, 20))
        for _ in range(a.warmup):
            cg.conv3d_device(n, sig, filt, out, b, flags)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            cg.conv3d_device(n, sig, filt, out, b, flags)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        model = (48 + 88 * b) * n ** 3  # one shared filter + b signals, per-axis pass model
        results[name] = {"conv_per_s": round(b / (ms / 1e3), 1), "ms_per_step": round(ms, 4),
                         "model_gbs": round(model / (ms / 1e3) / 1e9, 1), "steps": steps,
                         "filter": "complex U[-1,1]" if name == "c64x1" else "real Gaussian (FILTER_REAL)",
                         "path": "tcgen05 split-TF32" if flags & cg.TENSOR_SPLIT else "plain FP32",
                         "plan": {k: cg.plan_variant(n, i) for i, k in enumerate(cg.PLAN_KINDS)}}
        del sig, filt, out
        torch.cuda.empty_cache()
    status = cg.device_status()
    line = {"metric": "3D FFT-conv/s per workload (64^3 x1, 128^3 x8, 512^3 x1), device buffers",
            "value": results["c128x8"]["conv_per_s"], "unit": "conv/s", "n_gpus": 1, "steps": a.steps,
            "warmup": a.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded torch generator)", "config": {"workload": "configs", "value_of": "c128x8"},
            "configs": results, "device_status": status}
    if not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_configs_baseline(["c64x1", "c128x8", "c512x1"])
    print(json.dumps(line), flush=True)


def _read_traffic(kernel: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary, if any
    (keys of the tensor-core path's kernels start with "tc/")."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            d = json.load(f)
        return d.get(kernel)
    except Exception:
        return None


def main():
    a = _args()
    if a.workload == "uneven96" and a.impl == "ours":
        run_uneven(a)
        return
    if a.workload == "configs" and a.impl == "ours":
        run_configs(a)
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
