"""Accuracy of each of the five workloads at full size against the FP64 oracle.

The oracle is the same pipeline in complex128 (pocketfft). Each case prints one line:
workload, path, relative L2 error, max-abs error, and max |reference|.
  - FP32 path: rel-L2 < 1e-6 (the reference's 120 dB criterion, src/fft_conv3D.cpp:236-258)
    and max-abs < 1e-5 * max |reference|.
  - Tensor-core split path (CONVGPU_TENSOR_SPLIT, TF32x3): rel-L2 <= 1e-5 at 256^3 and 512^3,
    both of which have tensor-core kernels (the result differs from the FP32 path's).
  - The workloads with real Gaussian filters (128^3 x8, the uneven batch, 512^3 x1) also
    through Hermitian half spectra (plan kind 7 = 1): FP32 bounds as above.
Inputs are the workloads' seeded synthetic cubes (oracle.make_config), with the
workloads' options: 64^3 normalised by 1/N^3, shared real Gaussian filters passed as real
(CONVGPU_FILTER_REAL), per-signal filters at 256^3, one filter per job in the uneven batch.
"""
import numpy as np
import pytest

from oracle import conv3d, make_config, max_abs, rel_l2

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
torch = pytest.importorskip("torch")

REL_FP32 = 1e-6
REL_TC = 1e-5


def _report(name, path, ref, out):
    e, m, peak = rel_l2(ref, out), max_abs(ref, out), float(np.abs(ref).max())
    print(f"\n{name} {path}: rel-L2 {e:.3e}, max-abs {m:.3e}, max|ref| {peak:.3e}")
    return e, m, peak


def _device(cg, sig, filt, flags, real):
    n, b = sig.shape[-1], sig.shape[0]
    s = torch.from_numpy(np.ascontiguousarray(sig)).cuda()
    fh = np.ascontiguousarray(filt.real.astype(np.float32)) if real else np.ascontiguousarray(filt)
    f = torch.from_numpy(fh).cuda()
    o = torch.empty_like(s)
    cg.conv3d_device(n, s, f, o, b, flags | (cg.FILTER_REAL if real else 0))
    torch.cuda.synchronize()
    out = o.cpu().numpy()
    del s, f, o
    torch.cuda.empty_cache()
    return out


@pytest.fixture
def half_spectra(gpu):
    keep = {n: gpu.plan_variant(n, 7) for n in (64, 128, 256, 512)}
    for n in keep:
        gpu.plan_variant(n, 7, 1)
    yield
    for n, v in keep.items():
        gpu.plan_variant(n, 7, v)


@pytest.mark.parametrize("name", ["c128x8", "c512x1"])
def test_real_filter_workloads_half_spectra_against_fp64(gpu, half_spectra, name):
    sig, filt, _ = make_config(name)
    ref = conv3d(sig, filt, "fp64", engine="pocketfft")
    out = _device(gpu, sig, filt, 0, True)
    e, m, peak = _report(name, "fp32 half spectrum", ref, out)
    assert e < REL_FP32
    assert m < 1e-5 * peak
    assert gpu.device_status() == 0


def test_uneven_workload_real_filters_half_spectra_against_fp64(gpu, half_spectra):
    """The 96-job batch with its real Gaussian filters passed as floats, one job at a time
    (CONVGPU_UNEVEN_PER_JOB): jobs of 64^3 and up use half spectra."""
    sigs, filts, _ = make_config("uneven96")
    sizes = [s.shape[0] for s in sigs]
    offs = np.cumsum([0] + [n ** 3 for n in sizes])
    s = torch.from_numpy(np.concatenate([x.ravel() for x in sigs])).cuda()
    f = torch.from_numpy(np.concatenate([x.real.astype(np.float32).ravel() for x in filts])).cuda()
    o = torch.empty_like(s)
    jobs = [(n, int(offs[i]), int(offs[i]), int(offs[i])) for i, n in enumerate(sizes)]
    gpu.conv3d_uneven_device(jobs, s, f, o, gpu.NORMALIZE | gpu.FILTER_REAL | gpu.UNEVEN_PER_JOB)
    torch.cuda.synchronize()
    out = o.cpu().numpy()
    refs = [conv3d(sigs[i], filts[i], "fp64", normalize=True, engine="pocketfft").ravel() for i in range(len(sizes))]
    worst = max(rel_l2(refs[i], out[offs[i]:offs[i + 1]]) for i in range(len(sizes)))
    e, m, peak = _report("uneven96", "fp32 half spectrum (per job)", np.concatenate(refs), out)
    print(f"uneven96 half spectrum: worst job rel-L2 {worst:.3e}")
    assert e < REL_FP32 and worst < REL_FP32
    assert gpu.device_status() == 0


@pytest.mark.parametrize("name", ["c64x1", "c128x8", "c256x4", "c512x1"])
def test_uniform_workloads_against_fp64(gpu, name):
    sig, filt, shared = make_config(name)
    norm = name == "c64x1"
    real = shared and name != "c64x1"  # the real Gaussian filters
    flags = (gpu.NORMALIZE if norm else 0) | (0 if shared else gpu.FILTER_PER_SIGNAL)
    ref = conv3d(sig, filt, "fp64", normalize=norm, engine="pocketfft")
    out = _device(gpu, sig, filt, flags, real)
    e, m, peak = _report(name, "fp32", ref, out)
    assert e < REL_FP32
    assert m < 1e-5 * peak
    if name in ("c256x4", "c512x1"):
        tc = _device(gpu, sig, filt, flags | gpu.TENSOR_SPLIT, real)
        e_tc, _, _ = _report(name, "tf32x3", ref, tc)
        assert e_tc <= REL_TC
        assert not np.array_equal(tc, out)  # the tensor-core kernels ran
    assert gpu.device_status() == 0


def test_uneven_workload_against_fp64(gpu):
    """All 96 jobs in one grouped call; the error of the whole batch and the worst job."""
    sigs, filts, _ = make_config("uneven96")
    sizes = [s.shape[0] for s in sigs]
    offs = np.cumsum([0] + [n ** 3 for n in sizes])
    s = torch.from_numpy(np.concatenate([x.ravel() for x in sigs])).cuda()
    f = torch.from_numpy(np.concatenate([x.ravel() for x in filts])).cuda()
    o = torch.empty_like(s)
    jobs = [(n, int(offs[i]), int(offs[i]), int(offs[i])) for i, n in enumerate(sizes)]
    gpu.conv3d_uneven_device(jobs, s, f, o, gpu.NORMALIZE)
    torch.cuda.synchronize()
    out = o.cpu().numpy()
    refs = [conv3d(sigs[i], filts[i], "fp64", normalize=True, engine="pocketfft").ravel() for i in range(len(sizes))]
    worst = max(rel_l2(refs[i], out[offs[i]:offs[i + 1]]) for i in range(len(sizes)))
    ref = np.concatenate(refs)
    e, m, peak = _report("uneven96", "fp32", ref, out)
    print(f"uneven96 fp32: worst job rel-L2 {worst:.3e}")
    assert e < REL_FP32 and worst < REL_FP32
    assert m < 1e-5 * peak
    assert gpu.device_status() == 0
