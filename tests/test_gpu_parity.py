"""GPU parity of the plain FP32 path, through the C ABI, against the oracle.

Criterion: the reference's own, SNR > 120 dB (relative L2 < 1e-6) against the FP32
pipeline of src/fft_conv3D.cpp:186-258 (src/fft_conv3D.cpp:236-258), and against the
golden vectors of the reference's FFT engine. Full-size workloads are also checked
against the FP64 oracle and through size-independent properties.
"""
import os

import numpy as np
import pytest

from oracle import conv3d, gaussian_filter, make_config, max_abs, rel_l2, snr_db

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GOLD = os.path.join(os.path.dirname(__file__), "golden")
SNR_DB = 120.0


def _c64(rng, shape):
    a = np.empty(shape, np.complex64)
    a.real = rng.uniform(-1, 1, shape)
    a.imag = rng.uniform(-1, 1, shape)
    return a


def dev_conv(cg, sig, filt, flags=0, inplace=False):
    n = sig.shape[-1]
    b = sig.shape[0]
    s = torch.from_numpy(np.ascontiguousarray(sig)).cuda()
    f = torch.from_numpy(np.ascontiguousarray(filt)).cuda()
    o = s if inplace else torch.empty_like(s)
    cg.conv3d_device(n, s, f, o, b, flags)
    torch.cuda.synchronize()
    return o.cpu().numpy()


@pytest.mark.parametrize("name", ["conv16x3", "conv16x2pf", "conv32x1"])
def test_golden_reference_engine(gpu, name):
    d = np.load(os.path.join(GOLD, f"{name}.npz"))
    flags = gpu.FILTER_PER_SIGNAL if d["filt"].ndim == 4 else 0
    out = dev_conv(gpu, d["sig"], d["filt"], flags)
    assert snr_db(d["out"], out) > SNR_DB


def test_golden_64_workload(gpu):
    d = np.load(os.path.join(GOLD, "conv64x1.npz"))
    sig, filt, _ = make_config("c64x1")
    out = dev_conv(gpu, sig, filt)
    assert snr_db(d["out"], out) > SNR_DB


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256])
@pytest.mark.parametrize("per_signal", [False, True])
def test_sizes_against_fp32_oracle(gpu, n, per_signal):
    rng = np.random.default_rng(n + 7 * per_signal)
    b = 2 if n <= 128 else 1
    sig = _c64(rng, (b, n, n, n))
    filt = _c64(rng, (b, n, n, n)) if per_signal else _c64(rng, (n, n, n))
    out = dev_conv(gpu, sig, filt, gpu.FILTER_PER_SIGNAL if per_signal else 0)
    ref = conv3d(sig, filt, "fp32", engine="pocketfft")
    assert snr_db(ref, out) > SNR_DB
    ref64 = conv3d(sig, filt, "fp64", engine="pocketfft")
    assert rel_l2(ref64, out) < 1e-6


@pytest.mark.parametrize("n", [16, 32])
@pytest.mark.parametrize("flags", ["shared", "per_signal", "normalize"])
def test_small_cubes_elementwise_against_fp64(gpu, n, flags):
    """Every output value, not only the relative L2 norm: |out - ref| <= 1e-5 * max |ref| for
    every element against the FP64 oracle (FP32 rounding of a 16- or 32-point transform
    per axis is ~1e-7 relative to the largest value)."""
    rng = np.random.default_rng(31 * n + len(flags))
    b = 3
    sig = _c64(rng, (b, n, n, n))
    per_signal = flags == "per_signal"
    filt = _c64(rng, (b, n, n, n) if per_signal else (n, n, n))
    f = (gpu.FILTER_PER_SIGNAL if per_signal else 0) | (gpu.NORMALIZE if flags == "normalize" else 0)
    out = dev_conv(gpu, sig, filt, f)
    ref = conv3d(sig, filt, "fp64", normalize=flags == "normalize", engine="pocketfft")
    err = np.abs(out.astype(np.complex128) - ref)
    assert err.max() <= 1e-5 * np.abs(ref).max(), (err.max(), np.abs(ref).max())
    assert gpu.device_status() == 0


@pytest.mark.parametrize("n", [32, 256])
@pytest.mark.parametrize("how_many", [1, 2, 3])
def test_shared_filter_batches_against_fp32_oracle(gpu, full_spectra, n, how_many):
    """A shared filter with one or two signals has its z transform fused into the signals'
    z pass; from three signals on it gets a pass of its own. Both routes, complex and real
    filters (the real one, as a full spectrum, bit-identical to the same filter given as
    complex)."""
    rng = np.random.default_rng(100 * how_many + n)
    sig = _c64(rng, (how_many, n, n, n))
    filt = _c64(rng, (n, n, n))
    out = dev_conv(gpu, sig, filt)
    ref = conv3d(sig, filt, "fp32", engine="pocketfft")
    assert snr_db(ref, out) > SNR_DB
    g = gaussian_filter(n, 3.0)
    out_c = dev_conv(gpu, sig, g)
    s = torch.from_numpy(sig).cuda()
    fr = torch.from_numpy(np.ascontiguousarray(g.real)).cuda()
    o = torch.empty_like(s)
    gpu.conv3d_device(n, s, fr, o, how_many, gpu.FILTER_REAL)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(o.cpu().numpy(), out_c)
    assert snr_db(conv3d(sig, g, "fp32", engine="pocketfft"), out_c) > SNR_DB
    assert gpu.device_status() == 0


@pytest.mark.parametrize("n", [16, 32, 64])
@pytest.mark.parametrize("per_signal", [False, True])
def test_single_small_cube_one_launch(gpu, n, per_signal):
    """One cube of N <= 64 runs as a single cooperative launch (the seven passes with grid
    barriers between their dependency levels): the reference's criterion against the FP32
    oracle, normalised and in place, one launch counted, device status clean."""
    rng = np.random.default_rng(900 + n + per_signal)
    sig = _c64(rng, (1, n, n, n))
    filt = _c64(rng, (1, n, n, n) if per_signal else (n, n, n))
    flags = gpu.FILTER_PER_SIGNAL if per_signal else 0
    l0 = gpu.launch_count()
    out = dev_conv(gpu, sig, filt, flags)
    assert gpu.launch_count() - l0 == 1
    assert snr_db(conv3d(sig, filt, "fp32", engine="pocketfft"), out) > SNR_DB
    outn = dev_conv(gpu, sig, filt, flags | gpu.NORMALIZE, inplace=True)
    np.testing.assert_allclose(outn, out / n ** 3, rtol=0, atol=1e-6 * np.abs(out).max() / n ** 3)
    for _ in range(3):  # repeated launches reuse the barrier-slot ring
        again = dev_conv(gpu, sig, filt, flags)
    np.testing.assert_array_equal(again, out)
    assert gpu.device_status() == 0


@pytest.mark.slow
def test_512_against_fp32_oracle(gpu):
    rng = np.random.default_rng(512)
    n = 512
    sig = _c64(rng, (1, n, n, n))
    filt = gaussian_filter(n, 6.0)
    out = dev_conv(gpu, sig, filt)
    ref = conv3d(sig, filt, "fp32", engine="pocketfft")
    assert snr_db(ref, out) > SNR_DB


def test_normalise_and_inplace(gpu):
    rng = np.random.default_rng(3)
    n = 64
    sig = _c64(rng, (3, n, n, n))
    filt = _c64(rng, (n, n, n))
    ref = conv3d(sig, filt, "fp32", normalize=True, engine="pocketfft")
    out = dev_conv(gpu, sig, filt, gpu.NORMALIZE, inplace=True)
    assert snr_db(ref, out) > SNR_DB


def test_filter_spectrum_reuse(gpu):
    rng = np.random.default_rng(4)
    n = 32
    sig = _c64(rng, (2, n, n, n))
    filt = _c64(rng, (n, n, n))
    f = torch.from_numpy(filt).cuda()
    spec = torch.empty_like(f)
    gpu.filter_spectrum_device(n, f, spec, 1)
    torch.cuda.synchronize()
    spec_ref = np.fft.fftn(filt.astype(np.complex128))
    assert rel_l2(spec_ref, spec.cpu().numpy()) < 1e-6
    out = dev_conv(gpu, sig, spec.cpu().numpy(), gpu.FILTER_IS_SPECTRUM)
    assert snr_db(conv3d(sig, filt, "fp32", engine="pocketfft"), out) > SNR_DB


@pytest.mark.parametrize("fn", ["fpgaf_conv3D", "fpgaf_conv3D_svm"])
def test_reference_host_entry_points(gpu, fn):
    rng = np.random.default_rng(5)
    n = 64
    sig = _c64(rng, (n, n, n))
    filt = _c64(rng, (n, n, n))
    out = np.zeros_like(sig)
    t = getattr(gpu, fn)(n, sig, filt, out)
    assert t.valid, gpu.last_error()
    assert t.filter_exec_t > 0 and t.sig_exec_t > 0 and t.sig_pcie_wr_t > 0 and t.sig_pcie_rd_t > 0
    assert snr_db(conv3d(sig, filt, "fp32", engine="pocketfft"), out) > SNR_DB


@pytest.mark.parametrize("how_many", [1, 3, 4])
def test_batch_entry_point_any_count_distinct_signals(gpu, how_many):
    """Odd counts and distinct signals per slot (the reference breaks on both:
    host/src/convfpga_svm_batch.c:302, 579-648; src/helper.cpp:159-171)."""
    rng = np.random.default_rng(6 + how_many)
    n = 32
    sig = _c64(rng, (how_many, n, n, n))
    filt = _c64(rng, (n, n, n))
    out = np.zeros_like(sig)
    t = gpu.fpgaf_conv3D_svm_batch(n, sig, filt, out, how_many)
    assert t.valid, gpu.last_error()
    ref = conv3d(sig, filt, "fp32", engine="pocketfft")
    for i in range(how_many):
        assert snr_db(ref[i], out[i]) > SNR_DB


def test_host_batch_chunked_per_signal(gpu):
    """More signals than one 64 MiB chunk: exercises the 3-buffer copy/compute pipeline."""
    rng = np.random.default_rng(8)
    n, b = 128, 7
    sig = _c64(rng, (b, n, n, n))
    filt = _c64(rng, (b, n, n, n))
    out = np.zeros_like(sig)
    t = gpu.conv3d_host(n, sig, filt, out, b, gpu.FILTER_PER_SIGNAL | gpu.NORMALIZE)
    assert t.valid, gpu.last_error()
    ref = conv3d(sig, filt, "fp32", normalize=True, engine="pocketfft")
    assert snr_db(ref, out) > SNR_DB


@pytest.mark.parametrize("slabs", [False, True], ids=["whole", "slabs"])
def test_host_filter_spectrum_cache(gpu, slabs):
    """CONVGPU_FILTER_CACHED: the second call with the same shared filter pointer reuses the
    kept spectrum (no filter copy or transform, bit-identical output); a filter changed in
    place is not seen while the flag promises it is unchanged; a call without the flag
    transforms it again and drops the kept spectrum."""
    rng = np.random.default_rng(21)
    n, b = (256, 2) if slabs else (64, 3)  # the slab pipeline takes cubes of 32 MiB and more
    extra = gpu.HOST_SLABS if slabs else 0
    sig = _c64(rng, (b, n, n, n))
    filt = _c64(rng, (n, n, n))
    filt2 = _c64(rng, (n, n, n))
    outs = []
    times = []
    for _ in range(2):
        out = np.zeros_like(sig)
        t = gpu.conv3d_host(n, sig, filt, out, b, gpu.FILTER_CACHED | extra)
        assert t.valid, gpu.last_error()
        outs.append(out)
        times.append(t)
    assert snr_db(conv3d(sig, filt, "fp32", engine="pocketfft"), outs[0]) > SNR_DB
    np.testing.assert_array_equal(outs[0], outs[1])
    assert times[0].filter_exec_t > 0.0 and times[1].filter_exec_t == 0.0
    assert times[1].filter_pcie_wr_t == 0.0
    filt[...] = filt2  # same pointer, new contents: the promise is broken on purpose
    stale = np.zeros_like(sig)
    assert gpu.conv3d_host(n, sig, filt, stale, b, gpu.FILTER_CACHED | extra).valid
    np.testing.assert_array_equal(stale, outs[0])
    fresh = np.zeros_like(sig)
    assert gpu.conv3d_host(n, sig, filt, fresh, b, extra).valid  # no flag: transformed again
    assert snr_db(conv3d(sig, filt2, "fp32", engine="pocketfft"), fresh) > SNR_DB
    again = np.zeros_like(sig)
    t = gpu.conv3d_host(n, sig, filt, again, b, gpu.FILTER_CACHED | extra)
    assert t.valid and t.filter_exec_t > 0.0  # the unflagged call dropped the kept spectrum
    np.testing.assert_array_equal(again, fresh)
    assert gpu.device_status() == 0


def test_uneven_jobs(gpu):
    rng = np.random.default_rng(9)
    sizes = [32, 64, 16, 128, 32]
    sigs = [_c64(rng, (n, n, n)) for n in sizes]
    filts = [gaussian_filter(n, 2.0 + i) for i, n in enumerate(sizes)]
    offs = np.cumsum([0] + [n ** 3 for n in sizes])
    s = torch.from_numpy(np.concatenate([x.ravel() for x in sigs])).cuda()
    f = torch.from_numpy(np.concatenate([x.ravel() for x in filts])).cuda()
    o = torch.empty_like(s)
    jobs = [(n, int(offs[i]), int(offs[i]), int(offs[i])) for i, n in enumerate(sizes)]
    gpu.conv3d_uneven_device(jobs, s, f, o, gpu.NORMALIZE)
    torch.cuda.synchronize()
    oh = o.cpu().numpy()
    for i, n in enumerate(sizes):
        ref = conv3d(sigs[i], filts[i], "fp32", normalize=True, engine="pocketfft")
        got = oh[offs[i]:offs[i + 1]].reshape(n, n, n)
        assert snr_db(ref, got) > SNR_DB


@pytest.mark.slow
def test_full_size_256x4_against_fp64(gpu):
    sig, filt, _ = make_config("c256x4")
    out = dev_conv(gpu, sig, filt, gpu.FILTER_PER_SIGNAL | gpu.NORMALIZE)
    ref = conv3d(sig[:1], filt[:1], "fp64", normalize=True, engine="pocketfft")
    assert rel_l2(ref, out[:1]) < 1e-6
    assert max_abs(ref, out[:1]) < 1e-5 * np.abs(ref).max()


@pytest.mark.slow
@pytest.mark.parametrize("n", [256, 512])
def test_full_size_properties(gpu, n):
    """Size-independent checks at the full cube sizes: a shifted delta filter is a
    circular shift (exact up to rounding), and the operator is linear."""
    rng = np.random.default_rng(n)
    sig = np.empty((1, n, n, n), np.complex64)
    sig.real = rng.standard_normal((1, n, n, n), dtype=np.float32)
    sig.imag = rng.standard_normal((1, n, n, n), dtype=np.float32)
    delta = np.zeros((n, n, n), np.complex64)
    delta[3, 5, 7] = 1.0
    out = dev_conv(gpu, sig, delta, gpu.NORMALIZE)
    shifted = np.roll(sig, shift=(3, 5, 7), axis=(1, 2, 3))
    assert rel_l2(shifted, out) < 1e-6
    if n == 256:
        g = gaussian_filter(n, 4.0)
        a = dev_conv(gpu, sig, g, gpu.NORMALIZE)
        b = dev_conv(gpu, 2.0 * sig, g, gpu.NORMALIZE)
        assert rel_l2(2.0 * a, b) < 1e-6


@pytest.mark.parametrize("n", [32, 128])
def test_unaligned_pointers_use_gather_kernels(gpu, n):
    """8-byte aligned (not 16) operands cannot be described by TMA tensor maps; the
    register-gather y / z kernels take over and give the same results."""
    rng = np.random.default_rng(n + 11)
    b = 2
    sig = _c64(rng, (b, n, n, n))
    filt = _c64(rng, (b, n, n, n))
    vol = b * n ** 3
    s_buf = torch.empty(vol + 1, dtype=torch.complex64, device="cuda")
    f_buf = torch.empty(vol + 1, dtype=torch.complex64, device="cuda")
    o_buf = torch.empty(vol + 1, dtype=torch.complex64, device="cuda")
    s, f, o = s_buf[1:], f_buf[1:], o_buf[1:]
    assert s.data_ptr() % 16 == 8
    s.copy_(torch.from_numpy(sig.ravel()))
    f.copy_(torch.from_numpy(filt.ravel()))
    gpu.conv3d_device(n, s, f, o, b, gpu.FILTER_PER_SIGNAL)
    torch.cuda.synchronize()
    out = o.cpu().numpy().reshape(b, n, n, n)
    assert snr_db(conv3d(sig, filt, "fp32", engine="pocketfft"), out) > SNR_DB


def test_device_status_clean(gpu):
    """No kernel gave up a bounded wait during the tests above."""
    assert gpu.device_status() == 0


def _uneven_inputs(sizes, seed):
    rng = np.random.default_rng(seed)
    sigs = [_c64(rng, (n, n, n)) for n in sizes]
    filts = [gaussian_filter(n, float(rng.uniform(1.0, 8.0))) for n in sizes]
    offs = np.cumsum([0] + [n ** 3 for n in sizes])
    return sigs, filts, offs


@pytest.mark.parametrize("mode", ["grouped", "queue", "per_job"])
def test_uneven_config_sizes_queue_and_replay(gpu, mode):
    """The uneven workload's size mix (drawn from {32,64,128,256}), first 20 jobs; the
    grouped and work-queue launches are replayed from their cached CUDA graphs with new
    data (new buffers, so the grouped plan re-encodes its tensor maps)."""
    from oracle import uneven_sizes

    sizes = uneven_sizes()[:20]
    flags = gpu.NORMALIZE | {"grouped": 0, "queue": gpu.UNEVEN_QUEUE, "per_job": gpu.UNEVEN_PER_JOB}[mode]
    for rep in range(2):
        sigs, filts, offs = _uneven_inputs(sizes, 100 + rep)
        s = torch.from_numpy(np.concatenate([x.ravel() for x in sigs])).cuda()
        f = torch.from_numpy(np.concatenate([x.ravel() for x in filts])).cuda()
        o = torch.empty_like(s)
        jobs = [(n, int(offs[i]), int(offs[i]), int(offs[i])) for i, n in enumerate(sizes)]
        gpu.conv3d_uneven_device(jobs, s, f, o, flags)
        torch.cuda.synchronize()
        oh = o.cpu().numpy()
        for i, n in enumerate(sizes):
            ref = conv3d(sigs[i], filts[i], "fp32", normalize=True, engine="pocketfft")
            assert snr_db(ref, oh[offs[i]:offs[i + 1]].reshape(n, n, n)) > SNR_DB, (i, n)
    assert gpu.device_status() == 0


def test_uneven_in_place_and_distinct_offsets(gpu):
    """Jobs whose signal, filter and output live at unrelated offsets, outputs in place."""
    rng = np.random.default_rng(77)
    sizes = [64, 32, 128, 64]
    sigs, filts, offs = _uneven_inputs(sizes, 78)
    total = int(offs[-1])
    s = torch.from_numpy(np.concatenate([x.ravel() for x in sigs])).cuda()
    f_perm = list(reversed(range(len(sizes))))
    f_offs, pos = {}, 0
    for i in f_perm:
        f_offs[i] = pos
        pos += sizes[i] ** 3
    f = torch.from_numpy(np.concatenate([filts[i].ravel() for i in f_perm])).cuda()
    jobs = [(n, int(offs[i]), f_offs[i], int(offs[i])) for i, n in enumerate(sizes)]
    gpu.conv3d_uneven_device(jobs, s, f, s, 0)
    torch.cuda.synchronize()
    oh = s.cpu().numpy()
    assert oh.size == total
    for i, n in enumerate(sizes):
        ref = conv3d(sigs[i], filts[i], "fp32", engine="pocketfft")
        assert snr_db(ref, oh[offs[i]:offs[i + 1]].reshape(n, n, n)) > SNR_DB


@pytest.mark.parametrize("per_signal,b,slabs", [(True, 4, True), (False, 2, True), (True, 4, False)])
def test_host_pipelines_256(gpu, per_signal, b, slabs):
    """256^3 cubes through the host pipelines: whole-cube chunks (default) and, with
    CONVGPU_HOST_SLABS, z-slab streaming (x / y passes per slab as it lands, fused z per
    cube, inverse per slab, slab downloads); 4 cubes wrap the 3-buffer ring."""
    rng = np.random.default_rng(256 + b)
    n = 256
    sig = _c64(rng, (b, n, n, n))
    filt = _c64(rng, (b, n, n, n)) if per_signal else _c64(rng, (n, n, n))
    out = np.zeros_like(sig)
    extra = gpu.HOST_SLABS if slabs else 0
    if per_signal:
        t = gpu.conv3d_host(n, sig, filt, out, b, gpu.FILTER_PER_SIGNAL | gpu.NORMALIZE | extra)
        ref = conv3d(sig, filt, "fp32", normalize=True, engine="pocketfft")
    else:
        t = gpu.conv3d_host(n, sig, filt, out, b, extra)
        ref = conv3d(sig, filt, "fp32", engine="pocketfft")
    assert t.valid, gpu.last_error()
    assert t.sig_pcie_wr_t > 0 and t.sig_pcie_rd_t > 0 and t.sig_exec_t > 0
    for i in range(b):
        assert snr_db(ref[i], out[i]) > SNR_DB


@pytest.mark.slow
def test_host_slab_pipeline_512(gpu):
    rng = np.random.default_rng(5120)
    n = 512
    sig = _c64(rng, (1, n, n, n))
    filt = gaussian_filter(n, 6.0)
    out = np.zeros_like(sig)
    t = gpu.conv3d_host(n, sig, filt, out, 1, gpu.HOST_SLABS)
    assert t.valid, gpu.last_error()
    assert snr_db(conv3d(sig, filt, "fp32", engine="pocketfft"), out) > SNR_DB


def _real(rng, shape):
    return rng.uniform(-1, 1, shape).astype(np.float32)


@pytest.fixture
def full_spectra(gpu):
    """Real filters as full spectra (plan kind 7 = 0), whatever an earlier autotune chose."""
    keep = {n: gpu.plan_variant(n, 7) for n in (64, 128, 256, 512)}
    for n in keep:
        gpu.plan_variant(n, 7, 0)
    yield
    for n, v in keep.items():
        gpu.plan_variant(n, 7, v)


@pytest.mark.parametrize("n,per_signal", [(32, False), (64, True), (128, False), (256, True)])
def test_real_filters_device(gpu, full_spectra, n, per_signal):
    """CONVGPU_FILTER_REAL on device buffers with full spectra: the same result, bit for
    bit, as the complex filter with zero imaginary parts (the real x pass uses the same
    radix plan and exchange order), and within the reference's SNR criterion of the FP32
    oracle."""
    rng = np.random.default_rng(n + per_signal)
    b = 2
    sig = _c64(rng, (b, n, n, n))
    filt = _real(rng, (b, n, n, n) if per_signal else (n, n, n))
    flags = gpu.FILTER_PER_SIGNAL if per_signal else 0
    s = torch.from_numpy(sig).cuda()
    fr = torch.from_numpy(filt).cuda()
    fc = torch.from_numpy(filt.astype(np.complex64)).cuda()
    o_real = torch.empty_like(s)
    o_cplx = torch.empty_like(s)
    gpu.conv3d_device(n, s, fr, o_real, b, flags | gpu.FILTER_REAL)
    gpu.conv3d_device(n, s, fc, o_cplx, b, flags)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(o_real.cpu().numpy(), o_cplx.cpu().numpy())
    if n <= 64:
        ref = conv3d(sig, filt.astype(np.complex64), "fp32", engine="pocketfft")
        assert snr_db(ref, o_real.cpu().numpy()) > SNR_DB
    assert gpu.device_status() == 0


@pytest.mark.parametrize("per_signal", [False, True])
def test_real_filters_host(gpu, full_spectra, per_signal):
    """CONVGPU_FILTER_REAL through the host entry point (float filters on the host, half
    the filter upload): equal to the complex-filter call."""
    rng = np.random.default_rng(40 + per_signal)
    n, b = 64, 5
    sig = _c64(rng, (b, n, n, n))
    filt = _real(rng, (b, n, n, n) if per_signal else (n, n, n))
    flags = gpu.FILTER_PER_SIGNAL if per_signal else 0
    out_r = np.zeros_like(sig)
    out_c = np.zeros_like(sig)
    assert gpu.conv3d_host(n, sig, filt, out_r, b, flags | gpu.FILTER_REAL).valid, gpu.last_error()
    assert gpu.conv3d_host(n, sig, filt.astype(np.complex64), out_c, b, flags).valid, gpu.last_error()
    np.testing.assert_array_equal(out_r, out_c)


def test_real_filters_rejected_where_unsupported(gpu):
    n = 32
    s = torch.zeros((1, n, n, n), dtype=torch.complex64, device="cuda")
    f = torch.zeros((n, n, n), dtype=torch.float32, device="cuda")
    with pytest.raises(gpu.ConvGpuError):
        gpu.conv3d_device(n, s, f, s, 1, gpu.FILTER_REAL | gpu.FILTER_IS_SPECTRUM)
    with pytest.raises(gpu.ConvGpuError):
        gpu.conv3d_uneven_device([(n, 0, 0, 0)], s, f, s, gpu.FILTER_REAL)


@pytest.mark.parametrize("offset", [0, 8])
def test_host_pageable_and_pinned_buffers_agree(gpu, offset):
    """The host entry point issues the downloads into a pageable output buffer (numpy,
    fpgaf_complex_malloc) from a second thread, since such a copy returns only when it has
    completed, and keeps pinned buffers on the calling thread. Pageable buffers (also at an
    8-byte offset) and pinned ones give the same bits, and the oracle's result."""
    rng = np.random.default_rng(91 + offset)
    n, b = 64, 3
    count = b * n ** 3
    raw = np.zeros(2 * count + 2, np.complex64)  # pageable, misaligned by `offset` bytes when asked
    sig = raw[offset // 8: offset // 8 + count].reshape(b, n, n, n)
    sig[...] = _c64(rng, (b, n, n, n))
    filt = _c64(rng, (n, n, n))
    out_pageable = np.zeros_like(sig)
    t = gpu.fpgaf_conv3D_svm_batch(n, sig, filt, out_pageable, b)
    assert t.valid, gpu.last_error()
    ps, pf, po = (gpu.PinnedBuffer.alloc(c * 8) for c in (count, n ** 3, count))
    try:
        ps.array(sig.shape)[...] = sig
        pf.array(filt.shape)[...] = filt
        t = gpu.fpgaf_conv3D_svm_batch(n, ps.ptr, pf.ptr, po.ptr, b)
        assert t.valid, gpu.last_error()
        np.testing.assert_array_equal(out_pageable, po.array(sig.shape))
    finally:
        for h in (ps, pf, po):
            h.free()
    assert snr_db(conv3d(sig, filt, "fp32"), out_pageable) > SNR_DB
