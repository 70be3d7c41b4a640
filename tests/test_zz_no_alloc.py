"""The no-allocation entry point, convgpu_conv3d_device_noalloc, against the oracle and
against the regular device entry point convgpu_conv3d_device.

It exists for callers that cannot call cudaMalloc: programs whose device memory is
owned by another allocator (a framework's caching allocator, a pool sized once at
start-up) and loops that cannot take the device-wide synchronisation of
cudaMalloc / cudaFree. Its scratch is a fixed 16 MiB array inside the library.

The file sorts last so that a run stopping at the first failure has already run every
other test; it also passes alone in a fresh process, where the no-allocation call is
the first call the library sees.
"""
import ctypes

import numpy as np
import pytest

import convfpga_gb300 as cg
from oracle import conv3d, snr_db

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SNR_DB = 120.0  # the tolerance of every parity test in this suite


def _c64(rng, shape):
    a = np.empty(shape, np.complex64)
    a.real = rng.uniform(-1, 1, shape)
    a.imag = rng.uniform(-1, 1, shape)
    return a


def _run(fn, n, sig, filt, b, flags):
    out = torch.empty_like(sig)
    fn(n, sig, filt, out, b, flags)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _oracle(sig, filt, flags):
    return conv3d(sig, filt, "fp32", normalize=bool(flags & cg.NORMALIZE))


def test_no_alloc_matches_oracle_and_device_entry_point_two_calls(built_lib):
    rng = np.random.default_rng(2024)
    cases = [
        (64, 3, cg.NORMALIZE),                     # shared filter: N^3 scratch
        (32, 4, cg.FILTER_PER_SIGNAL),             # per-signal filters: 4*N^3 scratch
    ]
    for n, b, flags in cases:  # two calls in a row, each checked
        sig_h = _c64(rng, (b, n, n, n))
        filt_h = _c64(rng, (b, n, n, n) if flags & cg.FILTER_PER_SIGNAL else (n, n, n))
        sig, filt = torch.from_numpy(sig_h).cuda(), torch.from_numpy(filt_h).cuda()
        got = _run(cg.conv3d_device_noalloc, n, sig, filt, b, flags)   # before the regular entry point
        assert snr_db(_oracle(sig_h, filt_h, flags), got) > SNR_DB
        ref = _run(cg.conv3d_device, n, sig, filt, b, flags)
        assert snr_db(ref, got) > SNR_DB
    assert cg.device_status() == 0


def test_no_alloc_at_its_scratch_limit(built_lib):
    """A shared 128^3 filter needs exactly 2^21 spectrum values: the whole array."""
    n, b = 128, 2
    assert n ** 3 == cg.NOALLOC_SCRATCH_ELEMS
    rng = np.random.default_rng(7)
    sig_h, filt_h = _c64(rng, (b, n, n, n)), _c64(rng, (n, n, n))
    sig, filt = torch.from_numpy(sig_h).cuda(), torch.from_numpy(filt_h).cuda()
    got = _run(cg.conv3d_device_noalloc, n, sig, filt, b, 0)
    assert snr_db(_oracle(sig_h, filt_h, 0), got) > SNR_DB
    assert cg.device_status() == 0


def test_no_alloc_stale_scratch_from_a_larger_call_is_harmless(built_lib):
    """A per-signal call that fills the array (8 x 64^3 = 2^21 values), then a smaller
    shared-filter call: the second reads only what it wrote itself."""
    rng = np.random.default_rng(11)
    n1, b1 = 64, 8
    s1, f1 = _c64(rng, (b1, n1, n1, n1)), _c64(rng, (b1, n1, n1, n1))
    n2, b2 = 32, 3
    s2, f2 = _c64(rng, (b2, n2, n2, n2)), _c64(rng, (n2, n2, n2))
    g1 = _run(cg.conv3d_device_noalloc, n1, torch.from_numpy(s1).cuda(), torch.from_numpy(f1).cuda(), b1,
              cg.FILTER_PER_SIGNAL)
    g2 = _run(cg.conv3d_device_noalloc, n2, torch.from_numpy(s2).cuda(), torch.from_numpy(f2).cuda(), b2, 0)
    assert snr_db(_oracle(s1, f1, cg.FILTER_PER_SIGNAL), g1) > SNR_DB
    assert snr_db(_oracle(s2, f2, 0), g2) > SNR_DB


@pytest.mark.parametrize("per_signal", [False, True])
def test_no_alloc_with_precomputed_spectra(gpu, per_signal):
    """CONVGPU_FILTER_IS_SPECTRUM: no scratch at all; spectra from the library."""
    rng = np.random.default_rng(5)
    n, b = 32, 3
    sig_h = _c64(rng, (b, n, n, n))
    filt_h = _c64(rng, (b, n, n, n) if per_signal else (n, n, n))
    sig, filt = torch.from_numpy(sig_h).cuda(), torch.from_numpy(filt_h).cuda()
    spec = torch.empty_like(filt)
    cg.filter_spectrum_device(n, filt, spec, b if per_signal else 1)
    flags = cg.FILTER_IS_SPECTRUM | (cg.FILTER_PER_SIGNAL if per_signal else 0)
    got = _run(cg.conv3d_device_noalloc, n, sig, spec, b, flags)
    assert snr_db(_oracle(sig_h, filt_h, cg.FILTER_PER_SIGNAL if per_signal else 0), got) > SNR_DB


def test_no_alloc_in_place(built_lib):
    rng = np.random.default_rng(13)
    n, b = 32, 2
    sig_h, filt_h = _c64(rng, (b, n, n, n)), _c64(rng, (n, n, n))
    buf, filt = torch.from_numpy(sig_h.copy()).cuda(), torch.from_numpy(filt_h).cuda()
    cg.conv3d_device_noalloc(n, buf, filt, buf, b, cg.NORMALIZE)
    torch.cuda.synchronize()
    assert snr_db(_oracle(sig_h, filt_h, cg.NORMALIZE), buf.cpu().numpy()) > SNR_DB


def test_no_alloc_allocates_no_device_memory(built_lib):
    """Device free memory is the same before and after a call. Everything else that could
    take device memory happens before the first reading: the inputs are made (torch's own
    kernels load lazily into device memory on their first use) and a warm-up call of the
    same size loads this library's kernels."""
    rng = np.random.default_rng(17)
    n, b = 64, 4
    sig = torch.from_numpy(_c64(rng, (b, n, n, n))).cuda()
    sig2 = torch.from_numpy(_c64(rng, (b, n, n, n))).cuda()
    filt = torch.from_numpy(_c64(rng, (b, n, n, n))).cuda()
    out = torch.empty_like(sig)
    cg.conv3d_device_noalloc(n, sig, filt, out, b, cg.FILTER_PER_SIGNAL)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    cg.conv3d_device_noalloc(n, sig2, filt, out, b, cg.FILTER_PER_SIGNAL)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_no_alloc_rejects_requests_beyond_its_scratch(built_lib):
    n = 256  # a shared 256^3 filter spectrum needs 16 Mi values > 2 Mi
    # buffers large enough for either request, so a wrong size check could not read out of bounds
    sig = torch.zeros((1, n, n, n), dtype=torch.complex64, device="cuda")
    rc = built_lib.convgpu_conv3d_device_noalloc(n, sig.data_ptr(), sig.data_ptr(), sig.data_ptr(), 1, 0, None)
    assert rc == cg.EINVAL
    assert "scratch" in cg.last_error()
    # per-signal filters: 128^3 x 2 = 4 Mi values > 2 Mi
    rc = built_lib.convgpu_conv3d_device_noalloc(128, sig.data_ptr(), sig.data_ptr(), sig.data_ptr(), 2,
                                                 cg.FILTER_PER_SIGNAL, None)
    assert rc == cg.EINVAL
    assert cg.NOALLOC_SCRATCH_ELEMS == 1 << 21


def test_no_alloc_rejects_unsupported_and_invalid_arguments(built_lib):
    """Argument checks come before any device work, so nothing here launches a kernel."""
    p = ctypes.c_void_p(64)  # never dereferenced: every call below is rejected first
    f = built_lib.convgpu_conv3d_device_noalloc
    assert f(32, p, p, p, 1, cg.TENSOR_SPLIT, None) == cg.EUNSUPPORTED
    assert f(32, p, p, p, 1, cg.FILTER_REAL, None) == cg.EUNSUPPORTED
    assert f(48, p, p, p, 1, 0, None) == cg.EINVAL      # not a power of two
    assert f(1024, p, p, p, 1, 0, None) == cg.EINVAL    # beyond N = 512
    assert f(32, None, p, p, 1, 0, None) == cg.EINVAL   # null signal
    assert f(32, p, p, None, 1, 0, None) == cg.EINVAL   # null output
