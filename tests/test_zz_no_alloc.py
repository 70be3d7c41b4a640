"""The no-allocation entry point, convgpu_conv3d_device_noalloc, against the regular
device entry point convgpu_conv3d_device.

It exists for callers that cannot call cudaMalloc: programs whose device memory is
owned by another allocator (a framework's caching allocator, a pool sized once at
start-up) and loops that cannot take the device-wide synchronisation of
cudaMalloc / cudaFree. Its scratch is a fixed 16 MiB array inside the library.

The file sorts last so that a run stopping at the first failure has already run every
other test; it also passes alone in a fresh process, where the no-allocation call is
the first call the library sees.
"""
import numpy as np
import pytest

import convfpga_gb300 as cg
from oracle import snr_db

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


def test_no_alloc_matches_device_entry_point_two_calls(built_lib):
    rng = np.random.default_rng(2024)
    cases = [
        (64, 3, cg.NORMALIZE),                     # shared filter: N^3 scratch
        (32, 4, cg.FILTER_PER_SIGNAL),             # per-signal filters: 4*N^3 scratch
    ]
    for n, b, flags in cases:  # two calls in a row, each checked
        sig = torch.from_numpy(_c64(rng, (b, n, n, n))).cuda()
        fshape = (b, n, n, n) if flags & cg.FILTER_PER_SIGNAL else (n, n, n)
        filt = torch.from_numpy(_c64(rng, fshape)).cuda()
        got = _run(cg.conv3d_device_noalloc, n, sig, filt, b, flags)   # before the regular entry point
        ref = _run(cg.conv3d_device, n, sig, filt, b, flags)
        assert snr_db(ref, got) > SNR_DB


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
