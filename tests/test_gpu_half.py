"""Hermitian half spectra of real filters (CONVGPU_FILTER_REAL with plan kind 7 = 1).

A real filter's spectrum obeys F(kx, ky, kz) = conj(F(N-kx, N-ky, N-kz)); the library keeps
kx < N/2 + 16 only and its fused z pass serves a column tile and its mirror from one read
of that half. The reference always transforms and multiplies full complex spectra
(src/fft_conv3D.cpp:95-99, 222-231), so the check is the reference's own criterion: the
result within 1e-6 relative L2 (120 dB) of the same convolution in FP64, on every route
(shared filter with its own z pass, per-signal filters, host buffers), and different bits
from the full-spectrum route (the half-spectrum kernels ran).
"""
import numpy as np
import pytest

from oracle import conv3d, rel_l2

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERM = 7
REL = 1e-6


@pytest.fixture
def herm(gpu):
    keep = {n: gpu.plan_variant(n, HERM) for n in (64, 128, 256, 512)}

    def use(v):
        for n in keep:
            gpu.plan_variant(n, HERM, v)

    yield use
    for n, v in keep.items():
        gpu.plan_variant(n, HERM, v)


def _c64(rng, shape):
    a = np.empty(shape, np.complex64)
    a.real = rng.uniform(-1, 1, shape)
    a.imag = rng.uniform(-1, 1, shape)
    return a


def _device(cg, sig, filt, b, flags):
    s = torch.from_numpy(sig).cuda()
    f = torch.from_numpy(np.ascontiguousarray(filt)).cuda()
    o = torch.empty_like(s)
    cg.conv3d_device(sig.shape[-1], s, f, o, b, flags | cg.FILTER_REAL)
    torch.cuda.synchronize()
    return o.cpu().numpy()


@pytest.mark.parametrize("n,b,per_signal", [(64, 2, False), (128, 3, False), (128, 1, False), (128, 2, True),
                                            (256, 3, False), (256, 2, True)])
def test_half_spectra_against_fp64(gpu, herm, n, b, per_signal):
    rng = np.random.default_rng(n * 10 + b + per_signal)
    sig = _c64(rng, (b, n, n, n))
    filt = rng.uniform(-1, 1, (b, n, n, n) if per_signal else (n, n, n)).astype(np.float32)
    flags = gpu.FILTER_PER_SIGNAL if per_signal else 0
    herm(1)
    half = _device(gpu, sig, filt, b, flags)
    herm(0)
    full = _device(gpu, sig, filt, b, flags)
    ref = conv3d(sig, filt.astype(np.complex64), "fp64", engine="pocketfft")
    e_half, e_full = rel_l2(ref, half), rel_l2(ref, full)
    print(f"{n}^3 x{b} {'per-signal' if per_signal else 'shared'}: half {e_half:.3e}, full {e_full:.3e}")
    assert e_half < REL and e_full < REL
    assert not np.array_equal(half, full)
    assert gpu.device_status() == 0


@pytest.mark.parametrize("shift", [(0, 0, 0), (64, 64, 64), (3, 127, 65), (100, 64, 127), (77, 1, 1)])
def test_half_spectrum_impulse_reproduces_filter(gpu, herm, shift):
    """A shifted unit impulse gives the real filter rolled by the shift: the pairing of
    column tiles with their mirrors, rows y and N - y, and the self-mirrored columns 0 and
    N/2, all land where they belong."""
    n = 128
    rng = np.random.default_rng(sum(shift))
    sig = np.zeros((2, n, n, n), np.complex64)
    sig[0][shift] = 1.0
    sig[1][tuple((n - v) % n for v in shift)] = 1.0
    filt = rng.uniform(-1, 1, (n, n, n)).astype(np.float32)
    herm(1)
    out = _device(gpu, sig, filt, 2, gpu.NORMALIZE)
    assert rel_l2(np.roll(filt, shift, axis=(0, 1, 2)).astype(np.complex64), out[0]) < REL
    back = tuple((n - v) % n for v in shift)
    assert rel_l2(np.roll(filt, back, axis=(0, 1, 2)).astype(np.complex64), out[1]) < REL


@pytest.mark.parametrize("per_signal", [False, True])
def test_half_spectra_host_entry_point(gpu, herm, per_signal):
    """Host buffers: float filters up, half spectra on the device, and the filter-spectrum
    cache keeps a half spectrum across calls."""
    rng = np.random.default_rng(55 + per_signal)
    n, b = 128, 3
    sig = _c64(rng, (b, n, n, n))
    filt = rng.uniform(-1, 1, (b, n, n, n) if per_signal else (n, n, n)).astype(np.float32)
    flags = (gpu.FILTER_PER_SIGNAL if per_signal else gpu.FILTER_CACHED) | gpu.FILTER_REAL
    herm(1)
    ref = conv3d(sig, filt.astype(np.complex64), "fp64", engine="pocketfft")
    for _ in range(2):
        out = np.zeros_like(sig)
        t = gpu.conv3d_host(n, sig, filt, out, b, flags)
        assert t.valid, gpu.last_error()
        assert rel_l2(ref, out) < REL


def test_half_spectrum_workspace(gpu, herm):
    herm(1)
    n = 128
    assert gpu.workspace_bytes(n, 3, gpu.FILTER_REAL) == n * n * (n // 2 + 16) * 8
    assert gpu.workspace_bytes(n, 3, gpu.FILTER_REAL | gpu.FILTER_PER_SIGNAL) == 3 * n * n * (n // 2 + 16) * 8
    assert gpu.workspace_bytes(n, 3, 0) == n ** 3 * 8  # complex filters keep full spectra
    herm(0)
    assert gpu.workspace_bytes(n, 3, gpu.FILTER_REAL) == n ** 3 * 8
