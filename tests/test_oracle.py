"""The oracle against the reference's own FFT engine (golden vectors) and FP64.

Golden vectors in tests/golden/ were produced by kernels/fft/fft_8.cl of pc2/ConvFPGA
compiled unchanged on the host (tests/golden/make_golden.py). The pass criterion is the
reference's SNR > 120 dB (src/fft_conv3D.cpp:236-258).
"""
import os

import numpy as np
import pytest

from oracle import (comp_mult, conv3d, dft_axis, gaussian_filter, make_config, max_abs, rel_l2, snr_db,
                    uneven_sizes)

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _bitrev(v: int, bits: int) -> int:
    return int(format(v, f"0{bits}b")[::-1], 2)


@pytest.mark.parametrize("logn", range(4, 10))
def test_1d_against_reference_engine(logn):
    d = np.load(os.path.join(GOLD, "fft1d.npz"))
    n = 1 << logn
    x = d[f"x{logn}"]
    perm = np.array([_bitrev(p, logn) for p in range(n)])
    for key, inv in (("fwd", False), ("inv", True)):
        raw = d[f"{key}{logn}"]
        nat = np.empty_like(raw)
        nat[perm] = raw  # the engine emits bit-reversed order (kernels/fft/fft_8.cl:28-30)
        ours = dft_axis(x, 0, inverse=inv)
        assert snr_db(nat, ours) > 120.0
        exact = np.fft.fft(x.astype(np.complex128)) if not inv else np.fft.ifft(x.astype(np.complex128)) * n
        assert rel_l2(exact, ours) < 3e-7


@pytest.mark.parametrize("name", ["conv16x3", "conv16x2pf", "conv32x1"])
@pytest.mark.parametrize("engine", ["stockham", "pocketfft"])
def test_conv_against_reference_engine(name, engine):
    d = np.load(os.path.join(GOLD, f"{name}.npz"))
    out = conv3d(d["sig"], d["filt"], "fp32", engine=engine)
    assert out.dtype == np.complex64
    assert snr_db(d["out"], out) > 120.0
    exact = conv3d(d["sig"], d["filt"], "fp64", engine=engine)
    assert rel_l2(exact, d["out"]) < 1e-6


def test_conv64_workload_against_reference_engine():
    d = np.load(os.path.join(GOLD, "conv64x1.npz"))
    sig, filt, shared = make_config("c64x1")
    assert shared and sig.shape == (1, 64, 64, 64)
    # the seeded generator must reproduce the inputs the golden output was made from
    np.testing.assert_allclose([sig.real.astype(np.float64).sum(), sig.imag.astype(np.float64).sum()],
                               d["sig_sum"], rtol=0, atol=1e-6)
    np.testing.assert_allclose([filt.real.astype(np.float64).sum(), filt.imag.astype(np.float64).sum()],
                               d["filt_sum"], rtol=0, atol=1e-6)
    out = conv3d(sig, filt, "fp32")
    assert snr_db(d["out"], out) > 120.0


def test_unnormalised_identity():
    """A delta filter reproduces the signal times N^3 (FFTW_BACKWARD has no 1/N)."""
    rng = np.random.default_rng(0)
    n = 16
    sig = (rng.uniform(-1, 1, (n, n, n)) + 1j * rng.uniform(-1, 1, (n, n, n))).astype(np.complex64)
    delta = np.zeros((n, n, n), np.complex64)
    delta[0, 0, 0] = 1
    out = conv3d(sig, delta, "fp64")
    assert rel_l2(sig * n ** 3, out) < 1e-12
    outn = conv3d(sig, delta, "fp64", normalize=True)
    assert rel_l2(sig, outn) < 1e-12


def test_comp_mult_order():
    a = np.array([1 + 2j, -3.5 + 0.25j], np.complex64)
    b = np.array([0.5 - 1j, 2 + 2j], np.complex64)
    np.testing.assert_array_equal(comp_mult(a, b), a * b)


def test_snr_matches_rel_l2():
    rng = np.random.default_rng(1)
    r = rng.standard_normal(100) + 1j * rng.standard_normal(100)
    o = r + 1e-7 * rng.standard_normal(100)
    assert abs(snr_db(r, o) - (-20 * np.log10(rel_l2(r, o)))) < 1e-9
    assert snr_db(r, r) == float("inf")
    assert max_abs(r, o) > 0


def test_planted_error_is_caught():
    """A mistake planted in the oracle's output must fail the 120 dB criterion."""
    d = np.load(os.path.join(GOLD, "conv32x1.npz"))
    out = conv3d(d["sig"], d["filt"], "fp32")
    out.flat[1234] += 1e-2 * np.abs(out).max()
    assert snr_db(d["out"], out) < 120.0


def test_generators():
    s, f, shared = make_config("c128x8", scale_n=16)
    assert s.shape == (8, 16, 16, 16) and f.shape == (16, 16, 16) and shared
    assert np.all(f.imag == 0) and abs(f[0, 0, 0] - 1) < 1e-6
    s, f, shared = make_config("c256x4", scale_n=16)
    assert s.shape == (4, 16, 16, 16) and f.shape == (4, 16, 16, 16) and not shared
    sizes = uneven_sizes()
    assert len(sizes) == 96 and set(sizes) <= {32, 64, 128, 256}
    g = gaussian_filter(32, 4.0)
    assert g[1, 0, 0] == g[31, 0, 0]  # periodic wrap
    s, f, shared = make_config("c512x1", scale_n=32)
    assert s.shape == (1, 32, 32, 32) and np.abs(s.imag).max() <= 1e-3
    s2, _, _ = make_config("c512x1", scale_n=32)
    np.testing.assert_array_equal(s, s2)


def test_fp32_pipeline_error_budget():
    """The FP32 restatement stays near 3e-7 rel-L2 from FP64, the level FFTW reaches."""
    s, f, _ = make_config("c64x1", scale_n=32)
    o32 = conv3d(s, f, "fp32")
    o64 = conv3d(s, f, "fp64", engine="pocketfft")
    assert rel_l2(o64, o32) < 6e-7
