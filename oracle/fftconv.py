"""CPU oracle for FFT-based 3D convolution — TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline leg and
its reference arm) may import this module, and only as the checker or as the timed CPU
baseline. The product (``convfpga_gb300`` and its CUDA library) never calls it.

What it restates
----------------
The reference computes ``out = IFFT3( FFT3(sig) (.) FFT3(filter) )`` on complex64 cubes
of power-of-two size N, x fastest (``idx = z*N*N + y*N + x``), with an UNNORMALISED
backward transform, so outputs carry a factor N^3:

* FPGA library: host/src/convfpga.c:32-409 (plain), host/src/convfpga_svm.c:34-461 (SVM),
  host/src/convfpga_svm_batch.c:36-724 (batched, one shared filter);
* CPU path / verifier: src/fft_conv3D.cpp:50-177 (``fft_conv3D_cpu``) and
  src/fft_conv3D.cpp:186-266 (``fft_conv3D_cpu_verify``), which call FFTW3f
  (``fftwf_plan_many_dft`` FFTW_FORWARD / FFTW_BACKWARD, src/fft_conv3D.cpp:95-99,
  201-205) — a third-party library that is not vendored in the reference and whose
  version is not pinned there (cmake/FindFFTW.cmake finds a system copy).

FFTW's published algorithm is the discrete Fourier transform computed by Cooley–Tukey
factorisation. This module restates it as a radix-2 Stockham autosort FFT
(:func:`dft_axis`), applied along x, y and z, in a chosen precision. numpy's pocketfft
(:func:`conv3d` with ``engine="pocketfft"``) is kept as a fast second engine for large
cubes and as the complex128 ("FP64 FFTW") oracle.

The pointwise product keeps the expression order of src/fft_conv3D.cpp:225-226 and of
``comp_mult`` (kernels/fft/fft_8.cl:180-185)::

    re = a.re*b.re - a.im*b.im ;  im = a.re*b.im + a.im*b.re

Pinning: the restatement is checked against vectors produced by the reference's own
FPGA FFT engine (kernels/fft/fft_8.cl built unchanged on the host), committed under
``tests/golden/``; see tests/golden/make_golden.py.

The pass criterion is the reference's: ``10*log10(sum|ref|^2 / sum|ref-out|^2) > 120``
dB (src/fft_conv3D.cpp:236-258), i.e. relative L2 error below 1e-6.
"""
from __future__ import annotations

import math
import os

import numpy as np

__all__ = [
    "dft_axis",
    "fft3d",
    "comp_mult",
    "conv3d",
    "snr_db",
    "rel_l2",
    "max_abs",
    "gaussian_filter",
    "make_config",
    "uneven_sizes",
    "CONFIG_NAMES",
]


# --------------------------------------------------------------------------- transforms
def dft_axis(a: np.ndarray, axis: int, inverse: bool = False) -> np.ndarray:
    """Unnormalised DFT of ``a`` along ``axis`` by the radix-2 Stockham autosort FFT.

    Forward uses exp(-2*pi*i*jk/N) (FFTW_FORWARD); ``inverse`` uses exp(+2*pi*i*jk/N)
    without the 1/N factor (FFTW_BACKWARD, fft_step inverse: kernels/fft/fft_8.cl:280-282,
    346-348). Arithmetic stays in ``a.dtype`` (complex64 or complex128); twiddles are
    generated in float64 and rounded once to that dtype.
    """
    if a.dtype not in (np.complex64, np.complex128):
        raise TypeError("dft_axis wants complex64 or complex128")
    x = np.moveaxis(a, axis, -1).copy()
    n = x.shape[-1]
    if n & (n - 1):
        raise ValueError("length must be a power of two")
    half = n // 2
    sign = 1.0 if inverse else -1.0
    j = np.arange(half)
    ns = 1
    while ns < n:
        k = j % ns
        w = np.exp(sign * 2j * np.pi * k / (2 * ns)).astype(x.dtype)
        v0 = x[..., :half]
        v1 = x[..., half:] * w
        y = np.empty_like(x)
        dst = (j // ns) * (2 * ns) + k
        y[..., dst] = v0 + v1
        y[..., dst + ns] = v0 - v1
        x = y
        ns *= 2
    return np.moveaxis(x, -1, axis)


def fft3d(vol: np.ndarray, inverse: bool = False, engine: str = "stockham", workers: int | None = None) -> np.ndarray:
    """Unnormalised 3D transform over the last three axes (z, y, x) of ``vol``."""
    if engine == "stockham":
        out = vol
        for ax in (-1, -2, -3):
            out = dft_axis(out, ax, inverse)
        return out
    if engine == "pocketfft":
        import scipy.fft as sfft

        w = workers if workers is not None else (os.cpu_count() or 1)
        if inverse:
            # norm="forward" leaves the backward transform unscaled (FFTW_BACKWARD).
            return sfft.ifftn(vol, axes=(-3, -2, -1), norm="forward", workers=w)
        return sfft.fftn(vol, axes=(-3, -2, -1), workers=w)
    raise ValueError(f"unknown engine {engine!r}")


def comp_mult(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Complex product with the reference's expression order (src/fft_conv3D.cpp:225-226)."""
    ar, ai = a.real, a.imag
    br, bi = b.real, b.imag
    out = np.empty(np.broadcast_shapes(a.shape, b.shape), dtype=np.result_type(a, b))
    out.real = (ar * br) - (ai * bi)
    out.imag = (ar * bi) + (ai * br)
    return out


def conv3d(
    sig: np.ndarray,
    filt: np.ndarray,
    precision: str = "fp32",
    normalize: bool = False,
    engine: str = "stockham",
    workers: int | None = None,
) -> np.ndarray:
    """FFT-based circular 3D convolution, the reference pipeline.

    ``sig``: (B, N, N, N) or (N, N, N). ``filt``: (N, N, N) shared by all signals
    (src/fft_conv3D.cpp:222-231, host/src/convfpga_svm_batch.c) or (B, N, N, N), one per
    signal. Returns complex64 for ``precision="fp32"`` and complex128 for ``"fp64"``.
    Unnormalised unless ``normalize`` (then scaled by 1/N^3).
    """
    dt = {"fp32": np.complex64, "fp64": np.complex128}[precision]
    s = np.asarray(sig).astype(dt, copy=True)
    f = np.asarray(filt).astype(dt, copy=True)
    squeeze = s.ndim == 3
    if squeeze:
        s = s[None]
    if f.ndim == 4 and f.shape[0] != s.shape[0]:
        raise ValueError("per-signal filters need one filter per signal")
    n = s.shape[-1]
    fs = fft3d(f, False, engine, workers).astype(dt, copy=False)
    ss = fft3d(s, False, engine, workers).astype(dt, copy=False)
    prod = comp_mult(ss, fs if fs.ndim == 4 else fs[None]).astype(dt, copy=False)
    out = fft3d(prod, True, engine, workers).astype(dt, copy=False)
    if normalize:
        out = (out * dt(1.0 / float(n) ** 3)).astype(dt, copy=False)
    return out[0] if squeeze else out


# --------------------------------------------------------------------------- error measures
def snr_db(ref: np.ndarray, out: np.ndarray) -> float:
    """Signal-to-noise ratio in dB as in src/fft_conv3D.cpp:236-258 (sums in float64)."""
    r = np.asarray(ref).astype(np.complex128).ravel()
    o = np.asarray(out).astype(np.complex128).ravel()
    mag = float(np.sum(r.real * r.real + r.imag * r.imag))
    noise = float(np.sum((r.real - o.real) ** 2 + (r.imag - o.imag) ** 2))
    if noise == 0.0:
        return math.inf
    return 10.0 * math.log10(mag / noise)


def rel_l2(ref: np.ndarray, out: np.ndarray) -> float:
    r = np.asarray(ref).astype(np.complex128).ravel()
    o = np.asarray(out).astype(np.complex128).ravel()
    return float(np.linalg.norm(r - o) / np.linalg.norm(r))


def max_abs(ref: np.ndarray, out: np.ndarray) -> float:
    r = np.asarray(ref).astype(np.complex128).ravel()
    o = np.asarray(out).astype(np.complex128).ravel()
    return float(np.max(np.abs(r - o)))


# --------------------------------------------------------------------------- inputs
def _uniform_c64(rng: np.random.Generator, shape, lo=-1.0, hi=1.0) -> np.ndarray:
    out = np.empty(shape, dtype=np.complex64)
    out.real = rng.uniform(lo, hi, size=shape).astype(np.float32)
    out.imag = rng.uniform(lo, hi, size=shape).astype(np.float32)
    return out


def gaussian_filter(n: int, sigma: float) -> np.ndarray:
    """Real isotropic Gaussian centred at the origin with periodic wrap, imag 0."""
    d = np.arange(n, dtype=np.float64)
    d = np.minimum(d, n - d)
    g1 = np.exp(-0.5 * (d / sigma) ** 2)
    g = g1[:, None, None] * g1[None, :, None] * g1[None, None, :]
    return g.astype(np.complex64)


def _blob_field(rng: np.random.Generator, n: int, nblobs: int = 64) -> np.ndarray:
    """Sum of periodic Gaussian blobs (separable per blob) plus tiny uniform noise."""
    field = np.zeros((n, n, n), dtype=np.float32)
    ax = np.arange(n, dtype=np.float64)
    for _ in range(nblobs):
        c = rng.uniform(0, n, size=3)
        w = rng.uniform(4.0, 32.0)
        amp = rng.uniform(-1.0, 1.0)
        prof = []
        for k in range(3):
            d = np.abs(ax - c[k])
            d = np.minimum(d, n - d)
            prof.append(np.exp(-0.5 * (d / w) ** 2).astype(np.float32))
        field += np.float32(amp) * (prof[0][:, None, None] * prof[1][None, :, None] * prof[2][None, None, :])
    out = np.empty((n, n, n), dtype=np.complex64)
    out.real = field + rng.uniform(-1e-3, 1e-3, size=(n, n, n)).astype(np.float32)
    out.imag = rng.uniform(-1e-3, 1e-3, size=(n, n, n)).astype(np.float32)
    return out


CONFIG_NAMES = ("c64x1", "c128x8", "c256x4", "uneven96", "c512x1")


def uneven_sizes(seed: int = 4, count: int = 96) -> list[int]:
    """Cube sizes of the uneven batch: drawn from {32,64,128,256}, p={.4,.3,.2,.1}."""
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.choice([32, 64, 128, 256], size=count, p=[0.4, 0.3, 0.2, 0.1])]


def make_config(name: str, seed: int | None = None, scale_n: int | None = None):
    """Seeded inputs for the five workloads.

    Returns ``(sigs, filters, shared)``: for the uniform-size configs ``sigs`` is
    (B, N, N, N) complex64 and ``filters`` is (N, N, N) when ``shared`` else
    (B, N, N, N). For ``uneven96`` both are lists of cubes (one filter per signal).
    ``scale_n`` replaces N (for quick checks at a smaller size with the same
    distributions).
    """
    if name == "c64x1":
        rng = np.random.default_rng(1 if seed is None else seed)
        n = scale_n or 64
        return _uniform_c64(rng, (1, n, n, n)), _uniform_c64(rng, (n, n, n)), True
    if name == "c128x8":
        rng = np.random.default_rng(2 if seed is None else seed)
        n = scale_n or 128
        return _uniform_c64(rng, (8, n, n, n)), gaussian_filter(n, 4.0), True
    if name == "c256x4":
        rng = np.random.default_rng(3 if seed is None else seed)
        n = scale_n or 256
        sig = np.empty((4, n, n, n), dtype=np.complex64)
        sig.real = rng.standard_normal((4, n, n, n), dtype=np.float32)
        sig.imag = rng.standard_normal((4, n, n, n), dtype=np.float32)
        return sig, _uniform_c64(rng, (4, n, n, n)), False
    if name == "uneven96":
        s = 4 if seed is None else seed
        sizes = uneven_sizes(s)
        if scale_n:
            sizes = [min(v, scale_n) for v in sizes]
        rng = np.random.default_rng(s + 1000)
        sigs, filts = [], []
        for n in sizes:
            sigs.append(_uniform_c64(rng, (n, n, n)))
            filts.append(gaussian_filter(n, float(rng.uniform(1.0, 8.0))))
        return sigs, filts, False
    if name == "c512x1":
        rng = np.random.default_rng(5 if seed is None else seed)
        n = scale_n or 512
        return _blob_field(rng, n)[None], gaussian_filter(n, 6.0), True
    raise ValueError(f"unknown config {name!r}")
