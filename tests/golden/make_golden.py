"""Generate the golden vectors under tests/golden/ from the reference's own FFT engine.

The vectors come from ``oracle/_ref/libfft8ref.so``: the reference's FPGA FFT engine
(kernels/fft/fft_8.cl of pc2/ConvFPGA, compiled unchanged on the host by
``make -C oracle``) driven the way the reference kernels drive it, plus its ``comp_mult``
for the pointwise product. They pin the oracle (oracle/fftconv.py) and, through it, the
CUDA path.

Run from the repository root, where the reference sources are available::

    make -C oracle && python tests/golden/make_golden.py

Files written (all complex64 unless noted):
  fft1d.npz       for logN = 4..9: seeded input ``x{logN}``, raw engine output
                  (bit-reversed order) ``fwd{logN}`` and ``inv{logN}``
  conv16x3.npz    3 distinct signals, one shared filter, N=16 (``sig``, ``filt``, ``out``)
  conv16x2pf.npz  2 signals with per-signal filters, N=16
  conv32x1.npz    1 signal, N=32
  conv64x1.npz    the 64^3 x 1 workload (inputs regenerated by oracle.make_config("c64x1"));
                  stores ``out`` and the float64 checksums ``sig_sum``/``filt_sum`` of the inputs
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import make_config  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(ROOT, "oracle", "_ref", "libfft8ref.so")


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _load():
    if not os.path.exists(LIB):
        raise SystemExit(f"{LIB} missing: run `make -C oracle` where the reference sources exist")
    lib = ctypes.CDLL(LIB)
    for fn in ("fft8ref_1d_raw", "fft8ref_fft3d", "fft8ref_conv3d"):
        getattr(lib, fn).restype = ctypes.c_int
    return lib


def _c64(rng, shape):
    a = np.empty(shape, np.complex64)
    a.real = rng.uniform(-1, 1, shape).astype(np.float32)
    a.imag = rng.uniform(-1, 1, shape).astype(np.float32)
    return a


def ref_conv(lib, sig: np.ndarray, filt: np.ndarray) -> np.ndarray:
    sig = np.ascontiguousarray(sig, np.complex64)
    filt = np.ascontiguousarray(filt, np.complex64)
    b, n = sig.shape[0], sig.shape[-1]
    per = 1 if filt.ndim == 4 else 0
    out = np.zeros_like(sig)
    rc = lib.fft8ref_conv3d(int(np.log2(n)), b, _ptr(sig), _ptr(filt), _ptr(out), per)
    if rc != 0:
        raise RuntimeError("fft8ref_conv3d failed")
    return out


def main() -> None:
    lib = _load()
    rng = np.random.default_rng(20240611)

    d = {}
    for logn in range(4, 10):
        n = 1 << logn
        x = _c64(rng, (n,))
        fwd = np.zeros(n, np.complex64)
        inv = np.zeros(n, np.complex64)
        lib.fft8ref_1d_raw(logn, 0, _ptr(x), _ptr(fwd))
        lib.fft8ref_1d_raw(logn, 1, _ptr(x), _ptr(inv))
        d[f"x{logn}"], d[f"fwd{logn}"], d[f"inv{logn}"] = x, fwd, inv
    np.savez(os.path.join(HERE, "fft1d.npz"), **d)

    sig, filt = _c64(rng, (3, 16, 16, 16)), _c64(rng, (16, 16, 16))
    np.savez(os.path.join(HERE, "conv16x3.npz"), sig=sig, filt=filt, out=ref_conv(lib, sig, filt))

    sig, filt = _c64(rng, (2, 16, 16, 16)), _c64(rng, (2, 16, 16, 16))
    np.savez(os.path.join(HERE, "conv16x2pf.npz"), sig=sig, filt=filt, out=ref_conv(lib, sig, filt))

    sig, filt = _c64(rng, (1, 32, 32, 32)), _c64(rng, (32, 32, 32))
    np.savez(os.path.join(HERE, "conv32x1.npz"), sig=sig, filt=filt, out=ref_conv(lib, sig, filt))

    sig, filt, _ = make_config("c64x1")
    out = ref_conv(lib, sig, filt)
    np.savez(
        os.path.join(HERE, "conv64x1.npz"),
        out=out,
        sig_sum=np.array([sig.real.astype(np.float64).sum(), sig.imag.astype(np.float64).sum()]),
        filt_sum=np.array([filt.real.astype(np.float64).sum(), filt.imag.astype(np.float64).sum()]),
    )
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
