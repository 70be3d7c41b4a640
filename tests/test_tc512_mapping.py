"""CPU check of the 512-point tensor-core pass's decomposition and index arithmetic
(tc05.cuh, k_tc05_512) before any GPU run: a radix-2 step on the CUDA cores around two
256-point transforms, with the kernel's thread mapping. numpy's DFT stands in for the
tensor-core 256-point stages (t5_fft256), which leave output k of sub-pencil (q, j, c) at
register k of the thread whose 256-positions are q + 16 k."""
import numpy as np
import pytest

N, P = 512, 4  # points per pencil, pencils per CTA


def w512(p, sign=-1):
    return np.exp(sign * 2j * np.pi * p / N)


def forward(x):
    """x: (P, N) pencils -> per thread (q, j, c) the 16 values X[2(q + 16k) + j]."""
    regs = {}
    for c in range(P):
        for j in range(2):
            # gather_dif: u[p] = x[p] + x[p+256], w[p] = (x[p] - x[p+256]) W512^p
            p = np.arange(256)
            sub = x[c, p] + (-1) ** j * x[c, p + 256]
            if j:
                sub = sub * w512(p)
            y = np.fft.fft(sub)  # the tensor-core 256-point transform
            for q in range(16):
                regs[(q, j, c)] = y[q + 16 * np.arange(16)]
    return regs


def inverse(regs):
    """Per thread (q, j, c) registers holding X[2(q + 16k) + j] -> (P, N) unnormalised
    inverse, through IDFT256 of each sub-pencil and the shuffle-partner combine."""
    out = np.zeros((P, N), np.complex128)
    for c in range(P):
        sub = {}
        for j in range(2):
            spec = np.zeros(256, np.complex128)
            for q in range(16):
                spec[q + 16 * np.arange(16)] = regs[(q, j, c)]
            sub[j] = np.conj(np.fft.fft(np.conj(spec)))  # swap -> forward -> swap: unnormalised inverse
        for q in range(16):
            n = q + 16 * np.arange(16)
            e, o = sub[0][n], sub[1][n]
            t1 = o * np.conj(w512(n))   # partner j = 1 sends O[n] W512^-n
            out[c, n] = e + t1          # j = 0 keeps x[n]
            out[c, n + 256] = e - t1    # j = 1 keeps x[n + 256]
    return out


def test_forward_registers_hold_the_dft_at_their_positions():
    rng = np.random.default_rng(512)
    x = rng.standard_normal((P, N)) + 1j * rng.standard_normal((P, N))
    regs = forward(x)
    ref = np.fft.fft(x, axis=1)
    for (q, j, c), v in regs.items():
        np.testing.assert_allclose(v, ref[c, 2 * (q + 16 * np.arange(16)) + j], rtol=0, atol=1e-9)


def test_inverse_of_forward_scales_by_n():
    rng = np.random.default_rng(513)
    x = rng.standard_normal((P, N)) + 1j * rng.standard_normal((P, N))
    np.testing.assert_allclose(inverse(forward(x)), N * x, rtol=0, atol=1e-8)


@pytest.mark.parametrize("rows", [False, True])
def test_lanes_of_a_pencil_pair_share_a_warp(rows):
    """The E/O partners of every pencil position are lanes m and m ^ partner of one warp."""
    for m in range(128):
        ia, ib = (m >> 4, m & 15) if rows else (m >> 3, m & 7)
        j, c, q = (ia & 1, ia >> 1, ib) if rows else (ib >> 2, ib & 3, ia)
        mp = m ^ (16 if rows else 4)
        ia2, ib2 = (mp >> 4, mp & 15) if rows else (mp >> 3, mp & 7)
        j2, c2, q2 = (ia2 & 1, ia2 >> 1, ib2) if rows else (ib2 >> 2, ib2 & 3, ia2)
        assert mp // 32 == m // 32 and (c2, q2) == (c, q) and j2 == 1 - j
