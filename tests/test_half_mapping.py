"""CPU check of the Hermitian half-spectrum fused z pass's index arithmetic (herm.cuh,
k_zconv_half), before any GPU run: for every CTA, tile A (columns x0.., row y) and tile B
(columns N-x0-C.., row N-y) together cover every pencil of the cube exactly once, every
filter value a CTA reads lies inside its C+2-column box of the half layout (width
N/2 + 16), and the mirror formula conj(H[x0+C-c, y, (N-kz) mod N]) reproduces the full
spectrum of a real filter at tile B's positions."""
import numpy as np
import pytest

COLS = {64: 16, 128: 16, 256: 8, 512: 8}  # columns per tile: shape variant 1 of each size


def half_pitch(n):
    return n // 2 + 16 if n >= 64 else 0


@pytest.mark.parametrize("n", [64, 128, 256, 512])
def test_tiles_cover_every_pencil_once(n):
    c = COLS[n]
    groups = n // 2 // c
    seen = np.zeros((n, n), np.int32)  # [y, x]
    for bid in range(n * groups):
        y, x0 = bid // groups, (bid % groups) * c
        yb, xb = (n - y) & (n - 1), n - x0 - c
        assert x0 % 2 == 0 and xb % 2 == 0          # TMA: x coordinate of 8-byte elements even
        assert x0 + c + 2 <= half_pitch(n)          # the filter box lies in the half layout
        for cc in range(c):
            seen[y, x0 + cc] += 1
            seen[yb, xb + cc] += 1
            assert 1 <= c - cc <= c                  # tile B's filter column inside the box
    assert (seen == 1).all()


@pytest.mark.parametrize("n", [64, 128])
def test_mirror_formula_reproduces_the_full_spectrum(n):
    c = COLS[n]
    w = half_pitch(n)
    rng = np.random.default_rng(n)
    full = np.fft.fftn(rng.uniform(-1, 1, (n, n, n)))   # [z, y, x] of a real cube
    half = full[:, :, :w]                                # what the half layout keeps
    groups = n // 2 // c
    # every (CTA, column) at once: y, x0 from the block index, cc the tile column
    bid, cc = np.meshgrid(np.arange(n * groups), np.arange(c), indexing="ij")
    y, x0 = bid // groups, (bid % groups) * c
    yb, xb = (n - y) & (n - 1), n - x0 - c
    kz = np.arange(n)[:, None, None]
    np.testing.assert_array_equal(half[:, y, x0 + cc], full[:, y, x0 + cc])              # tile A
    mirrored = np.conj(half[(n - kz) & (n - 1), y[None], (x0 + c - cc)[None]])          # tile B
    np.testing.assert_allclose(mirrored, full[:, yb, xb + cc], rtol=0, atol=1e-9 * np.abs(full).max())
