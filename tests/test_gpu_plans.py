"""Shape variants and the autotuner's plan cache (convgpu_autotune / convgpu_plan_variant).

Every cube size has two shape variants (radix split, pencils per CTA, rows per CTA);
both must give the oracle's results (SNR > 120 dB, the reference's criterion). The
autotuner's choices survive a save / fpga_final / fpga_initialize round trip.
"""
import os

import numpy as np
import pytest

from oracle import conv3d, snr_db

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

KINDS = 4  # shape-variant kinds; kind 4 (fused x+y) is tested separately


def _c64(rng, shape):
    a = np.empty(shape, np.complex64)
    a.real = rng.uniform(-1, 1, shape)
    a.imag = rng.uniform(-1, 1, shape)
    return a


@pytest.fixture
def restore_plans(gpu):
    """Puts every plan kind of every size back as it was: the autotuner below also sets the
    tensor-core and half-spectrum kinds, which later tests in the session rely on."""
    keep = {(n, k): gpu.plan_variant(n, k) for n in (16, 32, 64, 128, 256, 512) for k in range(len(gpu.PLAN_KINDS))}
    yield
    for (n, k), v in keep.items():
        gpu.plan_variant(n, k, v)


def _check(gpu, n, b, per_signal):
    rng = np.random.default_rng(n * 3 + per_signal)
    sig = _c64(rng, (b, n, n, n))
    filt = _c64(rng, (b, n, n, n)) if per_signal else _c64(rng, (n, n, n))
    s = torch.from_numpy(sig).cuda()
    f = torch.from_numpy(filt).cuda()
    o = torch.empty_like(s)
    gpu.conv3d_device(n, s, f, o, b, gpu.FILTER_PER_SIGNAL if per_signal else 0)
    torch.cuda.synchronize()
    ref = conv3d(sig, filt, "fp32", engine="pocketfft")
    assert snr_db(ref, o.cpu().numpy()) > 120.0


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256])
@pytest.mark.parametrize("variant", [0, 1])
def test_every_variant_matches_the_oracle(gpu, restore_plans, n, variant):
    for k in range(KINDS):
        assert gpu.plan_variant(n, k, variant) == variant
    b = 2 if n <= 128 else 1
    _check(gpu, n, b, per_signal=False)  # x, y/z and fused z (CONV) kernels
    _check(gpu, n, b, per_signal=True)   # fused z with the filter's z transform (CONV_FZ)
    assert gpu.device_status() == 0


@pytest.mark.slow
@pytest.mark.parametrize("variant", [0, 1])
def test_512_variants(gpu, restore_plans, variant):
    for k in range(KINDS):
        gpu.plan_variant(512, k, variant)
    _check(gpu, 512, 1, per_signal=True)


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("xy", [1, 2], ids=["l2_staged", "cluster"])
def test_fused_xy_pass_256(gpu, restore_plans, variant, xy):
    """x and y of 256^3 cubes as one pass (plan kind 4): variant 1 stages the x-transformed
    planes through an L2-resident scratch ring, variant 2 holds each plane in an 8-CTA
    cluster's shared memory. Forward and inverse, shared and per-signal filters, host path."""
    assert gpu.plan_variant(256, 4, xy) == xy
    for k in range(KINDS):
        gpu.plan_variant(256, k, variant)
    _check(gpu, 256, 2, per_signal=False)
    _check(gpu, 256, 3, per_signal=True)
    rng = np.random.default_rng(99)
    sig = _c64(rng, (2, 256, 256, 256))
    filt = _c64(rng, (256, 256, 256))
    out = np.zeros_like(sig)
    t = gpu.fpgaf_conv3D_svm_batch(256, sig, filt, out, 2)
    assert t.valid, gpu.last_error()
    assert snr_db(conv3d(sig, filt, "fp32", engine="pocketfft"), out) > 120.0
    assert gpu.device_status() == 0


@pytest.mark.parametrize("variant", [0, 1])
def test_fused_xy_pass_128(gpu, restore_plans, variant):
    """x and y of 128^3 cubes as one pass staged through an L2-resident scratch ring (plan
    kind 4, variant 1; 16-row / 16-column items): forward and inverse, shared and
    per-signal filters, in place, and the host path; the same results as the separate
    passes within rounding (both within the reference's 120 dB criterion)."""
    for k in range(KINDS):
        gpu.plan_variant(128, k, variant)
    gpu.plan_variant(128, 4, 0)
    rng = np.random.default_rng(128)
    sig = _c64(rng, (3, 128, 128, 128))
    filt = _c64(rng, (3, 128, 128, 128))
    s = torch.from_numpy(sig).cuda()
    f = torch.from_numpy(filt).cuda()
    o_sep = torch.empty_like(s)
    gpu.conv3d_device(128, s, f, o_sep, 3, gpu.FILTER_PER_SIGNAL)
    assert gpu.plan_variant(128, 4, 1) == 1
    _check(gpu, 128, 2, per_signal=False)
    _check(gpu, 128, 3, per_signal=True)
    o_xy = torch.empty_like(s)
    gpu.conv3d_device(128, s, f, o_xy, 3, gpu.FILTER_PER_SIGNAL)
    s2 = s.clone()
    gpu.conv3d_device(128, s2, f, s2, 3, gpu.FILTER_PER_SIGNAL | gpu.NORMALIZE)
    torch.cuda.synchronize()
    assert snr_db(o_sep.cpu().numpy(), o_xy.cpu().numpy()) > 120.0
    np.testing.assert_allclose(s2.cpu().numpy(), o_xy.cpu().numpy() / 128 ** 3, rtol=0, atol=1e-6)
    out = np.zeros_like(sig[:2])
    t = gpu.fpgaf_conv3D_svm_batch(128, sig[:2], filt[0], out, 2)
    assert t.valid, gpu.last_error()
    assert snr_db(conv3d(sig[:2], filt[0], "fp32", engine="pocketfft"), out) > 120.0
    assert gpu.device_status() == 0


def test_autotune_plan_cache_round_trip(gpu, restore_plans, tmp_path):
    path = str(tmp_path / "plans.json")
    gpu.fpga_final()
    assert gpu.fpga_initialize("cuda:0", path, False) == 0
    gpu.autotune([32, 128, 256], write_cache=True)
    chosen = {n: [gpu.plan_variant(n, k) for k in range(KINDS)] for n in (32, 128, 256)}
    text = open(path).read()
    assert '"256": {' in text and '"us_v1"' in text
    for n in (32, 128, 256):      # scramble, then reload from the file
        for k in range(KINDS):
            gpu.plan_variant(n, k, 1 - chosen[n][k])
    gpu.fpga_final()
    assert gpu.fpga_initialize("cuda:0", path, False) == 0
    assert {n: [gpu.plan_variant(n, k) for k in range(KINDS)] for n in (32, 128, 256)} == chosen
    gpu.fpga_final()
    assert gpu.fpga_initialize("cuda:0", "convgpu_plans.json", False) == 0


def test_initialize_ignores_a_file_that_is_not_a_plan_cache(gpu, restore_plans, tmp_path):
    p = tmp_path / "kernel.aocx"
    p.write_bytes(os.urandom(4096))
    gpu.fpga_final()
    assert gpu.fpga_initialize("cuda:0", str(p), False) == 0
    gpu.fpga_final()
    assert gpu.fpga_initialize("cuda:0", "convgpu_plans.json", False) == 0


def test_uneven_graph_with_fused_xy(gpu, restore_plans):
    """The uneven batch's CUDA graph runs its 256^3 and 128^3 jobs through the table-mode
    L2-staged x+y pass when the plan fuses x and y (kind 4, variant 1) and through separate
    passes otherwise; both match the oracle and each other. A second call with new buffers
    re-encodes the per-job maps of the cached graph."""
    sizes = [256, 64, 256, 32, 128, 256, 128]
    offs = np.cumsum([0] + [n ** 3 for n in sizes])
    outs = {}
    for xy in (1, 0):
        gpu.plan_variant(256, 4, xy)
        gpu.plan_variant(128, 4, xy)
        for rep in range(2):
            rng = np.random.default_rng(500 + rep)
            sigs = [_c64(rng, (n, n, n)) for n in sizes]
            filts = [_c64(rng, (n, n, n)) for n in sizes]
            s = torch.from_numpy(np.concatenate([x.ravel() for x in sigs])).cuda()
            f = torch.from_numpy(np.concatenate([x.ravel() for x in filts])).cuda()
            o = torch.empty_like(s)
            jobs = [(n, int(offs[i]), int(offs[i]), int(offs[i])) for i, n in enumerate(sizes)]
            gpu.conv3d_uneven_device(jobs, s, f, o, gpu.NORMALIZE)
            torch.cuda.synchronize()
            oh = o.cpu().numpy()
            for i, n in enumerate(sizes):
                ref = conv3d(sigs[i], filts[i], "fp32", normalize=True, engine="pocketfft")
                assert snr_db(ref, oh[offs[i]:offs[i + 1]].reshape(n, n, n)) > 120.0, (xy, rep, i, n)
            outs[(xy, rep)] = oh
            del s, f, o
    for rep in range(2):
        assert snr_db(outs[(0, rep)], outs[(1, rep)]) > 130.0
    assert gpu.device_status() == 0


@pytest.mark.slow
def test_fused_xy_pass_512(gpu, restore_plans):
    """x and y of 512^3 cubes as one L2-staged pass (plan kind 4, variant 1; 4-row /
    4-column items, two TMA boxes per column tile): a shifted delta filter gives the
    circular shift of the signal, and the result equals the separate passes' within
    rounding, forward and inverse."""
    n = 512
    rng = np.random.default_rng(512)
    sig = np.empty((1, n, n, n), np.complex64)
    sig.real = rng.standard_normal((1, n, n, n), dtype=np.float32)
    sig.imag = rng.standard_normal((1, n, n, n), dtype=np.float32)
    delta = np.zeros((n, n, n), np.complex64)
    delta[3, 5, 7] = 1.0
    s = torch.from_numpy(sig).cuda()
    d = torch.from_numpy(delta).cuda()
    f = torch.from_numpy(_c64(rng, (n, n, n))).cuda()
    outs = {}
    for xy in (0, 1):
        assert gpu.plan_variant(n, 4, xy) == xy
        o = torch.empty_like(s)
        gpu.conv3d_device(n, s, d, o, 1, gpu.NORMALIZE)
        torch.cuda.synchronize()
        shifted = np.roll(sig, shift=(3, 5, 7), axis=(1, 2, 3))
        from oracle import rel_l2
        assert rel_l2(shifted, o.cpu().numpy()) < 1e-6, xy
        gpu.conv3d_device(n, s, f, o, 1, 0)
        torch.cuda.synchronize()
        outs[xy] = o.cpu().numpy()
        del o
    assert snr_db(outs[0], outs[1]) > 120.0
    assert gpu.device_status() == 0
