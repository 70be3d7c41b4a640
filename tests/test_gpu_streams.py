"""Calls on different streams that overlap in time: the library orders them on the GPU
(they share the workspace and the fused x+y pass's scratch ring and counters), so both
results stay exact. The reference is single-stream and blocking (host/src/fpga_init.c:18-29:
process-global state); its callers never overlap calls."""
import numpy as np
import pytest

from oracle import conv3d, rel_l2

pytestmark = [pytest.mark.gpu, pytest.mark.slow]
torch = pytest.importorskip("torch")


def test_two_streams_with_the_fused_pass_both_exact(gpu):
    cg = gpu
    n, b = 256, 2
    keep = cg.plan_variant(n, 4)
    cg.plan_variant(n, 4, 1)  # x+y through the shared L2 scratch ring
    try:
        rng = np.random.default_rng(31)
        shape = (b, n, n, n)
        sig = [(rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64) for _ in range(2)]
        filt = [(rng.uniform(-1, 1, shape) + 1j * rng.uniform(-1, 1, shape)).astype(np.complex64) for _ in range(2)]
        s = [torch.from_numpy(x).cuda() for x in sig]
        f = [torch.from_numpy(x).cuda() for x in filt]
        o = [torch.empty_like(x) for x in s]
        streams = [torch.cuda.Stream(), torch.cuda.Stream()]
        torch.cuda.synchronize()
        for _ in range(3):  # back to back, no host wait between the two streams
            for k in range(2):
                cg.conv3d_device(n, s[k], f[k], o[k], b, cg.FILTER_PER_SIGNAL, streams[k])
        torch.cuda.synchronize()
        assert cg.device_status() == 0
        for k in range(2):
            got = o[k].cpu().numpy()
            for i in range(b):
                ref = conv3d(sig[k][i], filt[k][i], "fp64", engine="pocketfft")
                assert rel_l2(ref, got[i]) < 1e-6
    finally:
        cg.plan_variant(n, 4, keep)
