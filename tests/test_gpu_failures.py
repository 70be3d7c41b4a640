"""The failure contract on the GPU, without faulting, trapping or hanging it.

The reference exit()s the process on any runtime error (host/src/opencl_utils.c:421-439);
this library instead bounds every wait in its kernels, records a wait that gave up in the
device status word, and reports it: host-buffer calls return an fpga_t with valid == 0,
device calls leave the bit for convgpu_device_status. These tests make the waits run out
on purpose through the testing hook that lowers every dependency-wait limit (to 0 probes:
the wait gives up at once, so the outcome does not depend on timing), check the report,
restore the limit and check that the next call is clean and matches the oracle. Waits on
copies or MMAs in flight are never shortened. Allocation failures are injected on the
host.
"""
import numpy as np
import pytest

from oracle import conv3d, snr_db

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

STATUS_QUEUE = 2      # uneven work queue / small-cube grid barrier gave up a dependency wait
STATUS_XY_L2 = 16     # fused x+y pass gave up a plane dependency wait


def _c64(rng, shape):
    a = np.empty(shape, np.complex64)
    a.real = rng.uniform(-1, 1, shape)
    a.imag = rng.uniform(-1, 1, shape)
    return a


@pytest.fixture
def cg(gpu):
    gpu.device_status()  # start clean
    yield gpu
    gpu.debug_dependency_wait_limit(-1)
    gpu.device_status()


def test_work_queue_dependency_timeout_is_reported_then_clean(cg):
    rng = np.random.default_rng(21)
    sizes = [64, 32, 64, 16]
    sigs = [_c64(rng, (n, n, n)) for n in sizes]
    filts = [_c64(rng, (n, n, n)) for n in sizes]
    offs = np.cumsum([0] + [n ** 3 for n in sizes])
    s = torch.from_numpy(np.concatenate([x.ravel() for x in sigs])).cuda()
    f = torch.from_numpy(np.concatenate([x.ravel() for x in filts])).cuda()
    o = torch.zeros_like(s)
    jobs = [(n, int(offs[i]), int(offs[i]), int(offs[i])) for i, n in enumerate(sizes)]
    cg.debug_dependency_wait_limit(0)
    cg.conv3d_uneven_device(jobs, s, f, o, cg.UNEVEN_QUEUE)
    assert cg.device_status() & STATUS_QUEUE
    cg.debug_dependency_wait_limit(-1)
    cg.conv3d_uneven_device(jobs, s, f, o, cg.UNEVEN_QUEUE)  # the same cached graph, replayed
    assert cg.device_status() == 0
    out = o.cpu().numpy()
    for i, n in enumerate(sizes):
        got = out[offs[i]:offs[i + 1]].reshape(n, n, n)
        assert snr_db(conv3d(sigs[i], filts[i], "fp32"), got) > 120.0


def test_small_cube_grid_barrier_timeout_is_reported_then_clean(cg):
    rng = np.random.default_rng(22)
    n = 64
    sig, filt = _c64(rng, (1, n, n, n)), _c64(rng, (n, n, n))
    s, f = torch.from_numpy(sig).cuda(), torch.from_numpy(filt).cuda()
    o = torch.empty_like(s)
    cg.debug_dependency_wait_limit(0)
    cg.conv3d_device(n, s, f, o, 1, 0)  # one cooperative launch with grid barriers
    assert cg.device_status() & STATUS_QUEUE
    cg.debug_dependency_wait_limit(-1)
    cg.conv3d_device(n, s, f, o, 1, 0)
    assert cg.device_status() == 0
    assert snr_db(conv3d(sig, filt, "fp32"), o.cpu().numpy()) > 120.0


def test_host_call_returns_invalid_on_a_dependency_timeout_then_clean(cg):
    """fpgaf_conv3D_svm_batch at 128^3 with the fused x+y pass in the plan."""
    n, b = 128, 2
    keep = cg.plan_variant(n, 4)
    cg.plan_variant(n, 4, 1)
    try:
        rng = np.random.default_rng(23)
        sig, filt = _c64(rng, (b, n, n, n)), _c64(rng, (n, n, n))
        out = np.zeros_like(sig)
        cg.debug_dependency_wait_limit(0)
        t = cg.fpgaf_conv3D_svm_batch(n, sig, filt, out, b)
        assert not t.valid
        assert "device status" in cg.last_error()
        cg.debug_dependency_wait_limit(-1)
        t = cg.fpgaf_conv3D_svm_batch(n, sig, filt, out, b)
        assert t.valid, cg.last_error()
        assert snr_db(conv3d(sig, filt, "fp32"), out) > 120.0
    finally:
        cg.plan_variant(n, 4, keep)


def test_allocation_failure_is_reported_then_the_next_call_allocates(cg):
    """After fpga_final every device buffer is released, so the next calls allocate."""
    rng = np.random.default_rng(24)
    n = 32
    sig, filt = _c64(rng, (n, n, n)), _c64(rng, (n, n, n))
    ref = conv3d(sig, filt, "fp32")
    cg.fpga_final()
    assert cg.fpga_initialize("cuda:0", "convgpu_plans.json", False) == 0
    out = np.zeros_like(sig)
    cg.debug_fail_allocations(1)
    t = cg.fpgaf_conv3D(n, sig, filt, out)
    assert not t.valid
    assert "out of memory" in cg.last_error()
    t = cg.fpgaf_conv3D(n, sig, filt, out)
    assert t.valid, cg.last_error()
    assert snr_db(ref, out) > 120.0
    # device entry point: its workspace is the first allocation it makes
    s, f = torch.from_numpy(sig[None]).cuda(), torch.from_numpy(filt).cuda()
    o = torch.empty_like(s)
    lib = cg.load_library()
    cg.debug_fail_allocations(1)
    assert lib.convgpu_conv3d_device(n, s.data_ptr(), f.data_ptr(), o.data_ptr(), 1, 0, None) == cg.ENOMEM
    cg.conv3d_device(n, s, f, o, 1, 0)
    torch.cuda.synchronize()
    assert snr_db(ref, o.cpu().numpy()[0]) > 120.0
    assert cg.device_status() == 0
