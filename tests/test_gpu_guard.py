"""Guard bands around every operand: no entry point writes outside its output or into its
inputs.

compute-sanitizer is not available on the GPUs these tests run on, so each buffer is carved
out of a larger allocation whose 1 MiB on either side hold a canary bit pattern (a NaN
payload). After the call and a synchronisation the canaries must be intact, the inputs
bit-identical to what was passed (except where the call is in place), and the device status
clean. The routes covered: the per-axis passes and the L2-staged fused x+y pass, the fused z
pass with shared and per-signal filters, the single-cube cooperative launch, real filters as
full and Hermitian half spectra, precomputed spectra, the tensor-core kernels at 256 and
512, uneven batches (per-size graph, work queue, one job at a time), the no-allocation entry
point and the host-buffer pipeline.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CANARY = 0x7FC0DEAD  # a float NaN bit pattern no kernel writes
GUARD = 1 << 20      # bytes on either side


class Guarded:
    """`nbytes` of device memory between two canary bands."""

    def __init__(self, nbytes, dtype=torch.complex64, init=None):
        self.nbytes = nbytes
        self.base = torch.empty(2 * GUARD + nbytes, dtype=torch.uint8, device="cuda")
        self.base.view(torch.int32).fill_(CANARY)
        self.body = self.base[GUARD:GUARD + nbytes].view(dtype)
        if init is not None:
            self.body.copy_(init.reshape(-1).to(dtype))
        self.snapshot = self.body.clone() if init is not None else None

    def guards_intact(self):
        iv = self.base.view(torch.int32)
        g = GUARD // 4
        return bool((iv[:g] == CANARY).all()) and bool((iv[g + self.nbytes // 4:] == CANARY).all())

    def unchanged(self):
        return torch.equal(self.body.view(torch.int32), self.snapshot.view(torch.int32))


def _c64(g, numel):
    return torch.complex(torch.rand(numel, device="cuda", generator=g) * 2 - 1,
                         torch.rand(numel, device="cuda", generator=g) * 2 - 1)


def _check(gpu, inputs, outputs):
    torch.cuda.synchronize()
    for name, buf in inputs.items():
        assert buf.guards_intact(), f"guard band of input {name} written"
        assert buf.unchanged(), f"input {name} modified"
    for name, buf in outputs.items():
        assert buf.guards_intact(), f"guard band of output {name} written"
    assert gpu.device_status() == 0


@pytest.fixture
def plan(gpu):
    """Sets plan kinds for one test and puts them back afterwards."""
    keep = []

    def set_(n, kind, v):
        keep.append((n, kind, gpu.plan_variant(n, kind)))
        gpu.plan_variant(n, kind, v)

    yield set_
    for n, kind, v in reversed(keep):
        gpu.plan_variant(n, kind, v)


# (N, batch, flag names, fused x+y variant for N >= 128)
DEVICE_CASES = [
    (16, 3, (), 0),
    (32, 2, ("FILTER_PER_SIGNAL", "NORMALIZE"), 0),
    (64, 1, (), 0),                       # one cube: one cooperative launch
    (64, 3, ("FILTER_PER_SIGNAL",), 0),
    (128, 2, (), 1),                      # L2-staged x+y
    (128, 2, ("FILTER_PER_SIGNAL",), 0),
    (256, 1, ("FILTER_PER_SIGNAL",), 1),
    (256, 2, (), 0),
    (256, 1, ("FILTER_PER_SIGNAL", "TENSOR_SPLIT"), 0),
    (512, 1, ("NORMALIZE",), 1),
    (512, 1, ("TENSOR_SPLIT",), 0),
]


@pytest.mark.parametrize("n,b,flag_names,xy", DEVICE_CASES)
def test_device_entry_point_stays_in_bounds(gpu, plan, n, b, flag_names, xy):
    if n >= 128:
        plan(n, 4, xy)
    flags = 0
    for f in flag_names:
        flags |= getattr(gpu, f)
    g = torch.Generator(device="cuda").manual_seed(n + b)
    vol = n ** 3
    nf = b if flags & gpu.FILTER_PER_SIGNAL else 1
    sig = Guarded(b * vol * 8, init=_c64(g, b * vol))
    filt = Guarded(nf * vol * 8, init=_c64(g, nf * vol))
    out = Guarded(b * vol * 8)
    gpu.conv3d_device(n, sig.body, filt.body, out.body, b, flags)
    _check(gpu, {"signal": sig, "filter": filt}, {"output": out})
    assert bool(torch.isfinite(out.body.view(torch.float32)).all())


@pytest.mark.parametrize("n,half", [(64, 0), (128, 1), (256, 1), (512, 1), (512, 0)])
def test_real_filters_stay_in_bounds(gpu, plan, n, half):
    plan(n, 7, half)
    g = torch.Generator(device="cuda").manual_seed(7 * n + half)
    vol = n ** 3
    sig = Guarded(vol * 8, init=_c64(g, vol))
    filt = Guarded(vol * 4, dtype=torch.float32, init=torch.rand(vol, device="cuda", generator=g))
    out = Guarded(vol * 8)
    gpu.conv3d_device(n, sig.body, filt.body, out.body, 1, gpu.FILTER_REAL | gpu.NORMALIZE)
    _check(gpu, {"signal": sig, "filter": filt}, {"output": out})


def test_in_place_and_precomputed_spectra_stay_in_bounds(gpu):
    n, b = 128, 2
    vol = n ** 3
    g = torch.Generator(device="cuda").manual_seed(3)
    filt = Guarded(vol * 8, init=_c64(g, vol))
    spec = Guarded(vol * 8)
    gpu.filter_spectrum_device(n, filt.body, spec.body, 1)
    _check(gpu, {"filter": filt}, {"spectrum": spec})
    spec.snapshot = spec.body.clone()
    io = Guarded(b * vol * 8, init=_c64(g, b * vol))
    gpu.conv3d_device(n, io.body, spec.body, io.body, b, gpu.FILTER_IS_SPECTRUM)
    _check(gpu, {"spectrum": spec}, {"in-place signal": io})


def test_no_alloc_entry_point_stays_in_bounds(gpu):
    g = torch.Generator(device="cuda").manual_seed(5)
    for n, b, per_signal in ((32, 3, True), (64, 2, False), (128, 1, False)):
        vol = n ** 3
        flags = gpu.FILTER_PER_SIGNAL if per_signal else 0
        sig = Guarded(b * vol * 8, init=_c64(g, b * vol))
        filt = Guarded((b if per_signal else 1) * vol * 8, init=_c64(g, (b if per_signal else 1) * vol))
        out = Guarded(b * vol * 8)
        gpu.conv3d_device_noalloc(n, sig.body, filt.body, out.body, b, flags)
        _check(gpu, {"signal": sig, "filter": filt}, {"output": out})


@pytest.mark.parametrize("mode", ["graph", "queue", "per_job"])
def test_uneven_batch_stays_in_its_jobs(gpu, plan, mode):
    """Jobs of four sizes laid out with canary gaps between them: every gap and every input
    stays as it was."""
    plan(256, 4, 1)
    sizes = [32, 256, 64, 128, 32, 64]
    gap = GUARD // 8  # complex elements between jobs
    offs, o = [], gap
    for n in sizes:
        offs.append(o)
        o += n ** 3 + gap
    total = o
    g = torch.Generator(device="cuda").manual_seed(11)
    sig = Guarded(total * 8)
    filt = Guarded(total * 8)
    out = Guarded(total * 8)
    for n, off in zip(sizes, offs):
        sig.body[off:off + n ** 3] = _c64(g, n ** 3)
        filt.body[off:off + n ** 3] = _c64(g, n ** 3)
    sig.snapshot, filt.snapshot = sig.body.clone(), filt.body.clone()
    out_before = out.body.clone()
    flags = {"graph": 0, "queue": gpu.UNEVEN_QUEUE, "per_job": gpu.UNEVEN_PER_JOB}[mode]
    jobs = [(n, off, off, off) for n, off in zip(sizes, offs)]
    gpu.conv3d_uneven_device(jobs, sig.body, filt.body, out.body, flags | gpu.NORMALIZE)
    _check(gpu, {"signals": sig, "filters": filt}, {"outputs": out})
    written = torch.zeros(total, dtype=torch.bool, device="cuda")
    for n, off in zip(sizes, offs):
        written[off:off + n ** 3] = True
    gaps = ~written
    assert torch.equal(out.body[gaps].view(torch.int32), out_before[gaps].view(torch.int32))


def test_host_pipeline_stays_in_bounds(gpu):
    """convgpu_conv3d_host on numpy buffers with canary bands: copies move exactly the
    operands' bytes."""
    n, b = 64, 5
    vol = n ** 3
    rng = np.random.default_rng(13)
    band = GUARD // 8

    def carve(count, fill):
        a = np.empty(2 * band + count * vol, np.complex64)
        a.view(np.int32)[...] = CANARY
        body = a[band:band + count * vol]
        if fill:
            body.real = rng.uniform(-1, 1, body.shape)
            body.imag = rng.uniform(-1, 1, body.shape)
        return a, body

    sa, sb = carve(b, True)
    fa, fb = carve(b, True)
    oa, ob = carve(b, False)
    s0, f0 = sa.copy(), fa.copy()
    t = gpu.conv3d_host(n, sb.reshape(b, n, n, n), fb.reshape(b, n, n, n), ob.reshape(b, n, n, n), b,
                        gpu.FILTER_PER_SIGNAL)
    assert t.valid, gpu.last_error()
    assert np.array_equal(sa.view(np.int32), s0.view(np.int32))
    assert np.array_equal(fa.view(np.int32), f0.view(np.int32))
    ov = oa.view(np.int32)
    assert (ov[:2 * band] == CANARY).all() and (ov[2 * (band + b * vol):] == CANARY).all()
    assert np.isfinite(ob).all()
