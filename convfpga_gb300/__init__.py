"""GB300 FFT-based 3D convolution: Python mirror of the convfpga.h C API.

Every call goes through the C ABI of ``libconvgpu.so`` (built in-tree by
``convfpga_gb300.build``); there is no Python or CPU compute path. If the library is
missing, importing the bindings raises instead of falling back.

Reference entry points (host/include/convfpga/convfpga.h:36-46 of pc2/ConvFPGA) keep
their names and meaning:

    fpga_initialize(platform_name, path, use_svm) -> int
    fpga_final()
    fpgaf_conv3D(N, sig, filter, out) -> FpgaT
    fpgaf_conv3D_svm(N, sig, filter, out) -> FpgaT
    fpgaf_conv3D_svm_batch(N, sig, filter, out, how_many) -> FpgaT

``sig``/``filter``/``out`` are host arrays of complex64 (numpy arrays or anything with
the buffer protocol / ``ctypes`` address). The extensions of convgpu.h are exposed as
``conv3d_device`` (device pointers, e.g. ``torch`` CUDA tensors), ``conv3d_host``,
``filter_spectrum_device`` and ``conv3d_uneven_device``.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libconvgpu.so")

NORMALIZE = 1 << 0
FILTER_PER_SIGNAL = 1 << 1
FILTER_IS_SPECTRUM = 1 << 2
TENSOR_SPLIT = 1 << 3
TENSOR_BF16X3 = 1 << 4
UNEVEN_PER_JOB = 1 << 5
UNEVEN_QUEUE = 1 << 6
HOST_SLABS = 1 << 7
FILTER_CACHED = 1 << 8
FILTER_REAL = 1 << 9

OK, EINVAL, ENOTINIT, ECUDA, ENOMEM, EUNSUPPORTED = 0, -1, -2, -3, -4, -5

#: Every symbol the C ABI exports (include/convfpga.h and include/convgpu.h).
EXPORTED_SYMBOLS = (
    "fpga_initialize",
    "fpga_final",
    "fpgaf_complex_malloc",
    "fpgaf_conv3D",
    "fpgaf_conv3D_svm",
    "fpgaf_conv3D_svm_batch",
    "convgpu_conv3d_device",
    "convgpu_conv3d_device_noalloc",
    "convgpu_conv3d_host",
    "convgpu_filter_spectrum_device",
    "convgpu_conv3d_uneven_device",
    "convgpu_workspace_bytes",
    "convgpu_host_alloc",
    "convgpu_host_free",
    "convgpu_device_info",
    "convgpu_launch_count",
    "convgpu_pass_timing",
    "convgpu_synchronize",
    "convgpu_device_status",
    "convgpu_autotune",
    "convgpu_plan_variant",
    "convgpu_debug_dependency_wait_limit",
    "convgpu_debug_fail_allocations",
    "convgpu_last_error",
)


class FpgaTiming(ctypes.Structure):
    """``fpga_t`` (host/include/convfpga/convfpga.h:24-34): milliseconds + valid."""

    _fields_ = [
        ("filter_pcie_wr_t", ctypes.c_double),
        ("filter_exec_t", ctypes.c_double),
        ("sig_pcie_wr_t", ctypes.c_double),
        ("sig_pcie_rd_t", ctypes.c_double),
        ("sig_exec_t", ctypes.c_double),
        ("siginv_exec_t", ctypes.c_double),
        ("valid", ctypes.c_bool),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class Job(ctypes.Structure):
    """``convgpu_job``: one convolution of an uneven batch."""

    _fields_ = [
        ("n", ctypes.c_uint),
        ("sig_offset", ctypes.c_ulonglong),
        ("filter_offset", ctypes.c_ulonglong),
        ("out_offset", ctypes.c_ulonglong),
    ]


class ConvGpuError(RuntimeError):
    pass


_lib = None


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Loads libconvgpu.so and declares every C signature. Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ConvGpuError(f"{p} not built: run `python -m convfpga_gb300.build` (no fallback path exists)")
    lib = ctypes.CDLL(p)
    vp, u, c_f2 = ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p
    lib.fpga_initialize.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_bool]
    lib.fpga_initialize.restype = ctypes.c_int
    lib.fpga_final.argtypes = []
    lib.fpga_final.restype = None
    lib.fpgaf_complex_malloc.argtypes = [ctypes.c_size_t]
    lib.fpgaf_complex_malloc.restype = vp
    for fn in ("fpgaf_conv3D", "fpgaf_conv3D_svm"):
        getattr(lib, fn).argtypes = [u, c_f2, c_f2, c_f2]
        getattr(lib, fn).restype = FpgaTiming
    lib.fpgaf_conv3D_svm_batch.argtypes = [u, c_f2, c_f2, c_f2, u]
    lib.fpgaf_conv3D_svm_batch.restype = FpgaTiming
    lib.convgpu_conv3d_device.argtypes = [u, vp, vp, vp, u, u, vp]
    lib.convgpu_conv3d_device.restype = ctypes.c_int
    lib.convgpu_conv3d_device_noalloc.argtypes = [u, vp, vp, vp, u, u, vp]
    lib.convgpu_conv3d_device_noalloc.restype = ctypes.c_int
    lib.convgpu_conv3d_host.argtypes = [u, vp, vp, vp, u, u]
    lib.convgpu_conv3d_host.restype = FpgaTiming
    lib.convgpu_filter_spectrum_device.argtypes = [u, vp, vp, u, vp]
    lib.convgpu_filter_spectrum_device.restype = ctypes.c_int
    lib.convgpu_conv3d_uneven_device.argtypes = [ctypes.POINTER(Job), u, vp, vp, vp, u, vp]
    lib.convgpu_conv3d_uneven_device.restype = ctypes.c_int
    lib.convgpu_workspace_bytes.argtypes = [u, u, u, ctypes.POINTER(ctypes.c_size_t)]
    lib.convgpu_workspace_bytes.restype = ctypes.c_int
    lib.convgpu_host_alloc.argtypes = [ctypes.c_size_t, ctypes.POINTER(vp)]
    lib.convgpu_host_alloc.restype = ctypes.c_int
    lib.convgpu_host_free.argtypes = [vp]
    lib.convgpu_host_free.restype = ctypes.c_int
    lib.convgpu_device_info.argtypes = [ctypes.POINTER(ctypes.c_int)] * 3
    lib.convgpu_device_info.restype = ctypes.c_int
    lib.convgpu_launch_count.argtypes = []
    lib.convgpu_launch_count.restype = ctypes.c_ulonglong
    lib.convgpu_pass_timing.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_double)]
    lib.convgpu_pass_timing.restype = ctypes.c_int
    lib.convgpu_synchronize.argtypes = []
    lib.convgpu_synchronize.restype = ctypes.c_int
    lib.convgpu_device_status.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    lib.convgpu_device_status.restype = ctypes.c_int
    lib.convgpu_autotune.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_uint, ctypes.c_int]
    lib.convgpu_autotune.restype = ctypes.c_int
    lib.convgpu_plan_variant.argtypes = [ctypes.c_uint, ctypes.c_int, ctypes.c_int]
    lib.convgpu_plan_variant.restype = ctypes.c_int
    lib.convgpu_debug_dependency_wait_limit.argtypes = [ctypes.c_int]
    lib.convgpu_debug_dependency_wait_limit.restype = ctypes.c_int
    lib.convgpu_debug_fail_allocations.argtypes = [ctypes.c_uint]
    lib.convgpu_debug_fail_allocations.restype = ctypes.c_int
    lib.convgpu_last_error.argtypes = []
    lib.convgpu_last_error.restype = ctypes.c_char_p
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    return (load_library().convgpu_last_error() or b"").decode()


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise ConvGpuError(f"{what} failed ({rc}): {last_error()}")


def _host_ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        # complex64; float32 for real filters (FILTER_REAL)
        if a.dtype not in (np.complex64, np.float32) or not a.flags.c_contiguous:
            raise TypeError("host arrays must be C-contiguous complex64 (or float32 real filters)")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):  # CPU torch tensor (e.g. pinned)
        return a.data_ptr()
    raise TypeError(f"unsupported host buffer {type(a)!r}")


def _dev_ptr(t) -> int | None:
    if t is None:
        return None
    if isinstance(t, int):
        return t
    return t.data_ptr()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


# ------------------------------------------------------------------ reference API
def fpga_initialize(platform_name: str | None = "cuda:0", path: str | None = "convgpu_plans.json",
                    use_svm: bool = False) -> int:
    lib = load_library()
    pn = platform_name.encode() if platform_name is not None else None
    pa = path.encode() if path is not None else None
    return lib.fpga_initialize(pn, pa, use_svm)


def fpga_final() -> None:
    load_library().fpga_final()


def fpgaf_conv3D(n: int, sig, filt, out) -> FpgaTiming:
    return load_library().fpgaf_conv3D(n, _host_ptr(sig), _host_ptr(filt), _host_ptr(out))


def fpgaf_conv3D_svm(n: int, sig, filt, out) -> FpgaTiming:
    return load_library().fpgaf_conv3D_svm(n, _host_ptr(sig), _host_ptr(filt), _host_ptr(out))


def fpgaf_conv3D_svm_batch(n: int, sig, filt, out, how_many: int) -> FpgaTiming:
    return load_library().fpgaf_conv3D_svm_batch(n, _host_ptr(sig), _host_ptr(filt), _host_ptr(out), how_many)


# ------------------------------------------------------------------ extensions
def conv3d_device(n: int, sig, filt, out, how_many: int, flags: int = 0, stream=None) -> None:
    """Device-pointer batch (torch CUDA tensors or raw addresses); raises on error."""
    rc = load_library().convgpu_conv3d_device(n, _dev_ptr(sig), _dev_ptr(filt), _dev_ptr(out), how_many, flags,
                                              _stream_ptr(stream))
    _check(rc, "convgpu_conv3d_device")


NOALLOC_SCRATCH_ELEMS = 1 << 21


def conv3d_device_noalloc(n: int, sig, filt, out, how_many: int, flags: int = 0, stream=None) -> None:
    """Like conv3d_device, for callers that cannot allocate device memory: its scratch
    is a fixed 16 MiB array inside the library (NOALLOC_SCRATCH_ELEMS complex values),
    shared by all calls (overlapping calls race). Raises on error."""
    rc = load_library().convgpu_conv3d_device_noalloc(n, _dev_ptr(sig), _dev_ptr(filt), _dev_ptr(out), how_many,
                                                      flags, _stream_ptr(stream))
    _check(rc, "convgpu_conv3d_device_noalloc")


def conv3d_host(n: int, sig, filt, out, how_many: int, flags: int = 0) -> FpgaTiming:
    return load_library().convgpu_conv3d_host(n, _host_ptr(sig), _host_ptr(filt), _host_ptr(out), how_many, flags)


def filter_spectrum_device(n: int, filt, spec, count: int = 1, stream=None) -> None:
    rc = load_library().convgpu_filter_spectrum_device(n, _dev_ptr(filt), _dev_ptr(spec), count, _stream_ptr(stream))
    _check(rc, "convgpu_filter_spectrum_device")


def conv3d_uneven_device(jobs, sig_base, filt_base, out_base, flags: int = 0, stream=None) -> None:
    """jobs: sequence of (n, sig_offset, filter_offset, out_offset) in complex elements."""
    arr = (Job * len(jobs))(*[Job(*j) for j in jobs])
    rc = load_library().convgpu_conv3d_uneven_device(arr, len(jobs), _dev_ptr(sig_base), _dev_ptr(filt_base),
                                                     _dev_ptr(out_base), flags, _stream_ptr(stream))
    _check(rc, "convgpu_conv3d_uneven_device")


def workspace_bytes(n: int, how_many: int, flags: int = 0) -> int:
    v = ctypes.c_size_t(0)
    _check(load_library().convgpu_workspace_bytes(n, how_many, flags, ctypes.byref(v)), "convgpu_workspace_bytes")
    return int(v.value)


def device_info() -> dict:
    d, p, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(load_library().convgpu_device_info(ctypes.byref(d), ctypes.byref(p), ctypes.byref(s)), "device_info")
    return {"device": d.value, "pageable_access": p.value, "sm_count": s.value}


def launch_count() -> int:
    return int(load_library().convgpu_launch_count())


PASS_SLOTS = 14
PASS_AXES = ("x", "y", "z")
PASS_OPS = ("fwd", "inv", "conv", "conv_fz")


def pass_timing_start() -> None:
    _check(load_library().convgpu_pass_timing(1, None, None, None), "convgpu_pass_timing")


def pass_timing_stop() -> None:
    _check(load_library().convgpu_pass_timing(0, None, None, None), "convgpu_pass_timing")


def pass_timing_read() -> dict:
    """{"y-fwd": {"ms": total, "launches": k, "bytes": algorithmic bytes}, ...}"""
    ms = (ctypes.c_double * PASS_SLOTS)()
    cnt = (ctypes.c_ulonglong * PASS_SLOTS)()
    by = (ctypes.c_double * PASS_SLOTS)()
    _check(load_library().convgpu_pass_timing(2, ms, cnt, by), "convgpu_pass_timing")
    out = {}
    for i in range(PASS_SLOTS):
        if cnt[i]:
            name = f"{PASS_AXES[i // 4]}-{PASS_OPS[i % 4]}" if i < 12 else ("xy-fwd", "xy-inv")[i - 12]
            out[name] = {"ms": ms[i], "launches": int(cnt[i]), "bytes": by[i]}
    return out


PLAN_KINDS = ("rows", "strided", "conv", "conv_fz", "xy", "tc", "tcxy", "herm")


def autotune(sizes, write_cache: bool = True) -> None:
    """Times both shape variants per pass kind for each size and keeps the faster."""
    arr = (ctypes.c_uint * len(sizes))(*sizes)
    _check(load_library().convgpu_autotune(arr, len(sizes), 1 if write_cache else 0), "convgpu_autotune")


def plan_variant(n: int, kind: int, set_to: int = -1) -> int:
    v = load_library().convgpu_plan_variant(n, kind, set_to)
    if v < 0:
        raise ConvGpuError(f"convgpu_plan_variant failed ({v}): {last_error()}")
    return v


def device_status() -> int:
    """Waits for the device; returns and clears the status word (0 = all kernels normal)."""
    v = ctypes.c_uint(0)
    _check(load_library().convgpu_device_status(ctypes.byref(v)), "convgpu_device_status")
    return int(v.value)


def debug_dependency_wait_limit(probes: int) -> None:
    """Testing hook: dependency waits give up after `probes` probes (< 0: default)."""
    _check(load_library().convgpu_debug_dependency_wait_limit(probes), "convgpu_debug_dependency_wait_limit")


def debug_fail_allocations(count: int) -> None:
    """Testing hook: the next `count` device-buffer allocations fail as out of memory."""
    _check(load_library().convgpu_debug_fail_allocations(count), "convgpu_debug_fail_allocations")


def synchronize() -> None:
    _check(load_library().convgpu_synchronize(), "convgpu_synchronize")


@dataclass
class ComplexMalloc:
    """Host block from fpgaf_complex_malloc (64-byte aligned, pageable), the buffers a
    reference caller hands to the conv entry points (src/main.cpp:64-74 of pc2/ConvFPGA);
    released with the C library's free(), as the reference's callers do."""

    ptr: int
    nbytes: int

    @classmethod
    def alloc(cls, nbytes: int) -> "ComplexMalloc":
        p = load_library().fpgaf_complex_malloc(nbytes)
        if not p:
            raise ConvGpuError(f"fpgaf_complex_malloc({nbytes}) returned NULL")
        return cls(int(p), nbytes)

    def array(self, shape) -> np.ndarray:
        count = int(np.prod(shape))
        buf = (ctypes.c_char * (count * 8)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=np.complex64, count=count).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            libc = ctypes.CDLL(None)
            libc.free.argtypes = [ctypes.c_void_p]
            libc.free.restype = None
            libc.free(self.ptr)
            self.ptr = 0


@dataclass
class PinnedBuffer:
    """Page-locked host block from convgpu_host_alloc, viewed as complex64."""

    ptr: int
    nbytes: int

    @classmethod
    def alloc(cls, nbytes: int) -> "PinnedBuffer":
        p = ctypes.c_void_p()
        _check(load_library().convgpu_host_alloc(nbytes, ctypes.byref(p)), "convgpu_host_alloc")
        return cls(int(p.value or 0), nbytes)

    def array(self, shape) -> np.ndarray:
        count = int(np.prod(shape))
        buf = (ctypes.c_char * (count * 8)).from_address(self.ptr)
        return np.frombuffer(buf, dtype=np.complex64, count=count).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            _check(load_library().convgpu_host_free(self.ptr), "convgpu_host_free")
            self.ptr = 0
