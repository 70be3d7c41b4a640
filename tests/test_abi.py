"""C-ABI checks that need no GPU: the library loads, exports exactly what include/*.h
declares, and rejects bad arguments the way the reference does, before touching CUDA."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import convfpga_gb300 as cg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions() -> set[str]:
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
        for m in re.finditer(r"\b([A-Za-z_]\w*)\s*\(([^;{}()]*)\)\s*;", text):
            names.add(m.group(1))
    return names


def test_headers_declare_the_python_symbol_list():
    assert _declared_functions() == set(cg.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(built_lib):
    for name in _declared_functions():
        assert hasattr(built_lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", cg.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert _declared_functions() <= exported


def test_reference_entry_points_are_the_same_names():
    ref = {"fpga_initialize", "fpga_final", "fpgaf_complex_malloc", "fpgaf_conv3D", "fpgaf_conv3D_svm",
           "fpgaf_conv3D_svm_batch"}
    assert ref <= _declared_functions()


def test_initialize_rejects_missing_path(built_lib):
    assert cg.fpga_initialize("cuda:0", None) == -1
    assert cg.fpga_initialize("cuda:0", "") == -1


def test_complex_malloc(built_lib):
    assert built_lib.fpgaf_complex_malloc(0) is None
    p = built_lib.fpgaf_complex_malloc(1000)
    assert p and p % 64 == 0
    ctypes.CDLL(None).free(ctypes.c_void_p(p))


def test_conv_rejects_bad_arguments_without_a_gpu(built_lib):
    a = np.zeros(16 ** 3, np.complex64)
    for n in (0, 3, 100, 1024, 8):
        assert not cg.fpgaf_conv3D(n, a, a, a).valid
    assert not cg.fpgaf_conv3D(16, None, a, a).valid
    assert not cg.fpgaf_conv3D_svm(16, a, None, a).valid
    assert not cg.fpgaf_conv3D_svm_batch(16, a, a, None, 1).valid
    assert not cg.fpgaf_conv3D_svm_batch(16, a, a, a, 0).valid
    assert built_lib.convgpu_conv3d_device(100, 1, 1, 1, 1, 0, None) == cg.EINVAL
    assert built_lib.convgpu_conv3d_device(16, None, 1, 1, 1, 0, None) == cg.EINVAL
    assert cg.last_error() != ""


def test_workspace_bytes(built_lib):
    v = 64 ** 3 * 8
    assert cg.workspace_bytes(64, 4) == v
    assert cg.workspace_bytes(64, 4, cg.FILTER_PER_SIGNAL) == 4 * v
    assert cg.workspace_bytes(64, 4, cg.FILTER_IS_SPECTRUM) == 0
    with pytest.raises(cg.ConvGpuError):
        cg.workspace_bytes(60, 1)


def test_fpga_t_layout():
    assert ctypes.sizeof(cg.FpgaTiming) == 56
    assert ctypes.sizeof(cg.Job) == 32


def test_flag_and_code_constants_match_the_header():
    """Every CONVGPU_* flag and return code in include/convgpu.h has the same value in the
    Python mirror (the mirror is how the tests and the bench pass them)."""
    import re

    text = open(os.path.join(ROOT, "include", "convgpu.h")).read()
    defs = dict(re.findall(r"#define CONVGPU_(\w+)\s+\(?(1u << \d+|-?\d+)\)?", text))
    checked = 0
    for name, val in defs.items():
        if not hasattr(cg, name):
            continue
        v = 1 << int(val.split("<<")[1]) if "<<" in val else int(val)
        assert getattr(cg, name) == v, name
        checked += 1
    for flag in ("NORMALIZE", "FILTER_PER_SIGNAL", "FILTER_IS_SPECTRUM", "TENSOR_SPLIT", "TENSOR_BF16X3",
                 "UNEVEN_PER_JOB", "UNEVEN_QUEUE", "HOST_SLABS", "FILTER_CACHED", "FILTER_REAL"):
        assert flag in defs and hasattr(cg, flag), flag
    assert checked >= 10


def test_uneven_batch_rejects_malformed_jobs_without_a_gpu(built_lib):
    """Descriptors are checked before anything runs (the base addresses below are never
    dereferenced): unsupported sizes, offsets past the address space, outputs that overlap
    another job's output or part of the job's own signal."""
    base = 1 << 20

    def call(jobs, same_io=False):
        arr = (cg.Job * len(jobs))(*[cg.Job(*j) for j in jobs])
        out = base if same_io else base + (1 << 30)
        return built_lib.convgpu_conv3d_uneven_device(arr, len(jobs), base, base + (1 << 29), out, 0, None)

    v = 32 ** 3
    assert call([(48, 0, 0, 0)]) == cg.EINVAL
    assert "size 48" in cg.last_error()
    assert call([(32, 0, 0, 1 << 62)]) == cg.EINVAL                  # byte offset wraps
    assert "address space" in cg.last_error()
    assert call([(32, 0, 0, 0), (32, v, v, v - 1)]) == cg.EINVAL     # outputs overlap by one value
    assert "overlap" in cg.last_error()
    assert call([(32, 0, 0, 10)], same_io=True) == cg.EINVAL         # shifted in-place output
    assert "own signal" in cg.last_error()
