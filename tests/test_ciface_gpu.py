"""The generated `_mlir_ciface_*` entry points on the GPU: called with MLIR
memref descriptors exactly as a reference driver calls them (through ctypes,
and from a compiled C driver of the same shape), the result matches the
oracle within 1e-12."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from golden_util import reference_stencil, resized
from gpu_util import assert_f64_close, run_oracle
from uxxxxxxxxh_gb300 import ciface

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


class Memref3(ctypes.Structure):
    _fields_ = [("allocated", ctypes.c_void_p), ("aligned", ctypes.c_void_p), ("offset", ctypes.c_int64),
                ("sizes", ctypes.c_int64 * 3), ("strides", ctypes.c_int64 * 3)]


class Memref2(ctypes.Structure):
    _fields_ = [("allocated", ctypes.c_void_p), ("aligned", ctypes.c_void_p), ("offset", ctypes.c_int64),
                ("sizes", ctypes.c_int64 * 2), ("strides", ctypes.c_int64 * 2)]


def _memref(t):
    if t.dim() == 3:
        m = Memref3(t.data_ptr(), t.data_ptr(), 0)
        for i in range(3):
            m.sizes[i], m.strides[i] = t.shape[i], t.stride(i)
    else:
        m = Memref2(t.data_ptr(), t.data_ptr(), 0)
        for i in range(2):
            m.sizes[i], m.strides[i] = t.shape[i], t.stride(i)
    return m


@pytest.mark.parametrize("case", ["3d1r_star", "2d1r_star", "3d2r_box", "2d3r_box"])
def test_ctypes_call_of_generated_entry(cuda, tmp_path, case):
    import torch
    st = resized(reference_stencil(case, "gpu"), (20, 24, 66) if case[0] == "3" else (70, 130), iterations=4)
    n = int(np.prod(st.sizes))
    a0 = np.empty(n)
    oracle.fill_rand50([a0])
    so = ciface.build_ciface(st, str(tmp_path))
    lib = ctypes.CDLL(so)
    a = torch.from_numpy(a0.reshape(st.shape)).cuda()
    b = a.clone()
    ma, mb = _memref(a), _memref(b)
    getattr(lib, f"_mlir_ciface_{st.name}_iteration")(ctypes.byref(ma), ctypes.byref(mb))
    torch.cuda.synchronize()
    assert getattr(lib, f"uhs_ciface_status_{st.name}")() == 0
    ra, rb = run_oracle(st, a0)
    assert_f64_close(st, ra, a.cpu().numpy().reshape(-1))
    assert_f64_close(st, rb, b.cpu().numpy().reshape(-1))


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not found")
@pytest.mark.parametrize("case", ["3d1r_star", "2d2r_star"])
def test_compiled_c_driver_calls_generated_entry(cuda, tmp_path, case):
    st = resized(reference_stencil(case, "gpu"), (30, 40, 64) if case[0] == "3" else (100, 200), iterations=4)
    so = ciface.build_ciface(st, str(tmp_path))
    exe = tmp_path / "driver"
    entry = f"_mlir_ciface_{st.name}_iteration"
    r = subprocess.run(["nvcc", "-O2", f"-DUHS_ENTRY={entry}", os.path.join(HERE, "c", "mlir_driver.c"), "-o",
                        str(exe), f"-L{tmp_path}", f"-l{st.name}_ciface", f"-Xlinker", f"-rpath={tmp_path}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = tmp_path / "out.bin"
    Z, Y, X = st.sizes
    r = subprocess.run([str(exe), str(Z), str(Y), str(X), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(out, dtype=np.float64)
    a0 = np.empty(got.size)
    oracle.fill_rand50([a0])  # the driver's rand() % 50 sequence
    ra, _ = run_oracle(st, a0)
    assert_f64_close(st, ra, got)
