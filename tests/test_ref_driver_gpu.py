"""The reference's own GPU drivers, run end to end on the GPU.

UH-GPU/3d1r_star/3d7pt_main.cpp (512^3, T = 4) and UH-GPU/2d1r_star/
2d5pt_main.cpp (8192^2, T = 4) fill their grids with rand() % 50, copy the
input to the device, call _mlir_ciface_stencil_<n>pt_iteration
(3d7pt_main.cpp:147-150) and check the device result against their own CPU
loop, cpu_verify (3d7pt_main.cpp:50-103: |cpu - gpu| <= 1e-6 on every
interior cell), printing "Verfiy Success" (their spelling) or "Verify
Failed".  Here each driver, compiled unmodified, is linked to the wrapper
ciface.py generates from the case's .dsl program (the drop-in for what
UHStencil's compiler emits) and run; it must report success.

The driver sources come from the reference checkout: oracle/build_ref.py
copies them into oracle/_ref/drivers/ (git-ignored).  Where that copy is
absent the test is skipped."""
import os
import subprocess

import pytest

from golden_util import reference_stencil
from oracle import build_ref
from uxxxxxxxxh_gb300 import ciface
from uxxxxxxxxh_gb300._lib import PKG

pytestmark = pytest.mark.gpu

CUDA_LIB = "/usr/local/cuda/lib64"


@pytest.mark.parametrize("case", sorted(build_ref.GPU_DRIVER_RUNS))
def test_reference_gpu_driver_verifies_the_wrapper(cuda, tmp_path, case):
    if not os.path.exists(build_ref.gpu_driver_source(case)):
        pytest.skip("reference driver source not present (oracle/build_ref.py copies it from the checkout)")
    st = reference_stencil(case, "gpu")
    ciface.build_ciface(st, str(tmp_path))
    exe = build_ref.build_gpu_driver(case, str(tmp_path), f"{st.name}_ciface", [str(tmp_path), PKG, CUDA_LIB])
    r = subprocess.run([exe], cwd=str(tmp_path), capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "Verfiy Success" in r.stdout and "Verify Failed" not in r.stdout, r.stdout[-2000:]
    assert "_mlir_ciface" not in r.stderr, r.stderr[-2000:]  # the wrapper reports a failed call there
