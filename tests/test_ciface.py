"""Generated `_mlir_ciface_*` entry points: every reference program's wrapper
compiles against include/uhs.h and exports the symbol UHStencil's compiler
would (no GPU needed)."""
import os
import subprocess

import pytest

from golden_util import load, reference_stencil
from oracle.build_ref import reference_root
from uxxxxxxxxh_gb300 import ciface

CASES = sorted(load("reference_stencils.json"))


@pytest.mark.parametrize("kind", ["sw", "gpu"])
@pytest.mark.parametrize("case", CASES)
def test_wrapper_builds_and_exports_the_reference_symbol(tmp_path, case, kind):
    st = reference_stencil(case, kind)
    name = f"{st.name}_{case}_{kind}"  # 2d3r_star and 2d3r_box share the program name
    so = ciface.build_ciface(st, str(tmp_path), name=name)
    syms = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    assert f"_mlir_ciface_{name}_iteration" in syms
    assert f"uhs_ciface_status_{name}" in syms


def test_single_sweep_program_exports_the_compute_function(tmp_path):
    st = reference_stencil("3d1r_star").with_(iterations=1)
    so = ciface.build_ciface(st, str(tmp_path))
    syms = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    assert f"_mlir_ciface_{st.name}\n" in syms or f"_mlir_ciface_{st.name} " in syms
    assert f"_mlir_ciface_{st.name}_iteration" not in syms


REF_DRIVER = os.path.join(reference_root() or "", "UH-GPU/3d1r_star/3d7pt_main.cpp")


@pytest.mark.skipif(not os.path.exists(REF_DRIVER), reason="reference checkout not present")
def test_reference_gpu_driver_links_against_the_wrapper(tmp_path):
    """The reference's own 3d7pt driver, compiled unmodified, resolves
    _mlir_ciface_stencil_3d7pt_iteration from the generated wrapper (link
    check only: this machine has no GPU to run it)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    st = reference_stencil("3d1r_star", "gpu")
    so = ciface.build_ciface(st, str(tmp_path))
    stub = tmp_path / "driver_api_stub.c"
    stub.write_text('extern "C" { void cuInit(void){} void cuDeviceGet(void){} void cuCtxCreate(void){} }\n')
    exe = tmp_path / "ref_driver"
    r = subprocess.run(["g++", "-O1", "-w", f"-I{root}/oracle/shim/gpu", REF_DRIVER, str(stub),
                        "-o", str(exe), f"-L{tmp_path}", f"-l{st.name}_ciface", f"-L{root}/uxxxxxxxxh_gb300",
                        "-luhs", "-L/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{tmp_path}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    und = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True).stdout
    assert "_mlir_ciface_stencil_3d7pt_iteration" in subprocess.run(
        ["nm", "-D", so], capture_output=True, text=True).stdout
    assert "_mlir_ciface" not in und or "_mlir_ciface_stencil_3d7pt_iteration" in und
