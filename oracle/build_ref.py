"""Compile the reference's own serial stencil drivers into oracle/_ref/.

(Also: the spatially fused program's driver as an executable, and copies of
two UH-GPU drivers for the end-to-end run on a GPU machine; see below.)

TEST INFRASTRUCTURE ONLY.  The shared objects made here are the reference
implementation that the C oracle (oracle/uhs_oracle.c) is pinned against; the
library never loads them.

Each UHStencil case directory holds a self-contained C (UH-SW) or C++ (UH-GPU)
driver whose CPU loop (mpe_verify / cpu_verify) is the reference CPU path.  The
drivers are compiled unmodified, straight from where they lie in the
reference checkout, with:
  * oracle/shim/athread.h standing in for the Sunway runtime header, and
    oracle/shim/gpu/cuda*.h declaring the few CUDA calls of the GPU drivers'
    main() (the installed CUDA headers changed cuCtxCreate's arguments),
  * -Dmain=uhs_ref_unused_main so the driver's main() is never run,
  * a generated stub file that defines every symbol the driver leaves
    undefined outside libc (the device entry point, the CUDA calls of the GPU
    drivers' main()); none of them is ever called.
Flags: gcc/g++ -O2 -ffp-contract=off, the same as the oracle.

Usage: python oracle/build_ref.py [REFERENCE_ROOT]
The checkout is found through reference_root(): the UHS_REFERENCE_ROOT
environment variable, else the checkout's location on the build machine.
Nothing is built when it is absent.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SHIM = os.path.join(HERE, "shim")
# where the reference checkout lies on the machine that builds the checker;
# UHS_REFERENCE_ROOT overrides it
_DEFAULT_ROOT = "/root/reference"


def reference_root() -> str | None:
    """The reference checkout, or None where it is absent (GPU machines)."""
    root = os.environ.get("UHS_REFERENCE_ROOT") or _DEFAULT_ROOT
    return root if os.path.isdir(os.path.join(root, "UH-SW")) else None

# case -> (UH-SW driver, UH-GPU driver), paths relative to the reference root
CASES = {
    "2d1r_star": ("UH-SW/2d1r_star/stencil_2d5pt_driver.serial.c", "UH-GPU/2d1r_star/2d5pt_main.cpp"),
    "2d2r_star": ("UH-SW/2d2r_star/stencil_2d9pt_driver.serial.c", "UH-GPU/2d2r_star/2d9pt_main.cpp"),
    "2d3r_star": ("UH-SW/2d3r_star/stencil_2d13pt_driver.serial.c", "UH-GPU/2d3r_star/2d3r_main.cpp"),
    "2d1r_box": ("UH-SW/2d1r_box/stencil_2d9pt_driver.serial.c", "UH-GPU/2d1r_box/2d9pt_main.cpp"),
    "2d2r_box": ("UH-SW/2d2r_box/stencil_2d25pt_driver.serial.c", "UH-GPU/2d2r_box/2d25pt_main.cpp"),
    "2d3r_box": ("UH-SW/2d3r_box/stencil_2d49pt_driver.serial.c", "UH-GPU/2d3r_box/2d3r_main.cpp"),
    "3d1r_star": ("UH-SW/3d1r_star/stencil_3d7pt_driver.serial.c", "UH-GPU/3d1r_star/3d7pt_main.cpp"),
    "3d2r_star": ("UH-SW/3d2r_star/stencil_3d13pt_driver.serial.c", "UH-GPU/3d2r_star/3d13pt_main.cpp"),
    "3d3r_star": ("UH-SW/3d3r_star/stencil_3d19pt_driver.serial.c", "UH-GPU/3d3r_star/3d3r_main.cpp"),
    "3d1r_box": ("UH-SW/3d1r_box/stencil_3d27pt_driver.serial.c", "UH-GPU/3d1r_box/3d27pt_main.cpp"),
    "3d2r_box": ("UH-SW/3d2r_box/stencil_3d125pt_driver.serial.c", "UH-GPU/3d2r_box/3d125pt_main.cpp"),
    "3d3r_box": ("UH-SW/3d3r_box/stencil_3d343pt_driver.serial.c", "UH-GPU/3d3r_box/3d3r_main.cpp"),
}


# Spatial kernel fusion (lib/Dialect/Stencil/StencilKernelFusion.cpp:70-183):
# the program `laplaceAddInput` inlines its producer kernel into the consumer
# (test/Examples/StencilDialect/laplaceAddInputIteration/*.dsl).  Its driver
# runs the fused serial loop inside main() (laplaceAddInputIteration_driver.c:
# 37-58) and writes the grid to the file mpe_result, so it is built as an
# executable and run in a scratch directory.
FUSION = ("fusion_laplaceAddInputIteration",
          "UHStencil/test/Examples/StencilDialect/laplaceAddInputIteration/laplaceAddInputIteration_driver.c")
FUSION_DSL = "UHStencil/test/Examples/StencilDialect/laplaceAddInputIteration/laplaceAddInputIteration.dsl"


# The reference's GPU drivers, run end to end against the generated
# _mlir_ciface_* wrappers on a GPU machine, which has no reference checkout:
# build() copies these driver sources, unmodified, into oracle/_ref/drivers/
# (git-ignored, like everything under oracle/_ref), and the GPU test compiles
# them there (build_gpu_driver).
GPU_DRIVER_RUNS = {"3d1r_star": "UH-GPU/3d1r_star/3d7pt_main.cpp", "2d1r_star": "UH-GPU/2d1r_star/2d5pt_main.cpp"}
DRIVERS = os.path.join(OUT, "drivers")


def gpu_driver_source(case: str) -> str:
    return os.path.join(DRIVERS, f"gpu_{case}_main.cpp")


def build_gpu_driver(case: str, out_dir: str, ciface_lib: str, lib_dirs: "list[str]") -> str:
    """Compile the copied driver of `case` into out_dir/ref_driver_<case>,
    linked to the generated wrapper library (lib<ciface_lib>.so), libuhs.so
    and the CUDA runtime.  The driver's three driver-API calls (cuInit,
    cuDeviceGet, cuCtxCreate, whose cuCtxCreate signature CUDA 13's headers no
    longer have) are no-op stubs: the runtime calls after them use the
    device's primary context, as do the library's."""
    exe = os.path.join(out_dir, f"ref_driver_{case}")
    stub = os.path.join(out_dir, "driver_api_stub.c")
    with open(stub, "w") as f:
        f.write("int cuInit(unsigned f) { (void)f; return 0; }\n"
                "int cuDeviceGet(int *d, int o) { *d = o; return 0; }\n"
                "int cuCtxCreate(void **c, unsigned f, int d) { (void)f; (void)d; *c = 0; return 0; }\n")
    stub_o = stub[:-2] + ".o"
    _run(["gcc", "-O2", "-c", stub, "-o", stub_o])
    cmd = ["g++", "-O2", "-w", f"-I{os.path.join(SHIM, 'gpu')}", gpu_driver_source(case), stub_o, "-o", exe,
           f"-l{ciface_lib}", "-luhs", "-lcudart"]
    for d in lib_dirs:
        cmd[-3:-3] = [f"-L{d}", f"-Wl,-rpath,{d}"]
    _run(cmd)
    return exe


def _copy_gpu_drivers(ref_root: str) -> "list[str]":
    os.makedirs(DRIVERS, exist_ok=True)
    out = []
    for case, rel in GPU_DRIVER_RUNS.items():
        dst = gpu_driver_source(case)
        with open(os.path.join(ref_root, rel), "rb") as f, open(dst, "wb") as g:
            g.write(f.read())
        out.append(dst)
    return out


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _undefined(obj: str, prefixes=("cu", "_mlir_ciface_", "stencil_", "athread")) -> list[str]:
    r = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True)
    syms = []
    for line in r.stdout.splitlines():
        name = line.split()[-1].split("@")[0]
        if name.startswith(prefixes):
            syms.append(name)
    return syms


def _build_fusion_exe(ref_root: str) -> str:
    """The fusion driver as an executable; its accelerator entry points
    (laplaceAddInput, laplaceAddInput_iteration) are never-called stubs, so
    only its serial loop computes."""
    tag, src_rel = FUSION
    src = os.path.join(ref_root, src_rel)
    obj = os.path.join(OUT, f"{tag}.o")
    exe = os.path.join(OUT, tag)
    stub_c = os.path.join(OUT, f"{tag}_stub.c")
    _run(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w", f"-I{SHIM}", "-c", src, "-o", obj])
    with open(stub_c, "w") as f:
        f.write("/* generated: definitions for the accelerator entry points the driver declares */\n")
        for sym in _undefined(obj, ("laplaceAddInput", "athread")):
            f.write(f"void {sym}(void) {{}}\n")
    _run(["gcc", "-O2", "-o", exe, obj, stub_c])
    return exe


def run_fusion_driver(workdir: str) -> "list[float]":
    """Run the fusion driver in workdir; returns the grid it wrote (mpe_result:
    its serial loop's result, printed with %.2lf, exact for its integer
    values) in row-major order."""
    exe = os.path.join(OUT, FUSION[0])
    subprocess.run([exe], cwd=workdir, capture_output=True, text=True, check=True)
    with open(os.path.join(workdir, "mpe_result")) as f:
        return [float(v) for v in f.read().split()]


def _build_one(ref_root: str, tag: str, src_rel: str) -> str:
    src = os.path.join(ref_root, src_rel)
    is_cpp = src.endswith(".cpp")
    obj = os.path.join(OUT, f"{tag}.o")
    so = os.path.join(OUT, f"{tag}.so")
    stub_c = os.path.join(OUT, f"{tag}_stub.c")
    comp = ["g++" if is_cpp else "gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-w",
            "-Dmain=uhs_ref_unused_main", f"-I{SHIM}"]
    if is_cpp:
        comp += [f"-I{os.path.join(SHIM, 'gpu')}"]
    _run(comp + ["-c", src, "-o", obj])
    with open(stub_c, "w") as f:
        f.write("/* generated: never-called definitions for symbols the driver leaves undefined */\n")
        for s in _undefined(obj):
            f.write(f"void {s}(void) {{}}\n")
    _run(["gcc", "-O2", "-fPIC", "-shared", "-o", so, obj, stub_c] + (["-lstdc++"] if is_cpp else []))
    return so


def build(ref_root: str | None = None) -> list[str]:
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "UH-SW")):
        return []
    os.makedirs(OUT, exist_ok=True)
    jobs = []
    for case, (sw, gpu) in CASES.items():
        jobs.append((f"sw_{case}", sw))
        jobs.append((f"gpu_{case}", gpu))
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        built = list(ex.map(lambda j: _build_one(ref_root, *j), jobs))
    built.append(_build_fusion_exe(ref_root))
    built += _copy_gpu_drivers(ref_root)
    return built


if __name__ == "__main__":
    built = build(sys.argv[1] if len(sys.argv) > 1 else None)
    print(f"built {len(built)} reference drivers into {OUT}")
