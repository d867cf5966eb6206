"""Per-program `_mlir_ciface_*` entry points.

UHStencil compiles each .dsl program to an object exporting
`_mlir_ciface_<name>_iteration(memref *a, memref *b)` (even T) or
`_mlir_ciface_<name>(memref *in, memref *in_output)` (T == 1), with MLIR's
ranked memref descriptors as arguments (UH-GPU/3d1r_star/3d7pt_main.cpp:17-25;
UHStencil/lib/Parser/MLIRGen.cpp:183-352 names the functions,
lib/Conversion/StencilToStandard/ConvertStencilToStandard.cpp:80 asks for the
C interface).  This module writes the same symbol as a thin C wrapper around
uhs_run / uhs_sweep with the program's descriptor baked in, so a reference
driver links against it unchanged.  The wrapper keeps the reference's `void`
signature; its status is kept and readable through
`uhs_ciface_status_<name>()` (and `uhs_last_error()` on the calling thread).
"""
from __future__ import annotations

import os
import subprocess

from .stencil import Stencil
from ._lib import LIB_PATH, PKG, UHS_F32, UHS_F64

INCLUDE = os.path.join(os.path.dirname(PKG), "include")


def _ctype(dtype: int) -> str:
    return {UHS_F64: "double", UHS_F32: "float"}[dtype]


def ciface_source(st: Stencil, name: str | None = None) -> str:
    """C source of the program's MLIR C-interface entry point."""
    name = name or st.name
    if st.dtype not in (UHS_F64, UHS_F32):
        raise ValueError("the MLIR entry points take f32 or f64 memrefs")
    T = _ctype(st.dtype)
    R = st.rank
    dt = "UHS_F64" if st.dtype == UHS_F64 else "UHS_F32"
    terms = ",\n    ".join(
        f"{{{t[0]}, {t[1]}, {t[2]}, {st.param_terms.get(i, -1)}, {float(t[3])!r}}}" for i, t in enumerate(st.terms))
    params = ", ".join(repr(float(p)) for p in st.params) if st.params else ""
    single = st.iterations == 1
    sym = f"_mlir_ciface_{name}" if single else f"_mlir_ciface_{name}_iteration"
    call = "uhs_sweep" if single else "uhs_run"
    if R == 3:
        conv = """    m->allocated = d->allocated; m->aligned = d->aligned; m->offset = d->offset;
    for (int i = 0; i < 3; ++i) { m->sizes[i] = d->sizes[i]; m->strides[i] = d->strides[i]; }"""
    else:
        conv = """    m->allocated = d->allocated; m->aligned = d->aligned; m->offset = d->offset;
    m->sizes[0] = 1; m->sizes[1] = d->sizes[0]; m->sizes[2] = d->sizes[1];
    m->strides[0] = d->sizes[0] * d->strides[0]; m->strides[1] = d->strides[0]; m->strides[2] = d->strides[1];"""
    return f"""/* Generated by uxxxxxxxxh_gb300.ciface for stencil program `{st.name}`:
 * the MLIR C-interface entry UHStencil's compiler would emit for it, routed to
 * the GB300 backend ({call}).  Rank {R}, {T}, T = {st.iterations}. */
#include <stdint.h>
#include <stdio.h>
#include "uhs.h"

/* MLIR StridedMemRefType<{T}, {R}> */
typedef struct {{
    {T} *allocated;
    {T} *aligned;
    int64_t offset;
    int64_t sizes[{R}];
    int64_t strides[{R}];
}} uhs_mlir_memref_{name};

static const uhs_term kTerms[] = {{
    {terms}
}};
{"static const double kParams[] = {" + params + "};" if params else ""}
static const uhs_stencil_desc kDesc = {{
    {R}, {dt}, {{{st.lb[0]}, {st.lb[1]}, {st.lb[2]}}}, {{{st.ub[0]}, {st.ub[1]}, {st.ub[2]}}},
    {st.nterms}, kTerms, {st.iterations}, {"kParams" if params else "0"}, {len(st.params)}
}};

static int g_status = UHS_OK;

/* Status of the last call of {sym} (UHS_OK or a uhs.h error code). */
int uhs_ciface_status_{name}(void) {{ return g_status; }}

static void to_uhs(const uhs_mlir_memref_{name} *d, uhs_memref *m) {{
{conv}
}}

void {sym}(uhs_mlir_memref_{name} *a, uhs_mlir_memref_{name} *b) {{
    uhs_memref A, B;
    to_uhs(a, &A);
    to_uhs(b, &B);
    g_status = {call}(&kDesc, &A, &B, 0, 0);
    if (g_status != UHS_OK) fprintf(stderr, "{sym}: %s\\n", uhs_last_error());
}}
"""


def build_ciface(st: Stencil, out_dir: str, name: str | None = None) -> str:
    """Compile the wrapper into out_dir/lib<name>_ciface.so, linked to libuhs.so."""
    name = name or st.name
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(out_dir, f"{name}_ciface.c")
    so = os.path.join(out_dir, f"lib{name}_ciface.so")
    with open(src, "w") as f:
        f.write(ciface_source(st, name))
    cmd = ["gcc", "-O2", "-fPIC", "-shared", f"-I{INCLUDE}", src, "-o", so, f"-L{PKG}", "-luhs",
           f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building {so} failed:\n{r.stderr}")
    return so
