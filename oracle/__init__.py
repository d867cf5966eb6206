"""Python access to the CPU oracle (oracle/uhs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, always as the checker or the timed CPU baseline,
never as part of the product path.  See uhs_oracle.c for what it restates.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


class _OStencil(ctypes.Structure):
    _fields_ = [("sizes", c_int64 * 3), ("lb", c_int64 * 3), ("ub", c_int64 * 3), ("nterms", c_int32),
                ("off", POINTER(c_int32)), ("coef", POINTER(c_double))]


_lib = None


def build() -> str:
    """Compile liboracle.so (gcc -O2 -ffp-contract=off -fopenmp)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "uhs_oracle.c")):
            build()
        l = ctypes.CDLL(LIB)
        P = POINTER(_OStencil)
        l.oracle_sweep_f64.argtypes = [P, c_void_p, c_void_p]
        l.oracle_iterate_f64.argtypes = [P, c_void_p, c_void_p, c_int]
        l.oracle_iterate_f64.restype = c_int
        l.oracle_sweep_f32.argtypes = [P, c_void_p, c_void_p]
        l.oracle_fill_rand50.argtypes = [POINTER(c_void_p), c_int, c_int64]
        l.oracle_error_f64.argtypes = [P, c_void_p, c_void_p, POINTER(c_double)]
        l.oracle_error_f32.argtypes = [P, c_void_p, c_void_p, POINTER(c_double)]
        l.oracle_halo_diff_bytes.argtypes = [P, c_void_p, c_void_p, c_int64]
        l.oracle_halo_diff_bytes.restype = c_int64
        l.oracle_set_threads.argtypes = [c_int]
        l.oracle_max_threads.restype = c_int
        _lib = l
    return _lib


class OracleStencil:
    """The oracle's view of a uxxxxxxxxh_gb300.Stencil (or any object with
    sizes/lb/ub/terms/coefficients())."""

    def __init__(self, st):
        self.st = st
        n = len(st.terms)
        coefs = st.coefficients() if hasattr(st, "coefficients") else [t[3] for t in st.terms]
        self._off = (c_int32 * (3 * n))(*[v for t in st.terms for v in t[:3]])
        self._coef = (c_double * n)(*coefs)
        self.s = _OStencil()
        for i in range(3):
            self.s.sizes[i] = st.sizes[i]
            self.s.lb[i] = st.lb[i]
            self.s.ub[i] = st.ub[i]
        self.s.nterms = n
        self.s.off = ctypes.cast(self._off, POINTER(c_int32))
        self.s.coef = ctypes.cast(self._coef, POINTER(c_double))

    def ref(self):
        return ctypes.byref(self.s)


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def max_threads() -> int:
    return lib().oracle_max_threads()


def iterate_f64(st, a: np.ndarray, b: np.ndarray, T: int | None = None) -> None:
    """Run the reference loop nest in place: T == 1 sweeps a -> b, even T runs
    T/2 pairs leaving step T in a (mpe_verify / cpu_verify)."""
    T = st.iterations if T is None else T
    assert a.dtype == np.float64 and b.dtype == np.float64
    o = OracleStencil(st)
    rc = lib().oracle_iterate_f64(o.ref(), _ptr(a), _ptr(b), T)
    if rc != 0:
        raise ValueError(f"oracle rejects T = {T}")


def sweep_f64(st, src: np.ndarray, dst: np.ndarray) -> None:
    o = OracleStencil(st)
    lib().oracle_sweep_f64(o.ref(), _ptr(src), _ptr(dst))


def sweep_f32(st, src: np.ndarray, dst: np.ndarray) -> None:
    o = OracleStencil(st)
    lib().oracle_sweep_f32(o.ref(), _ptr(src), _ptr(dst))


def fill_rand50(arrays: list) -> None:
    """rand() % 50 into every cell of every array, as the drivers' main() does."""
    n = arrays[0].size
    ptrs = (c_void_p * len(arrays))(*[_ptr(a) for a in arrays])
    lib().oracle_fill_rand50(ptrs, len(arrays), n)


def error(st, ref: np.ndarray, x: np.ndarray) -> dict:
    """Relative L2, max abs, max abs / max|ref| over the domain."""
    o = OracleStencil(st)
    out = (c_double * 4)()
    if x.dtype == np.float64:
        lib().oracle_error_f64(o.ref(), _ptr(ref), _ptr(x), out)
    elif x.dtype == np.float32:
        lib().oracle_error_f32(o.ref(), _ptr(ref), _ptr(x), out)
    else:
        raise TypeError(x.dtype)
    return {"l2_rel": out[0], "max_abs": out[1], "max_rel": out[2], "max_ref": out[3]}


def cell_error(st, ref: np.ndarray, x: np.ndarray, floor: float = 0.0) -> float:
    """Largest per-cell relative error over the domain,
    max |x - ref| / max(|ref|, floor): unlike max_rel of error(), which
    divides by the field's largest magnitude, it sees small cells that lost
    precision.  Cells where both are equal count 0 (a zero reference cell
    with floor 0 then counts only when x differs).  Chunked by planes."""
    sz = st.sizes
    r3 = ref.reshape(sz)
    x3 = x.reshape(sz)
    worst = 0.0
    y0, y1, x0, x1 = st.lb[1], st.ub[1], st.lb[2], st.ub[2]
    for z in range(st.lb[0], st.ub[0]):
        r = r3[z, y0:y1, x0:x1]
        d = np.abs(x3[z, y0:y1, x0:x1].astype(np.float64) - r)
        den = np.maximum(np.abs(r), floor)
        with np.errstate(divide="ignore", invalid="ignore"):
            q = np.where(d == 0.0, 0.0, d / den)
        if q.size:
            worst = max(worst, float(np.nanmax(np.where(np.isnan(q), np.inf, q))))
    return worst


def halo_diff(st, a: np.ndarray, b: np.ndarray) -> int:
    """Cells outside the domain whose bytes differ."""
    o = OracleStencil(st)
    return int(lib().oracle_halo_diff_bytes(o.ref(), _ptr(a), _ptr(b), a.itemsize))


# ---------------------------------------------------------------------------
# The reference's own drivers, compiled by oracle/build_ref.py (present only
# where the reference checkout was available at build time).
# ---------------------------------------------------------------------------
def ref_available(case: str, kind: str = "sw") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"{kind}_{case}.so"))


def run_ref_sw(case: str, n_cells: int) -> np.ndarray:
    """Run mpe_verify() of UH-SW/<case>/stencil_*_driver.serial.c on the data
    its main() would have produced; returns a copy of input_mpe afterwards."""
    l = ctypes.CDLL(os.path.join(REF_DIR, f"sw_{case}.so"))
    arrs = [np.ctypeslib.as_array((c_double * n_cells).in_dll(l, nm)) for nm in
            ("input_mpe", "input_spe", "tmp_mpe", "tmp_spe")]
    fill_rand50(arrs)
    l.mpe_verify()
    return arrs[0].copy()


def run_ref_gpu_cpu_verify(case: str, n_cells: int) -> np.ndarray:
    """Run cpu_verify() of UH-GPU/<case>/*_main.cpp.  The driver's tmp_cpu is
    an unset malloc; here it is zeroed (what a fresh mmap'd block holds)."""
    l = ctypes.CDLL(os.path.join(REF_DIR, f"gpu_{case}.so"))
    inp = np.empty(n_cells, np.float64)
    gpu = np.empty(n_cells, np.float64)
    fill_rand50([inp, gpu])
    tmp = np.zeros(n_cells, np.float64)
    for nm, arr in (("input_cpu", inp), ("input_gpu", gpu), ("tmp_cpu", tmp)):
        c_void_p.in_dll(l, nm).value = arr.ctypes.data
    getattr(l, "_Z10cpu_verifyv")()
    return inp
