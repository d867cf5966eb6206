"""Helpers for the gpu-marked tests: run a program through the C ABI on
device copies of host grids and bring both grids back."""
import numpy as np

import oracle
import uxxxxxxxxh_gb300 as uhs


def to_dev(a: np.ndarray, st, dtype=None):
    import torch
    t = torch.from_numpy(a.reshape(st.sizes if st.rank == 3 else st.sizes[1:]))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda().contiguous()


def run_gpu(st, a0: np.ndarray, params=None, b0: np.ndarray | None = None, dtype=None):
    """Device run of st on (a0, b0 or a copy of a0); returns host (a, b)."""
    import torch
    a = to_dev(a0, st, dtype)
    b = to_dev(a0 if b0 is None else b0, st, dtype)
    uhs.run(st, a, b, params)
    torch.cuda.synchronize()
    return a.cpu().numpy().reshape(-1), b.cpu().numpy().reshape(-1)


def run_oracle(st, a0: np.ndarray, b0: np.ndarray | None = None, T=None):
    a = a0.astype(np.float64).copy()
    b = (a0 if b0 is None else b0).astype(np.float64).copy()
    oracle.iterate_f64(st, a, b, T)
    return a, b


def assert_f64_close(st, ref, got, tol=1e-12):
    e = oracle.error(st, ref, got)
    assert e["max_rel"] <= tol, e
    return e


def assert_halo_exact(st, ref, got):
    assert oracle.halo_diff(st, ref, got) == 0


def assert_cells_close(st, ref, got, tol=1e-12, floor=0.0):
    """Per-cell relative error (oracle.cell_error) within tol."""
    e = oracle.cell_error(st, ref, got, floor)
    assert e <= tol, e
    return e
