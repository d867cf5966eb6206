"""The single-grid benchmark configurations at their full sizes against the
FP64 oracle (a restatement of the reference's serial loops, run on all host
cores): cfg1 (2D 5-point star, 4096^2, constant halo, T = 100) and cfg3
(343-point Gaussian box, 256^3, T = 10), each in the default FP64 path and in
FP32.  FP64: max |x - ref| / max |ref| <= 1e-12 after T steps, every cell
within 1e-12 of itself (these fields and coefficients are positive, so each
cell's relative error is well defined), both grids' halos bit-exact.  FP32:
relative L2 <= 1e-6 against the oracle on the same (rounded) input.  The
third single-grid configuration, cfg4 (13-point star, 512^3, T = 200), is
scored against the oracle every 20 steps by tests/test_precision_gpu.py at
its full size.  The reference checks its own GPU run the same way, against
its CPU loop on the host (UH-GPU/3d1r_star/3d7pt_main.cpp:50-103)."""
import os

import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from uxxxxxxxxh_gb300.workloads import cfg1, cfg3
from gpu_util import assert_cells_close, assert_f64_close, assert_halo_exact, run_gpu

pytestmark = pytest.mark.gpu


def _oracle(st, a0):
    oracle.set_threads(os.cpu_count() or 1)
    ra, rb = a0.copy(), a0.copy()
    oracle.iterate_f64(st, ra, rb)
    return ra, rb


@pytest.mark.parametrize("cfg", [cfg1, cfg3], ids=["cfg1_4096sq_T100", "cfg3_256cube_T10"])
def test_full_size_config_matches_oracle(cuda, cfg):
    import torch
    st, a0 = cfg()
    ra, rb = _oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams())
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_cells_close(st, ra, ga, 1e-12)
    assert_halo_exact(st, ra, ga)
    assert_halo_exact(st, rb, gb)
    # FP32 grids on the same workload, against the oracle on the rounded input
    st32 = st.with_(dtype=_lib.UHS_F32)
    a32 = a0.astype(np.float32)
    r32a, _ = _oracle(st, a32.astype(np.float64))
    g32, _ = run_gpu(st32, a32, uhs.RunParams(), dtype=torch.float32)
    e = oracle.error(st, r32a, g32)
    assert e["l2_rel"] <= 1e-6, e
