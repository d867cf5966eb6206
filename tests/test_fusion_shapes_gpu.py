"""Temporal fusion (k timesteps per pass over HBM, stream_fused.cuh) of every
star and box shape, rank 2 and 3, radius 1-3, against the oracle: FP64 (native
and float pairs) within 1e-12 of the field's largest magnitude with the halo
bit-exact, for both grids (a holds step T, b step T-1, as the reference's
ping-pong leaves them); FP32 within a relative L2 of 1e-6.  Depth 4 runs in
2D for every radius and in 3D for radius 1; the odd extents leave ragged
tiles on every axis."""
import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from gpu_util import assert_f64_close, assert_halo_exact, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu

CASES = [(rank, r, kind, k) for rank, r, kind in uhs.SHAPES for k in (2, 4) if not (k == 4 and rank == 3 and r > 1)]


def _interior(rank, r):
    return (13, 19, 37) if rank == 3 else (61, 517)


@pytest.mark.parametrize("rank,r,kind,k", CASES)
@pytest.mark.parametrize("arith", [uhs.UHS_ARITH_FMA, uhs.UHS_ARITH_DF32])
def test_fused_shapes_f64(cuda, rank, r, kind, k, arith):
    st, a0 = random_case(rank, r, kind, _interior(rank, r), 8, 400 + 10 * r + rank)
    p = uhs.RunParams(kernel=uhs.UHS_KERNEL_STREAM, arith=arith, k_temporal=k)
    assert uhs.plan(st, params=p).k_temporal == k
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, p)
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)
    assert_halo_exact(st, rb, gb)


@pytest.mark.parametrize("rank,r,kind,k", CASES)
def test_fused_shapes_f32(cuda, rank, r, kind, k):
    import torch
    st, a0 = random_case(rank, r, kind, _interior(rank, r), 8, 500 + 10 * r + rank)
    a32 = a0.astype(np.float32)
    ra, _ = run_oracle(st, a32.astype(np.float64))
    ga, _ = run_gpu(st.with_(dtype=uhs.UHS_F32), a32, uhs.RunParams(kernel=uhs.UHS_KERNEL_STREAM, k_temporal=k),
                    dtype=torch.float32)
    assert oracle.error(st, ra, ga.astype(np.float64))["l2_rel"] <= 1e-6


@pytest.mark.parametrize("k", [2, 4])
def test_fused_2d_offset_domain(cuda, k):
    """A domain strictly inside the grid on both axes (cells between the
    domain and the grid's edge are halo at every level)."""
    st, a0 = random_case(2, 2, "star", (70, 600), 12, 77)
    st = st.with_(lb=(st.lb[0], 5, 7), ub=(st.ub[0], st.ub[1] - 3, st.ub[2] - 9))
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(k_temporal=k))
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)
