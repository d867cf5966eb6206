"""Temporal fusion (k timesteps per pass) and the separable-box path, both
against the oracle: FP64 within 1e-12 (max, relative to the field), FP32
within a relative L2 of 1e-6, halo bit-exact."""
import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from golden_util import reference_stencil, resized
from gpu_util import assert_f64_close, assert_halo_exact, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import cfg3, random_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [2, 4])
@pytest.mark.parametrize("T", [2, 4, 6, 50])
@pytest.mark.parametrize("arith", [uhs.UHS_ARITH_FMA, uhs.UHS_ARITH_DF32])
def test_fused_f64_matches_oracle(cuda, k, T, arith):
    st, a0 = random_case(3, 1, "star", (37, 21, 70), T, 31)
    # both grids must hold the same halo: use a copy of a0 for b
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(arith=arith, k_temporal=k))
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)  # b holds step T-1, as the reference leaves it
    assert_halo_exact(st, ra, ga)


@pytest.mark.parametrize("k", [2, 4])
def test_fused_f32(cuda, k):
    import torch
    st, a0 = random_case(3, 1, "star", (40, 33, 64), 20, 32)
    a32 = a0.astype(np.float32)
    ra, _ = run_oracle(st, a32.astype(np.float64))
    ga, _ = run_gpu(st.with_(dtype=uhs.UHS_F32), a32, uhs.RunParams(k_temporal=k), dtype=torch.float32)
    assert oracle.error(st, ra, ga)["l2_rel"] <= 1e-6


def test_fused_offset_domain_and_ragged_tiles(cuda):
    st, a0 = random_case(3, 1, "star", (19, 23, 45), 8, 33)
    st = st.with_(lb=(2, 1, 3), ub=(st.ub[0] - 1, st.ub[1] - 2, st.ub[2]))
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(k_temporal=4))
    assert_f64_close(st, ra, ga)
    assert_halo_exact(st, ra, ga)


def test_fused_rejects_different_halos_and_other_shapes(cuda):
    st, a0 = random_case(3, 1, "star", (10, 10, 40), 4, 34)
    b0 = a0.copy()
    b0[0] += 1.0  # a halo cell differs
    with pytest.raises(uhs.UhsError) as ei:
        run_gpu(st, a0, uhs.RunParams(k_temporal=2), b0=b0)
    assert ei.value.code == uhs._lib.UHS_EINVAL
    # depth 4 of a radius-2 3D star does not fit shared memory; float-pair grids are not fused
    st2, _ = random_case(3, 2, "star", (10, 10, 40), 4, 35)
    uhs.plan(st2, params=uhs.RunParams(k_temporal=2))
    with pytest.raises(uhs.UhsError):
        uhs.plan(st2, params=uhs.RunParams(k_temporal=4))
    with pytest.raises(uhs.UhsError):
        uhs.plan(st.with_(dtype=uhs._lib.UHS_F32X2), params=uhs.RunParams(k_temporal=2))


@pytest.mark.parametrize("case", ["3d1r_box", "3d2r_box", "3d3r_box", "2d2r_box", "2d3r_box"])
@pytest.mark.parametrize("arith", [uhs.UHS_ARITH_FMA, uhs.UHS_ARITH_DF32])
def test_reference_boxes_run_factored(cuda, case, arith):
    """The reference's box programs have rank-1 coefficient tensors: the
    planner sweeps them as 1D passes."""
    st = reference_stencil(case, "gpu")
    st = resized(st, (26, 30, 70) if st.rank == 3 else (150, 260), iterations=4)
    p = uhs.RunParams(arith=arith)
    assert uhs.plan(st, params=p).factored == 1
    n = int(np.prod(st.sizes))
    a0 = np.empty(n)
    oracle.fill_rand50([a0])
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, p)
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)


def test_gaussian_box_factored_f32_and_opt_out(cuda):
    import torch
    st, a0 = cfg3(n=40, T=4)
    assert uhs.plan(st).factored == 1
    assert uhs.plan(st, params=uhs.RunParams(flags=uhs._lib.UHS_FLAG_NO_FACTOR)).factored == 0
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0)
    assert_f64_close(st, ra, ga)
    gn, _ = run_gpu(st, a0, uhs.RunParams(flags=uhs._lib.UHS_FLAG_NO_FACTOR))
    assert_f64_close(st, ra, gn)
    a32 = a0.astype(np.float32)
    r32, _ = run_oracle(st, a32.astype(np.float64))
    g32, _ = run_gpu(st.with_(dtype=uhs.UHS_F32), a32, dtype=torch.float32)
    assert oracle.error(st, r32, g32)["l2_rel"] <= 1e-6


def test_non_separable_box_is_not_factored(cuda):
    st, a0 = random_case(3, 2, "box", (20, 20, 40), 2, 36)
    assert uhs.plan(st).factored == 0
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0)
    assert_f64_close(st, ra, ga)
