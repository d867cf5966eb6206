"""The tensor-core box path (UHS_KERNEL_MMA: tcgen05 kind::tf32 with split
hi/lo operands) for FP32 3D boxes of radius 2 and 3, against the FP64 oracle,
cells outside the domain untouched.

Tolerance: the split operands make every product exact to 2^-22, but the
tensor core rounds its FP32 accumulator once per MMA instruction, toward
zero, and one output's sum runs through 225 (radius 2) to 441 (radius 3)
MMAs.  Measured on GB300 that leaves a relative L2 of 2e-6 to 5e-6 per
step, growing about linearly with T (4.5e-5 for the 343-point Gaussian box
after 10 steps), against 2e-7 to 3e-7 for the CUDA-core FP32 sweep.  The bar
here is MMA_L2 for up to 10 steps."""
import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from gpu_util import run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import cfg3, random_case

pytestmark = pytest.mark.gpu

MMA = uhs.UHS_KERNEL_MMA
MMA_L2 = 1e-4


def f32_case(r, interior, T, seed):
    st, a0 = random_case(3, r, "box", interior, T, seed, dtype=uhs.UHS_F32)
    return st, a0.astype(np.float32)


def check_f32(st, a0, params, l2=MMA_L2):
    import torch
    ra, rb = run_oracle(st, a0.astype(np.float64))
    ga, gb = run_gpu(st, a0, params, dtype=torch.float32)
    e = oracle.error(st, ra, ga.astype(np.float64))
    assert e["l2_rel"] <= l2, e
    eb = oracle.error(st, rb, gb.astype(np.float64))
    assert eb["l2_rel"] <= l2, eb
    # the halo is never written: bit-identical to the input's
    assert oracle.halo_diff(st, a0.astype(np.float64), ga.astype(np.float64)) == 0
    return e


TMEM_A = uhs._lib.UHS_FLAG_MMA_TMEM_A


# A operand read from shared memory (the default), or staged in tensor memory
# by tcgen05.cp (flag, 16-column tiles)
@pytest.mark.parametrize("r,xtile,flags", [(2, 16, 0), (3, 16, 0), (2, 16, TMEM_A), (3, 16, TMEM_A), (2, 32, 0)])
@pytest.mark.parametrize("T", [1, 2, 6])
def test_mma_box_matches_oracle(cuda, r, xtile, flags, T):
    # 150 rows: two 128-row tiles, the second ragged; 45 columns: ragged x tiles
    st, a0 = f32_case(r, (21, 150, 45), T, 40 + r)
    p = uhs.RunParams(kernel=MMA, tile_x=xtile, flags=flags)
    assert uhs.plan(st, params=p).kernel == MMA
    check_f32(st, a0, p)


@pytest.mark.parametrize("r", [2, 3])
def test_mma_box_agrees_with_cuda_cores(cuda, r):
    import torch
    st, a0 = f32_case(r, (30, 64, 80), 4, 50 + r)
    ga, _ = run_gpu(st, a0, uhs.RunParams(kernel=MMA), dtype=torch.float32)
    gc, _ = run_gpu(st, a0, uhs.RunParams(kernel=uhs.UHS_KERNEL_STREAM, flags=uhs._lib.UHS_FLAG_NO_FACTOR),
                    dtype=torch.float32)
    d = np.abs(ga.astype(np.float64) - gc.astype(np.float64)).max()
    assert d <= MMA_L2 * np.abs(gc).max()


def test_mma_box_offset_domain_and_wide_halo(cuda):
    """Domain narrower than the grid on every axis, with halos wider than R:
    cells beyond lb - R / ub + R must not enter the sum, and stay untouched."""
    st, a0 = f32_case(3, (40, 140, 70), 2, 61)
    st = st.with_(lb=(5, 4, 6), ub=(st.ub[0] - 2, st.ub[1] - 4, st.ub[2] - 5))
    a0 = a0.copy()
    # poison cells the stencil never reads
    full = a0.reshape(st.sizes)
    full[:, :, 0] = np.nan
    full[:, 0, :] = np.nan
    full[0, :, :] = np.nan
    import torch
    ra, _ = run_oracle(st, a0.astype(np.float64))
    ga, _ = run_gpu(st, a0, uhs.RunParams(kernel=MMA), dtype=torch.float32)
    e = oracle.error(st, ra, ga.astype(np.float64))
    assert e["l2_rel"] <= MMA_L2, e
    assert np.isfinite(ga.reshape(st.sizes)[5:-2, 4:-4, 6:-5]).all()
    ha = np.nan_to_num(a0.astype(np.float64), nan=7.0)
    hg = np.nan_to_num(ga.astype(np.float64), nan=7.0)
    assert oracle.halo_diff(st, ha, hg) == 0


def test_mma_cfg3_gaussian_box(cuda):
    """The 343-point Gaussian box at 96^3, T = 10, on both paths: the
    CUDA-core FP32 sweep (term by term) within 1e-6 of the FP64 oracle, the
    split-tf32 tensor-core sweep within MMA_L2."""
    st, a0 = cfg3(n=96, T=10)
    st = st.with_(dtype=uhs.UHS_F32)
    check_f32(st, a0.astype(np.float32), uhs.RunParams(kernel=MMA))
    check_f32(st, a0.astype(np.float32),
              uhs.RunParams(kernel=uhs.UHS_KERNEL_STREAM, flags=uhs._lib.UHS_FLAG_NO_FACTOR), l2=1e-6)


def test_mma_refusals(cuda):
    st, _ = f32_case(3, (8, 8, 16), 2, 70)
    with pytest.raises(uhs.UhsError) as ei:
        uhs.plan(st.with_(dtype=uhs.UHS_F64), params=uhs.RunParams(kernel=MMA))
    assert ei.value.code == uhs._lib.UHS_EUNSUPPORTED
    st1, _ = f32_case(1, (8, 8, 16), 2, 71)
    with pytest.raises(uhs.UhsError):
        uhs.plan(st1, params=uhs.RunParams(kernel=MMA))
    with pytest.raises(uhs.UhsError) as ei:
        uhs.plan(st, params=uhs.RunParams(kernel=MMA, tile_x=32))
    assert ei.value.code == uhs._lib.UHS_EINVAL
    with pytest.raises(uhs.UhsError):
        uhs.plan(st, params=uhs.RunParams(kernel=MMA, k_temporal=2))
    st2, _ = f32_case(2, (8, 8, 16), 2, 73)
    with pytest.raises(uhs.UhsError) as ei:
        uhs.plan(st2, params=uhs.RunParams(kernel=MMA, tile_x=32, flags=TMEM_A))
    assert ei.value.code == uhs._lib.UHS_EINVAL
    stars, _ = random_case(3, 2, "star", (8, 8, 16), 2, 72, dtype=uhs.UHS_F32)
    with pytest.raises(uhs.UhsError):
        uhs.plan(stars, params=uhs.RunParams(kernel=MMA))


@pytest.mark.parametrize("flags", [0, TMEM_A])
def test_mma_many_planes_per_cta_and_tiny_grid(cuda, flags):
    """More plane tiles than CTAs (each CTA walks several segments) and a grid
    smaller than one tile."""
    st, a0 = f32_case(2, (300, 20, 20), 2, 80)
    check_f32(st, a0, uhs.RunParams(kernel=MMA, flags=flags))
    st2, b0 = f32_case(3, (3, 5, 7), 2, 81)
    check_f32(st2, b0, uhs.RunParams(kernel=MMA, flags=flags))
