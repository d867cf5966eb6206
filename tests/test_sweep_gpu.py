"""Parity of the CUDA sweep kernels with the oracle (gpu-marked).

Bar: UHS_ARITH_EXACT is bit-identical to the oracle (and so to the reference's
serial loops); UHS_ARITH_FMA and the float-pair path stay within a max error of
1e-12 relative to the field's largest magnitude after T steps; FP32 grids stay
within a relative L2 error of 1e-6 of the FP64 oracle.  Cells outside the
domain come back bit-exact in both grids in every mode.
"""
import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from golden_util import reference_stencil, resized
from gpu_util import assert_f64_close, assert_halo_exact, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu

SHAPES = uhs.SHAPES
ODD_3D = (19, 37, 45)
ODD_2D = (131, 157)


def _case(rank, r, kind, T=4, seed=5, interior=None):
    interior = interior or (ODD_3D if rank == 3 else ODD_2D)
    return random_case(rank, r, kind, interior, T, seed)


@pytest.mark.parametrize("rank,r,kind", SHAPES)
def test_generic_exact_is_bit_identical(cuda, rank, r, kind):
    st, a0 = _case(rank, r, kind)
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(kernel=uhs.UHS_KERNEL_GENERIC, arith=uhs.UHS_ARITH_EXACT))
    assert np.array_equal(ra.view(np.uint64), ga.view(np.uint64))
    assert np.array_equal(rb.view(np.uint64), gb.view(np.uint64))


@pytest.mark.parametrize("rank,r,kind", SHAPES)
def test_generic_fma_within_1e12(cuda, rank, r, kind):
    st, a0 = _case(rank, r, kind, T=6)
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(kernel=uhs.UHS_KERNEL_GENERIC, arith=uhs.UHS_ARITH_FMA))
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)
    assert_halo_exact(st, rb, gb)


@pytest.mark.parametrize("rank,r,kind", [(3, 1, "star"), (2, 2, "box"), (3, 3, "box")])
def test_generic_f32_against_f64_oracle(cuda, rank, r, kind):
    import torch
    st, a0 = _case(rank, r, kind, T=4)
    a32 = a0.astype(np.float32)
    ra, _ = run_oracle(st, a32.astype(np.float64))
    st32 = st.with_(dtype=uhs.UHS_F32)
    ga, _ = run_gpu(st32, a32, uhs.RunParams(kernel=uhs.UHS_KERNEL_GENERIC), dtype=torch.float32)
    e = oracle.error(st, ra, ga)
    assert e["l2_rel"] <= 1e-6, e
    assert oracle.halo_diff(st32, a32, ga) == 0


@pytest.mark.parametrize("case", ["2d1r_star", "2d3r_box", "3d1r_star", "3d2r_box", "3d3r_box"])
def test_reference_programs_exact(cuda, case):
    """The reference's own expressions (term order and coefficients from its
    .dsl files) on the reference's rand() % 50 data, smaller grids."""
    st = reference_stencil(case, "sw")
    st = resized(st, (23, 29, 31) if st.rank == 3 else (97, 101), iterations=4)
    n = int(np.prod(st.sizes))
    a0 = np.empty(n)
    oracle.fill_rand50([a0])
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(arith=uhs.UHS_ARITH_EXACT))
    assert np.array_equal(ra.view(np.uint64), ga.view(np.uint64))
    assert np.array_equal(rb.view(np.uint64), gb.view(np.uint64))


def test_single_sweep_writes_b_only_in_domain(cuda):
    st, a0 = _case(3, 2, "star", T=1)
    b0 = np.full_like(a0, 7.0)
    ra, rb = run_oracle(st, a0, b0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(arith=uhs.UHS_ARITH_EXACT), b0=b0)
    assert np.array_equal(ga, a0)
    assert np.array_equal(rb.view(np.uint64), gb.view(np.uint64))


def test_tiny_and_ragged_grids(cuda):
    for interior in [(1, 1, 1), (2, 3, 1), (1, 40, 33), (33, 1, 65)]:
        st, a0 = random_case(3, 1, "box", interior, 2, 9)
        ra, _ = run_oracle(st, a0)
        ga, _ = run_gpu(st, a0, uhs.RunParams(arith=uhs.UHS_ARITH_EXACT))
        assert np.array_equal(ra, ga), interior


def test_zero_iterations_is_a_no_op(cuda):
    st, a0 = _case(2, 1, "star", T=0)
    ga, gb = run_gpu(st, a0)
    assert np.array_equal(ga, a0) and np.array_equal(gb, a0)


def test_padded_pitch_memref(cuda):
    """Row pitch larger than the row (a view into a wider allocation)."""
    import torch
    st, a0 = _case(3, 1, "star", T=2, interior=(9, 10, 11))
    sz = st.sizes
    big_a = torch.zeros((sz[0], sz[1], sz[2] + 5), dtype=torch.float64, device="cuda")
    big_b = torch.zeros_like(big_a)
    va, vb = big_a[:, :, :sz[2]], big_b[:, :, :sz[2]]
    src = torch.from_numpy(a0.reshape(sz)).cuda()
    va.copy_(src)
    vb.copy_(src)
    uhs.run(st, va, vb, uhs.RunParams(arith=uhs.UHS_ARITH_EXACT))
    ra, _ = run_oracle(st, a0)
    assert np.array_equal(va.cpu().numpy().reshape(-1), ra)
    assert torch.all(big_a[:, :, sz[2]:] == 0)
