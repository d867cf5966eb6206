"""The range guard and the power-of-two scale of FP64 grids in float pairs.

A float pair holds a value to 2^-48 of itself only between 2^-74 and 2^128
(below 2^-74 it keeps 24 bits, below 2^-126 it flushes to zero).  Under
UHS_ARITH_AUTO a run keeps its pairs scaled by 2^s, with s chosen from a
device scan of both grids so that the largest magnitude, grown by
(sum |c|)^T, stays below 2^120; the run keeps float pairs when every nonzero
magnitude, scaled, is at least 2^-50, and computes in native FP64 otherwise.
A linear sweep commutes with the scale exactly, so fields of any magnitude
run in float pairs as long as they span less than about 2^169.

These tests score every cell on its own (oracle.cell_error:
|x - ref| / |ref|), which a max-normalised error cannot do: on a field
spanning 1 ... 1e-30, float pairs without the scale (explicit
UHS_ARITH_DF32) lose the small cells' precision while their normalised error
stays far below 1e-12.  The fields and coefficients are positive, so each
cell's relative error is well defined.  The reference computes in IEEE
binary64 throughout (UH-SW/3d1r_star/stencil_3d7pt_driver.serial.c:44-63).

With either float-pair mode a value that outgrows the float range returns
UHS_ERANGE, on the pair-resident path (checked at the join) as in place.
"""
import math

import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from uxxxxxxxxh_gb300.stencil import make_stencil, star_offsets
from uxxxxxxxxh_gb300.workloads import normalised, splitmix_uniform
from gpu_util import assert_cells_close, assert_f64_close, assert_halo_exact, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

AUTO = uhs.RunParams()
FMA = uhs.RunParams(arith=_lib.UHS_ARITH_FMA)
DF32 = uhs.RunParams(arith=_lib.UHS_ARITH_DF32)


def _stencil(rank, r, interior, T, seed, name):
    offs = star_offsets(rank, r)
    coefs = normalised(splitmix_uniform(seed, len(offs)) + 0.1)
    st = make_stencil(name, rank, interior, r, offs, coefs, iterations=T)
    return st, (st.sizes if rank == 3 else st.sizes[1:])


def _bump(rank, r, interior, T, smallest, seed=5):
    """A Gaussian bump centred in the grid, 1 at the centre and `smallest`
    in the corners (halo included), under a star of positive normalised
    coefficients."""
    st, sz = _stencil(rank, r, interior, T, seed, f"bump{rank}d{r}r")
    axes = [np.arange(n) - (n - 1) / 2.0 for n in sz]
    d2 = sum(np.meshgrid(*[a * a for a in axes], indexing="ij"))
    s2 = d2.max() / (2.0 * math.log(1.0 / smallest))
    return st, np.exp(-d2 / (2.0 * s2)).reshape(-1)


def _two_level(rank, r, interior, T, small=1e-30, seed=6):
    """Positive values near 1 in the lower half of the slowest axis and near
    `small` in the upper half: the upper half's cells are computed from
    values of that size only."""
    st, sz = _stencil(rank, r, interior, T, seed, f"two{rank}d{r}r")
    a = 1.0 + 0.5 * splitmix_uniform(seed + 1, int(np.prod(sz))).reshape(sz)
    a[sz[0] // 2:] *= small
    return st, a.reshape(-1)


def _uniform(rank, r, interior, T, scale, seed=7):
    st, sz = _stencil(rank, r, interior, T, seed, f"uni{rank}d{r}r")
    return st, scale * (1.0 + 0.5 * splitmix_uniform(seed + 1, int(np.prod(sz))))


CASES = [(3, 1, (40, 36, 52), 8),  # pair-resident
         (3, 2, (30, 34, 40), 4),  # in place
         (2, 1, (150, 170), 8)]
FIELDS = {
    "bump_1e-30": lambda *a: _bump(*a, 1e-30),
    "two_level_1e-30": lambda *a: _two_level(*a, 1e-30),
    "uniform_1e-40": lambda *a: _uniform(*a, 1e-40),
    "uniform_1e200": lambda *a: _uniform(*a, 1e200),
}


@pytest.mark.parametrize("field", sorted(FIELDS))
@pytest.mark.parametrize("rank,r,interior,T", CASES)
def test_scaled_float_pairs_hold_every_cell(cuda, field, rank, r, interior, T):
    """Fields far outside the float range, or spanning 2^100, keep float pairs
    under AUTO (the result is not the native run's) and every cell within
    1e-12 of the oracle."""
    st, a0 = FIELDS[field](rank, r, interior, T)
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, AUTO)
    assert_cells_close(st, ra, ga, 1e-12)
    assert_cells_close(st, rb, gb, 1e-12)
    assert_halo_exact(st, ra, ga)
    assert_halo_exact(st, rb, gb)
    fa, _ = run_gpu(st, a0, FMA)
    assert not np.array_equal(ga.view(np.uint64), fa.view(np.uint64))


@pytest.mark.parametrize("rank,r,interior,T", CASES)
def test_unscaled_float_pairs_lose_small_cells(cuda, rank, r, interior, T):
    """What the scale avoids: float pairs forced without it (explicit
    UHS_ARITH_DF32) keep 24 bits in the 1e-30 half, which the max-normalised
    error does not show."""
    st, a0 = _two_level(rank, r, interior, T, 1e-30)
    ra, _ = run_oracle(st, a0)
    da, _ = run_gpu(st, a0, DF32)
    assert oracle.error(st, ra, da)["max_rel"] <= 1e-12
    assert oracle.cell_error(st, ra, da) > 1e-9


@pytest.mark.parametrize("rank,r,interior,T", CASES)
def test_field_wider_than_the_window_runs_native(cuda, rank, r, interior, T):
    """Values near 1 and near 1e-60 (a span of 2^200): AUTO computes in
    native FP64, bit-identical to UHS_ARITH_FMA, every cell within 1e-12."""
    st, a0 = _two_level(rank, r, interior, T, 1e-60)
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, AUTO)
    fa, _ = run_gpu(st, a0, FMA)
    assert np.array_equal(ga.view(np.uint64), fa.view(np.uint64))
    assert_cells_close(st, ra, ga, 1e-12)
    assert_cells_close(st, rb, gb, 1e-12)


def _growing(T):
    """Unit coefficients (sum 7) on values in [2^125, 1.5 * 2^125): most sums
    of the first sweep pass 2^128."""
    st = make_stencil("grow3d", 3, (20, 24, 36), 1, star_offsets(3, 1), [1.0] * 7, iterations=T)
    a0 = (2.0 ** 125) * (1.0 + 0.5 * splitmix_uniform(3, int(np.prod(st.sizes))))
    return st, a0


@pytest.mark.parametrize("T,flags", [(8, 0), (2, _lib.UHS_FLAG_IN_PLACE), (8, _lib.UHS_FLAG_IN_PLACE)])
def test_explicit_float_pairs_report_overflow(cuda, T, flags):
    st, a0 = _growing(T)
    with pytest.raises(_lib.UhsError) as ei:
        run_gpu(st, a0, uhs.RunParams(arith=_lib.UHS_ARITH_DF32, flags=flags))
    assert ei.value.code == _lib.UHS_ERANGE
    # the status word is cleared: the next call on the stream succeeds
    st2, b0 = _bump(3, 1, (20, 24, 36), 2, 1e-3)
    ra, _ = run_oracle(st2, b0)
    ga, _ = run_gpu(st2, b0, DF32)
    assert_f64_close(st2, ra, ga)


@pytest.mark.parametrize("T", [2, 8])
def test_auto_scales_a_growing_field(cuda, T):
    """The same growth under AUTO: the scale takes the growth bound (sum |c|)^T
    into account, so the run stays in float pairs and every cell matches the
    oracle within 1e-12 (values reach 2^148 at T = 8)."""
    st, a0 = _growing(T)
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, AUTO)
    assert np.isfinite(ga).all()
    assert_cells_close(st, ra, ga, 1e-12)
    assert_cells_close(st, rb, gb, 1e-12)
