"""The range guard of FP64 grids in float-pair arithmetic.

A float pair holds a value to 2^-48 of itself only between 2^-74 and 2^128
(below 2^-74 it keeps 24 bits, below 2^-126 it flushes to zero).  Under
UHS_ARITH_AUTO a device scan of both grids keeps float pairs only when every
nonzero magnitude is at least 2^-50 and the largest, grown by (sum |c|)^T,
stays below 2^120; otherwise the run computes in native FP64.  These tests
score every cell on its own (oracle.cell_error: |x - ref| / |ref|), which a
max-normalised error cannot do: on a field spanning 1 ... 1e-30 the explicit
float-pair run loses the small cells' precision while its normalised error
stays far below 1e-12.  The reference computes in IEEE binary64 throughout
(UH-SW/3d1r_star/stencil_3d7pt_driver.serial.c:44-63).

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


def _bump(rank, r, interior, T, smallest, seed=5):
    """A Gaussian bump centred in the grid, 1 at the centre and `smallest`
    in the corners (halo included), under a star of positive normalised
    coefficients: every cell and every term is positive, so each cell's
    relative error is well defined."""
    offs = star_offsets(rank, r)
    coefs = normalised(splitmix_uniform(seed, len(offs)) + 0.1)
    st = make_stencil(f"bump{rank}d{r}r", rank, interior, r, offs, coefs, iterations=T)
    sz = st.sizes if rank == 3 else st.sizes[1:]
    axes = [np.arange(n) - (n - 1) / 2.0 for n in sz]
    d2 = sum(np.meshgrid(*[a * a for a in axes], indexing="ij"))
    s2 = d2.max() / (2.0 * math.log(1.0 / smallest))
    return st, np.exp(-d2 / (2.0 * s2)).reshape(-1)


def _two_level(rank, r, interior, T, seed=6):
    """Positive values near 1 in the lower half of the slowest axis and near
    1e-30 in the upper half, under positive normalised star coefficients:
    the upper half's cells are computed from values below 2^-74 only."""
    offs = star_offsets(rank, r)
    coefs = normalised(splitmix_uniform(seed, len(offs)) + 0.1)
    st = make_stencil(f"two{rank}d{r}r", rank, interior, r, offs, coefs, iterations=T)
    sz = st.sizes if rank == 3 else st.sizes[1:]
    a = 1.0 + 0.5 * splitmix_uniform(seed + 1, int(np.prod(sz))).reshape(sz)
    a[sz[0] // 2:] *= 1e-30
    return st, a.reshape(-1)


FIELDS = {"bump": lambda *a: _bump(*a, 1e-30), "two_level": _two_level}


@pytest.mark.parametrize("field", ["bump", "two_level"])
@pytest.mark.parametrize("rank,r,interior,T", [
    (3, 1, (40, 36, 52), 8),   # pair-resident when float pairs run
    (3, 2, (30, 34, 40), 4),   # in place
    (2, 1, (150, 170), 8),
])
def test_wide_range_field_runs_native_and_holds_every_cell(cuda, field, rank, r, interior, T):
    st, a0 = FIELDS[field](rank, r, interior, T)
    assert a0.min() < 2.0 ** -74
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, AUTO)
    assert_cells_close(st, ra, ga, 1e-12)
    assert_cells_close(st, rb, gb, 1e-12)
    assert_halo_exact(st, ra, ga)
    # the guard chose native FP64: bit-identical to an explicit UHS_ARITH_FMA run
    fa, _ = run_gpu(st, a0, FMA)
    assert np.array_equal(ga.view(np.uint64), fa.view(np.uint64))
    if field == "two_level":
        # what the guard avoids: float pairs forced on this field keep 24
        # bits in the small half, which the max-normalised error does not show
        da, _ = run_gpu(st, a0, DF32)
        assert oracle.error(st, ra, da)["max_rel"] <= 1e-12
        assert oracle.cell_error(st, ra, da) > 1e-9


def test_moderate_range_field_keeps_float_pairs(cuda):
    """A bump spanning 1 ... 1e-10 (all magnitudes above 2^-50) keeps float
    pairs under AUTO -- the result differs from the native FP64 run in its
    low bits -- and still holds every cell within 1e-12."""
    st, a0 = _bump(3, 1, (40, 36, 52), 8, 1e-10)
    assert a0.min() > 2.0 ** -50
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0, AUTO)
    assert_cells_close(st, ra, ga, 1e-12)
    fa, _ = run_gpu(st, a0, FMA)
    assert not np.array_equal(ga.view(np.uint64), fa.view(np.uint64))


def test_uniformly_tiny_field_runs_native(cuda):
    """Every value near 1e-40 (below the float range): AUTO computes in native
    FP64, bit-identical to UHS_ARITH_FMA and within 1e-12 of the oracle per cell."""
    from uxxxxxxxxh_gb300.workloads import random_case
    st, a0 = random_case(3, 1, "star", (24, 28, 40), 8, 9)
    a0 = 1e-40 * (1.5 + a0)  # positive, in [0.5e-40, 2.5e-40)
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0, AUTO)
    fa, _ = run_gpu(st, a0, FMA)
    assert np.array_equal(ga.view(np.uint64), fa.view(np.uint64))
    assert_cells_close(st, ra, ga, 1e-12)


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


def test_auto_with_growth_runs_native(cuda):
    """The same growth under AUTO: the scan's growth bound sends it to native
    FP64, which represents it (no error), bit-identical to UHS_ARITH_FMA."""
    st, a0 = _growing(2)
    ga, _ = run_gpu(st, a0, AUTO)
    fa, _ = run_gpu(st, a0, FMA)
    assert np.isfinite(ga).all()
    assert np.array_equal(ga.view(np.uint64), fa.view(np.uint64))
