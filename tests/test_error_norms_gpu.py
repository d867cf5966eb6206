"""uhs_error_norms (FP64 error reduction on the GPU) against the oracle's host
reduction of the same grids."""
import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from gpu_util import to_dev
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu


def _close(got, want, rel=1e-10):
    for k in ("l2_rel", "max_abs", "max_rel", "max_ref"):
        assert got[k] == pytest.approx(want[k], rel=rel, abs=1e-300), (k, got, want)


# the last two have few long rows: each row block is also cut along x
@pytest.mark.parametrize("rank,interior", [(3, (17, 33, 70)), (2, (300, 129)), (2, (40, 2999)), (3, (2, 3, 5000))])
def test_error_norms_f64_f32_pairs(cuda, rank, interior):
    import torch
    st, ref = random_case(rank, 1, "star", interior, 2, 21)
    rng = np.random.default_rng(5)
    x = ref + 1e-9 * rng.standard_normal(ref.size)
    want = oracle.error(st, ref, x)
    got = uhs.error_norms(st, to_dev(x, st), to_dev(ref, st))
    _close(got, want)
    x32 = ref.astype(np.float32)
    want32 = oracle.error(st, ref, x32)
    got32 = uhs.error_norms(st.with_(dtype=uhs.UHS_F32), to_dev(x32, st, torch.float32), to_dev(ref, st))
    _close(got32, want32)
    hi = ref.astype(np.float32)
    lo = (ref - hi.astype(np.float64)).astype(np.float32)
    pairs = np.stack([hi, lo], -1).reshape(-1).view(np.float64)
    gotp = uhs.error_norms(st.with_(dtype=uhs.UHS_F32X2), to_dev(pairs, st), to_dev(ref, st))
    wantp = oracle.error(st, ref, hi.astype(np.float64) + lo.astype(np.float64))
    _close(gotp, wantp, rel=1e-6)


def test_error_norms_identical_grids_and_empty_domain(cuda):
    st, ref = random_case(3, 2, "box", (9, 10, 11), 2, 4)
    d = to_dev(ref, st)
    got = uhs.error_norms(st, d, d.clone())
    assert got["l2_rel"] == 0.0 and got["max_abs"] == 0.0
    assert got["max_ref"] == pytest.approx(oracle.error(st, ref, ref)["max_ref"])
    empty = st.with_(ub=st.lb)
    assert uhs.error_norms(empty, d, d)["l2_rel"] == 0.0


def test_error_norms_special_values(cuda):
    """Zeros of both signs, subnormal, huge and infinite FP32 values are
    widened exactly (the results equal the oracle's); a NaN in the result
    makes max |x - r| infinite and the L2 norm NaN; a NaN in the reference
    does not raise max |r|."""
    import torch
    st, ref = random_case(3, 1, "star", (6, 7, 40), 2, 8)
    x32 = ref.astype(np.float32)
    sz = st.sizes
    flat = lambda z, y, xx: (z * sz[1] + y) * sz[2] + xx  # noqa: E731
    specials = [0.0, -0.0, 1e-40, -3e-39, 3.0e38, -1.5e-45]
    for j, v in enumerate(specials):
        x32[flat(1 + j % 6, 1 + j, 1 + 5 * j)] = np.float32(v)
    got = uhs.error_norms(st.with_(dtype=uhs.UHS_F32), to_dev(x32, st, torch.float32), to_dev(ref, st))
    _close(got, oracle.error(st, ref, x32), rel=1e-12)
    x32[flat(3, 3, 3)] = np.float32("inf")
    got = uhs.error_norms(st.with_(dtype=uhs.UHS_F32), to_dev(x32, st, torch.float32), to_dev(ref, st))
    assert got["max_abs"] == float("inf")
    x32[flat(2, 4, 9)] = np.float32("nan")
    got = uhs.error_norms(st.with_(dtype=uhs.UHS_F32), to_dev(x32, st, torch.float32), to_dev(ref, st))
    assert np.isnan(got["l2_rel"]) and got["max_abs"] == float("inf")
    ref2 = ref.copy()
    ref2[flat(4, 2, 7)] = float("nan")
    got = uhs.error_norms(st, to_dev(ref2, st), to_dev(ref2, st))
    want = oracle.error(st, ref2, ref2)
    assert np.isfinite(want["max_ref"]) and got["max_ref"] == want["max_ref"]
    assert got["max_abs"] == want["max_abs"] == float("inf")
