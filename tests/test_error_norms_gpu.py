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


@pytest.mark.parametrize("rank,interior", [(3, (17, 33, 70)), (2, (300, 129))])
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
