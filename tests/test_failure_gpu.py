"""Failure detection without a GPU fault: a device wait that nothing
completes runs out of its bound, the kernel records the timeout in the
device status word and returns, the host reports UHS_ETIMEOUT with where it
happened -- and the context stays usable: the next sweeps run and match the
oracle, and the status word is clear again."""
import numpy as np
import pytest

import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from gpu_util import assert_f64_close, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cycles", [1, 1 << 16, 1 << 24])
def test_bounded_wait_reports_timeout_and_device_recovers(cuda, cycles):
    import torch
    rc = uhs.probe_wait_timeout(cycles)
    assert rc == _lib.UHS_ETIMEOUT
    assert "bounded wait" in _lib.last_error()
    # the context is usable and the status word was cleared by the report
    st, a0 = random_case(3, 1, "star", (20, 24, 40), 4, 91)
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0)
    assert_f64_close(st, ra, ga)
    torch.cuda.synchronize()


def test_timeout_on_a_stream_then_sweeps_on_it(cuda):
    import torch
    s = torch.cuda.Stream()
    assert uhs.probe_wait_timeout(1 << 12, stream=s) == _lib.UHS_ETIMEOUT
    st, a0 = random_case(3, 2, "box", (12, 20, 36), 2, 92)
    a = torch.from_numpy(a0.reshape(st.sizes)).cuda()
    b = a.clone()
    uhs.run(st, a, b, stream=s)
    ra, _ = run_oracle(st, a0)
    assert_f64_close(st, ra, a.cpu().numpy().reshape(-1))
    assert np.isfinite(a.cpu().numpy()).all()


def test_allocation_failure_is_reported_and_recovers(cuda):
    """A simulated out-of-memory (every library allocation above 64 bytes
    fails): batch creation and the MLP report UHS_ENOMEM and leak nothing;
    with the cap removed the same calls succeed."""
    import torch
    from uxxxxxxxxh_gb300.costmodel import MLP
    L = _lib.lib()
    st, a0 = random_case(3, 1, "star", (16, 16, 32), 2, 93)
    a = torch.from_numpy(a0.reshape(st.sizes)).cuda()
    b = a.clone()
    assert L.uhs_set_alloc_cap(64) == _lib.UHS_OK
    try:
        with pytest.raises(uhs.UhsError) as ei:
            uhs.Batch([st], [a], [b], uhs.RunParams())
        assert ei.value.code == _lib.UHS_ENOMEM
        with pytest.raises(uhs.UhsError) as ei:
            MLP(8, 16, 2)
        assert ei.value.code == _lib.UHS_ENOMEM
    finally:
        assert L.uhs_set_alloc_cap(0) == _lib.UHS_OK
    batch = uhs.Batch([st], [a], [b], uhs.RunParams())
    batch.run()
    ra, _ = run_oracle(st, a0)
    assert_f64_close(st, ra, a.cpu().numpy().reshape(-1))
    assert MLP(8, 16, 2).num_params > 0
    assert L.uhs_set_alloc_cap(-1) == _lib.UHS_EINVAL
