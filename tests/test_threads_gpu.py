"""Concurrent host threads: four threads, each with its own stream and
grids, run programs of different shapes, element types and kernels at the
same time (shared state: the TMA map cache, the tuner database, per-stream
status words, error-reduction scratch).  Every result matches the oracle."""
import threading

import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from gpu_util import assert_f64_close, run_oracle
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu

JOBS = [  # (rank, r, kind, interior, T, seed, dtype)
    (3, 1, "star", (40, 48, 64), 6, 201, uhs.UHS_F64),
    (3, 2, "box", (20, 24, 40), 4, 202, uhs.UHS_F64),
    (2, 3, "star", (300, 256), 8, 203, uhs.UHS_F32),
    (3, 3, "star", (24, 32, 48), 4, 204, uhs.UHS_F32),
]


def test_concurrent_calls_from_host_threads(cuda):
    import torch
    results, errors = {}, []

    def worker(i, rank, r, kind, interior, T, seed, dtype):
        try:
            st, a0 = random_case(rank, r, kind, interior, T, seed, dtype=dtype)
            tdt = torch.float32 if dtype == uhs.UHS_F32 else torch.float64
            s = torch.cuda.Stream()
            shape = st.sizes if rank == 3 else st.sizes[1:]
            host = a0.astype(np.float32) if dtype == uhs.UHS_F32 else a0
            for rep in range(3):
                with torch.cuda.stream(s):
                    a = torch.from_numpy(host.reshape(shape)).to(device="cuda", dtype=tdt)
                    b = a.clone()
                uhs.run(st, a, b, stream=s)
                with torch.cuda.stream(s):
                    ref = a.double()
                e = uhs.error_norms(st, a, ref, stream=s)  # shared scratch, per-device lock
                assert e["max_abs"] == 0.0, e
                s.synchronize()
                results[(i, rep)] = (st, host.astype(np.float64), a.double().cpu().numpy().reshape(-1))
                del a, b, ref
        except Exception as e:  # reported below
            errors.append((i, repr(e)))

    threads = [threading.Thread(target=worker, args=(i,) + job) for i, job in enumerate(JOBS)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    assert len(results) == 3 * len(JOBS)
    for (i, rep), (st, x0, got) in results.items():
        ra, _ = run_oracle(st, x0)
        if st.dtype == uhs.UHS_F32:
            assert oracle.error(st, ra, got)["l2_rel"] <= 1e-6
        else:
            assert_f64_close(st, ra, got)
