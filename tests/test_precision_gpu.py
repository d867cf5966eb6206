"""Precision study (configuration 4): 3d2r_star with a smooth field
sin(x)cos(y)sin(z) + 1e-3 noise, run in FP32 grids, float-pair grids
(UHS_F32X2), FP64 grids in float-pair arithmetic and FP64 grids in native
arithmetic; every 20 steps each is scored on the GPU (uhs_error_norms)
against the FP64 oracle's state.

It runs at 96^3 and at the configuration's full size, 512^3, both with
T = 200 (the bars, at every 20th step: FP64 paths and float pairs within
1e-12 of the oracle, FP32 within a relative L2 of 1e-6).  With
UHS_PRECISION_N set only that size runs, and the table is written to
UHS_PRECISION_OUT when that is set.
"""
import json
import os
import time

import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from uxxxxxxxxh_gb300.workloads import cfg4

pytestmark = pytest.mark.gpu


SIZES = [int(os.environ["UHS_PRECISION_N"])] if os.environ.get("UHS_PRECISION_N") else [96, 512]


@pytest.mark.parametrize("n", SIZES)
def test_precision_study(cuda, n):
    import torch
    T, every = 200, 20
    oracle.set_threads(os.cpu_count() or 1)
    st, a0 = cfg4(n=n, T=T)
    shape = st.sizes

    def dev(x, dt):
        return torch.from_numpy(x.reshape(shape)).to(dt).cuda()

    hi = a0.astype(np.float32)
    lo = (a0 - hi.astype(np.float64)).astype(np.float32)
    pairs = np.stack([hi, lo], -1).reshape(-1).view(np.float64)
    variants = {
        "f32": (st.with_(dtype=_lib.UHS_F32, iterations=every), dev(a0, torch.float32), uhs.RunParams()),
        "f32x2": (st.with_(dtype=_lib.UHS_F32X2, iterations=every), dev(pairs, torch.float64), uhs.RunParams()),
        "f64_df32": (st.with_(iterations=every), dev(a0, torch.float64), uhs.RunParams(arith=_lib.UHS_ARITH_DF32)),
        "f64_native": (st.with_(iterations=every), dev(a0, torch.float64), uhs.RunParams(arith=_lib.UHS_ARITH_FMA)),
    }
    grids = {k: (v[1], v[1].clone()) for k, v in variants.items()}
    ra, rb = a0.copy(), a0.copy()
    ref = torch.empty(shape, dtype=torch.float64, device="cuda")
    rows = []
    for step in range(every, T + 1, every):
        t0 = time.time()
        oracle.iterate_f64(st, ra, rb, every)
        row = {"step": step, "oracle_seconds": time.time() - t0}
        ref.copy_(torch.from_numpy(ra.reshape(shape)))
        for k, (s, _, p) in variants.items():
            a, b = grids[k]
            torch.cuda.synchronize()
            t1 = time.time()
            uhs.run(s, a, b, p)
            row[k + "_seconds"] = time.time() - t1
            row[k] = uhs.error_norms(s, a, ref)
        rows.append(row)
    out = os.environ.get("UHS_PRECISION_OUT")
    if out:
        with open(out, "w") as f:
            json.dump({"config": f"cfg4 3d2r_star {n}^3 T={T}", "every": every, "rows": rows}, f, indent=1)
    for row in rows:
        for k in ("f32x2", "f64_df32", "f64_native"):
            assert row[k]["max_rel"] <= 1e-12, (row["step"], k, row[k])
        assert row["f32"]["l2_rel"] <= 1e-6, (row["step"], row["f32"])
    # the FP64 grids' halos are never written: bit-identical to the oracle's
    for k in ("f64_df32", "f64_native"):
        for g, r in zip(grids[k], (ra, rb)):
            assert oracle.halo_diff(st, r, g.cpu().numpy().reshape(-1)) == 0, k
