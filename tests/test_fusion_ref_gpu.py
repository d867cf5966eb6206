"""Spatial kernel fusion against the reference's own fused program.

laplaceAddInput (UHStencil/test/Examples/StencilDialect/
laplaceAddInputIteration) has a producer kernel, laplace, read by its consumer
addInput at the same point; the reference's kernel-fusion pass inlines the
producer into the consumer (lib/Dialect/Stencil/StencilKernelFusion.cpp:
70-183), and the DSL reader does the same, giving one sweep of six terms over
the two slowest axes whose domain covers the fastest axis whole (no halo on
it).  Swept on the GPU on the driver's own data (rand() % 50 in both grids,
T = 10), both grids must equal the grid the driver's serial loop leaves
(laplaceAddInputIteration_driver.c:37-58, recorded by its digest) bit for bit
in every arithmetic mode: the values are integers below 2^32, so every
product and sum is exact.  On random non-integer data at a larger size the
sweep must match the oracle within 1e-12."""
import hashlib

import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from golden_util import load
from gpu_util import assert_f64_close, assert_halo_exact, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import splitmix_uniform

pytestmark = pytest.mark.gpu


def fusion_program():
    rec = load("fusion_pins.json")["program"]
    return uhs.Stencil(name=rec["name"], rank=rec["rank"], sizes=tuple(rec["sizes"]), lb=tuple(rec["lb"]),
                       ub=tuple(rec["ub"]), terms=[tuple(t) for t in rec["terms"]], iterations=rec["iterations"],
                       exact_order=rec["exact_order"])


@pytest.mark.parametrize("arith", [_lib.UHS_ARITH_AUTO, _lib.UHS_ARITH_FMA, _lib.UHS_ARITH_EXACT])
def test_fused_program_equals_reference_loop(cuda, arith):
    pin = load("fusion_pins.json")
    st = fusion_program()
    n = int(np.prod(st.sizes))
    a0, b0 = np.empty(n), np.empty(n)
    oracle.fill_rand50([a0, b0])
    ga, gb = run_gpu(st, a0, uhs.RunParams(arith=arith), b0)
    assert hashlib.sha256(ga.tobytes()).hexdigest() == pin["sha256"]
    ra, rb = run_oracle(st, a0, b0)
    assert np.array_equal(gb.view(np.uint64), rb.view(np.uint64))
    assert_halo_exact(st, ra, ga)


def test_fused_program_at_a_larger_size_matches_oracle(cuda):
    st0 = fusion_program()
    st = st0.with_(sizes=(130, 66, 200), lb=(1, 1, 0), ub=(129, 65, 200))
    a0 = 2.0 * splitmix_uniform(31, int(np.prod(st.sizes))) - 1.0
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams())
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)
