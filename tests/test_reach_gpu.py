"""Programs whose reach is shorter than their radius on some axis, or one-
sided: no z offsets at all on a grid without a z halo, and upwind stencils
reaching only down or only up in z with the halo on that side only.  They
run on the generic kernel (the planner keeps the templated star/box kernels
for full symmetric reach) and must match the oracle: exact mode bit-identical,
FMA within 1e-12; cells outside the domain are never written."""
import numpy as np
import pytest

import uxxxxxxxxh_gb300 as uhs
from gpu_util import assert_f64_close, assert_halo_exact, run_gpu, run_oracle
from uxxxxxxxxh_gb300.stencil import Stencil
from uxxxxxxxxh_gb300.workloads import splitmix_uniform

pytestmark = pytest.mark.gpu

CASES = {
    # in-plane 5-point star in a 3D grid with no z halo
    "inplane": dict(sizes=(6, 20, 40), lb=(0, 1, 1), ub=(6, 19, 39),
                    terms=[(0, -1, 0, 0.2), (0, 0, -1, 0.2), (0, 0, 0, 0.2), (0, 0, 1, 0.2), (0, 1, 0, 0.2)]),
    # reaches one plane down only; halo below, none above
    "down": dict(sizes=(9, 20, 40), lb=(1, 1, 1), ub=(9, 19, 39),
                 terms=[(-1, 0, 0, 0.25), (0, -1, 0, 0.125), (0, 0, -1, 0.125), (0, 0, 0, 0.25), (0, 0, 1, 0.125),
                        (0, 1, 0, 0.125)]),
    # reaches up to two planes up only; no halo below (planes -1, -2 never exist)
    "up": dict(sizes=(10, 20, 40), lb=(0, 1, 1), ub=(8, 19, 39),
               terms=[(0, 0, 0, 0.4), (1, 0, 0, 0.2), (2, 0, 0, 0.1), (0, -1, 0, 0.075), (0, 1, 0, 0.075),
                      (0, 0, -1, 0.075), (0, 0, 1, 0.075)]),
}


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("arith", [uhs.UHS_ARITH_EXACT, uhs.UHS_ARITH_FMA])
def test_short_and_one_sided_reach(cuda, name, arith):
    c = CASES[name]
    st = Stencil(name=name, rank=3, sizes=c["sizes"], lb=c["lb"], ub=c["ub"], terms=c["terms"], iterations=6)
    assert uhs.plan(st).kernel == uhs.UHS_KERNEL_GENERIC
    a0 = 2.0 * splitmix_uniform(77, int(np.prod(st.sizes))) - 1.0
    ra, rb = run_oracle(st, a0)
    ga, gb = run_gpu(st, a0, uhs.RunParams(arith=arith))
    if arith == uhs.UHS_ARITH_EXACT:
        assert np.array_equal(ra, ga) and np.array_equal(rb, gb)
    else:
        assert_f64_close(st, ra, ga)
        assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)
