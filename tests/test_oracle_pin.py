"""The oracle is pinned to the reference's own CPU loops.

Where oracle/_ref exists (built by oracle/build_ref.py from the reference
checkout) each UH-SW driver's mpe_verify() runs on its own data and the oracle
must reproduce its grid bit-for-bit.  Everywhere, the oracle's result must
hash to the digest tests/golden/make_golden.py recorded from that comparison.
"""
import hashlib
import os
import tempfile

import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from golden_util import load, reference_stencil

PINS = load("reference_pins.json")
FAST = [c for c, p in PINS.items() if p["driver"] == "sw"]


def _oracle_run(case, kind):
    st = reference_stencil(case, kind)
    n = int(np.prod(st.sizes))
    a = np.empty(n)
    if kind == "sw":
        b = np.empty(n)
        oracle.fill_rand50([a, b])
    else:
        b = np.zeros(n)
        oracle.fill_rand50([a])
    oracle.iterate_f64(st, a, b)
    return st, a


@pytest.mark.parametrize("case", FAST)
def test_oracle_matches_reference_driver(case):
    st, a = _oracle_run(case, "sw")
    assert hashlib.sha256(a.tobytes()).hexdigest() == PINS[case]["sha256"]
    if oracle.ref_available(case, "sw"):
        ref = oracle.run_ref_sw(case, a.size)
        assert np.array_equal(ref.view(np.uint64), a.view(np.uint64))


def test_oracle_matches_343pt_box_digest():
    """UH-SW/3d3r_box/stencil_3d343pt_driver.serial.c:43 skips its own loops,
    so the 343-point box is pinned through UH-GPU/3d3r_box's cpu_verify
    (512^3, T = 4); its digest was recorded after a bit-exact comparison."""
    st, a = _oracle_run("3d3r_box", "gpu")
    assert hashlib.sha256(a.tobytes()).hexdigest() == PINS["3d3r_box"]["sha256"]


def fusion_program():
    rec = load("fusion_pins.json")["program"]
    return uhs.Stencil(name=rec["name"], rank=rec["rank"], sizes=tuple(rec["sizes"]), lb=tuple(rec["lb"]),
                       ub=tuple(rec["ub"]), terms=[tuple(t) for t in rec["terms"]], iterations=rec["iterations"],
                       exact_order=rec["exact_order"])


def test_oracle_matches_fused_reference_program():
    """Spatial kernel fusion: the program laplaceAddInput inlines its producer
    kernel (laplace) into its consumer (addInput), as the reference's
    kernel-fusion pass does (lib/Dialect/Stencil/StencilKernelFusion.cpp:
    70-183).  The DSL reader's fused term list, run by the oracle on the
    driver's own rand() % 50 data, reproduces the grid the driver's serial
    loop leaves (laplaceAddInputIteration_driver.c:37-58): through the
    recorded digest everywhere, and bit-for-bit against the driver itself
    where oracle/_ref holds it."""
    pin = load("fusion_pins.json")
    st = fusion_program()
    n = int(np.prod(st.sizes))
    a, b = np.empty(n), np.empty(n)
    oracle.fill_rand50([a, b])
    oracle.iterate_f64(st, a, b)
    assert hashlib.sha256(a.tobytes()).hexdigest() == pin["sha256"]
    exe = os.path.join(oracle.REF_DIR, "fusion_laplaceAddInputIteration")
    if os.path.exists(exe):
        from oracle.build_ref import run_fusion_driver
        with tempfile.TemporaryDirectory() as d:
            ref = np.array(run_fusion_driver(d))
        assert np.array_equal(ref.view(np.uint64), a.view(np.uint64))


def test_oracle_rejects_odd_iteration_counts():
    st = reference_stencil("2d1r_star").with_(sizes=(1, 6, 6), lb=(0, 1, 1), ub=(1, 5, 5))
    a, b = np.zeros(36), np.zeros(36)
    with pytest.raises(ValueError):
        oracle.iterate_f64(st, a, b, T=3)


def test_oracle_thread_count_does_not_change_results():
    st = reference_stencil("3d1r_box").with_(sizes=(20, 21, 22), lb=(1, 1, 1), ub=(19, 20, 21), iterations=4)
    n = int(np.prod(st.sizes))
    rng = np.random.default_rng(3)
    a0 = rng.random(n)
    outs = []
    for th in (1, 3):
        oracle.set_threads(th)
        a, b = a0.copy(), a0.copy()
        oracle.iterate_f64(st, a, b)
        outs.append(a)
    oracle.set_threads(oracle.max_threads())
    assert np.array_equal(outs[0], outs[1])
