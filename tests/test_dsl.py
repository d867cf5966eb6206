"""The DSL reader (include/uhs_dsl.h) on the CPU: the grammar and its
reduction to a term list on programs written for these tests, rejection of
malformed text with UHS_EPARSE and a position, a mutation fuzz (every
mutated text parses or is rejected, nothing crashes), and -- where the
reference checkout is present -- all 24 reference programs against the
recorded fixture."""
import ctypes
import glob
import json
import os
import random

import pytest

import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
from oracle.build_ref import reference_root

REF = reference_root() or ""

HEAT3D = """# seven-point heat step
stencil heat3d(double t[18][20][22]) {
    iteration(6)
    operation(step)
    kernel step {
        tile(2, 4, 8)
        domain([1, 17][1, 19][1, 21])
        expr {
            0.125*t[z-1][y][x] + 0.0625*t[z+1][y][x] +
            0.25*t[z][y-1][x] + 0.125*t[z][y+1][x] +   # rows
            0.0625*t[z][y][x-1] + 0.125*t[z][y][x+1] +
            0.25*t[z][y][x]
        }
    }
}
"""

BLUR2D = """stencil blur2d(float img[30][40]) {
    iteration(1)
    operation(b)
    kernel b {
        domain([1, 29][1, 39])
        expr {
            0.0625*img[y-1][x-1] + 0.125*img[y-1][x] + 0.0625*img[y-1][x+1] +
            0.125*img[y][x-1] + 0.25*img[y][x] + 0.125*img[y][x+1] +
            0.0625*img[y+1][x-1] + 0.125*img[y+1][x] + 0.0625*img[y+1][x+1]
        }
    }
}
"""


def test_heat3d_program():
    st = uhs.parse_dsl(HEAT3D, "heat3d.dsl")
    assert st.name == "heat3d" and st.rank == 3 and st.dtype == _lib.UHS_F64
    assert st.sizes == (18, 20, 22) and st.lb == (1, 1, 1) and st.ub == (17, 19, 21)
    assert st.iterations == 6 and st.exact_order
    assert st.terms == [(-1, 0, 0, 0.125), (1, 0, 0, 0.0625), (0, -1, 0, 0.25), (0, 1, 0, 0.125),
                        (0, 0, -1, 0.0625), (0, 0, 1, 0.125), (0, 0, 0, 0.25)]
    prog = _program(HEAT3D)
    tile = (ctypes.c_int64 * 3)()
    assert _lib.lib().uhs_program_tile(prog, tile) == 3 and tuple(tile) == (2, 4, 8)
    assert _lib.lib().uhs_program_num_kernels(prog) == 1
    _lib.lib().uhs_program_free(prog)


def test_blur2d_float_program():
    st = uhs.parse_dsl(BLUR2D)
    assert st.rank == 2 and st.dtype == _lib.UHS_F32 and st.sizes == (1, 30, 40)
    assert st.lb == (0, 1, 1) and st.ub == (1, 29, 39) and st.iterations == 1
    assert len(st.terms) == 9 and sum(t[3] for t in st.terms) == 1.0
    assert uhs.plan(st).kernel == _lib.UHS_KERNEL_STREAM


def test_precedence_leading_minus_and_division():
    st = uhs.parse_dsl("""stencil p(double u[12][16]) {
        iteration(2) operation(k)
        kernel k { domain([1, 11][1, 15]) expr { -0.5*u[y][x] + 2*u[y][x-1] * 0.25 - u[y][x+1]/4 } } }""")
    assert st.terms == [(0, 0, 0, -0.5), (0, 0, -1, 0.5), (0, 0, 1, -0.25)]
    assert not st.exact_order  # 2 * u * 0.25 is rounded twice in the expression tree


def test_kernel_references_are_inlined():
    """A consumer kernel reading a producer kernel's output: the producer is
    inlined (spatial fusion) into one sweep."""
    st = uhs.parse_dsl("""stencil fuse(float v[20][24]) {
        iteration(4)
        operation(vert)
        kernel horiz { domain([1, 19][1, 23]) expr { 0.5*v[y][x-1] + 0.5*v[y][x+1] } }
        kernel vert { domain([1, 19][1, 23]) expr { 0.5*horiz[y-1][x] + 0.5*horiz[y+1][x] } }
    }""")
    assert sorted(st.terms) == [(0, -1, -1, 0.25), (0, -1, 1, 0.25), (0, 1, -1, 0.25), (0, 1, 1, 0.25)]


def test_parameter_arrays():
    text = """stencil par(double w[10][12][14], c[3]) {
        iteration(2) operation(k)
        kernel k { domain([1, 9][1, 11][1, 13]) expr { c[0]*w[z][y][x] + c[1]*w[z-1][y][x] + c[2]*w[z+1][y][x] } } }"""
    st = uhs.parse_dsl(text)
    assert [t[:3] for t in st.terms] == [(0, 0, 0), (-1, 0, 0), (1, 0, 0)]
    assert st.param_terms == {0: 0, 1: 1, 2: 2}
    prog = _program(text)
    L = _lib.lib()
    assert L.uhs_program_num_param_arrays(prog) == 1
    vals = (ctypes.c_double * 3)(0.5, 0.25, 0.25)
    assert L.uhs_program_set_params(prog, vals, 3) == _lib.UHS_OK
    L.uhs_program_free(prog)


def test_odd_iteration_count_is_rejected_by_the_runtime():
    st = uhs.parse_dsl(HEAT3D.replace("iteration(6)", "iteration(3)"))
    assert st.iterations == 3
    with pytest.raises(uhs.UhsError) as ei:
        uhs.plan(st)
    assert ei.value.code == _lib.UHS_EINVAL


@pytest.mark.parametrize("text,where", [
    ("", "1:"),
    ("stencil s(double a[4][4]) { iteration(2) operation(k) kernel k { domain([1,3][1,3]) expr { a[y][x] }",
     None),
    ("stencil s(double a[4][4]) { iteration(2) operation(nope) kernel k { domain([1,3][1,3]) expr { a[y][x] } } }",
     None),
    ("stencil s(double a[4][4]) { iteration(2) operation(k) kernel k { domain([1,3][1,3]) expr { b[y][x] } } }",
     None),
    ("stencil s(double a[4][4]) { iteration(2) operation(k) kernel k { domain([1,3][1,3]) expr { a[y][x] + } } }",
     None),
    ("stencil s(double a[4][4]) { iteration(two) operation(k) kernel k { domain([1,3][1,3]) expr { a[y][x] } } }",
     "1:"),
    ("stencil s(int a[4][4]) { iteration(2) operation(k) kernel k { domain([1,3][1,3]) expr { a[y][x] } } }", "1:"),
])
def test_malformed_programs_are_rejected_with_a_position(text, where):
    prog = ctypes.c_void_p()
    rc = _lib.lib().uhs_dsl_parse(text.encode(), b"bad.dsl", ctypes.byref(prog))
    assert rc in (_lib.UHS_EPARSE, _lib.UHS_EUNSUPPORTED)
    assert not prog.value
    msg = _lib.last_error()
    assert msg
    if where:
        assert "bad.dsl@" + where in msg


def test_mutation_fuzz_never_crashes():
    """600 seeded mutations of two programs (a character deleted, inserted,
    replaced, or the text cut short): each parses or is rejected cleanly."""
    rng = random.Random(2024)
    alphabet = "[](){}+-*/.,#0123456789xyzabc \n"
    L = _lib.lib()
    outcomes = {"ok": 0, "rejected": 0}
    for base in (HEAT3D, BLUR2D):
        for _ in range(300):
            t = list(base)
            for _ in range(rng.randint(1, 4)):
                op = rng.randrange(4)
                i = rng.randrange(len(t))
                if op == 0:
                    del t[i]
                elif op == 1:
                    t.insert(i, rng.choice(alphabet))
                elif op == 2:
                    t[i] = rng.choice(alphabet)
                else:
                    t = t[:i]
                if not t:
                    break
            prog = ctypes.c_void_p()
            rc = L.uhs_dsl_parse("".join(t).encode(), b"fuzz.dsl", ctypes.byref(prog))
            if rc == _lib.UHS_OK:
                outcomes["ok"] += 1
                d = _lib.StencilDesc()
                sizes = (ctypes.c_int64 * 3)()
                L.uhs_program_desc(prog, ctypes.byref(d), sizes)
                L.uhs_program_free(prog)
            else:
                assert rc in (_lib.UHS_EPARSE, _lib.UHS_EUNSUPPORTED, _lib.UHS_EINVAL), rc
                assert not prog.value
                outcomes["rejected"] += 1
    assert outcomes["rejected"] > 0 and outcomes["ok"] > 0


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_reference_programs_match_the_recorded_fixture():
    """Every UH-SW and UH-GPU .dsl of the reference parses to the program
    recorded in tests/golden/reference_stencils.json."""
    with open(os.path.join(HERE, "golden", "reference_stencils.json")) as f:
        recs = json.load(f)
    n = 0
    for case, kinds in recs.items():
        for kind, rec in kinds.items():
            path = os.path.join(REF, rec["dsl"])
            st = uhs.parse_dsl_file(path)
            assert st.name == rec["name"] and st.rank == rec["rank"]
            assert list(st.sizes) == rec["sizes"] and list(st.lb) == rec["lb"] and list(st.ub) == rec["ub"]
            assert st.iterations == rec["iterations"] and st.exact_order == rec["exact_order"]
            assert [list(t) for t in st.terms] == rec["terms"]
            n += 1
    assert n == 24
    assert len(glob.glob(os.path.join(REF, "UH-GPU", "*", "*.dsl"))) == 12


def _program(text):
    prog = ctypes.c_void_p()
    _lib.check(_lib.lib().uhs_dsl_parse(text.encode(), b"t.dsl", ctypes.byref(prog)))
    return prog


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_reader_fuses_the_reference_producer_consumer_program():
    """laplaceAddInputIteration.dsl has two kernels: laplace (a 5-point
    expression over the two slowest axes) and addInput, which reads laplace at
    the same point.  The reader inlines the producer into the consumer -- the
    reference's kernel-fusion pass (lib/Dialect/Stencil/StencilKernelFusion.cpp:
    70-183) -- giving one sweep with the recorded term list.  The domain
    covers the fastest axis whole ([0, 16), no halo on it)."""
    from oracle.build_ref import FUSION_DSL
    rec = json.load(open(os.path.join(HERE, "golden", "fusion_pins.json")))["program"]
    st = uhs.parse_dsl_file(os.path.join(REF, FUSION_DSL))
    assert st.name == rec["name"] and list(st.sizes) == rec["sizes"]
    assert list(st.lb) == rec["lb"] and list(st.ub) == rec["ub"] and st.iterations == rec["iterations"]
    assert [list(t) for t in st.terms] == rec["terms"]
    assert st.lb[2] == 0 and st.ub[2] == st.sizes[2]
    # consumer's own access first, then the inlined producer's five terms;
    # the consumer adds a subtree, so the linear form is not a left-deep sum
    assert st.terms[0][:3] == (0, 0, 0) and len(st.terms) == 6 and not st.exact_order
