"""The float-pair bounded sum's arithmetic (df32.cuh: bound_add, sigma_of,
dfs_mul, dfs_fma, then one TwoSum), restated in C on the host with the C
library's correctly rounded fmaf (tests/c/bounded_sum_check.c): on random
stencil sums of 3-19 float-pair terms -- coefficients of one or mixed sign,
values of one or mixed sign spread over up to 2^79 -- every partial sum of
the extracted high parts is exact in a float, and the result is within
n^2 2^-46 of B = sum |ch_k| |xh_k| of the exact sum (computed in
binary128)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_bounded_sum_is_exact_in_its_high_part_and_within_its_bound(tmp_path):
    exe = tmp_path / "bounded_sum_check"
    r = subprocess.run(["gcc", "-O2", "-ffp-contract=off", os.path.join(HERE, "c", "bounded_sum_check.c"), "-lm",
                        "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0 and "float128" in r.stderr:
        pytest.skip("this compiler has no binary128 type")
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe), "120000", "11"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "violations=0" in out.stdout
