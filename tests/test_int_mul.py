"""The IEEE-754 binary64 multiplication on the integer pipes (golikov_2d_gb300/csrc/gd_swfp.cuh)
that the fast Euler and MHD kernels use for part of their products, and its exact halving and
doubling.  On the CPU the header is compiled for the host and checked against the host's
multiplication bit for bit on random bit patterns, typical magnitudes, products near the
overflow and underflow limits, short significands (exact products and halfway cases), zeros,
all-ones significands, subnormal operands, infinities and NaNs (two NaNs count as equal: the
integer path returns the canonical quiet NaN); halving and doubling against x * 0.5 and x + x
on random bit patterns and on subnormals and the exponent range's edges.  On the GPU,
gd_check_int_mul compares the device code with the FP64 unit's multiply, and
gd_check_fast_roots measures the two-operation reciprocal and root against IEEE results."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_integer_multiply_matches_host_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "swfp_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "swfp_check.cpp")],
                   check=True)
    r = subprocess.run([exe, "2000000", "20260904"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if "cases" in ln]
    assert len(lines) == 11
    assert all(ln.split()[ln.split().index("mismatches") + 1] == "0" for ln in lines)


@pytest.mark.gpu
def test_integer_multiply_matches_fp64_unit():
    import golikov_2d_gb300 as g
    c = g.check_int_mul(1 << 26, seed=7)
    assert c["checked"] >= 1 << 26
    assert c["mismatches"] == 0, c
    assert c["slow_path"] > 0  # the subnormal and limit classes take the general path


@pytest.mark.gpu
def test_two_operation_roots_within_two_ulp():
    """The Euler step's reciprocal and sound-speed root in two FP64 operations (the Newton
    correction's quadratic term added to the bit pattern on the integer pipe) stay within a
    unit or two of the IEEE results (the IEEE root of a quotient rounds twice itself)."""
    import golikov_2d_gb300 as g
    c = g.check_fast_roots(1 << 24, seed=3)
    assert c["checked"] >= 1 << 24
    assert c["rcp_2op_ulp"] <= 1, c
    assert c["sqrt_over_2op_ulp"] <= 2, c
    assert c["sqrt_over_ulp"] <= 2, c
