"""CPU: the float-float helpers of the FP64 pair kernel (csrc/ff.cuh),
compiled for the host from the same header, against long double arithmetic.

Bars: the double -> float-float split keeps 2^-47 of the value; the way back
to double is within half an ulp; sums, products, reciprocal, rsqrt and sqrt
stay within 2^-45 relative; the pair velocity factor f0 (1/|d| - 1/(r1 + r2))
within 2^-45 of 1/|d|; the chord area r2^2 - w^2 / 4 within 2^-45 of
r1^2 + r2^2 + |d|^2. These bound the FP64 form's pair terms well inside its
1e-12 parity bar. The FP64 reciprocal and reciprocal square root built on
them (one or two FP64 instructions) stay within 1 ulp."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def errors():
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "ff_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(HERE, "ff_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout
    return {ln.split()[0]: float(ln.split()[1]) for ln in out.splitlines() if ln.strip()}


def test_split_and_back(errors):
    assert errors["split"] <= 2.0 ** -47
    assert errors["to_double_ulps"] <= 0.5
    assert errors["to_double"] <= 2.0 ** -53


@pytest.mark.parametrize("op", ["add", "add_cancel_abs", "mul", "sqr", "rcp", "rsqrt", "sqrt",
                                "pair_velocity", "chord_area_abs", "sqrt_ffd"])
def test_operations(errors, op):
    assert errors[op] <= 2.0 ** -45, (op, errors[op])


def test_exact_subtraction_bit_identical(errors):
    """sub_exact (the FP64 pair kernel's position differences on the integer
    pipe) equals the FP64 subtraction bit for bit."""
    assert errors["sub_exact_mismatches"] == 0


def test_fp64_results_with_few_fp64_instructions(errors):
    """1/sqrt and 1/x of the FP64 kernels (float-float estimate, one FP64
    residual, the correction added on the integer pipe): within 1 ulp; the
    small addition within 1/2 ulp plus its FP32 rounding."""
    assert errors["rsqrt_d_ulps"] <= 1.0
    assert errors["rcp_d_ulps"] <= 1.0
    assert errors["add_small_ulps"] <= 0.51
