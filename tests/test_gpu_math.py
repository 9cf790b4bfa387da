"""GPU check of the FP64 helpers the step kernels use instead of IEEE
division and rsqrt: they must agree with CUDA's results to a few ulp over the
argument range of the step (radii, squared distances, areas)."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

from cubble_gb300 import buildlib

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def checker():
    d = tempfile.mkdtemp()
    so = os.path.join(d, "fp64_check.so")
    subprocess.run([buildlib.nvcc()] + buildlib.ARCH +
                   ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
                    "-I", buildlib.INCLUDE, os.path.join(HERE, "fp64_helpers_check.cu"),
                    "-o", so], check=True)
    lib = C.CDLL(so)
    lib.fp64_check.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    return lib


def test_rcp_rsqrt_within_a_few_ulp(checker):
    rng = np.random.default_rng(0)
    x = np.concatenate([np.logspace(-12, 12, 200001), rng.uniform(1e-3, 50.0, 200000),
                        np.array([1.0, 2.0, 4.0, 0.25, 1e-300 * 1e290])])
    out = np.zeros((len(x), 8))
    assert checker.fp64_check(x.ctypes.data, len(x), out.ctypes.data) == 0
    rel = lambda a, b: np.max(np.abs(a - b) / np.abs(b))  # noqa: E731
    eps = np.finfo(np.float64).eps
    assert rel(out[:, 0], out[:, 1]) <= 4 * eps
    assert rel(out[:, 2], out[:, 3]) <= 4 * eps
    # the helpers of the FP64 pair, predict and correct kernels (1 and 2
    # FP64 instructions): within 2 ulp of IEEE division and rsqrt()
    assert rel(out[:, 4], out[:, 1]) <= 2 * eps
    assert rel(out[:, 5], out[:, 3]) <= 2 * eps


def test_min_image_matches_reference_formula(checker):
    x = np.linspace(-30.0, 130.0, 100003)
    x = x[np.abs(np.abs(x - 50.0) - 40.0) > 1e-9]  # away from the half-box tie
    out = np.zeros((len(x), 8))
    assert checker.fp64_check(x.ctypes.data, len(x), out.ctypes.data) == 0
    assert np.array_equal(out[:, 6], out[:, 7])


def test_float_float_helpers_on_device(checker):
    """The FP64 pair kernel's float-float reciprocal, rsqrt and sqrt with the
    hardware FP32 estimates: within 2^-45 of the exact values (long double),
    and the split of a double keeps 2^-47 of it."""
    checker.ff_check.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    rng = np.random.default_rng(1)
    x = np.concatenate([np.logspace(-20, 20, 100001), rng.uniform(1e-3, 50.0, 100000)])
    out = np.zeros((len(x), 4))
    assert checker.ff_check(x.ctypes.data, len(x), out.ctypes.data) == 0
    L = x.astype(np.longdouble)
    rel = lambda a, b: np.max(np.abs(a.astype(np.longdouble) - b) / np.abs(b))  # noqa: E731
    assert rel(out[:, 0], L) <= 2.0 ** -47
    assert rel(out[:, 1], 1 / L) <= 2.0 ** -45
    assert rel(out[:, 2], 1 / np.sqrt(L)) <= 2.0 ** -45
    assert rel(out[:, 3], np.sqrt(L)) <= 2.0 ** -45


def test_exact_subtraction_on_device(checker):
    """The FP64 pair kernel's position differences (sub_exact: integer
    significands when the difference needs no rounding, the FP64 subtraction
    otherwise) are bit-identical to the FP64 subtraction: nearby values of
    both signs, across binade edges, equal, far apart, of opposite sign,
    zeros and subnormals."""
    checker.sub_check.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    rng = np.random.default_rng(2)
    n = 400000
    a = rng.choice([-1.0, 1.0], n) * np.exp2(rng.uniform(-40, 40, n))
    a[::3] = np.sign(a[::3]) * np.exp2(np.round(rng.uniform(-30, 30, len(a[::3]))))
    b = a + rng.choice([-1.0, 1.0], n) * np.abs(a) * np.exp2(rng.uniform(-55, 2, n))
    b[::11] = a[::11]
    b[::13] = -b[::13]
    b[::17] = 0.0
    a[::19] = a[::19] * 2.0 ** -1060
    box = rng.uniform(0.0, 175.0, n // 4)  # positions of nearby bubbles in a box
    a = np.concatenate([a, box])
    b = np.concatenate([b, box + rng.normal(0.0, 2.0, len(box))])
    out = np.zeros((len(a), 2))
    assert checker.sub_check(a.ctypes.data, b.ctypes.data, len(a), out.ctypes.data) == 0
    assert np.array_equal(out[:, 0].view(np.int64), out[:, 1].view(np.int64))
