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
