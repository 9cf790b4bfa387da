"""GPU check of the FP64 helpers the step kernels use instead of IEEE
division / rsqrt / sqrt: they must agree with CUDA's results to a few ulp
over the argument range of the step (radii, squared distances, areas)."""
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


def test_rcp_rsqrt_sqrt_within_a_few_ulp(checker):
    rng = np.random.default_rng(0)
    x = np.concatenate([np.logspace(-12, 12, 200001), rng.uniform(1e-3, 50.0, 200000),
                        np.array([1.0, 2.0, 4.0, 0.25, 1e-300 * 1e290])])
    out = np.zeros((len(x), 8))
    assert checker.fp64_check(x.ctypes.data, len(x), out.ctypes.data) == 0
    rel = lambda a, b: np.max(np.abs(a - b) / np.abs(b))  # noqa: E731
    eps = np.finfo(np.float64).eps
    assert rel(out[:, 0], out[:, 1]) <= 4 * eps
    assert rel(out[:, 2], out[:, 3]) <= 4 * eps
    assert rel(out[:, 4], out[:, 5]) <= 4 * eps


def test_min_image_matches_reference_formula(checker):
    x = np.linspace(-30.0, 130.0, 100003)
    x = x[np.abs(np.abs(x - 50.0) - 40.0) > 1e-9]  # away from the half-box tie
    out = np.zeros((len(x), 8))
    assert checker.fp64_check(x.ctypes.data, len(x), out.ctypes.data) == 0
    assert np.array_equal(out[:, 6], out[:, 7])
