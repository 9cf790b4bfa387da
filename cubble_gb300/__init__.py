"""cubble_gb300 — GB300-native (sm_103a) Durian wet-foam time step.

The compute path is libcubble_gb300.so (hand-written CUDA kernels behind the
C ABI of include/cubble_gb300.h). This package only loads it and mirrors the
reference's step-loop interface in Python (`GpuFoam`, see foam.py). There is
no CPU fallback: when the library cannot be built or loaded, every entry
point raises.
"""
import ctypes as C
import os

from . import _abi
from .foam import CubbleError, Foam, make_config  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcubble_gb300.so")
_lib = None


def build(force=False, verbose=False):
    from . import buildlib as _build
    return _build.build(force=force, verbose=verbose)


def lib():
    """Loads libcubble_gb300.so (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _abi.declare(_lib, "cb_")
    return _lib


def exported_symbols():
    """Names of the C-ABI functions declared in include/cubble_gb300.h."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "cubble_gb300.h")
    with open(hdr) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(cb_[a-z_0-9]+)\s*\(", text)))


class GpuFoam(Foam):
    """One foam on the current CUDA device (a `cb_context`)."""

    def __init__(self, config):
        super().__init__(lib(), "cb_", config)

    def integrate_timed(self, n_steps):
        r = _abi.Report()
        ms = C.c_double()
        self._call("integrate_timed", self._ctx, int(n_steps), C.byref(r), C.byref(ms))
        return r.as_dict(), ms.value

    def profile_kernels(self, reps=5):
        """Mean device ms of (predict, pairwise interaction, correct)."""
        ms = (C.c_double * 3)()
        self._call("profile_kernels", self._ctx, int(reps), ms)
        return tuple(ms)

    def launch_count(self):
        n = C.c_int64()
        self._call("launch_count", self._ctx, C.byref(n))
        return n.value
