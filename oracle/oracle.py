"""TEST INFRASTRUCTURE: ctypes binding of the CPU FP64 oracle.

The oracle exports the C ABI of include/cubble_gb300.h with the prefix
`cbo_`, so it is driven through the same `Foam` class as the CUDA library.
"""
import ctypes as C
import os
import subprocess

from cubble_gb300 import _abi
from cubble_gb300.foam import Foam

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libcubble_oracle.so")
_lib = None


def build(force=False):
    """Compiles the oracle with the recipe in oracle/Makefile."""
    if force or not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        _abi.declare(_lib, "cbo_")
    return _lib


class OracleFoam(Foam):
    def __init__(self, config, threads=1):
        super().__init__(lib(), "cbo_", config)
        if threads != 1:
            self._call("set_threads", self._ctx, int(threads))

    def cell_dims(self):
        d = _abi.I3()
        self._call("cell_dims", self._ctx, d)
        return tuple(d)
