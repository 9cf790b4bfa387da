"""Python host mirror of the reference's step-loop interface.

`Foam` wraps one context of a library that exports the C ABI of
include/cubble_gb300.h. Its methods carry the reference's names and meaning:

    integrate(n)        -> integrate() x n        src/simulator.cu:251-337
    attempt()           -> step() without accept  src/simulator.cu:192-249
    search_neighbors()  -> searchNeighbors()      src/simulator.cu:60-178
    bootstrap()         -> init()'s Euler start   src/simulator.cu:727-787
    energy()            -> totalEnergy()          src/simulator.cu:39-58
    total_volume()      -> totalVolume()          src/simulator.cu:362-379

Errors follow the reference's throwing wrappers (`CUDA_ASSERT`,
src/util.cuh:104-111): a non-zero status raises `CubbleError` with the
library's last error message.
"""
import ctypes as C

import numpy as np

from . import _abi

DROWS = _abi.STATE_D_ROWS
IROWS = _abi.STATE_I_ROWS


class CubbleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%s): %s" % (
            _abi.STATUS_NAMES.get(code, "error"), code, msg))
        self.code = code


def _dptr(a):
    return a.ctypes.data_as(_abi.PD) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(_abi.PI) if a is not None else None


def make_config(**kw):
    """Builds a cb_config from keyword arguments (names of the C fields)."""
    cfg = _abi.Config()
    cfg.dimensionality = 3
    cfg.time_step = 1e-4
    cfg.error_tolerance = 1e-5
    cfg.f0_per_mu0 = 1.0
    cfg.skin_radius = 0.3
    cfg.use_gas_exchange = 1
    cfg.increment_path = 1
    for k, v in kw.items():
        if k in ("wall",):
            cfg.wall = _abi.I3(*[int(t) for t in v])
        elif k in ("lbb", "tfr", "flow_lbb", "flow_tfr", "flow_vel"):
            setattr(cfg, k, _abi.D3(*[float(t) for t in v]))
        else:
            setattr(cfg, k, v)
    return cfg


class Foam:
    """One foam (context) of a C-ABI library with symbol prefix `prefix`."""

    def __init__(self, lib, prefix, config):
        self._lib = lib
        self._p = prefix
        self.config = config
        self._ctx = C.c_void_p()
        self._call("create", C.byref(config), C.byref(self._ctx))

    # ------------------------------------------------------------ plumbing
    def _fn(self, name):
        return getattr(self._lib, self._p + name)

    def _call(self, name, *args):
        rc = self._fn(name)(*args)
        if rc != 0:
            msg = self._fn("last_error")()
            raise CubbleError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if self._ctx:
            self._fn("destroy")(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # --------------------------------------------------------------- state
    def load_state(self, state):
        """state: dict of numpy rows (float64 for DROWS, int32 for IROWS);
        missing rows are zero (saved_* default to positions, index to 0..n-1)."""
        n = len(state["x"])
        keep = {}
        v = _abi.StateView()
        v.count = n
        for k in DROWS:
            if k in state and state[k] is not None:
                a = np.ascontiguousarray(state[k], dtype=np.float64)
                assert a.shape == (n,), k
                keep[k] = a
                setattr(v, k, _dptr(a))
        for k in IROWS:
            if k in state and state[k] is not None:
                a = np.ascontiguousarray(state[k], dtype=np.int32)
                assert a.shape == (n,), k
                keep[k] = a
                setattr(v, k, _iptr(a))
        self._call("load_state", self._ctx, C.byref(v))

    def count(self):
        return self.report()["count"]

    def get_state(self, rows=None, out=None):
        """The persistent rows (all, or `rows`) as numpy arrays; `out` may
        give the destination arrays (e.g. pinned host buffers, each holding at
        least count() elements of the row's type)."""
        n = self.count()
        res = {}
        v = _abi.StateView()
        for k in DROWS:
            if rows is None or k in rows:
                if out is not None and k in out:
                    res[k] = out[k][:n]
                    assert res[k].dtype == np.float64 and res[k].flags.c_contiguous, k
                else:
                    res[k] = np.zeros(n, np.float64)
                setattr(v, k, _dptr(res[k]))
        for k in IROWS:
            if rows is None or k in rows:
                if out is not None and k in out:
                    res[k] = out[k][:n]
                    assert res[k].dtype == np.int32 and res[k].flags.c_contiguous, k
                else:
                    res[k] = np.zeros(n, np.int32)
                setattr(v, k, _iptr(res[k]))
        self._call("get_state", self._ctx, C.byref(v))
        return res

    def set_options(self, use_gas_exchange, use_flow, increment_path):
        self._call("set_options", self._ctx, int(use_gas_exchange),
                   int(use_flow), int(increment_path))

    def set_time(self, time_step, time_integer=0, time_fraction=0.0):
        self._call("set_time", self._ctx, float(time_step), int(time_integer),
                   float(time_fraction))

    def set_box(self, lbb, tfr, bubble_volume_multiplier, flow_lbb=None,
                flow_tfr=None):
        fl = flow_lbb if flow_lbb is not None else self.config.flow_lbb
        ft = flow_tfr if flow_tfr is not None else self.config.flow_tfr
        self._call("set_box", self._ctx, _abi.D3(*lbb), _abi.D3(*tfr),
                   float(bubble_volume_multiplier), _abi.D3(*fl), _abi.D3(*ft))

    # ---------------------------------------------------------- operations
    def bootstrap(self):
        self._call("bootstrap", self._ctx)

    def search_neighbors(self):
        self._call("search_neighbors", self._ctx)

    def pairs(self):
        cnt = C.c_int32()
        self._call("get_pairs", self._ctx, None, None, 0, C.byref(cnt))
        i = np.zeros(cnt.value, np.int32)
        j = np.zeros(cnt.value, np.int32)
        self._call("get_pairs", self._ctx, _iptr(i), _iptr(j), cnt.value,
                   C.byref(cnt))
        return i, j

    def set_pairs(self, i, j):
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        self._call("set_pairs", self._ctx, _iptr(i), _iptr(j), len(i))

    def attempt(self):
        n = self.count()
        v = _abi.AttemptView()
        out = {}
        for k in _abi.ATTEMPT_D_ROWS:
            out[k] = np.zeros(n, np.float64)
            setattr(v, k, _dptr(out[k]))
        out["delete_flags"] = np.zeros(n, np.int32)
        v.delete_flags = _iptr(out["delete_flags"])
        self._call("attempt", self._ctx, C.byref(v))
        for k in _abi.ATTEMPT_SCALARS + ["num_to_be_deleted"]:
            out[k] = getattr(v, k)
        return out

    def integrate(self, n_steps=1):
        r = _abi.Report()
        self._call("integrate", self._ctx, int(n_steps), C.byref(r))
        return r.as_dict()

    def report(self):
        r = _abi.Report()
        self._call("get_report", self._ctx, C.byref(r))
        return r.as_dict()

    def energy(self):
        e = C.c_double()
        self._call("energy", self._ctx, C.byref(e))
        return e.value

    def bubble_energies(self):
        n = self.count()
        e = np.zeros(n, np.float64)
        self._call("bubble_energies", self._ctx, _dptr(e), n)
        return e

    def total_volume(self):
        v = C.c_double()
        self._call("total_volume", self._ctx, C.byref(v))
        return v.value
