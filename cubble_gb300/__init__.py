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

    def profile_search(self, reps=3):
        """Mean device ms of one neighbour search of the current state."""
        ms = C.c_double()
        self._call("profile_search", self._ctx, int(reps), C.byref(ms))
        return ms.value

    def launch_count(self):
        n = C.c_int64()
        self._call("launch_count", self._ctx, C.byref(n))
        return n.value

    def set_tuning(self, cell_scale=1.0, pair_run=4, pair_blocks=0, step_blocks=0):
        t = _abi.Tuning(float(cell_scale), int(pair_run), int(pair_blocks), int(step_blocks), 0)
        self._call("set_tuning", self._ctx, C.byref(t))

    def tuning(self):
        t = _abi.Tuning()
        self._call("get_tuning", self._ctx, C.byref(t))
        return t.as_dict()

    def autotune(self, reps=3):
        """Times the knobs of cb_tuning on the current (searched) state, keeps
        the fastest (also for later contexts of the same kind), returns them."""
        t = _abi.Tuning()
        self._call("autotune", self._ctx, int(reps), C.byref(t))
        return t.as_dict()

    def integrate_until(self, max_steps, time=None, min_count=-1, max_radius=float("inf")):
        """Up to max_steps accepted steps, ending after the first one that
        reaches `time` (the simulation clock), leaves <= min_count bubbles
        or makes the largest radius >= max_radius."""
        st = _abi.Stop()
        t = float("inf") if time is None else float(time)
        if t == float("inf"):
            st.time_integer, st.time_fraction = (1 << 63), 0.0
        else:
            st.time_integer = int(t)
            st.time_fraction = t - int(t)
        st.min_count = int(min_count)
        st.max_radius = float(max_radius)
        r = _abi.Report()
        self._call("integrate_until", self._ctx, int(max_steps), C.byref(st), C.byref(r))
        return r.as_dict()

    def transform_positions(self, normalize):
        self._call("transform_positions", self._ctx, 1 if normalize else 0)

    def averages(self):
        """Means of r, dxdt, dydt, dzdt, drdt, path."""
        out = (C.c_double * 6)()
        self._call("averages", self._ctx, out)
        return tuple(out)

    def reset_rows(self, which):
        self._call("reset_rows", self._ctx, int(which))

    def set_average_area(self, area):
        self._call("set_average_area", self._ctx, float(area))

    def assign_lattice(self, bubbles_per_dim, avg_rad, ux, uy, uz, uw, nr):
        """init()'s lattice placement from the generator's draws; returns
        (average initial area, largest radius)."""
        import numpy as np
        n = len(ux)
        rows = [np.ascontiguousarray(a, dtype=np.float64) for a in (ux, uy, uz, uw, nr)]
        bpd = _abi.I3(*[int(v) for v in bubbles_per_dim])
        area, mr = C.c_double(), C.c_double()
        ptr = [r.ctypes.data_as(_abi.PD) for r in rows]
        self._call("assign_lattice", self._ctx, bpd, float(avg_rad), *ptr, int(n),
                   C.byref(area), C.byref(mr))
        return area.value, mr.value


class _BatchFoam(GpuFoam):
    """A foam owned by a GpuFoamBatch (its context lives as long as the batch)."""

    def __init__(self, batch, index, config):
        self._lib = batch._lib
        self._p = "cb_"
        self.config = config
        self._batch = batch  # keeps the batch alive
        self._ctx = C.c_void_p()
        batch._call("batch_context", batch._b, int(index), C.byref(self._ctx))

    def close(self):
        self._ctx = C.c_void_p()


class GpuFoamBatch:
    """Independent foams advanced together, one launch per stage for all of
    them (a `cb_batch`). `foams[f]` is foam f's single-foam interface (load
    its state, search, bootstrap, read it back); `integrate(n)` advances
    every foam by n accepted steps."""

    def __init__(self, configs):
        self._lib = lib()
        self._b = C.c_void_p()
        arr = (_abi.Config * len(configs))(*configs)
        self._call("batch_create", arr, len(configs), C.byref(self._b))
        self.foams = [_BatchFoam(self, f, cfg) for f, cfg in enumerate(configs)]

    def _call(self, name, *args):
        rc = getattr(self._lib, "cb_" + name)(*args)
        if rc != 0:
            msg = self._lib.cb_last_error()
            raise CubbleError(rc, msg.decode() if msg else "")
        return rc

    def __len__(self):
        return len(self.foams)

    def integrate(self, n_steps=1):
        reps = (_abi.Report * len(self.foams))()
        self._call("batch_integrate", self._b, int(n_steps), reps)
        return [r.as_dict() for r in reps]

    def integrate_timed(self, n_steps):
        reps = (_abi.Report * len(self.foams))()
        ms = C.c_double()
        self._call("batch_integrate_timed", self._b, int(n_steps), reps, C.byref(ms))
        return [r.as_dict() for r in reps], ms.value

    def set_tile(self, bubbles_per_block):
        self._call("batch_set_tile", self._b, int(bubbles_per_block))

    def autotune(self, steps_per_trial):
        """Tile, cell scale and (mixed form) pairs per thread, each timed over
        `steps_per_trial` steps that advance the foams; returns the tile (the
        other knobs: foams[0].tuning())."""
        t = C.c_int32()
        self._call("batch_autotune", self._b, int(steps_per_trial), C.byref(t))
        return t.value

    def set_tuning(self, cell_scale=1.0, pair_run=4, pair_blocks=0, step_blocks=0):
        t = _abi.Tuning(float(cell_scale), int(pair_run), int(pair_blocks), int(step_blocks), 0)
        self._call("batch_set_tuning", self._b, C.byref(t))

    def launch_count(self):
        n = C.c_int64()
        self._call("batch_launch_count", self._b, C.byref(n))
        return n.value

    def close(self):
        if self._b:
            for f in self.foams:
                f.close()
            self._lib.cb_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
