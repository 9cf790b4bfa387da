"""ctypes mirror of include/cubble_gb300.h (structures and prototypes).

The same structures describe the CUDA library's entry points (prefix `cb_`)
and, in the test harness, the CPU oracle's (prefix `cbo_`), so both can be
driven through one Python binding.
"""
import ctypes as C

D3 = C.c_double * 3
I3 = C.c_int32 * 3
PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int32)

CB_OK = 0
CB_ERR_INVALID_ARGUMENT = 1
CB_ERR_CUDA = 2
CB_ERR_CAPACITY = 3
CB_ERR_MAX_ATTEMPTS = 4
CB_ERR_NONFINITE = 5
CB_ERR_DT_UNDERFLOW = 6
CB_ERR_NO_DEVICE = 7
CB_ERR_STATE = 8

CB_PRECISION_FP64 = 0
CB_PRECISION_MIXED = 1
CB_PRECISION_FP64_FF = 2

STATUS_NAMES = {
    0: "ok", 1: "invalid argument", 2: "cuda error", 3: "capacity exceeded",
    4: "max attempts", 5: "non-finite", 6: "dt underflow", 7: "no device",
    8: "state",
}


class Config(C.Structure):
    _fields_ = [
        ("dimensionality", C.c_int32),
        ("wall", I3),
        ("use_gas_exchange", C.c_int32),
        ("use_flow", C.c_int32),
        ("increment_path", C.c_int32),
        ("capacity", C.c_int32),
        ("pair_capacity", C.c_int32),
        ("max_attempts", C.c_int32),
        ("precision", C.c_int32),
        ("use_graph", C.c_int32),
        ("lbb", D3),
        ("tfr", D3),
        ("flow_lbb", D3),
        ("flow_tfr", D3),
        ("flow_vel", D3),
        ("wall_drag", C.c_double),
        ("min_rad", C.c_double),
        ("f0_per_mu0", C.c_double),
        ("k_parameter", C.c_double),
        ("kappa", C.c_double),
        ("skin_radius", C.c_double),
        ("bubble_volume_multiplier", C.c_double),
        ("average_surface_area_in", C.c_double),
        ("error_tolerance", C.c_double),
        ("time_step", C.c_double),
        ("shear_speed", C.c_double),
    ]


STATE_D_ROWS = ["x", "y", "z", "r", "dxdt", "dydt", "dzdt", "drdt",
                "dxdto", "dydto", "dzdto", "drdto", "path", "error",
                "saved_x", "saved_y", "saved_z", "saved_r"]
STATE_I_ROWS = ["wrap_count_x", "wrap_count_y", "wrap_count_z", "index",
                "num_neighbors"]


class StateView(C.Structure):
    _fields_ = ([("count", C.c_int32), ("pad_", C.c_int32)]
                + [(n, PD) for n in STATE_D_ROWS]
                + [(n, PI) for n in STATE_I_ROWS])


class Report(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("attempts", C.c_int64),
        ("searches", C.c_int64),
        ("deleted", C.c_int64),
        ("bubble_steps", C.c_int64),
        ("time_integer", C.c_uint64),
        ("time_fraction", C.c_double),
        ("time_step", C.c_double),
        ("max_error", C.c_double),
        ("max_radius", C.c_double),
        ("max_expansion", C.c_double),
        ("count", C.c_int32),
        ("num_pairs", C.c_int32),
        ("status", C.c_int32),
        ("pad_", C.c_int32),
        ("dt_min", C.c_double),
        ("dt_max", C.c_double),
        ("dt_sum", C.c_double),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad_"}


ATTEMPT_D_ROWS = ["xp", "yp", "zp", "rp", "dxdtp", "dydtp", "dzdtp", "drdtp",
                  "error", "path_new", "overlap"]
ATTEMPT_SCALARS = ["total_area", "total_area_per_radius", "total_overlap_area",
                   "total_overlap_area_per_radius", "total_volume_new",
                   "max_error", "max_radius", "max_expansion"]


class Stop(C.Structure):
    _fields_ = [("time_integer", C.c_uint64), ("time_fraction", C.c_double),
                ("max_radius", C.c_double), ("min_count", C.c_int32), ("pad_", C.c_int32)]


class AttemptView(C.Structure):
    _fields_ = ([(n, PD) for n in ATTEMPT_D_ROWS]
                + [("delete_flags", PI)]
                + [(n, C.c_double) for n in ATTEMPT_SCALARS]
                + [("num_to_be_deleted", C.c_int32), ("pad_", C.c_int32)])


class Tuning(C.Structure):
    """cb_tuning: launch and search knobs of a context."""
    _fields_ = [("cell_scale", C.c_double), ("pair_run", C.c_int32),
                ("pair_blocks", C.c_int32), ("step_blocks", C.c_int32), ("pad_", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


def declare(lib, prefix):
    """Declares the prototypes of include/cubble_gb300.h on `lib` for the
    given symbol prefix ("cb_" for the CUDA library)."""
    vp = C.c_void_p
    sig = {
        "last_error": (C.c_char_p, []),
        "create": (C.c_int, [C.POINTER(Config), C.POINTER(vp)]),
        "destroy": (C.c_int, [vp]),
        "load_state": (C.c_int, [vp, C.POINTER(StateView)]),
        "get_state": (C.c_int, [vp, C.POINTER(StateView)]),
        "set_options": (C.c_int, [vp, C.c_int32, C.c_int32, C.c_int32]),
        "set_time": (C.c_int, [vp, C.c_double, C.c_uint64, C.c_double]),
        "set_box": (C.c_int, [vp, D3, D3, C.c_double, D3, D3]),
        "bootstrap": (C.c_int, [vp]),
        "search_neighbors": (C.c_int, [vp]),
        "get_pairs": (C.c_int, [vp, PI, PI, C.c_int32, C.POINTER(C.c_int32)]),
        "set_pairs": (C.c_int, [vp, PI, PI, C.c_int32]),
        "attempt": (C.c_int, [vp, C.POINTER(AttemptView)]),
        "integrate": (C.c_int, [vp, C.c_int64, C.POINTER(Report)]),
        "get_report": (C.c_int, [vp, C.POINTER(Report)]),
        "energy": (C.c_int, [vp, C.POINTER(C.c_double)]),
        "bubble_energies": (C.c_int, [vp, PD, C.c_int32]),
        "total_volume": (C.c_int, [vp, C.POINTER(C.c_double)]),
    }
    extra = {
        "cb_": {
            "integrate_timed": (C.c_int, [vp, C.c_int64, C.POINTER(Report),
                                          C.POINTER(C.c_double)]),
            "launch_count": (C.c_int, [vp, C.POINTER(C.c_int64)]),
            "profile_kernels": (C.c_int, [vp, C.c_int32, C.POINTER(C.c_double)]),
            "profile_search": (C.c_int, [vp, C.c_int32, C.POINTER(C.c_double)]),
            "set_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
            "get_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
            "autotune": (C.c_int, [vp, C.c_int32, C.POINTER(Tuning)]),
            "forget_tuning": (C.c_int, []),
            "batch_set_tuning": (C.c_int, [vp, C.POINTER(Tuning)]),
            "energy_noalloc": (C.c_int, [C.POINTER(Config), vp, vp, vp, vp, vp, vp,
                                         C.c_int32, C.c_int32, vp, vp]),
            "integrate_until": (C.c_int, [vp, C.c_int64, C.POINTER(Stop), C.POINTER(Report)]),
            "transform_positions": (C.c_int, [vp, C.c_int32]),
            "averages": (C.c_int, [vp, C.POINTER(C.c_double)]),
            "reset_rows": (C.c_int, [vp, C.c_int32]),
            "set_average_area": (C.c_int, [vp, C.c_double]),
            "assign_lattice": (C.c_int, [vp, I3, C.c_double, PD, PD, PD, PD, PD, C.c_int32,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "batch_create": (C.c_int, [C.POINTER(Config), C.c_int32, C.POINTER(vp)]),
            "batch_destroy": (C.c_int, [vp]),
            "batch_context": (C.c_int, [vp, C.c_int32, C.POINTER(vp)]),
            "batch_integrate": (C.c_int, [vp, C.c_int64, C.POINTER(Report)]),
            "batch_integrate_timed": (C.c_int, [vp, C.c_int64, C.POINTER(Report),
                                                C.POINTER(C.c_double)]),
            "batch_set_tile": (C.c_int, [vp, C.c_int32]),
            "batch_autotune": (C.c_int, [vp, C.c_int32, C.POINTER(C.c_int32)]),
            "batch_launch_count": (C.c_int, [vp, C.POINTER(C.c_int64)]),
        },
        "cbo_": {
            "set_threads": (C.c_int, [vp, C.c_int32]),
            "cell_dims": (C.c_int, [vp, I3]),
        },
    }
    sig.update(extra.get(prefix, {}))
    for name, (res, args) in sig.items():
        f = getattr(lib, prefix + name)
        f.restype = res
        f.argtypes = args
    return sorted(prefix + n for n in sig)
