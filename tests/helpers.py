"""Shared test helpers: rows keyed by the persistent bubble index, brute-force
pair sets, tolerant comparisons."""
import numpy as np

from cubble_gb300 import _abi

DROWS = _abi.STATE_D_ROWS
IROWS = _abi.STATE_I_ROWS


def by_index(state):
    """Rows reordered by the persistent `index` (the reference's parity key)."""
    order = np.argsort(state["index"], kind="stable")
    return {k: np.asarray(v)[order] for k, v in state.items()}


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if a.size == 0:
        return 0.0
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


# Rows that are differences of two positions: the predictor-corrector error
# |x_predicted - x_corrected| and the path increments |x_corrected - x|. Their
# FP64 resolution is the ulp of the largest coordinate, so a corrected
# position whose last bit differs (velocities that agree to ~1e-14 but not
# bit for bit) moves them by that much, which can be more than 1e-12 of the
# row's maximum when the errors are small.
POSITION_DIFFERENCES = ("error", "path_new", "path", "max_error")


def position_ulp(state, ulps=4):
    """`ulps` units in the last place of the largest coordinate."""
    m = max(float(np.max(np.abs(state[k]))) for k in ("x", "y", "z")
            if k in state and np.size(state[k]))
    return ulps * float(np.spacing(m))


def assert_rows_close(a, b, rows, rtol, what="", floor=0.0):
    """max |a - b| <= rtol max |b| per row; a row in POSITION_DIFFERENCES may
    also differ by up to `floor` (position_ulp of the state)."""
    for k in rows:
        x = np.asarray(a[k], np.float64)
        y = np.asarray(b[k], np.float64)
        if y.size == 0:
            continue
        diff = float(np.max(np.abs(x - y)))
        scale = max(float(np.max(np.abs(y))), 1e-300)
        allowed = rtol * scale
        if k in POSITION_DIFFERENCES:
            allowed = max(allowed, floor)
        assert diff <= allowed, "%s%s: max |diff| %.3e > %.3e (%.1e of max |ref| %.3e)" % (
            what, k, diff, allowed, rtol, scale)


def pair_set(i, j, index=None):
    i = np.asarray(i, np.int64)
    j = np.asarray(j, np.int64)
    if index is not None:
        i = np.asarray(index)[i]
        j = np.asarray(index)[j]
    lo = np.minimum(i, j)
    hi = np.maximum(i, j)
    return set(zip(lo.tolist(), hi.tolist()))


def wrapped_sq(cfg, x1, y1, z1, x2, y2, z2):
    """wrappedDifference + getSquaredLength (src/kernels.cu:1094-1114,
    src/vec.h:41-49) with numpy, operation by operation."""
    dim = cfg.dimensionality
    iv = [cfg.tfr[a] - cfg.lbb[a] for a in range(3)]
    ds = []
    for a, (p, q) in enumerate(((x1, x2), (y1, y2), (z1, z2))):
        d1 = p - q if (a < 2 or dim == 3) else np.zeros_like(p - q)
        t = iv[a] - np.abs(d1)
        d = d1
        if not cfg.wall[a] and (a < 2 or dim == 3):
            flip = t * t < d1 * d1
            d = np.where(flip, t * np.where(d1 < 0, 1.0, -1.0), d1)
        ds.append(d)
    s = 0.0 + ds[0] * ds[0]
    s = s + ds[1] * ds[1]
    s = s + ds[2] * ds[2]
    return s


def brute_pairs(cfg, state):
    """All pairs (by row) within r_i + r_j + skin, O(N^2)."""
    x, y, z, r = (np.asarray(state[k], np.float64) for k in ("x", "y", "z", "r"))
    n = len(x)
    out = set()
    for i in range(n - 1):
        j = np.arange(i + 1, n)
        sq = wrapped_sq(cfg, x[i], y[i], z[i], x[j], y[j], z[j])
        maxd = r[i] + r[j] + cfg.skin_radius
        hit = j[sq < maxd * maxd]
        out.update((i, int(k)) for k in hit)
    return out
