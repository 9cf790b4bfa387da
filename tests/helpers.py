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


def assert_rows_close(a, b, rows, rtol, what=""):
    for k in rows:
        e = max_rel(a[k], b[k])
        assert e <= rtol, "%s%s: max |diff| / max |ref| = %.3e > %.1e" % (what, k, e, rtol)


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
