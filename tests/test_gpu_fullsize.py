"""GPU: the benchmark's 3D N = 10^6 foam at full size, checked through
properties that do not depend on an oracle run of that size:

  * the pair list: rows grouped by i ascending, j > i ascending inside a
    row, no duplicates, every pair within r_i + r_j + skin in the exact FP64
    minimum-image distance (comparePair, src/kernels.cu:619-623), and no
    pair missing for a random sample of bubbles (brute force over all N);
  * the pair forces are antisymmetric: without flow or walls the overlap
    velocities of one attempt sum to zero over the foam (relative to the sum
    of their magnitudes, 1e-12 in FP64);
  * a second search of an unchanged state reproduces the list (idempotence);
  * the mixed form matches the FP64 form within its stated bars at full
    size (one attempt 1e-6 per row, 20 steps: same counts, volume 1e-10);
  * the FP64 form with float-float pair terms matches the plain FP64 form
    within the FP64 bar (one attempt 1e-12 per row, 20 steps: same counts,
    volume 1e-12).
"""
import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads

pytestmark = pytest.mark.gpu

N = 1_000_000


@pytest.fixture(scope="module")
def c2():
    cfg, st = workloads.config_c2(n=N)
    return cfg, st


def min_image(d, L):
    return d - L * np.round(d / L)


def test_pair_list_properties(c2):
    cfg, st = c2
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    g.search_neighbors()
    s = g.get_state()
    i, j = g.pairs()
    assert len(i) > 3 * N
    assert np.all(i < j)
    assert np.all(np.diff(i) >= 0)
    same = i[1:] == i[:-1]
    assert np.all(j[1:][same] > j[:-1][same])  # j ascending and unique in a row
    L = np.array([cfg.tfr[a] - cfg.lbb[a] for a in range(3)])
    x, y, z, r = s["x"], s["y"], s["z"], s["r"]
    dx = min_image(x[i] - x[j], L[0])
    dy = min_image(y[i] - y[j], L[1])
    dz = min_image(z[i] - z[j], L[2])
    d2 = dx * dx + dy * dy + dz * dz
    cut = r[i] + r[j] + cfg.skin_radius
    assert np.all(d2 < cut * cut)
    # completeness for sampled rows: every partner within the cutoff is listed
    rng = np.random.default_rng(5)
    for b in rng.choice(N, size=60, replace=False):
        ex = min_image(x - x[b], L[0])
        ey = min_image(y - y[b], L[1])
        ez = min_image(z - z[b], L[2])
        c = r + r[b] + cfg.skin_radius
        near = np.nonzero(ex * ex + ey * ey + ez * ez < c * c)[0]
        near = set(near.tolist()) - {int(b)}
        listed = set(j[i == b].tolist()) | set(i[j == b].tolist())
        assert listed == near, b
    # idempotence: a second search of the unchanged (now cell-ordered) state
    g.search_neighbors()
    i2, j2 = g.pairs()
    s2 = g.get_state()
    assert len(i2) == len(i)
    a = np.stack([s["index"][i], s["index"][j]], 1)
    b2 = np.stack([s2["index"][i2], s2["index"][j2]], 1)
    key = lambda m: np.sort(np.minimum(m[:, 0], m[:, 1]).astype(np.int64) * N  # noqa: E731
                            + np.maximum(m[:, 0], m[:, 1]))
    assert np.array_equal(key(a), key(b2))
    g.close()


def test_pair_forces_balance(c2):
    cfg, st = c2
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    g.search_neighbors()
    g.set_options(0, 0, 0)  # overlap velocities only
    a = g.attempt()
    for k in ("dxdtp", "dydtp", "dzdtp"):
        v = a[k]
        assert abs(v.sum()) <= 1e-12 * np.abs(v).sum(), k
    g.close()


def test_mixed_matches_fp64_at_full_size(c2):
    cfg, st = c2
    a = cb.GpuFoam(cfg)
    a.load_state(st)
    workloads.prepare(a)
    a.integrate(3)
    s0 = a.get_state()
    i, j = a.pairs()
    cfg_m, _ = workloads.config_c2(n=N, precision=1)
    b = cb.GpuFoam(cfg_m)
    b.load_state(s0)
    b.set_pairs(i, j)
    b.set_time(a.report()["time_step"])
    aa, ab = a.attempt(), b.attempt()
    for k, base in (("xp", "x"), ("yp", "y"), ("zp", "z")):
        d = ab[k] - aa[k]
        m = aa[k] - s0[base]
        assert np.max(np.abs(d)) <= 1e-6 * np.max(np.abs(m)), k
    for k in ("dxdtp", "dydtp", "dzdtp", "drdtp"):
        assert np.max(np.abs(ab[k] - aa[k])) <= 1e-6 * np.max(np.abs(aa[k])), k
    v0 = a.total_volume()
    qa, qb = a.report(), b.report()
    ra, rb = a.integrate(20), b.integrate(20)
    for k in ("steps", "searches", "deleted"):
        assert ra[k] - qa[k] == rb[k] - qb[k], k
    assert ra["count"] == rb["count"]
    assert b.total_volume() == pytest.approx(a.total_volume(), rel=1e-10)
    assert a.total_volume() == pytest.approx(v0, rel=1e-9)
    a.close()
    b.close()


def test_ff_form_matches_fp64_at_full_size(c2):
    cfg, st = c2
    a = cb.GpuFoam(cfg)
    a.load_state(st)
    workloads.prepare(a)
    a.integrate(3)
    s0 = a.get_state()
    i, j = a.pairs()
    cfg_f, _ = workloads.config_c2(n=N, precision=2)
    b = cb.GpuFoam(cfg_f)
    b.load_state(s0)
    b.set_pairs(i, j)
    b.set_time(a.report()["time_step"])
    aa, ab = a.attempt(), b.attempt()
    for k, base in (("xp", "x"), ("yp", "y"), ("zp", "z")):
        d = ab[k] - aa[k]
        m = aa[k] - s0[base]
        assert np.max(np.abs(d)) <= 1e-12 * np.max(np.abs(m)) + 4 * np.spacing(
            np.max(np.abs(aa[k]))), k
    for k in ("dxdtp", "dydtp", "dzdtp", "drdtp", "overlap"):
        assert np.max(np.abs(ab[k] - aa[k])) <= 1e-12 * np.max(np.abs(aa[k])), k
    for k in ("total_overlap_area", "total_overlap_area_per_radius"):
        assert ab[k] == pytest.approx(aa[k], rel=1e-12), k
    qa, qb = a.report(), b.report()
    ra, rb = a.integrate(20), b.integrate(20)
    for k in ("steps", "attempts", "searches", "deleted"):
        assert ra[k] - qa[k] == rb[k] - qb[k], k
    assert ra["count"] == rb["count"]
    assert b.total_volume() == pytest.approx(a.total_volume(), rel=1e-12)
    a.close()
    b.close()
