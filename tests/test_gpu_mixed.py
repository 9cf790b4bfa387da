"""GPU: the mixed-precision form against the FP64 oracle on the same inputs.

Errors are norm-wise: max |mixed - fp64| over bubbles divided by the largest
|fp64| of the same row (for positions and radii, of their change in the
step). Bars: 1e-6 per step for positions, velocities and radius rates in 3D
(2e-6 for the 2D radius rate and 4e-6 for 2D overlap lengths, where the
chord of nearly tangent circles is a square root of a small difference);
total gas volume within 1e-10 of the FP64 run; pair sets, deletion sets and
the compaction order bit-exact (they are computed from the FP64 positions).
"""
import math

import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads
from helpers import by_index, max_rel, pair_set

pytestmark = pytest.mark.gpu


def case(dim, n, **kw):
    if dim == 3:
        return workloads.foam(n, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=41, **kw)
    return workloads.foam(n, 2, 0.9, seed=42, min_rad=0.05, **kw)


def prepared(oracle_mod, dim, n, steps=5):
    cfg, st = case(dim, n)
    o = oracle_mod.OracleFoam(cfg)
    o.load_state(st)
    workloads.prepare(o)
    o.integrate(steps)
    return cfg, o


def mixed_from(o, dim, n, **kw):
    cfg_m, _ = case(dim, n, precision=1, **kw)
    g = cb.GpuFoam(cfg_m)
    g.load_state(o.get_state())
    i, j = o.pairs()
    g.set_pairs(i, j)
    g.set_time(o.report()["time_step"])
    return g


def test_mixed_volume_over_200_steps():
    """The benchmark's foam at N = 10^5: the mixed and the FP64 forms run 200
    accepted steps from the same prepared state, with no deletion in between
    to reset the volumes. Each form's total gas volume moves (the AM2 radius
    update conserves it to first order); the mixed form must follow the FP64
    one to 3e-11 — values that enter every bubble's update alike (half step,
    mean-field factor, the radius of the gas-exchange term) rounded toward
    zero instead of to nearest made it ~1e-10 by this step at N = 10^6."""
    cfg, st = workloads.config_c2(n=100_000, use_graph=1)
    a = cb.GpuFoam(cfg)
    a.load_state(st)
    workloads.prepare(a)
    a.integrate(3)
    s0 = a.get_state()
    i, j = a.pairs()
    dt = a.report()["time_step"]
    b = cb.GpuFoam(workloads.sweep_config_as(cfg, precision=1))
    b.load_state(s0)
    b.set_pairs(i, j)
    b.set_time(dt)
    a.set_time(dt)
    ra0, rb0 = a.report(), b.report()
    ra, rb = a.integrate(200), b.integrate(200)
    assert ra["deleted"] == ra0["deleted"] and rb["deleted"] == rb0["deleted"]
    assert b.total_volume() == pytest.approx(a.total_volume(), rel=3e-11)
    a.close()
    b.close()


def test_mixed_large_radii(oracle_mod):
    """Radii of 6-12 length units: most overlapping pairs have r1 + r2 above
    16, where the overlap product (r1 + r2)^2 - d^2 is no longer formed from
    exact integers and the FP32 expression is used; one attempt against the
    oracle at the same bars as the unit-radius foams."""
    cfg, st = workloads.foam(3000, 3, 0.8, rmean=9.0, rstd=1.0, rclip=(6.0, 12.0), seed=43)
    o = oracle_mod.OracleFoam(cfg)
    o.load_state(st)
    workloads.prepare(o)
    o.integrate(5)
    s = o.get_state()
    cfg_m, _ = workloads.foam(3000, 3, 0.8, rmean=9.0, rstd=1.0, rclip=(6.0, 12.0), seed=43,
                              precision=1)
    g = cb.GpuFoam(cfg_m)
    g.load_state(s)
    i, j = o.pairs()
    g.set_pairs(i, j)
    g.set_time(o.report()["time_step"])
    ag, ao = g.attempt(), o.attempt()
    lim = 1e-6
    for k, base in (("xp", "x"), ("yp", "y"), ("zp", "z"), ("rp", "r")):
        assert max_rel(ag[k] - s[base], ao[k] - s[base]) <= lim, k
    for k in ("dxdtp", "dydtp", "dzdtp", "drdtp", "overlap", "path_new"):
        assert max_rel(ag[k], ao[k]) <= lim, k
    for k in ("total_area", "total_area_per_radius", "total_overlap_area",
              "total_overlap_area_per_radius"):
        assert ag[k] == pytest.approx(ao[k], rel=lim), k
    g.close()
    o.close()


@pytest.mark.parametrize("dim", [3, 2])
def test_mixed_single_attempt(oracle_mod, dim):
    cfg, o = prepared(oracle_mod, dim, 8000)
    s = o.get_state()
    g = mixed_from(o, dim, 8000)
    ag, ao = g.attempt(), o.attempt()
    lim = 1e-6
    for k, base in (("xp", "x"), ("yp", "y"), ("zp", "z"), ("rp", "r")):
        if dim == 2 and k == "zp":
            continue
        assert max_rel(ag[k] - s[base], ao[k] - s[base]) <= lim, k
    for k in ("dxdtp", "dydtp", "dzdtp"):
        if dim == 2 and k == "dzdtp":
            continue
        assert max_rel(ag[k], ao[k]) <= lim, k
    assert max_rel(ag["drdtp"], ao["drdtp"]) <= (lim if dim == 3 else 2e-6)
    assert max_rel(ag["overlap"], ao["overlap"]) <= (lim if dim == 3 else 4e-6)
    assert max_rel(ag["path_new"], ao["path_new"]) <= lim
    for k in ("total_area", "total_area_per_radius", "total_overlap_area",
              "total_overlap_area_per_radius"):
        assert ag[k] == pytest.approx(ao[k], rel=lim), k
    assert np.array_equal(ag["delete_flags"], ao["delete_flags"])


@pytest.mark.parametrize("graph", [0, 1])
@pytest.mark.parametrize("dim", [3, 2])
def test_mixed_trajectory(oracle_mod, dim, graph):
    cfg, o = prepared(oracle_mod, dim, 8000)
    s0 = by_index(o.get_state())
    g = mixed_from(o, dim, 8000, use_graph=graph)
    rg0, ro0 = g.report(), o.report()
    rg, ro = g.integrate(60), o.integrate(60)
    for k in ("steps", "attempts", "searches", "deleted"):
        assert rg[k] - rg0[k] == ro[k] - ro0[k], k
    for k in ("count", "num_pairs"):
        assert rg[k] == ro[k], k
    sg, so = by_index(g.get_state()), by_index(o.get_state())
    for a, k in enumerate(("x", "y", "z")):
        if dim == 2 and k == "z":
            continue
        L = cfg.tfr[a] - cfg.lbb[a]
        wrap = lambda d: d - L * np.round(d / L)  # noqa: E731  (searches wrap positions)
        err = np.max(np.abs(wrap(sg[k] - so[k]))) / np.max(np.abs(wrap(so[k] - s0[k])))
        assert err <= 1e-6, (k, err)
    assert max_rel(sg["r"], so["r"]) <= 1e-8
    assert g.total_volume() == pytest.approx(o.total_volume(), rel=1e-10)
    assert g.energy() == pytest.approx(o.energy(), rel=1e-6)
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    assert pair_set(gi, gj, g.get_state()["index"]) == pair_set(oi, oj, o.get_state()["index"])


@pytest.mark.parametrize("dim", [3, 2])
def test_mixed_deletion_and_volume_fix(oracle_mod, dim):
    kw = dict(rstd=0.3, rclip=(0.01, 2.0), seed=43, min_rad=0.2)
    cfg, st = workloads.foam(4000, dim, 0.85, **kw)
    cfg_m, _ = workloads.foam(4000, dim, 0.85, precision=1, **kw)
    o = oracle_mod.OracleFoam(cfg)
    g = cb.GpuFoam(cfg_m)
    for f in (o, g):
        f.load_state(st)
        workloads.prepare(f)
    ro, rg = o.integrate(1), g.integrate(1)
    assert ro["deleted"] > 0
    for k in ("deleted", "count", "num_pairs"):
        assert rg[k] == ro[k], k
    sg, so = g.get_state(), o.get_state()
    assert np.array_equal(sg["index"], so["index"])
    M = cfg.bubble_volume_multiplier
    target = math.pi * M ** 2 if dim == 2 else 4.0 / 3.0 * math.pi * M ** 3
    assert g.total_volume() == pytest.approx(target, rel=1e-12)


def test_mixed_search_is_exact(oracle_mod):
    cfg, st = case(3, 6000)
    cfg_m, _ = case(3, 6000, precision=1)
    o = oracle_mod.OracleFoam(cfg)
    g = cb.GpuFoam(cfg_m)
    for f in (o, g):
        f.load_state(st)
        f.search_neighbors()
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    assert np.array_equal(gi, oi) and np.array_equal(gj, oj)
    sg, so = g.get_state(), o.get_state()
    for k in ("x", "y", "z", "r", "saved_x"):
        assert np.array_equal(sg[k], so[k]), k
    assert np.array_equal(sg["index"], so["index"])


@pytest.mark.parametrize("dim", [3, 2])
def test_mixed_containment_threshold(oracle_mod, dim):
    """A pair on the threshold where the overlap area jumps (one centre just
    inside the other bubble, src/kernels.cu:240-249): the centres are
    1 - 2^-30 apart and the larger radius is 1, so FP64 takes the containment
    branch while the FP32 distance rounds to exactly 1 (the lens branch, an
    area 6 % smaller in 3D). The mixed form decides such pairs again in FP64
    and matches the oracle."""
    d = 1.0 - 2.0 ** -30
    L = 40.0
    x = np.array([10.0, 10.0 + d, 25.0])
    y = np.array([10.0, 10.0, 25.0])
    z = np.array([10.0, 10.0, 25.0]) if dim == 3 else np.zeros(3)
    r = np.array([1.0, 0.5, 0.8])
    st = {"x": x, "y": y, "z": z, "r": r, "index": np.arange(3, dtype=np.int32)}
    kw = dict(dimensionality=dim, lbb=(0.0, 0.0, 0.0), tfr=(L, L, L if dim == 3 else 0.0),
              min_rad=0.1, f0_per_mu0=1.0, k_parameter=0.1, kappa=0.01, skin_radius=0.3,
              bubble_volume_multiplier=1.0, average_surface_area_in=4.0,
              error_tolerance=1e-5, time_step=1e-6, capacity=3)
    o = oracle_mod.OracleFoam(cb.make_config(**kw))
    g = cb.GpuFoam(cb.make_config(precision=1, **kw))
    for f in (o, g):
        f.load_state(st)
        f.search_neighbors()
    assert len(o.pairs()[0]) == 1
    ag, ao = g.attempt(), o.attempt()
    sg, so = g.get_state(), o.get_state()
    og, oo = np.argsort(sg["index"]), np.argsort(so["index"])
    # the containment branch: pi min(r)^2 (3D), 2 min(r) (2D)
    expect = 0.25 * 3.1415926535897932 if dim == 3 else 1.0
    assert ao["overlap"][oo][0] == pytest.approx(expect, rel=1e-12)
    for k in ("overlap", "drdtp", "dxdtp"):
        assert max_rel(ag[k][og], ao[k][oo]) <= 1e-6, k
    assert ag["total_overlap_area"] == pytest.approx(ao["total_overlap_area"], rel=1e-6)
