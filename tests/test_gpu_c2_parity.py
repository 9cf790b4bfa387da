"""GPU: the benchmark's own workload — 3D periodic foam, N = 10^6, phi 0.80,
r ~ N(1, 0.15) clipped to [0.3, 2.5] — against the FP64 oracle at full size,
through the C ABI, on the same seeded input.

The compared step is the reference's searchNeighbors (src/simulator.cu:60-178,
src/kernels.cu:598-770), step() (src/simulator.cu:192-249: preIntegrate,
pairwiseInteraction, postIntegrate, src/kernels.cu:40-593) and integrate()
(src/simulator.cu:251-337). The oracle runs on all host threads.

Bars:
  * search: every row (cell order, wrapped positions, wrap counts, index,
    neighbour counts) and the pair list bit-exact;
  * bootstrap and one attempt, both FP64 forms: every row within 1e-12 of
    its largest magnitude (position differences also within 4 ulp of the
    largest coordinate), the global sums within 1e-12, deletion flags
    exact;
  * 10 accepted steps: the same attempt, search and deletion counts and
    dt, every state row within 1e-9;
  * 60 accepted steps in lockstep, compared after every step (counts, dt,
    pair count, positions, radii and rates within 1e-9), through at least
    one neighbour search;
  * the mixed form's attempt on the oracle's state: positions (their
    change), velocities, radius rates, overlap areas and path increments
    within 1e-6 of each row's largest magnitude, the global sums within
    1e-6; its error estimate within 1e-6 of the tolerance it is compared
    with (the estimate is a difference of nearly equal FP32 rates, so its
    own relative error is about 2^-24 |v| / |2v - v_old - v_p|).
"""
import os

import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads
from helpers import DROWS, IROWS, assert_rows_close, by_index, max_rel, position_ulp

pytestmark = pytest.mark.gpu

N = 1_000_000
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def c2():
    return workloads.config_c2(n=N, use_graph=1)


def both(oracle_mod, cfg, st, precision=0):
    g = cb.GpuFoam(workloads.sweep_config_as(cfg, precision=precision) if precision else cfg)
    o = oracle_mod.OracleFoam(cfg, threads=THREADS)
    g.load_state(st)
    o.load_state(st)
    return g, o


def test_c2_search_bit_exact(oracle_mod, c2):
    cfg, st = c2
    g, o = both(oracle_mod, cfg, st)
    g.search_neighbors()
    o.search_neighbors()
    sg, so = g.get_state(), o.get_state()
    for k in DROWS:
        assert np.array_equal(sg[k], so[k]), k
    for k in IROWS:
        assert np.array_equal(sg[k], so[k]), k
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    assert len(oi) > 4 * N
    assert np.array_equal(gi, oi) and np.array_equal(gj, oj)
    g.close()
    o.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_c2_bootstrap_and_attempt(oracle_mod, c2, precision):
    cfg, st = c2
    g, o = both(oracle_mod, cfg, st, precision)
    for f in (g, o):
        workloads.prepare(f)
    sg, so = g.get_state(), o.get_state()
    assert_rows_close(sg, so, ["dxdto", "dydto", "dzdto"], 1e-12, "bootstrap ")
    ag, ao = g.attempt(), o.attempt()
    floor = position_ulp(so)
    assert_rows_close(ag, ao, ["xp", "yp", "zp", "rp", "dxdtp", "dydtp", "dzdtp", "drdtp",
                               "error", "path_new", "overlap"], 1e-12, "attempt ", floor=floor)
    for k in ("total_area", "total_area_per_radius", "total_overlap_area",
              "total_overlap_area_per_radius", "total_volume_new", "max_radius",
              "max_expansion"):
        assert ag[k] == pytest.approx(ao[k], rel=1e-12, abs=1e-300), k
    assert ag["max_error"] == pytest.approx(ao["max_error"], rel=1e-12, abs=floor)
    assert np.array_equal(ag["delete_flags"], ao["delete_flags"])
    assert g.report()["time_step"] == o.report()["time_step"]
    g.close()
    o.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_c2_ten_steps(oracle_mod, c2, precision):
    cfg, st = c2
    g, o = both(oracle_mod, cfg, st, precision)
    for f in (g, o):
        workloads.prepare(f)
    rg, ro = g.integrate(10), o.integrate(10)
    for k in ("steps", "attempts", "searches", "deleted", "count", "num_pairs"):
        assert rg[k] == ro[k], k
    assert rg["time_step"] == pytest.approx(ro["time_step"], rel=1e-12)
    sg, so = by_index(g.get_state()), by_index(o.get_state())
    assert np.array_equal(sg["index"], so["index"])
    assert_rows_close(sg, so, ["x", "y", "z", "r", "dxdt", "dydt", "dzdt", "drdt", "path",
                               "dxdto", "error"], 1e-9, "10 steps ")
    assert g.total_volume() == pytest.approx(o.total_volume(), rel=1e-12)
    g.close()
    o.close()


def test_c2_mixed_attempt(oracle_mod, c2):
    cfg, st = c2
    o = oracle_mod.OracleFoam(cfg, threads=THREADS)
    o.load_state(st)
    workloads.prepare(o)
    o.integrate(3)
    s = o.get_state()
    g = cb.GpuFoam(workloads.sweep_config_as(cfg, precision=1))
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
              "total_overlap_area_per_radius", "total_volume_new"):
        assert ag[k] == pytest.approx(ao[k], rel=lim), k
    tol = cfg.error_tolerance
    assert abs(ag["max_error"] - ao["max_error"]) <= lim * tol
    assert np.array_equal(ag["delete_flags"], ao["delete_flags"])
    g.close()
    o.close()


def test_c2_mixed_attempt_relaxed(c2):
    """The mixed form's attempt late in a run, where the relaxing foam's net
    velocities have fallen ~10x below its pair forces: the FP64 form (equal
    to the oracle within 1e-12 per step, the tests above) runs 1500 accepted
    steps, then one attempt of each form from that state. Every row within
    1e-6 of its largest magnitude, as on the fresh foam; the error estimate
    (a difference of nearly equal FP32 rates) within 1e-4 of the tolerance."""
    cfg, st = c2
    a = cb.GpuFoam(cfg)
    a.load_state(st)
    workloads.prepare(a)
    a.integrate(1500)
    s = a.get_state()
    i, j = a.pairs()
    dt = a.report()["time_step"]
    ref = cb.GpuFoam(cfg)
    g = cb.GpuFoam(workloads.sweep_config_as(cfg, precision=1))
    for f in (ref, g):
        f.load_state(s)
        f.set_pairs(i, j)
        f.set_time(dt)
    ag, ar = g.attempt(), ref.attempt()
    lim = 1e-6
    for k, base in (("xp", "x"), ("yp", "y"), ("zp", "z"), ("rp", "r")):
        assert max_rel(ag[k] - s[base], ar[k] - s[base]) <= lim, k
    for k in ("dxdtp", "dydtp", "dzdtp", "drdtp", "overlap", "path_new"):
        assert max_rel(ag[k], ar[k]) <= lim, k
    for k in ("total_area", "total_area_per_radius", "total_overlap_area",
              "total_overlap_area_per_radius", "total_volume_new"):
        assert ag[k] == pytest.approx(ar[k], rel=lim), k
    assert abs(ag["max_error"] - ar["max_error"]) <= 1e-4 * cfg.error_tolerance
    assert np.array_equal(ag["delete_flags"], ar["delete_flags"])
    for f in (a, ref, g):
        f.close()


def test_c2_every_step(oracle_mod, c2):
    """60 accepted steps of the 3D N = 10^6 foam with the CUDA path and the
    oracle in lockstep, compared after every step: the same attempt, search
    and deletion counts, dt and pair count, and positions, radii and their
    rates within 1e-9 of each row's maximum, by bubble index. The window
    holds at least one neighbour search."""
    cfg, st = c2
    g, o = both(oracle_mod, cfg, st)
    for f in (g, o):
        workloads.prepare(f)
    rows = ["x", "y", "z", "r", "dxdt", "dydt", "dzdt", "drdt", "index"]
    s0 = g.report()["searches"]
    for step in range(60):
        rg, ro = g.integrate(1), o.integrate(1)
        for k in ("steps", "attempts", "searches", "deleted", "count", "num_pairs"):
            assert rg[k] == ro[k], (step, k)
        assert rg["time_step"] == pytest.approx(ro["time_step"], rel=1e-12), step
        sg, so = by_index(g.get_state(rows=rows)), by_index(o.get_state(rows=rows))
        assert np.array_equal(sg["index"], so["index"]), step
        assert_rows_close(sg, so, rows[:-1], 1e-9, "step %d " % step)
    assert g.report()["searches"] > s0
    g.close()
    o.close()
