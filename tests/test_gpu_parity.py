"""GPU parity: the CUDA path (through the C ABI) against the FP64 oracle on
the same seeded inputs.

Bars (FP64 form):
  * cell order, permutation, pair lists, deletion / compaction order and all
    integer rows: bit-exact;
  * one attempt (velocities, radius rates, corrected positions, errors,
    overlap areas, the global sums): max |gpu - oracle| <= 1e-12 max |oracle|
    per row (FP64 atomics reorder the per-bubble sums, and the pair terms are
    float-float, ~1e-14); rows that are differences of two positions (the
    predictor-corrector error, the path) may also differ by 4 ulp of the
    largest coordinate, their FP64 resolution;
  * short trajectories (<= 30 accepted steps): 1e-9 of the row maximum, same
    step / attempt / search / deletion counts.
"""
import math

import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads
from cubble_gb300.foam import CubbleError
from helpers import (DROWS, IROWS, assert_rows_close, brute_pairs, by_index, max_rel, pair_set,
                     position_ulp)

pytestmark = pytest.mark.gpu

CASES = {
    "2d": dict(n=3000, dim=2, phi=0.9, seed=101),
    "3d": dict(n=3000, dim=3, phi=0.8, seed=102, rstd=0.15, rclip=(0.3, 2.5)),
    "2d-wallx": dict(n=2000, dim=2, phi=0.85, seed=103, wall=(1, 0, 0), wall_drag=0.2),
    "3d-wallz": dict(n=2000, dim=3, phi=0.8, seed=104, wall=(0, 0, 1), wall_drag=0.1),
    "2d-small": dict(n=12, dim=2, phi=0.9, seed=105),
    "3d-small": dict(n=40, dim=3, phi=0.8, seed=106),
}


def make(case, **over):
    c = dict(CASES[case])
    c.update(over)
    n, dim, phi = c.pop("n"), c.pop("dim"), c.pop("phi")
    return workloads.foam(n, dim, phi, **c)


def pair_both(oracle_mod, cfg, st, precision=0):
    """The GPU foam in `precision` (0: FP64, 2: FP64 with float-float pair
    terms) and the FP64 oracle on the same state."""
    g = cb.GpuFoam(workloads.sweep_config_as(cfg, precision=precision) if precision else cfg)
    o = oracle_mod.OracleFoam(cfg)
    g.load_state(st)
    o.load_state(st)
    return g, o


def int_rows_equal(a, b):
    for k in IROWS:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("case", list(CASES))
def test_search_bit_exact(oracle_mod, case):
    cfg, st = make(case)
    g, o = pair_both(oracle_mod, cfg, st)
    g.search_neighbors()
    o.search_neighbors()
    sg, so = g.get_state(), o.get_state()
    for k in DROWS:
        assert np.array_equal(sg[k], so[k]), k
    int_rows_equal(sg, so)
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    assert np.array_equal(gi, oi) and np.array_equal(gj, oj)
    assert set(zip(gi.tolist(), gj.tolist())) == brute_pairs(cfg, sg)


@pytest.mark.parametrize("dim", [2, 3])
def test_search_rows_beyond_stash(oracle_mod, dim):
    """Rows with more partners than the counting pass keeps (a few large
    bubbles among small ones) take the second enumeration; the pair list is
    still the oracle's, bit for bit."""
    n = 3000 if dim == 2 else 4000
    cfg, st = workloads.foam(n, dim, 0.85, rmean=0.4, rstd=0.05, rclip=(0.3, 0.5), seed=107)
    r = st["r"].copy()
    r[:: n // 5] = 4.0  # five large bubbles
    st["r"] = r
    g, o = pair_both(oracle_mod, cfg, st)
    g.search_neighbors()
    o.search_neighbors()
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    counts = np.bincount(oi, minlength=n)
    assert counts.max() > (16 if dim == 2 else 32)
    assert np.array_equal(gi, oi) and np.array_equal(gj, oj)
    int_rows_equal(g.get_state(), o.get_state())


@pytest.mark.parametrize("cells", [3, 4])
def test_search_thin_periodic_box(oracle_mod, cells):
    """A 3D periodic box with only 3 or 4 cells along x (9 along y and z):
    at 4 the warp-per-cell counting pass takes it (every stencil offset a
    distinct cell, one periodic image each), at 3 the thread-per-bubble pass
    with the minimum image. Pair list bit-exact against the oracle and equal
    to the brute-force set."""
    rng = np.random.default_rng(110 + cells)
    r = np.clip(rng.normal(1.0, 0.1, 4000), 0.5, 1.3)
    r[0] = 1.3  # the largest radius, whatever the sample size below
    cut = 2.0 * r.max() + 0.3
    lx, ly = (cells + 0.5) * cut, 9.5 * cut
    n = int(0.8 * lx * ly * ly / (4.0 / 3.0 * math.pi * float(np.mean(r ** 3))))
    r = r[:n]
    cfg, st = workloads.foam(n, 3, 0.8, seed=110 + cells, rclip=(0.5, 1.3))
    cfg.tfr[0], cfg.tfr[1], cfg.tfr[2] = lx, ly, ly
    st = {"x": rng.uniform(0.0, lx, n), "y": rng.uniform(0.0, ly, n),
          "z": rng.uniform(0.0, ly, n), "r": r, "index": np.arange(n, dtype=np.int32)}
    g, o = pair_both(oracle_mod, cfg, st)
    g.search_neighbors()
    o.search_neighbors()
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    assert len(gi) > n
    assert np.array_equal(gi, oi) and np.array_equal(gj, oj)
    sg = g.get_state()
    int_rows_equal(sg, o.get_state())
    assert set(zip(gi.tolist(), gj.tolist())) == brute_pairs(cfg, sg)


def test_search_dense_cluster_in_sparse_grid(oracle_mod):
    """A 3D grid that is sparse on average (six cells per axis) with one
    crowded spot: a large bubble in a shell of 300 small ones. The home cell
    and its neighbours hold hundreds of bubbles, so the warp-per-cell
    counting pass runs home blocks beyond 32 bubbles, candidate windows
    beyond 512 and rows beyond the stash; the pair list is still the
    oracle's, bit for bit, and the brute-force set."""
    cfg, st = workloads.foam(2300, 3, 0.3, rmean=1.0, rstd=0.1, rclip=(0.5, 1.5), seed=108)
    side = cfg.tfr[0]
    rng = np.random.default_rng(109)
    x, y, z, r = (np.array(st[k], dtype=np.float64) for k in ("x", "y", "z", "r"))
    c = 0.5 * side
    x[0] = y[0] = z[0] = c
    r[0] = 2.5
    d = rng.normal(size=(300, 3))
    d *= (rng.uniform(0.5, 3.0, 300) / np.linalg.norm(d, axis=1))[:, None]
    x[1:301], y[1:301], z[1:301] = c + d[:, 0], c + d[:, 1], c + d[:, 2]
    r[1:301] = 0.3
    st.update(x=x, y=y, z=z, r=r)
    g, o = pair_both(oracle_mod, cfg, st)
    g.search_neighbors()
    o.search_neighbors()
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    assert np.bincount(oi, minlength=len(x)).max() > 32
    assert np.array_equal(gi, oi) and np.array_equal(gj, oj)
    sg = g.get_state()
    int_rows_equal(sg, o.get_state())
    assert set(zip(gi.tolist(), gj.tolist())) == brute_pairs(cfg, sg)


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("case", ["2d", "3d", "2d-wallx", "3d-wallz"])
def test_bootstrap_and_attempt(oracle_mod, case, precision):
    cfg, st = make(case)
    g, o = pair_both(oracle_mod, cfg, st, precision)
    for f in (g, o):
        workloads.prepare(f)
    sg, so = g.get_state(), o.get_state()
    assert_rows_close(sg, so, ["dxdto", "dydto", "dzdto"], 1e-12, "bootstrap ")
    ag, ao = g.attempt(), o.attempt()
    rows = ["xp", "yp", "zp", "rp", "dxdtp", "dydtp", "dzdtp", "drdtp", "error",
            "path_new", "overlap"]
    floor = position_ulp(so)
    assert_rows_close(ag, ao, rows, 1e-12, "attempt ", floor=floor)
    for k in ("total_area", "total_area_per_radius", "total_overlap_area",
              "total_overlap_area_per_radius", "total_volume_new", "max_radius",
              "max_expansion"):
        assert ag[k] == pytest.approx(ao[k], rel=1e-12, abs=1e-300), k
    assert ag["max_error"] == pytest.approx(ao["max_error"], rel=1e-12, abs=floor)
    assert np.array_equal(ag["delete_flags"], ao["delete_flags"])
    assert ag["num_to_be_deleted"] == ao["num_to_be_deleted"]
    assert g.report()["time_step"] == o.report()["time_step"]


@pytest.mark.parametrize("precision", [0, 2])
def test_flow_attempt(oracle_mod, precision):
    cfg, st = make("2d", use_flow=1, flow_lbb=(0.0, 20.0, 0.0), flow_tfr=(30.0, 40.0, 0.0),
                   flow_vel=(0.01, 0.0, 0.0))
    g, o = pair_both(oracle_mod, cfg, st, precision)
    for f in (g, o):
        workloads.prepare(f)
        f.integrate(3)
    ag, ao = g.attempt(), o.attempt()
    assert_rows_close(ag, ao, ["xp", "yp", "dxdtp", "dydtp", "drdtp"], 1e-11, "flow ")


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_shear_attempt_and_trajectory(oracle_mod, precision):
    """The linear shear extension (walls in z, shear along x) against the
    oracle's restatement: the FP64 forms within 1e-11, the mixed form within
    1e-6."""
    cfg, st = make("3d-wallz", use_flow=1, shear_speed=0.05)
    cfg_g, _ = make("3d-wallz", use_flow=1, shear_speed=0.05, precision=precision)
    g = cb.GpuFoam(cfg_g)
    o = oracle_mod.OracleFoam(cfg)
    for f in (g, o):
        f.load_state(st)
        workloads.prepare(f)
        f.integrate(3)
    if precision == 1:
        i, j = o.pairs()
        g.load_state(o.get_state())
        g.set_pairs(i, j)
        g.set_time(o.report()["time_step"])
    ag, ao = g.attempt(), o.attempt()
    tol = 1e-6 if precision == 1 else 1e-11
    assert_rows_close(ag, ao, ["dxdtp", "dydtp", "dzdtp", "drdtp"], tol, "shear ")
    # the imposed profile: mean x velocity grows with height
    s = o.get_state()
    z, vx = s["z"], ao["dxdtp"]
    lo, hi = z < np.quantile(z, 0.2), z > np.quantile(z, 0.8)
    assert vx[hi].mean() - vx[lo].mean() > 0.02
    rg, ro = g.integrate(10), o.integrate(10)
    for k in ("steps", "searches", "deleted", "count"):
        assert rg[k] == ro[k], k


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("graph", [0, 1])
@pytest.mark.parametrize("case", ["2d", "3d", "3d-wallz"])
def test_trajectory(oracle_mod, case, graph, precision):
    cfg, st = make(case, use_graph=graph)
    g, o = pair_both(oracle_mod, cfg, st, precision)
    for f in (g, o):
        workloads.prepare(f)
    rg = g.integrate(30)
    ro = o.integrate(30)
    for k in ("steps", "attempts", "searches", "deleted", "count", "num_pairs"):
        assert rg[k] == ro[k], k
    assert rg["time_step"] == pytest.approx(ro["time_step"], rel=1e-12)
    sg, so = by_index(g.get_state()), by_index(o.get_state())
    assert_rows_close(sg, so, ["x", "y", "z", "r", "dxdt", "dydt", "drdt", "path",
                               "dxdto", "error"], 1e-9, "trajectory ")


@pytest.mark.parametrize("precision", [0, 2])
def test_c1_full_run(oracle_mod, precision):
    """The 2D configuration at its stated size and length: N = 10^4, phi 0.90,
    1000 adaptive steps with gas exchange and deletions, GPU FP64 forms
    against the oracle. Same accepted steps, attempts, searches, deletions
    and pair count; states within 1e-8 of each row's maximum (rounding of
    FP64 atomics over 1000 steps of a dissipative flow), total volume and
    energy within 1e-10."""
    import os
    cfg, st = workloads.config_c1(use_graph=1)
    g = cb.GpuFoam(workloads.sweep_config_as(cfg, precision=precision) if precision else cfg)
    o = oracle_mod.OracleFoam(cfg, threads=os.cpu_count() or 1)
    for f in (g, o):
        f.load_state(st)
        workloads.prepare(f)
    rg, ro = g.integrate(1000), o.integrate(1000)
    for k in ("steps", "attempts", "searches", "deleted", "count", "num_pairs"):
        assert rg[k] == ro[k], k
    assert rg["time_step"] == pytest.approx(ro["time_step"], rel=1e-9)
    sg, so = by_index(g.get_state()), by_index(o.get_state())
    assert np.array_equal(sg["index"], so["index"])
    assert_rows_close(sg, so, ["x", "y", "r", "dxdt", "dydt", "drdt", "path"], 1e-8, "c1 ")
    assert g.total_volume() == pytest.approx(o.total_volume(), rel=1e-10)
    assert g.energy() == pytest.approx(o.energy(), rel=1e-10)


@pytest.mark.parametrize("graph", [0, 1])
@pytest.mark.parametrize("dim", [2, 3])
def test_deletion_bit_exact_order(oracle_mod, dim, graph):
    cfg, st = workloads.foam(3000, dim, 0.85, rstd=0.3, rclip=(0.01, 2.0), seed=110 + dim,
                             min_rad=0.2, use_graph=graph)
    g, o = pair_both(oracle_mod, cfg, st)
    for f in (g, o):
        workloads.prepare(f)
    rg, ro = g.integrate(1), o.integrate(1)
    assert ro["deleted"] > 0
    for k in ("deleted", "count", "num_pairs", "searches"):
        assert rg[k] == ro[k], k
    sg, so = g.get_state(), o.get_state()
    int_rows_equal(sg, so)
    assert_rows_close(sg, so, ["x", "y", "z", "r", "dxdt", "drdt", "saved_r"], 1e-12, "delete ")
    gi, gj = g.pairs()
    oi, oj = o.pairs()
    if rg["searches"] == 1:  # no re-search: compaction order itself
        assert np.array_equal(gi, oi) and np.array_equal(gj, oj)
    assert pair_set(gi, gj, sg["index"]) == pair_set(oi, oj, so["index"])
    M = cfg.bubble_volume_multiplier
    target = math.pi * M ** 2 if dim == 2 else 4.0 / 3.0 * math.pi * M ** 3
    assert g.total_volume() == pytest.approx(target, rel=1e-12)


@pytest.mark.parametrize("dim", [2, 3])
def test_energy_volume(oracle_mod, dim):
    cfg, st = make("2d" if dim == 2 else "3d")
    g, o = pair_both(oracle_mod, cfg, st)
    for f in (g, o):
        f.search_neighbors()
    assert g.energy() == pytest.approx(o.energy(), rel=1e-12)
    assert g.total_volume() == pytest.approx(o.total_volume(), rel=1e-12)
    assert max_rel(g.bubble_energies(), o.bubble_energies()) <= 1e-12


@pytest.mark.parametrize("case", ["2d", "3d"])
def test_graph_matches_eager(oracle_mod, case):
    """The same 40 steps as one graph and as eager launches: same counts and
    states, and the graph's launch count (kernels per attempt, deletion and
    search, counted when the graph was captured) equal to the eager one."""
    cfg0, st = make(case, use_graph=0)
    cfg1, _ = make(case, use_graph=1)
    a, b = cb.GpuFoam(cfg0), cb.GpuFoam(cfg1)
    for f in (a, b):
        f.load_state(st)
        workloads.prepare(f)
    la, lb = a.launch_count(), b.launch_count()
    ra, rb = a.integrate(40), b.integrate(40)
    for k in ("steps", "attempts", "searches", "deleted", "count"):
        assert ra[k] == rb[k], k
    sa, sb = by_index(a.get_state()), by_index(b.get_state())
    assert_rows_close(sa, sb, ["x", "y", "z", "r"], 1e-10, "graph ")
    assert b.launch_count() - lb == a.launch_count() - la > 0


@pytest.mark.parametrize("precision", [0, 2])
def test_single_steps_with_calls_between(oracle_mod, precision):
    """Back-to-back graph cb_integrate(1) calls reuse the host copy of the
    control block; any other call in between makes the next one read it from
    the device again. Here a neighbour search (it changes the pair count on
    the device only) and an option change sit between single steps; the
    oracle runs the same sequence: same counts and pairs, states within the
    trajectory bar."""
    cfg, st = make("2d", use_graph=1)
    g, o = pair_both(oracle_mod, cfg, st, precision)
    for f in (g, o):
        workloads.prepare(f)
    for phase in range(3):
        for _ in range(4):
            rg, ro = g.integrate(1), o.integrate(1)
            for k in ("steps", "attempts", "searches", "count", "num_pairs"):
                assert rg[k] == ro[k], (phase, k)
        if phase == 0:
            for f in (g, o):
                f.search_neighbors()
        else:
            for f in (g, o):
                f.set_options(1, 0, 0)  # path no longer incremented
    assert g.report()["num_pairs"] == o.report()["num_pairs"]
    sg, so = by_index(g.get_state()), by_index(o.get_state())
    assert_rows_close(sg, so, ["x", "y", "r", "path", "error"], 1e-9, "single steps ")


def test_two_foams_alternating_single_steps():
    """Single graph steps alternating between two contexts: each call finds
    the other context's call in between and reads its control block again,
    and each foam follows the trajectory it has when run alone."""
    cfg, st = make("2d", use_graph=1)
    a, b, solo = cb.GpuFoam(cfg), cb.GpuFoam(cfg), cb.GpuFoam(cfg)
    for f in (a, b, solo):
        f.load_state(st)
        workloads.prepare(f)
    for _ in range(12):
        a.integrate(1)
        b.integrate(1)
        solo.integrate(1)
    ra, rb, rs = a.report(), b.report(), solo.report()
    for k in ("steps", "attempts", "searches", "count", "num_pairs"):
        assert ra[k] == rs[k] and rb[k] == rs[k], k
    ss = by_index(solo.get_state())
    for f in (a, b):
        assert_rows_close(by_index(f.get_state()), ss, ["x", "y", "r"], 1e-10, "alternating ")
    for f in (a, b, solo):
        f.close()


def test_pair_capacity_error(oracle_mod):
    cfg, st = make("2d", pair_capacity=100)
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    with pytest.raises(CubbleError) as e:
        g.search_neighbors()
    assert e.value.code == 3


@pytest.mark.parametrize("graph", [0, 1])
def test_reject_loop_cap(oracle_mod, graph):
    cfg, st = make("2d", tol=1e-30, max_attempts=5, use_graph=graph)
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    workloads.prepare(g)
    with pytest.raises(CubbleError) as e:
        g.integrate(1)
    assert e.value.code == 4
    assert g.report()["attempts"] == 5
