"""GPU: batched foams (cb_batch_*) against the same foams run one at a time.

A batch runs the single-foam kernel bodies on per-foam virtual grids, so a
foam in a batch must behave as the same foam in its own context: the same
accepted steps, attempts, searches and deletions, the same bubble count,
pair set and compaction order, and positions equal up to the rounding of
reductions over a different block partition (FP64 form: 1e-12 relative to
the displacement; mixed form: 1e-6, the FP32 atomics' order being free).
The FP64 batch is also checked against the FP64 oracle."""
import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads
from helpers import by_index, pair_set

pytestmark = pytest.mark.gpu


def small_sweep(count=6, precision=1, graph=1, **kw):
    return workloads.sweep(count=count, seed=7, n_range=(1_500, 9_000),
                           precision=precision, use_graph=graph, **kw)


def load_prepared(f, st):
    f.load_state(st)
    workloads.prepare(f)


def displacement_err(cfg, s_a, s_b, s0):
    err = 0.0
    axes = ("x", "y", "z") if cfg.dimensionality == 3 else ("x", "y")
    for a, k in enumerate(axes):
        L = cfg.tfr[a] - cfg.lbb[a]
        d = s_a[k] - s_b[k]
        d = d - L * np.round(d / L)
        m = s_b[k] - s0[k]
        m = m - L * np.round(m / L)
        err = max(err, float(np.max(np.abs(d)) / max(np.max(np.abs(m)), 1e-300)))
    return err


def compare_with_single(items, precision, graph, steps, tol):
    batch = cb.GpuFoamBatch([c for c, _ in items])
    singles = []
    for (cfg, st), bf in zip(items, batch.foams):
        load_prepared(bf, st)
        g = cb.GpuFoam(cfg)
        load_prepared(g, st)
        singles.append(g)
    s0 = [by_index(bf.get_state()) for bf in batch.foams]
    r0 = [g.report() for g in singles]
    reps = batch.integrate(steps)
    for f, ((cfg, _), bf, g) in enumerate(zip(items, batch.foams, singles)):
        rg = g.integrate(steps)
        rb = reps[f]
        for k in ("steps", "attempts", "searches", "deleted", "count", "num_pairs"):
            assert rb[k] == rg[k], (f, k, rb[k], rg[k])
        assert rb["steps"] - r0[f]["steps"] == steps
        sb, sg = bf.get_state(), g.get_state()
        assert np.array_equal(sb["index"], sg["index"]), f
        assert displacement_err(cfg, by_index(sb), by_index(sg), s0[f]) <= tol, f
        bi, bj = bf.pairs()
        gi, gj = g.pairs()
        assert pair_set(bi, bj, sb["index"]) == pair_set(gi, gj, sg["index"]), f
        g.close()
    n = batch.launch_count()
    batch.close()
    return n


@pytest.mark.parametrize("graph", [1, 0])
def test_batch_mixed_matches_single(graph):
    n = compare_with_single(small_sweep(precision=1, graph=graph), 1, graph, 40, 1e-6)
    assert n > 0


def foams_3d(precision, walls, graph=1):
    """3D foams of uneven sizes (six or more cells per periodic axis: the
    search's counting pass is the warp-per-cell one), periodic or all with
    walls in z (a batch holds foams of one wall presence)."""
    wall = (0, 0, 1) if walls else (0, 0, 0)
    return [workloads.foam(n, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=70 + f, wall=wall,
                           wall_drag=0.1 if walls else 0.0, precision=precision,
                           use_graph=graph)
            for f, n in enumerate((6000, 11000, 3500))]


@pytest.mark.parametrize("walls", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_batch_3d_matches_single(precision, walls):
    """3D foams batched and alone: the batched forms of the 3D search and
    attempt kernels on virtual grids."""
    tol = 1e-12 if precision == 0 else 1e-6
    compare_with_single(foams_3d(precision, walls), precision, 1, 30, tol)


def test_batch_fp64_matches_single():
    compare_with_single(small_sweep(count=4, precision=0, graph=1), 0, 1, 25, 1e-12)


def test_batch_fp64_ff_matches_single():
    """The FP64 form with float-float pair terms, batched and alone."""
    compare_with_single(small_sweep(count=4, precision=2, graph=1), 2, 1, 25, 1e-12)


def test_batch_fp64_against_oracle(oracle_mod):
    items = small_sweep(count=3, precision=0, graph=1)
    batch = cb.GpuFoamBatch([c for c, _ in items])
    oracles = []
    for (cfg, st), bf in zip(items, batch.foams):
        load_prepared(bf, st)
        o = oracle_mod.OracleFoam(cfg)
        load_prepared(o, st)
        oracles.append(o)
    s0 = [by_index(bf.get_state()) for bf in batch.foams]
    reps = batch.integrate(10)
    for f, ((cfg, _), bf, o) in enumerate(zip(items, batch.foams, oracles)):
        ro = o.integrate(10)
        for k in ("steps", "attempts", "searches", "deleted", "count", "num_pairs"):
            assert reps[f][k] == ro[k], (f, k)
        assert displacement_err(cfg, by_index(bf.get_state()), by_index(o.get_state()),
                                s0[f]) <= 1e-11
        assert bf.total_volume() == pytest.approx(o.total_volume(), rel=1e-12)
    batch.close()


def test_batch_deletion_matches_single():
    # small radii and a large minimum radius: deletions in the first steps
    items = [workloads.foam(n, 2, 0.85, 1.0, 0.3, (0.01, 2.0), seed=50 + f, min_rad=0.2,
                            precision=1, use_graph=1)
             for f, n in enumerate((3000, 5200, 1800))]
    batch = cb.GpuFoamBatch([c for c, _ in items])
    singles = []
    for (cfg, st), bf in zip(items, batch.foams):
        load_prepared(bf, st)
        g = cb.GpuFoam(cfg)
        load_prepared(g, st)
        singles.append(g)
    reps = batch.integrate(3)
    assert sum(r["deleted"] for r in reps) > 0
    for f, (bf, g) in enumerate(zip(batch.foams, singles)):
        rg = g.integrate(3)
        for k in ("deleted", "count", "num_pairs", "attempts"):
            assert reps[f][k] == rg[k], (f, k)
        assert np.array_equal(bf.get_state()["index"], g.get_state()["index"])
        assert bf.total_volume() == pytest.approx(g.total_volume(), rel=1e-12)
        g.close()
    batch.close()


def test_batch_foam_error_is_isolated():
    # foam 1 may take one attempt per step and starts with a time step far
    # too large: its first attempt is rejected and it stops with
    # CB_ERR_MAX_ATTEMPTS; the other foams still advance all their steps
    items = small_sweep(count=3, precision=1, graph=1)
    cfgs = [c for c, _ in items]
    cfgs[1].max_attempts = 1
    batch = cb.GpuFoamBatch(cfgs)
    for (cfg, st), bf in zip(items, batch.foams):
        load_prepared(bf, st)
    r0 = [bf.report()["steps"] for bf in batch.foams]
    batch.foams[1].set_time(5.0)
    with pytest.raises(cb.CubbleError) as e:
        batch.integrate(20)
    assert e.value.code in (4, 5)  # CB_ERR_MAX_ATTEMPTS (or NONFINITE)
    for f in (0, 2):
        r = batch.foams[f].report()
        assert r["status"] == 0 and r["steps"] - r0[f] == 20
    assert batch.foams[1].report()["status"] in (4, 5)
    batch.close()


def test_batch_rejects_mixed_options():
    a, _ = workloads.foam(1000, 2, 0.9, precision=1)
    b, _ = workloads.foam(1000, 2, 0.9, precision=0)
    with pytest.raises(cb.CubbleError):
        cb.GpuFoamBatch([a, b])


def test_batch_autotune_keeps_results():
    items = small_sweep(count=4, precision=1, graph=1)
    batch = cb.GpuFoamBatch([c for c, _ in items])
    for (cfg, st), bf in zip(items, batch.foams):
        load_prepared(bf, st)
    r0 = [bf.report()["steps"] for bf in batch.foams]
    tile = batch.autotune(3)
    assert tile in (512, 1024, 2048, 4096, 8192)
    reps = batch.integrate(5)
    # trials of 3 steps: 5 tiles, 3 cell scales, 3 pairs-per-thread values
    for f, r in enumerate(reps):
        assert r["steps"] - r0[f] == (5 + 3 + 3) * 3 + 5
        assert r["status"] == 0
    batch.close()
