"""GPU: the launch and search knobs (cb_tuning) and the autotuner.

A tuned context must compute the same physics as a default one: the pair set
of a search, keyed by bubble index, bit-exact (a larger cell changes which
candidates are tested and the bubble order, never the set); one attempt
within 1e-12 (FP64 form: only the order of FP64 reductions moves) or 1e-6
(mixed form: FP32 reductions in another order); short trajectories with the
same step, attempt, search and deletion counts and states within 1e-9 (FP64).
The autotuner picks valid knobs, keeps them for later contexts of the same
kind, and cb_forget_tuning drops them."""
import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads
from helpers import assert_rows_close, by_index, pair_set

pytestmark = pytest.mark.gpu


def case(dim, precision, n=20000):
    if dim == 3:
        return workloads.foam(n, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=61,
                              precision=precision, use_graph=1)
    return workloads.foam(n, 2, 0.9, seed=62, min_rad=0.05, precision=precision, use_graph=1)


@pytest.fixture(autouse=True)
def fresh_cache():
    cb.lib().cb_forget_tuning()
    yield
    cb.lib().cb_forget_tuning()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("dim", [3, 2])
def test_tuned_knobs_keep_pairs_and_physics(dim, precision):
    cfg, st = case(dim, precision)
    a, b = cb.GpuFoam(cfg), cb.GpuFoam(cfg)
    b.set_tuning(cell_scale=1.3, pair_run=2 if precision == 1 else 4, pair_blocks=2,
                 step_blocks=1)
    assert b.tuning()["cell_scale"] == 1.3
    for f in (a, b):
        f.load_state(st)
        f.search_neighbors()
    sa, sb = a.get_state(), b.get_state()
    assert not np.array_equal(sa["index"], sb["index"])  # another cell order
    assert pair_set(*a.pairs(), sa["index"]) == pair_set(*b.pairs(), sb["index"])
    for f in (a, b):
        f.bootstrap()
        f.integrate(3)
    # one attempt from the same state: b takes a's rows and pair list
    s0 = a.get_state()
    b.load_state(s0)
    b.set_pairs(*a.pairs())
    dt0 = a.report()["time_step"]
    b.set_time(dt0)
    ra, rb = a.attempt(), b.attempt()
    tol = 1e-12 if precision == 0 else 1e-6
    assert_rows_close(rb, ra, ["dxdtp", "dydtp", "drdtp", "overlap"], tol, "tuned attempt ")
    if precision == 0:
        a.set_time(dt0)
        b.set_time(dt0)
        qa, qb = a.integrate(20), b.integrate(20)
        for k in ("steps", "attempts", "searches", "deleted", "count", "num_pairs"):
            assert qa[k] == qb[k], k
        sa, sb = by_index(a.get_state()), by_index(b.get_state())
        assert_rows_close(sb, sa, ["x", "y", "r", "dxdt", "drdt"], 1e-9, "tuned trajectory ")


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_picks_and_keeps_knobs(precision):
    cfg, st = case(3, precision)
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    g.search_neighbors()
    t = g.autotune(2)
    assert 1.0 <= t["cell_scale"] <= 1.5
    assert t["pair_run"] in ((2, 4, 8) if precision == 1 else (4,))
    assert 0 <= t["pair_blocks"] <= 3 and 0 <= t["step_blocks"] <= 3
    assert g.tuning() == t
    # the state is left searched and steps on
    g.bootstrap()
    r = g.integrate(5)
    assert r["steps"] == 5 and r["status"] == 0
    h = cb.GpuFoam(cfg)  # same dimensionality, precision and capacity bucket
    assert h.tuning() == t
    cb.lib().cb_forget_tuning()
    assert cb.GpuFoam(cfg).tuning()["cell_scale"] == 1.0


def test_batch_autotune_sets_knobs():
    items = workloads.sweep(count=6, seed=9, n_range=(1000, 4000), precision=1, use_graph=1)
    batch = cb.GpuFoamBatch([c for c, _ in items])
    for (cfg, st), f in zip(items, batch.foams):
        f.load_state(st)
        workloads.prepare(f)
    tile = batch.autotune(3)
    assert tile in (512, 1024, 2048, 4096, 8192)
    t = batch.foams[0].tuning()
    assert all(f.tuning() == t for f in batch.foams)
    assert t["pair_run"] in (2, 4, 8) and 1.0 <= t["cell_scale"] <= 1.3
    reps = batch.integrate(10)
    assert all(r["status"] == 0 for r in reps)
    batch.close()
