"""GPU: init()'s device steps against the reference's own kernels.

tests/golden/init_{2,3}d.npz hold, for seeded draws, the output of the
reference's assignDataToBubbles (src/kernels.cu:1026-1071) and of
transformPositions (src/kernels.cu:971-990) both ways, recorded by
tests/golden/make_golden.py --init on a GB300. cb_assign_lattice and
cb_transform_positions must reproduce them bit for bit; the mean initial
area (averageSurfaceAreaIn) is a sum whose order differs (1e-14)."""
import os

import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def fixture(dim):
    return np.load(os.path.join(HERE, "golden", "init_%dd.npz" % dim))


def lattice_foam(g, dim, tfr=None):
    n = int(np.prod(g["bpd"]))
    cfg, _ = workloads.foam(n, dim, 0.9, seed=1, min_rad=float(g["min_rad"]))
    box = g["tfr"] if tfr is None else tfr
    for a in range(3):
        cfg.lbb[a] = 0.0
        cfg.tfr[a] = float(box[a])
    return cb.GpuFoam(cfg), n


@pytest.mark.parametrize("dim", [2, 3])
def test_assign_lattice_matches_reference(dim):
    g = fixture(dim)
    f, n = lattice_foam(g, dim)
    area, mr = f.assign_lattice(g["bpd"], float(g["avg_rad"]), g["in_ux"], g["in_uy"],
                                g["in_uz"], g["in_uw"], g["in_nr"])
    s = f.get_state()
    for k in ("x", "y", "r"):
        assert np.array_equal(s[k], g["out_" + k]), k
    if dim == 3:
        assert np.array_equal(s["z"], g["out_z"])
    assert np.array_equal(s["index"], g["out_index"])
    assert area == pytest.approx(float(np.sum(g["out_rp"])), rel=1e-13)
    assert mr == float(np.max(g["out_r"]))
    f.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_transform_positions_matches_reference(dim):
    g = fixture(dim)
    f, n = lattice_foam(g, dim)
    st = {"x": g["out_x"], "y": g["out_y"], "z": g["out_z"], "r": g["out_r"]}
    f.load_state(st)
    f.transform_positions(True)
    s = f.get_state()
    for k in ("x", "y") + (("z",) if dim == 3 else ()):
        assert np.array_equal(s[k], g["norm_" + k]), k
    tfr = g["new_tfr"]
    M = f.config.bubble_volume_multiplier
    f.set_box((0.0, 0.0, 0.0), tuple(float(v) for v in tfr), M)
    f.transform_positions(False)
    s = f.get_state()
    for k in ("x", "y") + (("z",) if dim == 3 else ()):
        assert np.array_equal(s[k], g["back_" + k]), k
    f.close()


def test_averages_and_resets():
    cfg, st = workloads.foam(3000, 2, 0.9, seed=9, precision=1)
    f = cb.GpuFoam(cfg)
    f.load_state(st)
    workloads.prepare(f)
    f.integrate(5)
    s = f.get_state()
    m = f.averages()
    ref = [s["r"].mean(), s["dxdt"].mean(), s["dydt"].mean(), s["dzdt"].mean(),
           s["drdt"].mean(), s["path"].mean()]
    for a, b in zip(m, ref):
        assert a == pytest.approx(b, rel=1e-12, abs=1e-15)
    assert np.any(s["error"] != 0)
    f.reset_rows(1)
    assert np.all(f.get_state()["error"] == 0)
    f.close()


@pytest.mark.parametrize("graph", [1, 0])
def test_integrate_until_stops_like_simulate(graph):
    cfg, st = workloads.foam(3000, 2, 0.9, seed=10, use_graph=graph)
    f = cb.GpuFoam(cfg)
    f.load_state(st)
    workloads.prepare(f)
    r0 = f.report()
    t0 = r0["time_integer"] + r0["time_fraction"]
    target = t0 + 50 * r0["time_step"]
    r = f.integrate_until(10_000, time=target)
    t = r["time_integer"] + r["time_fraction"]
    assert t >= target and r["steps"] > r0["steps"]
    # the step before ended short of the target: one step less does not reach it
    assert t - r["dt_max"] * 1.0001 < target or r["steps"] - r0["steps"] == 1
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    workloads.prepare(g)
    rg = g.integrate(r["steps"] - r0["steps"])
    assert rg["time_integer"] + rg["time_fraction"] == pytest.approx(t, rel=1e-12)
    # max_steps bounds the stretch; a count floor stops at once
    r2 = f.integrate_until(7)
    assert r2["steps"] - r["steps"] == 7
    r3 = f.integrate_until(100, min_count=10**9)
    assert r3["steps"] - r2["steps"] == 1
    f.close()
    g.close()
