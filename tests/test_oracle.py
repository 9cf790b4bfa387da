"""CPU tests of the FP64 oracle (the checker) against brute force, analytic
two-bubble cases and conservation laws."""
import math

import numpy as np
import pytest

from cubble_gb300 import workloads
from cubble_gb300.foam import CubbleError, make_config
from helpers import brute_pairs, by_index, pair_set, wrapped_sq


def oracle_foam(oracle_mod, cfg, state, threads=1):
    f = oracle_mod.OracleFoam(cfg, threads=threads)
    f.load_state(state)
    return f


CASES = [
    dict(n=1500, dim=2, phi=0.9, seed=11),
    dict(n=1500, dim=3, phi=0.8, seed=12, rstd=0.15, rclip=(0.3, 2.5)),
    dict(n=800, dim=2, phi=0.85, seed=13, wall=(1, 0, 0)),
    dict(n=800, dim=3, phi=0.8, seed=14, wall=(0, 0, 1)),
    dict(n=12, dim=2, phi=0.9, seed=15),   # two cells per axis
    dict(n=4, dim=2, phi=0.9, seed=16),    # one cell per axis
    dict(n=40, dim=3, phi=0.8, seed=17),   # two cells per axis in 3D
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%dD-n%d-w%s" % (
    c["dim"], c["n"], "".join(map(str, c.get("wall", (0, 0, 0))))))
def test_pairs_match_brute_force(oracle_mod, case):
    case = dict(case)
    n, dim, phi = case.pop("n"), case.pop("dim"), case.pop("phi")
    cfg, st = workloads.foam(n, dim, phi, **case)
    f = oracle_foam(oracle_mod, cfg, st)
    f.search_neighbors()
    s = f.get_state()
    i, j = f.pairs()
    assert np.all(i < j)
    # rows ascending, j ascending inside a row
    key = i.astype(np.int64) * (n + 1) + j
    assert np.all(np.diff(key) > 0)
    expect = brute_pairs(cfg, s)
    assert set(zip(i.tolist(), j.tolist())) == expect
    # the permutation keeps every bubble once; saved == positions
    assert sorted(s["index"].tolist()) == list(range(n))
    for a, b in (("x", "saved_x"), ("y", "saved_y"), ("r", "saved_r")):
        assert np.array_equal(s[a], s[b])
    nn = np.bincount(np.concatenate([i, j]), minlength=n)
    assert np.array_equal(nn, s["num_neighbors"])


def test_cell_order_is_stable(oracle_mod):
    cfg, st = workloads.foam(2000, 2, 0.9, seed=3)
    f = oracle_foam(oracle_mod, cfg, st)
    f.search_neighbors()
    s = f.get_state()
    cd = f.cell_dims()
    iv = [cfg.tfr[a] - cfg.lbb[a] for a in range(3)]
    kx = np.clip(np.floor(cd[0] * (s["x"] - cfg.lbb[0]) / iv[0]), 0, cd[0] - 1)
    ky = np.clip(np.floor(cd[1] * (s["y"] - cfg.lbb[1]) / iv[1]), 0, cd[1] - 1)
    cell = (ky * cd[0] + kx).astype(np.int64)
    # sorted by (cell, previous position == original index here)
    key = cell * 10 ** 7 + s["index"]
    assert np.all(np.diff(key) > 0)


def test_wrap_counts(oracle_mod):
    cfg, st = workloads.foam(500, 2, 0.9, seed=4)
    L = cfg.tfr[0]
    st = dict(st)
    st["x"] = st["x"].copy()
    st["x"][:10] += L          # pushed out on the high side
    st["x"][10:20] -= L        # and on the low side
    f = oracle_foam(oracle_mod, cfg, st)
    f.search_neighbors()
    s = by_index(f.get_state())
    assert np.all(s["wrap_count_x"][:10] == 1)
    assert np.all(s["wrap_count_x"][10:20] == -1)
    assert np.all(s["wrap_count_x"][20:] == 0)
    assert np.all((s["x"] >= 0) & (s["x"] <= L))


def two_bubble(dim, d, r1, r2, gas=1, kappa=0.01, K=0.1):
    L = 100.0
    cfg = make_config(dimensionality=dim, lbb=(0, 0, 0),
                      tfr=(L, L, L if dim == 3 else 0.0), capacity=2,
                      min_rad=0.05, f0_per_mu0=1.0, k_parameter=K, kappa=kappa,
                      skin_radius=0.3, bubble_volume_multiplier=1.0,
                      average_surface_area_in=4.0, error_tolerance=1.0,
                      time_step=1e-3, use_gas_exchange=gas)
    st = {"x": np.array([50.0, 50.0 + d]), "y": np.array([50.0, 50.0]),
          "z": np.array([50.0 if dim == 3 else 0.0] * 2),
          "r": np.array([r1, r2])}
    return cfg, st


@pytest.mark.parametrize("dim", [2, 3])
def test_two_bubble_analytic(oracle_mod, dim):
    d, r1, r2 = 1.3, 1.0, 0.8
    cfg, st = two_bubble(dim, d, r1, r2)
    f = oracle_foam(oracle_mod, cfg, st)
    f.search_neighbors()
    out = f.attempt()
    s = f.get_state()
    i0 = int(np.where(s["index"] == 0)[0][0])
    i1 = 1 - i0
    R = r1 + r2
    fx = -(1.0 - d / R)  # f0 d (1/|d| - 1/R) with d = x0 - x1 = -d
    assert out["dxdtp"][i0] == pytest.approx(fx, rel=1e-14)
    assert out["dxdtp"][i1] == pytest.approx(-fx, rel=1e-14)
    assert abs(out["dydtp"][i0]) == 0.0
    a2 = r2 ** 2 - ((r2 ** 2 - r1 ** 2 + d * d) / (2 * d)) ** 2
    oa = math.pi * a2 if dim == 3 else 2.0 * math.sqrt(a2)
    assert out["overlap"][i0] == pytest.approx(oa, rel=1e-13)
    area = [4 * math.pi * r * r if dim == 3 else 2 * math.pi * r for r in (r1, r2)]
    sA = sum(area)
    sAr = sum(a / r for a, r in zip(area, (r1, r2)))
    sAo = 2 * oa
    sAor = oa * (1 / r1 + 1 / r2)
    assert out["total_area"] == pytest.approx(sA, rel=1e-14)
    assert out["total_overlap_area"] == pytest.approx(sAo, rel=1e-14)
    assert out["total_overlap_area_per_radius"] == pytest.approx(sAor, rel=1e-14)
    pair = [oa * (1 / r2 - 1 / r1), -oa * (1 / r2 - 1 / r1)]
    for k, (r, A, pw) in enumerate(zip((r1, r2), area, pair)):
        vr = (sAr - sAor) / (sA - sAo) - 1 / r
        vr *= cfg.kappa * cfg.average_surface_area_in * 2 / sA * (A - oa)
        vr = (vr + pw) * cfg.k_parameter / A
        row = i0 if k == 0 else i1
        assert out["drdtp"][row] == pytest.approx(vr, rel=1e-12)
        # AM2 correct from rest: r + dt/2 (0 + vr)
        assert out["rp"][row] == pytest.approx(r + 0.5 * cfg.time_step * vr, rel=1e-14)


def test_pairwise_flux_conserves(oracle_mod):
    cfg, st = workloads.foam(2000, 2, 0.9, seed=5, kappa=0.0)
    f = oracle_foam(oracle_mod, cfg, st)
    workloads.prepare(f)
    out = f.attempt()
    s = f.get_state()
    area = 2 * math.pi * s["r"]  # predicted r == r: drdt == drdto == 0
    pairwise = out["drdtp"] * area / cfg.k_parameter
    assert abs(pairwise.sum()) <= 1e-12 * np.abs(pairwise).sum()
    # overlap velocities are equal and opposite
    assert abs(out["dxdtp"].sum()) <= 1e-12 * np.abs(out["dxdtp"]).sum()
    assert abs(out["dydtp"].sum()) <= 1e-12 * np.abs(out["dydtp"]).sum()


@pytest.mark.parametrize("dim", [2, 3])
def test_volume_fix_restores_gas_fraction(oracle_mod, dim):
    cfg, st = workloads.foam(1500, dim, 0.85, rstd=0.3, rclip=(0.01, 2.0),
                             seed=6, min_rad=0.2)
    f = oracle_foam(oracle_mod, cfg, st)
    workloads.prepare(f)
    before = f.count()
    rep = f.integrate(1)
    assert rep["deleted"] > 0 and f.count() == before - rep["deleted"]
    M = cfg.bubble_volume_multiplier
    target = math.pi * M ** 2 if dim == 2 else 4.0 / 3.0 * math.pi * M ** 3
    assert f.total_volume() == pytest.approx(target, rel=1e-12)


def test_deletion_compaction_order(oracle_mod):
    n = 60
    cfg, st = workloads.foam(n, 2, 0.5, seed=7, rstd=0.05, min_rad=0.05, pair_capacity=n * n)
    st = dict(st)
    r = st["r"].copy()
    doomed = np.array([3, 10, 11, 40, 55, 58])
    r[doomed] = 0.01
    st["r"] = r
    cfg.skin_radius = 100.0  # no search after the step
    f = oracle_foam(oracle_mod, cfg, st)
    f.search_neighbors()
    pre = f.get_state()
    pi0, pj0 = f.pairs()
    f.integrate(1)
    post = f.get_state()
    assert f.count() == n - len(doomed)
    rows_doomed = {int(np.where(pre["index"] == d)[0][0]) for d in doomed}
    nnew = n - len(doomed)
    holes = sorted(k for k in rows_doomed if k < nnew)
    movers = [k for k in range(n - 1, nnew - 1, -1) if k not in rows_doomed]
    expect = pre["index"].copy()
    for h, m in zip(holes, movers):
        expect[h] = pre["index"][m]
    assert np.array_equal(post["index"], expect[:nnew])
    # pair set: pairs touching a doomed bubble are gone, the rest survive
    i, j = f.pairs()
    got = pair_set(i, j, post["index"])
    want = {p for p in pair_set(pi0, pj0, pre["index"]) if p[0] not in doomed and p[1] not in doomed}
    assert got == want


def test_reject_loop_cap(oracle_mod):
    cfg, st = workloads.foam(300, 2, 0.9, seed=8, tol=1e-30, max_attempts=5)
    f = oracle_foam(oracle_mod, cfg, st)
    workloads.prepare(f)
    with pytest.raises(CubbleError) as e:
        f.integrate(1)
    assert e.value.code == 4
    assert f.report()["attempts"] == 5


def test_time_accumulator_uses_updated_dt(oracle_mod):
    cfg, st = workloads.foam(400, 2, 0.9, seed=9)
    f = oracle_foam(oracle_mod, cfg, st)
    workloads.prepare(f)
    dts = []
    for _ in range(20):
        f.integrate(1)
        dts.append(f.report()["time_step"])
    rep = f.report()
    # src/simulator.cu:311-314 adds the dt after step() has updated it
    assert rep["time_integer"] + rep["time_fraction"] == pytest.approx(sum(dts), rel=1e-12)


def test_threads_agree(oracle_mod):
    cfg, st = workloads.foam(3000, 3, 0.8, seed=10, rstd=0.15, rclip=(0.3, 2.5))
    outs = []
    for t in (1, 4):
        f = oracle_foam(oracle_mod, cfg, st, threads=t)
        workloads.prepare(f)
        f.integrate(5)
        outs.append(by_index(f.get_state()))
    for k in ("x", "y", "z", "r", "dxdt"):
        np.testing.assert_allclose(outs[1][k], outs[0][k], rtol=0, atol=1e-11 * np.abs(outs[0][k]).max())


def test_energy_and_volume(oracle_mod):
    cfg, st = workloads.foam(500, 3, 0.8, seed=21)
    f = oracle_foam(oracle_mod, cfg, st)
    f.search_neighbors()
    s = f.get_state()
    i, j = f.pairs()
    sq = wrapped_sq(cfg, s["x"][i], s["y"][i], s["z"][i], s["x"][j], s["y"][j], s["z"][j])
    e = s["r"][i] + s["r"][j] - np.sqrt(sq)
    e = np.where(e > 0, e * e, 0.0)
    assert f.energy() == pytest.approx(2 * e.sum(), rel=1e-12)
    assert f.total_volume() == pytest.approx(float(np.sum(4 / 3 * math.pi * s["r"] ** 3)), rel=1e-12)


def test_oracle_shear_profile():
    """Linear shear (extension): an isolated bubble at height q gains
    shear_speed * (2 (q - lbb) / L - 1) along x and nothing else."""
    from cubble_gb300 import workloads
    from oracle.oracle import OracleFoam
    cfg, _ = workloads.foam(4, 3, 0.5, seed=3, wall=(0, 0, 1), use_flow=1,
                            shear_speed=0.05)
    L = 40.0
    for a in range(3):
        cfg.tfr[a] = L
    st = {"x": np.array([5.0, 15.0, 25.0, 35.0]), "y": np.full(4, 20.0),
          "z": np.array([10.0, 20.0, 30.0, 5.0]), "r": np.full(4, 1.0)}
    o = OracleFoam(cfg)
    o.load_state(st)
    o.search_neighbors()
    z = o.get_state()["z"]  # cell order after the search
    a = o.attempt()
    expect = 0.05 * (2.0 * z / L - 1.0)
    np.testing.assert_allclose(a["dxdtp"], expect, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(a["dydtp"], 0.0, atol=1e-15)


@pytest.mark.parametrize("dim", [2, 3])
def test_degenerate_foams(oracle_mod, dim):
    """No bubbles, one bubble, two overlapping and two apart: the step runs,
    a lone bubble stays where it is, an overlapping pair separates
    symmetrically and the gas volume is unchanged."""
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    for n, overlap in ((0, True), (1, True), (2, True), (2, False)):
        cfg, st = workloads.foam(4, dim, 0.5, seed=3)
        cfg.lbb = cb._abi.D3(0.0, 0.0, 0.0)
        cfg.tfr = cb._abi.D3(10.0, 10.0, 10.0 if dim == 3 else 0.0)
        st = {k: np.asarray(v)[:n].copy() for k, v in st.items()}
        if n:
            st["x"][:] = [4.0, 5.5][:n]
            st["y"][:] = 5.0
            st["r"][:] = 1.0
            if dim == 3:
                st["z"][:] = 5.0
            if n == 2 and not overlap:
                st["x"][1] = 7.5
            st["index"] = np.arange(n, dtype=np.int32)
        o = oracle_mod.OracleFoam(cfg)
        o.load_state(st)
        workloads.prepare(o)
        v0 = o.total_volume()
        r = o.integrate(5)
        assert r["status"] == 0 and r["steps"] == 5 and r["count"] == n
        s = o.get_state()
        if n == 1:
            assert s["x"][0] == 4.0
        if n == 2:
            assert r["num_pairs"] == 1 if overlap else True
            if overlap:
                assert s["x"][0] < 4.0 and s["x"][1] > 5.5
                assert s["x"][0] - 4.0 == pytest.approx(-(s["x"][1] - 5.5), rel=1e-12)
        assert o.total_volume() == pytest.approx(v0, rel=1e-12, abs=1e-300)
