"""GPU: degenerate foams against the FP64 oracle, in every form, eager and as
a graph: no bubbles, one bubble (no pairs, no motion), two overlapping
bubbles (one pair pushing them apart symmetrically) and two apart (a listed
pair that does not overlap). Same steps, counts and pairs; positions and
radii within the form's bar (FP64 forms 1e-12 of the displacement, mixed
1e-6); total volume within 1e-12 (mixed 1e-10). A batch that mixes such foams with a
normal one runs them alongside and leaves the normal one as it runs alone."""
import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads

pytestmark = pytest.mark.gpu

L = 10.0


def tiny(n, dim, overlap=True, precision=0, graph=0):
    cfg, st = workloads.foam(4, dim, 0.5, seed=3, precision=precision, use_graph=graph)
    cfg.lbb = cb._abi.D3(0.0, 0.0, 0.0)
    cfg.tfr = cb._abi.D3(L, L, L if dim == 3 else 0.0)
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
    return cfg, st


CASES = [(0, True), (1, True), (2, True), (2, False)]


@pytest.mark.parametrize("graph", [0, 1])
@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("n,overlap", CASES)
def test_tiny_foam(oracle_mod, dim, n, overlap, precision, graph):
    cfg, st = tiny(n, dim, overlap, precision, graph)
    cfg_o, _ = tiny(n, dim, overlap)
    g = cb.GpuFoam(cfg)
    o = oracle_mod.OracleFoam(cfg_o)
    for f in (g, o):
        f.load_state(st)
        workloads.prepare(f)
    rg, ro = g.integrate(5), o.integrate(5)
    for k in ("steps", "count", "num_pairs", "deleted", "status"):
        assert rg[k] == ro[k], k
    sg, so = g.get_state(), o.get_state()
    tol = 1e-6 if precision == 1 else 1e-12
    for k in ("x", "y", "z", "r") if dim == 3 else ("x", "y", "r"):
        d = np.abs(sg[k] - so[k])
        moved = np.abs(so[k] - st[k]) if n else d
        assert np.all(d <= tol * max(float(np.max(moved, initial=0.0)), 1e-300) + 4 * np.spacing(L)), k
    if n == 2 and overlap:
        assert sg["x"][0] < 4.0 and sg["x"][1] > 5.5  # pushed apart
        assert sg["x"][0] - 4.0 == pytest.approx(-(sg["x"][1] - 5.5), rel=1e-6)
    if n == 1:
        assert sg["x"][0] == 4.0
    assert g.total_volume() == pytest.approx(o.total_volume(), rel=1e-10 if precision == 1 else 1e-12,
                                             abs=1e-300)
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_with_degenerate_foams(precision):
    normal = workloads.foam(2000, 2, 0.9, seed=11, precision=precision, use_graph=1)
    items = [tiny(0, 2, precision=precision, graph=1), tiny(1, 2, precision=precision, graph=1),
             normal, tiny(2, 2, precision=precision, graph=1)]
    batch = cb.GpuFoamBatch([c for c, _ in items])
    for (cfg, st), bf in zip(items, batch.foams):
        bf.load_state(st)
        workloads.prepare(bf)
    alone = cb.GpuFoam(normal[0])
    alone.load_state(normal[1])
    workloads.prepare(alone)
    reps = batch.integrate(10)
    ra = alone.integrate(10)
    assert [r["count"] for r in reps] == [0, 1, 2000, 2]
    assert all(r["status"] == 0 for r in reps)
    for k in ("steps", "attempts", "searches", "count", "num_pairs"):
        assert reps[2][k] == ra[k], k
    s_b, s_a = batch.foams[2].get_state(), alone.get_state()
    tol = 1e-6 if precision else 1e-12
    assert np.max(np.abs(s_b["r"] - s_a["r"])) <= tol * np.max(np.abs(s_a["r"]))
    alone.close()
    batch.close()
