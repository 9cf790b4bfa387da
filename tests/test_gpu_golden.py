"""GPU: the CUDA path, through the C ABI, against the golden vectors recorded
from the reference's own kernels (tests/golden/make_golden.py). Same bars as
tests/test_golden.py, which checks the oracle against the same files, except
that rows that are differences of two positions (the predictor-corrector
error, the path) may also differ by 4 ulp of the largest coordinate: the
FP64 form's pair terms agree with the reference's to ~1e-14, not bit for bit,
so a corrected position can differ in its last bit."""
import numpy as np
import pytest

import cubble_gb300 as cb
from helpers import assert_rows_close, position_ulp
from test_golden import FILES, config, ids, load, rel, state

pytestmark = pytest.mark.gpu


def sorted_pairs(s, i, j):
    a, b = s["index"][i], s["index"][j]
    got = np.stack([np.minimum(a, b), np.maximum(a, b)], 1)
    return got[np.lexsort((got[:, 1], got[:, 0]))]


@pytest.mark.parametrize("path", FILES, ids=ids)
def test_gpu_search_matches_reference(path):
    d = load(path)
    g = cb.GpuFoam(config(d))
    g.load_state(state(d, "search_in_"))
    g.search_neighbors()
    s = g.get_state()
    i, j = g.pairs()
    assert np.array_equal(sorted_pairs(s, i, j), d["search_pairs"])
    order = np.argsort(s["index"])
    for k in ("x", "y", "z"):
        assert np.array_equal(s[k][order], d["search_out_" + k]), k


@pytest.mark.parametrize("precision", [0, 2])
@pytest.mark.parametrize("path", FILES, ids=ids)
def test_gpu_attempt_matches_reference(path, precision):
    """Both FP64 forms: plain, and float-float pair terms (precision 2)."""
    d = load(path)
    cfg = config(d, precision=precision)
    g = cb.GpuFoam(cfg)
    g.load_state(state(d, "attempt_in_"))
    g.set_pairs(d["attempt_pi"], d["attempt_pj"])
    g.set_time(float(d["attempt_ts"]))
    out = g.attempt()
    floor = position_ulp(state(d, "attempt_in_"))
    for mine, ref in (("xp", "xp"), ("yp", "yp"), ("zp", "zp"), ("rp", "rp"),
                      ("dxdtp", "dxdtp"), ("dydtp", "dydtp"), ("dzdtp", "dzdtp"),
                      ("drdtp", "drdtp"), ("error", "error"), ("path_new", "pathNew"),
                      ("overlap", "overlap")):
        if cfg.dimensionality == 2 and mine in ("zp", "dzdtp"):
            continue
        assert_rows_close({mine: out[mine]}, {mine: d["attempt_out_" + ref]}, [mine], 1e-12,
                          floor=floor)
    for mine, ref in (("total_area", "TotalArea"), ("total_overlap_area", "TotalOverlapArea"),
                      ("total_overlap_area_per_radius", "TotalOverlapAreaPerRadius"),
                      ("total_volume_new", "TotalVolumeNew"), ("max_radius", "max_radius"),
                      ("max_expansion", "max_expansion")):
        assert out[mine] == pytest.approx(float(d["attempt_out_" + ref]), rel=1e-12), mine
    assert out["max_error"] == pytest.approx(float(d["attempt_out_max_error"]), rel=1e-12,
                                             abs=floor)
    assert np.array_equal(np.flatnonzero(out["delete_flags"]), d["attempt_out_to_be_deleted"])


@pytest.mark.parametrize("path", FILES, ids=ids)
def test_gpu_bootstrap_and_energy_match_reference(path):
    d = load(path)
    cfg = config(d, time_step=float(d["boot_ts"]))
    g = cb.GpuFoam(cfg)
    g.load_state(state(d, "attempt_in_"))
    g.set_pairs(d["attempt_pi"], d["attempt_pj"])
    assert rel(g.bubble_energies(), d["energy_out"]) <= 1e-12
    g.bootstrap()
    s = g.get_state()
    for k in ("dxdto", "dydto") + (("dzdto",) if cfg.dimensionality == 3 else ()):
        assert rel(s[k], d["boot_out_" + k]) <= 1e-12, k


@pytest.mark.parametrize("graph", [0, 1])
@pytest.mark.parametrize("path", FILES, ids=ids)
def test_gpu_deletion_matches_reference(path, graph):
    d = load(path)
    cfg = config(d, error_tolerance=1.0, skin_radius=1e9, time_step=1e-5, use_graph=graph)
    g = cb.GpuFoam(cfg)
    g.load_state(state(d, "delete_in_"))
    g.set_pairs(d["attempt_pi"], d["attempt_pj"])
    rep = g.integrate(1)
    assert rep["deleted"] == len(d["delete_out_to_be_deleted"])
    s = g.get_state()
    assert np.array_equal(s["index"], d["delete_out_index"])
    floor = position_ulp(state(d, "delete_in_"))
    for k, ref in (("x", "x"), ("y", "y"), ("r", "r"), ("dxdt", "dxdt"), ("drdt", "drdt"),
                   ("path", "path"), ("error", "error")):
        assert_rows_close({k: s[k]}, {k: d["delete_out_" + ref]}, [k], 1e-12, floor=floor)
    i, j = g.pairs()
    assert np.array_equal(sorted_pairs(s, i, j), d["delete_out_pairs"])
