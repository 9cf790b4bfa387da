"""cb_energy_noalloc: the energy entry point for callers that cannot allocate
device memory (their HBM belongs to their own pool, or allocation is not
allowed where they call from). It must give what cb_energy gives, call after
call, with its scratch in the library's static device array.

This file is collected last so that a failure here comes after every other
test has run."""
import ctypes as C
import math

import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads

MAX_BUBBLES = 1 << 18


def _noalloc(cfg, rows, pi, pj, n, npairs, out, stream):
    lib = cb.lib()
    return lib.cb_energy_noalloc(C.byref(cfg), rows[0], rows[1], rows[2], rows[3],
                                 pi, pj, int(n), int(npairs), out, stream)


def _case(case):
    if case == "3d":
        return workloads.foam(50000, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=31)
    if case == "2d":
        return workloads.foam(50000, 2, 0.9, seed=32)
    # walls in z: no minimum image on that axis (cfg.wall)
    return workloads.foam(50000, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=33,
                          wall=(0, 0, 1), wall_drag=0.1)


def _device_inputs(case):
    """A searched foam: cb_energy's value, and the rows and pairs copied to
    device tensors that the caller owns."""
    import torch
    cfg, st = _case(case)
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    g.search_neighbors()
    expect = g.energy()  # the existing entry point
    s = g.get_state(rows=["x", "y", "z", "r"])
    i, j = g.pairs()
    dev = torch.device("cuda", torch.cuda.current_device())
    t = [torch.from_numpy(np.ascontiguousarray(s[k])).to(dev) for k in ("x", "y", "z", "r")]
    ti = torch.from_numpy(i).to(dev)
    tj = torch.from_numpy(j).to(dev)
    g.close()
    return cfg, expect, t, ti, tj, len(s["x"])


def _call(cfg, t, ti, tj, n, npairs, out):
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    rows = [C.c_void_p(a.data_ptr()) for a in t]
    rc = _noalloc(cfg, rows, C.c_void_p(ti.data_ptr()), C.c_void_p(tj.data_ptr()),
                  n, npairs, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    assert rc == 0, cb.lib().cb_last_error()
    return float(out.item())


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["3d", "2d", "3d-wallz"])
def test_energy_noalloc_matches_energy(case):
    import torch
    cfg, expect, t, ti, tj, n = _device_inputs(case)
    out = torch.full((1,), -1.0, dtype=torch.float64, device=t[0].device)
    assert expect > 0
    for call in range(2):  # the array keeps the last call's contents
        out.fill_(-1.0)
        got = _call(cfg, t, ti, tj, n, len(ti), out)
        assert got == pytest.approx(expect, rel=1e-12), (call, got, expect)


@pytest.mark.gpu
def test_energy_noalloc_allocates_nothing():
    """After the first call (which may load the library's device code),
    further calls leave the device's free memory unchanged."""
    import torch
    cfg, expect, t, ti, tj, n = _device_inputs("3d")
    out = torch.full((1,), -1.0, dtype=torch.float64, device=t[0].device)
    assert _call(cfg, t, ti, tj, n, len(ti), out) == pytest.approx(expect, rel=1e-12)
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _call(cfg, t, ti, tj, n, len(ti), out) == pytest.approx(expect, rel=1e-12)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


@pytest.mark.gpu
def test_energy_noalloc_rejects_bad_pair_indices():
    """A pair index outside [0, count) is skipped before any load (nothing
    outside the caller's rows or the scratch array is touched) and makes the
    result NaN; the next call with valid pairs is exact again."""
    import torch
    cfg, expect, t, ti, tj, n = _device_inputs("3d")
    out = torch.full((1,), -1.0, dtype=torch.float64, device=t[0].device)
    for bad_i, bad_j in ((0, n), (-1, 1), (n + 5000, 2), (3, 1 << 30)):
        bi = torch.cat([ti, torch.tensor([bad_i], dtype=torch.int32, device=ti.device)])
        bj = torch.cat([tj, torch.tensor([bad_j], dtype=torch.int32, device=tj.device)])
        got = _call(cfg, t, bi, bj, n, len(bi), out)
        assert math.isnan(got), (bad_i, bad_j, got)
        assert _call(cfg, t, ti, tj, n, len(ti), out) == pytest.approx(expect, rel=1e-12)


@pytest.mark.gpu
def test_energy_noalloc_rejects_oversized_input():
    cfg = cb.make_config(dimensionality=3, tfr=(10.0, 10.0, 10.0), capacity=1)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = _noalloc(cfg, [dummy] * 4, dummy, dummy, MAX_BUBBLES + 1, 0, dummy, None)
    assert rc == 3
    assert b"static scratch limit" in cb.lib().cb_last_error()
