"""cb_energy_noalloc: the energy entry point for callers that cannot allocate
device memory (their HBM belongs to their own pool, or allocation is not
allowed where they call from). It must give what cb_energy gives, call after
call, with its scratch in the library's static device array.

This file is collected last so that a failure here comes after every other
test has run."""
import ctypes as C

import numpy as np
import pytest

import cubble_gb300 as cb
from cubble_gb300 import workloads

MAX_BUBBLES = 1 << 18


def _noalloc(cfg, rows, pi, pj, n, npairs, out, stream):
    lib = cb.lib()
    return lib.cb_energy_noalloc(C.byref(cfg), rows[0], rows[1], rows[2], rows[3],
                                 pi, pj, int(n), int(npairs), out, stream)


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [3, 2])
def test_energy_noalloc_matches_energy(dim):
    import torch
    if dim == 3:
        cfg, st = workloads.foam(50000, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=31)
    else:
        cfg, st = workloads.foam(50000, 2, 0.9, seed=32)
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
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    rows = [C.c_void_p(a.data_ptr()) for a in t]
    assert expect > 0
    for call in range(2):  # the array keeps the last call's contents
        out.fill_(-1.0)
        rc = _noalloc(cfg, rows, C.c_void_p(ti.data_ptr()), C.c_void_p(tj.data_ptr()),
                      len(s["x"]), len(i), C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        torch.cuda.synchronize()
        assert rc == 0, cb.lib().cb_last_error()
        got = float(out.item())
        assert got == pytest.approx(expect, rel=1e-12), (call, got, expect)
    g.close()


@pytest.mark.gpu
def test_energy_noalloc_rejects_oversized_input():
    cfg = cb.make_config(dimensionality=3, tfr=(10.0, 10.0, 10.0), capacity=1)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = _noalloc(cfg, [dummy] * 4, dummy, dummy, MAX_BUBBLES + 1, 0, dummy, None)
    assert rc == 3
    assert b"static scratch limit" in cb.lib().cb_last_error()
