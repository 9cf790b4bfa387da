"""Times the REFERENCE's own step() kernels on a GB300 next to this library's
two forms, on the same state. Test infrastructure: it runs the reference's
unmodified device code (KJLankinen/cubble src/kernels.cu, compiled by
oracle/ref/build_ref.py into oracle/_ref/kernels_ref.cubin) through the
harness of make_golden.py; nothing of the library's product path uses it.

State: the 3D periodic N = 10^6 foam of bench.py (phi 0.80, r ~ N(1, 0.15) in
[0.3, 2.5]) after this library's search, bootstrap and 3 accepted steps,
loaded into the reference's Bubbles / Pairs layout with the same pair list
and dt. One reference attempt is step() without the accept
(src/simulator.cu:197-221): initGlobals, preIntegrate, pairwiseInteraction,
postIntegrate at the reference's launch shape (5120 x 384), then the copy of
dNumToBeDeleted and of the 3 x 5120 block maxima to the host that step()
makes every time. Attempts repeat from the same state (no accept), timed
with CUDA events after 3 warm-up attempts; this library's attempts are timed
the same way (cb_profile_kernels: predict + pairs + correct, no accept).

    python tests/golden/time_reference_step.py [attempts] [c2|c1]

prints one JSON line. c1 is the 2D periodic N = 10^4 foam of the CPU-runnable
configuration, prepared the same way.
"""
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import make_golden as mg  # noqa: E402


def main(reps, wl="c2"):
    import torch
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    cb.build()
    make = workloads.config_c1 if wl == "c1" else workloads.config_c2
    cfg, st = make()
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    workloads.prepare(g)
    g.integrate(3)
    s = g.get_state()
    pi, pj = g.pairs()
    dt = g.report()["time_step"]
    ours64 = g.profile_kernels(reps=reps)
    g.close()
    cfg_m, _ = make(precision=1)
    m = cb.GpuFoam(cfg_m)
    m.load_state(s)
    m.set_pairs(pi, pj)
    m.set_time(dt)
    oursmx = m.profile_kernels(reps=reps)
    m.close()

    drv = mg.Driver(mg.CUBIN)
    n = len(s["x"])
    f = mg.Foam(drv, cfg, n, len(pi) + 64)
    mg.load(f, s)
    f.set_pairs(pi, pj)
    tbd = torch.zeros(2 * f.stride, dtype=torch.int32, device="cuda")
    dim = cfg.dimensionality
    smem = (dim + 4) * mg.BLOCK * 8  # gas exchange on, flow off
    host_max = np.zeros(3 * mg.GRID)

    def attempt(copies):
        drv.launch("initGlobals", [])
        drv.launch("preIntegrate", [C.c_double(dt), C.c_bool(True), f.bubbles(),
                                    C.c_void_p(f.tempD1.data_ptr())])
        drv.launch("pairwiseInteraction", [f.bubbles(), f.pairs(),
                                           C.c_void_p(f.tempD1.data_ptr()), C.c_bool(True),
                                           C.c_bool(False)], smem)
        drv.launch("postIntegrate", [C.c_double(dt), C.c_bool(True), C.c_bool(True),
                                     C.c_bool(False), f.bubbles(),
                                     C.c_void_p(f.blockMax.data_ptr()),
                                     C.c_void_p(f.tempD1.data_ptr()),
                                     C.c_void_p(tbd.data_ptr())])
        if copies:  # step()'s two host copies (src/simulator.cu:212-221)
            drv.get_global("dNumToBeDeleted", C.c_int32)
            drv._ok(drv.cu.cuMemcpyDtoH_v2(host_max.ctypes.data_as(C.c_void_p),
                                           C.c_uint64(f.blockMax.data_ptr()),
                                           C.c_size_t(host_max.nbytes)), "DtoH")

    def timed(copies):
        for _ in range(3):
            attempt(copies)
        drv.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            attempt(copies)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    ref_kernels = timed(False)
    ref_step = timed(True)
    line = {
        "what": ("one step() attempt of the %s foam, same state and pair list"
                 % ("2D periodic N=1e4" if wl == "c1" else "3D periodic N=1e6")),
        "bubbles": n, "pairs": int(len(pi)), "attempts_timed": reps,
        "reference_cuda_ms_per_attempt": ref_step,
        "reference_cuda_kernels_only_ms_per_attempt": ref_kernels,
        "gb300_fp64_ms_per_attempt": float(sum(ours64)),
        "gb300_fp64_kernel_ms": dict(zip(("predict", "pairs", "correct"), ours64)),
        "gb300_mixed_ms_per_attempt": float(sum(oursmx)),
        "gb300_mixed_kernel_ms": dict(zip(("predict", "pairs", "correct"), oursmx)),
        "speedup_fp64_vs_reference": ref_step / float(sum(ours64)),
        "speedup_mixed_vs_reference": ref_step / float(sum(oursmx)),
        "note": "the mixed form's predict is skipped after accepted steps; its sum here "
                "includes a full predict (the profile does not accept)",
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 20, sys.argv[2] if len(sys.argv) > 2 else "c2")
