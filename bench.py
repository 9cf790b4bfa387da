"""Benchmark: accepted bubble-steps per second of the Durian foam step.

Default workload: 3D periodic foam, N = 1,000,000, FP64, phi = 0.80,
r ~ Normal(1, 0.15) clipped to [0.3, 2.5], kappa = 0.01, K = 0.1,
tolerance 1e-5 (seeded synthetic input, uniform positions). One "step" is
one accepted integrate() step (rejected attempts, neighbour searches and
deletions inside it are part of its cost).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the reference's path on the host cores: the
reference has no CPU implementation, so this is the FP64 OpenMP restatement
(oracle/) with all host threads, on the same workload.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
METRIC = "bubble-steps/s at 1 GB300, 3D N=1e6: FP64 vs mixed/batched at stated error; HBM %"


def workload(name, seed, precision=0, use_graph=1):
    from cubble_gb300 import workloads
    if name == "c2":
        cfg, st = workloads.config_c2(seed=seed, precision=precision, use_graph=use_graph)
        desc = ("3D periodic foam N=1e6, phi=0.80, r~N(1,0.15) in [0.3,2.5], kappa=0.01, "
                "K=0.1, tol 1e-5")
    elif name == "c1":
        cfg, st = workloads.config_c1(seed=seed, precision=precision, use_graph=use_graph)
        desc = "2D periodic foam N=1e4, phi=0.90, r~N(1,0.1) in [0.3,2.0], kappa=0.01, K=0.1, tol 1e-5"
    elif name.startswith("c5"):
        # "c5" is N=1e7; "c5:<n>" the same foam at another size
        n = int(float(name.split(":")[1])) if ":" in name else 10_000_000
        cfg, st = workloads.config_c5(seed=seed, n=n, precision=1, use_graph=use_graph)
        desc = ("3D foam N=%d, walls in z, periodic x/y, linear shear along x (max speed "
                "0.05), phi=0.80, r~N(1,0.15) in [0.3,2.5], kappa=0.01, K=0.1, tol 1e-5, "
                "mixed" % n)
    else:
        raise SystemExit("unknown workload " + name)
    return cfg, st, desc


def run_until_deleted(args):
    """The large sheared foam run until a fraction of its bubbles is gone:
    device time, bubble-steps/s over the whole run (searches and every
    compaction included), the device memory it holds, progress samples."""
    import torch
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    torch.cuda.set_device(0)
    cb.build()
    cfg, st, desc = workload(args.workload, args.seed, precision=1, use_graph=1)
    n0 = len(st["x"])
    free0, total = torch.cuda.mem_get_info()
    sim = cb.GpuFoam(cfg)
    sim.load_state(st)
    free1, _ = torch.cuda.mem_get_info()
    workloads.prepare(sim)
    target = int(n0 * (1.0 - args.until_deleted))
    r0 = sim.report()
    samples, dev_ms = [], 0.0
    t0 = time.perf_counter()
    r = r0
    while r["count"] > target and r["steps"] - r0["steps"] < args.max_run_steps:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        r = sim.integrate_until(args.chunk_steps, min_count=target)
        ev1.record()
        torch.cuda.synchronize()
        dev_ms += ev0.elapsed_time(ev1)
        samples.append({"steps": r["steps"] - r0["steps"], "count": r["count"],
                        "searches": r["searches"] - r0["searches"],
                        "time": r["time_integer"] + r["time_fraction"],
                        "wall_s": time.perf_counter() - t0})
    bs = r["bubble_steps"] - r0["bubble_steps"]
    line = {"metric": "bubble-steps/s, large sheared foam run to %.0f%% deleted"
                      % (100 * args.until_deleted),
            "value": bs / (dev_ms / 1e3), "unit": "bubble-steps/s", "workload": desc,
            "bubbles_start": n0, "bubbles_end": r["count"],
            "reached_target": r["count"] <= target,
            "steps": r["steps"] - r0["steps"], "attempts": r["attempts"] - r0["attempts"],
            "searches": r["searches"] - r0["searches"], "deleted": r["deleted"] - r0["deleted"],
            "device_s": dev_ms / 1e3, "device_bytes_held": int(free0 - free1),
            "device_total_bytes": int(total), "samples": samples[-20:]}
    sim.close()
    print(json.dumps(line))


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for ln in f:
                parts = [p.strip() for p in ln.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce(x, op, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def algorithmic_bytes(dim, np_per_n, mixed=False, ff=False):
    """Algorithmic HBM bytes per bubble of each attempt kernel.

    FP64 form, 3D: predict reads x,y,z,r, v x4, v_old x4 (96) and writes the
    packed prediction + 1/r (40); pairs reads the pair indices (8 P/N), the
    prediction once (40) and writes the accumulators once (40); correct reads
    accumulators (40), prediction (32), x (32), v (32), saved (32), path (8),
    error (8) and writes x' (32), v' (32), path' (8), error (8), clears the
    accumulators (40). The whole step's compulsory traffic is 224 + 8 P/N.
    Mixed form (FP32 rates, 32-byte fixed-point prediction, 20-byte FP32
    accumulators), 3D: predict 64 + 32, pairs 8 P/N + 32 + 20, correct
    132 + 88; step 176 + 8 P/N (q FP64 r/w 64, f FP32 r/w 32, f_old 16,
    saved 32, path 16, error 16). The float-float form (CB_PRECISION_FP64_FF)
    adds its 32-byte per-bubble records: written by predict, read by pairs
    (which reads them instead of the 16-byte (1/r, r^2) row in 3D); the
    step's compulsory traffic is the FP64 form's."""
    if ff:
        b = algorithmic_bytes(dim, np_per_n)
        b["predict"] += 32.0
        b["pairs"] += 32.0 - (16.0 if dim == 3 else 0.0)
        return b
    if mixed:
        if dim == 3:
            return {"predict": 96.0, "pairs": 52.0 + 8.0 * np_per_n, "correct": 220.0,
                    "step": 176.0 + 8.0 * np_per_n}
        return {"predict": 80.0, "pairs": 48.0 + 8.0 * np_per_n, "correct": 176.0,
                "step": 136.0 + 8.0 * np_per_n}
    if dim == 3:
        return {"predict": 136.0, "pairs": 80.0 + 8.0 * np_per_n, "correct": 304.0,
                "step": 224.0 + 8.0 * np_per_n}
    return {"predict": 104.0, "pairs": 64.0 + 8.0 * np_per_n, "correct": 272.0,
            "step": 176.0 + 8.0 * np_per_n}


def profiled_traffic(kernel_name):
    """DRAM bytes per launch of `kernel_name` from the committed ncu summaries
    in profiles/ (lines "- `name`: traffic_bytes=N"), or None."""
    import glob
    import re
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        with open(path) as f:
            for ln in f:
                m = re.match(r"- `(.+)`: traffic_bytes=(\d+)", ln.strip())
                if m and m.group(1) == kernel_name:
                    return int(m.group(2)), os.path.relpath(path, ROOT)
    return None


def profiled_metric(kernel_name, label):
    """A value of the committed ncu summary tables in profiles/ (rows
    "| label | v1 | v2 |" under a header "| metric | kernel1 | kernel2 |"), or
    None."""
    import glob
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        cols = None
        with open(path) as f:
            for ln in f:
                cells = [c.strip() for c in ln.strip().strip("|").split("|")]
                if len(cells) > 1 and cells[0] == "metric":
                    cols = cells[1:]
                elif cols and len(cells) == len(cols) + 1 and cells[0] == label:
                    if kernel_name in cols:
                        try:
                            return float(cells[1 + cols.index(kernel_name)].split()[0]), \
                                os.path.relpath(path, ROOT)
                        except ValueError:
                            return None
    return None


def state_bytes(st):
    return int(sum(np.asarray(v).nbytes for v in st.values()))


def pinned_copy(st):
    """Host copy of the state in pinned (page-locked) memory."""
    import torch
    out = {}
    for k, v in st.items():
        v = np.ascontiguousarray(v)
        t = torch.empty(v.shape, dtype=torch.from_numpy(v[:1]).dtype, pin_memory=True)
        a = t.numpy()
        a[...] = v
        out[k] = (a, t)
    return {k: a for k, (a, _) in out.items()}, [t for _, t in out.values()]


def cpu_baseline(cfg, st, steps):
    from oracle.oracle import OracleFoam
    from cubble_gb300 import workloads
    threads = os.cpu_count() or 1
    f = OracleFoam(cfg, threads=threads)
    f.load_state(st)
    workloads.prepare(f)
    f.integrate(1)
    r0 = f.report()
    t0 = time.perf_counter()
    f.integrate(steps)
    dt = time.perf_counter() - t0
    r1 = f.report()
    bs = r1["bubble_steps"] - r0["bubble_steps"]
    return bs / dt, threads, steps, dt


def run_reference(args, world, rank):
    if rank != 0:
        return
    cfg, st, desc = workload(args.workload, args.seed)
    from oracle.oracle import OracleFoam
    from cubble_gb300 import workloads
    threads = os.cpu_count() or 1
    f = OracleFoam(cfg, threads=threads)
    f.load_state(st)
    workloads.prepare(f)
    f.integrate(args.warmup)
    r0 = f.report()
    steps = args.steps if args.ref_steps is None else min(args.steps, args.ref_steps)
    t0 = time.perf_counter()
    f.integrate(steps)
    el = time.perf_counter() - t0
    r1 = f.report()
    bs = r1["bubble_steps"] - r0["bubble_steps"]
    value = bs / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "bubble-steps/s",
        "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / max(steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, uniform positions)",
        "config": {"workload": desc, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "bubble-steps/s", "cores": threads,
                         "kind": "port",
                         "sample": "%d accepted steps of the full workload after %d warm-up "
                                   "steps (the reference has no CPU path; FP64 OpenMP "
                                   "restatement)" % (steps, args.warmup)},
        "e2e": {"value": value, "unit": "bubble-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "attempts": r1["attempts"] - r0["attempts"],
        "searches": r1["searches"] - r0["searches"],
    }
    print(json.dumps(line))


def measure_form(args, world, rank, precision, clocks_on=True):
    """Times K accepted steps of one form; returns its numbers."""
    import torch
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    cfg, st, desc = workload(args.workload, args.seed + rank, precision=precision,
                             use_graph=args.graph)
    dim = cfg.dimensionality
    sim = cb.GpuFoam(cfg)
    sim.load_state(st)
    workloads.prepare(sim)
    # launch and search knobs picked by the autotuner on the prepared foam
    # (kept for the later contexts of this kind in the process)
    tuning = sim.autotune(3) if args.autotune else sim.tuning()
    sim.integrate(args.warmup)
    r0 = sim.report()
    l0 = sim.launch_count()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    barrier(world)
    torch.cuda.synchronize()
    if clocks_on:
        clocks.start()
    r1, dev_ms = sim.integrate_timed(args.steps)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop() if clocks_on else None
    launches = sim.launch_count() - l0
    bs = r1["bubble_steps"] - r0["bubble_steps"]
    el = allreduce(dev_ms / 1e3, _op("max"), world)
    bs_all = allreduce(bs, _op("sum"), world)
    np_per_n = r1["num_pairs"] / max(r1["count"], 1)
    kms = sim.profile_kernels(reps=5)
    # the steady-state rate with its searches: a longer run continuing from
    # the timed steps (integrate() searches when the largest expansion since
    # the last search reaches half the skin), and the device time of one
    # search of the current state
    amort = None
    if args.amortised_steps > 0:
        qa0 = sim.report()
        qa1, ams = sim.integrate_timed(args.amortised_steps)
        na = qa1["steps"] - qa0["steps"]
        sa = qa1["searches"] - qa0["searches"]
        amort = {"value": (qa1["bubble_steps"] - qa0["bubble_steps"]) / (ams / 1e3),
                 "unit": "bubble-steps/s", "steps": na, "ms_per_step": ams / max(na, 1),
                 "attempts": qa1["attempts"] - qa0["attempts"], "searches": sa,
                 "deleted": qa1["deleted"] - qa0["deleted"],
                 "steps_per_search": (na / sa) if sa else None,
                 "what": "%d accepted steps after the timed ones, searches and deletions "
                         "included, one graph launch, CUDA events" % na}
    search_ms = sim.profile_search(reps=3)
    names = ["predict", "pairs", "correct"]
    top = int(np.argmax(kms))
    mixed = precision == 1
    ab = algorithmic_bytes(dim, np_per_n, mixed=mixed, ff=precision == 2)
    n_now = r1["count"]
    hbm, src = peaks()
    achieved = ab[names[top]] * n_now / (kms[top] * 1e-3) / 1e9
    # the whole step (searches, rejects, deletions and the skipped predict
    # of a speculated prediction included): algorithmic bytes x measured rate
    step_gbs = ab["step"] * (bs_all / el) / 1e9
    gas, flow = int(cfg.use_gas_exchange), int(cfg.use_flow)
    sfx = "_mx" if mixed else ""
    walls = int(any(cfg.wall[:dim]))
    kcorr = ("k_correct_mx<%d, %d, %d, %d>" % (dim, gas, flow, walls) if mixed
             else "k_correct<%d>" % dim)
    kpairs = "k_pairs%s<%d, %d, %d>" % (sfx if mixed else ("_ff" if precision == 2 else ""),
                                        dim, gas, flow)
    if mixed:  # the mixed pair kernel's pairs per thread (a template argument)
        run = tuning["pair_run"] if (gas and not flow) else 4
        kpairs = "k_pairs_mx<%d, %d, %d, %d>" % (dim, gas, flow, run)
    kname = {"predict": "k_predict%s<%d>" % (sfx, dim), "correct": kcorr,
             "pairs": kpairs}[names[top]]
    tr = profiled_traffic(kname)
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm,
            "unit": "GB/s", "frac": achieved / hbm,
            "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": tr[0] if tr else None,
            "traffic_source": ("%s (ncu dram__bytes_read.sum + dram__bytes_write.sum of %s)"
                               % (tr[1], kname)) if tr else None,
            "algorithmic_bytes_per_launch": ab[names[top]] * n_now,
            "kernel_ms": dict(zip(names, kms)),
            "algorithmic_bytes_per_bubble": ab,
            "step_achieved_gbs": step_gbs, "step_frac": step_gbs / hbm}
    fp64 = profiled_metric(kname, "FP64 pipe % active")
    if fp64 and precision == 0:
        # the FP64 form is bound by FP64 issue (2 FP64 thread-instructions per
        # SM and cycle on GB300), not by HBM: the ncu pipe utilisation says how
        # close the dominant kernel is to that bound
        roof["fp64_issue_bound"] = {"pipe_active_frac": fp64[0] / 100.0,
                                    "source": "%s (ncu sm__pipe_fp64_cycles_active of %s)"
                                              % (fp64[1], kname)}
    sim.close()
    return {"value": bs_all / el, "el": el, "cfg": cfg, "st": st, "desc": desc, "r0": r0,
            "r1": r1, "roofline": roof, "launches": launches, "clocks": clk,
            "np_per_n": np_per_n, "amortised": amort, "search_ms": search_ms,
            "tuning": tuning}


def form_errors(args, precision=1, steps=50):
    """Per-quantity error of another form (mixed, or the float-float FP64
    form) against the FP64 form (which matches the FP64 oracle within 1e-12
    per step) from the same prepared state: one attempt, then `steps`
    accepted steps."""
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    cfg64, st, _ = workload(args.workload, args.seed, precision=0, use_graph=1)
    cfgmx, _, _ = workload(args.workload, args.seed, precision=precision, use_graph=1)
    a = cb.GpuFoam(cfg64)
    a.load_state(st)
    workloads.prepare(a)
    a.integrate(args.warmup)
    s0 = a.get_state()
    i, j = a.pairs()
    b = cb.GpuFoam(cfgmx)
    b.load_state(s0)
    b.set_pairs(i, j)
    dt = a.report()["time_step"]
    b.set_time(dt)

    def rel(x, y):
        return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))
    def ulps(x, y):  # largest difference in units in the last place of y
        return float(np.max(np.abs(x - y) / np.spacing(np.maximum(np.abs(y), 1e-300))))
    aa, ab_ = a.attempt(), b.attempt()
    out = {"attempt": {}}
    for k, base in (("xp", "x"), ("yp", "y"), ("zp", "z"), ("rp", "r")):
        out["attempt"]["d" + base] = rel(ab_[k] - s0[base], aa[k] - s0[base])
        out["attempt"][base + "_ulps"] = ulps(ab_[k], aa[k])
    for k in ("dxdtp", "dydtp", "dzdtp", "drdtp", "overlap"):
        out["attempt"][k] = rel(ab_[k], aa[k])
    for k in ("total_area", "total_overlap_area", "total_overlap_area_per_radius"):
        out["attempt"][k] = abs(ab_[k] / aa[k] - 1.0)
    out["attempt"]["max_error"] = abs(ab_["max_error"] / aa["max_error"] - 1.0)
    a.set_time(dt)
    b.set_time(dt)
    v0 = a.total_volume()
    ra0, rb0 = a.report(), b.report()
    ra, rb = a.integrate(steps), b.integrate(steps)
    sa, sb = a.get_state(), b.get_state()
    oa_, ob_ = np.argsort(sa["index"]), np.argsort(sb["index"])
    o0 = np.argsort(s0["index"])
    traj = {"steps": steps,
            "same_attempts_searches_deletions": all(
                ra[k] - ra0[k] == rb[k] - rb0[k] for k in ("attempts", "searches", "deleted"))}
    for k in ("x", "y", "z"):
        traj["d" + k] = rel(sb[k][ob_] - s0[k][o0], sa[k][oa_] - s0[k][o0])
        traj[k + "_ulps"] = ulps(sb[k][ob_], sa[k][oa_])
    traj["r"] = rel(sb["r"][ob_], sa["r"][oa_])
    traj["volume_drift"] = abs(b.total_volume() / a.total_volume() - 1.0)
    traj["volume_change_fp64"] = a.total_volume() / v0 - 1.0
    traj["energy"] = abs(b.energy() / a.energy() - 1.0)
    out["trajectory"] = traj
    out["reference"] = "the FP64 form of this library on the same input (equal to the FP64 oracle within 1e-12 per step)"
    out["error_definition"] = ("max over bubbles |form - fp64| / max |fp64| per row (positions, "
                               "radii: their change over the attempt or the run, which can be "
                               "a few 1e-6 at small dt); *_ulps: the largest difference in "
                               "units in the last place of the FP64 value")
    a.close()
    b.close()
    return out


def _attempt_errors(ga, gb, s, tol):
    """Largest per-row error of attempt `gb` against attempt `ga` from state
    `s`: positions and radii by their change over the attempt, rates and
    overlap areas by each row's largest magnitude, the error estimate
    relative to the tolerance it is compared with."""
    def rel(x, y):
        return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))
    e = {}
    for k, base in (("xp", "x"), ("yp", "y"), ("zp", "z"), ("rp", "r")):
        e["d" + base] = rel(gb[k] - s[base], ga[k] - s[base])
    for k in ("dxdtp", "dydtp", "dzdtp", "drdtp", "overlap", "path_new"):
        e[k] = rel(gb[k], ga[k])
    e["max_error_vs_tol"] = abs(gb["max_error"] - ga["max_error"]) / tol
    e["max_error_rel"] = abs(gb["max_error"] / ga["max_error"] - 1.0)
    return e


def long_horizon_errors(args, steps, every):
    """The mixed form against the FP64 form over `steps` accepted steps from
    the same prepared state (the survey's C3 beside C2). Every `every`
    steps: both runs' energies (the energy-decay curve), the mixed run's
    total gas volume against the FP64 run's, and the mixed form's per-step
    error measured on the FP64 run's own state (one attempt of each form
    from that state, `_attempt_errors`)."""
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    cfg64, st, _ = workload(args.workload, args.seed, precision=0, use_graph=1)
    cfgmx, _, _ = workload(args.workload, args.seed, precision=1, use_graph=1)
    a = cb.GpuFoam(cfg64)
    a.load_state(st)
    workloads.prepare(a)
    a.integrate(args.warmup)
    s0 = a.get_state()
    i0, j0 = a.pairs()
    dt = a.report()["time_step"]
    b = cb.GpuFoam(cfgmx)
    b.load_state(s0)
    b.set_pairs(i0, j0)
    b.set_time(dt)
    a.set_time(dt)
    p64, pmx = cb.GpuFoam(cfg64), cb.GpuFoam(cfgmx)
    tol = cfg64.error_tolerance
    v0 = a.total_volume()
    ra0, rb0 = a.report(), b.report()
    curve, worst = [], {}
    done = 0
    part = None  # first sample where the two runs' attempt / deletion counts differ
    while True:
        sa = a.get_state()
        ia, ja = a.pairs()
        q = a.report()
        for f in (p64, pmx):
            f.load_state(sa)
            f.set_pairs(ia, ja)
            f.set_time(q["time_step"])
        err = _attempt_errors(p64.attempt(), pmx.attempt(), sa, tol)
        for k, v in err.items():
            worst[k] = max(worst.get(k, 0.0), v)
        ea, eb = a.energy(), b.energy()
        qa, qb = a.report(), b.report()
        same = all(qa[k] - ra0[k] == qb[k] - rb0[k] for k in ("attempts", "deleted"))
        if not same and part is None:
            part = done
        curve.append({"step": done, "same_counts": same,
                      "energy_fp64": ea, "energy_mixed": eb,
                      "energy_rel": abs(eb / ea - 1.0),
                      "volume_drift": abs(b.total_volume() / a.total_volume() - 1.0),
                      "per_step_max": max(v for k, v in err.items()
                                          if k not in ("max_error_rel", "max_error_vs_tol")),
                      "error_estimate_vs_tol": err["max_error_vs_tol"]})
        if done >= steps:
            break
        a.integrate(every)
        b.integrate(every)
        done += every
    ra, rb = a.report(), b.report()
    out = {"steps": done, "sample_every": every,
           "same_attempts_searches_deletions": all(
               ra[k] - ra0[k] == rb[k] - rb0[k] for k in ("attempts", "searches", "deleted")),
           "counts_fp64": {k: ra[k] - ra0[k] for k in ("attempts", "searches", "deleted")},
           "counts_mixed": {k: rb[k] - rb0[k] for k in ("attempts", "searches", "deleted")},
           "counts_part_by_step": part,
           "note": "once an accept / reject or deletion decision near its threshold goes "
                   "the other way, the two runs reach a step count at different times, and "
                   "the energies of later samples compare different moments of a relaxing "
                   "foam; the per-step error is measured on the FP64 run's own state and "
                   "is unaffected",
           "volume_drift": abs(b.total_volume() / a.total_volume() - 1.0),
           "volume_change_fp64": a.total_volume() / v0 - 1.0,
           "energy_rel_end": curve[-1]["energy_rel"],
           "per_step_worst": worst, "curve": curve,
           "reference": "the FP64 form of this library (equal to the FP64 oracle within "
                        "1e-12 per step) on the same input",
           "error_definition": "per step: one attempt of each form from the FP64 run's state "
                               "every sample; max over bubbles |mixed - fp64| / max |fp64| per "
                               "row (positions, radii: their change over the attempt; "
                               "per_step_max: the largest row); the error estimate relative to "
                               "the tolerance (max_error_vs_tol, error_estimate_vs_tol) and to "
                               "itself (max_error_rel, a difference of nearly equal FP32 rates)"}
    for f in (a, b, p64, pmx):
        f.close()
    return out


def batch_errors(items, steps=50):
    """Mixed batch against the FP64 batch of the same foams from the same
    FP64-prepared state (positions, rates, pairs, dt): max over foams of the
    displacement-relative position error, the radius error and the total
    volume drift after `steps` accepted steps. Over thousands of steps the
    two runs of a chaotic foam part (a deletion may land a step apart), so
    positions and radii are compared on the bubbles both runs still hold;
    the total gas volume is what stays comparable."""
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    cf64 = [c for c, _ in items]
    cfmx = [workloads.sweep_config_as(c, precision=1) for c in cf64]
    b64, bmx = cb.GpuFoamBatch(cf64), cb.GpuFoamBatch(cfmx)
    s0 = []
    for (cfg, st), f64, fmx in zip(items, b64.foams, bmx.foams):
        f64.load_state(st)
        workloads.prepare(f64)
        s = f64.get_state()
        i, j = f64.pairs()
        fmx.load_state(s)
        fmx.set_pairs(i, j)
        fmx.set_time(f64.report()["time_step"])
        s0.append(s)
    r64, rmx = b64.integrate(steps), bmx.integrate(steps)
    out = {"steps": steps, "foams": len(items), "same_attempts_searches_deletions": True,
           "foams_with_same_counts": 0, "dx": 0.0, "r": 0.0, "volume_drift": 0.0,
           "volume_vs_target_fp64": 0.0, "volume_vs_target_mixed": 0.0,
           "deleted_fp64": 0, "deleted_mixed": 0,
           "note": "volume_drift compares the two runs; volume_vs_target_* is each run's own "
                   "total gas volume against pi M^2, the value every deletion's volume fix "
                   "restores (src/kernels.cu:859-867): the AM2 update keeps it to first order "
                   "in dt only, so both runs drift between deletions, and runs whose "
                   "deletions fall on different steps differ by that drift"}
    for f, ((cfg, _), f64, fmx) in enumerate(zip(items, b64.foams, bmx.foams)):
        same = all(r64[f][k] == rmx[f][k] for k in ("attempts", "searches", "deleted"))
        out["same_attempts_searches_deletions"] &= same
        out["foams_with_same_counts"] += int(same)
        out["deleted_fp64"] += r64[f]["deleted"]
        out["deleted_mixed"] += rmx[f]["deleted"]
        a, b = f64.get_state(), fmx.get_state()
        common = np.intersect1d(a["index"], b["index"])
        pa = np.argsort(a["index"])[np.searchsorted(np.sort(a["index"]), common)]
        pb = np.argsort(b["index"])[np.searchsorted(np.sort(b["index"]), common)]
        p0 = np.argsort(s0[f]["index"])[np.searchsorted(np.sort(s0[f]["index"]), common)]
        for ax, k in enumerate(("x", "y")):
            L = cfg.tfr[ax] - cfg.lbb[ax]
            d = b[k][pb] - a[k][pa]
            d -= L * np.round(d / L)
            m = a[k][pa] - s0[f][k][p0]
            m -= L * np.round(m / L)
            out["dx"] = max(out["dx"], float(np.max(np.abs(d)) / max(np.max(np.abs(m)), 1e-300)))
        out["r"] = max(out["r"], float(np.max(np.abs(b["r"][pb] - a["r"][pa])) /
                                        np.max(np.abs(a["r"]))))
        v64, vmx = f64.total_volume(), fmx.total_volume()
        out["volume_drift"] = max(out["volume_drift"], abs(vmx - v64) / v64)
        vt = math.pi * cfg.bubble_volume_multiplier ** 2
        out["volume_vs_target_fp64"] = max(out["volume_vs_target_fp64"], abs(v64 / vt - 1.0))
        out["volume_vs_target_mixed"] = max(out["volume_vs_target_mixed"], abs(vmx / vt - 1.0))
    b64.close()
    bmx.close()
    return out


def measure_batch(args, world, rank):
    """The batched parameter sweep: `--batch-count` independent 2D periodic
    foams (N log-uniform in [1e3, 1e5], phi in [0.85, 0.95], kappa
    log-uniform in [1e-3, 1e-1]) in the mixed form, all advanced by one
    graph launch per call, tile picked by the autotuner."""
    import torch
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    items = workloads.sweep(count=args.batch_count, seed=4 + 1000 * rank, precision=1,
                            use_graph=args.batch_graph)
    t0 = time.perf_counter()
    batch = cb.GpuFoamBatch([c for c, _ in items])
    for (cfg, st), f in zip(items, batch.foams):
        f.load_state(st)
        workloads.prepare(f)
    setup_s = time.perf_counter() - t0
    tile = batch.autotune(args.batch_tune_steps)
    tuning = batch.foams[0].tuning()
    batch.integrate(args.warmup)
    r0 = [f.report() for f in batch.foams]
    l0 = batch.launch_count()
    barrier(world)
    torch.cuda.synchronize()
    reps, ms = batch.integrate_timed(args.batch_steps)
    torch.cuda.synchronize()
    barrier(world)
    launches = batch.launch_count() - l0
    bs = sum(r["bubble_steps"] - q["bubble_steps"] for r, q in zip(reps, r0))
    el = allreduce(ms / 1e3, _op("max"), world)
    bs_all = allreduce(bs, _op("sum"), world)
    n_now = sum(r["count"] for r in reps)
    np_now = sum(r["num_pairs"] for r in reps)
    ab = algorithmic_bytes(2, np_now / max(n_now, 1), mixed=True)
    value = bs_all / el
    hbm, src = peaks()
    achieved = ab["step"] * bs / (ms / 1e3) / 1e9
    out = {"value": value, "unit": "bubble-steps/s",
           "ms_per_batch_step": ms / args.batch_steps,
           "foams": len(items), "bubbles": int(sum(st["x"].size for _, st in items)),
           "steps_each": args.batch_steps, "tile_bubbles_per_block": tile,
           "tuning": tuning,
           "attempts": sum(r["attempts"] - q["attempts"] for r, q in zip(reps, r0)),
           "searches": sum(r["searches"] - q["searches"] for r, q in zip(reps, r0)),
           "deleted": sum(r["deleted"] - q["deleted"] for r, q in zip(reps, r0)),
           "gpu_launches": launches, "setup_s": setup_s,
           "roofline": {"bound": "hbm", "kernel": "whole batched step",
                        "achieved": achieved, "peak": hbm, "unit": "GB/s",
                        "frac": achieved / hbm,
                        "peak_source": src + " (MEASURED_PEAKS.json hbm_gbs)",
                        "algorithmic_bytes_per_bubble_step": ab["step"]},
           "workload": "%d independent 2D periodic foams, N log-uniform in [1e3, 1e5] "
                       "(seeded), phi U[0.85, 0.95], kappa log-uniform [1e-3, 1e-1], "
                       "r~N(1, 0.1) in [0.3, 2.0], mixed precision, one graph launch, "
                       "autotuned tile" % len(items)}
    batch.close()
    if rank == 0:
        pick = sorted(range(len(items)), key=lambda f: items[f][1]["x"].size)
        sub = [items[f] for f in pick[:: max(1, len(pick) // 4)][:4]]
        sub = [(workloads.sweep_config_as(c, precision=0), st) for c, st in sub]
        out["error_vs_fp64"] = batch_errors(sub, steps=args.batch_error_steps)
    return out


def reference_cuda(args, steps):
    """The reference's own CUDA step loop on the same GB300: KJLankinen/cubble's
    src/kernels.cu compiled unmodified for sm_103a (oracle/ref/build_ref.py),
    driven by oracle/ref/harness.py's restatement of integrate()
    (src/simulator.cu:60-337: per attempt four launches and the blocking
    copy of the block maxima, host dt decision, pointer rotation, searches
    and deletions). It starts from this library's prepared foam (state, pair
    list, dt); this library's FP64 and mixed forms run the same `steps`
    accepted steps from the same state. A reported baseline, never the
    measured path: the harness runs only here and in the golden-vector
    recorder."""
    import torch
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    from oracle.ref import harness
    if not os.path.exists(harness.CUBIN):
        return {"unavailable": "reference cubin oracle/_ref/kernels_ref.cubin not built "
                               "(the reference sources were absent when build() ran)"}
    cfg, st, desc = workload(args.workload, args.seed, precision=0, use_graph=1)
    g = cb.GpuFoam(cfg)
    g.load_state(st)
    workloads.prepare(g)
    g.integrate(args.warmup)
    s = g.get_state()
    pi, pj = g.pairs()
    rep = g.report()
    g.close()
    dt, max_r = rep["time_step"], rep["max_radius"]
    drv = harness.Driver(harness.CUBIN)
    warm = harness.RefSim(drv, cfg, s, pi, pj, dt, max_r)
    warm.integrate(3)  # loads the kernels' code; the timed run starts afresh
    drv.sync()
    del warm
    sim = harness.RefSim(drv, cfg, s, pi, pj, dt, max_r)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    e0.record()
    sim.integrate(steps)
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ref_ms = e0.elapsed_time(e1)
    out = {"value": sim.bubble_steps / (ref_ms / 1e3), "unit": "bubble-steps/s",
           "steps": steps, "ms_per_step": ref_ms / steps, "wall_s": wall,
           "attempts": sim.attempts, "searches": sim.searches, "deleted": sim.deleted,
           "what": "the reference's src/kernels.cu (unmodified, sm_103a) under its own "
                   "integrate() host loop, from the same prepared foam; CUDA events on the "
                   "default stream around the whole loop (host round trips included)"}
    forms = {}
    for prec, name in ((0, "fp64"), (1, "mixed")):
        cfgp, _, _ = workload(args.workload, args.seed, precision=prec, use_graph=1)
        f = cb.GpuFoam(cfgp)
        f.load_state(s)
        f.set_pairs(pi, pj)
        f.set_time(dt)
        q0 = f.report()
        q1, ms = f.integrate_timed(steps)
        forms[name] = {"value": (q1["bubble_steps"] - q0["bubble_steps"]) / (ms / 1e3),
                       "ms_per_step": ms / steps,
                       "attempts": q1["attempts"] - q0["attempts"],
                       "searches": q1["searches"] - q0["searches"],
                       "deleted": q1["deleted"] - q0["deleted"]}
        forms[name]["speedup_vs_reference_cuda"] = forms[name]["value"] / out["value"]
        f.close()
    out["gb300"] = forms
    return out


def measure_sheared(args):
    """A sample of the large sheared foam (3D, N = 1e7, walls in z, linear
    shear along x, mixed form): `--c5-steps` accepted steps after its search,
    bootstrap and warm-up, one graph launch, CUDA events. The run until half
    the bubbles are deleted (`--workload c5 --until-deleted 0.5`) takes
    minutes and is reported from its own runs."""
    import torch
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    n = args.c5_n
    t0 = time.perf_counter()
    cfg, st = workloads.config_c5(n=n, precision=1, use_graph=1)
    free0, _ = torch.cuda.mem_get_info()
    sim = cb.GpuFoam(cfg)
    sim.load_state(st)
    free1, _ = torch.cuda.mem_get_info()
    workloads.prepare(sim)
    sim.integrate(args.warmup)
    setup_s = time.perf_counter() - t0
    r0 = sim.report()
    r1, ms = sim.integrate_timed(args.c5_steps)
    out = {"value": (r1["bubble_steps"] - r0["bubble_steps"]) / (ms / 1e3),
           "unit": "bubble-steps/s", "steps": r1["steps"] - r0["steps"],
           "ms_per_step": ms / max(r1["steps"] - r0["steps"], 1),
           "attempts": r1["attempts"] - r0["attempts"],
           "searches": r1["searches"] - r0["searches"],
           "deleted": r1["deleted"] - r0["deleted"],
           "bubbles_start": n, "bubbles_end": r1["count"],
           "device_bytes_held": int(free0 - free1), "setup_s": setup_s,
           "workload": "3D foam N=%d, walls in z, periodic x/y, linear shear along x (max "
                       "speed 0.05), phi=0.80, r~N(1,0.15) in [0.3,2.5], kappa=0.01, K=0.1, "
                       "tol 1e-5, mixed precision; a %d-step sample of the run to 50%% "
                       "deleted" % (n, args.c5_steps)}
    sim.close()
    return out


def run_gb300(args, world, rank, local):
    import torch
    import cubble_gb300 as cb
    from cubble_gb300 import workloads
    torch.cuda.set_device(local)
    cb.build()
    main = measure_form(args, world, rank, args.precision)
    cfg, st, desc, r0, r1 = main["cfg"], main["st"], main["desc"], main["r0"], main["r1"]
    value, el = main["value"], main["el"]
    attempts = r1["attempts"] - r0["attempts"]
    searches = r1["searches"] - r0["searches"]

    # end to end through the C ABI with pinned host buffers: upload, search +
    # bootstrap, K steps each returning its report to the host, download.
    e2e = None
    if not args.no_e2e:
        host, keep = pinned_copy(st)
        down, keep_down = pinned_copy({k: np.zeros_like(v) for k, v in st.items()})
        g2 = cb.GpuFoam(cfg)
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g2.load_state(host)
        t1 = time.perf_counter()
        workloads.prepare(g2)
        t2 = time.perf_counter()
        q0 = g2.report()
        calls = []
        for _ in range(args.warmup + args.steps):
            tc = time.perf_counter()
            g2.integrate(1)
            calls.append(1e3 * (time.perf_counter() - tc))
        q1 = g2.report()
        t3 = time.perf_counter()
        fin = g2.get_state(rows=list(host.keys()), out=down)
        torch.cuda.synchronize()
        t4 = time.perf_counter()
        e2e_s = t4 - t0
        parts = {"upload_ms": 1e3 * (t1 - t0), "search_bootstrap_ms": 1e3 * (t2 - t1),
                 "steps_ms": 1e3 * (t3 - t2), "download_ms": 1e3 * (t4 - t3),
                 "call_ms_first": calls[:3], "call_ms_median": statistics.median(calls),
                 "attempts": q1["attempts"] - q0["attempts"]}
        barrier(world)
        e2e_s = allreduce(e2e_s, _op("max"), world)
        e2e_bs = allreduce(q1["bubble_steps"] - q0["bubble_steps"], _op("sum"), world)
        nsteps = args.warmup + args.steps
        import ctypes
        rep = ctypes.sizeof(cb._abi.Report)
        e2e = {"value": e2e_bs / e2e_s, "unit": "bubble-steps/s",
               "h2d_bytes_per_step": state_bytes(host) // nsteps,
               "d2h_bytes_per_step": rep + state_bytes(fin) // nsteps,
               "steps": nsteps, "host_wall_ms": parts,
               "note": "state upload, search, bootstrap, %d steps each reading "
                       "its report back, state download (pinned host buffers)" % nsteps}
        g2.close()
        del keep, keep_down

    mixed = None
    if args.precision == 0 and not args.no_mixed:
        mx = measure_form(args, world, rank, 1, clocks_on=False)
        mixed = {"value": mx["value"], "unit": "bubble-steps/s",
                 "ms_per_step": 1e3 * mx["el"] / args.steps,
                 "speedup_vs_fp64": mx["value"] / value,
                 "attempts": mx["r1"]["attempts"] - mx["r0"]["attempts"],
                 "searches": mx["r1"]["searches"] - mx["r0"]["searches"],
                 "roofline": mx["roofline"], "gpu_launches": mx["launches"],
                 "tuning": mx["tuning"],
                 "workload": "same foam, mixed precision: FP32 pair geometry on exact 64-bit "
                             "fixed-point differences, FP32 rates; FP64 positions, radii, "
                             "volume sum and fix, error norm, energy"}
        if rank == 0:
            mixed["error_vs_fp64"] = form_errors(args, 1)
            if args.long_steps > 0:
                mixed["long_horizon_vs_fp64"] = long_horizon_errors(args, args.long_steps,
                                                                    args.long_every)
        mixed["amortised"] = mx["amortised"]
        mixed["search_ms"] = mx["search_ms"]

    fp64_ff = None
    if args.precision == 0 and not args.no_ff:
        fx = measure_form(args, world, rank, 2, clocks_on=False)
        fp64_ff = {"value": fx["value"], "unit": "bubble-steps/s",
                   "ms_per_step": 1e3 * fx["el"] / args.steps,
                   "speedup_vs_fp64": fx["value"] / value,
                   "attempts": fx["r1"]["attempts"] - fx["r0"]["attempts"],
                   "searches": fx["r1"]["searches"] - fx["r0"]["searches"],
                   "roofline": fx["roofline"], "gpu_launches": fx["launches"],
                   "dtype": "f64 state and update; pair terms in float-float (2 x f32)",
                   "workload": "same foam, CB_PRECISION_FP64_FF: the FP64 form with the pair "
                               "kernel's distance, velocities, gas flux and overlap areas in "
                               "float-float (~2^-46 relative) on the FP32 pipe"}
        if rank == 0:
            fp64_ff["error_vs_fp64"] = form_errors(args, 2)

    batched = None
    if not args.no_batch:
        batched = measure_batch(args, world, rank)

    sheared = None
    if args.c5_steps > 0:
        sheared = measure_sheared(args)

    ref_cuda = None
    if rank == 0 and args.ref_cuda_steps > 0:
        try:
            ref_cuda = reference_cuda(args, args.ref_cuda_steps)
        except Exception as e:  # the baseline is reported, never required
            ref_cuda = {"unavailable": "%s: %s" % (type(e).__name__, e)}

    base = None
    if rank == 0 and not args.no_cpu:
        v, cores, n_steps, secs = cpu_baseline(cfg, st, args.cpu_steps)
        base = {"value": v, "unit": "bubble-steps/s", "cores": cores, "kind": "port",
                "sample": "%d accepted steps of the same workload after its first step "
                          "(%.1f s, FP64 OpenMP restatement of the reference step)" % (n_steps, secs)}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "bubble-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {0: "f64", 1: "f64/f32 mixed", 2: "f64 + float-float (2 x f32) pair terms"}[
            args.precision],
        "data": "synthetic (seeded, uniform positions)",
        "config": {"workload": desc,
                   "precision": {0: "fp64", 1: "mixed", 2: "fp64_ff"}[args.precision],
                   "graph": bool(args.graph), "parallelism": "replicas" if world > 1 else "single foam",
                   "l2": "working set larger than L2 (state + pairs > 129 MB)",
                   "attempts": attempts, "searches": searches,
                   "steps_per_search": (args.steps / searches) if searches else None,
                   "pairs_per_bubble": main["np_per_n"], "bubbles_end": r1["count"],
                   "tuning": main["tuning"],
                   "deleted": r1["deleted"] - r0["deleted"], "dt_end": r1["time_step"]},
        "search": {"search_ms": main["search_ms"],
                   "what": "device time of one neighbour search of the N-bubble foam "
                           "(CUDA events, mean of 3)"},
        "amortised": main["amortised"], "reference_cuda": ref_cuda,
        "roofline": main["roofline"], "cpu_baseline": base, "e2e": e2e,
        "gpu_launches": main["launches"], "clocks": main["clocks"], "mixed": mixed,
        "fp64_ff": fp64_ff, "batched": batched, "sheared": sheared,
    }
    print(json.dumps(line))


def _op(name):
    try:
        import torch.distributed as dist
        return {"max": dist.ReduceOp.MAX, "sum": dist.ReduceOp.SUM}[name]
    except Exception:
        return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--graph", type=int, default=1)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--cpu-steps", type=int, default=30)
    ap.add_argument("--ref-steps", type=int, default=200)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-ff", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    # accepted steps of the search-inclusive run after the timed ones (0: off)
    ap.add_argument("--amortised-steps", type=int, default=500)
    # accepted steps of the reference's CUDA step loop and of both forms from
    # the same state (0: off)
    ap.add_argument("--ref-cuda-steps", type=int, default=200)
    # the mixed form against the FP64 form over this many steps (0: off),
    # sampled every --long-every steps; the batched sweep's mixed-vs-FP64
    # drift over --batch-error-steps steps per foam
    ap.add_argument("--long-steps", type=int, default=2000)
    ap.add_argument("--long-every", type=int, default=100)
    ap.add_argument("--batch-error-steps", type=int, default=5000)
    # 1: the autotuner picks the cb_tuning knobs before the warm-up
    ap.add_argument("--autotune", type=int, default=1)
    # the large sheared foam's sample: bubbles and accepted steps (0: off)
    ap.add_argument("--c5-n", type=int, default=10_000_000)
    ap.add_argument("--c5-steps", type=int, default=1000)
    ap.add_argument("--until-deleted", type=float, default=0.0)
    ap.add_argument("--chunk-steps", type=int, default=2000)
    ap.add_argument("--max-run-steps", type=int, default=200000)
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=5000)  # the sweep runs 5,000 steps per foam
    ap.add_argument("--batch-tune-steps", type=int, default=10)
    # 0: eager batched launches (each batched kernel a separate launch, for
    # a profiler's launch list); the measurement uses the graph
    ap.add_argument("--batch-graph", type=int, default=1)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        # the CPU arm needs no process group: rank 0 works, the others exit
        world = int(os.environ.get("WORLD_SIZE", "1"))
        run_reference(args, world, int(os.environ.get("RANK", "0")))
        return
    if args.until_deleted > 0.0:
        run_until_deleted(args)
        return
    world, rank, local = dist_setup()
    run_gb300(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
