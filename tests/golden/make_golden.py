"""Generates the golden vectors of tests/golden/ by running the REFERENCE's own
device code (KJLankinen/cubble src/kernels.cu, compiled unmodified by
oracle/ref/build_ref.py into oracle/_ref/kernels_ref.cubin) on a GB300,
through the driver-API harness of oracle/ref/harness.py.

It restates only the host glue of src/simulator.cu that the kernels need
(launch shapes, the CUB scans as host prefix sums, the pointer rotations) and
records, for seeded foams (2D, 3D, a wall in x, a wall in z, box flow in 2D
and 3D, and the 2D N = 10^4 configuration):

  search   wrapOverPeriodicBoundaries -> cellByPosition -> scan ->
           indexByCell -> reorganizeByIndex -> neighborSearch
           (src/simulator.cu:60-163): the pair set keyed by bubble index and
           the wrapped positions;
  attempt  initGlobals -> preIntegrate -> pairwiseInteraction ->
           postIntegrate (src/simulator.cu:192-210) on a given pair list:
           corrected positions and radii, new velocities, error, pathNew,
           overlap areas, the global sums, the block maxima, the deletion set;
  boot     the Euler bootstrap of the AB2 history (src/simulator.cu:744-787);
  delete   an attempt whose bubbles fall below minRad, the rotation of
           integrate() and removeBubbles() (swapDataCountPairs,
           addVolumeFixPairs) with the deletion list in ascending order;
  energy   potentialEnergy (src/kernels.cu:941-957).
With --init it writes init_2d.npz / init_3d.npz instead: init()'s
assignDataToBubbles on seeded draws and transformPositions both ways.

Run on a GB300 (torch provides the device buffers, ctypes the CUDA driver API):
    python tests/golden/make_golden.py [--init] [--only=NAME,...] OUT_DIR
(OUT_DIR is required; --only records just the named cases). The .npz files
it writes are committed under tests/golden/.
"""
import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.ref.harness import (BLOCK, CUBIN, DROWS, GRID, IROWS, Constants,  # noqa: E402,F401
                                Driver, DVec, Foam, IVec, load)


# ------------------------------------------------------------------ flows
def ref_search(drv, cfg, st):
    """searchNeighbors() (src/simulator.cu:60-163) up to the unsorted pairs."""
    n = len(st["x"])
    f = Foam(drv, cfg, n, 64 * n + 64)
    load(f, st)
    drv.launch("wrapOverPeriodicBoundaries", [f.bubbles()])
    iv = np.array([cfg.tfr[a] - cfg.lbb[a] for a in range(3)])
    max_r = float(np.max(st["r"]))
    cd = np.floor(iv / (2 * (max_r + cfg.skin_radius))).astype(int)
    cd[2] = cd[2] if cd[2] > 0 else 1
    ncell = int(cd[0] * cd[1] * cd[2])
    t = drv.torch
    cell_idx = t.zeros(n, dtype=t.int32, device="cuda")
    sizes = t.zeros(ncell, dtype=t.int32, device="cuda")
    drv.launch("cellByPosition", [C.c_void_p(cell_idx.data_ptr()), C.c_void_p(sizes.data_ptr()),
                                  IVec(*cd.tolist()), f.bubbles()])
    drv.sync()
    offsets = t.cumsum(sizes, 0, dtype=t.int32)  # CUB InclusiveSum, :90-91
    bidx = t.zeros(n, dtype=t.int32, device="cuda")
    off_work = offsets.clone()
    drv.launch("indexByCell", [C.c_void_p(cell_idx.data_ptr()), C.c_void_p(off_work.data_ptr()),
                               C.c_void_p(bidx.data_ptr()), C.c_int32(n)])
    drv.launch("reorganizeByIndex", [f.bubbles(), C.c_void_p(bidx.data_ptr())])
    drv.sync()
    # host pointer rotation, src/simulator.cu:99-146
    for a, b in (("xp", "x"), ("yp", "y"), ("zp", "z"), ("rp", "r"), ("dxdtp", "dxdt"),
                 ("dydtp", "dydt"), ("dzdtp", "dzdt"), ("drdtp", "drdt")):
        f.swap(a, b)
    d = f.d
    sw = d["error"]
    d["error"], d["path"], d["drdto"], d["dzdto"], d["dydto"], d["dxdto"], d["flowVx"] = \
        d["path"], d["drdto"], d["dzdto"], d["dydto"], d["dxdto"], d["flowVx"], sw
    ii = f.i
    swi = ii["index"]
    ii["index"], ii["wrapCountZ"], ii["wrapCountY"], ii["wrapCountX"], ii["numNeighbors"] = \
        ii["wrapCountZ"], ii["wrapCountY"], ii["wrapCountX"], ii["numNeighbors"], swi
    drv.set_global("dNumPairs", C.c_int32(0))
    # offsets after indexByCell hold the cell starts (atomicSub down to them)
    hist = t.zeros(n, dtype=t.int32, device="cuda")
    ncs = 14 if cfg.dimensionality == 3 else 5
    drv.launch("neighborSearch", [C.c_int32(ncell), C.c_int32(ncs), IVec(*cd.tolist()),
                                  C.c_void_p(off_work.data_ptr()), C.c_void_p(sizes.data_ptr()),
                                  C.c_void_p(hist.data_ptr()), C.c_void_p(f.pi.data_ptr()),
                                  C.c_void_p(f.pj.data_ptr()), f.bubbles()])
    npairs = drv.get_global("dNumPairs", C.c_int32)
    index = f.get("index")
    pi = f.pi[:npairs].cpu().numpy()
    pj = f.pj[:npairs].cpu().numpy()
    a, b = index[pi], index[pj]
    pairs = np.stack([np.minimum(a, b), np.maximum(a, b)], 1)
    pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
    order = np.argsort(index)
    wrapped = {k: f.get(k)[order] for k in ("x", "y", "z")}
    wc = {k: f.get(k)[order] for k in ("wrapCountX", "wrapCountY", "wrapCountZ")}
    return pairs, wrapped, wc, cd


def ref_attempt(drv, cfg, st, pi, pj, ts, gas=True, flow=False, path=True):
    """step() kernels (src/simulator.cu:197-210) on the given pair list."""
    n = len(st["x"])
    f = Foam(drv, cfg, n, max(len(pi), 1))
    load(f, st)
    f.set_pairs(pi, pj)
    return f, attempt_on(drv, cfg, f, ts, gas, flow, path)


def attempt_on(drv, cfg, f, ts, gas, flow, path):
    dim = cfg.dimensionality
    t = drv.torch
    tbd = t.zeros(2 * f.stride, dtype=t.int32, device="cuda")
    f.tbd = tbd
    drv.launch("initGlobals", [])
    drv.launch("preIntegrate", [C.c_double(ts), C.c_bool(gas), f.bubbles(),
                                C.c_void_p(f.tempD1.data_ptr())])
    smem = (dim + 4 * int(gas) + dim * int(flow)) * BLOCK * 8
    drv.launch("pairwiseInteraction", [f.bubbles(), f.pairs(), C.c_void_p(f.tempD1.data_ptr()),
                                       C.c_bool(gas), C.c_bool(flow)], smem)
    drv.launch("postIntegrate", [C.c_double(ts), C.c_bool(gas), C.c_bool(path), C.c_bool(flow),
                                 f.bubbles(), C.c_void_p(f.blockMax.data_ptr()),
                                 C.c_void_p(f.tempD1.data_ptr()), C.c_void_p(tbd.data_ptr())])
    drv.sync()
    out = {k: f.get(k) for k in ("xp", "yp", "zp", "rp", "dxdtp", "dydtp", "dzdtp", "drdtp",
                                 "error", "pathNew")}
    out["overlap"] = f.tempD1[:f.n].cpu().numpy()
    for g in ("TotalArea", "TotalAreaPerRadius", "TotalOverlapArea",
              "TotalOverlapAreaPerRadius", "TotalVolumeNew"):
        out[g] = np.array(drv.get_global("d" + g, C.c_double))
    ntbd = drv.get_global("dNumToBeDeleted", C.c_int32)
    out["to_be_deleted"] = np.sort(tbd[:ntbd].cpu().numpy()) if gas else np.zeros(0, np.int32)
    bm = f.blockMax.cpu().numpy()
    nb = min(max(1, math.ceil(f.n / BLOCK)), GRID)
    out["max_error"] = np.array(bm[:nb].max())
    out["max_radius"] = np.array(bm[GRID:GRID + nb].max())
    out["max_expansion"] = np.array(bm[2 * GRID:2 * GRID + nb].max())
    return out


def ref_bootstrap(drv, cfg, st, pi, pj, ts):
    """init()'s Euler bootstrap (src/simulator.cu:727-787): returns dxdto.."""
    n = len(st["x"])
    f = Foam(drv, cfg, n, max(len(pi), 1))
    load(f, st)
    f.set_pairs(pi, pj)
    for k in ("x", "y", "z", "r"):
        f.d[k[0] + "p" if k != "r" else "rp"].copy_(f.d[k])
    for k in ("dxdto", "dydto", "dzdto", "drdto", "dxdtp", "dydtp", "dzdtp", "drdtp", "path"):
        f.d[k].zero_()
    smem = cfg.dimensionality * BLOCK * 8
    args = lambda: [f.bubbles(), f.pairs(), C.c_void_p(f.tempD1.data_ptr()),  # noqa: E731
                    C.c_bool(False), C.c_bool(False)]
    drv.launch("pairwiseInteraction", args(), smem)
    drv.launch("euler", [C.c_double(ts), f.bubbles()])
    for a, b in (("dxdto", "dxdtp"), ("dydto", "dydtp"), ("dzdto", "dzdtp")):
        f.swap(a, b)
    drv.launch("pairwiseInteraction", args(), smem)
    drv.sync()
    for a, b in (("dxdto", "dxdtp"), ("dydto", "dydtp"), ("dzdto", "dzdtp")):
        f.swap(a, b)
    return {k: f.get(k) for k in ("dxdto", "dydto", "dzdto")}


def ref_delete(drv, cfg, st, pi, pj, ts, flow=False):
    """An accepted attempt with deletions: rotation of integrate()
    (src/simulator.cu:258-301) then removeBubbles() with the deletion list
    in ascending order."""
    n = len(st["x"])
    f, out = ref_attempt(drv, cfg, st, pi, pj, ts, flow=flow)
    for a, b in (("x", "xp"), ("y", "yp"), ("z", "zp"), ("r", "rp"), ("path", "pathNew")):
        f.swap(a, b)
    for ax in ("x", "y", "z", "r"):
        o, c, p = "d%sdto" % ax, "d%sdt" % ax, "d%sdtp" % ax
        f.d[o], f.d[c], f.d[p] = f.d[c], f.d[p], f.d[o]
    tbd = out["to_be_deleted"].astype(np.int32)
    D = len(tbd)
    f.tbd[:D].copy_(drv.torch.from_numpy(tbd))
    drv.launch("swapDataCountPairs", [f.bubbles(), f.pairs(), C.c_void_p(f.tbd.data_ptr())])
    drv.launch("addVolumeFixPairs", [f.bubbles(), f.pairs(), C.c_void_p(f.tbd.data_ptr())])
    drv.sync()
    nn = n - D
    npairs = drv.get_global("dNumPairs", C.c_int32)
    res = {k: f.get(k, nn) for k in ("x", "y", "z", "r", "dxdt", "dydt", "dzdt", "drdt",
                                      "dxdto", "path", "error", "savedR")}
    res["index"] = f.get("index", nn)
    pi2 = f.pi[:npairs].cpu().numpy()
    pj2 = f.pj[:npairs].cpu().numpy()
    a, b = res["index"][pi2], res["index"][pj2]
    pr = np.stack([np.minimum(a, b), np.maximum(a, b)], 1)
    res["pairs"] = pr[np.lexsort((pr[:, 1], pr[:, 0]))]
    res["to_be_deleted"] = tbd
    return res


def ref_energy(drv, cfg, st, pi, pj):
    n = len(st["x"])
    f = Foam(drv, cfg, n, max(len(pi), 1))
    load(f, st)
    f.set_pairs(pi, pj)
    f.tempD1.zero_()
    drv.launch("potentialEnergy", [f.bubbles(), f.pairs(), C.c_void_p(f.tempD1.data_ptr())])
    drv.sync()
    return f.tempD1[:n].cpu().numpy()


def ref_init(drv, dim, seed):
    """assignDataToBubbles (src/kernels.cu:1026-1071) on seeded uniform and
    normal draws for a lattice box, then transformPositions
    (src/kernels.cu:971-990) to [0, 1] and back into a rescaled box."""
    from cubble_gb300 import workloads
    rng = np.random.default_rng(seed)
    bpd = (23, 19, 7 if dim == 3 else 1)
    n = bpd[0] * bpd[1] * bpd[2]
    avg_rad = 1.0
    side = [2.0 * avg_rad * bpd[a] if a < dim else 0.0 for a in range(3)]
    cfg, _ = workloads.foam(4, dim, 0.9, seed=1)
    cfg.lbb[0] = cfg.lbb[1] = cfg.lbb[2] = 0.0
    for a in range(3):
        cfg.tfr[a] = side[a]
    cfg.min_rad = 0.1 * avg_rad
    data = {"bpd": np.array(bpd, np.int32), "avg_rad": np.array(avg_rad),
            "lbb": np.zeros(3), "tfr": np.array(side), "min_rad": np.array(cfg.min_rad)}
    draws = {"ux": rng.random(n), "uy": rng.random(n), "uz": rng.random(n) * (dim == 3),
             "uw": rng.random(n), "nr": rng.normal(avg_rad, 0.21, n)}
    draws["nr"][:5] = [-0.4, 0.05, -0.02, 0.0999, 0.1001]  # negative and small radii
    data.update({"in_" + k: v for k, v in draws.items()})
    f = Foam(drv, cfg, n, 64)
    f.put("x", draws["ux"])
    f.put("y", draws["uy"])
    f.put("z", draws["uz"])
    f.put("rp", draws["uw"])
    f.put("r", draws["nr"])
    drv.launch("assignDataToBubbles", [IVec(*bpd), C.c_double(avg_rad), f.bubbles()])
    drv.sync()
    for k in ("x", "y", "z", "r", "rp", "index"):
        data["out_" + k] = f.get(k)
    # box rescale: to [0, 1], new box, back (src/simulator.cu:793-833)
    drv.launch("transformPositions", [C.c_bool(True), f.bubbles()])
    drv.sync()
    for k in ("x", "y", "z"):
        data["norm_" + k] = f.get(k)
    new_tfr = [0.9 * side[0], 1.1 * side[1], 0.95 * side[2] if dim == 3 else 0.0]
    cfg2, _ = workloads.foam(4, dim, 0.9, seed=1)
    for a in range(3):
        cfg2.lbb[a] = 0.0
        cfg2.tfr[a] = new_tfr[a]
    g = Foam(drv, cfg2, n, 64)
    for k in ("x", "y", "z"):
        g.put(k, data["norm_" + k])
    drv.launch("transformPositions", [C.c_bool(False), g.bubbles()])
    drv.sync()
    data["new_tfr"] = np.array(new_tfr)
    for k in ("x", "y", "z"):
        data["back_" + k] = g.get(k)
    return data


# ------------------------------------------------------------------ cases
def flow_box(cfg, frac_lo, frac_hi, vel):
    """Sets the imposed-flow region to the fraction [frac_lo, frac_hi] of the
    box on every axis of the foam and its velocity to `vel` (already scaled
    by f0/mu0, as after src/simulator.cu:569-570)."""
    dim = cfg.dimensionality
    lo, hi = [0.0, 0.0, 0.0], [0.0, 0.0, 0.0]
    for a in range(dim):
        L = cfg.tfr[a] - cfg.lbb[a]
        lo[a] = cfg.lbb[a] + frac_lo[a] * L
        hi[a] = cfg.lbb[a] + frac_hi[a] * L
    cfg.use_flow = 1
    for a in range(3):
        cfg.flow_lbb[a], cfg.flow_tfr[a] = lo[a], hi[a]
        cfg.flow_vel[a] = vel[a] if a < dim else 0.0
    return cfg


def cases():
    """(name, (config, state)) of every recorded foam. The flow cases run the
    reference's box flow: pairwiseInteraction's neighbour-velocity sums
    (src/kernels.cu:191-208, :281-283) and addFlowVelocity
    (src/kernels.cu:497-544) in every attempt and in the deletion step."""
    from cubble_gb300 import workloads
    out = []
    out.append(("2d", workloads.foam(1200, 2, 0.9, seed=501, min_rad=0.05)))
    out.append(("3d", workloads.foam(1500, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=502)))
    out.append(("2d_wallx", workloads.foam(1000, 2, 0.85, seed=503, wall=(1, 0, 0),
                                           wall_drag=0.2)))
    out.append(("3d_wallz", workloads.foam(1200, 3, 0.8, seed=504, wall=(0, 0, 1),
                                           wall_drag=0.1)))
    cfg, st = workloads.foam(1200, 2, 0.9, seed=505, min_rad=0.05)
    out.append(("2d_flow", (flow_box(cfg, (0.0, 0.3, 0.0), (1.0, 0.6, 0.0),
                                     (0.02, -0.005, 0.0)), st)))
    cfg, st = workloads.foam(1500, 3, 0.8, rstd=0.15, rclip=(0.3, 2.5), seed=506)
    out.append(("3d_flow", (flow_box(cfg, (0.2, 0.0, 0.4), (0.7, 1.0, 0.8),
                                     (0.01, 0.004, -0.003)), st)))
    # the 2D configuration at its stated size: N = 10^4, phi 0.90, min_rad 0.05
    out.append(("2d_c1", workloads.config_c1(seed=507)))
    return out


def oracle_pairs(cfg, st):
    from oracle.oracle import OracleFoam
    o = OracleFoam(cfg)
    o.load_state(st)
    o.search_neighbors()
    s = o.get_state()
    i, j = o.pairs()
    return s, i, j


def main(out_dir, only=None):
    os.makedirs(out_dir, exist_ok=True)
    drv = Driver(CUBIN)
    for name, (cfg, st) in cases():
        if only and name not in only:
            continue
        flow = bool(cfg.use_flow)
        rng = np.random.default_rng(7)
        n = len(st["x"])
        data = {"cfg_" + f: np.array(getattr(cfg, f)) for f, _ in type(cfg)._fields_}
        # 1. search on the raw (unwrapped) positions, shifted by up to a box length
        st_s = dict(st)
        for a, k in enumerate(("x", "y", "z")):
            if a < cfg.dimensionality and not cfg.wall[a]:
                L = cfg.tfr[a] - cfg.lbb[a]
                # only bubbles well inside the box move out by one box length,
                # so the reference's wrap lands strictly inside [lbb, tfr)
                inner = (st[k] > cfg.lbb[a] + 0.01 * L) & (st[k] < cfg.tfr[a] - 0.01 * L)
                sh = rng.integers(-1, 2, n) * L * ((rng.random(n) < 0.05) & inner)
                st_s[k] = st[k] + sh
        pairs, wrapped, wc, cd = ref_search(drv, cfg, st_s)
        for k in ("x", "y", "z", "r"):
            data["search_in_" + k] = st_s[k]
        data["search_pairs"] = pairs
        for k, v in list(wrapped.items()) + list(wc.items()):
            data["search_out_" + k] = v
        data["search_ref_cell_dims"] = cd
        # 2. an attempt from a searched, bootstrapped, moving state
        s, pi, pj = oracle_pairs(cfg, st)
        ts = 1e-3
        st_a = {k: s[k] for k in ("x", "y", "z", "r", "saved_x", "saved_y", "saved_z", "saved_r",
                                   "index", "num_neighbors")}
        for k in ("dxdt", "dydt", "dzdt", "dxdto", "dydto", "dzdto"):
            st_a[k] = rng.normal(0.0, 0.05, n) * (k[1] != "z" or cfg.dimensionality == 3)
        st_a["drdt"] = rng.normal(0.0, 0.01, n)
        st_a["drdto"] = rng.normal(0.0, 0.01, n)
        st_a["path"] = rng.random(n)
        st_a["error"] = rng.random(n) * 1e-6
        for k, v in st_a.items():
            data["attempt_in_" + k] = v
        data["attempt_pi"], data["attempt_pj"] = pi, pj
        data["attempt_ts"] = np.array(ts)
        _, out = ref_attempt(drv, cfg, st_a, pi, pj, ts, flow=flow)
        for k, v in out.items():
            data["attempt_out_" + k] = v
        # 3. bootstrap
        bo = ref_bootstrap(drv, cfg, st_a, pi, pj, 1e-4)
        data["boot_ts"] = np.array(1e-4)
        for k, v in bo.items():
            data["boot_out_" + k] = v
        # 4. energy
        data["energy_out"] = ref_energy(drv, cfg, st_a, pi, pj)
        # 5. deletion: shrink a few bubbles below minRad
        st_d = dict(st_a)
        r = st_d["r"].copy()
        doomed = rng.choice(n, size=max(3, n // 100), replace=False)
        r[doomed] = 0.5 * cfg.min_rad
        st_d["r"] = r
        st_d["saved_r"] = r
        st_d["drdt"] = np.zeros(n)
        st_d["drdto"] = np.zeros(n)
        st_d["error"] = np.zeros(n)
        for k, v in st_d.items():
            data["delete_in_" + k] = v
        res = ref_delete(drv, cfg, st_d, pi, pj, 1e-5, flow=flow)
        for k, v in res.items():
            data["delete_out_" + k] = v
        path = os.path.join(out_dir, "ref_%s.npz" % name)
        np.savez_compressed(path, **data)
        print("wrote", path, "pairs", len(pairs), "deleted", len(res["to_be_deleted"]))


def main_init(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    drv = Driver(CUBIN)
    for dim in (2, 3):
        path = os.path.join(out_dir, "init_%dd.npz" % dim)
        np.savez_compressed(path, **ref_init(drv, dim, 600 + dim))
        print("wrote", path)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if len(args) != 1:
        raise SystemExit("usage: make_golden.py [--init] [--only=NAME,...] OUT_DIR")
    out = args[0]
    only = None
    for a in sys.argv[1:]:
        if a.startswith("--only="):
            only = set(a[len("--only="):].split(","))
    if "--init" in sys.argv:
        main_init(out)
    else:
        main(out, only)
