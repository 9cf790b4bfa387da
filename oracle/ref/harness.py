"""TEST INFRASTRUCTURE and reference timing: runs the REFERENCE's own device code.

KJLankinen/cubble's src/kernels.cu, compiled unmodified by
oracle/ref/build_ref.py into oracle/_ref/kernels_ref.cubin, is loaded on the
GPU through the CUDA driver API (ctypes on libcuda). This module restates
only the reference's host glue around those kernels: its device layout
(`Bubbles`, `Pairs`, `Constants`, src/data_definitions.h:41-225), its launch
shape (5120 x 384, src/data_definitions.h:28-29), the CUB scans as prefix
sums and the host pointer rotations of src/simulator.cu.

Two users, neither of them the product:
  * tests/golden/make_golden.py records golden vectors from single kernels;
  * bench.py's `reference_cuda` baseline leg times `RefSim`, the reference's
    whole integrate() loop (src/simulator.cu:60-337) on the same foam as the
    library's forms.
Nothing in cubble_gb300/ imports it.
"""
import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

CUBIN = os.path.join(ROOT, "oracle", "_ref", "kernels_ref.cubin")
BLOCK, GRID = 384, 5120  # src/data_definitions.h:28-29

DROWS = ["x", "y", "z", "r", "xp", "yp", "zp", "rp", "dxdt", "dydt", "dzdt", "drdt",
         "dxdtp", "dydtp", "dzdtp", "drdtp", "dxdto", "dydto", "dzdto", "drdto",
         "path", "pathNew", "error", "flowVx", "flowVy", "flowVz",
         "savedX", "savedY", "savedZ", "savedR"]
IROWS = ["wrapCountX", "wrapCountY", "wrapCountZ", "index", "numNeighbors"]


class Bubbles(C.Structure):  # src/data_definitions.h:41-153
    _fields_ = ([(n, C.c_void_p) for n in DROWS] + [(n, C.c_void_p) for n in IROWS]
                + [("count", C.c_int32), ("stride", C.c_uint64),
                   ("numDP", C.c_uint64), ("numIP", C.c_uint64)])


class Pairs(C.Structure):  # src/data_definitions.h:157-178
    _fields_ = [("i", C.c_void_p), ("j", C.c_void_p), ("count", C.c_int32),
                ("stride", C.c_uint64)]


class DVec(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class IVec(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32)]


class Constants(C.Structure):  # src/data_definitions.h:183-225
    _fields_ = [("lbb", DVec), ("tfr", DVec), ("interval", DVec), ("flowLbb", DVec),
                ("flowTfr", DVec), ("flowVel", DVec),
                ("averageSurfaceAreaIn", C.c_double), ("minRad", C.c_double),
                ("fZeroPerMuZero", C.c_double), ("kParameter", C.c_double),
                ("kappa", C.c_double), ("wallDragStrength", C.c_double),
                ("skinRadius", C.c_double), ("bubbleVolumeMultiplier", C.c_double),
                ("dimensionality", C.c_int32), ("xWall", C.c_bool), ("yWall", C.c_bool),
                ("zWall", C.c_bool)]


class Driver:
    def __init__(self, cubin):
        import torch
        self.torch = torch
        torch.zeros(1, device="cuda")  # primary context current on this thread
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        self._ok(self.cu.cuModuleLoad(C.byref(self.mod), cubin.encode()), "cuModuleLoad")
        cnt = C.c_uint()
        self._ok(self.cu.cuModuleGetFunctionCount(C.byref(cnt), self.mod), "count")
        funcs = (C.c_void_p * cnt.value)()
        self._ok(self.cu.cuModuleEnumerateFunctions(funcs, cnt, self.mod), "enumerate")
        self.funcs = {}
        for f in funcs:
            name = C.c_char_p()
            self._ok(self.cu.cuFuncGetName(C.byref(name), C.c_void_p(f)), "name")
            self.funcs[name.value.decode()] = C.c_void_p(f)

    @staticmethod
    def _ok(rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, rc))

    def func(self, short):
        key = "%d%s" % (len(short), short)
        hits = [n for n in self.funcs if n.startswith("_ZN6cubble" + key)]
        if len(hits) != 1:
            raise KeyError(short)
        return self.funcs[hits[0]]

    def global_ptr(self, short):
        name = "_ZN6cubble%d%sE" % (len(short), short)
        ptr, size = C.c_uint64(), C.c_size_t()
        self._ok(self.cu.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod,
                                              name.encode()), name)
        return ptr.value, size.value

    def get_global(self, short, ctype):
        p, _ = self.global_ptr(short)
        v = ctype()
        self.sync()
        self._ok(self.cu.cuMemcpyDtoH_v2(C.byref(v), C.c_uint64(p), C.sizeof(v)), "DtoH")
        return v.value

    def set_global(self, short, value):
        p, _ = self.global_ptr(short)
        self._ok(self.cu.cuMemcpyHtoD_v2(C.c_uint64(p), C.byref(value), C.sizeof(value)), "HtoD")

    def launch(self, short, args, smem=0):
        params = (C.c_void_p * len(args))(*[C.cast(C.pointer(a), C.c_void_p) for a in args])
        self._ok(self.cu.cuLaunchKernel(self.func(short), GRID, 1, 1, BLOCK, 1, 1, smem, None,
                                        params, None), short)

    def sync(self):
        self._ok(self.cu.cuCtxSynchronize(), "sync")


class Foam:
    """The reference's device state for one foam (Bubbles rows, pairs,
    temporaries), in torch device buffers."""

    def __init__(self, drv, cfg, n, pair_stride):
        t = drv.torch
        self.drv, self.cfg, self.n = drv, cfg, n
        self.stride = n + (32 - n % 32) % 32
        dev = "cuda"
        self.d = {k: t.zeros(self.stride, dtype=t.float64, device=dev) for k in DROWS}
        self.i = {k: t.zeros(self.stride, dtype=t.int32, device=dev) for k in IROWS}
        self.pstride = pair_stride
        self.pi = t.zeros(pair_stride, dtype=t.int32, device=dev)
        self.pj = t.zeros(pair_stride, dtype=t.int32, device=dev)
        self.tmpi = t.zeros(max(self.stride, 1) * 2, dtype=t.int32, device=dev)
        self.tempD1 = t.zeros(self.stride, dtype=t.float64, device=dev)
        self.blockMax = t.zeros(3 * GRID, dtype=t.float64, device=dev)
        self.const = t.zeros(C.sizeof(Constants), dtype=t.uint8, device=dev)
        self.np = 0
        k = Constants()
        dim = cfg.dimensionality
        k.lbb = DVec(*cfg.lbb)
        k.tfr = DVec(*cfg.tfr)
        k.interval = DVec(*[cfg.tfr[a] - cfg.lbb[a] for a in range(3)])
        k.flowLbb = DVec(*cfg.flow_lbb)
        k.flowTfr = DVec(*cfg.flow_tfr)
        k.flowVel = DVec(*cfg.flow_vel)
        k.averageSurfaceAreaIn = cfg.average_surface_area_in
        k.minRad = cfg.min_rad
        k.fZeroPerMuZero = cfg.f0_per_mu0
        k.kParameter = cfg.k_parameter
        k.kappa = cfg.kappa
        k.wallDragStrength = cfg.wall_drag
        k.skinRadius = cfg.skin_radius
        k.bubbleVolumeMultiplier = cfg.bubble_volume_multiplier
        k.dimensionality = dim
        k.xWall, k.yWall, k.zWall = (bool(w) for w in cfg.wall)
        host = t.frombuffer(bytearray(bytes(k)), dtype=t.uint8)
        self.const.copy_(host)
        drv.set_global("dConstants", C.c_uint64(self.const.data_ptr()))
        drv.set_global("dNumPairs", C.c_int32(0))
        drv.launch("initGlobals", [])

    def bubbles(self):
        b = Bubbles()
        for k in DROWS:
            setattr(b, k, self.d[k].data_ptr())
        for k in IROWS:
            setattr(b, k, self.i[k].data_ptr())
        b.count = self.n
        b.stride = self.stride
        b.numDP, b.numIP = 30, 5
        return b

    def pairs(self):
        p = Pairs()
        p.i, p.j = self.pi.data_ptr(), self.pj.data_ptr()
        p.count = self.np
        p.stride = self.pstride
        return p

    def put(self, key, arr):
        t = self.drv.torch
        src = t.from_numpy(np.ascontiguousarray(arr))
        (self.d if key in self.d else self.i)[key][:len(arr)].copy_(src)

    def get(self, key, n=None):
        n = self.n if n is None else n
        return (self.d if key in self.d else self.i)[key][:n].cpu().numpy().copy()

    def set_pairs(self, i, j):
        t = self.drv.torch
        self.pi[:len(i)].copy_(t.from_numpy(np.asarray(i, np.int32)))
        self.pj[:len(j)].copy_(t.from_numpy(np.asarray(j, np.int32)))
        self.np = len(i)
        self.drv.set_global("dNumPairs", C.c_int32(self.np))

    def swap(self, a, b):
        self.d[a], self.d[b] = self.d[b], self.d[a]


def load(f, st):
    for k_ref, k_st in (("x", "x"), ("y", "y"), ("z", "z"), ("r", "r"),
                        ("dxdt", "dxdt"), ("dydt", "dydt"), ("dzdt", "dzdt"), ("drdt", "drdt"),
                        ("dxdto", "dxdto"), ("dydto", "dydto"), ("dzdto", "dzdto"),
                        ("drdto", "drdto"), ("path", "path"), ("error", "error"),
                        ("savedX", "saved_x"), ("savedY", "saved_y"), ("savedZ", "saved_z"),
                        ("savedR", "saved_r")):
        if k_st in st:
            f.put(k_ref, st[k_st])
    for k_ref, k_st in (("index", "index"), ("numNeighbors", "num_neighbors")):
        if k_st in st:
            f.put(k_ref, st[k_st].astype(np.int32))
    f.put("rp", st["r"])  # rp == r before the first step (src/simulator.cu:737-742)




def cell_dims(cfg, max_radius):
    """searchNeighbors()' cell grid (src/simulator.cu:69-75): floor(interval /
    (2 (maxR + skin))) per axis, z = 1 in 2D."""
    iv = np.array([cfg.tfr[a] - cfg.lbb[a] for a in range(3)])
    cd = np.floor(iv / (2 * (max_radius + cfg.skin_radius))).astype(int)
    cd[2] = cd[2] if cd[2] > 0 else 1
    return cd


class RefSim:
    """The reference's step loop on its own kernels, from a given state.

    integrate() (src/simulator.cu:251-337): step() until the error is
    acceptable — initGlobals, preIntegrate, pairwiseInteraction,
    postIntegrate, then the copy of dNumToBeDeleted and the blocking copy of
    the 3 x 5120 block maxima to the host, the host maximum over the used
    blocks and the dt decision (x0.37 on reject, x1.269 when the error is
    below 0.45 tol and dt < 10, :192-249) — then the pointer rotation, the
    two-part clock, removeBubbles() (swapDataCountPairs, addVolumeFixPairs)
    when bubbles fell below minRad and searchNeighbors() (:60-178) when the
    largest expansion reaches half the skin.

    `st` holds the persistent rows (x, y, z, r, velocities, previous
    velocities, path, error, saved_*, index, num_neighbors); (pi, pj) is a
    pair list grouped by i, as sortPairs leaves it; `dt` the next step size.
    Options as integrate() with useGasExchange and incrementPath on and the
    flow of cfg.use_flow."""

    def __init__(self, drv, cfg, st, pi, pj, dt, max_radius, pair_stride=None):
        t = drv.torch
        n = len(st["x"])
        self.drv, self.cfg = drv, cfg
        per = 16 if cfg.dimensionality == 3 else 8
        stride = n + (32 - n % 32) % 32
        self.f = Foam(drv, cfg, n, pair_stride or per * max(stride, 32))
        load(self.f, st)
        self.f.put("rp", st["r"])
        self.f.set_pairs(pi, pj)
        self.dt = float(dt)
        self.max_radius = float(max_radius)
        self.gas, self.path = True, True
        self.flow = bool(cfg.use_flow)
        self.tbd = t.zeros(2 * self.f.stride, dtype=t.int32, device="cuda")
        self.host_max = np.zeros(3 * GRID)
        self.steps = self.attempts = self.searches = self.deleted = 0
        self.bubble_steps = 0
        self.time_integer, self.time_fraction = 0, 0.0

    # ----------------------------------------------------------- step()
    def step(self):
        drv, f, cfg = self.drv, self.f, self.cfg
        dim = cfg.dimensionality
        b = f.bubbles()
        drv.launch("initGlobals", [])
        drv.launch("preIntegrate", [C.c_double(self.dt), C.c_bool(self.gas), b,
                                    C.c_void_p(f.tempD1.data_ptr())])
        smem = (dim + 4 * int(self.gas) + dim * int(self.flow)) * BLOCK * 8
        drv.launch("pairwiseInteraction", [b, f.pairs(), C.c_void_p(f.tempD1.data_ptr()),
                                           C.c_bool(self.gas), C.c_bool(self.flow)], smem)
        drv.launch("postIntegrate", [C.c_double(self.dt), C.c_bool(self.gas),
                                     C.c_bool(self.path), C.c_bool(self.flow), b,
                                     C.c_void_p(f.blockMax.data_ptr()),
                                     C.c_void_p(f.tempD1.data_ptr()),
                                     C.c_void_p(self.tbd.data_ptr())])
        self.attempts += 1
        ntbd = drv.get_global("dNumToBeDeleted", C.c_int32) if self.gas else 0
        drv._ok(drv.cu.cuMemcpyDtoH_v2(self.host_max.ctypes.data_as(C.c_void_p),
                                       C.c_uint64(f.blockMax.data_ptr()),
                                       C.c_size_t(self.host_max.nbytes)), "DtoH")
        nb = 1
        if f.n > BLOCK:
            nb = min(int(math.ceil(np.float32(f.n) / np.float32(BLOCK))), GRID)
        p = self.host_max
        max_error = float(np.max(p[:nb]))
        max_radius = float(np.max(p[GRID:GRID + nb]))
        max_expansion = float(np.max(p[2 * GRID:2 * GRID + nb]))
        tol = self.cfg.error_tolerance
        too_large = max_error > tol
        if too_large:
            self.dt *= 0.37
        elif max_error < 0.45 * tol and self.dt < 10:
            self.dt *= 1.269
        return too_large, ntbd, max_radius, max_expansion

    # ------------------------------------------------------ integrate()
    def integrate(self, n_steps=1):
        f = self.f
        d = f.d
        for _ in range(n_steps):
            while True:
                too_large, ntbd, max_radius, max_expansion = self.step()
                if not too_large:
                    break
            for ax in ("x", "y", "z"):
                o, c, p = "d%sdto" % ax, "d%sdt" % ax, "d%sdtp" % ax
                d[o], d[c], d[p] = d[c], d[p], d[o]
                d[ax], d[ax + "p"] = d[ax + "p"], d[ax]
            if self.gas:
                d["r"], d["rp"] = d["rp"], d["r"]
                d["drdto"], d["drdt"], d["drdtp"] = d["drdt"], d["drdtp"], d["drdto"]
            if self.path:
                d["path"], d["pathNew"] = d["pathNew"], d["path"]
            self.steps += 1
            self.bubble_steps += f.n
            self.time_fraction += self.dt
            whole = int(self.time_fraction)
            self.time_integer += whole
            self.time_fraction -= whole
            if self.gas:
                self.max_radius = max_radius
                if ntbd > 0:
                    self.remove(ntbd)
            if max_expansion >= 0.5 * self.cfg.skin_radius:
                self.search()

    # -------------------------------------------------- removeBubbles()
    def remove(self, ntbd):
        drv, f = self.drv, self.f
        b = f.bubbles()
        drv.launch("swapDataCountPairs", [b, f.pairs(), C.c_void_p(self.tbd.data_ptr())])
        drv.launch("addVolumeFixPairs", [b, f.pairs(), C.c_void_p(self.tbd.data_ptr())])
        f.n -= ntbd
        self.deleted += ntbd

    # ------------------------------------------------- searchNeighbors()
    def search(self):
        drv, f, cfg = self.drv, self.f, self.cfg
        t = drv.torch
        self.searches += 1
        drv.launch("wrapOverPeriodicBoundaries", [f.bubbles()])
        f.pi.zero_()
        f.pj.zero_()
        cd = cell_dims(cfg, self.max_radius)
        ncell = int(cd[0] * cd[1] * cd[2])
        n = f.n
        cell_idx = t.zeros(f.stride, dtype=t.int32, device="cuda")
        sizes = t.zeros(ncell, dtype=t.int32, device="cuda")
        bidx = t.zeros(f.stride, dtype=t.int32, device="cuda")
        hist = t.zeros(f.stride, dtype=t.int32, device="cuda")
        tp1 = t.zeros(f.pstride, dtype=t.int32, device="cuda")
        tp2 = t.zeros(f.pstride, dtype=t.int32, device="cuda")
        ivec = IVec(*[int(v) for v in cd])
        # cellByPosition has no range check (a bubble on the top face would
        # count into the cell past the end): the same IEEE operations here
        # first, and no launch when any index falls outside the grid
        for a, k in enumerate(("x", "y", "z")[:cfg.dimensionality]):
            q = t.floor(float(cd[a]) * (f.d[k][:n] - cfg.lbb[a]) / (cfg.tfr[a] - cfg.lbb[a]))
            if n and (bool((q < 0).any()) or bool((q >= int(cd[a])).any())):
                raise RuntimeError("a bubble lies outside the reference's cell grid on axis "
                                   "%s; its cellByPosition would index past the cells" % k)
        drv.launch("cellByPosition", [C.c_void_p(cell_idx.data_ptr()),
                                      C.c_void_p(sizes.data_ptr()), ivec, f.bubbles()])
        offsets = t.cumsum(sizes, 0, dtype=t.int32)  # CUB InclusiveSum, :90-91
        drv.launch("indexByCell", [C.c_void_p(cell_idx.data_ptr()),
                                   C.c_void_p(offsets.data_ptr()),
                                   C.c_void_p(bidx.data_ptr()), C.c_int32(n)])
        drv.launch("reorganizeByIndex", [f.bubbles(), C.c_void_p(bidx.data_ptr())])
        d, ii = f.d, f.i  # host pointer rotation, src/simulator.cu:99-146
        for a, b in (("xp", "x"), ("yp", "y"), ("zp", "z"), ("rp", "r"), ("dxdtp", "dxdt"),
                     ("dydtp", "dydt"), ("dzdtp", "dzdt"), ("drdtp", "drdt")):
            d[a], d[b] = d[b], d[a]
        sw = d["error"]
        d["error"], d["path"], d["drdto"], d["dzdto"], d["dydto"], d["dxdto"], d["flowVx"] = \
            d["path"], d["drdto"], d["dzdto"], d["dydto"], d["dxdto"], d["flowVx"], sw
        swi = ii["index"]
        ii["index"], ii["wrapCountZ"], ii["wrapCountY"], ii["wrapCountX"], ii["numNeighbors"] = \
            ii["wrapCountZ"], ii["wrapCountY"], ii["wrapCountX"], ii["numNeighbors"], swi
        drv.set_global("dNumPairs", C.c_int32(0))
        ncs = 14 if cfg.dimensionality == 3 else 5
        drv.launch("neighborSearch", [C.c_int32(ncell), C.c_int32(ncs), ivec,
                                      C.c_void_p(offsets.data_ptr()),
                                      C.c_void_p(sizes.data_ptr()),
                                      C.c_void_p(hist.data_ptr()), C.c_void_p(tp1.data_ptr()),
                                      C.c_void_p(tp2.data_ptr()), f.bubbles()])
        f.np = drv.get_global("dNumPairs", C.c_int32)
        nn = ii["numNeighbors"]
        nn[:n].copy_(t.cumsum(hist[:n], 0, dtype=t.int32))  # CUB InclusiveSum, :165-167
        drv.launch("sortPairs", [f.bubbles(), f.pairs(), C.c_void_p(tp1.data_ptr()),
                                 C.c_void_p(tp2.data_ptr())])
        nn[:n].zero_()
        drv.launch("countNumNeighbors", [f.bubbles(), f.pairs()])

    def state(self):
        """The current rows keyed like cb_state_view (in the reference's
        current bubble order)."""
        f = self.f
        out = {k: f.get(k) for k in ("x", "y", "z", "r", "dxdt", "dydt", "dzdt", "drdt",
                                      "dxdto", "dydto", "dzdto", "drdto", "path", "error")}
        out["index"] = f.get("index")
        return out
