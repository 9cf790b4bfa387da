// Host side of the C ABI (include/cubble_gb300.h): the context owns every
// device buffer of one foam, runs the step loop either eagerly (one small
// control-block read per attempt, like the reference's per-step copy at
// src/simulator.cu:219-221) or as a single CUDA graph whose while/if
// conditional nodes are driven by the device (no host round trip per step).
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "context.cuh"

using namespace cbg;

namespace {
thread_local std::string g_err;
}  // namespace

namespace cbg {
int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

const char *status_text(int s) {
    switch (s) {
    case CB_OK: return "ok";
    case CB_ERR_CAPACITY: return "pair capacity exceeded";
    case CB_ERR_MAX_ATTEMPTS: return "reject loop exceeded max_attempts";
    case CB_ERR_NONFINITE: return "non-finite value in the step";
    case CB_ERR_DT_UNDERFLOW: return "time step underflow";
    default: return "device status error";
    }
}

void set_last_error(const std::string &msg) { g_err = msg; }
std::atomic<unsigned long long> g_calls{0};
}  // namespace cbg


namespace {

void fill_const(cb_context *c) {
    DevConst &k = c->hk;
    const cb_config &f = c->cfg;
    k.dim = f.dimensionality;
    for (int a = 0; a < 3; a++) {
        k.wall[a] = f.wall[a] ? 1 : 0;
        k.lbb[a] = f.lbb[a];
        k.tfr[a] = f.tfr[a];
        k.iv[a] = f.tfr[a] - f.lbb[a];
        k.flow_lbb[a] = f.flow_lbb[a];
        k.flow_tfr[a] = f.flow_tfr[a];
        k.flow_vel[a] = f.flow_vel[a];
    }
    k.any_wall = k.wall[0] || k.wall[1] || k.wall[2];
    k.max_attempts = f.max_attempts > 0 ? f.max_attempts : 64;
    k.cap = f.capacity;
    k.pcap = f.pair_capacity > 0 ? f.pair_capacity : (k.dim == 3 ? 16 : 8) * f.capacity;
    k.ccap = 2 * f.capacity + 64;
    k.wall_drag = f.wall_drag;
    k.min_rad = f.min_rad;
    k.f0 = f.f0_per_mu0;
    k.K = f.k_parameter;
    k.kappa = f.kappa;
    k.skin = f.skin_radius;
    k.vol_mul_const = f.bubble_volume_multiplier;
    k.ain = f.average_surface_area_in;
    k.tol = f.error_tolerance;
    double maxabs = 0.0, maxiv = 0.0;
    for (int a = 0; a < 3; a++) {
        maxabs = std::max(maxabs, std::max(std::fabs(k.lbb[a]), std::fabs(k.tfr[a])));
        maxiv = std::max(maxiv, k.iv[a]);
        k.half_iv[a] = 0.5 * k.iv[a];
        k.half_iv32[a] = (float)(0.5 * k.iv[a]);
        k.iv32[a] = (float)k.iv[a];
    }
    k.mixed = f.precision == CB_PRECISION_MIXED ? 1 : 0;
    k.ffpair = f.precision == CB_PRECISION_FP64_FF ? 1 : 0;
    k.f0_f = (float)k.f0;
    k.f0_l = (float)(k.f0 - (double)k.f0_f);
    k.skin_f = (float)k.skin;
    for (int a = 0; a < 3; a++) k.lbb_f[a] = (float)k.lbb[a];
    k.kq_f = (float)(k.dim == 3 ? k.K / (4.0 * 3.1415926535897932384626433832795) :
                                  k.K / (2.0 * 3.1415926535897932384626433832795));
    for (int a = 0; a < 3; a++) {
        k.lq[a] = (long long)std::llround(k.iv[a] * 1099511627776.0);  // 2^40
        k.hq[a] = k.lq[a] / 2;
        k.lbq[a] = (long long)std::llround(k.lbb[a] * 1099511627776.0);
    }
    // Guard band of the FP32 pair prefilters. An FP32 coordinate carries up
    // to 2^-24 |x| rounding, a periodic shift or minimum image another
    // 2^-24 (|x| + L) (the box edge L rounded to FP32, the shifted value
    // rounded), so a difference is off by at most 2^-24 (3 maxabs + 2 L)
    // per axis, the distance by sqrt(3) times that: < 5.2e-7 (maxabs + L).
    // The squared-distance and cutoff roundings add < 1e-6 absolute.
    // 2e-6 (maxabs + L) + 1e-5 is about 4x the worst case.
    k.pre_margin = (float)(2e-6 * (maxabs + maxiv) + 1e-5);
    // fix_from_double needs |x| < 2^23: box corners within 2^21 leave room
    // for bubbles past a wall
    k.fix_range = maxabs < 2097152.0 ? 1 : 0;
    k.shear_on = f.shear_speed != 0.0 ? 1 : 0;
    k.shear_axis = k.dim - 1;
    k.shear = f.shear_speed;
    k.shear_il = k.iv[k.shear_axis] > 0.0 ? 2.0 / k.iv[k.shear_axis] : 0.0;
    k.shear_f = (float)k.shear;
    k.shear_il_f = (float)k.shear_il;
    k.cell_scale = c->tune.cell_scale >= 1.0 ? c->tune.cell_scale : 1.0;
}

// Process-wide choices of cb_autotune, by dimensionality, precision and
// capacity bucket floor(log2(capacity)).
std::mutex g_tune_mu;
std::map<long long, cb_tuning> g_tune_cache;

long long tune_key(const cb_config &f) {
    int b = 0;
    while (b < 31 && (1LL << (b + 1)) <= (long long)f.capacity) b++;
    return (long long)f.dimensionality * 1000 + (long long)f.precision * 100 + b;
}

// Largest radius of a row into ctrl->max_bubble_radius, which the caller
// zeroed: positive finite doubles order as their bit patterns do.
__global__ void __launch_bounds__(kBlock) k_max_radius(const double *R, int n, Ctrl *ctrl) {
    long long m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long v = __double_as_longlong(R[i]);
        if (v < 0x7ff0000000000000LL) m = max(m, v);  // finite and positive radii only
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0)
        atomicMax(reinterpret_cast<unsigned long long *>(&ctrl->max_bubble_radius),
                  (unsigned long long)m);
}

}  // namespace

namespace cbg {
int sync_status(cb_context *c) {
    int rc = c->pull();
    if (rc) return rc;
    if (c->hctrl->status != CB_OK) return fail(c->hctrl->status, status_text(c->hctrl->status));
    return CB_OK;
}

// A state change from the host (new rows, pairs, dt, options, box) makes
// the candidate predictions of the mixed form stale.
int invalidate_prediction(cb_context *c) {
    int rc = c->pull();
    if (rc) return rc;
    c->hctrl->pred_ready = 0;
    c->hctrl->pred_slot = 0;
    return c->push();
}

// The three kernels of one step() attempt, in the context's precision.
void launch_attempt_kernels(const cb_context *c, const Launch &l, const Bufs &b, int which) {
    const int dim = c->hk.dim;
    if (c->hk.mixed) {
        if (which & 1) launch_predict_mx(l, b, dim);
        if (which & 2) launch_pairs_mx(l, b, dim, c->mode());
        if (which & 4) launch_correct_mx(l, b, dim, c->mode(), c->hk.any_wall != 0);
    } else {
        if (which & 1) launch_predict(l, b, dim);
        if (which & 2) launch_pairs(l, b, dim, c->mode(), c->hk.ffpair != 0);
        if (which & 4) launch_correct(l, b, dim);
    }
}

}  // namespace cbg

namespace {

int run_attempt(cb_context *c) {
    NvtxRange nv("Integration step");
    launch_attempt_kernels(c, c->launch, c->bufs);
    return c->check_launch();
}

int run_search(cb_context *c) {
    launch_search(c->launch, c->bufs, c->hk.dim);
    return c->check_launch();
}

// Eager integrate(): one control-block read per attempt.
int integrate_eager(cb_context *c, int64_t n_steps) {
    for (int64_t s = 0; s < n_steps; s++) {
        for (;;) {
            int rc = run_attempt(c);
            if (rc) return rc;
            rc = sync_status(c);
            if (rc) return rc;
            if (!c->hctrl->too_large) break;
        }
        if (c->hctrl->need_delete) {
            NvtxRange nv("Removal");
            launch_remove(c->launch, c->bufs, c->hk.dim);
            int rc = c->check_launch();
            if (rc) return rc;
        }
        if (c->hctrl->need_search) {
            int rc = run_search(c);
            if (rc) return rc;
            rc = sync_status(c);
            if (rc) return rc;
        }
        if (c->hctrl->stop_hit) break;
    }
    return sync_status(c);
}

}  // namespace

namespace cbg {
// Adds a conditional node to the graph that `stream` is capturing into and
// returns its body graph; the capture continues after the node.
int capture_conditional(cudaStream_t stream, cudaGraphConditionalNodeType type,
                        cudaGraphConditionalHandle *handle, unsigned int dflt,
                        cudaGraph_t *body) {
    cudaStreamCaptureStatus st;
    cudaGraph_t cg;
    const cudaGraphNode_t *deps = nullptr;
    const cudaGraphEdgeData *edges = nullptr;
    size_t nd = 0;
    CB_CUDA(cudaStreamGetCaptureInfo(stream, &st, nullptr, &cg, &deps, &edges, &nd));
    CB_CUDA(cudaGraphConditionalHandleCreate(handle, cg, dflt, cudaGraphCondAssignDefault));
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = *handle;
    p.conditional.type = type;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    CB_CUDA(cudaGraphAddNode(&node, cg, deps, edges, nd, &p));
    CB_CUDA(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1,
                                                cudaStreamSetCaptureDependencies));
    *body = p.conditional.phGraph_out[0];
    return CB_OK;
}

}  // namespace cbg

namespace {

// integrate(n) as one graph:
//   WHILE(h_loop) { predict; pairs; correct; IF(h_delete) remove; IF(h_search) search }
// k_correct's last block sets the three conditions on the device.
int build_graph(cb_context *c) {
    const int key = c->mode() | (c->hk.dim << 4);
    if (c->gexec && c->graph_key == key) return CB_OK;
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    cudaGraph_t g;
    CB_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle hloop, hdel, hsearch;
    CB_CUDA(cudaGraphConditionalHandleCreate(&hloop, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp{};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hloop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    CB_CUDA(cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    long long dummy = 0;
    Launch l = c->launch;
    l.launches = &dummy;
    cudaStream_t s = c->stream;
    CB_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    const int dim = c->hk.dim;
    launch_attempt_kernels(c, l, c->bufs);
    const long long n_attempt = dummy;
    cudaGraph_t delbody, searchbody;
    int rc = capture_conditional(s, cudaGraphCondTypeIf, &hdel, 0, &delbody);
    if (!rc) rc = capture_conditional(s, cudaGraphCondTypeIf, &hsearch, 0, &searchbody);
    cudaGraph_t out;
    cudaError_t e = cudaStreamEndCapture(s, &out);
    if (rc) return rc;
    CB_CUDA(e);
    CB_CUDA(cudaStreamBeginCaptureToGraph(s, delbody, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    launch_remove(l, c->bufs, dim);
    const long long n_remove = dummy - n_attempt;
    CB_CUDA(cudaStreamEndCapture(s, &out));
    CB_CUDA(cudaStreamBeginCaptureToGraph(s, searchbody, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    launch_search(l, c->bufs, dim);
    c->graph_kernels.attempt = n_attempt;
    c->graph_kernels.remove = n_remove;
    c->graph_kernels.search = dummy - n_attempt - n_remove;
    CB_CUDA(cudaStreamEndCapture(s, &out));
    CB_CUDA(cudaGraphInstantiate(&c->gexec, g, 0));
    // upload now, so that the first integrate's launch does not carry it
    CB_CUDA(cudaGraphUpload(c->gexec, c->stream));
    CB_CUDA(cudaGraphDestroy(g));
    c->graph_key = key;
    int r2 = c->pull();
    if (r2) return r2;
    c->hctrl->h_loop = (unsigned long long)hloop;
    c->hctrl->h_delete = (unsigned long long)hdel;
    c->hctrl->h_search = (unsigned long long)hsearch;
    return c->push();
}

// Expects hctrl to hold the device's control block (integrate_impl has just
// read it, or the previous graph integration left it so). One asynchronous
// write of the control block, the graph launch and one read back: the device
// clears graph_mode when its loop ends.
int integrate_graph(cb_context *c, int64_t n_steps) {
    int rc = build_graph(c);
    if (rc) return rc;
    Ctrl &h = *c->hctrl;
    const long long a0 = h.attempts, s0 = h.searches, d0 = h.delete_events;
    h.steps_target = h.steps + n_steps;
    h.graph_mode = 1;
    // hctrl is pinned and not touched again before the synchronising read
    CB_CUDA(cudaMemcpyAsync(c->dctrl, c->hctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream));
    CB_CUDA(cudaGraphLaunch(c->gexec, c->stream));
    rc = c->pull();
    if (rc) return rc;
    c->launches += (h.attempts - a0) * c->graph_kernels.attempt +
                   (h.searches - s0) * c->graph_kernels.search +
                   (h.delete_events - d0) * c->graph_kernels.remove;
    if (h.graph_mode) {  // the loop did not run to its end (a launch failure)
        h.graph_mode = 0;
        if ((rc = c->push())) return rc;
    }
    if (h.status != CB_OK) return fail(h.status, status_text(h.status));
    return CB_OK;
}

}  // namespace

namespace cbg {
void fill_report(const cb_context *c, cb_report *r) {
    const Ctrl &h = *c->hctrl;
    std::memset(r, 0, sizeof(*r));
    r->steps = h.steps;
    r->attempts = h.attempts;
    r->searches = h.searches;
    r->deleted = h.deleted;
    r->bubble_steps = h.bubble_steps;
    r->time_integer = h.tint;
    r->time_fraction = h.tfrac;
    r->time_step = h.dt;
    r->max_error = h.max_err;
    r->max_radius = h.max_bubble_radius;
    r->max_expansion = h.max_exp;
    r->count = h.n;
    r->num_pairs = h.np;
    r->status = h.status;
    r->dt_min = h.dt_min;
    r->dt_max = h.dt_max;
    r->dt_sum = h.dt_sum;
}

}  // namespace cbg

namespace {

}  // namespace

// ====================================================================== ABI
extern "C" {

const char *cb_last_error(void) { return g_err.c_str(); }

int cb_create(const cb_config *cfg, cb_context **out) {
    return cbg::create_context(cfg, out, true);
}

}  // extern "C"

// cb_create; with `graph` and cfg->use_graph the integrate() graph of the
// context's options is built and instantiated here, so that the first
// cb_integrate does not pay for it (the foams of a batch skip it: the batch
// runs its own graph).
int cbg::create_context(const cb_config *cfg, cb_context **out, bool graph) {
    if (!cfg || !out) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (cfg->dimensionality != 2 && cfg->dimensionality != 3)
        return fail(CB_ERR_INVALID_ARGUMENT, "dimensionality must be 2 or 3");
    if (cfg->capacity <= 0) return fail(CB_ERR_INVALID_ARGUMENT, "capacity must be positive");
    if ((long long)cfg->capacity * 2 + 64 > 0x7fffffffLL)
        return fail(CB_ERR_INVALID_ARGUMENT, "capacity too large");
    {  // pair-list offsets are int32 (row starts, the pair count)
        const long long pcap = cfg->pair_capacity > 0
                                   ? (long long)cfg->pair_capacity
                                   : (long long)(cfg->dimensionality == 3 ? 16 : 8) * cfg->capacity;
        if (cfg->pair_capacity < 0 || pcap + 1 > 0x7fffffffLL)
            return fail(CB_ERR_INVALID_ARGUMENT,
                        "pair capacity beyond 2^31 - 2 (set pair_capacity or lower capacity)");
    }
    if (cfg->precision != CB_PRECISION_FP64 && cfg->precision != CB_PRECISION_MIXED &&
        cfg->precision != CB_PRECISION_FP64_FF)
        return fail(CB_ERR_INVALID_ARGUMENT, "unknown precision");
    if (cfg->precision == CB_PRECISION_MIXED) {
        for (int a = 0; a < 3; a++)
            if (std::fabs(cfg->lbb[a]) > 2097152.0 || std::fabs(cfg->tfr[a]) > 2097152.0)
                return fail(CB_ERR_INVALID_ARGUMENT,
                            "mixed precision needs box corners within +-2^21 (fixed point 2^40)");
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
        return fail(CB_ERR_NO_DEVICE, "no CUDA device");
    cb_context *c = new cb_context();
    c->cfg = *cfg;
    int rc = CB_OK;
    auto bail = [&](int code) {
        cb_destroy(c);
        return code;
    };
    if (cudaGetDevice(&c->dev) != cudaSuccess) return bail(fail(CB_ERR_CUDA, "cudaGetDevice"));
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->dev);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(CB_ERR_CUDA, "cudaStreamCreate"));
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    fill_const(c);
    const size_t cap = (size_t)c->hk.cap, pcap = (size_t)c->hk.pcap, ccap = (size_t)c->hk.ccap;
    c->launch.grid = std::max(1, c->sms) * 8;
    c->launch.sms = std::max(1, c->sms);
    c->launch.scan_grid = std::min(1024, std::max(1, c->sms) * 4);
    c->launch.cover = (int)((cap + kBlock - 1) / kBlock);
    c->launch.stream = c->stream;
    c->launch.launches = &c->launches;
    const int G = std::max(c->launch.grid, c->launch.cover);
    if (cudaMallocHost(&c->hctrl, sizeof(Ctrl)) != cudaSuccess)
        return bail(fail(CB_ERR_CUDA, "cudaMallocHost"));
    std::memset(c->hctrl, 0, sizeof(Ctrl));
    Bufs &b = c->bufs;
    if ((rc = c->alloc(&c->dk, 1))) return bail(rc);
    if ((rc = c->alloc(&c->dctrl, 1))) return bail(rc);
    for (int r = 0; r < ND_ROLES; r++)
        if ((rc = c->alloc(&c->dslot[r], cap))) return bail(rc);
    for (int r = 0; r < NI_ROLES; r++)
        if ((rc = c->alloc(&c->islot[r], cap))) return bail(rc);
    for (int r = 0; r < NP_ROLES; r++)
        if ((rc = c->alloc(&c->pslot[r], pcap))) return bail(rc);
    if ((rc = c->alloc(&c->d_dslots, ND_ROLES))) return bail(rc);
    if ((rc = c->alloc(&c->d_islots, NI_ROLES))) return bail(rc);
    if ((rc = c->alloc(&c->d_pslots, NP_ROLES))) return bail(rc);
    if ((rc = c->alloc(&b.pred, 4 * cap))) return bail(rc);
    if (c->hk.mixed && (rc = c->alloc(&b.predc, 8 * cap))) return bail(rc);
    if ((rc = c->alloc(&b.invr, 2 * cap))) return bail(rc);
    if (c->hk.ffpair && (rc = c->alloc(&b.ffr, 2 * cap))) return bail(rc);
    if ((rc = c->alloc(&b.acc, (size_t)kAcc * cap))) return bail(rc);
    if ((rc = c->alloc(&b.part, (size_t)kPartSlots * G))) return bail(rc);
    if ((rc = c->alloc(&b.delflag, cap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.iscan, cap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.blocksums, (size_t)c->launch.scan_grid + 1))) return bail(rc);
    if ((rc = c->alloc(&b.cellOf, cap))) return bail(rc);
    if ((rc = c->alloc(&b.cellSorted, cap))) return bail(rc);
    if ((rc = c->alloc(&b.perm, cap))) return bail(rc);
    if ((rc = c->alloc(&b.permSorted, cap))) return bail(rc);
    if ((rc = c->alloc(&b.cellCount, ccap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.cellStart, ccap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.cellFill, ccap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.rowCount, cap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.rowStart, cap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.pos32, cap))) return bail(rc);
    if (c->hk.dim == 3 && (rc = c->alloc(&b.pos32r, cap))) return bail(rc);
    if ((rc = c->alloc(&b.holes, cap))) return bail(rc);
    if ((rc = c->alloc(&b.moveDst, cap))) return bail(rc);
    if ((rc = c->alloc(&b.keep, pcap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.keepScan, pcap + 1))) return bail(rc);
    if ((rc = c->alloc(&b.stash, cap * (size_t)kStash(c->hk.dim)))) return bail(rc);
    if ((rc = c->alloc(&b.energy, std::max<size_t>(cap, 8)))) return bail(rc);
    if (cudaMemcpyAsync(c->d_dslots, c->dslot, sizeof(c->dslot), cudaMemcpyHostToDevice,
                        c->stream) != cudaSuccess ||
        cudaMemcpyAsync(c->d_islots, c->islot, sizeof(c->islot), cudaMemcpyHostToDevice,
                        c->stream) != cudaSuccess ||
        cudaMemcpyAsync(c->d_pslots, c->pslot, sizeof(c->pslot), cudaMemcpyHostToDevice,
                        c->stream) != cudaSuccess)
        return bail(fail(CB_ERR_CUDA, "slot table upload"));
    b.ctrl = c->dctrl;
    b.k = c->dk;
    b.ds = c->d_dslots;
    b.is = c->d_islots;
    b.ps = c->d_pslots;
    b.dbg_ov = nullptr;
    Ctrl &h = *c->hctrl;
    for (int r = 0; r < ND_ROLES; r++) h.drole[r] = r;
    for (int r = 0; r < NI_ROLES; r++) h.irole[r] = r;
    for (int r = 0; r < NP_ROLES; r++) h.prole[r] = r;
    h.dt = cfg->time_step;
    h.dt_min = 9999999.9;
    h.dt_max = -1.0;
    h.dt_sum = 0.0;
    h.use_gas = cfg->use_gas_exchange ? 1 : 0;
    h.use_flow = cfg->use_flow ? 1 : 0;
    h.inc_path = cfg->increment_path ? 1 : 0;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune_cache.find(tune_key(*cfg));
        if (it != g_tune_cache.end()) {
            c->tune = it->second;
            c->launch.pair_run = c->tune.pair_run;
            c->launch.pair_bps = c->tune.pair_blocks;
            c->launch.step_bps = c->tune.step_blocks;
            fill_const(c);
        }
    }
    if ((rc = c->upload_const())) return bail(rc);
    if ((rc = c->push())) return bail(rc);
    if (graph && cfg->use_graph && (rc = build_graph(c))) return bail(rc);
    *out = c;
    return CB_OK;
}

extern "C" {

int cb_destroy(cb_context *c) {
    if (!c) return CB_OK;
    cudaSetDevice(c->dev);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    for (void *p : c->allocs) cudaFree(p);
    if (c->hctrl) cudaFreeHost(c->hctrl);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return CB_OK;
}

#define CB_ENTER(c)                                                                         \
    do {                                                                                    \
        if (!(c)) return fail(CB_ERR_INVALID_ARGUMENT, "null context");                     \
        cbg::note_call();                                                                   \
        CB_CUDA(cudaSetDevice((c)->dev));                                                   \
    } while (0)

int cb_load_state(cb_context *c, const cb_state_view *s) {
    CB_ENTER(c);
    if (!s) return fail(CB_ERR_INVALID_ARGUMENT, "null state");
    if (s->count < 0 || s->count > c->hk.cap) return fail(CB_ERR_CAPACITY, "count exceeds capacity");
    if (!s->x || !s->y || !s->r || (c->hk.dim == 3 && !s->z))
        return fail(CB_ERR_INVALID_ARGUMENT, "positions and radii required");
    int rc = c->pull();
    if (rc) return rc;
    Ctrl &h = *c->hctrl;
    const size_t n = (size_t)s->count;
    const double *drows[ND_ROLES] = {};
    drows[RX] = s->x;
    drows[RY] = s->y;
    drows[RZ] = s->z;
    drows[RR] = s->r;
    drows[RV0] = s->dxdt;
    drows[RV1] = s->dydt;
    drows[RV2] = s->dzdt;
    drows[RV3] = s->drdt;
    drows[RVO0] = s->dxdto;
    drows[RVO1] = s->dydto;
    drows[RVO2] = s->dzdto;
    drows[RVO3] = s->drdto;
    drows[RPATH] = s->path;
    drows[RERR] = s->error;
    drows[RS0] = s->saved_x;
    drows[RS1] = s->saved_y;
    drows[RS2] = s->saved_z;
    drows[RS3] = s->saved_r;
    std::vector<std::vector<float>> fl;
    for (int r = 0; r < ND_ROLES; r++) {
        double *dst = c->dslot[h.drole[r]];
        const bool rate = r >= RV0 && r <= RVP3;
        if (drows[r] && c->hk.mixed && rate) {  // FP32 rate rows
            fl.emplace_back(drows[r], drows[r] + n);
            CB_CUDA(cudaMemcpyAsync(dst, fl.back().data(), n * 4, cudaMemcpyHostToDevice,
                                    c->stream));
        } else if (drows[r]) {
            CB_CUDA(cudaMemcpyAsync(dst, drows[r], n * 8, cudaMemcpyHostToDevice, c->stream));
        } else if (r >= RS0 && r <= RS3 && n && drows[RX + (r - RS0)]) {
            // saved position / radius not given: the uploaded current ones,
            // copied on the device
            CB_CUDA(cudaMemcpyAsync(dst, c->dslot[h.drole[RX + (r - RS0)]], n * 8,
                                    cudaMemcpyDeviceToDevice, c->stream));
        } else {
            CB_CUDA(cudaMemsetAsync(dst, 0, (size_t)c->hk.cap * 8, c->stream));
        }
    }
    const int32_t *irows[NI_ROLES] = {};
    irows[IWX] = s->wrap_count_x;
    irows[IWY] = s->wrap_count_y;
    irows[IWZ] = s->wrap_count_z;
    irows[INN] = s->num_neighbors;
    std::vector<int32_t> idx;
    if (!s->index) {
        idx.resize(n);
        for (size_t i = 0; i < n; i++) idx[i] = (int32_t)i;
    }
    irows[IIDX] = s->index ? s->index : idx.data();
    for (int r = 0; r < NI_ROLES; r++) {
        int *dst = c->islot[h.irole[r]];
        if (irows[r] && n)
            CB_CUDA(cudaMemcpyAsync(dst, irows[r], n * 4, cudaMemcpyHostToDevice, c->stream));
        else
            CB_CUDA(cudaMemsetAsync(dst, 0, (size_t)c->hk.cap * 4, c->stream));
    }
    CB_CUDA(cudaMemsetAsync(c->bufs.acc, 0, (size_t)kAcc * c->hk.cap * 8, c->stream));
    h.n = s->count;
    h.np = 0;
    h.ndel = 0;
    h.status = CB_OK;
    h.max_bubble_radius = 0.0;
    h.too_large = h.need_search = h.need_delete = h.attempts_this_step = 0;
    h.pred_ready = 0;
    h.pred_slot = 0;
    CB_CUDA(cudaMemcpyAsync(c->dctrl, c->hctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, c->stream));
    // the largest radius (HostData.maxBubbleRadius) from the uploaded row
    if (n) {
        k_max_radius<<<std::min<int>(c->launch.grid, (int)((n + kBlock - 1) / kBlock)), kBlock, 0,
                       c->stream>>>(c->dslot[h.drole[RR]], (int)n, c->dctrl);
        c->launches += 1;
        if ((rc = c->check_launch())) return rc;
    }
    rc = c->pull();  // synchronises, so the caller's buffers are free
    if (rc) return rc;
    c->loaded = true;
    return CB_OK;
}

int cb_get_state(cb_context *c, cb_state_view *s) {
    CB_ENTER(c);
    if (!s) return fail(CB_ERR_INVALID_ARGUMENT, "null state");
    int rc = c->pull();
    if (rc) return rc;
    const Ctrl &h = *c->hctrl;
    const size_t n = (size_t)h.n;
    s->count = h.n;
    double *drows[ND_ROLES] = {};
    drows[RX] = s->x;
    drows[RY] = s->y;
    drows[RZ] = s->z;
    drows[RR] = s->r;
    drows[RV0] = s->dxdt;
    drows[RV1] = s->dydt;
    drows[RV2] = s->dzdt;
    drows[RV3] = s->drdt;
    drows[RVO0] = s->dxdto;
    drows[RVO1] = s->dydto;
    drows[RVO2] = s->dzdto;
    drows[RVO3] = s->drdto;
    drows[RPATH] = s->path;
    drows[RERR] = s->error;
    drows[RS0] = s->saved_x;
    drows[RS1] = s->saved_y;
    drows[RS2] = s->saved_z;
    drows[RS3] = s->saved_r;
    std::vector<std::pair<double *, std::vector<float>>> fl;
    for (int r = 0; r < ND_ROLES; r++) {
        if (!drows[r] || !n) continue;
        if (c->hk.mixed && r >= RV0 && r <= RVP3) {  // FP32 rate rows
            fl.emplace_back(drows[r], std::vector<float>(n));
            CB_CUDA(cudaMemcpyAsync(fl.back().second.data(), c->dslot[h.drole[r]], n * 4,
                                    cudaMemcpyDeviceToHost, c->stream));
            continue;
        }
        CB_CUDA(cudaMemcpyAsync(drows[r], c->dslot[h.drole[r]], n * 8, cudaMemcpyDeviceToHost,
                                c->stream));
    }
    int32_t *irows[NI_ROLES] = {};
    irows[IWX] = s->wrap_count_x;
    irows[IWY] = s->wrap_count_y;
    irows[IWZ] = s->wrap_count_z;
    irows[IIDX] = s->index;
    irows[INN] = s->num_neighbors;
    for (int r = 0; r < NI_ROLES; r++)
        if (irows[r] && n)
            CB_CUDA(cudaMemcpyAsync(irows[r], c->islot[h.irole[r]], n * 4, cudaMemcpyDeviceToHost,
                                    c->stream));
    CB_CUDA(cudaStreamSynchronize(c->stream));
    for (auto &f : fl)
        for (size_t i = 0; i < n; i++) f.first[i] = f.second[i];
    return CB_OK;
}

int cb_set_options(cb_context *c, int32_t g, int32_t f, int32_t p) {
    {
        if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null context");
        CB_CUDA(cudaSetDevice(c->dev));
        const int rc0 = invalidate_prediction(c);
        if (rc0) return rc0;
    }
    CB_ENTER(c);
    int rc = c->pull();
    if (rc) return rc;
    c->hctrl->use_gas = g ? 1 : 0;
    c->hctrl->use_flow = f ? 1 : 0;
    c->hctrl->inc_path = p ? 1 : 0;
    return c->push();
}

int cb_set_time(cb_context *c, double dt, uint64_t ti, double tf) {
    {
        if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null context");
        CB_CUDA(cudaSetDevice(c->dev));
        const int rc0 = invalidate_prediction(c);
        if (rc0) return rc0;
    }
    CB_ENTER(c);
    int rc = c->pull();
    if (rc) return rc;
    c->hctrl->dt = dt;
    c->hctrl->tint = ti;
    c->hctrl->tfrac = tf;
    return c->push();
}

int cb_set_box(cb_context *c, const double lbb[3], const double tfr[3], double m,
               const double flbb[3], const double ftfr[3]) {
    {
        if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null context");
        CB_CUDA(cudaSetDevice(c->dev));
        const int rc0 = invalidate_prediction(c);
        if (rc0) return rc0;
    }
    CB_ENTER(c);
    if (!lbb || !tfr) return fail(CB_ERR_INVALID_ARGUMENT, "null box");
    for (int a = 0; a < 3; a++) {
        c->cfg.lbb[a] = lbb[a];
        c->cfg.tfr[a] = tfr[a];
        if (flbb) c->cfg.flow_lbb[a] = flbb[a];
        if (ftfr) c->cfg.flow_tfr[a] = ftfr[a];
    }
    c->cfg.bubble_volume_multiplier = m;
    fill_const(c);
    return c->upload_const();
}

int cb_bootstrap(cb_context *c) {
    NvtxRange nv("Bootstrap");
    {
        if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null context");
        CB_CUDA(cudaSetDevice(c->dev));
        const int rc0 = invalidate_prediction(c);
        if (rc0) return rc0;
    }
    CB_ENTER(c);
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    const int dim = c->hk.dim;
    if (c->hk.mixed) {
        launch_boot_mx(c->launch, c->bufs, dim, 0);
        launch_pairs_mx(c->launch, c->bufs, dim, 0);
        launch_boot_mx(c->launch, c->bufs, dim, 1);
        launch_pairs_mx(c->launch, c->bufs, dim, 0);
        launch_boot_mx(c->launch, c->bufs, dim, 2);
    } else {
        launch_boot(c->launch, c->bufs, dim, 0);
        launch_pairs(c->launch, c->bufs, dim, 0, c->hk.ffpair != 0);
        launch_boot(c->launch, c->bufs, dim, 1);
        launch_pairs(c->launch, c->bufs, dim, 0, c->hk.ffpair != 0);
        launch_boot(c->launch, c->bufs, dim, 2);
    }
    int rc = c->check_launch();
    if (rc) return rc;
    return sync_status(c);
}

int cb_search_neighbors(cb_context *c) {
    NvtxRange nv("Neighbors");
    CB_ENTER(c);
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    int rc = run_search(c);
    if (rc) return rc;
    return sync_status(c);
}

int cb_get_pairs(cb_context *c, int32_t *i, int32_t *j, int32_t capacity, int32_t *count) {
    CB_ENTER(c);
    if (!count) return fail(CB_ERR_INVALID_ARGUMENT, "null count");
    int rc = c->pull();
    if (rc) return rc;
    const Ctrl &h = *c->hctrl;
    *count = h.np;
    if (!i || !j) return CB_OK;
    if (capacity < h.np) return fail(CB_ERR_CAPACITY, "buffer too small");
    if (h.np) {
        CB_CUDA(cudaMemcpyAsync(i, c->pslot[h.prole[PI0]], (size_t)h.np * 4,
                                cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaMemcpyAsync(j, c->pslot[h.prole[PJ0]], (size_t)h.np * 4,
                                cudaMemcpyDeviceToHost, c->stream));
    }
    CB_CUDA(cudaStreamSynchronize(c->stream));
    return CB_OK;
}

int cb_set_pairs(cb_context *c, const int32_t *i, const int32_t *j, int32_t count) {
    {
        if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null context");
        CB_CUDA(cudaSetDevice(c->dev));
        const int rc0 = invalidate_prediction(c);
        if (rc0) return rc0;
    }
    CB_ENTER(c);
    if (count < 0 || (count && (!i || !j))) return fail(CB_ERR_INVALID_ARGUMENT, "bad pairs");
    if (count > c->hk.pcap) return fail(CB_ERR_CAPACITY, "pair capacity exceeded");
    int rc = c->pull();
    if (rc) return rc;
    Ctrl &h = *c->hctrl;
    std::vector<int32_t> nn((size_t)h.n, 0);
    for (int p = 0; p < count; p++) {
        if (i[p] < 0 || j[p] < 0 || i[p] >= h.n || j[p] >= h.n || i[p] == j[p])
            return fail(CB_ERR_INVALID_ARGUMENT, "pair index out of range");
        nn[i[p]]++;
        nn[j[p]]++;
    }
    if (count) {
        CB_CUDA(cudaMemcpyAsync(c->pslot[h.prole[PI0]], i, (size_t)count * 4,
                                cudaMemcpyHostToDevice, c->stream));
        CB_CUDA(cudaMemcpyAsync(c->pslot[h.prole[PJ0]], j, (size_t)count * 4,
                                cudaMemcpyHostToDevice, c->stream));
    }
    if (h.n)
        CB_CUDA(cudaMemcpyAsync(c->islot[h.irole[INN]], nn.data(), (size_t)h.n * 4,
                                cudaMemcpyHostToDevice, c->stream));
    h.np = count;
    return c->push();
}

int cb_attempt(cb_context *c, cb_attempt_view *o) {
    CB_ENTER(c);
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    int rc = c->pull();
    if (rc) return rc;
    c->hctrl->no_accept = 1;
    if ((rc = c->push())) return rc;
    Bufs b = c->bufs;
    b.dbg_ov = c->bufs.energy;  // scratch row for the overlap copy
    const int dim = c->hk.dim;
    launch_attempt_kernels(c, c->launch, b);
    if ((rc = c->check_launch())) return rc;
    if ((rc = c->pull())) return rc;
    Ctrl &h = *c->hctrl;
    const size_t n = (size_t)h.n;
    if (o) {
        const int gas = h.use_gas;
        double *rows[] = {o->xp, o->yp, o->zp, o->rp, o->dxdtp, o->dydtp, o->dzdtp, o->drdtp,
                          o->error, o->path_new, o->overlap};
        const int roles[] = {RXN, RYN, dim == 3 ? RZN : RZ, gas ? RRN : RR, RVP0, RVP1,
                             RVP2, RVP3, RERR, RPATHN, -1};
        std::vector<float> tmp;
        for (int q = 0; q < 11; q++) {
            if (!rows[q] || !n) continue;
            const double *src = roles[q] >= 0 ? c->dslot[h.drole[roles[q]]] : c->bufs.energy;
            if (c->hk.mixed && q >= 4 && q < 8) {  // FP32 rate rows
                tmp.resize(n);
                CB_CUDA(cudaMemcpyAsync(tmp.data(), src, n * 4, cudaMemcpyDeviceToHost, c->stream));
                CB_CUDA(cudaStreamSynchronize(c->stream));
                for (size_t i = 0; i < n; i++) rows[q][i] = tmp[i];
                continue;
            }
            CB_CUDA(cudaMemcpyAsync(rows[q], src, n * 8, cudaMemcpyDeviceToHost, c->stream));
        }
        if (o->delete_flags && n)
            CB_CUDA(cudaMemcpyAsync(o->delete_flags, c->bufs.delflag, n * 4,
                                    cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaStreamSynchronize(c->stream));
        if (!gas && o->drdtp) std::memset(o->drdtp, 0, n * 8);
        if (dim == 2) {
            if (o->zp) std::memset(o->zp, 0, n * 8);
            if (o->dzdtp) std::memset(o->dzdtp, 0, n * 8);
        }
        o->total_area = h.sumA;
        o->total_area_per_radius = h.sumAr;
        o->total_overlap_area = h.sumAo;
        o->total_overlap_area_per_radius = h.sumAor;
        o->total_volume_new = h.vol_new;
        o->max_error = h.max_err;
        o->max_radius = h.max_rad;
        o->max_expansion = h.max_exp;
        o->num_to_be_deleted = gas ? h.ndel : 0;
    }
    h.no_accept = 0;
    h.attempts_this_step = 0;
    if ((rc = c->push())) return rc;
    if (h.status != CB_OK) return fail(h.status, status_text(h.status));
    return CB_OK;
}

// fresh: hctrl already holds the device's control block (no read needed)
static int integrate_impl(cb_context *c, int64_t n_steps, bool fresh) {
    NvtxRange nv("Integration");
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    if (n_steps < 0) return fail(CB_ERR_INVALID_ARGUMENT, "negative step count");
    if (!fresh) {
        int rc = c->pull();
        if (rc) return rc;
    }
    if (c->hctrl->status != CB_OK) return fail(c->hctrl->status, status_text(c->hctrl->status));
    if (n_steps == 0) return CB_OK;
    return c->cfg.use_graph ? integrate_graph(c, n_steps) : integrate_eager(c, n_steps);
}

int cb_integrate(cb_context *c, int64_t n_steps, cb_report *r) {
    // back-to-back graph integrations skip the control-block read: no call
    // has run on any context since the last one returned
    const bool fresh = c && c->mirror_call == cbg::g_calls.load(std::memory_order_relaxed);
    CB_ENTER(c);
    c->mirror_call = ~0ull;
    const int rc = integrate_impl(c, n_steps, fresh);
    if (rc == CB_OK && c->cfg.use_graph) c->mirror_call = cbg::g_calls.load(std::memory_order_relaxed);
    // integrate_impl leaves hctrl as read from the device after its last
    // launch (or before, when it returned early)
    if (r) fill_report(c, r);
    return rc;
}

int cb_integrate_timed(cb_context *c, int64_t n_steps, cb_report *r, double *ms) {
    CB_ENTER(c);
    CB_CUDA(cudaStreamSynchronize(c->stream));
    CB_CUDA(cudaEventRecord(c->ev0, c->stream));
    const int rc = integrate_impl(c, n_steps, false);
    CB_CUDA(cudaEventRecord(c->ev1, c->stream));
    CB_CUDA(cudaEventSynchronize(c->ev1));
    float t = 0.f;
    CB_CUDA(cudaEventElapsedTime(&t, c->ev0, c->ev1));
    if (ms) *ms = (double)t;
    if (r) {
        c->pull();
        fill_report(c, r);
    }
    return rc;
}

int cb_integrate_until(cb_context *c, int64_t max_steps, const cb_stop *stop, cb_report *r) {
    CB_ENTER(c);
    if (!stop) return fail(CB_ERR_INVALID_ARGUMENT, "null stop conditions");
    int rc = c->pull();
    if (rc) return rc;
    Ctrl &h = *c->hctrl;
    h.stop_on = 1;
    h.stop_hit = 0;
    h.stop_tint = stop->time_integer;
    h.stop_tfrac = stop->time_fraction;
    h.stop_nmin = stop->min_count;
    h.stop_rmax = stop->max_radius;
    if ((rc = c->push())) return rc;
    rc = integrate_impl(c, max_steps, false);
    int rc2 = c->pull();
    h.stop_on = 0;
    h.stop_hit = 0;
    if (!rc2) rc2 = c->push();
    if (r) fill_report(c, r);
    return rc ? rc : rc2;
}

int cb_get_report(cb_context *c, cb_report *r) {
    CB_ENTER(c);
    if (!r) return fail(CB_ERR_INVALID_ARGUMENT, "null report");
    int rc = c->pull();
    if (rc) return rc;
    fill_report(c, r);
    return CB_OK;
}

int cb_energy(cb_context *c, double *out) {
    NvtxRange nv("Energy");
    CB_ENTER(c);
    if (!out) return fail(CB_ERR_INVALID_ARGUMENT, "null output");
    launch_energy(c->launch, c->bufs, c->hk.dim, 0);
    int rc = c->check_launch();
    if (rc) return rc;
    if ((rc = c->pull())) return rc;
    *out = c->hctrl->misc_result;
    return CB_OK;
}

int cb_bubble_energies(cb_context *c, double *e, int32_t capacity) {
    CB_ENTER(c);
    int rc = c->pull();
    if (rc) return rc;
    const int n = c->hctrl->n;
    if (!e || capacity < n) return fail(CB_ERR_INVALID_ARGUMENT, "bad energy buffer");
    CB_CUDA(cudaMemsetAsync(c->bufs.energy, 0, (size_t)c->hk.cap * 8, c->stream));
    launch_energy(c->launch, c->bufs, c->hk.dim, 1);
    if ((rc = c->check_launch())) return rc;
    if (n)
        CB_CUDA(cudaMemcpyAsync(e, c->bufs.energy, (size_t)n * 8, cudaMemcpyDeviceToHost,
                                c->stream));
    CB_CUDA(cudaStreamSynchronize(c->stream));
    return CB_OK;
}

int cb_total_volume(cb_context *c, double *out) {
    NvtxRange nv("Volume");
    CB_ENTER(c);
    if (!out) return fail(CB_ERR_INVALID_ARGUMENT, "null output");
    launch_volume(c->launch, c->bufs, c->hk.dim);
    int rc = c->check_launch();
    if (rc) return rc;
    if ((rc = c->pull())) return rc;
    *out = c->hctrl->misc_result;
    return CB_OK;
}

}  // extern "C"

namespace {

// Mean device ms of predict, pairs and correct over `reps` attempts that are
// not accepted; the control block (dt, counters) is restored afterwards.
int profile_attempts(cb_context *c, int32_t reps, double ms[3]) {
    int rc = c->pull();
    if (rc) return rc;
    Ctrl saved = *c->hctrl;
    c->hctrl->no_accept = 1;
    if ((rc = c->push())) return rc;
    cudaEvent_t ev[4];
    for (int q = 0; q < 4; q++) CB_CUDA(cudaEventCreate(&ev[q]));
    double acc[3] = {0, 0, 0};
    // one attempt untimed: the first launch of a kernel also loads its code
    launch_attempt_kernels(c, c->launch, c->bufs);
    CB_CUDA(cudaStreamSynchronize(c->stream));
    for (int r = 0; r < reps; r++) {
        CB_CUDA(cudaEventRecord(ev[0], c->stream));
        launch_attempt_kernels(c, c->launch, c->bufs, 1);
        CB_CUDA(cudaEventRecord(ev[1], c->stream));
        launch_attempt_kernels(c, c->launch, c->bufs, 2);
        CB_CUDA(cudaEventRecord(ev[2], c->stream));
        launch_attempt_kernels(c, c->launch, c->bufs, 4);
        CB_CUDA(cudaEventRecord(ev[3], c->stream));
        CB_CUDA(cudaEventSynchronize(ev[3]));
        for (int q = 0; q < 3; q++) {
            float t = 0.f;
            CB_CUDA(cudaEventElapsedTime(&t, ev[q], ev[q + 1]));
            acc[q] += t;
        }
    }
    for (int q = 0; q < 4; q++) cudaEventDestroy(ev[q]);
    for (int q = 0; q < 3; q++) ms[q] = acc[q] / reps;
    if ((rc = c->check_launch())) return rc;
    if ((rc = c->pull())) return rc;
    const int status = c->hctrl->status;
    *c->hctrl = saved;
    c->hctrl->status = status;
    return c->push();
}

// Mean device ms of one search over `reps` searches of the current state
// (after one untimed search); the search counter is restored.
int profile_searches(cb_context *c, int32_t reps, double *ms) {
    int rc = c->pull();
    if (rc) return rc;
    const long long searches0 = c->hctrl->searches;
    if ((rc = run_search(c))) return rc;
    CB_CUDA(cudaStreamSynchronize(c->stream));
    CB_CUDA(cudaEventRecord(c->ev0, c->stream));
    for (int r = 0; r < reps; r++) launch_search(c->launch, c->bufs, c->hk.dim);
    CB_CUDA(cudaEventRecord(c->ev1, c->stream));
    CB_CUDA(cudaEventSynchronize(c->ev1));
    float t = 0.f;
    CB_CUDA(cudaEventElapsedTime(&t, c->ev0, c->ev1));
    *ms = (double)t / reps;
    if ((rc = c->check_launch())) return rc;
    if ((rc = sync_status(c))) return rc;
    c->hctrl->searches = searches0;  // measurement searches are not the run's
    return c->push();
}

}  // namespace

// Validates and applies a tuning: the launch knobs, the cell scale of the
// device constants, and a rebuild of the integrate graph at its next use.
int cbg::apply_tuning(cb_context *c, const cb_tuning &t) {
    if (!(t.cell_scale >= 1.0 && t.cell_scale <= 4.0))
        return fail(CB_ERR_INVALID_ARGUMENT, "cell_scale must lie in [1, 4]");
    if (t.pair_run != 0 && t.pair_run != 2 && t.pair_run != 4 && t.pair_run != 8)
        return fail(CB_ERR_INVALID_ARGUMENT, "pair_run must be 0, 2, 4 or 8");
    if (t.pair_blocks < 0 || t.pair_blocks > 8 || t.step_blocks < 0 || t.step_blocks > 8)
        return fail(CB_ERR_INVALID_ARGUMENT, "blocks per SM must lie in 0 ... 8");
    c->tune = t;
    if (c->tune.pair_run == 0) c->tune.pair_run = 4;
    c->launch.pair_run = c->tune.pair_run;
    c->launch.pair_bps = c->tune.pair_blocks;
    c->launch.step_bps = c->tune.step_blocks;
    fill_const(c);
    if (c->gexec) {
        cudaGraphExecDestroy(c->gexec);
        c->gexec = nullptr;
    }
    c->graph_key = -1;
    return c->upload_const();
}

extern "C" {

int cb_profile_kernels(cb_context *c, int32_t reps, double ms[3]) {
    CB_ENTER(c);
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    if (reps < 1 || !ms) return fail(CB_ERR_INVALID_ARGUMENT, "bad arguments");
    return profile_attempts(c, reps, ms);
}

int cb_profile_search(cb_context *c, int32_t reps, double *ms) {
    NvtxRange nv("Neighbors");
    CB_ENTER(c);
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    if (reps < 1 || !ms) return fail(CB_ERR_INVALID_ARGUMENT, "bad arguments");
    return profile_searches(c, reps, ms);
}

int cb_set_tuning(cb_context *c, const cb_tuning *t) {
    CB_ENTER(c);
    if (!t) return fail(CB_ERR_INVALID_ARGUMENT, "null tuning");
    return apply_tuning(c, *t);
}

int cb_forget_tuning(void) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_cache.clear();
    return CB_OK;
}

int cb_get_tuning(cb_context *c, cb_tuning *t) {
    if (!c || !t) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    *t = c->tune;
    return CB_OK;
}

int cb_autotune(cb_context *c, int32_t reps, cb_tuning *best) {
    CB_ENTER(c);
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    if (reps < 1 || !best) return fail(CB_ERR_INVALID_ARGUMENT, "bad arguments");
    int rc = c->pull();
    if (rc) return rc;
    if (c->hctrl->np < 1) return fail(CB_ERR_STATE, "no pair list: search first");
    cb_tuning t = c->tune;
    double ms[3];
    // pair kernel: pairs per thread x resident blocks per SM
    const int runs_mx[] = {2, 4, 8}, runs_one[] = {4};
    const int *runs = c->hk.mixed ? runs_mx : runs_one;
    const int nruns = c->hk.mixed ? 3 : 1;
    const int blocks[] = {0, 2, 3};
    double best_pairs = 1e300;
    cb_tuning bt = t;
    for (int r = 0; r < nruns; r++)
        for (int bl : blocks) {
            cb_tuning q = t;
            q.pair_run = runs[r];
            q.pair_blocks = bl;
            if ((rc = apply_tuning(c, q)) || (rc = profile_attempts(c, reps, ms))) return rc;
            if (ms[1] < best_pairs) {
                best_pairs = ms[1];
                bt.pair_run = q.pair_run;
                bt.pair_blocks = q.pair_blocks;
            }
        }
    // predict + correct: resident blocks per SM
    double best_step = 1e300;
    for (int bl : {0, 1, 2, 3}) {
        cb_tuning q = bt;
        q.step_blocks = bl;
        if ((rc = apply_tuning(c, q)) || (rc = profile_attempts(c, reps, ms))) return rc;
        if (ms[0] + ms[2] < best_step) {
            best_step = ms[0] + ms[2];
            bt.step_blocks = bl;
        }
    }
    // neighbour search: cell edge
    double best_search = 1e300;
    for (double cs : {1.0, 1.15, 1.3, 1.5}) {
        cb_tuning q = bt;
        q.cell_scale = cs;
        double sm = 0.0;
        if ((rc = apply_tuning(c, q)) || (rc = profile_searches(c, reps, &sm))) return rc;
        if (sm < best_search) {
            best_search = sm;
            bt.cell_scale = cs;
        }
    }
    if ((rc = apply_tuning(c, bt))) return rc;
    // leave the state searched with the chosen cells
    if ((rc = run_search(c)) || (rc = sync_status(c))) return rc;
    if ((rc = c->pull())) return rc;
    c->hctrl->searches -= 1;  // a measurement search, not the run's
    if ((rc = c->push())) return rc;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_cache[tune_key(c->cfg)] = bt;
    }
    *best = bt;
    return CB_OK;
}

int cb_launch_count(cb_context *c, int64_t *count) {
    if (!c || !count) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    *count = c->launches;
    return CB_OK;
}

}  // extern "C"
