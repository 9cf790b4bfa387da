// Batched foams: many independent cb_contexts advanced by one launch per
// stage. The kernels are the single-foam bodies on a virtual grid (see
// CB_KERNEL_PAIR in common.cuh): a phase's work list names the selected
// foams and the prefix sums of their virtual grids (attempt: capacity / tile
// blocks, tile tuned; search and deletion: capacity / 256), and a fixed grid
// of resident blocks loops over the work items, so the reductions,
// last-block finishes and scans of every foam are exactly its own. After
// each attempt one block (k_batch_decide) reads every foam's outcome, picks
// the phases each foam takes part in next (Ctrl::bsel), rebuilds the three
// work lists and drives the graph's conditional nodes:
//
//   WHILE(any foam still stepping) {
//       predict; pairs; correct              (attempt list)
//       decide
//       IF(any foam deletes) remove          (delete list)
//       IF(any foam searches) search         (search list)
//   }
#include <algorithm>
#include <cstring>
#include <vector>

#include "context.cuh"

using namespace cbg;

namespace {

// Batch-level flags and graph handles (device, one per batch).
struct BatchCtl {
    unsigned long long h_loop, h_delete, h_search;
    int graph_mode;
    int any_attempt, any_delete, any_search;
    long long decides, any_delete_phases, any_search_phases;
};

// Block-wide exclusive scan of one int per thread (blockDim.x a multiple of
// 32, at most 1024); *total receives the block's sum.
__device__ __forceinline__ int block_scan_ex(int v, int *smem, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += t;
    }
    __syncthreads();
    if (lane == 31) smem[warp] = x;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        int w = lane < nw ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) smem[lane] = w;
    }
    __syncthreads();
    *total = smem[(blockDim.x >> 5) - 1];
    return (warp > 0 ? smem[warp - 1] : 0) + x - v;
}

// After every batched attempt (init = 0) or before the first one (init = 1,
// selections as the host set them): the phases each foam takes part in
// next, from its own outcome (the decisions finish_attempt made for it),
// and the work lists of the three phases. One block.
__global__ void __launch_bounds__(1024) k_batch_decide(const Bufs *bb, int count, BatchCtl *bc,
                                                      BatchWork *wk, int init) {
    __shared__ int smem[32];
    __shared__ int carry[3][2];
    if (threadIdx.x < 6) carry[threadIdx.x / 2][threadIdx.x % 2] = 0;
    __syncthreads();
    for (int base = 0; base < count; base += blockDim.x) {
        const int f = base + threadIdx.x;
        int sel = 0, va = 0, vs = 0;
        if (f < count) {
            Ctrl *c = bb[f].ctrl;
            if (init) {
                sel = c->bsel;
            } else if (c->bsel & SEL_ATTEMPT) {
                const int ok = c->status == CB_OK;
                const int accepted = !c->too_large;
                if (ok && accepted && c->need_delete) sel |= SEL_DELETE;
                if (ok && accepted && c->need_search) sel |= SEL_SEARCH;
                if (ok && (c->too_large || (c->steps < c->steps_target && !c->stop_hit)))
                    sel |= SEL_ATTEMPT;
            }
            c->bsel = sel;
            va = c->vgrid_a;
            vs = c->vgrid_s;
        }
        for (int p = 0; p < 3; p++) {
            const int in = (sel >> p) & 1;
            const int vg = in ? (p == 0 ? va : vs) : 0;
            int tn, tt;
            const int en = block_scan_ex(in, smem, &tn);
            const int et = block_scan_ex(vg, smem, &tt);
            const int cn = carry[p][0], ct = carry[p][1];
            if (in) {
                wk[p].foam[cn + en] = f;
                wk[p].pre[cn + en] = ct + et;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                carry[p][0] = cn + tn;
                carry[p][1] = ct + tt;
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        for (int p = 0; p < 3; p++) {
            wk[p].nsel = carry[p][0];
            wk[p].total = carry[p][1];
            wk[p].pre[carry[p][0]] = carry[p][1];
        }
        const int act = carry[0][0] > 0, del = carry[1][0] > 0, srch = carry[2][0] > 0;
        bc->any_attempt = act;
        bc->any_delete = del;
        bc->any_search = srch;
        if (!init) {
            bc->decides += 1;
            bc->any_delete_phases += del;
            bc->any_search_phases += srch;
        }
        if (bc->graph_mode && !init) {
            set_cond(bc->h_delete, del);
            set_cond(bc->h_search, srch);
            set_cond(bc->h_loop, act);
        }
    }
}

}  // namespace

struct cb_batch {
    std::vector<cb_context *> foams;
    int dev = 0;
    cudaStream_t stream = nullptr;
    Bufs *dbufs = nullptr;
    BatchCtl *dbc = nullptr;
    BatchCtl *hbc = nullptr;  // pinned mirror
    BatchWork *dwork = nullptr;  // attempt, delete, search work lists
    int *dlists = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int graph_tile = -1;
    cbg::PhaseKernels graph_kernels;
    int tile = 2048;
    int gmax = 1;  // blocks of every batched launch
    long long launches = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    const cb_context *first() const { return foams[0]; }
    int pull_bc() {
        CB_CUDA(cudaMemcpyAsync(hbc, dbc, sizeof(BatchCtl), cudaMemcpyDeviceToHost, stream));
        CB_CUDA(cudaStreamSynchronize(stream));
        return CB_OK;
    }
    int push_bc() {
        CB_CUDA(cudaMemcpyAsync(dbc, hbc, sizeof(BatchCtl), cudaMemcpyHostToDevice, stream));
        CB_CUDA(cudaStreamSynchronize(stream));
        return CB_OK;
    }
    // The launch parameters of a batched phase (0 attempt, 1 delete, 2 search).
    Launch launch(int phase, long long *counter) const {
        Launch l = first()->launch;
        l.stream = stream;
        l.launches = counter;
        l.batch = dbufs;
        l.work = dwork + phase;
        l.gmax = gmax;
        return l;
    }
};

namespace {

// Virtual grid of a foam: capacity / tile blocks (the attempt's tile is
// tuned; the search and the deletion, which run for few foams at a time,
// use 256 bubbles per block). Partials, block sums and the scan's top level
// are sized for at most launch.grid / launch.scan_grid blocks.
int vgrid_of(const cb_context *c, int tile) {
    const long long cap = c->hk.cap;
    long long g = (cap + tile - 1) / tile;
    g = std::min<long long>(g, std::min(c->launch.grid, c->launch.scan_grid));
    return (int)std::max<long long>(1, g);
}

// One batched attempt, the decision, and (eager mode) the phases the host
// reads back. Graph mode records the same launches into the loop body.
void launch_batch_attempt(const cb_batch *b, long long *counter) {
    const Launch l = b->launch(0, counter);
    launch_attempt_kernels(b->first(), l, b->first()->bufs);
    k_batch_decide<<<1, 1024, 0, b->stream>>>(b->dbufs, (int)b->foams.size(), b->dbc, b->dwork,
                                              0);
    *counter += 1;
}

void launch_batch_remove(const cb_batch *b, long long *counter) {
    launch_remove(b->launch(1, counter), b->first()->bufs, b->first()->hk.dim);
}

void launch_batch_search(const cb_batch *b, long long *counter) {
    launch_search(b->launch(2, counter), b->first()->bufs, b->first()->hk.dim);
}

int build_batch_graph(cb_batch *b) {
    if (b->gexec && b->graph_tile == b->tile) return CB_OK;
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
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
    cudaStream_t s = b->stream;
    CB_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    launch_batch_attempt(b, &dummy);  // the attempt kernels and the decision
    const long long n_attempt = dummy;
    cudaGraph_t delbody, searchbody, out;
    int rc = capture_conditional(s, cudaGraphCondTypeIf, &hdel, 0, &delbody);
    if (!rc) rc = capture_conditional(s, cudaGraphCondTypeIf, &hsearch, 0, &searchbody);
    cudaError_t e = cudaStreamEndCapture(s, &out);
    if (rc) return rc;
    CB_CUDA(e);
    CB_CUDA(cudaStreamBeginCaptureToGraph(s, delbody, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    launch_batch_remove(b, &dummy);
    const long long n_remove = dummy - n_attempt;
    CB_CUDA(cudaStreamEndCapture(s, &out));
    CB_CUDA(cudaStreamBeginCaptureToGraph(s, searchbody, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal));
    launch_batch_search(b, &dummy);
    b->graph_kernels.attempt = n_attempt;
    b->graph_kernels.remove = n_remove;
    b->graph_kernels.search = dummy - n_attempt - n_remove;
    CB_CUDA(cudaStreamEndCapture(s, &out));
    CB_CUDA(cudaGraphInstantiate(&b->gexec, g, 0));
    CB_CUDA(cudaGraphUpload(b->gexec, b->stream));
    CB_CUDA(cudaGraphDestroy(g));
    b->graph_tile = b->tile;
    b->hbc->h_loop = (unsigned long long)hloop;
    b->hbc->h_delete = (unsigned long long)hdel;
    b->hbc->h_search = (unsigned long long)hsearch;
    return CB_OK;
}

}  // namespace

namespace {

int batch_fail_status(cb_batch *b) {
    for (size_t f = 0; f < b->foams.size(); f++) {
        const int st = b->foams[f]->hctrl->status;
        if (st != CB_OK)
            return fail(st, std::string("foam ") + std::to_string(f) + ": " + status_text(st));
    }
    return CB_OK;
}

int batch_integrate(cb_batch *b, int64_t n_steps, cb_report *reports, double *ms) {
    cbg::note_call();  // runs every foam's kernels
    NvtxRange nv("Batch integration");
    CB_CUDA(cudaSetDevice(b->dev));
    if (n_steps < 0) return fail(CB_ERR_INVALID_ARGUMENT, "n_steps must be >= 0");
    const int mode0 = b->first()->mode();
    const bool graph = b->first()->cfg.use_graph != 0;
    // work items loop over a fixed grid of resident blocks
    b->gmax = b->first()->launch.grid;
    for (size_t f = 0; f < b->foams.size(); f++) {
        cb_context *c = b->foams[f];
        if (!c->loaded) return fail(CB_ERR_STATE, "foam " + std::to_string(f) + " has no state");
        int rc = c->pull();
        if (rc) return rc;
        Ctrl &h = *c->hctrl;
        if (c->mode() != mode0)
            return fail(CB_ERR_INVALID_ARGUMENT, "foams of a batch need the same gas/flow options");
        h.steps_target = h.steps + n_steps;
        h.graph_mode = 0;
        h.bsel = (h.status == CB_OK && n_steps > 0) ? SEL_ATTEMPT : 0;
        h.vgrid_a = vgrid_of(c, b->tile);
        h.vgrid_s = vgrid_of(c, 256);
        if ((rc = c->push())) return rc;
    }
    if (graph) {
        int rc = build_batch_graph(b);
        if (rc) return rc;
    }
    b->hbc->graph_mode = graph ? 1 : 0;
    b->hbc->decides = b->hbc->any_delete_phases = b->hbc->any_search_phases = 0;
    int rc = b->push_bc();
    if (rc) return rc;
    k_batch_decide<<<1, 1024, 0, b->stream>>>(b->dbufs, (int)b->foams.size(), b->dbc, b->dwork, 1);
    CB_CUDA(cudaGetLastError());
    CB_CUDA(cudaEventRecord(b->ev0, b->stream));
    if (n_steps > 0) {
        if (graph) {
            CB_CUDA(cudaGraphLaunch(b->gexec, b->stream));
        } else {
            for (;;) {
                launch_batch_attempt(b, &b->launches);
                CB_CUDA(cudaGetLastError());
                if ((rc = b->pull_bc())) return rc;
                if (b->hbc->any_delete) launch_batch_remove(b, &b->launches);
                if (b->hbc->any_search) launch_batch_search(b, &b->launches);
                CB_CUDA(cudaGetLastError());
                if (!b->hbc->any_attempt) break;
            }
        }
    }
    CB_CUDA(cudaEventRecord(b->ev1, b->stream));
    CB_CUDA(cudaEventSynchronize(b->ev1));
    if (ms) {
        float t = 0.f;
        CB_CUDA(cudaEventElapsedTime(&t, b->ev0, b->ev1));
        *ms = t;
    }
    if ((rc = b->pull_bc())) return rc;
    for (size_t f = 0; f < b->foams.size(); f++) {
        cb_context *c = b->foams[f];
        if ((rc = c->pull())) return rc;
        if (reports) fill_report(c, reports + f);
    }
    if (graph && n_steps > 0) {
        // attempt kernels + decide per loop iteration; a remove / search
        // phase is one launch of each of its kernels for all foams together
        b->launches += b->hbc->decides * b->graph_kernels.attempt;
        b->launches += b->hbc->any_delete_phases * b->graph_kernels.remove;
        b->launches += b->hbc->any_search_phases * b->graph_kernels.search;
    }
    return batch_fail_status(b);
}

}  // namespace

extern "C" {

int cb_batch_create(const cb_config *cfgs, int32_t count, cb_batch **out) {
    if (!cfgs || !out) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    if (count < 1) return fail(CB_ERR_INVALID_ARGUMENT, "count must be positive");
    auto any_wall = [](const cb_config &c) {
        return (c.wall[0] || c.wall[1] || (c.dimensionality == 3 && c.wall[2])) ? 1 : 0;
    };
    for (int f = 1; f < count; f++) {
        const cb_config &a = cfgs[0], &c = cfgs[f];
        if (c.dimensionality != a.dimensionality || c.precision != a.precision ||
            (c.use_gas_exchange != 0) != (a.use_gas_exchange != 0) ||
            (c.use_flow != 0) != (a.use_flow != 0) || any_wall(c) != any_wall(a))
            return fail(CB_ERR_INVALID_ARGUMENT,
                        "foams of a batch need the same dimensionality, precision, gas/flow "
                        "options and wall presence");
    }
    cb_batch *b = new cb_batch();
    auto bail = [&](int code) {
        std::string msg = cb_last_error();
        cb_batch_destroy(b);
        fail(code, msg);
        return code;
    };
    for (int f = 0; f < count; f++) {
        cb_context *c = nullptr;
        int rc = cbg::create_context(cfgs + f, &c, false);
        if (rc) return bail(rc);
        b->foams.push_back(c);
    }
    b->dev = b->foams[0]->dev;
    for (cb_context *c : b->foams)
        if (c->dev != b->dev) return bail(fail(CB_ERR_INVALID_ARGUMENT, "foams on different devices"));
    if (cudaSetDevice(b->dev) != cudaSuccess) return bail(fail(CB_ERR_CUDA, "cudaSetDevice"));
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(CB_ERR_CUDA, "cudaStreamCreate"));
    cudaEventCreate(&b->ev0);
    cudaEventCreate(&b->ev1);
    if (cudaMalloc(&b->dbufs, sizeof(Bufs) * count) != cudaSuccess ||
        cudaMalloc(&b->dbc, sizeof(BatchCtl)) != cudaSuccess ||
        cudaMallocHost(&b->hbc, sizeof(BatchCtl)) != cudaSuccess ||
        cudaMalloc(&b->dwork, sizeof(BatchWork) * 3) != cudaSuccess ||
        cudaMalloc(&b->dlists, sizeof(int) * 3 * (2 * (size_t)count + 1)) != cudaSuccess)
        return bail(fail(CB_ERR_CUDA, "batch allocation"));
    BatchWork hw[3];
    for (int p = 0; p < 3; p++) {
        hw[p].nsel = hw[p].total = 0;
        hw[p].foam = b->dlists + (size_t)p * (2 * count + 1);
        hw[p].pre = hw[p].foam + count;
    }
    if (cudaMemcpy(b->dwork, hw, sizeof(hw), cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(CB_ERR_CUDA, "batch work lists"));
    std::memset(b->hbc, 0, sizeof(BatchCtl));
    std::vector<Bufs> hb(count);
    for (int f = 0; f < count; f++) hb[f] = b->foams[f]->bufs;
    if (cudaMemcpy(b->dbufs, hb.data(), sizeof(Bufs) * count, cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return bail(fail(CB_ERR_CUDA, "batch table upload"));
    if (b->push_bc()) return bail(CB_ERR_CUDA);
    *out = b;
    return CB_OK;
}

int cb_batch_destroy(cb_batch *b) {
    if (!b) return CB_OK;
    cudaSetDevice(b->dev);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->dbufs) cudaFree(b->dbufs);
    if (b->dbc) cudaFree(b->dbc);
    if (b->dwork) cudaFree(b->dwork);
    if (b->dlists) cudaFree(b->dlists);
    if (b->hbc) cudaFreeHost(b->hbc);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    for (cb_context *c : b->foams) cb_destroy(c);
    delete b;
    return CB_OK;
}

int cb_batch_context(cb_batch *b, int32_t index, cb_context **ctx) {
    if (!b || !ctx) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    if (index < 0 || index >= (int)b->foams.size())
        return fail(CB_ERR_INVALID_ARGUMENT, "foam index out of range");
    *ctx = b->foams[index];
    return CB_OK;
}

int cb_batch_integrate(cb_batch *b, int64_t n_steps, cb_report *reports) {
    if (!b) return fail(CB_ERR_INVALID_ARGUMENT, "null batch");
    return batch_integrate(b, n_steps, reports, nullptr);
}

int cb_batch_integrate_timed(cb_batch *b, int64_t n_steps, cb_report *reports, double *ms) {
    if (!b || !ms) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    return batch_integrate(b, n_steps, reports, ms);
}

int cb_batch_set_tile(cb_batch *b, int32_t tile) {
    if (!b) return fail(CB_ERR_INVALID_ARGUMENT, "null batch");
    if (tile < 256 || tile % 256) return fail(CB_ERR_INVALID_ARGUMENT, "tile must be a multiple of 256");
    b->tile = tile;
    return CB_OK;
}

int cb_batch_set_tuning(cb_batch *b, const cb_tuning *t) {
    if (!b || !t) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    for (cb_context *c : b->foams) {
        CB_CUDA(cudaSetDevice(c->dev));
        int rc = cbg::apply_tuning(c, *t);
        if (rc) return rc;
    }
    if (b->gexec) {  // the batched graph holds the old launches
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return CB_OK;
}

int cb_batch_autotune(cb_batch *b, int32_t steps, int32_t *tile_out) {
    if (!b || !tile_out) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    if (steps < 1) return fail(CB_ERR_INVALID_ARGUMENT, "steps must be positive");
    std::vector<cb_report> r0(b->foams.size()), r1(b->foams.size());
    // bubble-steps per ms of `steps` steps with the current settings
    auto trial = [&](double *rate) -> int {
        for (size_t f = 0; f < b->foams.size(); f++) {
            int rc = cb_get_report(b->foams[f], &r0[f]);
            if (rc) return rc;
        }
        double ms = 0.0;
        int rc = batch_integrate(b, steps, r1.data(), &ms);
        if (rc) return rc;
        long long bs = 0;
        for (size_t f = 0; f < b->foams.size(); f++) bs += r1[f].bubble_steps - r0[f].bubble_steps;
        *rate = ms > 0.0 ? (double)bs / ms : 0.0;
        return CB_OK;
    };
    double best = -1.0, rate = 0.0;
    int best_tile = b->tile;
    for (int t : {512, 1024, 2048, 4096, 8192}) {
        b->tile = t;
        int rc = trial(&rate);
        if (rc) return rc;
        if (rate > best) {
            best = rate;
            best_tile = t;
        }
    }
    b->tile = best_tile;
    // the cell edge, then the mixed pair kernel's pairs per thread
    cb_tuning bt = b->first()->tune;
    const cb_tuning keep0 = bt;
    best = -1.0;
    for (double cs : {1.0, 1.15, 1.3}) {
        cb_tuning q = keep0;
        q.cell_scale = cs;
        int rc = cb_batch_set_tuning(b, &q);
        if (!rc) rc = trial(&rate);
        if (rc) return rc;
        if (rate > best) {
            best = rate;
            bt = q;
        }
    }
    if (b->first()->hk.mixed) {
        const cb_tuning keep1 = bt;
        best = -1.0;
        for (int run : {2, 4, 8}) {
            cb_tuning q = keep1;
            q.pair_run = run;
            int rc = cb_batch_set_tuning(b, &q);
            if (!rc) rc = trial(&rate);
            if (rc) return rc;
            if (rate > best) {
                best = rate;
                bt = q;
            }
        }
    }
    int rc = cb_batch_set_tuning(b, &bt);
    if (rc) return rc;
    *tile_out = best_tile;
    return CB_OK;
}

int cb_batch_launch_count(cb_batch *b, int64_t *count) {
    if (!b || !count) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    *count = b->launches;
    return CB_OK;
}

}  // extern "C"
