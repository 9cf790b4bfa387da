// Host-side internals shared by the single-foam context (context.cu) and
// the batched foams (batch.cu). Not part of the C ABI.
#pragma once

#include <atomic>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace cbg {
int fail(int code, const std::string &msg);
const char *status_text(int s);
// Kernels per phase of a captured graph (attempt, removal, search), counted
// while the graph is captured; graph executions add them to the launch
// counter per attempt, deletion and search the device reports.
struct PhaseKernels {
    long long attempt = 0, remove = 0, search = 0;
};
// Count of C-ABI calls that may touch a context, process wide: a context
// whose host mirror was left current by a call knows, by this count, that no
// call has run since.
extern std::atomic<unsigned long long> g_calls;
inline unsigned long long note_call() { return g_calls.fetch_add(1, std::memory_order_relaxed) + 1; }
}  // namespace cbg

#define CB_CUDA(x)                                                                          \
    do {                                                                                    \
        cudaError_t e_ = (x);                                                               \
        if (e_ != cudaSuccess)                                                              \
            return cbg::fail(CB_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));      \
    } while (0)

using cbg::Bufs;
using cbg::Ctrl;
using cbg::DevConst;
using cbg::Launch;

struct cb_context {
    cb_config cfg{};
    int dev = 0, sms = 0;
    cudaStream_t stream = nullptr;
    DevConst hk{};
    DevConst *dk = nullptr;
    Ctrl *dctrl = nullptr;
    Ctrl *hctrl = nullptr;  // pinned mirror
    std::vector<void *> allocs;
    double *dslot[cbg::ND_ROLES] = {};
    int *islot[cbg::NI_ROLES] = {};
    int *pslot[cbg::NP_ROLES] = {};
    double **d_dslots = nullptr;
    int **d_islots = nullptr;
    int **d_pslots = nullptr;
    Bufs bufs{};
    Launch launch{};
    long long launches = 0;
    bool loaded = false;
    cudaGraphExec_t gexec = nullptr;
    int graph_key = -1;
    cbg::PhaseKernels graph_kernels;
    long long graph_attempts0 = 0, graph_searches0 = 0, graph_deletes0 = 0;
    // g_calls when a graph cb_integrate returned with hctrl equal to the
    // device's control block and the stream idle
    unsigned long long mirror_call = ~0ull;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // launch / search knobs (cb_tuning); their launch parts live in `launch`
    cb_tuning tune{1.0, 4, 0, 0, 0};

    template <typename T>
    int alloc(T **p, size_t n) {
        void *q = nullptr;
        CB_CUDA(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
        CB_CUDA(cudaMemsetAsync(q, 0, std::max<size_t>(n, 1) * sizeof(T), stream));
        allocs.push_back(q);
        *p = static_cast<T *>(q);
        return CB_OK;
    }
    int pull() {
        CB_CUDA(cudaMemcpyAsync(hctrl, dctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, stream));
        CB_CUDA(cudaStreamSynchronize(stream));
        return CB_OK;
    }
    int push() {
        CB_CUDA(cudaMemcpyAsync(dctrl, hctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, stream));
        CB_CUDA(cudaStreamSynchronize(stream));
        return CB_OK;
    }
    int upload_const() {
        CB_CUDA(cudaMemcpyAsync(dk, &hk, sizeof(DevConst), cudaMemcpyHostToDevice, stream));
        CB_CUDA(cudaStreamSynchronize(stream));
        return CB_OK;
    }
    // kernel variant: bit 1 gas exchange, bit 2 the box-region flow (its
    // neighbour sums); the shear flow needs no pair work
    int mode() const {
        return (hctrl->use_gas ? 1 : 0) | (hctrl->use_flow && !hk.shear_on ? 2 : 0);
    }
    int check_launch() {
        CB_CUDA(cudaGetLastError());
        return CB_OK;
    }
};

namespace cbg {
// NVTX range over a scope, named like the reference's ranges
// (src/simulator.cu:40-376); costs nothing without a tool attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

int sync_status(cb_context *c);
int invalidate_prediction(cb_context *c);
void launch_attempt_kernels(const cb_context *c, const Launch &l, const Bufs &b, int which = 7);
int capture_conditional(cudaStream_t stream, cudaGraphConditionalNodeType type,
                        cudaGraphConditionalHandle *handle, unsigned int dflt,
                        cudaGraph_t *body);
void fill_report(const cb_context *c, cb_report *r);
int create_context(const cb_config *cfg, cb_context **out, bool graph);
int apply_tuning(cb_context *c, const cb_tuning &t);
}  // namespace cbg
