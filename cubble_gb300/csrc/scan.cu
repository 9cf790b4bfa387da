// Device-wide exclusive scan of int32 rows whose length lives in device
// memory, so that the call can sit inside a CUDA graph whose sizes change
// from one execution to the next. Replaces the reference's
// cub::DeviceScan::InclusiveSum calls (src/simulator.cu:90-91, :165-167).
//
// Three launches, no inter-block waiting:
//   1. every block sums one contiguous chunk of the input,
//   2. one block scans the chunk sums,
//   3. every block scans its chunk again and adds its offset.
// Output: out[0..count] with out[count] = total.
#include "common.cuh"

namespace cbg {
namespace {

// What a scan reads and writes, per use in the search and the deletion.
struct ScanIO {
    const int *in;
    int *out;
    int count;
    int *total_out;
};

__device__ __forceinline__ ScanIO scan_io(const Bufs &b, int kind) {
    Ctrl *c = b.ctrl;
    switch (kind) {
        case SCAN_CELLS: return {b.cellCount, b.cellStart, c->ncell, nullptr};
        case SCAN_ROWS: return {b.rowCount, b.rowStart, c->n, &c->np_found};
        case SCAN_DEL: return {b.delflag, b.iscan, c->n, nullptr};
        default: return {b.keep, b.keepScan, c->np, nullptr};
    }
}

template <int KIND>
__device__ __forceinline__ void k_scan_sums_body(const Bufs &b, const int vb, const int vg) {
    __shared__ int smem[32];
    const ScanIO io = scan_io(b, KIND);
    const int chunk = (io.count + vg - 1) / vg;
    const int s = vb * chunk;
    const int e = min(s + chunk, io.count);
    int v = 0;
    for (int i = s + threadIdx.x; i < e; i += blockDim.x) v += io.in[i];
    v = block_reduce_int(v, smem);
    if (threadIdx.x == 0) b.blocksums[vb] = v;
}
CB_KERNEL_PAIR((template <int KIND>), k_scan_sums, (<KIND>), __launch_bounds__(kBlock))

// Block-wide exclusive scan; returns the exclusive prefix of `v` and writes
// the block total into *total.
__device__ __forceinline__ int block_exclusive_scan(int v, int *smem, int *total) {
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
        if (lane < nw) smem[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const int warp_off = warp > 0 ? smem[warp - 1] : 0;
    *total = smem[(blockDim.x >> 5) - 1];
    return warp_off + x - v;
}

__device__ __forceinline__ void k_scan_top_body(int *blocksums, int nblocks) {
    __shared__ int smem[32];
    __shared__ int carry_s;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    for (int base = 0; base < nblocks; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < nblocks ? blocksums[i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, smem, &tot);
        const int carry = carry_s;
        if (i < nblocks) blocksums[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) blocksums[nblocks] = carry_s;
}

__global__ void __launch_bounds__(1024) k_scan_top(int *blocksums, int nblocks) {
    k_scan_top_body(blocksums, nblocks);
}

// Batched form: the selected foams in turn, over their virtual grids' sums.
__global__ void __launch_bounds__(1024) k_scan_top_batch(const Bufs *bb, const BatchWork *wk) {
    for (int k = blockIdx.x; k < wk->nsel; k += gridDim.x) {
        k_scan_top_body(bb[wk->foam[k]].blocksums, wk->pre[k + 1] - wk->pre[k]);
        __syncthreads();
    }
}

template <int KIND>
__device__ __forceinline__ void k_scan_apply_body(const Bufs &b, const int vb, const int vg) {
    __shared__ int smem[32];
    __shared__ int carry_s;
    const ScanIO io = scan_io(b, KIND);
    const int chunk = (io.count + vg - 1) / vg;
    const int s = vb * chunk;
    const int e = min(s + chunk, io.count);
    if (threadIdx.x == 0) carry_s = b.blocksums[vb];
    __syncthreads();
    for (int base = s; base < e; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < e ? io.in[i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, smem, &tot);
        const int carry = carry_s;
        if (i < e) io.out[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + tot;
        __syncthreads();
    }
    if (vb == vg - 1 && threadIdx.x == 0) {
        const int total = b.blocksums[vg];
        io.out[io.count] = total;
        if (io.total_out) *io.total_out = total;
    }
}
CB_KERNEL_PAIR((template <int KIND>), k_scan_apply, (<KIND>), __launch_bounds__(kBlock))

template <int KIND>
void launch_scan_t(const Launch &l, const Bufs &b) {
    CB_LAUNCH(l, k_scan_sums, (<KIND>), l.scan_grid, b);
    if (l.batch)
        k_scan_top_batch<<<l.sms, 1024, 0, l.stream>>>(l.batch, l.work);
    else
        k_scan_top<<<1, 1024, 0, l.stream>>>(b.blocksums, l.scan_grid);
    *l.launches += 1;
    CB_LAUNCH(l, k_scan_apply, (<KIND>), l.scan_grid, b);
}

}  // namespace

void launch_scan(const Launch &l, const Bufs &b, int kind) {
    switch (kind) {
        case SCAN_CELLS: launch_scan_t<SCAN_CELLS>(l, b); break;
        case SCAN_ROWS: launch_scan_t<SCAN_ROWS>(l, b); break;
        case SCAN_DEL: launch_scan_t<SCAN_DEL>(l, b); break;
        default: launch_scan_t<SCAN_KEEP>(l, b); break;
    }
}

}  // namespace cbg
