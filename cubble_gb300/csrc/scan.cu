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

__device__ __forceinline__ int read_count(const int *count_ptr, int add) {
    return *count_ptr + add;
}

__global__ void __launch_bounds__(kBlock) k_scan_sums(const int *in, const int *count_ptr,
                                                      int add, int *blocksums) {
    __shared__ int smem[32];
    const int count = read_count(count_ptr, add);
    const int chunk = (count + gridDim.x - 1) / gridDim.x;
    const int s = blockIdx.x * chunk;
    const int e = min(s + chunk, count);
    int v = 0;
    for (int i = s + threadIdx.x; i < e; i += blockDim.x) v += in[i];
    v = block_reduce_int(v, smem);
    if (threadIdx.x == 0) blocksums[blockIdx.x] = v;
}

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

__global__ void __launch_bounds__(1024) k_scan_top(int *blocksums, int nblocks) {
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

__global__ void __launch_bounds__(kBlock) k_scan_apply(const int *in, int *out, const int *count_ptr,
                                                       int add, const int *blocksums,
                                                       int *total_out) {
    __shared__ int smem[32];
    __shared__ int carry_s;
    const int count = read_count(count_ptr, add);
    const int chunk = (count + gridDim.x - 1) / gridDim.x;
    const int s = blockIdx.x * chunk;
    const int e = min(s + chunk, count);
    if (threadIdx.x == 0) carry_s = blocksums[blockIdx.x];
    __syncthreads();
    for (int base = s; base < e; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const int v = i < e ? in[i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, smem, &tot);
        const int carry = carry_s;
        if (i < e) out[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + tot;
        __syncthreads();
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        const int total = blocksums[gridDim.x];
        out[count] = total;
        if (total_out) *total_out = total;
    }
}

}  // namespace

void launch_scan(const Launch &l, const Bufs &b, const int *in, int *out, const int *count_ptr,
                 int count_add, int *total_out) {
    k_scan_sums<<<l.scan_grid, kBlock, 0, l.stream>>>(in, count_ptr, count_add, b.blocksums);
    k_scan_top<<<1, 1024, 0, l.stream>>>(b.blocksums, l.scan_grid);
    k_scan_apply<<<l.scan_grid, kBlock, 0, l.stream>>>(in, out, count_ptr, count_add, b.blocksums,
                                                      total_out);
    *l.launches += 3;
}

}  // namespace cbg
