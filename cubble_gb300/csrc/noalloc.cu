// cb_energy_noalloc: total potential energy of a foam for callers that must
// not allocate device memory.
//
// Some callers cannot call cudaMalloc: applications whose device memory is
// owned by their own pool or arena (a host code that hands out every byte of
// HBM itself), or code running where an allocation would synchronise the
// device or is forbidden (inside a tight time-stepping loop of another
// solver). They own the input rows and the output; this entry point brings
// its scratch with it: one file-scope static __device__ array, sized for at
// most kMaxBubbles bubbles, that every GPU loading the library keeps until
// the process exits.
//
// Same arithmetic as potentialEnergy + the per-bubble sum of totalEnergy
// (src/kernels.cu:941-957, src/simulator.cu:39-58): per pair
// e = r_i + r_j - |d| (minimum image), e^2 added to both bubbles when e > 0,
// then the per-bubble energies are summed.
#include <string>

#include "common.cuh"

namespace cbg {
void set_last_error(const std::string &msg);
}

namespace {

using namespace cbg;

constexpr int kMaxBubbles = 1 << 18;  // 262,144 bubbles
constexpr int kBlocks = 512;          // reduction blocks (fixed)
// [0, kMaxBubbles): per-bubble energies; [kMaxBubbles, +kBlocks): block
// partials; then the last-block counter and the count of rejected pairs
// (pairs with an index outside [0, count)), one word each.
constexpr int kDoneWord = kMaxBubbles + kBlocks;
constexpr int kBadWord = kDoneWord + 1;
constexpr int kScratchWords = kBadWord + 1;

static __device__ __align__(256) double g_scratch[kScratchWords];

struct Box {
    int dim;
    int wall[3];
    double iv[3];
};

__global__ void __launch_bounds__(kBlock) k_na_clear(double *s, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        s[i] = 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *reinterpret_cast<unsigned int *>(s + kDoneWord) = 0u;
        *reinterpret_cast<unsigned int *>(s + kBadWord) = 0u;
    }
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_na_pairs(Box box, const double *X, const double *Y,
                                                     const double *Z, const double *R,
                                                     const int *PI, const int *PJ, int np,
                                                     int n, double *s) {
    DevConst k{};
    for (int a = 0; a < 3; a++) {
        k.wall[a] = box.wall[a];
        k.iv[a] = box.iv[a];
    }
    unsigned int bad = 0u;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int i = PI[p], j = PJ[p];
        // the indices come from the caller: one outside [0, n) would read
        // past the caller's rows and add into scratch words that are not
        // per-bubble energies, so it is skipped and counted instead
        if ((unsigned)i >= (unsigned)n || (unsigned)j >= (unsigned)n) {
            bad++;
            continue;
        }
        double dx, dy, dz;
        wrapped_diff<DIM>(k, X[i], Y[i], DIM == 3 ? Z[i] : 0.0, X[j], Y[j],
                          DIM == 3 ? Z[j] : 0.0, dx, dy, dz);
        double m = dx * dx + dy * dy;
        if (DIM == 3) m += dz * dz;
        double e = R[i] + R[j] - sqrt(m);
        if (e > 0) {
            e *= e;
            atomicAdd(s + i, e);
            atomicAdd(s + j, e);
        }
    }
    if (bad) atomicAdd(reinterpret_cast<unsigned int *>(s + kBadWord), bad);
}

__global__ void __launch_bounds__(kBlock) k_na_sum(double *s, int n, double *out) {
    __shared__ double smem[32];
    // contiguous chunk per block, summed in a fixed order
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int b0 = blockIdx.x * chunk, b1 = min(b0 + chunk, n);
    double v = 0.0;
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) v += s[i];
    const double t = block_reduce(v, OpSum(), smem);
    double *part = s + kMaxBubbles;
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    unsigned int *done = reinterpret_cast<unsigned int *>(s + kDoneWord);
    if (last_block(done, gridDim.x)) {
        const double f = fold_partials(part, gridDim.x, false, smem);
        if (threadIdx.x == 0) {
            const unsigned int bad = *reinterpret_cast<volatile unsigned int *>(s + kBadWord);
            *out = bad ? __longlong_as_double(0x7ff8000000000000LL) : f;  // NaN: bad pairs
            *done = 0u;
        }
    }
}

// The device address of g_scratch for the current device and context, looked
// up on every call: after the module is loaded this is a host-side lookup,
// and it stays right when the caller has reset the device or switched to
// another context since the last call. Host code must not use &g_scratch
// itself: on the host it names a stand-in, not device memory.
int scratch_for_current_device(double **out) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
        set_last_error(std::string("cudaGetSymbolAddress(g_scratch): ") + cudaGetErrorString(e));
        return CB_ERR_CUDA;
    }
    *out = static_cast<double *>(p);
    return CB_OK;
}

}  // namespace

extern "C" int cb_energy_noalloc(const cb_config *cfg, const double *x, const double *y,
                                 const double *z, const double *r, const int32_t *pair_i,
                                 const int32_t *pair_j, int32_t count, int32_t num_pairs,
                                 double *energy_out, void *stream) {
    if (!cfg || !x || !y || !r || !energy_out || (num_pairs > 0 && (!pair_i || !pair_j))) {
        set_last_error("cb_energy_noalloc: null pointer");
        return CB_ERR_INVALID_ARGUMENT;
    }
    if (cfg->dimensionality != 2 && cfg->dimensionality != 3) {
        set_last_error("cb_energy_noalloc: dimensionality must be 2 or 3");
        return CB_ERR_INVALID_ARGUMENT;
    }
    if (cfg->dimensionality == 3 && !z) {
        set_last_error("cb_energy_noalloc: z is required in 3D");
        return CB_ERR_INVALID_ARGUMENT;
    }
    if (count < 0 || num_pairs < 0) {
        set_last_error("cb_energy_noalloc: negative size");
        return CB_ERR_INVALID_ARGUMENT;
    }
    if (count > kMaxBubbles) {
        set_last_error("cb_energy_noalloc: " + std::to_string(count) +
                       " bubbles exceed the static scratch limit of " +
                       std::to_string(kMaxBubbles));
        return CB_ERR_CAPACITY;
    }
    double *s = nullptr;
    int rc = scratch_for_current_device(&s);
    if (rc != CB_OK) return rc;
    Box box{};
    box.dim = cfg->dimensionality;
    for (int a = 0; a < 3; a++) {
        box.wall[a] = cfg->wall[a] ? 1 : 0;
        box.iv[a] = cfg->tfr[a] - cfg->lbb[a];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int grid = kBlocks;
    k_na_clear<<<grid, kBlock, 0, st>>>(s, count);
    if (box.dim == 3)
        k_na_pairs<3><<<grid, kBlock, 0, st>>>(box, x, y, z, r, pair_i, pair_j, num_pairs,
                                               count, s);
    else
        k_na_pairs<2><<<grid, kBlock, 0, st>>>(box, x, y, z, r, pair_i, pair_j, num_pairs,
                                               count, s);
    k_na_sum<<<grid, kBlock, 0, st>>>(s, count, energy_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(std::string("cb_energy_noalloc launch: ") + cudaGetErrorString(e));
        return CB_ERR_CUDA;
    }
    return CB_OK;
}
