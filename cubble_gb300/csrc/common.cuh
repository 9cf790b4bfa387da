// Shared device-side definitions of the GB300 Durian foam step.
//
// Memory layout in HBM (one context):
//   * persistent per-bubble rows are FP64 / int32 SoA "slots" of `capacity`
//     elements; which slot plays which role (current x, corrected x, the
//     three velocity generations, ...) lives in the device control block, so
//     buffer rotation after an accepted step (src/simulator.cu:258-301) and
//     the cell-order permutation of a search (src/simulator.cu:96-147) are
//     role swaps done on the device; no host round trip is needed;
//   * `pred` packs the predicted state of a bubble into one 32-byte sector
//     (3D: xp,yp,zp,rp; 2D: xp,yp,rp,1/rp) because the pair kernel gathers
//     it for both members of every pair;
//   * `acc` holds 8 FP64 accumulators per bubble (64 bytes: vx,vy,vz,vr,
//     overlap, flow vx,vy,vz) that the pair kernel adds into with FP64
//     atomics; it is all zero between attempts (the correct kernel reads
//     and clears it);
//   * pairs are two int32 rows (i, j), double-buffered for compaction.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/cubble_gb300.h"
#include "ff.cuh"

namespace cbg {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993;
constexpr int kBlock = 256;  // threads per block of every grid-stride kernel
constexpr int kAcc = 8;      // FP64 accumulators per bubble
constexpr int kPartSlots = 8;
// Partners j > i per bubble the search's counting pass keeps (a bubble with
// more sends the search through its second enumeration pass).
__host__ __device__ constexpr int kStash(int dim) { return dim == 3 ? 32 : 16; }

// Double-row roles (slot table indices are in Ctrl::drole).
enum DRole : int {
    RX = 0, RY, RZ, RR,          // current position and radius
    RXN, RYN, RZN, RRN,          // corrected (next) position and radius
    RV0, RV1, RV2, RV3,          // dxdt, dydt, dzdt, drdt
    RVO0, RVO1, RVO2, RVO3,      // dxdto ... (previous step)
    RVP0, RVP1, RVP2, RVP3,      // dxdtp ... (this attempt)
    RPATH, RPATHN, RERR, RERR2,  // path, pathNew, error, spare
    RS0, RS1, RS2, RS3,          // saved position / radius of the last search
    RVQ0, RVQ1, RVQ2, RVQ3,      // spares: the search's gather of the previous rates
    ND_ROLES
};
enum IRole : int {
    IWX = 0, IWY, IWZ, IIDX, INN,  // wrap counts, index, numNeighbors
    IWX2, IWY2, IWZ2, IIDX2,       // spares for the permutation
    NI_ROLES
};
enum PRole : int { PI0 = 0, PJ0, PI1, PJ1, NP_ROLES };

// Counters of the "last block finishes the reduction" pattern.
enum DoneCounter : int {
    DC_PREDICT = 0, DC_PAIRS, DC_CORRECT, DC_WRAP, DC_PERMUTE, DC_REMOVE,
    DC_SCAN, DC_MISC, DC_COUNT
};

// Values that change only through cb_set_box / cb_create.
struct DevConst {
    int dim;
    int wall[3];
    int any_wall;
    int max_attempts;
    int cap, pcap, ccap;
    int pad_;
    double lbb[3], tfr[3], iv[3];
    double flow_lbb[3], flow_tfr[3], flow_vel[3];
    double wall_drag, min_rad, f0, K, kappa, skin, vol_mul_const, ain, tol;
    double half_iv[3];
    // Mixed form: 64-bit fixed-point coordinates q = x * 2^40 (see
    // step_mixed.cu); lq / hq are the periodic box length and half of it in
    // those units.
    long long lq[3], hq[3];
    int mixed;
    float f0_f;  // f0/mu0 as FP32
    float f0_l;  // f0/mu0 - f0_f: the float-float f0 of k_pairs_ff
    // FP32 copies for the search's candidate tests (a double -> float
    // conversion is an FP64-pipe instruction)
    float skin_f, lbb_f[3];
    int ffpair;  // CB_PRECISION_FP64_FF: pair terms in float-float
    float kq_f;  // K / (4 pi) in 3D, K / (2 pi) in 2D, as FP32
    float pre_margin;  // FP32 pair-search prefilter margin (length units)
    long long lbq[3];  // the box's lower corner in fixed point (x 2^40)
    int fix_range;     // box corners within 2^21: coordinates fit the fixed point
    float half_iv32[3];
    float iv32[3];
    // Linear shear flow (cb_config.shear_speed): v_x += shear (2 (q - lbb_q)
    // / L_q - 1) on the last axis q; shear_il = 2 / L_q.
    int shear_on, shear_axis;
    double shear, shear_il;
    float shear_f, shear_il_f;
    // Cell edge of the neighbour search in units of 2 maxR + skin (>= 1; a
    // tuning knob, cb_tuning.cell_scale)
    double cell_scale;
};

// Device control block. The host reads it after each eager phase or at the
// end of a graph launch (one small copy).
struct Ctrl {
    int n, np, ndel, status;
    int use_gas, use_flow, inc_path, graph_mode;
    double dt;
    double sumA, sumAr, sumAo, sumAor;
    double max_err, max_rad, max_exp, vol_new;
    double max_bubble_radius;
    int too_large, need_search, need_delete, attempts_this_step;
    unsigned long long tint;
    double tfrac;
    long long steps, attempts, searches, deleted, bubble_steps;
    long long steps_target;
    long long delete_events;  // removeBubbles() calls
    unsigned long long h_loop, h_delete, h_search;  // conditional handles
    int drole[ND_ROLES];
    int irole[NI_ROLES];
    int prole[NP_ROLES];
    int cell_dims[3];
    int ncell;
    int nnew;
    int np_found;        // pairs found by the last search (may exceed capacity)
    int no_accept;       // cb_attempt: decide dt but do not accept
    double misc_result;  // energy / volume results
    double mfa, mfb;     // mean-field factors of the attempt (src/kernels.cu:399-404)
    // Order-independent attempt reductions of the one-bubble-per-thread
    // correct kernel: maxima as 64-bit patterns of doubles >= 0 and counts;
    // zero between attempts (the kernel's last block reads and clears them).
    long long amax_err, amax_rad, amax_exp;
    int acnt_del, acnt_bad;
    // Batched launches (several foams per launch): which phases this foam
    // takes part in next (BatchSel bits, set between launches) and the
    // blocks of its virtual grid in the attempt and in the search / deletion.
    int bsel, vgrid_a, vgrid_s;
    int stash_over;    // a row of the last search exceeded kStash partners
    int sparse_cells;  // < 24 bubbles per cell: thread-per-bubble pair pass
    float search_maxr;  // the search's largest radius, rounded up to FP32
    // Mixed form: the correct kernel also writes the next attempt's
    // prediction for both dt it can have after an accept (unchanged, x1.269)
    // with their area sums; pred_ready says the prediction for the coming
    // attempt is in slot pred_slot (0 = pred, 1 / 2 = the candidates).
    int pred_ready, pred_slot;
    double cand_sumA[2], cand_sumAr[2];
    // Stop conditions of cb_integrate_until, checked after every accepted
    // step (simulate()'s loop, src/simulator.cu:1002-1011 and the print and
    // snapshot times of :1017-1029, :1090-1104): time >= (stop_tint,
    // stop_tfrac), bubbles left <= stop_nmin, largest radius >= stop_rmax.
    int stop_on, stop_hit;
    int stop_nmin, pad_stop;
    unsigned long long stop_tint;
    double stop_tfrac, stop_rmax;
    // Smallest, largest and summed dt after the accepted steps since the
    // last reset (simulate()'s min / max / avg ts, src/simulator.cu:1013-1016).
    double dt_min, dt_max, dt_sum;
    unsigned int done[DC_COUNT];
};

// Every device buffer of a context; kernels take it by value.
struct Bufs {
    Ctrl *ctrl;
    const DevConst *k;
    double *const *ds;  // double slots
    int *const *is;     // int slots
    int *const *ps;     // pair slots
    double *pred;       // 4 doubles per bubble
    double *predc;      // mixed form: two candidate predictions, 8 doubles per bubble
    double *invr;       // FP64 form, 3D: (1 / rp, rp^2) per bubble
    float4 *ffr;        // CB_PRECISION_FP64_FF: float-float (rp, 1 / rp), (rp^2, 0)
    double *acc;        // kAcc doubles per bubble
    double *part;       // kPartSlots x grid partials
    int *delflag;       // deletion marks of the last attempt
    int *iscan;         // cap + 1 scan output
    int *blocksums;     // grid + 1
    int *cellOf;        // cell of each bubble (old order)
    int *cellSorted;    // cell of each bubble (cell order)
    int *perm;          // new position -> old position (atomic order)
    int *permSorted;    // new position -> old position (sorted in cell)
    int *cellCount;     // ccap + 1
    int *cellStart;     // ccap + 1
    int *cellFill;      // ccap + 1
    int *rowCount;      // cap + 1
    int *rowStart;      // cap + 1
    float4 *pos32;      // FP32 copy of x, y, z, r for the search prefilter
    float4 *pos32r;     // the same with x, y, z relative to the bubble's cell (3D tile pass)
    int *holes;         // cap
    int *moveDst;       // cap
    int *keep;          // pcap + 1
    int *keepScan;      // pcap + 1
    int *stash;         // cap x kStash(dim): pair partners found by the counting pass
    double *dbg_ov;     // optional copy of the overlap row (cb_attempt)
    double *energy;     // per-bubble energies
};

// ------------------------------------------------------------- helpers
__device__ __forceinline__ double *drow(const Bufs &b, const Ctrl *c, int role) {
    return b.ds[c->drole[role]];
}
__device__ __forceinline__ int *irow(const Bufs &b, const Ctrl *c, int role) {
    return b.is[c->irole[role]];
}

// 64-bit fixed point x * 2^40 (the mixed form's predicted positions, the
// search's cell-relative coordinates), converted on the integer pipe: GB300
// runs every 64-bit conversion on its 1/64-rate FP64 unit.
constexpr int kFixBits = 40;
constexpr float kFixInv = 9.094947017729282e-13f;  // 2^-40

// x * 2^40 rounded toward zero, from the bits of x (|x| < 2^23).
__device__ __forceinline__ long long fix_from_double(double x) {
    const long long b = __double_as_longlong(x);
    const int e = (int)(((unsigned long long)b >> 52) & 0x7ff);
    const long long m = (b & 0x000fffffffffffffLL) | 0x0010000000000000LL;
    const int sh = e - (1075 - kFixBits);  // x = m 2^(e - 1075)
    long long q = sh >= 0 ? (m << min(sh, 10)) : (sh > -64 ? (m >> -sh) : 0LL);
    if (e == 0) q = 0;
    return b < 0 ? -q : q;
}

// A fixed-point difference in length units as FP32: |d| = hi 2^32 + lo with
// two 32-bit conversions (the 64-bit one would take the FP64 unit); relative
// error below 2^-23.
__device__ __forceinline__ float len_from_fix(long long d) {
    const unsigned long long a = (unsigned long long)(d < 0 ? -d : d);
    const float f = fmaf(__uint2float_rn((unsigned int)(a >> 32)), 4294967296.f,
                         __uint2float_rn((unsigned int)a));
    return (d < 0 ? -f : f) * kFixInv;
}

// Row pointers of the correct kernels come from a per-block table in shared
// memory, fetched at each use with a volatile load: a grid-stride loop would
// otherwise keep all ~27 role-resolved 64-bit pointers in registers across
// its iterations (mixed form, 3D: 119 registers and two blocks per SM; with
// the table 64 registers and four blocks per SM).
__device__ __forceinline__ void *tab_ptr(const unsigned long long *tab, int r) {
    unsigned long long p;
    asm volatile("ld.shared.u64 %0, [%1];"
                 : "=l"(p)
                 : "r"((unsigned int)__cvta_generic_to_shared(tab + r)));
    return reinterpret_cast<void *>(p);
}

// Deterministic block reduction (fixed tree for a fixed blockDim).
template <typename Op>
__device__ __forceinline__ double block_reduce(double v, Op op, double *smem,
                                               double identity = 0.0) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    double r = 0.0;
    if (warp == 0) {
        r = lane < nw ? smem[lane] : identity;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r = op(r, __shfl_down_sync(0xffffffffu, r, o));
    }
    return r;  // valid in thread 0
}

struct OpSum {
    __device__ __forceinline__ double operator()(double a, double b) const { return a + b; }
};
struct OpMax {
    __device__ __forceinline__ double operator()(double a, double b) const { return fmax(a, b); }
};

__device__ __forceinline__ int block_reduce_int(int v, int *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    int r = 0;
    if (warp == 0) {
        r = lane < nw ? smem[lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;
}

// Block sum of FP32 values: FP32 inside each warp (no FP64 instruction per
// thread), FP64 across the warps. Result valid in thread 0.
__device__ __forceinline__ double block_sum_f(float v, double *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) smem[warp] = (double)v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r += smem[w];
    return r;
}

// Block maximum of 64-bit patterns (doubles >= 0 order like their bits).
__device__ __forceinline__ long long block_max_bits(long long v, long long *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    long long r = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) r = max(r, smem[w]);
    return r;
}

// "Last block" pattern: every block publishes its partials, fences, and the
// block that finishes last does the final (deterministic, in-order)
// reduction. No block ever waits on another, so nothing can hang.
// `total` is the number of blocks that take part (the virtual grid size).
__device__ __forceinline__ bool last_block(unsigned int *counter, int total) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int prev = atomicAdd(counter, 1u);
        am_last = (prev == (unsigned int)total - 1u);
    }
    __syncthreads();
    if (am_last) __threadfence();
    return am_last;
}

// Sum / max of this kernel's partials in block order (last block only).
__device__ __forceinline__ double fold_partials(const double *p, int nblocks, bool is_max,
                                                double *smem) {
    if (is_max) {  // maxima of values >= 0: integer max of the bit patterns
        long long m = 0;
        for (int k = threadIdx.x; k < nblocks; k += blockDim.x)
            m = max(m, __double_as_longlong(__ldcg(p + k)));
        return __longlong_as_double(block_max_bits(m, reinterpret_cast<long long *>(smem)));
    }
    double v = 0.0;
    // each thread folds a strided subset in order, then a fixed tree
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) v += __ldcg(p + k);
    return block_reduce(v, OpSum(), smem);
}

// ---------------------------------------------------------- FP64 helpers
// GB300 issues 2 FP64 thread-instructions per SM and cycle (1/64 of FP32),
// so the FP64 kernels avoid the multi-instruction IEEE divide and square
// root where full IEEE rounding is not needed.
//
// Reciprocal and reciprocal square root: an estimate y0 (~2^-22 relative,
// from the FP32 unit, see rcp_seed / rsqrt_seed) refined by one third-order
// Householder (Newton-Raphson with the second order term) correction. With
// e = 1 - a y0 (resp. 1 - a y0^2):
//   1/a       = y0 (1 + e + e^2 + ...)            -> error ~ e^3
//   1/sqrt(a) = y0 (1 + e/2 + 3 e^2 / 8 + ...)    -> error ~ 5/16 e^3
// i.e. a few ulp, for positive normal arguments. 3 and 5 FP64 instructions.
// Seeds from the FP32 special-function unit for positive normal doubles in
// FP32 range: the double is truncated to FP32 and the FP32 estimate widened
// back, both from the bit patterns on the integer pipe, so neither the
// estimate nor the conversions take FP64 issue slots (~2^-22 relative, the
// same quality as the FP64 approximate instructions). false when a or the
// estimate falls outside the FP32 normal range.
__device__ __forceinline__ bool f32_of(double a, float &f) {
    const int hi = __double2hiint(a);
    const unsigned int lo = (unsigned int)__double2loint(a);
    const int fe = ((hi >> 20) & 0x7ff) - 896;
    f = __uint_as_float(((unsigned int)fe << 23) | (((unsigned int)hi & 0xfffffu) << 3) |
                        (lo >> 29));
    return hi > 0 && fe > 0 && fe < 255;
}
__device__ __forceinline__ bool f64_of(float f, double &d) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xffu;
    d = __hiloint2double((int)(((e + 896u) << 20) | ((b & 0x7fffffu) >> 3)), (int)((b & 7u) << 29));
    return e > 0 && e < 255 && !(b >> 31);
}
__device__ __forceinline__ double rcp_seed(double a) {
    float f, r;
    double y;
    if (f32_of(a, f)) {
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
        if (f64_of(r, y)) return y;
    }
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
    return y;
}
__device__ __forceinline__ double rsqrt_seed(double a) {
    float f, r;
    double y;
    if (f32_of(a, f)) {
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
        if (f64_of(r, y)) return y;
    }
    asm("rsqrt.approx.f64 %0, %1;" : "=d"(y) : "d"(a));
    return y;
}
__device__ __forceinline__ double rcp_hn(double a) {
    const double y = rcp_seed(a);
    const double e = fma(-a, y, 1.0);
    return fma(y, fma(e, e, e), y);
}
__device__ __forceinline__ double rsqrt_hn(double a) {
    const double y = rsqrt_seed(a);
    const double t = a * y;
    const double e = fma(-t, y, 1.0);
    return fma(y * e, fma(e, 0.375, 0.5), y);
}
// 1/sqrt(a) and 1/a to ~1 ulp with 2 and 1 FP64 instructions (ff.cuh);
// rsqrt_hn / rcp_hn outside the float-float range.
static __device__ __noinline__ double rsqrt_slow(double a) { return rsqrt_hn(a); }
static __device__ __noinline__ double rcp_slow(double a) { return rcp_hn(a); }
__device__ __forceinline__ double rsqrt_d(double a) {
    return ff_in_range(a) ? rsqrt_d_core(a) : rsqrt_slow(a);
}
__device__ __forceinline__ double rcp_d(double a) {
    return ff_in_range(a) ? rcp_d_core(a) : rcp_slow(a);
}

// Sign and ordering on the integer pipe (no FP64 instruction): negation and
// absolute value flip / clear the sign bit of the high word; for doubles
// >= 0 (and +0) the signed 64-bit patterns order like the values.
__device__ __forceinline__ double neg_bits(double x) {
    int hi;
    asm("xor.b32 %0, %1, 0x80000000;" : "=r"(hi) : "r"(__double2hiint(x)));
    return __hiloint2double(hi, __double2loint(x));
}
__device__ __forceinline__ double abs_bits(double x) {
    int hi;
    asm("and.b32 %0, %1, 0x7fffffff;" : "=r"(hi) : "r"(__double2hiint(x)));
    return __hiloint2double(hi, __double2loint(x));
}
__device__ __forceinline__ bool nonneg_bits(double x) { return __double2hiint(x) >= 0; }
__device__ __forceinline__ bool less_nonneg(double a, double b) {
    return __double_as_longlong(a) < __double_as_longlong(b);
}
__device__ __forceinline__ double min_nonneg(double a, double b) {
    return __longlong_as_double(min(__double_as_longlong(a), __double_as_longlong(b)));
}

// Minimum image on a periodic axis: |d| > L/2 is tested on the 32-bit words
// of the bit patterns (non-negative doubles order like their bits; compared
// as one 64-bit integer, the test is turned back into an FP64 compare), so
// it costs no FP64 instruction; d - sign(d) L, the reference's (L - |d|)
// (+-1), is a call: inlined it would be computed for every pair.
static __device__ __noinline__ double wrap_slow(double d, double iv) {
    return d - copysign(iv, d);
}
__device__ __forceinline__ double min_image(double d, double half_iv, double iv) {
    const unsigned h = (unsigned)__double2hiint(d) & 0x7fffffffu, l = (unsigned)__double2loint(d);
    const unsigned H = (unsigned)__double2hiint(half_iv), L = (unsigned)__double2loint(half_iv);
    if (h > H || (h == H && l > L)) d = wrap_slow(d, iv);
    return d;
}

// Running maximum of doubles >= 0 (or any double against a running maximum
// that starts at 0) on the integer pipe: for x >= 0 the signed 64-bit
// pattern orders like the value, and negative values lose against 0.
__device__ __forceinline__ long long max_bits(long long m, double x) {
    return max(m, __double_as_longlong(x));
}
__device__ __forceinline__ bool finite_bits(double x) {
    return (__double_as_longlong(x) & 0x7ff0000000000000LL) != 0x7ff0000000000000LL;
}

// wrappedDifference, src/kernels.cu:1094-1114 (minimum image on periodic axes)
template <int DIM>
__device__ __forceinline__ void wrapped_diff(const DevConst &k, double x1, double y1, double z1,
                                             double x2, double y2, double z2, double &dx,
                                             double &dy, double &dz) {
    const double d1x = x1 - x2, d1y = y1 - y2, d1z = DIM == 3 ? z1 - z2 : 0.0;
    dx = d1x;
    dy = d1y;
    dz = d1z;
    const double tx = k.iv[0] - fabs(d1x);
    const double ty = k.iv[1] - fabs(d1y);
    if (!k.wall[0] && tx * tx < d1x * d1x) dx = d1x < 0 ? tx : -tx;
    if (!k.wall[1] && ty * ty < d1y * d1y) dy = d1y < 0 ? ty : -ty;
    if (DIM == 3) {
        const double tz = k.iv[2] - fabs(d1z);
        if (!k.wall[2] && tz * tz < d1z * d1z) dz = d1z < 0 ? tz : -tz;
    }
}

// Same, with every operation rounded separately (no contraction), so the
// pair acceptance test is bit-identical to the oracle's.
template <int DIM>
__device__ __forceinline__ double exact_sqdist(const DevConst &k, double x1, double y1, double z1,
                                               double x2, double y2, double z2) {
    const double d1x = __dsub_rn(x1, x2), d1y = __dsub_rn(y1, y2);
    const double d1z = DIM == 3 ? __dsub_rn(z1, z2) : 0.0;
    double dx = d1x, dy = d1y, dz = d1z;
    const double tx = __dsub_rn(k.iv[0], fabs(d1x));
    const double ty = __dsub_rn(k.iv[1], fabs(d1y));
    if (!k.wall[0] && __dmul_rn(tx, tx) < __dmul_rn(d1x, d1x)) dx = d1x < 0 ? tx : -tx;
    if (!k.wall[1] && __dmul_rn(ty, ty) < __dmul_rn(d1y, d1y)) dy = d1y < 0 ? ty : -ty;
    if (DIM == 3) {
        const double tz = __dsub_rn(k.iv[2], fabs(d1z));
        if (!k.wall[2] && __dmul_rn(tz, tz) < __dmul_rn(d1z, d1z)) dz = d1z < 0 ? tz : -tz;
    }
    double t = __dmul_rn(dx, dx);
    t = __dadd_rn(t, __dmul_rn(dy, dy));
    t = __dadd_rn(t, __dmul_rn(dz, dz));
    return t;
}

__device__ __forceinline__ void swap_role(int *r, int a, int b) {
    const int t = r[a];
    r[a] = r[b];
    r[b] = t;
}

__device__ __forceinline__ void set_cond(unsigned long long h, unsigned int v) {
    cudaGraphSetConditional((cudaGraphConditionalHandle)h, v);
}

// step(): accept / reject and the new dt (src/simulator.cu:239-246); on
// accept, integrate()'s rotation and clock (src/simulator.cu:258-314) and the
// delete / search decisions (:316-334). Run by one thread of the last block.
template <int DIM>
__device__ void finish_attempt(Ctrl *c, const DevConst &k, double fErr, double fRad,
                               double fExp, double fVol, double fDel, double fBad) {
    const int gas = c->use_gas, path = c->inc_path;
    const int n = c->n;
    c->done[DC_CORRECT] = 0;
    c->max_err = fErr;
    c->max_rad = fRad;
    c->max_exp = fExp;
    c->vol_new = fVol;
    c->ndel = gas ? (int)fDel : 0;
    c->attempts += 1;
    c->attempts_this_step += 1;
    const double tol = k.tol;
    const int too_large = fErr > tol;
    const int increase = fErr < 0.45 * tol && c->dt < 10;
    if (too_large)
        c->dt *= 0.37;
    else if (increase)
        c->dt *= 1.269;
    c->too_large = too_large;
    if (k.mixed) {  // speculative prediction of the next attempt (step_mixed.cu)
        const int use = !too_large && !c->no_accept;
        c->pred_ready = use;
        c->pred_slot = use ? (increase ? 2 : 1) : 0;
        if (use) {
            c->sumA = c->cand_sumA[increase ? 1 : 0];
            c->sumAr = c->cand_sumAr[increase ? 1 : 0];
        }
        c->cand_sumA[0] = c->cand_sumA[1] = c->cand_sumAr[0] = c->cand_sumAr[1] = 0.0;
    }
    if (fBad > 0.0 || isnan(fErr)) c->status = CB_ERR_NONFINITE;
    c->need_delete = 0;
    c->need_search = 0;
    if (too_large && c->status == CB_OK) {
        if (c->attempts_this_step >= k.max_attempts) c->status = CB_ERR_MAX_ATTEMPTS;
        if (c->dt < 1e-300) c->status = CB_ERR_DT_UNDERFLOW;
    }
    if (!too_large && !c->no_accept && c->status == CB_OK) {
        int *r = c->drole;
        for (int a = 0; a < DIM; a++) {
            swap_role(r, RX + a, RXN + a);
            const int old = r[RVO0 + a];
            r[RVO0 + a] = r[RV0 + a];
            r[RV0 + a] = r[RVP0 + a];
            r[RVP0 + a] = old;
        }
        if (gas) {
            swap_role(r, RR, RRN);
            const int old = r[RVO3];
            r[RVO3] = r[RV3];
            r[RV3] = r[RVP3];
            r[RVP3] = old;
        }
        if (path) swap_role(r, RPATH, RPATHN);
        c->steps += 1;
        c->bubble_steps += n;
        c->attempts_this_step = 0;
        // time accumulator, src/simulator.cu:311-314 (adds the updated dt)
        c->tfrac += c->dt;
        c->tint += (unsigned long long)c->tfrac;
        c->tfrac = c->tfrac - (double)(unsigned long long)c->tfrac;
        c->dt_min = fmin(c->dt_min, c->dt);
        c->dt_max = fmax(c->dt_max, c->dt);
        c->dt_sum += c->dt;
        if (gas) {
            c->max_bubble_radius = fRad;
            c->need_delete = c->ndel > 0;
        }
        c->need_search = fExp >= 0.5 * k.skin;
        if (c->stop_on) {
            const int left = n - (c->need_delete ? c->ndel : 0);
            const int time_up = c->tint > c->stop_tint ||
                                (c->tint == c->stop_tint && c->tfrac >= c->stop_tfrac);
            c->stop_hit = time_up || left <= c->stop_nmin ||
                          (gas && c->max_bubble_radius >= c->stop_rmax);
        }
    }
    if (c->graph_mode) {
        const int ok = c->status == CB_OK;
        const int accepted = !too_large;
        set_cond(c->h_delete, ok && accepted && c->need_delete);
        set_cond(c->h_search, ok && accepted && c->need_search);
        const int more = ok && (too_large || (c->steps < c->steps_target && !c->stop_hit));
        set_cond(c->h_loop, more);
        // the last iteration's removal / search are decided above; clearing
        // the mode here spares the host a control-block write per launch
        if (!more) c->graph_mode = 0;
    }
}

// ------------------------------------------------------ kernel launchers
struct Launch {
    int grid;         // upper bound of the blocks of a grid-stride kernel
    int sms;          // streaming multiprocessors of the device
    int scan_grid;    // blocks of the scan kernels
    int cover;        // blocks of a one-bubble-per-thread kernel over capacity
    cudaStream_t stream;
    long long *launches;  // host-side launch counter
    // Batched launches: when `batch` is set, every launcher runs its kernel's
    // batched form over the work list `work` (device) of the foams in the
    // device table `batch`, on a 1D grid of `gmax` blocks.
    const struct Bufs *batch = nullptr;
    const struct BatchWork *work = nullptr;
    int gmax = 0;
    // Tuning (cb_tuning): consecutive pairs per thread of the mixed pair
    // kernel, and resident blocks per SM of the pair kernels and of the
    // predict / correct kernels (0: as many as fit)
    int pair_run = 4;
    int pair_bps = 0;
    int step_bps = 0;
};

// Phases of a batched step a foam takes part in (Ctrl::bsel bits).
enum BatchSel : int { SEL_ATTEMPT = 1, SEL_DELETE = 2, SEL_SEARCH = 4 };

// Work list of one batched phase: the selected foams and the prefix sums of
// their virtual grids; work item w belongs to the foam k with
// pre[k] <= w < pre[k + 1] and is its block w - pre[k].
struct BatchWork {
    int nsel, total;
    int *foam;  // nsel entries
    int *pre;   // nsel + 1 entries
};

__device__ __forceinline__ int batch_item(const BatchWork *wk, int item, int &vb, int &vg) {
    const int *pre = wk->pre;
    int lo = 0, hi = wk->nsel - 1;  // largest k with pre[k] <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= item)
            lo = mid;
        else
            hi = mid - 1;
    }
    vb = item - pre[lo];
    vg = pre[lo + 1] - pre[lo];
    return wk->foam[lo];
}

#define CB_ID(...) __VA_ARGS__

// Declares the single-foam kernel NAME(Bufs) and its batched form
// NAME_batch(const Bufs *, const BatchWork *) around the body
// NAME_body(b, vb, vg): the batched form loops over the phase's work items
// on a fixed grid (no block waits for another).
// TPL is the parenthesised template header ("(template <int DIM>)" or "()"),
// ARGS the parenthesised template arguments ("(<DIM>)" or "()").
// Programmatic dependent launch: the kernels below are launched so that they
// may begin while the previous kernel on the stream drains (launch_pdl). The
// first thing each does is wait for that kernel's completion and memory
// (griddepcontrol.wait); it then lets its own successor be scheduled.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

#define CB_KERNEL_PAIR(TPL, NAME, ARGS, BOUNDS)                                  \
    CB_ID TPL __global__ void BOUNDS NAME(Bufs b) {                                \
        pdl_enter();                                                               \
        NAME##_body CB_ID ARGS(b, blockIdx.x, gridDim.x);                          \
    }                                                                              \
    CB_ID TPL __global__ void BOUNDS NAME##_batch(const Bufs *bb, const BatchWork *wk) { \
        pdl_enter();                                                               \
        const int total = wk->total;                                               \
        for (int item = blockIdx.x; item < total; item += gridDim.x) {             \
            int vb, vg;                                                            \
            const Bufs b = bb[batch_item(wk, item, vb, vg)];                       \
            NAME##_body CB_ID ARGS(b, vb, vg);                                     \
            __syncthreads();                                                       \
        }                                                                          \
    }

// Launch of a CB_KERNEL_PAIR kernel with programmatic stream serialisation
// (a failure is left for the caller's cudaGetLastError, as for <<<>>>).
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), int grid, cudaStream_t stream, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Launches NAME<ARGS> in its single or batched form per the Launch `l`.
#define CB_LAUNCH(l, NAME, ARGS, GRID, b)                                             \
    do {                                                                             \
        if ((l).batch)                                                               \
            launch_pdl(NAME##_batch CB_ID ARGS, (l).gmax, (l).stream, (l).batch, (l).work); \
        else                                                                         \
            launch_pdl(NAME CB_ID ARGS, (GRID), (l).stream, (b));                    \
        *(l).launches += 1;                                                          \
    } while (0)

// One wave of resident blocks of `kernel` (a multiple of the SM count),
// bounded by l.grid (the size of the per-block partial arrays).
// `want` > 0 caps the resident blocks per SM (a tuning knob).
template <typename K>
inline int wave_grid(K kernel, const Launch &l, int want = 0) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kBlock, 0) != cudaSuccess ||
        nb < 1)
        nb = 1;
    if (want > 0 && want < nb) nb = want;
    const int g = l.sms * nb;
    return g < l.grid ? g : l.grid;
}

// step.cu
void launch_predict(const Launch &l, const Bufs &b, int dim);
void launch_pairs(const Launch &l, const Bufs &b, int dim, int mode,
                  bool ff);  // mode: gas 1 | flow 2; ff: float-float kernel
void launch_correct(const Launch &l, const Bufs &b, int dim);
void launch_boot(const Launch &l, const Bufs &b, int dim, int phase);
// step_mixed.cu (mixed form)
void launch_predict_mx(const Launch &l, const Bufs &b, int dim);
void launch_pairs_mx(const Launch &l, const Bufs &b, int dim, int mode);
void launch_correct_mx(const Launch &l, const Bufs &b, int dim, int mode, bool walls);
void launch_boot_mx(const Launch &l, const Bufs &b, int dim, int phase);
void launch_energy(const Launch &l, const Bufs &b, int dim, int per_bubble);
void launch_volume(const Launch &l, const Bufs &b, int dim);
// search.cu
void launch_search(const Launch &l, const Bufs &b, int dim);
// remove.cu
void launch_remove(const Launch &l, const Bufs &b, int dim);
// scan.cu
// Exclusive scans of the search and the deletion: cellCount -> cellStart
// (ncell), rowCount -> rowStart (n, total -> np_found), delflag -> iscan (n),
// keep -> keepScan (np); out[count] = total.
enum ScanKind : int { SCAN_CELLS = 0, SCAN_ROWS, SCAN_DEL, SCAN_KEEP };
void launch_scan(const Launch &l, const Bufs &b, int kind);

}  // namespace cbg
