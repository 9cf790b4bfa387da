// One attempt of the Adams-Bashforth-Moulton step, FP64 form:
//   k_predict  : AB2 predict of x, y, (z), r into the packed `pred` rows and
//                the area sums (preIntegrate, src/kernels.cu:40-170)
//   k_pairs    : overlap velocities, pairwise gas flux, overlap areas and
//                flow neighbour sums per pair (pairwiseInteraction,
//                src/kernels.cu:172-337)
//   k_correct  : flow and wall velocities, the mean-field gas exchange, AM2
//                correct, error / expansion / radius maxima, deletion marks,
//                path; its last block takes the accept/reject decision and
//                the dt update of step() (src/simulator.cu:219-246) and, on
//                accept, rotates the buffers and advances the clock as
//                integrate() does (src/simulator.cu:258-334) — on the device
//                (postIntegrate, correct, addFlowVelocity, addWallVelocity,
//                src/kernels.cu:339-593)
// plus the Euler bootstrap of init() (src/simulator.cu:727-787) and the
// energy / volume reductions (src/kernels.cu:941-957, :1013-1024).
#include "common.cuh"

namespace cbg {
namespace {

__device__ __forceinline__ double4_32a ld4(const double *p, int i) {
    return reinterpret_cast<const double4_32a *>(p)[i];
}

// Float-float records of the float-float pair kernel (CB_PRECISION_FP64_FF):
// (r, 1/r) and (r^2, 0) per bubble, written where the predicted radius is
// known.
struct FfRec {
    ff r, inv, rsq;
};
__device__ __forceinline__ FfRec ld_rec(const float4 *R, int i) {
    const float4 u = R[2 * (size_t)i], v = R[2 * (size_t)i + 1];
    return {{u.x, u.y}, {u.z, u.w}, {v.x, v.y}};
}
__device__ __forceinline__ void st_rec(float4 *R, int i, double r, double inv, double rsq) {
    const ff a = ff_of(r), b = ff_of(inv), c = ff_of(rsq);
    R[2 * (size_t)i] = make_float4(a.h, a.l, b.h, b.l);
    R[2 * (size_t)i + 1] = make_float4(c.h, c.l, 0.f, 0.f);
}
__device__ __forceinline__ bool ff_less(ff a, ff b) {  // normalised pairs
    return a.h < b.h || (a.h == b.h && a.l < b.l);
}
// Reduction of a float-float value into an FP64 row: both parts widened
// exactly on the integer pipe and summed by one FP64 add (correctly rounded).
// The float-float pair kernel is bound by issue slots and leaves the FP64
// pipe mostly idle, so this costs fewer slots than the integer-pipe rounding.
__device__ __forceinline__ void add_d(double *p, ff v) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(ff_f2d(v.h) + ff_f2d(v.l)));
}

// ---------------------------------------------------------------- predict
template <int DIM>
__device__ __forceinline__ void k_predict_body(const Bufs &b, const int vb, const int vg) {
    __shared__ double smem[32];
    const Ctrl *c = b.ctrl;
    const int n = c->n;
    const double h = 0.5 * c->dt;
    const int gas = c->use_gas;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    const double *V0 = drow(b, c, RV0), *V1 = drow(b, c, RV1), *V2 = drow(b, c, RV2),
                 *V3 = drow(b, c, RV3);
    const double *O0 = drow(b, c, RVO0), *O1 = drow(b, c, RVO1), *O2 = drow(b, c, RVO2),
                 *O3 = drow(b, c, RVO3);
    double sA = 0.0, sAr = 0.0;
    int na = 0;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += vg * blockDim.x) {
        // p + 0.5 ts (3 v - vo), src/kernels.cu:48-50
        const double xp = fma(h, fma(3.0, V0[i], -O0[i]), X[i]);
        const double yp = fma(h, fma(3.0, V1[i], -O1[i]), Y[i]);
        double rp = R[i];
        if (gas) rp = fma(h, fma(3.0, V3[i], -O3[i]), rp);
        const double inv = rcp_d(rp);
        const double rsq = rp * rp;
        if (b.ffr) st_rec(b.ffr, i, rp, inv, rsq);
        double4_32a p;
        if (DIM == 3) {
            p.x = xp;
            p.y = yp;
            p.z = fma(h, fma(3.0, V2[i], -O2[i]), Z[i]);
            p.w = rp;
            reinterpret_cast<double2 *>(b.invr)[i] = make_double2(inv, rsq);
        } else {
            p.x = xp;
            p.y = yp;
            p.z = rp;
            p.w = inv;
        }
        reinterpret_cast<double4_32a *>(b.pred)[i] = p;
        if (gas) {  // area and area per radius, src/kernels.cu:103-112, with
                    // the constant factor (4 pi, 2 pi) applied to the block sums
            if (DIM == 3) {
                sA += rsq;
                sAr += rp;
            } else {
                sA += rp;
                na++;
            }
        }
    }
    if (DIM == 2) sAr = (double)na;
    constexpr double kArea = DIM == 3 ? 4.0 * kPi : 2.0 * kPi;
    const double tA = kArea * block_reduce(sA, OpSum(), smem);
    const double tAr = kArea * block_reduce(sAr, OpSum(), smem);
    if (threadIdx.x == 0) {
        b.part[0 * vg + vb] = tA;
        b.part[1 * vg + vb] = tAr;
    }
    if (last_block(&b.ctrl->done[DC_PREDICT], vg)) {
        const double fA = fold_partials(b.part + 0 * vg, vg, false, smem);
        const double fAr = fold_partials(b.part + 1 * vg, vg, false, smem);
        if (threadIdx.x == 0) {
            b.ctrl->sumA = fA;
            b.ctrl->sumAr = fAr;
            b.ctrl->done[DC_PREDICT] = 0;
        }
    }
}
CB_KERNEL_PAIR((template <int DIM>), k_predict, (<DIM>), __launch_bounds__(kBlock))


// ------------------------------------------------------------------ pairs
// Overlap velocities, pairwise gas flux and overlap areas in FP64
// (pairwiseInteraction, src/kernels.cu:172-337). FP64-issue bound on GB300
// (2 FP64 thread-instructions per SM and cycle), so:
//   * each warp takes 32 consecutive pairs, computes their FP64 differences
//     and overlap test (3 FP64 instructions a pair; the test in FP32 with a
//     guard band), and queues the overlapping ones (about 70 % of the listed
//     pairs) in shared memory; the distance, force and gas-exchange
//     arithmetic then runs on full warps of overlapping pairs, not on warps
//     with idle lanes;
//   * minimum image by bit compare; 1/sqrt(m) and 1/(r1 + r2) to ~1 ulp by
//     rsqrt_d / rcp_d (2 and 1 FP64 instructions, the rest on the FP32 and
//     integer pipes); the division by m of the overlap formula as a product
//     with (1/sqrt(m))^2; -w/4 on the exponent field; no product by f0 when
//     it is 1;
//   * contributions to both members go through FP64 reductions into the
//     per-bubble accumulator rows;
//   * overlap areas are accumulated in units of ov_unit (pi in 3D, 2 in 2D),
//     one FP64 product less per overlapping pair; the unit is applied to the
//     global sums and in the correct kernel.
__device__ __forceinline__ void red_add(double *p, double v) {
    asm volatile("red.global.add.f64 [%0], %1;" ::"l"(p), "d"(v));
}
// -w/4, exact: the exponent field lowered by 2 and the sign flipped when the
// exponent allows it (|w| > 2^-1020), else the FP64 product (a call, so that
// it is not computed for every pair).
static __device__ __noinline__ double neg_quarter_slow(double w) { return -0.25 * w; }
__device__ __forceinline__ double neg_quarter(double w) {
    const int hi = __double2hiint(w);
    if ((hi & 0x7ff00000) > 0x00200000)
        return __hiloint2double((hi - 0x00200000) ^ (int)0x80000000, __double2loint(w));
    return neg_quarter_slow(w);
}

constexpr int kQueue = 64;  // per-warp queue of overlapping pairs

// Unit of the overlap rows the pair kernels write: pi in 3D (an overlap area
// is pi (chord radius)^2), 2 in 2D (an overlap length is 2 (half chord)).
__host__ __device__ constexpr double ov_unit(int dim) { return dim == 3 ? kPi : 2.0; }

// The last block of a pair kernel: the attempt's total overlap area and
// overlap area per radius (src/kernels.cu:264-267; each pair adds 2 A_overlap)
// from the blocks' partial sums, which are in units of ov_unit, and the
// mean-field factors of every bubble (src/kernels.cu:399-404).
template <int DIM>
__device__ __forceinline__ void pairs_fold(const Bufs &b, const int vb, const int vg,
                                           double *smem) {
    if (!last_block(&b.ctrl->done[DC_PAIRS], vg)) return;
    const double fAo = fold_partials(b.part + 2 * vg, vg, false, smem);
    const double fAor = fold_partials(b.part + 3 * vg, vg, false, smem);
    if (threadIdx.x == 0) {
        Ctrl *cc = b.ctrl;
        cc->sumAo = (2.0 * ov_unit(DIM)) * fAo;
        cc->sumAor = ov_unit(DIM) * fAor;
        cc->mfa = (cc->sumAr - cc->sumAor) / (cc->sumA - cc->sumAo);
        cc->mfb = b.k->kappa * b.k->ain * (double)cc->n / cc->sumA;
        cc->done[DC_PAIRS] = 0;
    }
}

// The overlap test of the reference in FP64 (the sign of the exact
// (r1 + r2)^2 - m), for pairs in the FP32 guard band.
template <int DIM>
static __device__ __noinline__ bool overlap_exact(double dx, double dy, double dz, double r1,
                                                  double r2) {
    double m = dx * dx;
    m = fma(dy, dy, m);
    if (DIM == 3) m = fma(dz, dz, m);
    const double radii = r1 + r2;
    return nonneg_bits(fma(radii, radii, -m));
}

template <int DIM, bool GAS, bool FLOW>
__device__ __forceinline__ void k_pairs_body(const Bufs &b, const int vb, const int vg) {
    constexpr int kW = kBlock / 32;
    __shared__ double smem[32];
    // queue slots: dx, dy, (3D: dz), r1, r2
    constexpr int kR1 = DIM == 3 ? 3 : 2, kSlots = kR1 + 2;
    __shared__ double qd[kW][kSlots][kQueue];
    __shared__ int qij[kW][2][kQueue];
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int np = c->np;
    const int *PI = b.ps[c->prole[PI0]];
    const int *PJ = b.ps[c->prole[PJ0]];
    const double *V0 = drow(b, c, RV0), *V1 = drow(b, c, RV1), *V2 = drow(b, c, RV2);
    const double f0 = k.f0;
    const bool px = !k.wall[0], py = !k.wall[1], pz = DIM == 3 && !k.wall[2];
    const double hx = k.half_iv[0], hy = k.half_iv[1], hz = k.half_iv[2];
    const double Lx = k.iv[0], Ly = k.iv[1], Lz = k.iv[2];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    double(*Q)[kQueue] = qd[w];
    int *QI = qij[w][0], *QJ = qij[w][1];
    double sAo = 0.0, sAor = 0.0;

    // the force and gas-exchange terms of queued (overlapping) pair e
    auto process = [&](int e) {
        const int i = QI[e], j = QJ[e];
        const double dx = Q[0][e], dy = Q[1][e], dz = DIM == 3 ? Q[2][e] : 0.0;
        const double r1 = Q[kR1][e], r2 = Q[kR1 + 1][e];
        double m = dx * dx;
        m = fma(dy, dy, m);
        if (DIM == 3) m = fma(dz, dz, m);
        const double radii = r1 + r2;
        double *ai = b.acc + (size_t)i * kAcc;
        double *aj = b.acc + (size_t)j * kAcc;
        // velocity f0 d (1/|d| - 1/(r1 + r2)), src/kernels.cu:218-233
        const double rs = rsqrt_d(m);
        double s = rs - rcp_d(radii);
        if (f0 != 1.0) s *= f0;
        const double fx = dx * s, fy = dy * s;
        red_add(ai + 0, fx);
        red_add(aj + 0, neg_bits(fx));
        red_add(ai + 1, fy);
        red_add(aj + 1, neg_bits(fy));
        if (DIM == 3) {
            const double fz = dz * s;
            red_add(ai + 2, fz);
            red_add(aj + 2, neg_bits(fz));
        }
        if (GAS) {  // pairwise gas exchange, src/kernels.cu:236-280
            double r1sq, r2sq, inv1, inv2;
            if (DIM == 3) {  // (1/r, r^2) records written by k_predict
                const double2 e1 = reinterpret_cast<const double2 *>(b.invr)[i];
                const double2 e2 = reinterpret_cast<const double2 *>(b.invr)[j];
                inv1 = e1.x;
                r1sq = e1.y;
                inv2 = e2.x;
                r2sq = e2.y;
            } else {
                r1sq = r1 * r1;
                r2sq = r2 * r2;
                inv1 = b.pred[4 * (size_t)i + 3];
                inv2 = b.pred[4 * (size_t)j + 3];
            }
            const bool inside = less_nonneg(m, r1sq) || less_nonneg(m, r2sq);
            // chord: r2^2 - t^2 / m with t = (r2^2 - r1^2 + m) / 2, as
            // r2^2 - w^2 / 4 with w = (r2^2 - r1^2 + m) / |d|; the overlap
            // area in units of ov_unit (pi in 3D, 2 in 2D)
            double oa;
            if (inside) {
                oa = DIM == 3 ? min_nonneg(r1sq, r2sq) : min_nonneg(r1, r2);
            } else {
                const double wv = (r2sq - r1sq + m) * rs;
                oa = abs_bits(fma(neg_quarter(wv), wv, r2sq));
                if (DIM == 2) oa = __double_as_longlong(oa) > 0 ? oa * rsqrt_d(oa) : 0.0;
            }
            const double g = oa * (inv2 - inv1);
            red_add(ai + 3, g);
            red_add(aj + 3, neg_bits(g));
            red_add(ai + 4, oa);
            red_add(aj + 4, oa);
            sAo += oa;
            sAor = fma(oa, inv1 + inv2, sAor);
        }
        if (FLOW) {  // src/kernels.cu:298-307 (overlapping pairs only)
            red_add(ai + 5, V0[j]);
            red_add(ai + 6, V1[j]);
            if (DIM == 3) red_add(ai + 7, V2[j]);
        }
    };

    int cnt = 0;  // queued pairs of this warp (uniform over its lanes)
    const int nch = (np + 31) >> 5;
    for (int ch = vb * kW + w; ch < nch; ch += vg * kW) {
        const int p = (ch << 5) + lane;
        bool over = false;
        int i = 0, j = 0;
        double dx = 0.0, dy = 0.0, dz = 0.0, r1 = 0.0, r2 = 0.0;
        if (p < np) {
            i = PI[p];
            j = PJ[p];
            if (FLOW) {  // src/kernels.cu:191-207 (added for every pair)
                double *aj = b.acc + (size_t)j * kAcc;
                red_add(aj + 5, V0[i]);
                red_add(aj + 6, V1[i]);
                if (DIM == 3) red_add(aj + 7, V2[i]);
            }
            const double4_32a a = ld4(b.pred, i), q = ld4(b.pred, j);
            r1 = DIM == 3 ? a.w : a.z;
            r2 = DIM == 3 ? q.w : q.z;
            // wrappedDifference, src/kernels.cu:1094-1114 (the FP64
            // differences, exact, mostly on the integer pipe)
            dx = sub_exact(a.x, q.x);
            dy = sub_exact(a.y, q.y);
            if (px) dx = min_image(dx, hx, Lx);
            if (py) dy = min_image(dy, hy, Ly);
            if (DIM == 3) {
                dz = sub_exact(a.z, q.z);
                if (pz) dz = min_image(dz, hz, Lz);
            }
            // overlap test (r1 + r2)^2 >= m: in FP32 on the exact differences
            // (truncated, ~2^-21 relative) outside a 1e-5 guard band, by the
            // FP64 test of the reference's sign inside it
            const float fx = ff_f32(dx), fy = ff_f32(dy), fz = DIM == 3 ? ff_f32(dz) : 0.f;
            float m32 = fx * fx;
            m32 = fmaf(fy, fy, m32);
            if (DIM == 3) m32 = fmaf(fz, fz, m32);
            const float R32 = ff_f32(r1) + ff_f32(r2);
            const float RR = R32 * R32;
            if (m32 < RR * (1.f - 1e-5f))
                over = true;
            else if (!(m32 > RR * (1.f + 1e-5f)))
                over = overlap_exact<DIM>(dx, dy, dz, r1, r2);
        }
        const unsigned mask = __ballot_sync(0xffffffffu, over);
        if (over) {
            const int e = cnt + __popc(mask & below);
            QI[e] = i;
            QJ[e] = j;
            Q[0][e] = dx;
            Q[1][e] = dy;
            if (DIM == 3) Q[2][e] = dz;
            Q[kR1][e] = r1;
            Q[kR1 + 1][e] = r2;
        }
        cnt += __popc(mask);
        __syncwarp();
        if (cnt >= 32) {  // a full warp of overlapping pairs
            process(lane);
            __syncwarp();
            cnt -= 32;
            if (lane < cnt) {
                QI[lane] = QI[32 + lane];
                QJ[lane] = QJ[32 + lane];
#pragma unroll
                for (int t = 0; t < kSlots; t++) Q[t][lane] = Q[t][32 + lane];
            }
            __syncwarp();
        }
    }
    if (lane < cnt) process(lane);

    const double tAo = block_reduce(sAo, OpSum(), smem);
    const double tAor = block_reduce(sAor, OpSum(), smem);
    if (threadIdx.x == 0) {
        b.part[2 * vg + vb] = tAo;
        b.part[3 * vg + vb] = tAor;
    }
    pairs_fold<DIM>(b, vb, vg, smem);
}
CB_KERNEL_PAIR((template <int DIM, bool GAS, bool FLOW>), k_pairs, (<DIM, GAS, FLOW>), __launch_bounds__(kBlock))


// ------------------------------------------------------ pairs, float-float
// CB_PRECISION_FP64_FF: the pair kernel of the FP64 form with its arithmetic
// in float-float. Overlap velocities, pairwise gas flux and overlap areas
// (pairwiseInteraction, src/kernels.cu:172-337). GB300 issues FP64 at 1/64 of
// the FP32 rate, so apart from the three FP64 position differences
// (wrappedDifference, src/kernels.cu:1094-1114) the pair arithmetic runs in
// float-float (ff.cuh, ~2^-46 relative) on the FP32 and integer pipes, from
// per-bubble float-float records (r, 1/r, r^2) written by k_predict. The
// overlap test and the inside tests of the gas exchange are decided in
// float-float unless the difference is within 2^-38 of its operands; then the
// FP64 comparisons of the reference decide, so the classification of every
// pair is the FP64 one.
//
// Each thread takes a run of kRun consecutive pairs (rows are grouped by i):
// the i-side sums stay in float-float registers and go out once per row; the
// j-side contributions go out per pair. Both are rounded to double on the
// integer pipe and added to the FP64 accumulator rows with FP64 atomics.
constexpr int kRun = 4;
constexpr float kAmb = 0x1p-38f;


template <int DIM, bool GAS, bool FLOW>
__device__ __forceinline__ void k_pairs_ff_body(const Bufs &b, const int vb, const int vg) {
    __shared__ double smem[32];
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int np = c->np;
    const int *PI = b.ps[c->prole[PI0]];
    const int *PJ = b.ps[c->prole[PJ0]];
    const double *V0 = drow(b, c, RV0), *V1 = drow(b, c, RV1), *V2 = drow(b, c, RV2);
    const float4 *REC = b.ffr;
    const ff f0 = {k.f0_f, k.f0_l};
    const bool px = !k.wall[0], py = !k.wall[1], pz = DIM == 3 && !k.wall[2];
    const double hx = k.half_iv[0], hy = k.half_iv[1], hz = k.half_iv[2];
    const double Lx = k.iv[0], Ly = k.iv[1], Lz = k.iv[2];
    ff sAo = {0.f, 0.f}, sAor = {0.f, 0.f};
    const int nrun = (np + kRun - 1) / kRun;
    for (int g = vb * blockDim.x + threadIdx.x; g < nrun; g += vg * blockDim.x) {
        const int p0 = g * kRun;
        int cur = -1;
        double4_32a a;
        FfRec ra;
        ff ax = {0.f, 0.f}, ay = ax, az = ax, ag = ax, ao = ax;
        bool hit = false;
        double vxi = 0.0, vyi = 0.0, vzi = 0.0;
        auto flush = [&](int i) {
            double *ai = b.acc + (size_t)i * kAcc;
            add_d(ai + 0, ax);
            add_d(ai + 1, ay);
            if (DIM == 3) add_d(ai + 2, az);
            if (GAS) {
                add_d(ai + 3, ag);
                add_d(ai + 4, ao);
            }
        };
#pragma unroll 1  // one pair body: the unrolled run overflows the instruction cache
        for (int t = 0; t < kRun; t++) {
            if (p0 + t >= np) break;
            const int i = PI[p0 + t], j = PJ[p0 + t];
            if (i != cur) {
                if (hit) flush(cur);
                cur = i;
                a = ld4(b.pred, i);
                ra = ld_rec(REC, i);
                ax = ay = az = ag = ao = ff{0.f, 0.f};
                hit = false;
                if (FLOW) {
                    vxi = V0[i];
                    vyi = V1[i];
                    vzi = DIM == 3 ? V2[i] : 0.0;
                }
            }
            double *aj = b.acc + (size_t)j * kAcc;
            if (FLOW) {  // src/kernels.cu:191-207 (added for every pair)
                atomicAdd(aj + 5, vxi);
                atomicAdd(aj + 6, vyi);
                if (DIM == 3) atomicAdd(aj + 7, vzi);
            }
            const double4_32a q = ld4(b.pred, j);
            const FfRec rb = ld_rec(REC, j);
            // wrappedDifference, src/kernels.cu:1094-1114 (FP64)
            double dx = a.x - q.x, dy = a.y - q.y, dz = 0.0;
            if (px) dx = min_image(dx, hx, Lx);
            if (py) dy = min_image(dy, hy, Ly);
            if (DIM == 3) {
                dz = a.z - q.z;
                if (pz) dz = min_image(dz, hz, Lz);
            }
            const ff X = ff_of(dx), Y = ff_of(dy), Z = ff_of(dz);
            ff m = ff_add(ff_sqr(X), ff_sqr(Y));
            if (DIM == 3) m = ff_add(m, ff_sqr(Z));
            const ff R = ff_add(ra.r, rb.r);
            const ff RR = ff_sqr(R);
            const float dov = ff_diff_f(RR, m);
            bool over = dov >= 0.f;
            bool amb = fabsf(dov) <= kAmb * RR.h;
            bool inside = false;
            if (GAS) {
                const float d1 = ff_diff_f(m, ra.rsq), d2 = ff_diff_f(m, rb.rsq);
                inside = d1 < 0.f || d2 < 0.f;
                amb |= fabsf(d1) <= kAmb * m.h || fabsf(d2) <= kAmb * m.h;
            }
            if (amb) {  // within 2^-38: the reference's FP64 tests decide
                double m64 = dx * dx;
                m64 = fma(dy, dy, m64);
                if (DIM == 3) m64 = fma(dz, dz, m64);
                const double r1 = DIM == 3 ? a.w : a.z, r2 = DIM == 3 ? q.w : q.z;
                const double radii = r1 + r2;
                over = nonneg_bits(fma(radii, radii, -m64));
                if (GAS) {
                    double r1sq, r2sq;
                    if (DIM == 3) {
                        r1sq = b.invr[2 * (size_t)i + 1];
                        r2sq = b.invr[2 * (size_t)j + 1];
                    } else {
                        r1sq = r1 * r1;
                        r2sq = r2 * r2;
                    }
                    inside = less_nonneg(m64, r1sq) || less_nonneg(m64, r2sq);
                }
            }
            if (!over) continue;
            // velocity f0 d (1/|d| - 1/(r1 + r2)), src/kernels.cu:218-233
            const ff rs = ff_rsqrt(m);
            const ff s = ff_mul(f0, ff_sub(rs, ff_rcp(R)));
            const ff fx = ff_mul(X, s), fy = ff_mul(Y, s);
            ax = ff_add(ax, fx);
            ay = ff_add(ay, fy);
            add_d(aj + 0, ff_neg(fx));
            add_d(aj + 1, ff_neg(fy));
            if (DIM == 3) {
                const ff fz = ff_mul(Z, s);
                az = ff_add(az, fz);
                add_d(aj + 2, ff_neg(fz));
            }
            hit = true;
            if (GAS) {  // pairwise gas exchange, src/kernels.cu:236-280
                // chord: r2^2 - t^2 / m with t = (r2^2 - r1^2 + m) / 2, as
                // r2^2 - w^2 / 4 with w = (r2^2 - r1^2 + m) / |d|; the
                // overlap area in units of ov_unit (pi in 3D, 2 in 2D)
                ff oa;
                if (inside) {
                    if (DIM == 3)
                        oa = ff_less(ra.rsq, rb.rsq) ? ra.rsq : rb.rsq;
                    else
                        oa = ff_less(ra.r, rb.r) ? ra.r : rb.r;
                } else {
                    const ff w = ff_mul(ff_add(ff_sub(rb.rsq, ra.rsq), m), rs);
                    const ff v = ff_abs(ff_sub(rb.rsq, ff_scale(ff_sqr(w), 0.25f)));
                    oa = DIM == 3 ? v : ff_sqrt(v);
                }
                const ff gf = ff_mul(oa, ff_sub(rb.inv, ra.inv));
                ag = ff_add(ag, gf);
                ao = ff_add(ao, oa);
                add_d(aj + 3, ff_neg(gf));
                add_d(aj + 4, oa);
                sAo = ff_add(sAo, oa);
                sAor = ff_add(sAor, ff_mul(oa, ff_add(ra.inv, rb.inv)));
            }
            if (FLOW) {  // src/kernels.cu:298-307 (overlapping pairs only)
                double *ai = b.acc + (size_t)i * kAcc;
                atomicAdd(ai + 5, V0[j]);
                atomicAdd(ai + 6, V1[j]);
                if (DIM == 3) atomicAdd(ai + 7, V2[j]);
            }
        }
        if (hit) flush(cur);
    }
    const double tAo = block_reduce(ff_to_double(sAo), OpSum(), smem);
    const double tAor = block_reduce(ff_to_double(sAor), OpSum(), smem);
    if (threadIdx.x == 0) {
        b.part[2 * vg + vb] = tAo;
        b.part[3 * vg + vb] = tAor;
    }
    pairs_fold<DIM>(b, vb, vg, smem);
}
CB_KERNEL_PAIR((template <int DIM, bool GAS, bool FLOW>), k_pairs_ff, (<DIM, GAS, FLOW>), __launch_bounds__(kBlock, 3))


// ---------------------------------------------------------------- correct
// touchesWall, src/kernels.cu:553-566
__device__ __forceinline__ bool touches_wall(double f0, double rad, double x, double low,
                                             double high, double &velocity) {
    double d1 = x - low;
    double d2 = x - high;
    d1 = d1 * d1 < d2 * d2 ? d1 : d2;
    if (rad * rad >= d1 * d1) {
        d2 = d1 < 0.0 ? -1.0 : 1.0;
        d1 *= d2;
        velocity = d2 * f0 * (1.0 - d1 / rad);
        return true;
    }
    return false;
}

// Flow, shear and wall terms of the velocity (addFlowVelocity,
// addWallVelocity, src/kernels.cu:497-593) as a call taken only when one of
// them is on: inlined, their FP64 arithmetic would be predicated into every
// bubble's path and take FP64 issue slots.
struct Vel3 {
    double x, y, z;
};
template <int DIM>
static __device__ __noinline__ Vel3 boundary_velocity(const DevConst &k, int flow, int shear,
                                                      double drag, double vpx, double vpy,
                                                      double vpz, double xp, double yp, double zp,
                                                      double rp, double f0, double f1, double f2,
                                                      int nn) {
    if (flow) {  // addFlowVelocity, src/kernels.cu:497-544
        double multiplier = nn;
        multiplier = (multiplier > 0 ? 1.0 / multiplier : 0.0);
        const double riSq = rp * rp;
        int inside = (int)((xp < k.flow_tfr[0] && xp > k.flow_lbb[0]) ||
                           ((k.flow_lbb[0] - xp) * (k.flow_lbb[0] - xp) <= riSq) ||
                           ((k.flow_tfr[0] - xp) * (k.flow_tfr[0] - xp) <= riSq));
        inside *= (int)((yp < k.flow_tfr[1] && yp > k.flow_lbb[1]) ||
                        ((k.flow_lbb[1] - yp) * (k.flow_lbb[1] - yp) <= riSq) ||
                        ((k.flow_tfr[1] - yp) * (k.flow_tfr[1] - yp) <= riSq));
        if (DIM == 3) {
            inside *= (int)((zp < k.flow_tfr[2] && zp > k.flow_lbb[2]) ||
                            ((k.flow_lbb[2] - zp) * (k.flow_lbb[2] - zp) <= riSq) ||
                            ((k.flow_tfr[2] - zp) * (k.flow_tfr[2] - zp) <= riSq));
            vpz += !inside * multiplier * f2 + k.flow_vel[2] * inside;
        }
        vpx += !inside * multiplier * f0 + k.flow_vel[0] * inside;
        vpy += !inside * multiplier * f1 + k.flow_vel[1] * inside;
    }
    if (shear) {  // linear shear along x over the last axis (cb_config.shear_speed)
        const double q = DIM == 3 ? zp : yp;
        vpx += k.shear * ((q - k.lbb[DIM - 1]) * k.shear_il - 1.0);
    }
    if (k.any_wall) {  // addWallVelocity, src/kernels.cu:546-593
        double xDrag = 1.0, yDrag = 1.0, velocity = 0.0;
        if (k.wall[0] && touches_wall(k.f0, rp, xp, k.lbb[0], k.tfr[0], velocity)) {
            vpx += velocity;
            vpy *= drag;
            vpz *= drag;
            xDrag = drag;
        }
        velocity = 0.0;
        if (k.wall[1] && touches_wall(k.f0, rp, yp, k.lbb[1], k.tfr[1], velocity)) {
            vpx *= drag;
            vpy += velocity * xDrag;
            vpz *= drag;
            yDrag = drag;
        }
        velocity = 0.0;
        if (k.wall[2] && touches_wall(k.f0, rp, zp, k.lbb[2], k.tfr[2], velocity)) {
            vpx *= drag;
            vpy *= drag;
            vpz += velocity * xDrag * yDrag;
        }
    }
    return {vpx, vpy, vpz};
}

// |(a, b, c)| of exact FP64 differences of nearby positions: squares, sum
// and root in float-float (~2^-46), no FP64 instruction.
static __device__ __noinline__ double norm_slow(double s) { return s > 0.0 ? sqrt(s) : 0.0; }
template <int DIM>
__device__ __forceinline__ double norm_ffd(double a, double b, double c) {
    ff s = ff_add(ff_sqr(ff_of(a)), ff_sqr(ff_of(b)));
    if (DIM == 3) s = ff_add(s, ff_sqr(ff_of(c)));
    if (!(s.h > 0x1p-100f && s.h < 0x1p100f)) {
        double d = a * a + b * b;
        if (DIM == 3) d += c * c;
        return norm_slow(d);
    }
    return ff_to_double(ff_sqrt(s));
}

template <int DIM>
__device__ __forceinline__ void k_correct_body(const Bufs &b, const int vb, const int vg) {
    __shared__ double smem[32];
    __shared__ int ismem[32];
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const double ts = c->dt;
    const double h = 0.5 * ts;
    const int gas = c->use_gas, path = c->inc_path;
    const int flow = c->use_flow && !k.shear_on, shear = c->use_flow && k.shear_on;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    double *XN = drow(b, c, RXN), *YN = drow(b, c, RYN), *ZN = drow(b, c, RZN),
           *RN = drow(b, c, RRN);
    const double *V0 = drow(b, c, RV0), *V1 = drow(b, c, RV1), *V2 = drow(b, c, RV2),
                 *V3 = drow(b, c, RV3);
    double *P0 = drow(b, c, RVP0), *P1 = drow(b, c, RVP1), *P2 = drow(b, c, RVP2),
           *P3 = drow(b, c, RVP3);
    const double *S0 = drow(b, c, RS0), *S1 = drow(b, c, RS1), *S2 = drow(b, c, RS2),
                 *S3 = drow(b, c, RS3);
    const double *PATH = drow(b, c, RPATH);
    double *PATHN = drow(b, c, RPATHN), *ERR = drow(b, c, RERR);
    const int *NN = irow(b, c, INN);
    // mean-field factors, src/kernels.cu:399-408 (uniform over bubbles).
    // The overlap row ov and the pairwise rate are in units of ov_unit, and
    // so is the area here: 4 r^2 (3D), pi r (2D); the unit goes into kq, the
    // factor K ov_unit / area = kq / r^2 (/ r)
    const double mfa = c->mfa, mfb = c->mfb;
    const double kq = DIM == 3 ? k.K * 0.25 : k.K * (1.0 / kPi);
    const double drag = 1.0 - k.wall_drag;
    long long merr = 0, mrad = 0, mexp = 0;
    double vol = 0.0;
    int ndel = 0, bad = 0;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += vg * blockDim.x) {
        double *acc = b.acc + (size_t)i * kAcc;
        const double4_32a a0 = reinterpret_cast<const double4_32a *>(acc)[0];
        double4_32a a1;
        a1.x = a1.y = a1.z = a1.w = 0.0;
        if (gas || flow) a1 = reinterpret_cast<const double4_32a *>(acc)[1];
        double vpx = a0.x, vpy = a0.y, vpz = a0.z, vpr = a0.w;
        const double ov = a1.x;
        const double4_32a p = ld4(b.pred, i);
        const double xp = p.x, yp = p.y, zp = DIM == 3 ? p.z : 0.0, rp = DIM == 3 ? p.w : p.z;
        if (flow | shear | k.any_wall) {
            const Vel3 v = boundary_velocity<DIM>(k, flow, shear, drag, vpx, vpy, vpz, xp, yp, zp,
                                                  rp, a1.y, a1.z, a1.w, flow ? NN[i] : 0);
            vpx = v.x;
            vpy = v.y;
            vpz = v.z;
        }
        // AM2 correct x + 0.5 ts (v + vp), src/kernels.cu:487-495 and :366-387
        long long e = 0;
        // inputs read after the first store below, loaded up front (a load
        // cannot move across a store the compiler thinks may alias it)
        const double err0 = ERR[i], path0 = path ? PATH[i] : 0.0;
        const double x0 = X[i], y0 = Y[i];
        const double cx = fma(h, V0[i] + vpx, x0);
        e = max_bits(e, abs_bits(xp - cx));
        const double cy = fma(h, V1[i] + vpy, y0);
        e = max_bits(e, abs_bits(yp - cy));
        double cz = 0.0, z0 = 0.0, sz = 0.0;
        if (DIM == 3) {
            z0 = Z[i];
            cz = fma(h, V2[i] + vpz, z0);
            e = max_bits(e, abs_bits(zp - cz));
            sz = cz - S2[i];
        }
        // distance from the position of the last search; only its maximum
        // over the foam is used (the search trigger)
        double dist = norm_ffd<DIM>(cx - S0[i], cy - S1[i], sz);
        int del = 0;
        if (gas) {  // mean-field gas exchange and radius, src/kernels.cu:390-431
            double inv, area;
            if (DIM == 3) {  // (1/rp, rp^2) record of k_predict
                const double2 e = reinterpret_cast<const double2 *>(b.invr)[i];
                inv = e.x;
                area = 4.0 * e.y;
            } else {
                inv = p.w;
                area = kPi * rp;
            }
            double vr = mfa - inv;
            vr *= mfb * (area - ov);
            vr += vpr;
            vr *= DIM == 3 ? kq * (inv * inv) : kq * inv;
            vpr = vr;
            const double cr = fma(h, V3[i] + vr, R[i]);
            e = max_bits(e, abs_bits(rp - cr));
            dist += cr - S3[i];
            if (__double_as_longlong(cr) > __double_as_longlong(k.min_rad)) {  // cr > minRad
                vol = fma(DIM == 3 ? cr * cr : cr, cr, vol);
            } else {
                del = 1;
                ndel++;
            }
            mrad = max_bits(mrad, cr);
            RN[i] = cr;
            P3[i] = vpr;
            bad |= !finite_bits(cr);
        }
        b.delflag[i] = del;
        mexp = max_bits(mexp, dist);
        if (path)  // src/kernels.cu:437-451; the increment to ~2^-46
            PATHN[i] = path0 + norm_ffd<DIM>(x0 - cx, y0 - cy, z0 - cz);
        ERR[i] = __longlong_as_double(max(e, __double_as_longlong(err0)));  // both >= 0
        merr = max(merr, e);
        XN[i] = cx;
        YN[i] = cy;
        P0[i] = vpx;
        P1[i] = vpy;
        if (DIM == 3) {
            ZN[i] = cz;
            P2[i] = vpz;
        }
        bad |= !(finite_bits(cx) && finite_bits(cy) && finite_bits(cz));
        if (b.dbg_ov) b.dbg_ov[i] = ov_unit(DIM) * ov;
        // leave the accumulators zeroed for the next attempt
        double4_32a zero;
        zero.x = zero.y = zero.z = zero.w = 0.0;
        reinterpret_cast<double4_32a *>(acc)[0] = zero;
        if (gas || flow) reinterpret_cast<double4_32a *>(acc)[1] = zero;
    }
    long long *lsm = reinterpret_cast<long long *>(smem);
    const double tErr = __longlong_as_double(block_max_bits(merr, lsm));
    const double tRad = __longlong_as_double(block_max_bits(mrad, lsm));
    const double tExp = __longlong_as_double(block_max_bits(mexp, lsm));
    const double tVol = block_reduce(vol, OpSum(), smem);
    const int tDel = block_reduce_int(ndel, ismem);
    const int tBad = block_reduce_int(bad, ismem);
    const int G = vg;
    if (threadIdx.x == 0) {
        b.part[0 * G + vb] = tErr;
        b.part[1 * G + vb] = tRad;
        b.part[2 * G + vb] = tExp;
        b.part[3 * G + vb] = tVol;
        b.part[4 * G + vb] = (double)tDel;
        b.part[5 * G + vb] = (double)tBad;
    }
    if (!last_block(&c->done[DC_CORRECT], vg)) return;
    const double fErr = fold_partials(b.part + 0 * G, G, true, smem);
    const double fRad = fold_partials(b.part + 1 * G, G, true, smem);
    const double fExp = fold_partials(b.part + 2 * G, G, true, smem);
    const double fVol = fold_partials(b.part + 3 * G, G, false, smem);
    const double fDel = fold_partials(b.part + 4 * G, G, false, smem);
    const double fBad = fold_partials(b.part + 5 * G, G, false, smem);
    if (threadIdx.x != 0) return;
    finish_attempt<DIM>(c, k, fErr, fRad, fExp, fVol, fDel, fBad);
}
CB_KERNEL_PAIR((template <int DIM>), k_correct, (<DIM>), __launch_bounds__(kBlock))


// --------------------------------------------------------------- bootstrap
// phase 0: pred := (x, r), vo := 0, path := 0
// phase 1: euler pred += acc * dt (src/kernels.cu:959-969), acc := 0
// phase 2: vo := acc (= F(x + dt F(x))), acc := 0
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_boot(Bufs b, int phase) {
    const Ctrl *c = b.ctrl;
    const int n = c->n;
    const double ts = c->dt;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    double *O0 = drow(b, c, RVO0), *O1 = drow(b, c, RVO1), *O2 = drow(b, c, RVO2),
           *O3 = drow(b, c, RVO3), *PATH = drow(b, c, RPATH);
    double4_32a *P = reinterpret_cast<double4_32a *>(b.pred);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double *acc = b.acc + (size_t)i * kAcc;
        if (phase == 0) {
            double4_32a p;
            const double r = R[i];
            p.x = X[i];
            p.y = Y[i];
            const double inv = 1.0 / r, rsq = r * r;
            if (b.ffr) st_rec(b.ffr, i, r, inv, rsq);
            if (DIM == 3) {
                p.z = Z[i];
                p.w = r;
                reinterpret_cast<double2 *>(b.invr)[i] = make_double2(inv, rsq);
            } else {
                p.z = r;
                p.w = inv;
            }
            P[i] = p;
            O0[i] = O1[i] = O2[i] = O3[i] = 0.0;
            PATH[i] = 0.0;
        } else {
            double4_32a a = reinterpret_cast<double4_32a *>(acc)[0];
            if (phase == 1) {
                double4_32a p = P[i];
                p.x += a.x * ts;
                p.y += a.y * ts;
                if (DIM == 3) p.z += a.z * ts;
                P[i] = p;
            } else {
                O0[i] = a.x;
                O1[i] = a.y;
                if (DIM == 3) O2[i] = a.z;
            }
            a.x = a.y = a.z = a.w = 0.0;
            reinterpret_cast<double4_32a *>(acc)[0] = a;
        }
    }
}

// ------------------------------------------------------- energy, volume
// potentialEnergy, src/kernels.cu:941-957, on the current positions.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_energy(Bufs b, int per_bubble) {
    __shared__ double smem[32];
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int np = c->np;
    const int *PI = b.ps[c->prole[PI0]];
    const int *PJ = b.ps[c->prole[PJ0]];
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    double tot = 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int i = PI[p], j = PJ[p];
        double dx, dy, dz;
        wrapped_diff<DIM>(k, X[i], Y[i], DIM == 3 ? Z[i] : 0.0, X[j], Y[j], DIM == 3 ? Z[j] : 0.0,
                          dx, dy, dz);
        double m = dx * dx + dy * dy;
        if (DIM == 3) m += dz * dz;
        double e = R[i] + R[j] - sqrt(m);
        if (e > 0) {
            e *= e;
            tot += 2.0 * e;
            if (per_bubble) {
                atomicAdd(b.energy + i, e);
                atomicAdd(b.energy + j, e);
            }
        }
    }
    const double t = block_reduce(tot, OpSum(), smem);
    if (threadIdx.x == 0) b.part[6 * gridDim.x + blockIdx.x] = t;
    if (last_block(&c->done[DC_MISC], gridDim.x)) {
        const double f = fold_partials(b.part + 6 * gridDim.x, gridDim.x, false, smem);
        if (threadIdx.x == 0) {
            c->misc_result = f;
            c->done[DC_MISC] = 0;
        }
    }
}

// calculateVolumes + sum, src/kernels.cu:1013-1024, src/simulator.cu:362-379
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_volume(Bufs b) {
    __shared__ double smem[32];
    Ctrl *c = b.ctrl;
    const int n = c->n;
    const double *R = drow(b, c, RR);
    double tot = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double radius = R[i];
        double volume = radius * radius * kPi;
        if (DIM == 3) volume *= radius * 1.33333333333333333333333333;
        tot += volume;
    }
    const double t = block_reduce(tot, OpSum(), smem);
    if (threadIdx.x == 0) b.part[6 * gridDim.x + blockIdx.x] = t;
    if (last_block(&c->done[DC_MISC], gridDim.x)) {
        const double f = fold_partials(b.part + 6 * gridDim.x, gridDim.x, false, smem);
        if (threadIdx.x == 0) {
            c->misc_result = f;
            c->done[DC_MISC] = 0;
        }
    }
}

}  // namespace

void launch_predict(const Launch &l, const Bufs &b, int dim) {
    if (dim == 3)
        CB_LAUNCH(l, k_predict, (<3>), wave_grid(k_predict<3>, l, l.step_bps), b);
    else
        CB_LAUNCH(l, k_predict, (<2>), wave_grid(k_predict<2>, l, l.step_bps), b);
}

// mode bits: 1 = gas exchange, 2 = flow. mode 0 is the bootstrap form.
void launch_pairs(const Launch &l, const Bufs &b, int dim, int mode, bool ff) {
    const bool gas = mode & 1, flow = mode & 2;
#define CB_PAIRS(D, G, F)                                                                     \
    do {                                                                                      \
        if (ff)                                                                               \
            CB_LAUNCH(l, k_pairs_ff, (<D, G, F>), wave_grid(k_pairs_ff<D, G, F>, l, l.pair_bps), b);      \
        else                                                                                  \
            CB_LAUNCH(l, k_pairs, (<D, G, F>), wave_grid(k_pairs<D, G, F>, l, l.pair_bps), b);            \
    } while (0)
    if (dim == 3) {
        if (gas && flow) CB_PAIRS(3, true, true);
        else if (gas) CB_PAIRS(3, true, false);
        else if (flow) CB_PAIRS(3, false, true);
        else CB_PAIRS(3, false, false);
    } else {
        if (gas && flow) CB_PAIRS(2, true, true);
        else if (gas) CB_PAIRS(2, true, false);
        else if (flow) CB_PAIRS(2, false, true);
        else CB_PAIRS(2, false, false);
    }
#undef CB_PAIRS
}

void launch_correct(const Launch &l, const Bufs &b, int dim) {
    if (dim == 3)
        CB_LAUNCH(l, k_correct, (<3>), wave_grid(k_correct<3>, l, l.step_bps), b);
    else
        CB_LAUNCH(l, k_correct, (<2>), wave_grid(k_correct<2>, l, l.step_bps), b);
}

void launch_boot(const Launch &l, const Bufs &b, int dim, int phase) {
    if (dim == 3)
        k_boot<3><<<l.grid, kBlock, 0, l.stream>>>(b, phase);
    else
        k_boot<2><<<l.grid, kBlock, 0, l.stream>>>(b, phase);
    *l.launches += 1;
}

void launch_energy(const Launch &l, const Bufs &b, int dim, int per_bubble) {
    if (dim == 3)
        k_energy<3><<<l.grid, kBlock, 0, l.stream>>>(b, per_bubble);
    else
        k_energy<2><<<l.grid, kBlock, 0, l.stream>>>(b, per_bubble);
    *l.launches += 1;
}

void launch_volume(const Launch &l, const Bufs &b, int dim) {
    if (dim == 3)
        k_volume<3><<<l.grid, kBlock, 0, l.stream>>>(b);
    else
        k_volume<2><<<l.grid, kBlock, 0, l.stream>>>(b);
    *l.launches += 1;
}

}  // namespace cbg
