// One attempt of the step in the mixed form (cb_config.precision =
// CB_PRECISION_MIXED). Same algorithm and control as step.cu; what changes is
// the arithmetic of the pair interaction and the storage of the rates:
//   * FP64: absolute positions and radii (x, y, z, r and their corrected
//     values), path, the predictor-corrector error norm and its reduction,
//     the volume sum of the survivors and the volume fix, the global area
//     sums, the energy;
//   * FP32: velocities and radius rates (the dxdt / dxdto / dxdtp rows hold
//     floats), the pair geometry, overlap velocities, overlap areas and the
//     gas flux, the mean-field arithmetic per bubble, the expansion since the
//     last search (from the FP64 difference to the saved position).
//
// GB300 runs FP64 arithmetic *and* every 64-bit conversion (double <-> int64,
// float <-> double, int64 -> float) on one unit at 1/64 of the FP32 rate.
// The mixed kernels therefore convert on the integer pipe, from the IEEE-754
// bit patterns (fix_from_double, fix_from_float, double_from_float,
// float_from_double below; float_rn_from_double, rounded to nearest, where a
// conversion toward zero would bias every bubble alike), and use FP64
// arithmetic only for the position,
// radius and path updates, the differences to the saved position and the
// volume sum (12 FP64 instructions per bubble in 3D).
//
// Pair geometry works on exact differences of 64-bit fixed-point coordinates
// q = x * 2^40 (|x| < 2^21): the integer difference q_i - q_j is exact at any
// separation (also for nearly coincident bubbles); the minimum image on a
// periodic axis is an integer compare against half the box
// (wrappedDifference, src/kernels.cu:1094-1114). Only the final conversion of
// the difference to FP32 rounds (relative 2^-24). The predicted radius is
// fixed point too, so the overlap product (r_1 + r_2)^2 - d^2, a difference
// of nearly equal squares for the shallow overlaps of a foam, is formed from
// exact integers (overlap_product). The packed predicted state is 32 bytes
// per bubble (q_x, q_y, q_z, q_r) and the pair kernel adds its results with
// 16-byte vector FP32 reductions.
#include "common.cuh"

namespace cbg {
namespace {

__device__ __forceinline__ float *frow(const Bufs &b, const Ctrl *c, int role) {
    return reinterpret_cast<float *>(b.ds[c->drole[role]]);
}

// ------------------------------------------------- integer-pipe conversions
// (fix_from_double and len_from_fix are in common.cuh)
// f * 2^40 rounded toward zero, from the bits of f (|f| < 2^23).
__device__ __forceinline__ long long fix_from_float(float f) {
    const int b = __float_as_int(f);
    const int e = (b >> 23) & 0xff;
    const long long m = (long long)((b & 0x7fffff) | 0x800000);
    const int sh = e - (150 - kFixBits);  // f = m 2^(e - 150)
    long long q = sh >= 0 ? (m << min(sh, 39)) : (sh > -64 ? (m >> -sh) : 0LL);
    if (e == 0) q = 0;
    return b < 0 ? -q : q;
}

// Exact float -> double from the bits (FP32 subnormals become 0).
__device__ __forceinline__ double double_from_float(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xffu;
    const unsigned long long s = (unsigned long long)(b >> 31) << 63;
    if (e == 0) return __longlong_as_double((long long)s);
    const unsigned long long de = e == 0xffu ? 0x7ffull : (unsigned long long)(e + 896u);
    return __longlong_as_double(
        (long long)(s | (de << 52) | ((unsigned long long)(b & 0x7fffffu) << 29)));
}

// double -> float rounded toward zero, from the bits.
__device__ __forceinline__ float float_from_double(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned int s = (unsigned int)(b >> 63) << 31;
    const unsigned int man = (unsigned int)((b >> 29) & 0x7fffffull);
    const int fe = e - 896;
    unsigned int bits;
    if (e == 0x7ff)
        bits = s | 0x7f800000u | man | ((b & 0xfffffffffffffull) ? 0x400000u : 0u);
    else if (fe <= 0)
        bits = s;
    else if (fe >= 255)
        bits = s | 0x7f800000u;
    else
        bits = s | ((unsigned int)fe << 23) | man;
    return __uint_as_float(bits);
}

// The same, rounded to nearest (ties to even) instead of truncated: for the
// values whose rounding direction would otherwise bias every bubble the same
// way (the half step h, the mean-field factor, the radius in the gas-exchange
// term). Truncated, they moved the total volume away from the FP64 form's by
// 1.5e-10 over 300 steps at N = 10^6; rounded, by 3e-12.
__device__ __forceinline__ float float_rn_from_double(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    const int fe = e - 896;
    if (e == 0x7ff || fe <= 0 || fe >= 255) return float_from_double(x);
    unsigned int bits = ((unsigned int)(b >> 63) << 31) | ((unsigned int)fe << 23) |
                        (unsigned int)((b >> 29) & 0x7fffffull);
    const unsigned long long low = b & 0x1fffffffull;  // the 29 dropped bits
    if (low > 0x10000000ull || (low == 0x10000000ull && (bits & 1u))) bits += 1u;  // carries into the exponent
    return __uint_as_float(bits);
}

// Minimum image of a fixed-point difference on a periodic axis.
__device__ __forceinline__ long long wrap_fix(long long d, long long half, long long len) {
    if (d > half) d -= len;
    else if (d < -half) d += len;
    return d;
}

// Accumulator layout of the mixed form inside `acc` (64 bytes per bubble):
// float4 velocity sums (vx, vy, vz, vr) at [0, 16 cap), float overlap at
// [16 cap, 20 cap), float4 flow sums at [32 cap, 48 cap) bytes. In 2D the
// velocity float4 is (vx, vy, overlap, vr) and the overlap row is unused.
__device__ __forceinline__ float4 *acc_v(const Bufs &b) { return reinterpret_cast<float4 *>(b.acc); }
__device__ __forceinline__ float *acc_ov(const Bufs &b, int cap) {
    return reinterpret_cast<float *>(b.acc) + 4 * (size_t)cap;
}
__device__ __forceinline__ float4 *acc_fl(const Bufs &b, int cap) {
    return reinterpret_cast<float4 *>(reinterpret_cast<float *>(b.acc) + 8 * (size_t)cap);
}
// The containment recheck list of the pair kernel (see k_pairs_mx) in the
// unused bytes [48 cap, 64 cap) of the accumulators: element 0 holds the
// count, then up to recheck_cap(cap) pairs (i, j). Zero between attempts.
__device__ __forceinline__ int2 *recheck_list(float4 *AV, int cap) {
    return reinterpret_cast<int2 *>(AV + 3 * (size_t)cap);
}
__device__ __forceinline__ int recheck_cap(int cap) { return min(1024 + cap / 128, 2 * cap - 1); }

__device__ __forceinline__ void red_add4(float4 *p, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b),
                 "f"(c), "f"(d)
                 : "memory");
}

// Predicted state of one bubble in the mixed form (32 bytes): position and
// radius as fixed point x 2^40.
struct __align__(16) PredMx {
    long long q[3];
    long long qr;
};

// One 32-byte load per record (a 256-bit vector load; records are 32-byte
// aligned). Not volatile: the records are read-only while a kernel reads
// them, so the compiler may schedule these loads freely.
__device__ __forceinline__ PredMx ld_pred(const double *base, int i) {
    const long long *p = reinterpret_cast<const long long *>(base) + 4 * (size_t)i;
    long long a, b, c, d;
    asm("ld.global.v4.u64 {%0, %1, %2, %3}, [%4];"
        : "=l"(a), "=l"(b), "=l"(c), "=l"(d)
        : "l"(p));
    PredMx r;
    r.q[0] = a;
    r.q[1] = b;
    r.q[2] = c;
    r.qr = d;
    return r;
}

__device__ __forceinline__ void st_pred(double *base, int i, const PredMx &r) {
    longlong2 *p = reinterpret_cast<longlong2 *>(base) + 2 * (size_t)i;
    p[0] = make_longlong2(r.q[0], r.q[1]);
    p[1] = make_longlong2(r.q[2], r.qr);
}

// The predicted radius as FP32 (one rounding of the fixed-point value, which
// is >= 0).
__device__ __forceinline__ float pred_r(const PredMx &p) {
    const unsigned long long a = (unsigned long long)p.qr;
    return fmaf(__uint2float_rn((unsigned int)(a >> 32)), 4294967296.f,
                __uint2float_rn((unsigned int)a)) *
           kFixInv;
}

// The prediction the coming attempt uses: slot 0 (k_predict_mx) or one of
// the two candidates the last correct wrote.
__device__ __forceinline__ const double *pred_base(const Bufs &b, const Ctrl *c, int cap) {
    const int s = c->pred_slot;
    return s == 0 ? b.pred : b.predc + (size_t)(s - 1) * 4 * cap;
}

// ---------------------------------------------------------------- predict
// Skipped (every block returns at once) when the last correct already
// wrote this attempt's prediction and its area sums.
template <int DIM>
__device__ __forceinline__ void k_predict_mx_body(const Bufs &b, const int vb, const int vg) {
    __shared__ double smem[32];
    const Ctrl *c = b.ctrl;
    if (c->pred_ready) return;
    const int n = c->n;
    const float h = float_rn_from_double(0.5 * c->dt);
    const int gas = c->use_gas;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    const float *V0 = frow(b, c, RV0), *V1 = frow(b, c, RV1), *V2 = frow(b, c, RV2),
                *V3 = frow(b, c, RV3);
    const float *O0 = frow(b, c, RVO0), *O1 = frow(b, c, RVO1), *O2 = frow(b, c, RVO2),
                *O3 = frow(b, c, RVO3);
    float sA = 0.f, sAr = 0.f;
    // two bubbles per iteration, all loads of both issued before any store
    // (twice the loads in flight of a one-bubble loop)
    const int stride = vg * blockDim.x;
    for (int i0 = vb * blockDim.x + threadIdx.x; i0 < n; i0 += 2 * stride) {
        const int i1 = i0 + stride < n ? i0 + stride : i0;
        const int ii[2] = {i0, i1};
        double x[2], y[2], z[2], r[2];
        float d[4][2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int i = ii[u];
            x[u] = __ldg(X + i);
            y[u] = __ldg(Y + i);
            z[u] = DIM == 3 ? __ldg(Z + i) : 0.0;
            r[u] = __ldg(R + i);
            // AB2 direction 3 v - vo
            d[0][u] = fmaf(3.f, __ldg(V0 + i), -__ldg(O0 + i));
            d[1][u] = fmaf(3.f, __ldg(V1 + i), -__ldg(O1 + i));
            d[2][u] = DIM == 3 ? fmaf(3.f, __ldg(V2 + i), -__ldg(O2 + i)) : 0.f;
            d[3][u] = gas ? fmaf(3.f, __ldg(V3 + i), -__ldg(O3 + i)) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (u == 1 && ii[1] == ii[0]) break;
            // AB2 increment h (3 v - vo) in FP32 on the fixed point of x
            PredMx p;
            p.q[0] = fix_from_double(x[u]) + fix_from_float(h * d[0][u]);
            p.q[1] = fix_from_double(y[u]) + fix_from_float(h * d[1][u]);
            p.q[2] = DIM == 3 ? fix_from_double(z[u]) + fix_from_float(h * d[2][u]) : 0LL;
            p.qr = fix_from_double(r[u]) + (gas ? fix_from_float(h * d[3][u]) : 0LL);
            st_pred(b.pred, ii[u], p);
            const float rp = pred_r(p);
            if (gas) {
                const float apr = DIM == 3 ? (4.f * (float)kPi) * rp : 2.f * (float)kPi;
                sA = fmaf(apr, rp, sA);
                sAr += apr;
            }
        }
    }
    const double tA = block_sum_f(sA, smem);
    const double tAr = block_sum_f(sAr, smem);
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
CB_KERNEL_PAIR((template <int DIM>), k_predict_mx, (<DIM>), __launch_bounds__(kBlock))


// ------------------------------------------------------------------ pairs
// FP32 geometry of a pair on exact fixed-point differences: the minimum image
// on periodic axes (wrappedDifference, src/kernels.cu:1094-1114), the
// differences as FP32 and the squared distance m.
// Periodic axes and the fixed-point box (half) lengths, read once per kernel.
struct FixBox {
    bool px, py, pz;
    long long hx, hy, hz, lx, ly, lz;
};

__device__ __forceinline__ FixBox fix_box(const DevConst &k, int dim) {
    return {!k.wall[0], !k.wall[1], dim == 3 && !k.wall[2], k.hq[0], k.hq[1], k.hq[2],
            k.lq[0], k.lq[1], k.lq[2]};
}

template <int DIM>
__device__ __forceinline__ void pair_diff(const PredMx &a, const PredMx &q, const FixBox &f,
                                          long long &ex, long long &ey, long long &ez,
                                          float &dx, float &dy, float &dz, float &m) {
    ex = a.q[0] - q.q[0];
    ey = a.q[1] - q.q[1];
    ez = 0;
    if (f.px) ex = wrap_fix(ex, f.hx, f.lx);
    if (f.py) ey = wrap_fix(ey, f.hy, f.ly);
    if (DIM == 3) {
        ez = a.q[2] - q.q[2];
        if (f.pz) ez = wrap_fix(ez, f.hz, f.lz);
    }
    dx = len_from_fix(ex);
    dy = len_from_fix(ey);
    dz = DIM == 3 ? len_from_fix(ez) : 0.f;
    m = dx * dx;
    m = fmaf(dy, dy, m);
    if (DIM == 3) m = fmaf(dz, dz, m);
}

// A 64-bit integer as FP32 on the integer pipe (two 32-bit conversions and
// an FMA; the 64-bit conversion would run on the FP64 unit).
__device__ __forceinline__ float f32_from_i64(long long v) {
    const unsigned long long a = (unsigned long long)(v < 0 ? -v : v);
    const float f = fmaf(__uint2float_rn((unsigned int)(a >> 32)), 4294967296.f,
                         __uint2float_rn((unsigned int)a));
    return v < 0 ? -f : f;
}

// (r_1 + r_2)^2 - d^2 of an overlapping pair from exact integers. For shallow
// overlaps it is a difference of nearly equal squares, and its FP32 form
// fmaf(R, R, -d^2) carries the roundings of d^2 and of the radii, ~10^-7 R^2,
// into the overlap velocity f0 (R - |d|) / (|d| R) and the lens area. Here the
// fixed-point differences e and radius sum rq (units 2^-40) are split as
// v = h 2^20 + l (0 <= l < 2^20), so that, in units 2^-80,
//   rq^2 - sum e^2 = (h_r^2 - sum h^2) 2^40 + 2 (h_r l_r - sum h l) 2^20 + (l_r^2 - sum l^2),
// the first two brackets exact in 64-bit integers while the radius sum is
// below 2^44 (16 length units; the pair overlaps, so every |e| is below it
// too); the third, below 2^-38 absolute, is left out, and the second enters
// to 2^19 of its units (2^-40 absolute). One FP32 rounding of the result.
// Larger radii take the FP32 expression.
__device__ __forceinline__ float overlap_product(long long ex, long long ey, long long ez,
                                                 long long rq, float radii, float m) {
    if (rq >= (1LL << 44)) return fmaf(radii, radii, -m);
    const int hx = (int)(ex >> 20), hy = (int)(ey >> 20), hz = (int)(ez >> 20),
              hr = (int)(rq >> 20);
    const int lx = (int)(ex & 0xfffff), ly = (int)(ey & 0xfffff), lz = (int)(ez & 0xfffff),
              lr = (int)(rq & 0xfffff);
    const long long k1 = (long long)hr * hr -
                         ((long long)hx * hx + (long long)hy * hy + (long long)hz * hz);
    const long long k2 = (long long)hr * lr -
                         ((long long)hx * lx + (long long)hy * ly + (long long)hz * lz);
    return f32_from_i64(k1 + (k2 >> 19)) * kFixInv;
}

// Overlap area of an overlapping pair (src/kernels.cu:236-256): min(r1, r2)^2
// (3D, times pi) or 2 min(r1, r2) (2D) when one centre lies inside the other
// bubble, else from the squared half chord a^2. The reference evaluates
// a^2 = r2^2 - (r2^2 - r1^2 + d^2)^2 / (4 d^2), which cancels badly when a
// small bubble sits on a large one (1.69 - 1.68 for radii 0.1 and 1.3); the
// same quantity is evaluated here in the product form of the height of the
// triangle (r1, r2, d), a^2 = ((r1 + r2)^2 - d^2) (d^2 - (r1 - r2)^2) / (4 d^2),
// whose two factors carry the FP32 rounding of d^2 and the radii only; p =
// (r1 + r2)^2 - d^2 comes from overlap_product.
template <int DIM>
__device__ __forceinline__ float overlap_area(float r1, float r2, float r1sq, float r2sq,
                                              float p, float m, float rs, bool inside) {
    if (inside) return DIM == 3 ? fminf(r1sq, r2sq) * (float)kPi : 2.f * fminf(r1, r2);
    const float rd = r1 - r2;
    const float q = fmaf(-rd, rd, m);
    const float oa = fabsf(p * q * (0.25f * (rs * rs)));
    return DIM == 3 ? oa * (float)kPi : 2.f * sqrtf(oa);
}

// The overlap area jumps where one centre enters the other bubble (at
// d^2 = max(r1^2, r2^2) the lens formula gives r1^2 - r1^4 / (4 r2^2), the
// containment branch r1^2: a step of pi r1^4 / (4 r2^2) in 3D). The FP32 test
// can decide a pair within its rounding error of that threshold either way.
// Such pairs (relative distance below kContainBand: a few per 10^6 bubbles
// and attempt) are appended to a list; the last block of the pair kernel
// decides them again in FP64 — on the exact fixed-point differences and on
// both predicted radii recomputed from the state rows, r + h (3 v_r -
// v_r,old), as the prediction defines them — and where the decision turns,
// adds the difference of the two areas to both bubbles and to the global
// sums before the mean-field factors are formed.
constexpr float kContainBand = 3.814697265625e-06f;  // 2^-18

__device__ __forceinline__ bool contained_exact(long long ex, long long ey, long long ez, int i,
                                                int j, double *const *ds, const Ctrl *c) {
    const double s = 9.094947017729282379e-13;  // 2^-40
    const double dx = (double)ex * s, dy = (double)ey * s, dz = (double)ez * s;
    const double m = dx * dx + dy * dy + dz * dz;
    const double *R = ds[c->drole[RR]];
    const float *V3 = reinterpret_cast<const float *>(ds[c->drole[RV3]]);
    const float *O3 = reinterpret_cast<const float *>(ds[c->drole[RVO3]]);
    const double h = (double)float_rn_from_double(0.5 * c->dt);
    const double r1 = R[i] + h * (double)fmaf(3.f, V3[i], -O3[i]);
    const double r2 = R[j] + h * (double)fmaf(3.f, V3[j], -O3[j]);
    return m < r1 * r1 || m < r2 * r2;
}

// Last block of the pair kernel: the listed pairs decided again (see above).
// Returns this thread's changes of the summed overlap area and of the summed
// area over radius.
template <int DIM>
__device__ __forceinline__ float2 recheck_containment(const int2 *RC, double *const *ds,
                                                      const Ctrl *c, const DevConst *kp,
                                                      const double *PB, float4 *AV, float *AO) {
    const DevConst &k = *kp;
    float so = 0.f, sor = 0.f;
    const int cnt = min(RC[0].x, recheck_cap(k.cap));
    const FixBox fb = fix_box(k, DIM);
    for (int e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int2 pr = RC[1 + e];
        const PredMx a = ld_pred(PB, pr.x), q = ld_pred(PB, pr.y);
        long long ex, ey, ez;
        float dx, dy, dz, m;
        pair_diff<DIM>(a, q, fb, ex, ey, ez, dx, dy, dz, m);
        const float r1 = pred_r(a), r2 = pred_r(q), r1sq = r1 * r1, r2sq = r2 * r2;
        const bool fast = m < fmaxf(r1sq, r2sq);
        const bool exact = contained_exact(ex, ey, ez, pr.x, pr.y, ds, c);
        if (fast == exact) continue;
        const float rs = rsqrtf(m), radii = r1 + r2;
        const float pp = overlap_product(ex, ey, ez, a.qr + q.qr, radii, m);
        const float d = overlap_area<DIM>(r1, r2, r1sq, r2sq, pp, m, rs, exact) -
                        overlap_area<DIM>(r1, r2, r1sq, r2sq, pp, m, rs, fast);
        const float inv1 = __fdividef(1.f, r1), inv2 = __fdividef(1.f, r2);
        const float dg = d * (inv2 - inv1);
        if (DIM == 3) {
            atomicAdd(AO + pr.x, d);
            atomicAdd(AO + pr.y, d);
            red_add4(AV + pr.x, 0.f, 0.f, 0.f, dg);
            red_add4(AV + pr.y, 0.f, 0.f, 0.f, -dg);
        } else {
            red_add4(AV + pr.x, 0.f, 0.f, d, dg);
            red_add4(AV + pr.y, 0.f, 0.f, d, -dg);
        }
        so += d;
        sor = fmaf(d, inv1 + inv2, sor);
    }
    return make_float2(so, sor);
}

// RUN consecutive entries of a pair-list row with vector loads (the run
// starts at a multiple of RUN, so the loads are aligned).
template <int RUN>
__device__ __forceinline__ void load_run(const int *P, int p0, int (&v)[RUN]) {
    if (RUN == 2) {
        const int2 u = *reinterpret_cast<const int2 *>(P + p0);
        v[0] = u.x;
        v[1] = u.y;
    } else {
#pragma unroll
        for (int h = 0; h < RUN; h += 4) {
            const int4 u = *reinterpret_cast<const int4 *>(P + p0 + h);
            v[h] = u.x;
            v[h + 1] = u.y;
            v[h + 2] = u.z;
            v[h + 3] = u.w;
        }
    }
}

// The search emits the pairs grouped by i in ascending order, so consecutive
// pairs mostly share their first bubble. Each thread takes a run of RUN
// consecutive pairs (vector loads of the i's and of the j's), loads the
// prediction of i once per distinct i, keeps i's sums in registers and adds
// them with one vector reduction per distinct i; the j side adds per pair.
// In 2D the overlap sum rides in the third lane of the velocity float4. RUN
// (pairs per thread, 32 RUN per warp) is a tuning knob: 4 by default, 2 or 8
// for the gas-exchange kernels without flow (cb_tuning.pair_run).
template <int DIM, bool GAS, bool FLOW, int RUN>
__device__ __forceinline__ void k_pairs_mx_body(const Bufs &b, const int vb, const int vg) {
    __shared__ double smem[32];
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int np = c->np;
    const int cap = k.cap;
    const int *PI = b.ps[c->prole[PI0]];
    const int *PJ = b.ps[c->prole[PJ0]];
    const float *V0 = frow(b, c, RV0), *V1 = frow(b, c, RV1), *V2 = frow(b, c, RV2);
    float4 *AV = acc_v(b);
    float *AO = acc_ov(b, cap);
    float4 *AF = acc_fl(b, cap);
    const float f0 = k.f0_f;
    const FixBox fb = fix_box(k, DIM);
    const double *PB = pred_base(b, c, cap);
    float sAo = 0.f, sAor = 0.f;
    const int nrun = (np + RUN - 1) / RUN;
    for (int g = vb * blockDim.x + threadIdx.x; g < nrun; g += vg * blockDim.x) {
        const int p0 = g * RUN;
        int I[RUN], J[RUN];
        if (p0 + RUN <= np) {
            load_run<RUN>(PI, p0, I);
            load_run<RUN>(PJ, p0, J);
        } else {
#pragma unroll
            for (int t = 0; t < RUN; t++) {
                I[t] = p0 + t < np ? PI[p0 + t] : -1;
                J[t] = p0 + t < np ? PJ[p0 + t] : 0;
            }
        }
        int cur = -1;
        PredMx a;
        // i's predicted radius and its reciprocal (the reciprocals of the gas
        // flux to ~2 ulp: the flux sums carry that into the radius rates at
        // ~10^-7 of their row maximum)
        float r1 = 0.f, inv1 = 0.f;
        float ax = 0.f, ay = 0.f, az = 0.f, ag = 0.f, ao = 0.f;
        float fx_i = 0.f, fy_i = 0.f, fz_i = 0.f, vxi = 0.f, vyi = 0.f, vzi = 0.f;
        bool hit = false;
        auto flush = [&]() {
            if (DIM == 3) {
                red_add4(AV + cur, ax, ay, az, ag);
                if (GAS) atomicAdd(AO + cur, ao);
            } else {
                red_add4(AV + cur, ax, ay, ao, ag);
            }
            if (FLOW) red_add4(AF + cur, fx_i, fy_i, fz_i, 0.f);
        };
#pragma unroll
        for (int t = 0; t < RUN; t++) {
            const int i = I[t], j = J[t];
            if (i < 0) break;
            if (i != cur) {
                if (hit) flush();
                cur = i;
                a = ld_pred(PB, i);
                r1 = pred_r(a);
                if (GAS) inv1 = __fdividef(1.f, r1);
                ax = ay = az = ag = ao = 0.f;
                fx_i = fy_i = fz_i = 0.f;
                hit = false;
                if (FLOW) {
                    vxi = V0[i];
                    vyi = V1[i];
                    vzi = DIM == 3 ? V2[i] : 0.f;
                }
            }
            if (FLOW)  // src/kernels.cu:191-207 (added for every pair)
                red_add4(AF + j, vxi, vyi, vzi, 0.f);
            const PredMx q = ld_pred(PB, j);
            long long ex, ey, ez;
            float dx, dy, dz, m;
            pair_diff<DIM>(a, q, fb, ex, ey, ez, dx, dy, dz, m);
            const float r2 = pred_r(q);
            const float radii = r1 + r2;
            if (radii * radii >= m) {
                // velocity f0 d (1/|d| - 1/(r1 + r2)), src/kernels.cu:218-233, as
                // f0 d ((r1 + r2)^2 - d^2) / (|d| (r1 + r2) (r1 + r2 + |d|))
                const float rs = rsqrtf(m);
                const float pp = overlap_product(ex, ey, ez, a.qr + q.qr, radii, m);
                const float s = f0 * __fdividef(pp * rs, radii * fmaf(m, rs, radii));
                const float fx = dx * s, fy = dy * s, fz = dz * s;
                float gf = 0.f, oa = 0.f;
                if (GAS) {  // pairwise gas exchange, src/kernels.cu:236-280
                    const float r1sq = r1 * r1, r2sq = r2 * r2;
                    const float rm = fmaxf(r1sq, r2sq);
                    if (fabsf(m - rm) <= kContainBand * rm) {  // decided again at the end
                        int2 *RC = recheck_list(AV, cap);
                        const int e = atomicAdd(&RC[0].x, 1);
                        if (e < recheck_cap(cap)) RC[1 + e] = make_int2(i, j);
                    }
                    oa = overlap_area<DIM>(r1, r2, r1sq, r2sq, pp, m, rs, m < rm);
                    const float inv2 = __fdividef(1.f, r2);
                    gf = oa * (inv2 - inv1);
                    sAo += oa;
                    sAor = fmaf(oa, inv1 + inv2, sAor);
                }
                ax += fx;
                ay += fy;
                az += fz;
                ag += gf;
                ao += oa;
                hit = true;
                if (DIM == 3) {
                    red_add4(AV + j, -fx, -fy, -fz, -gf);
                    if (GAS) atomicAdd(AO + j, oa);
                } else {
                    red_add4(AV + j, -fx, -fy, oa, -gf);
                }
                if (FLOW) {  // src/kernels.cu:298-307 (overlapping pairs only)
                    fx_i += V0[j];
                    fy_i += V1[j];
                    if (DIM == 3) fz_i += V2[j];
                }
            }
        }
        if (hit) flush();
    }
    const double tAo = block_sum_f(sAo, smem);
    const double tAor = block_sum_f(sAor, smem);
    if (threadIdx.x == 0) {
        b.part[2 * vg + vb] = tAo;
        b.part[3 * vg + vb] = tAor;
    }
    if (last_block(&b.ctrl->done[DC_PAIRS], vg)) {
        double fAo = fold_partials(b.part + 2 * vg, vg, false, smem);
        double fAor = fold_partials(b.part + 3 * vg, vg, false, smem);
        if (GAS) {
            int2 *RC = recheck_list(AV, cap);
            const float2 d = recheck_containment<DIM>(RC, b.ds, c, b.k, PB, AV, AO);
            const double tdo = block_sum_f(d.x, smem);
            const double tdor = block_sum_f(d.y, smem);
            fAo += tdo;
            fAor += tdor;
            if (threadIdx.x == 0) RC[0].x = 0;  // every thread has read the count
        }
        if (threadIdx.x == 0) {
            Ctrl *cc = b.ctrl;
            cc->sumAo = 2.0 * fAo;
            cc->sumAor = fAor;
            // mean-field factors for every bubble, src/kernels.cu:399-404
            cc->mfa = (cc->sumAr - cc->sumAor) / (cc->sumA - cc->sumAo);
            cc->mfb = k.kappa * k.ain * (double)cc->n / cc->sumA;
            cc->done[DC_PAIRS] = 0;
        }
    }
}
CB_KERNEL_PAIR((template <int DIM, bool GAS, bool FLOW, int RUN>), k_pairs_mx, (<DIM, GAS, FLOW, RUN>), __launch_bounds__(kBlock, 4))


// ---------------------------------------------------------------- correct
// touchesWall, src/kernels.cu:553-566, on FP32 distances to both walls.
__device__ __forceinline__ bool touches_wall_f(float f0, float rad, float d1, float d2,
                                               float &velocity) {
    d1 = d1 * d1 < d2 * d2 ? d1 : d2;
    if (rad * rad >= d1 * d1) {
        d2 = d1 < 0.f ? -1.f : 1.f;
        d1 *= d2;
        velocity = d2 * f0 * (1.f - d1 / rad);
        return true;
    }
    return false;
}

// One pass over the block for the correct kernel's five reductions: maxima of
// error, radius and expansion (64-bit patterns of doubles >= 0), the volume
// sum (FP64, fixed order for a fixed block size) and the deletion and
// non-finite counts. Results valid in thread 0.
struct CorrRed {
    long long err, rad, exp;
    double vol;
    int del, bad;
    float cA[2], cAr[2];  // area sums of the two candidate predictions
};

__device__ __forceinline__ CorrRed block_reduce_corr(CorrRed v, CorrRed *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.err = max(v.err, __shfl_down_sync(0xffffffffu, v.err, o));
        v.rad = max(v.rad, __shfl_down_sync(0xffffffffu, v.rad, o));
        v.exp = max(v.exp, __shfl_down_sync(0xffffffffu, v.exp, o));
        v.vol += __shfl_down_sync(0xffffffffu, v.vol, o);
        v.del += __shfl_down_sync(0xffffffffu, v.del, o);
        v.bad += __shfl_down_sync(0xffffffffu, v.bad, o);
#pragma unroll
        for (int u = 0; u < 2; u++) {
            v.cA[u] += __shfl_down_sync(0xffffffffu, v.cA[u], o);
            v.cAr[u] += __shfl_down_sync(0xffffffffu, v.cAr[u], o);
        }
    }
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            const CorrRed u = smem[w];
            v.err = max(v.err, u.err);
            v.rad = max(v.rad, u.rad);
            v.exp = max(v.exp, u.exp);
            v.vol += u.vol;
            v.del += u.del;
            v.bad += u.bad;
#pragma unroll
            for (int q = 0; q < 2; q++) {
                v.cA[q] += u.cA[q];
                v.cAr[q] += u.cAr[q];
            }
        }
    return v;
}

// Grid-stride over the bubbles (one wave of blocks). The maxima and counts go
// to the control block with integer atomics (order-independent); only the
// volume sum keeps per-block partials for its in-order FP64 fold.
template <int DIM, bool GAS, bool FLOW, bool WALLS>
__device__ __forceinline__ void k_correct_mx_body(const Bufs &b, const int vb, const int vg) {
    __shared__ double smem[32];
    __shared__ CorrRed rsm[kBlock / 32];
    __shared__ unsigned long long tab[ND_ROLES];
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const int cap = k.cap;
    if (threadIdx.x < ND_ROLES)
        tab[threadIdx.x] = reinterpret_cast<unsigned long long>(b.ds[c->drole[threadIdx.x]]);
    __syncthreads();
#define CB_D(r) reinterpret_cast<double *>(tab_ptr(tab, r))
#define CB_F(r) reinterpret_cast<float *>(tab_ptr(tab, r))
    const float h = float_rn_from_double(0.5 * c->dt);
    const int path = c->inc_path;
    float4 *AV = acc_v(b);
    float *AO = acc_ov(b, cap);
    float4 *AF = acc_fl(b, cap);
    // mean-field factors, src/kernels.cu:399-408 (computed once per attempt)
    // mfa (the area-weighted mean of 1/r) as float-float: mfa - 1/r is a
    // difference of nearly equal terms, and one rounding of mfa would shift
    // every bubble's gas flux the same way; mfb only scales the term
    const ff mfa = ff_of(c->mfa);
    const float mfb = float_rn_from_double(c->mfb);
    const float kq = k.kq_f;
    const long long minr = __double_as_longlong(k.min_rad);
    const bool shear = c->use_flow && k.shear_on;
    // the two dt the next attempt can have after an accept (finish_attempt)
    const float hI = float_rn_from_double(0.5 * (c->dt * 1.269));
    float cA0 = 0.f, cA1 = 0.f, cAr0 = 0.f, cAr1 = 0.f;
    long long merr = 0, mrad = 0;
    float mexp = 0.f;
    double vol = 0.0;
    int ndel = 0, bad = 0;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += vg * blockDim.x) {
        const float4 a = AV[i];
        float vpx = a.x, vpy = a.y, vpz = DIM == 3 ? a.z : 0.f, vpr = a.w;
        const float ovl = GAS ? (DIM == 3 ? AO[i] : a.z) : 0.f;  // overlap area sum
        const float vx = CB_F(RV0)[i], vy = CB_F(RV1)[i], vz = DIM == 3 ? CB_F(RV2)[i] : 0.f;
        const float ox = CB_F(RVO0)[i], oy = CB_F(RVO1)[i], oz = DIM == 3 ? CB_F(RVO2)[i] : 0.f;
        const double x0 = CB_D(RX)[i], y0 = CB_D(RY)[i], z0 = DIM == 3 ? CB_D(RZ)[i] : 0.0;
        const double r0 = CB_D(RR)[i];
        // every other input up front, before the first store: the compiler
        // cannot move a load across a store it may alias, and loads issued
        // late leave their latency exposed
        const double s0 = CB_D(RS0)[i], s1 = CB_D(RS1)[i], s2 = DIM == 3 ? CB_D(RS2)[i] : 0.0;
        const double s3 = GAS ? CB_D(RS3)[i] : 0.0;
        const double err0 = CB_D(RERR)[i];
        const double path0 = path ? CB_D(RPATH)[i] : 0.0;
        float vr = 0.f, or_ = 0.f;
        float rp = float_rn_from_double(r0);
        if (GAS) {
            vr = CB_F(RV3)[i];
            or_ = CB_F(RVO3)[i];
            rp = fmaf(h, fmaf(3.f, vr, -or_), rp);  // as k_predict_mx
        }
        if (FLOW || WALLS || shear) {
            // predicted coordinates as x0 + e (e the FP32 AB2 increment)
            const float ex = h * fmaf(3.f, vx, -ox), ey = h * fmaf(3.f, vy, -oy),
                        ez = h * fmaf(3.f, vz, -oz);
            const float f0 = k.f0_f;
            if (FLOW) {  // addFlowVelocity, src/kernels.cu:497-544
                const float4 fl = AF[i];
                float multiplier = (float)irow(b, c, INN)[i];
                multiplier = multiplier > 0.f ? 1.f / multiplier : 0.f;
                const float riSq = rp * rp;
                const float lx = float_from_double(k.flow_lbb[0] - x0) - ex;
                const float tx = float_from_double(k.flow_tfr[0] - x0) - ex;
                const float ly = float_from_double(k.flow_lbb[1] - y0) - ey;
                const float ty = float_from_double(k.flow_tfr[1] - y0) - ey;
                int inside = (int)((tx > 0.f && lx < 0.f) || lx * lx <= riSq || tx * tx <= riSq);
                inside *= (int)((ty > 0.f && ly < 0.f) || ly * ly <= riSq || ty * ty <= riSq);
                if (DIM == 3) {
                    const float lz = float_from_double(k.flow_lbb[2] - z0) - ez;
                    const float tz = float_from_double(k.flow_tfr[2] - z0) - ez;
                    inside *= (int)((tz > 0.f && lz < 0.f) || lz * lz <= riSq || tz * tz <= riSq);
                    vpz += !inside * multiplier * fl.z + (float)k.flow_vel[2] * inside;
                }
                vpx += !inside * multiplier * fl.x + (float)k.flow_vel[0] * inside;
                vpy += !inside * multiplier * fl.y + (float)k.flow_vel[1] * inside;
            }
            if (shear) {  // linear shear along x over the last axis (cb_config.shear_speed)
                const float q = DIM == 3 ? float_from_double(z0 - k.lbb[2]) + ez
                                         : float_from_double(y0 - k.lbb[1]) + ey;
                vpx += k.shear_f * fmaf(q, k.shear_il_f, -1.f);
            }
            if (WALLS) {  // addWallVelocity, src/kernels.cu:546-593
                const float drag = (float)(1.0 - k.wall_drag);
                float xDrag = 1.f, yDrag = 1.f, velocity = 0.f;
                if (k.wall[0] && touches_wall_f(f0, rp, float_from_double(x0 - k.lbb[0]) + ex,
                                                float_from_double(x0 - k.tfr[0]) + ex, velocity)) {
                    vpx += velocity;
                    vpy *= drag;
                    vpz *= drag;
                    xDrag = drag;
                }
                velocity = 0.f;
                if (k.wall[1] && touches_wall_f(f0, rp, float_from_double(y0 - k.lbb[1]) + ey,
                                                float_from_double(y0 - k.tfr[1]) + ey, velocity)) {
                    vpx *= drag;
                    vpy += velocity * xDrag;
                    vpz *= drag;
                    yDrag = drag;
                }
                velocity = 0.f;
                if (k.wall[2] && touches_wall_f(f0, rp, float_from_double(z0 - k.lbb[2]) + ez,
                                                float_from_double(z0 - k.tfr[2]) + ez, velocity)) {
                    vpx *= drag;
                    vpy *= drag;
                    vpz += velocity * xDrag * yDrag;
                }
            }
        }
        // corrector x + 0.5 ts (v + vp): FP32 increment, FP64 sum; the error
        // |predicted - corrected| = 0.5 ts |2 v - vo - vp| (src/kernels.cu:487-495)
        const float ix = h * (vx + vpx), iy = h * (vy + vpy), iz = h * (vz + vpz);
        const double cx = x0 + double_from_float(ix);
        const double cy = y0 + double_from_float(iy);
        const double cz = DIM == 3 ? z0 + double_from_float(iz) : 0.0;
        float e = fmaxf(fabsf(fmaf(2.f, vx, -ox) - vpx), fabsf(fmaf(2.f, vy, -oy) - vpy));
        if (DIM == 3) e = fmaxf(e, fabsf(fmaf(2.f, vz, -oz) - vpz));
        // expansion since the last search, src/kernels.cu:366-387
        const float dx = float_from_double(cx - s0);
        const float dy = float_from_double(cy - s1);
        const float dz = DIM == 3 ? float_from_double(cz - s2) : 0.f;
        float dist = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
        int del = 0;
        double cr_keep = r0;
        if (GAS) {  // mean-field gas exchange, src/kernels.cu:390-431
            const float inv = 1.f / rp;
            const float area = DIM == 3 ? (4.f * (float)kPi) * (rp * rp) : (2.f * (float)kPi) * rp;
            float w = ((mfa.h - inv) + mfa.l) * (mfb * (area - ovl)) + vpr;
            w *= DIM == 3 ? kq * (inv * inv) : kq * inv;
            vpr = w;
            const float ir = h * (vr + w);
            const double cr = r0 + double_from_float(ir);
            cr_keep = cr;
            e = fmaxf(e, fabsf(fmaf(2.f, vr, -or_) - w));
            dist += float_from_double(cr - s3);
            if (__double_as_longlong(cr) > minr) {
                vol = fma(DIM == 3 ? cr * cr : cr, cr, vol);  // sum of r^D
            } else {
                del = 1;
                ndel++;
            }
            mrad = max(mrad, __double_as_longlong(cr));
            CB_D(RRN)[i] = cr;
            CB_F(RVP3)[i] = vpr;
            bad |= !finite_bits(cr);
        }
        b.delflag[i] = del;
        mexp = fmaxf(mexp, dist);
        const double ed = double_from_float(h * e);
        merr = max(merr, __double_as_longlong(ed));
        CB_D(RERR)[i] = __longlong_as_double(max(__double_as_longlong(err0), __double_as_longlong(ed)));
        if (path) {  // src/kernels.cu:437-451
            CB_D(RPATHN)[i] = path0 +
                              double_from_float(sqrtf(fmaf(iz, iz, fmaf(iy, iy, ix * ix))));
        }
        CB_D(RXN)[i] = cx;
        CB_D(RYN)[i] = cy;
        CB_F(RVP0)[i] = vpx;
        CB_F(RVP1)[i] = vpy;
        if (DIM == 3) {
            CB_D(RZN)[i] = cz;
            CB_F(RVP2)[i] = vpz;
        }
        bad |= !(finite_bits(cx) && finite_bits(cy) && finite_bits(cz));
        {  // the next attempt's prediction, as k_predict_mx would compute it
           // from the rotated state, for both dt: x' = cx, v' = vp, vo' = v
            const long long q0 = fix_from_double(cx), q1 = fix_from_double(cy);
            const long long q2 = DIM == 3 ? fix_from_double(cz) : 0LL;
            const float d0 = fmaf(3.f, vpx, -vx), d1 = fmaf(3.f, vpy, -vy);
            const float d2 = DIM == 3 ? fmaf(3.f, vpz, -vz) : 0.f;
            const long long qb = fix_from_double(GAS ? cr_keep : r0);
            const float d3 = GAS ? fmaf(3.f, vpr, -vr) : 0.f;
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const float hh = u ? hI : h;
                PredMx p;
                p.q[0] = q0 + fix_from_float(hh * d0);
                p.q[1] = q1 + fix_from_float(hh * d1);
                p.q[2] = DIM == 3 ? q2 + fix_from_float(hh * d2) : 0LL;
                p.qr = GAS ? qb + fix_from_float(hh * d3) : qb;
                st_pred(b.predc + (size_t)u * 4 * cap, i, p);
                const float rp1 = pred_r(p);
                if (GAS) {
                    const float apr = DIM == 3 ? (4.f * (float)kPi) * rp1 : 2.f * (float)kPi;
                    if (u) {
                        cA1 = fmaf(apr, rp1, cA1);
                        cAr1 += apr;
                    } else {
                        cA0 = fmaf(apr, rp1, cA0);
                        cAr0 += apr;
                    }
                }
            }
        }
        if (b.dbg_ov) b.dbg_ov[i] = double_from_float(ovl);
        AV[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (GAS && DIM == 3) AO[i] = 0.f;
        if (FLOW) AF[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
#undef CB_D
#undef CB_F
    CorrRed v{merr, mrad, __double_as_longlong(double_from_float(mexp)), vol, ndel, bad,
              {cA0, cA1}, {cAr0, cAr1}};
    v = block_reduce_corr(v, rsm);
    if (threadIdx.x == 0) {
        if (GAS) {
            atomicAdd(&c->cand_sumA[0], (double)v.cA[0]);
            atomicAdd(&c->cand_sumA[1], (double)v.cA[1]);
            atomicAdd(&c->cand_sumAr[0], (double)v.cAr[0]);
            atomicAdd(&c->cand_sumAr[1], (double)v.cAr[1]);
        }
        atomicMax(&c->amax_err, v.err);
        atomicMax(&c->amax_rad, v.rad);
        atomicMax(&c->amax_exp, v.exp);
        if (v.del) atomicAdd(&c->acnt_del, v.del);
        if (v.bad) atomicAdd(&c->acnt_bad, v.bad);
        b.part[vb] = v.vol;
    }
    if (!last_block(&c->done[DC_CORRECT], vg)) return;
    const double fVol = fold_partials(b.part, vg, false, smem);
    if (threadIdx.x != 0) return;
    volatile Ctrl *vc = c;
    const double fErr = __longlong_as_double(vc->amax_err);
    const double fRad = __longlong_as_double(vc->amax_rad);
    const double fExp = __longlong_as_double(vc->amax_exp);
    const double fDel = (double)vc->acnt_del, fBad = (double)vc->acnt_bad;
    c->amax_err = c->amax_rad = c->amax_exp = 0;
    c->acnt_del = c->acnt_bad = 0;
    finish_attempt<DIM>(c, k, fErr, fRad, fExp, fVol, fDel, fBad);
}
CB_KERNEL_PAIR((template <int DIM, bool GAS, bool FLOW, bool WALLS>), k_correct_mx, (<DIM, GAS, FLOW, WALLS>), __launch_bounds__(kBlock, 4))


// --------------------------------------------------------------- bootstrap
// phase 0: pred := fixed point of (x, r), vo := 0, path := 0
// phase 1: euler q += fix(acc dt) (src/kernels.cu:959-969), acc := 0
// phase 2: vo := acc, acc := 0
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_boot_mx(Bufs b, int phase) {
    const Ctrl *c = b.ctrl;
    const int n = c->n;
    const float ts = (float)c->dt;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    float *O0 = frow(b, c, RVO0), *O1 = frow(b, c, RVO1), *O2 = frow(b, c, RVO2),
          *O3 = frow(b, c, RVO3);
    double *PATH = drow(b, c, RPATH);
    float4 *AV = acc_v(b);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (phase == 0) {
            PredMx p;
            p.q[0] = fix_from_double(X[i]);
            p.q[1] = fix_from_double(Y[i]);
            p.q[2] = DIM == 3 ? fix_from_double(Z[i]) : 0LL;
            p.qr = fix_from_double(R[i]);
            st_pred(b.pred, i, p);
            O0[i] = O1[i] = O2[i] = O3[i] = 0.f;
            PATH[i] = 0.0;
        } else {
            const float4 a = AV[i];
            if (phase == 1) {
                PredMx p = ld_pred(b.pred, i);
                p.q[0] += fix_from_float(a.x * ts);
                p.q[1] += fix_from_float(a.y * ts);
                if (DIM == 3) p.q[2] += fix_from_float(a.z * ts);
                st_pred(b.pred, i, p);
            } else {
                O0[i] = a.x;
                O1[i] = a.y;
                if (DIM == 3) O2[i] = a.z;
            }
            AV[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

template <int DIM, bool GAS>
void launch_correct_mx_t(const Launch &l, const Bufs &b, bool flow, bool walls) {
    if (flow && walls)
        CB_LAUNCH(l, k_correct_mx, (<DIM, GAS, true, true>),
                  wave_grid(k_correct_mx<DIM, GAS, true, true>, l, l.step_bps), b);
    else if (flow)
        CB_LAUNCH(l, k_correct_mx, (<DIM, GAS, true, false>),
                  wave_grid(k_correct_mx<DIM, GAS, true, false>, l, l.step_bps), b);
    else if (walls)
        CB_LAUNCH(l, k_correct_mx, (<DIM, GAS, false, true>),
                  wave_grid(k_correct_mx<DIM, GAS, false, true>, l, l.step_bps), b);
    else
        CB_LAUNCH(l, k_correct_mx, (<DIM, GAS, false, false>),
                  wave_grid(k_correct_mx<DIM, GAS, false, false>, l, l.step_bps), b);
}

}  // namespace

void launch_predict_mx(const Launch &l, const Bufs &b, int dim) {
    if (dim == 3)
        CB_LAUNCH(l, k_predict_mx, (<3>), wave_grid(k_predict_mx<3>, l, l.step_bps), b);
    else
        CB_LAUNCH(l, k_predict_mx, (<2>), wave_grid(k_predict_mx<2>, l, l.step_bps), b);
}

void launch_pairs_mx(const Launch &l, const Bufs &b, int dim, int mode) {
    const bool gas = mode & 1, flow = mode & 2;
    const int run = l.pair_run;
#define CB_PAIRS(D, G, F, R) \
    CB_LAUNCH(l, k_pairs_mx, (<D, G, F, R>), wave_grid(k_pairs_mx<D, G, F, R>, l, l.pair_bps), b)
    if (dim == 3) {
        if (gas && flow) CB_PAIRS(3, true, true, 4);
        else if (gas && run == 2) CB_PAIRS(3, true, false, 2);
        else if (gas && run == 8) CB_PAIRS(3, true, false, 8);
        else if (gas) CB_PAIRS(3, true, false, 4);
        else if (flow) CB_PAIRS(3, false, true, 4);
        else CB_PAIRS(3, false, false, 4);
    } else {
        if (gas && flow) CB_PAIRS(2, true, true, 4);
        else if (gas && run == 2) CB_PAIRS(2, true, false, 2);
        else if (gas && run == 8) CB_PAIRS(2, true, false, 8);
        else if (gas) CB_PAIRS(2, true, false, 4);
        else if (flow) CB_PAIRS(2, false, true, 4);
        else CB_PAIRS(2, false, false, 4);
    }
#undef CB_PAIRS
}

void launch_correct_mx(const Launch &l, const Bufs &b, int dim, int mode, bool walls) {
    const bool gas = mode & 1, flow = mode & 2;
    if (dim == 3) {
        if (gas)
            launch_correct_mx_t<3, true>(l, b, flow, walls);
        else
            launch_correct_mx_t<3, false>(l, b, flow, walls);
    } else {
        if (gas)
            launch_correct_mx_t<2, true>(l, b, flow, walls);
        else
            launch_correct_mx_t<2, false>(l, b, flow, walls);
    }
}

void launch_boot_mx(const Launch &l, const Bufs &b, int dim, int phase) {
    if (dim == 3)
        k_boot_mx<3><<<l.grid, kBlock, 0, l.stream>>>(b, phase);
    else
        k_boot_mx<2><<<l.grid, kBlock, 0, l.stream>>>(b, phase);
    *l.launches += 1;
}

}  // namespace cbg
