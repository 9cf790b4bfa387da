// One attempt of the step in the mixed form (cb_config.precision =
// CB_PRECISION_MIXED). Same algorithm and control as step.cu; what changes is
// the arithmetic of the pair interaction and the storage of the rates:
//   * FP64: absolute positions and radii (x, y, z, r and their corrected
//     values), path, the predictor-corrector error norm and its reduction,
//     the volume sum of the survivors and the volume fix, the global area
//     sums, the energy;
//   * FP32: velocities and radius rates (the dxdt / dxdto / dxdtp rows hold
//     floats), the pair geometry, overlap velocities, overlap areas and the
//     gas flux, the mean-field arithmetic per bubble;
//   * pair geometry works on exact differences of 64-bit fixed-point
//     coordinates: q = x * 2^64 / L (mod 2^64) on a periodic axis, so the
//     integer difference q_i - q_j wraps to the minimum image by itself
//     (wrappedDifference, src/kernels.cu:1094-1114, becomes one integer
//     subtraction) and is exact at any separation, also for nearly
//     coincident bubbles; on a wall axis q = (x - lbb + L/4) 2^61 / (1.5 L)
//     without wrapping. Only the conversion of the exact difference to FP32
//     rounds (relative 2^-24).
// The packed predicted state is 32 bytes per bubble (q_x, q_y, q_z, r_p,
// 1/r_p) and the pair kernel adds its results with 16-byte vector FP32
// reductions.
#include "common.cuh"

namespace cbg {
namespace {

__device__ __forceinline__ float *frow(const Bufs &b, const Ctrl *c, int role) {
    return reinterpret_cast<float *>(b.ds[c->drole[role]]);
}

// Accumulator layout of the mixed form inside `acc` (64 bytes per bubble):
// float4 velocity sums (vx, vy, vz, vr) at [0, 16 cap), float overlap at
// [16 cap, 20 cap), float4 flow sums at [32 cap, 48 cap) bytes.
__device__ __forceinline__ float4 *acc_v(const Bufs &b) { return reinterpret_cast<float4 *>(b.acc); }
__device__ __forceinline__ float *acc_ov(const Bufs &b, int cap) {
    return reinterpret_cast<float *>(b.acc) + 4 * (size_t)cap;
}
__device__ __forceinline__ float4 *acc_fl(const Bufs &b, int cap) {
    return reinterpret_cast<float4 *>(reinterpret_cast<float *>(b.acc) + 8 * (size_t)cap);
}

__device__ __forceinline__ void red_add4(float4 *p, float a, float b, float c, float d) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b),
                 "f"(c), "f"(d)
                 : "memory");
}

// Predicted state of one bubble in the mixed form (32 bytes).
struct __align__(16) PredMx {
    unsigned long long q[3];
    float r, inv;
};

__device__ __forceinline__ unsigned long long fixq(const DevConst &k, int a, double x) {
    return (unsigned long long)__double2ll_rn(fma(x, k.fx_scale[a], k.fx_off[a]))
           << k.fx_shift[a];
}

// Adds a length increment (FP32) to a fixed-point coordinate.
__device__ __forceinline__ unsigned long long fixadd(unsigned long long q, float inc, float unit) {
    return q + (unsigned long long)__float2ll_rn(inc * unit);
}

__device__ __forceinline__ float qdiff(unsigned long long qi, unsigned long long qj, float inv) {
    return (float)(long long)(qi - qj) * inv;
}

__device__ __forceinline__ PredMx ld_pred(const Bufs &b, int i) {
    const int4 *p = reinterpret_cast<const int4 *>(b.pred) + 2 * (size_t)i;
    const int4 u = p[0], v = p[1];
    PredMx r;
    r.q[0] = (unsigned long long)(unsigned)u.x | ((unsigned long long)(unsigned)u.y << 32);
    r.q[1] = (unsigned long long)(unsigned)u.z | ((unsigned long long)(unsigned)u.w << 32);
    r.q[2] = (unsigned long long)(unsigned)v.x | ((unsigned long long)(unsigned)v.y << 32);
    r.r = __int_as_float(v.z);
    r.inv = __int_as_float(v.w);
    return r;
}

__device__ __forceinline__ void st_pred(const Bufs &b, int i, const PredMx &r) {
    int4 *p = reinterpret_cast<int4 *>(b.pred) + 2 * (size_t)i;
    p[0] = make_int4((int)(unsigned)r.q[0], (int)(unsigned)(r.q[0] >> 32), (int)(unsigned)r.q[1],
                     (int)(unsigned)(r.q[1] >> 32));
    p[1] = make_int4((int)(unsigned)r.q[2], (int)(unsigned)(r.q[2] >> 32), __float_as_int(r.r),
                     __float_as_int(r.inv));
}

// ---------------------------------------------------------------- predict
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_predict_mx(Bufs b) {
    __shared__ double smem[32];
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const float h = (float)(0.5 * c->dt);
    const int gas = c->use_gas;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    const float *V0 = frow(b, c, RV0), *V1 = frow(b, c, RV1), *V2 = frow(b, c, RV2),
                *V3 = frow(b, c, RV3);
    const float *O0 = frow(b, c, RVO0), *O1 = frow(b, c, RVO1), *O2 = frow(b, c, RVO2),
                *O3 = frow(b, c, RVO3);
    const float u0 = (float)k.fx_unit[0], u1 = (float)k.fx_unit[1], u2 = (float)k.fx_unit[2];
    float sA = 0.f, sAr = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // AB2 increment h (3 v - vo) in FP32, added to the exact fixed point of x
        PredMx p;
        p.q[0] = fixadd(fixq(k, 0, X[i]), h * fmaf(3.f, V0[i], -O0[i]), u0);
        p.q[1] = fixadd(fixq(k, 1, Y[i]), h * fmaf(3.f, V1[i], -O1[i]), u1);
        p.q[2] = DIM == 3 ? fixadd(fixq(k, 2, Z[i]), h * fmaf(3.f, V2[i], -O2[i]), u2) : 0ull;
        float rp = (float)R[i];
        if (gas) rp = fmaf(h, fmaf(3.f, V3[i], -O3[i]), rp);
        p.r = rp;
        p.inv = 1.f / rp;
        st_pred(b, i, p);
        if (gas) {
            const float apr = DIM == 3 ? (4.f * (float)kPi) * rp : 2.f * (float)kPi;
            sA = fmaf(apr, rp, sA);
            sAr += apr;
        }
    }
    const double tA = block_reduce((double)sA, OpSum(), smem);
    const double tAr = block_reduce((double)sAr, OpSum(), smem);
    if (threadIdx.x == 0) {
        b.part[0 * gridDim.x + blockIdx.x] = tA;
        b.part[1 * gridDim.x + blockIdx.x] = tAr;
    }
    if (last_block(&b.ctrl->done[DC_PREDICT])) {
        const double fA = fold_partials(b.part + 0 * gridDim.x, gridDim.x, false, smem);
        const double fAr = fold_partials(b.part + 1 * gridDim.x, gridDim.x, false, smem);
        if (threadIdx.x == 0) {
            b.ctrl->sumA = fA;
            b.ctrl->sumAr = fAr;
            b.ctrl->done[DC_PREDICT] = 0;
        }
    }
}

// ------------------------------------------------------------------ pairs
template <int DIM, bool GAS, bool FLOW>
__global__ void __launch_bounds__(kBlock) k_pairs_mx(Bufs b) {
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
    const float f0 = (float)k.f0;
    const float ix = k.fx_inv[0], iy = k.fx_inv[1], iz = k.fx_inv[2];
    float sAo = 0.f, sAor = 0.f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int i = PI[p], j = PJ[p];
        if (FLOW)  // src/kernels.cu:191-207 (added for every pair)
            red_add4(AF + j, V0[i], V1[i], DIM == 3 ? V2[i] : 0.f, 0.f);
        const PredMx a = ld_pred(b, i), q = ld_pred(b, j);
        const float dx = qdiff(a.q[0], q.q[0], ix);
        const float dy = qdiff(a.q[1], q.q[1], iy);
        const float dz = DIM == 3 ? qdiff(a.q[2], q.q[2], iz) : 0.f;
        const float r1 = a.r, r2 = q.r;
        float m = dx * dx;
        m = fmaf(dy, dy, m);
        if (DIM == 3) m = fmaf(dz, dz, m);
        const float radii = r1 + r2;
        if (radii * radii >= m) {
            const float rs = rsqrtf(m);
            const float s = f0 * (rs - __fdividef(1.f, radii));
            const float fx = dx * s, fy = dy * s, fz = dz * s;
            float g = 0.f;
            if (GAS) {
                const float r1sq = r1 * r1, r2sq = r2 * r2;
                float oa;
                if (m < r1sq || m < r2sq) {
                    oa = DIM == 3 ? fminf(r1sq, r2sq) * (float)kPi : 2.f * fminf(r1, r2);
                } else {
                    const float t = 0.5f * (r2sq - r1sq + m);
                    oa = fabsf(r2sq - (t * t) * (rs * rs));
                    oa = DIM == 3 ? oa * (float)kPi : 2.f * sqrtf(oa);
                }
                const float inv1 = a.inv, inv2 = q.inv;
                g = oa * (inv2 - inv1);
                atomicAdd(AO + i, oa);
                atomicAdd(AO + j, oa);
                sAo += oa;
                sAor = fmaf(oa, inv1 + inv2, sAor);
            }
            red_add4(AV + i, fx, fy, fz, g);
            red_add4(AV + j, -fx, -fy, -fz, -g);
            if (FLOW)  // src/kernels.cu:298-307 (overlapping pairs only)
                red_add4(AF + i, V0[j], V1[j], DIM == 3 ? V2[j] : 0.f, 0.f);
        }
    }
    const double tAo = block_reduce((double)sAo, OpSum(), smem);
    const double tAor = block_reduce((double)sAor, OpSum(), smem);
    if (threadIdx.x == 0) {
        b.part[2 * gridDim.x + blockIdx.x] = tAo;
        b.part[3 * gridDim.x + blockIdx.x] = tAor;
    }
    if (last_block(&b.ctrl->done[DC_PAIRS])) {
        const double fAo = fold_partials(b.part + 2 * gridDim.x, gridDim.x, false, smem);
        const double fAor = fold_partials(b.part + 3 * gridDim.x, gridDim.x, false, smem);
        if (threadIdx.x == 0) {
            b.ctrl->sumAo = 2.0 * fAo;
            b.ctrl->sumAor = fAor;
            b.ctrl->done[DC_PAIRS] = 0;
        }
    }
}

// ---------------------------------------------------------------- correct
// touchesWall, src/kernels.cu:553-566 (FP32; x is the predicted coordinate)
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

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_correct_mx(Bufs b) {
    __shared__ double smem[32];
    __shared__ int ismem[32];
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const int cap = k.cap;
    const double h64 = 0.5 * c->dt;
    const float h = (float)h64;
    const int gas = c->use_gas, flow = c->use_flow, path = c->inc_path;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    double *XN = drow(b, c, RXN), *YN = drow(b, c, RYN), *ZN = drow(b, c, RZN),
           *RN = drow(b, c, RRN);
    const float *V0 = frow(b, c, RV0), *V1 = frow(b, c, RV1), *V2 = frow(b, c, RV2),
                *V3 = frow(b, c, RV3);
    const float *O0 = frow(b, c, RVO0), *O1 = frow(b, c, RVO1), *O2 = frow(b, c, RVO2),
                *O3 = frow(b, c, RVO3);
    float *P0 = frow(b, c, RVP0), *P1 = frow(b, c, RVP1), *P2 = frow(b, c, RVP2),
          *P3 = frow(b, c, RVP3);
    const double *S0 = drow(b, c, RS0), *S1 = drow(b, c, RS1), *S2 = drow(b, c, RS2),
                 *S3 = drow(b, c, RS3);
    const double *PATH = drow(b, c, RPATH);
    double *PATHN = drow(b, c, RPATHN), *ERR = drow(b, c, RERR);
    const int *NN = irow(b, c, INN);
    float4 *AV = acc_v(b);
    float *AO = acc_ov(b, cap);
    float4 *AF = acc_fl(b, cap);
    // mean-field factors, src/kernels.cu:399-408, from the FP64 sums
    const double sA = c->sumA, sAr = c->sumAr, sAo = c->sumAo, sAor = c->sumAor;
    const float mfa = (float)((sAr - sAor) / (sA - sAo));
    const float mfb = (float)(k.kappa * k.ain * (double)n / sA);
    const float kq = (float)(DIM == 3 ? k.K / (4.0 * kPi) : k.K / (2.0 * kPi));
    const float f0 = (float)k.f0;
    const float drag = (float)(1.0 - k.wall_drag);
    long long merr = 0, mrad = 0;
    float mexp = 0.f;
    double vol = 0.0;
    int ndel = 0, bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 a = AV[i];
        float vpx = a.x, vpy = a.y, vpz = a.z, vpr = a.w;
        const float vx = V0[i], vy = V1[i], vz = DIM == 3 ? V2[i] : 0.f;
        const float ox = O0[i], oy = O1[i], oz = DIM == 3 ? O2[i] : 0.f;
        const double x0 = X[i], y0 = Y[i], z0 = DIM == 3 ? Z[i] : 0.0, r0 = R[i];
        float vr = 0.f, or_ = 0.f;
        float rp = (float)r0;
        if (gas) {
            vr = V3[i];
            or_ = O3[i];
            rp = fmaf(h, fmaf(3.f, vr, -or_), rp);  // as k_predict_mx
        }
        if (flow || k.any_wall) {
            // predicted coordinates relative to the box corner (FP32)
            const float ex = h * fmaf(3.f, vx, -ox), ey = h * fmaf(3.f, vy, -oy),
                        ez = h * fmaf(3.f, vz, -oz);
            if (flow) {  // addFlowVelocity, src/kernels.cu:497-544
                const float4 fl = AF[i];
                float multiplier = (float)NN[i];
                multiplier = multiplier > 0.f ? 1.f / multiplier : 0.f;
                const float riSq = rp * rp;
                const float lx = (float)(k.flow_lbb[0] - x0) - ex, tx = (float)(k.flow_tfr[0] - x0) - ex;
                const float ly = (float)(k.flow_lbb[1] - y0) - ey, ty = (float)(k.flow_tfr[1] - y0) - ey;
                int inside = (int)((tx > 0.f && lx < 0.f) || lx * lx <= riSq || tx * tx <= riSq);
                inside *= (int)((ty > 0.f && ly < 0.f) || ly * ly <= riSq || ty * ty <= riSq);
                if (DIM == 3) {
                    const float lz = (float)(k.flow_lbb[2] - z0) - ez,
                                tz = (float)(k.flow_tfr[2] - z0) - ez;
                    inside *= (int)((tz > 0.f && lz < 0.f) || lz * lz <= riSq || tz * tz <= riSq);
                    vpz += !inside * multiplier * fl.z + (float)k.flow_vel[2] * inside;
                }
                vpx += !inside * multiplier * fl.x + (float)k.flow_vel[0] * inside;
                vpy += !inside * multiplier * fl.y + (float)k.flow_vel[1] * inside;
            }
            if (k.any_wall) {  // addWallVelocity, src/kernels.cu:546-593
                float xDrag = 1.f, yDrag = 1.f, velocity = 0.f;
                if (k.wall[0] && touches_wall_f(f0, rp, (float)(x0 - k.lbb[0]) + ex,
                                                (float)(x0 - k.tfr[0]) + ex, velocity)) {
                    vpx += velocity;
                    vpy *= drag;
                    vpz *= drag;
                    xDrag = drag;
                }
                velocity = 0.f;
                if (k.wall[1] && touches_wall_f(f0, rp, (float)(y0 - k.lbb[1]) + ey,
                                                (float)(y0 - k.tfr[1]) + ey, velocity)) {
                    vpx *= drag;
                    vpy += velocity * xDrag;
                    vpz *= drag;
                    yDrag = drag;
                }
                velocity = 0.f;
                if (k.wall[2] && touches_wall_f(f0, rp, (float)(z0 - k.lbb[2]) + ez,
                                                (float)(z0 - k.tfr[2]) + ez, velocity)) {
                    vpx *= drag;
                    vpy *= drag;
                    vpz += velocity * xDrag * yDrag;
                }
            }
        }
        // corrector x + 0.5 ts (v + vp) in FP64 on FP32 rates; the error
        // |predicted - corrected| = 0.5 ts |2 v - vo - vp| (src/kernels.cu:487-495)
        const float sx = vx + vpx, sy = vy + vpy, sz = vz + vpz;
        const double cx = fma(h64, (double)sx, x0);
        const double cy = fma(h64, (double)sy, y0);
        const double cz = DIM == 3 ? fma(h64, (double)sz, z0) : 0.0;
        float e = fmaxf(fabsf(fmaf(2.f, vx, -ox) - vpx), fabsf(fmaf(2.f, vy, -oy) - vpy));
        if (DIM == 3) e = fmaxf(e, fabsf(fmaf(2.f, vz, -oz) - vpz));
        float tx = (float)(cx - S0[i]), ty = (float)(cy - S1[i]);
        float dist = fmaf(tx, tx, ty * ty);
        if (DIM == 3) {
            const float tz = (float)(cz - S2[i]);
            dist = fmaf(tz, tz, dist);
        }
        dist = sqrtf(dist);
        int del = 0;
        if (gas) {  // mean-field gas exchange, src/kernels.cu:390-431
            const float inv = 1.f / rp;
            const float area = DIM == 3 ? (4.f * (float)kPi) * (rp * rp) : (2.f * (float)kPi) * rp;
            float w = (mfa - inv) * (mfb * (area - AO[i])) + vpr;
            w *= DIM == 3 ? kq * (inv * inv) : kq * inv;
            vpr = w;
            const double cr = fma(h64, (double)(vr + w), r0);
            e = fmaxf(e, fabsf(fmaf(2.f, vr, -or_) - w));
            dist += (float)(cr - S3[i]);
            if (cr > k.min_rad) {
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
        mexp = fmaxf(mexp, dist);
        const double ed = (double)(h * e);
        merr = max_bits(merr, ed);
        ERR[i] = fmax(ed, ERR[i]);
        if (path) {  // src/kernels.cu:437-451
            float d2 = fmaf(sx, sx, sy * sy);
            if (DIM == 3) d2 = fmaf(sz, sz, d2);
            PATHN[i] = PATH[i] + (double)(h * sqrtf(d2));
        }
        XN[i] = cx;
        YN[i] = cy;
        P0[i] = vpx;
        P1[i] = vpy;
        if (DIM == 3) {
            ZN[i] = cz;
            P2[i] = vpz;
        }
        bad |= !(finite_bits(cx) && finite_bits(cy) && finite_bits(cz));
        if (b.dbg_ov) b.dbg_ov[i] = gas ? (double)AO[i] : 0.0;
        AV[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gas) AO[i] = 0.f;
        if (flow) AF[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const double tErr = block_reduce(__longlong_as_double(merr), OpMax(), smem);
    const double tRad = block_reduce(__longlong_as_double(mrad), OpMax(), smem);
    const double tExp = block_reduce((double)mexp, OpMax(), smem);
    const double tVol = block_reduce(vol, OpSum(), smem);
    const int tDel = block_reduce_int(ndel, ismem);
    const int tBad = block_reduce_int(bad, ismem);
    const int G = gridDim.x;
    if (threadIdx.x == 0) {
        b.part[0 * G + blockIdx.x] = tErr;
        b.part[1 * G + blockIdx.x] = tRad;
        b.part[2 * G + blockIdx.x] = tExp;
        b.part[3 * G + blockIdx.x] = tVol;
        b.part[4 * G + blockIdx.x] = (double)tDel;
        b.part[5 * G + blockIdx.x] = (double)tBad;
    }
    if (!last_block(&c->done[DC_CORRECT])) return;
    const double fErr = fold_partials(b.part + 0 * G, G, true, smem);
    const double fRad = fold_partials(b.part + 1 * G, G, true, smem);
    const double fExp = fold_partials(b.part + 2 * G, G, true, smem);
    const double fVol = fold_partials(b.part + 3 * G, G, false, smem);
    const double fDel = fold_partials(b.part + 4 * G, G, false, smem);
    const double fBad = fold_partials(b.part + 5 * G, G, false, smem);
    if (threadIdx.x != 0) return;
    finish_attempt<DIM>(c, k, fErr, fRad, fExp, fVol, fDel, fBad);
}

// --------------------------------------------------------------- bootstrap
// phase 0: pred := fixed point of (x, r), vo := 0, path := 0
// phase 1: euler q += round(acc dt scale), acc := 0
// phase 2: vo := acc, acc := 0
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_boot_mx(Bufs b, int phase) {
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const double ts = c->dt;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    float *O0 = frow(b, c, RVO0), *O1 = frow(b, c, RVO1), *O2 = frow(b, c, RVO2),
          *O3 = frow(b, c, RVO3);
    double *PATH = drow(b, c, RPATH);
    float4 *AV = acc_v(b);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (phase == 0) {
            PredMx p;
            p.q[0] = fixq(k, 0, X[i]);
            p.q[1] = fixq(k, 1, Y[i]);
            p.q[2] = DIM == 3 ? fixq(k, 2, Z[i]) : 0ull;
            p.r = (float)R[i];
            p.inv = 1.f / p.r;
            st_pred(b, i, p);
            O0[i] = O1[i] = O2[i] = O3[i] = 0.f;
            PATH[i] = 0.0;
        } else {
            const float4 a = AV[i];
            if (phase == 1) {  // euler, src/kernels.cu:959-969
                PredMx p = ld_pred(b, i);
                p.q[0] += (unsigned long long)__double2ll_rn((double)a.x * ts * k.fx_unit[0]);
                p.q[1] += (unsigned long long)__double2ll_rn((double)a.y * ts * k.fx_unit[1]);
                if (DIM == 3)
                    p.q[2] += (unsigned long long)__double2ll_rn((double)a.z * ts * k.fx_unit[2]);
                st_pred(b, i, p);
            } else {
                O0[i] = a.x;
                O1[i] = a.y;
                if (DIM == 3) O2[i] = a.z;
            }
            AV[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

}  // namespace

void launch_predict_mx(const Launch &l, const Bufs &b, int dim) {
    if (dim == 3)
        k_predict_mx<3><<<l.grid, kBlock, 0, l.stream>>>(b);
    else
        k_predict_mx<2><<<l.grid, kBlock, 0, l.stream>>>(b);
    *l.launches += 1;
}

void launch_pairs_mx(const Launch &l, const Bufs &b, int dim, int mode) {
    const bool gas = mode & 1, flow = mode & 2;
#define CB_PAIRS(D, G, F) k_pairs_mx<D, G, F><<<l.grid, kBlock, 0, l.stream>>>(b)
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
    *l.launches += 1;
}

void launch_correct_mx(const Launch &l, const Bufs &b, int dim) {
    if (dim == 3)
        k_correct_mx<3><<<l.grid, kBlock, 0, l.stream>>>(b);
    else
        k_correct_mx<2><<<l.grid, kBlock, 0, l.stream>>>(b);
    *l.launches += 1;
}

void launch_boot_mx(const Launch &l, const Bufs &b, int dim, int phase) {
    if (dim == 3)
        k_boot_mx<3><<<l.grid, kBlock, 0, l.stream>>>(b, phase);
    else
        k_boot_mx<2><<<l.grid, kBlock, 0, l.stream>>>(b, phase);
    *l.launches += 1;
}

}  // namespace cbg
