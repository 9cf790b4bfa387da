// Neighbour search, searchNeighbors() (src/simulator.cu:60-178):
//   k_wrap        wrap positions into the box (wrapOverPeriodicBoundaries,
//                 src/kernels.cu:992-1011), exact maximum radius -> cell grid
//   k_cell_count  cell of every bubble (cellByPosition, src/kernels.cu:598-607)
//   scan          cell offsets
//   k_cell_fill   counting-sort scatter (indexByCell, src/kernels.cu:609-615)
//   k_cell_order  one warp per cell orders its bubbles by previous position,
//                 so the cell order is deterministic
//   k_permute     gather every persistent row into cell order in one pass and
//                 set saved := positions (reorganizeByIndex,
//                 src/kernels.cu:721-770); the pointer rotation of
//                 src/simulator.cu:99-146 becomes a role swap in the control
//                 block
//   k_pair_cells, k_pair_tiles, k_pair_rows
//                 per bubble, the pairs (i, j > i) within r_i + r_j + skin
//                 (neighborSearch / comparePair, src/kernels.cu:617-701),
//                 by the pass that suits the grid (dense cells, sparse 3D,
//                 sparse 2D): one enumeration that counts each row and keeps
//                 its partners, a scan, k_pair_compact writing the rows, so
//                 the list is ordered by (i, j) without atomics (a second
//                 enumeration only when a row outgrew its stash); candidates
//                 are screened in FP32 with a conservative margin and
//                 accepted by the exact FP64 test of the reference, so the
//                 pair set is bit-exact
//   k_degree      neighbour counts (countNumNeighbors, src/kernels.cu:713-719)
#include "common.cuh"

namespace cbg {
namespace {

// Cell grid: cellDim_a = max(1, floor(interval_a / (s (2 maxR + skin)))) on
// the used axes, s = k.cell_scale >= 1 (1 by default); while the product
// exceeds the cell capacity the largest dimension (lowest axis on ties)
// shrinks by one. Larger cells change which candidates are tested and the
// bubble order, never the pair set.
__device__ void cell_grid(const DevConst &k, double max_r, int cd[3]) {
    const double cutoff = __dmul_rn(__dadd_rn(__dmul_rn(2.0, max_r), k.skin), k.cell_scale);
    for (int a = 0; a < 3; a++) {
        cd[a] = 1;
        if (a < k.dim) {
            double q = floor(__ddiv_rn(k.iv[a], cutoff));
            if (q > 1048576.0) q = 1048576.0;
            cd[a] = q >= 1.0 ? (int)q : 1;
        }
    }
    for (;;) {
        const long long tot = (long long)cd[0] * cd[1] * cd[2];
        if (tot <= (long long)k.ccap) break;
        int m = 0;
        for (int a = 1; a < 3; a++)
            if (cd[a] > cd[m]) m = a;
        cd[m] -= 1;
    }
}

// getCellIdxFromPos, src/kernels.cu:1191-1203, clamped to the grid.
__device__ __forceinline__ int cell_coord(double x, double lbb, double iv, int cd) {
    const double q = floor(__ddiv_rn(__dmul_rn((double)cd, __dsub_rn(x, lbb)), iv));
    return q < 0.0 ? 0 : (q >= (double)cd ? cd - 1 : (int)q);
}
__device__ __noinline__ int cell_coord_slow(double x, double lbb, double iv, int cd) {
    return cell_coord(x, lbb, iv, cd);
}

// The same cell coordinate with the FP64 division (about ten FP64-pipe
// instructions) only where it matters: q = cd (x - lbb) / iv in FP32 from the
// truncated x is within `band` of the FP64 value (|x - x32| <= 2^-23 |x|,
// three FP32 roundings of 2^-24 each), so unless its fractional part lies
// within `band` of a cell face, or outside the grid, its floor is the FP64
// expression's floor.
struct CellAxis {
    float lbb, scale, band;
    double lbb_d, iv;
    int cd;
};

__device__ __forceinline__ CellAxis cell_axis(const DevConst &k, int a, int cd) {
    CellAxis c;
    c.lbb = k.lbb_f[a];
    c.scale = (float)cd / k.iv32[a];
    const float ma = fmaxf(fabsf(k.lbb_f[a]), fabsf(k.lbb_f[a] + k.iv32[a]));
    c.band = 9.5367431640625e-07f * (float)cd * (1.f + ma / k.iv32[a]);  // 2^-20 cd (1 + |x|/L)
    c.lbb_d = k.lbb[a];
    c.iv = k.iv[a];
    c.cd = cd;
    return c;
}

__device__ __forceinline__ int cell_coord_fast(double x, const CellAxis &c) {
    const float q = (ff_f32(x) - c.lbb) * c.scale;
    const float fl = floorf(q);
    const float fr = q - fl;
    if (fr > c.band && fr < 1.f - c.band && fl >= 0.f && fl < (float)c.cd) return (int)fl;
    return cell_coord_slow(x, c.lbb_d, c.iv, c.cd);
}

__device__ __forceinline__ bool is_nan_bits(double x) {
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
}
// A double's bit pattern as a signed integer that orders like the value
// (-0 and +0 both 0; NaN patterns beyond the infinities).
__device__ __forceinline__ long long order_key(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (long long)(0x8000000000000000ULL - (unsigned long long)b);
}
// The wrap itself (rare): x + (hi - lo) mult and the wrap count, a call so
// that its FP64 arithmetic is not predicated into every bubble.
static __device__ __noinline__ void wrap_one(double *xp, int *wp, double x, double lo, double hi,
                                             int mult) {
    *xp = x + (hi - lo) * (double)mult;
    *wp -= mult;
}

template <int DIM>
__device__ __forceinline__ void k_wrap_body(const Bufs &b, const int vb, const int vg) {
    __shared__ double smem[32];
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    double *XR[3] = {drow(b, c, RX), drow(b, c, RY), drow(b, c, RZ)};
    int *WR[3] = {irow(b, c, IWX), irow(b, c, IWY), irow(b, c, IWZ)};
    const double *R = drow(b, c, RR);
    // box constants in registers: the stores below may alias them for the
    // compiler, which would reload them per bubble. The compares of
    // wrapOverPeriodicBoundaries (src/kernels.cu:992-1011) run on the integer
    // pipe, on order keys of the bit patterns (-0 and +0 alike; a NaN
    // coordinate is left alone and a NaN radius ignored, as the FP64
    // compares and fmax do).
    bool per[3];
    long long lo3[3], hi3[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        per[a] = a < DIM && !k.wall[a];
        lo3[a] = order_key(k.lbb[a]);
        hi3[a] = order_key(k.tfr[a]);
    }
    long long mr = 0;  // largest radius as the bits of a double >= 0
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += vg * blockDim.x) {
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            if (!per[a]) continue;
            const double x = XR[a][i];
            const long long kx = order_key(x);
            const int mult = is_nan_bits(x) ? 0 : (kx < lo3[a] ? 1 : (kx > hi3[a] ? -1 : 0));
            if (mult) wrap_one(XR[a] + i, WR[a] + i, x, k.lbb[a], k.tfr[a], mult);
        }
        const double r = R[i];
        if (!is_nan_bits(r)) mr = max(mr, __double_as_longlong(r));  // fmax over radii >= 0
    }
    const double t = __longlong_as_double(block_max_bits(mr, reinterpret_cast<long long *>(smem)));
    if (threadIdx.x == 0) b.part[7 * vg + vb] = t;
    if (last_block(&c->done[DC_WRAP], vg)) {
        const double f = fold_partials(b.part + 7 * vg, vg, true, smem);
        if (threadIdx.x == 0) {
            int cd[3];
            cell_grid(k, f, cd);
            c->cell_dims[0] = cd[0];
            c->cell_dims[1] = cd[1];
            c->cell_dims[2] = cd[2];
            c->ncell = cd[0] * cd[1] * cd[2];
            c->searches += 1;
            c->stash_over = 0;
            c->sparse_cells = (long long)c->n < 24LL * c->ncell;
            c->search_maxr = __double2float_ru(f);
            c->pred_ready = 0;  // the bubbles move to new slots
            c->pred_slot = 0;
            c->done[DC_WRAP] = 0;
        }
    }
}
CB_KERNEL_PAIR((template <int DIM>), k_wrap, (<DIM>), __launch_bounds__(kBlock))


template <int DIM>
__device__ __forceinline__ void k_cell_count_body(const Bufs &b, const int vb, const int vg) {
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const int cd0 = c->cell_dims[0], cd1 = c->cell_dims[1], cd2 = c->cell_dims[2];
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ);
    const CellAxis ax = cell_axis(k, 0, cd0), ay = cell_axis(k, 1, cd1);
    const CellAxis az = cell_axis(k, 2, DIM == 3 ? cd2 : 1);
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += vg * blockDim.x) {
        const int kx = cell_coord_fast(X[i], ax);
        const int ky = cell_coord_fast(Y[i], ay);
        const int kz = DIM == 3 ? cell_coord_fast(Z[i], az) : 0;
        const int ci = (kz * cd1 + ky) * cd0 + kx;
        b.cellOf[i] = ci;
        atomicAdd(b.cellCount + ci, 1);
    }
}
CB_KERNEL_PAIR((template <int DIM>), k_cell_count, (<DIM>), __launch_bounds__(kBlock))


__device__ __forceinline__ void k_cell_fill_body(const Bufs &b, const int vb, const int vg) {
    const int n = b.ctrl->n;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += vg * blockDim.x) {
        const int ci = b.cellOf[i];
        b.perm[b.cellStart[ci] + atomicAdd(b.cellFill + ci, 1)] = i;
    }
}
CB_KERNEL_PAIR((), k_cell_fill, (), __launch_bounds__(kBlock))


// One warp per cell: rank each member by its previous position (values are
// distinct), giving the stable counting-sort order. The cell's count and
// fill counters are spent by now and are cleared here for the next search
// (they start zeroed, and a search only touches its own ncell cells).
__device__ __forceinline__ void k_cell_order_body(const Bufs &b, const int vb, const int vg) {
    const int ncell = b.ctrl->ncell;
    const int lane = threadIdx.x & 31;
    const int warps = vg * (blockDim.x >> 5);
    for (int q = vb * (blockDim.x >> 5) + (threadIdx.x >> 5); q < ncell; q += warps) {
        if (lane == 0) {
            b.cellCount[q] = 0;
            b.cellFill[q] = 0;
        }
        const int s = b.cellStart[q], e = b.cellStart[q + 1], m = e - s;
        for (int t0 = 0; t0 < m; t0 += 32) {
            const int t = t0 + lane;
            const int v = t < m ? b.perm[s + t] : 0x7fffffff;
            int rank = 0;
            for (int u = 0; u < m; u++) rank += b.perm[s + u] < v;
            if (t < m) {
                b.permSorted[s + rank] = v;
                b.cellSorted[s + rank] = q;
            }
        }
    }
}
CB_KERNEL_PAIR((), k_cell_order, (), __launch_bounds__(kBlock))


// Sparse 3D grids whose periodic axes have at least four cells (and fewer
// than 2^26 cells, in a box whose corners lie within 2^21 of the origin) are
// counted by k_pair_tiles: a neighbour cell is then reached through at most
// one periodic image, and never twice.
template <int DIM>
__device__ __forceinline__ bool tile_grid(const DevConst &k, const int cd[3], int ncell) {
    // cell index and stencil offset in one sort key; fixed-point coordinates
    bool ok = DIM == 3 && ncell < (1 << 26) && k.fix_range;
#pragma unroll
    for (int a = 0; a < DIM; a++) ok &= k.wall[a] || cd[a] >= 4;
    return ok;
}

// Gather of every persistent row into cell order: positions (+ saved),
// velocities, previous velocities, path, error, wrap counts and indices into
// their spare slots, then swap the roles. One pass over the bubbles: every
// row of a bubble is gathered in the same iteration (the permutation read
// once, all loads of the bubble in flight together).
template <int DIM>
__device__ __forceinline__ void k_permute_body(const Bufs &b, const int vb, const int vg) {
    Ctrl *c = b.ctrl;
    const int n = c->n;
    const int *src = b.permSorted;
    const bool f32 = b.k->mixed;  // rate rows hold floats in the mixed form
    const int roles[4][2] = {{RX, RXN}, {RY, RYN}, {RZ, RZN}, {RR, RRN}};
    const double *pf[4];
    double *pt[4], *sv[4];
    const double *vf[4], *of[4];
    double *vt[4], *ot[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        pf[a] = drow(b, c, roles[a][0]);
        pt[a] = drow(b, c, roles[a][1]);
        sv[a] = drow(b, c, RS0 + a);
        vf[a] = drow(b, c, RV0 + a);
        vt[a] = drow(b, c, RVP0 + a);
        of[a] = drow(b, c, RVO0 + a);
        ot[a] = drow(b, c, RVQ0 + a);
    }
    const double *f1 = drow(b, c, RPATH), *f2 = drow(b, c, RERR);
    double *t1 = drow(b, c, RPATHN), *t2 = drow(b, c, RERR2);
    const int *fi[4] = {irow(b, c, IWX), irow(b, c, IWY), irow(b, c, IWZ), irow(b, c, IIDX)};
    int *ti[4] = {irow(b, c, IWX2), irow(b, c, IWY2), irow(b, c, IWZ2), irow(b, c, IIDX2)};
    // for the 3D tile pass: x, y, z relative to the lower corner of the
    // bubble's cell, from exact fixed-point differences (x 2^40; the cell
    // edge L / cd in that unit, off by at most one unit); the FP32 copy of
    // the positions is for the other passes
    const DevConst &k = *b.k;
    const int cd[3] = {c->cell_dims[0], c->cell_dims[1], c->cell_dims[2]};
    const bool rel = DIM == 3 && c->sparse_cells && tile_grid<DIM>(k, cd, c->ncell);
    long long cwq[3], lbq[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        cwq[a] = k.lq[a] / cd[a];
        lbq[a] = k.lbq[a];
    }
    for (int q = vb * blockDim.x + threadIdx.x; q < n; q += vg * blockDim.x) {
        const int s = src[q];
        double p[4];
#pragma unroll
        for (int a = 0; a < 4; a++) p[a] = (DIM == 2 && a == 2) ? 0.0 : pf[a][s];
        double v[4], vo[4];
        float vf32[4], vo32[4];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            if (DIM == 2 && a == 2) continue;
            if (f32) {
                vf32[a] = reinterpret_cast<const float *>(vf[a])[s];
                vo32[a] = reinterpret_cast<const float *>(of[a])[s];
            } else {
                v[a] = vf[a][s];
                vo[a] = of[a][s];
            }
        }
        const double g1 = f1[s], g2 = f2[s];
        const int w0 = fi[0][s], w1 = fi[1][s], w2 = fi[2][s], w3 = fi[3][s];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            if (DIM == 2 && a == 2) continue;
            pt[a][q] = p[a];
            sv[a][q] = p[a];
            if (f32) {
                reinterpret_cast<float *>(vt[a])[q] = vf32[a];
                reinterpret_cast<float *>(ot[a])[q] = vo32[a];
            } else {
                vt[a][q] = v[a];
                ot[a][q] = vo[a];
            }
        }
        t1[q] = g1;
        t2[q] = g2;
        ti[0][q] = w0;
        ti[1][q] = w1;
        ti[2][q] = w2;
        ti[3][q] = w3;
        if (!rel) {
            b.pos32[q] = make_float4((float)p[0], (float)p[1], DIM == 3 ? (float)p[2] : 0.0f,
                                     (float)p[3]);
        } else {
            const int cell = b.cellSorted[q];
            const int kc[3] = {cell % cd[0], (cell / cd[0]) % cd[1], cell / (cd[0] * cd[1])};
            float o[3];
#pragma unroll
            for (int a = 0; a < 3; a++)
                o[a] = len_from_fix(fix_from_double(p[a]) - (lbq[a] + (long long)kc[a] * cwq[a]));
            b.pos32r[q] = make_float4(o[0], o[1], o[2], (float)p[3]);
        }
    }
    if (last_block(&c->done[DC_PERMUTE], vg) && threadIdx.x == 0) {
        int *r = c->drole;
        for (int a = 0; a < 4; a++) {
            if (DIM == 2 && a == 2) continue;
            swap_role(r, roles[a][0], roles[a][1]);
            swap_role(r, RV0 + a, RVP0 + a);
            swap_role(r, RVO0 + a, RVQ0 + a);
        }
        swap_role(r, RPATH, RPATHN);
        swap_role(r, RERR, RERR2);
        int *ir = c->irole;
        swap_role(ir, IWX, IWX2);
        swap_role(ir, IWY, IWY2);
        swap_role(ir, IWZ, IWZ2);
        swap_role(ir, IIDX, IIDX2);
        c->done[DC_PERMUTE] = 0;
    }
}
CB_KERNEL_PAIR((template <int DIM>), k_permute, (<DIM>), __launch_bounds__(kBlock, 3))




// Neighbour cell `k` (0..26, offsets dx,dy,dz in -1..1) of `cell`, or
// INT_MAX when it is below `cell` in linear order, outside a wall, on an
// unused axis, or a duplicate of another offset on a periodic axis with
// fewer than three cells (one cell: offset 0 only; two: 0 and +1).
template <int DIM>
__device__ __forceinline__ int neighbor_cell(const DevConst &k, const int cd[3], int cell, int o) {
    const int off[3] = {o % 3 - 1, (o / 3) % 3 - 1, o / 9 - 1};
    const int kk[3] = {cell % cd[0], (cell / cd[0]) % cd[1], cell / (cd[0] * cd[1])};
    int q[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int d = cd[a];
        if (a >= DIM) {
            if (off[a] != 0) return 0x7fffffff;
            q[a] = 0;
        } else if (!k.wall[a]) {
            if (d == 1 && off[a] != 0) return 0x7fffffff;
            if (d == 2 && off[a] == -1) return 0x7fffffff;
            q[a] = (kk[a] + off[a] + d) % d;
        } else {
            q[a] = kk[a] + off[a];
            if (q[a] < 0 || q[a] >= d) return 0x7fffffff;
        }
    }
    const int v = (q[2] * cd[1] + q[1]) * cd[0] + q[0];
    return v >= cell ? v : 0x7fffffff;
}

// Warp-wide ascending bitonic sort of one int per lane.
__device__ __forceinline__ int warp_sort(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int size = 2; size <= 32; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            const int o = __shfl_xor_sync(0xffffffffu, v, stride);
            const bool up = ((lane & size) == 0);
            const bool lower = ((lane & stride) == 0);
            v = (lower == up) ? min(v, o) : max(v, o);
        }
    }
    return v;
}

constexpr int kWarpsPerBlock = kBlock / 32;

// Is j a pair partner of i (comparePair, src/kernels.cu:619-623)? Decided in
// FP32 unless the distance lies within the guard band `pre_margin` of the
// cutoff; there the reference's exact FP64 test decides. That test is a
// call: inlined, its FP64 loads and arithmetic are predicated into every
// candidate and take FP64 issue slots.
template <int DIM>
static __device__ __noinline__ bool pair_take_exact(const DevConst &k, int i, int j,
                                                    const double *X, const double *Y,
                                                    const double *Z, const double *R) {
    const double maxd = __dadd_rn(__dadd_rn(R[i], R[j]), k.skin);
    const double sq = exact_sqdist<DIM>(k, X[i], Y[i], DIM == 3 ? Z[i] : 0.0, X[j], Y[j],
                                        DIM == 3 ? Z[j] : 0.0);
    return sq < __dmul_rn(maxd, maxd);
}
// The FP32 part of the test: 0 not a partner, 1 a partner, 2 within the
// guard band (the exact test decides).
template <int DIM>
__device__ __forceinline__ int pair_class(const DevConst &k, const float4 &pi, const float4 &pj) {
    const bool per[3] = {!k.wall[0], !k.wall[1], !k.wall[2]};
    float dx = fabsf(pi.x - pj.x), dy = fabsf(pi.y - pj.y);
    float dz = DIM == 3 ? fabsf(pi.z - pj.z) : 0.f;
    if (per[0] && dx > k.half_iv32[0]) dx = k.iv32[0] - dx;
    if (per[1] && dy > k.half_iv32[1]) dy = k.iv32[1] - dy;
    if (DIM == 3 && per[2] && dz > k.half_iv32[2]) dz = k.iv32[2] - dz;
    float d2 = fmaf(dx, dx, dy * dy);
    if (DIM == 3) d2 = fmaf(dz, dz, d2);
    const float cut = pi.w + pj.w + k.skin_f;
    const float band = k.pre_margin;
    const float hi = cut + band, lo = fmaxf(cut - band, 0.f);
    if (d2 >= hi * hi) return 0;
    if (d2 < lo * lo) return 1;
    return 2;
}
template <int DIM>
__device__ __forceinline__ bool pair_take(const DevConst &k, const float4 &pi, const float4 &pj,
                                          int i, int j, const double *X, const double *Y,
                                          const double *Z, const double *R) {
    const int cls = pair_class<DIM>(k, pi, pj);
    return cls == 1 || (cls == 2 && pair_take_exact<DIM>(k, i, j, X, Y, Z, R));
}

// Pair rows of one cell per warp: lanes are the cell's bubbles (32 at a
// time); each neighbour cell with a linear index >= the home cell is staged
// 32 bubbles at a time in shared memory (FP32 x, y, z, r) and every lane
// tests its bubble against the staged ones. A candidate is decided in FP32
// unless its distance lies within the guard band `pre_margin` of the cutoff;
// only there the exact FP64 test of comparePair (src/kernels.cu:619-623)
// runs, so the pair set equals the FP64 one bit for bit.
// WRITE = false counts rows and keeps the first kStash partners of each row
// in `stash` (k_pair_compact then writes the list without a second
// enumeration); WRITE = true, needed only when some row had more partners,
// enumerates again and writes the rows at rowStart.
template <int DIM, bool WRITE>
__device__ __forceinline__ void k_pair_cells_body(const Bufs &b, const int vb, const int vg) {
    __shared__ float4 stage[kWarpsPerBlock][32];
    Ctrl *c = b.ctrl;
    if (WRITE && !c->stash_over) return;  // k_pair_compact wrote the list
    if (!WRITE && c->sparse_cells) return;  // k_pair_rows counts sparse grids
    constexpr int M = kStash(DIM);
    bool over = false;
    const DevConst &k = *b.k;
    const int ncell = c->ncell;
    const int cd[3] = {c->cell_dims[0], c->cell_dims[1], c->cell_dims[2]};
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    int *PI = b.ps[c->prole[PI0]];
    int *PJ = b.ps[c->prole[PJ0]];
    int *NN = irow(b, c, INN);
    const int pcap = k.pcap;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int warps = vg * kWarpsPerBlock;
    // The FP32 positions: the gather's copy, or, where the tile pass counted
    // (its gather wrote only cell-relative coordinates), the same values
    // converted here from the FP64 rows
    const bool conv = WRITE && DIM == 3 && c->sparse_cells && tile_grid<DIM>(k, cd, ncell);
    auto pos_f = [&](int q) {
        return conv ? make_float4((float)X[q], (float)Y[q], (float)Z[q], (float)R[q]) : b.pos32[q];
    };
    for (int cell = vb * kWarpsPerBlock + w; cell < ncell; cell += warps) {
        const int s0 = b.cellStart[cell], e0 = b.cellStart[cell + 1];
        if (s0 == e0) continue;
        const int nbr = warp_sort(lane < 27 ? neighbor_cell<DIM>(k, cd, cell, lane) : 0x7fffffff);
        const int m = __popc(__ballot_sync(0xffffffffu, nbr != 0x7fffffff));
        for (int h0 = s0; h0 < e0; h0 += 32) {
            const int i = h0 + lane;
            const bool active = i < e0;
            float4 pi = make_float4(0.f, 0.f, 0.f, 0.f);
            int base = 0, cnt = 0;
            if (active) {
                pi = pos_f(i);
                if (WRITE) base = b.rowStart[i];
            }
            for (int qn = 0; qn < m; qn++) {
                const int q = __shfl_sync(0xffffffffu, nbr, qn);
                const int cs = b.cellStart[q], ce = b.cellStart[q + 1];
                for (int c0 = cs; c0 < ce; c0 += 32) {
                    const int nc = min(32, ce - c0);
                    __syncwarp();
                    if (lane < nc) stage[w][lane] = pos_f(c0 + lane);
                    __syncwarp();
                    for (int t = 0; t < nc; t++) {
                        const int j = c0 + t;
                        const float4 pj = stage[w][t];
                        if (!active || j <= i) continue;
                        const bool take = pair_take<DIM>(k, pi, pj, i, j, X, Y, Z, R);
                        if (take) {
                            if (WRITE && base + cnt < pcap) {
                                PI[base + cnt] = i;
                                PJ[base + cnt] = j;
                            }
                            if (!WRITE && cnt < M) b.stash[(size_t)i * M + cnt] = j;
                            cnt++;
                        }
                    }
                }
            }
            if (active) {
                NN[i] = cnt;
                if (!WRITE) {
                    b.rowCount[i] = cnt;
                    over |= cnt > M;
                }
            }
        }
    }
    if (!WRITE) {
        if (__syncthreads_or(over) && threadIdx.x == 0) atomicOr(&c->stash_over, 1);
        return;
    }
    if (last_block(&c->done[DC_MISC], vg) && threadIdx.x == 0) {
        const int found = c->np_found;
        if (found > pcap) {
            c->status = CB_ERR_CAPACITY;
            c->np = 0;
        } else {
            c->np = found;
        }
        c->need_search = 0;
        c->done[DC_MISC] = 0;
    }
}
CB_KERNEL_PAIR((template <int DIM, bool WRITE>), k_pair_cells, (<DIM, WRITE>), __launch_bounds__(kBlock))

// Counting pass for sparse 2D cell grids (fewer than 24 bubbles per cell on
// average; 2D cells hold ~3) and the sparse 3D grids k_pair_tiles does not
// take (an axis with fewer than four cells): one thread per bubble walks its
// neighbour cells >= its own cell in ascending order and the bubbles j > i
// in them, so the rows and their order are those of the warp-per-cell pass,
// with all lanes busy (a warp per cell of ~3 bubbles would leave 90 % of its
// lanes idle).
template <int DIM>
__device__ __forceinline__ void k_pair_rows_body(const Bufs &b, const int vb, const int vg) {
    Ctrl *c = b.ctrl;
    if (!c->sparse_cells) return;
    const DevConst &k = *b.k;
    constexpr int M = kStash(DIM);
    constexpr int NO = DIM == 3 ? 27 : 9;  // stencil offsets
    const int n = c->n;
    const int cd[3] = {c->cell_dims[0], c->cell_dims[1], c->cell_dims[2]};
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    int *NN = irow(b, c, INN);
    // cell widths and the reach beyond a bubble's radius (FP32, padded so the
    // cell pruning below never drops a partner)
    float cw[3];
#pragma unroll
    for (int a = 0; a < 3; a++) cw[a] = k.iv32[a] / (float)cd[a];
    const float reach0 = c->search_maxr + k.skin_f + k.pre_margin + 1e-3f;
    if (DIM == 3 && tile_grid<DIM>(k, cd, c->ncell)) return;  // k_pair_tiles counts it
    bool over = false;
    for (int i = vb * blockDim.x + threadIdx.x; i < n; i += vg * blockDim.x) {
        const int cell = b.cellSorted[i];
        const int kk[3] = {cell % cd[0], (cell / cd[0]) % cd[1], cell / (cd[0] * cd[1])};
        const float4 pi = b.pos32[i];
        const float pr[3] = {pi.x - k.lbb_f[0], pi.y - k.lbb_f[1],
                             DIM == 3 ? pi.z - k.lbb_f[2] : 0.f};
        const float reach = pi.w + reach0;
        // distance from the bubble to the lower / upper face of its cell
        float lo[3], hi[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            lo[a] = fmaxf(pr[a] - (float)kk[a] * cw[a], 0.f);
            hi[a] = fmaxf((float)(kk[a] + 1) * cw[a] - pr[a], 0.f);
        }
        int nb[NO];
        int nq = 0;
#pragma unroll
        for (int t = 0; t < NO; t++) {
            const int o = DIM == 3 ? t : 9 + t;  // 2D: the z-offset-0 plane
            const int off[3] = {o % 3 - 1, (o / 3) % 3 - 1, o / 9 - 1};
            // neighbour cell index (getNeighborCellIndex, src/kernels.cu:1157-1189)
            int q[3];
            bool ok = true;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const int d = cd[a];
                if (a >= DIM) {
                    ok &= off[a] == 0;
                    q[a] = 0;
                } else if (!k.wall[a]) {
                    ok &= !(d == 1 && off[a] != 0) && !(d == 2 && off[a] == -1);
                    q[a] = kk[a] + off[a];
                    q[a] = q[a] < 0 ? q[a] + d : (q[a] >= d ? q[a] - d : q[a]);
                } else {
                    q[a] = kk[a] + off[a];
                    ok &= q[a] >= 0 && q[a] < d;
                }
            }
            const int v = (q[2] * cd[1] + q[1]) * cd[0] + q[0];
            if (!ok || v < cell) continue;
            // skip a neighbour cell no partner of this bubble can be in
            float d2 = 0.f;
#pragma unroll
            for (int a = 0; a < DIM; a++) {
                // with two cells on a periodic axis the other cell touches
                // both faces (only its +1 offset is enumerated)
                const float up = (!k.wall[a] && cd[a] == 2) ? fminf(lo[a], hi[a]) : hi[a];
                const float f = off[a] > 0 ? up : (off[a] < 0 ? lo[a] : 0.f);
                d2 = fmaf(f, f, d2);
            }
            if (d2 > reach * reach) continue;
            int p = nq++;  // insertion into the ascending list
            while (p > 0 && nb[p - 1] > v) {
                nb[p] = nb[p - 1];
                p--;
            }
            nb[p] = v;
        }
        // the candidates of all listed cells as one flat sequence: a lane
        // moves to its next cell inside the loop, so the warp runs for its
        // longest lane's candidate count, not for the sum over cells of the
        // longest lane's count in each
        int cnt = 0;
        int t = -1, j = 0, je = 0;
        while (true) {
            while (j >= je && ++t < nq) {
                const int qc = nb[t];
                j = max(b.cellStart[qc], i + 1);
                je = b.cellStart[qc + 1];
            }
            if (t >= nq) break;
            const float4 pj = b.pos32[j];
            const int cls = pair_class<DIM>(k, pi, pj);
            if (cls == 1 || (cls == 2 && pair_take_exact<DIM>(k, i, j, X, Y, Z, R))) {
                if (cnt < M) b.stash[(size_t)i * M + cnt] = j;
                cnt++;
            }
            j++;
        }
        NN[i] = cnt;
        b.rowCount[i] = cnt;
        over |= cnt > M;
    }
    if (__syncthreads_or(over) && threadIdx.x == 0) atomicOr(&c->stash_over, 1);
}
CB_KERNEL_PAIR((template <int DIM>), k_pair_rows, (<DIM>), __launch_bounds__(kBlock))

// Counting pass for sparse 3D grids with at least four cells on every
// periodic axis, one warp per home cell. The candidates of the cell (its own
// bubbles and those of its neighbour cells >= it, cells ascending, bubbles
// ascending inside a cell) are laid over the lanes 32 at a time, each lane
// loading one candidate (a cell's bubbles are contiguous, so the loads are
// coalesced). Coordinates are FP32 relative to each bubble's cell corner
// (written by the gather into cell order from exact fixed-point
// differences), and a candidate moves into the home cell's frame by its
// cell's stencil offset times the cell edge, across a periodic face too
// (four or more cells per axis make the offset unique): the FP32 rounding
// is relative to a cell edge, not to the box, and the guard band where the
// reference's FP64 test decides is ~40x narrower. A candidate out of reach
// of the box around the home bubbles is dropped, the kept ones are packed
// (in candidate order) into chunks of 32. The home cell's bubbles are then
// broadcast from shared memory one at a time and every lane tests its
// candidate against the bubble; the warp's hit mask of each (bubble, chunk)
// goes to shared memory, and after a window of up to kTileChunks tested
// chunks each lane walks the masks of its home bubble and appends the
// partners to the bubble's row in candidate order, the order of the thread
// pass, so stash, counts and pair list are the same. All lanes work on every
// test, against a thread per bubble that walks its own cells with, in 3D,
// less than half of its warp's lanes busy.
constexpr int kTileChunks = 16;  // window: 16 tested chunks of 32

// The tests of one chunk against home bubbles 0..nh-1 (home cell bubbles
// among the candidates: CMP, the j > i order test): the warp's hit mask of
// each home bubble goes to masks[a]. Tests in the guard band (d2 - cut^2
// within +-tb of zero, tb = 2 cutmax band >= 2 cut band; 2 cut band + band^2
// would be the exact band, the narrower one is within its margin) are only
// flagged here; the return value says whether any lane had one, and
// tile_exact then decides them.
template <bool CMP>
__device__ __forceinline__ bool tile_tests(const float4 *home, int nh, int h0, int j,
                                           const float4 &pj, float wj, float tb,
                                           unsigned *masks) {
    float bmin = 3.4e38f;  // min over the home bubbles of |e| (<= tb: in the band)
#pragma unroll 4
    for (int a = 0; a < nh; a++) {
        const float4 pi = home[a];
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float cut = pi.w + wj;
        const float e = fmaf(-cut, cut, d2);
        bool take = e < -tb;
        if (CMP) take &= j > h0 + a;
        masks[a] = __ballot_sync(0xffffffffu, take);
        bmin = fminf(bmin, fabsf(e));
    }
    return __any_sync(0xffffffffu, bmin <= tb);
}
// The FP64 test of the reference for the guard-band pairs of a chunk: the
// chunk's tests are repeated and each band pair's bit set by the exact
// decision (comparePair, src/kernels.cu:619-623). Rare: with the
// cell-relative band about 300 tests per search at N = 10^6.
template <int DIM>
__device__ __forceinline__ void tile_exact(const DevConst &k, const float4 *home, int nh, int h0,
                                           int j, float4 pj, float wj, float tb, unsigned *masks,
                                           const double *X, const double *Y, const double *Z,
                                           const double *R) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    for (int a = 0; a < nh; a++) {
        const float4 pi = home[a];
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float cut = pi.w + wj;
        const float e = fmaf(-cut, cut, d2);
        const bool amb = j > h0 + a && !(e < -tb) && e < tb;
        if (amb && pair_take_exact<DIM>(k, h0 + a, j, X, Y, Z, R))
            atomicOr(masks + a, 1u << lane);
    }
    __syncwarp();
}

// Each lane (home bubble lane < nh) appends its partners among the tc
// tested chunks of a window to its row, in candidate order.
template <int M>
__device__ __forceinline__ void tile_rows(const unsigned (*hitmask)[32], const int *candj, int tc,
                                          int nh, int *row, int &mycnt) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    if (lane < nh) {
        for (int ch = 0; ch < tc; ch++) {
            unsigned hm = hitmask[ch][lane];
            while (hm) {
                const int bit = __ffs(hm) - 1;
                hm &= hm - 1;
                if (mycnt < M) row[mycnt] = candj[(ch << 5) + bit];
                mycnt++;
            }
        }
    }
    __syncwarp();
}

template <int DIM>
__device__ __forceinline__ void k_pair_tiles_body(const Bufs &b, const int vb, const int vg) {
    __shared__ float4 home[kWarpsPerBlock][32];
    __shared__ unsigned hitmask[kWarpsPerBlock][kTileChunks][32];  // [chunk][home bubble]
    __shared__ int candj[kWarpsPerBlock][kTileChunks * 32];
    __shared__ float4 stp[kWarpsPerBlock][64];  // kept candidates (home frame)
    __shared__ int stj[kWarpsPerBlock][64];
    Ctrl *c = b.ctrl;
    if (!c->sparse_cells) return;
    const DevConst &k = *b.k;
    const int cd[3] = {c->cell_dims[0], c->cell_dims[1], c->cell_dims[2]};
    const int ncell = c->ncell;
    if (!tile_grid<DIM>(k, cd, ncell)) return;  // k_pair_rows counts it
    constexpr int M = kStash(DIM);
    constexpr unsigned kAll = 0xffffffffu;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    int *NN = irow(b, c, INN);
    int *stash = b.stash, *rowCount = b.rowCount;
    const int *cellStart = b.cellStart;
    const float4 *pos = b.pos32r;  // x, y, z relative to the bubble's cell
    // constants in registers (a store through `stash` could alias them)
    const float skin = k.skin_f;
    // cell edges (the unit of the fixed-point cell corners, rounded to FP32)
    float cw[3], cwmax = 0.f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        cw[a] = (float)(k.lq[a] / cd[a]) * kFixInv;
        cwmax = fmaxf(cwmax, cw[a]);
    }
    // Guard band of the cell-relative FP32 test. A coordinate relative to
    // its cell's corner is off by < 2^-23 cw (its conversion), the cell
    // offset of a candidate by 2^-24 cw, the moved candidate (|x| < 2 cw)
    // and the difference by 2^-24 2 cw each: < 8 2^-24 cw per axis, so the
    // distance by < 8.3e-7 cw; the squared-distance and cutoff roundings add
    // < 1e-6. 4e-6 cw + 2e-6 is about 4x that. In d2 - cut^2 units: 2 cut
    // band for the largest cut.
    const float band = 4e-6f * cwmax + 2e-6f;
    const float tb = 2.f * band * (2.f * (c->search_maxr + 1e-3f) + skin);
    const bool per[3] = {!k.wall[0], !k.wall[1], !k.wall[2]};
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int plane = cd[0] * cd[1];
    const int warps = vg * kWarpsPerBlock;
    bool over = false;
    for (int cell = vb * kWarpsPerBlock + w; cell < ncell; cell += warps) {
        const int s0 = cellStart[cell], e0 = cellStart[cell + 1];
        if (s0 == e0) continue;
        // lane t < m: the t-th neighbour cell >= cell in ascending order
        // (getNeighborCellIndex, src/kernels.cu:1157-1189) with its stencil
        // offset o (0..26: (o % 3 - 1, o / 3 % 3 - 1, o / 9 - 1) cells) in
        // the low 5 bits of the key: a candidate moves into the home cell's
        // frame by the offset times the cell edge, across a periodic face
        // too. Away from the box faces these are the offsets 13..26 in order.
        const int hk[3] = {cell % cd[0], (cell / cd[0]) % cd[1], cell / plane};
        const bool inner = hk[0] >= 1 && hk[0] <= cd[0] - 2 && hk[1] >= 1 &&
                           hk[1] <= cd[1] - 2 && hk[2] >= 1 && hk[2] <= cd[2] - 2;
        int key = 0x7fffffff, m = 14;
        if (inner) {
            if (lane < 14) {
                const int o = 13 + lane;
                key = ((cell + (o / 9 - 1) * plane + ((o / 3) % 3 - 1) * cd[0] + (o % 3 - 1)) << 5) | o;
            }
        } else {
            if (lane < 27) {
                const int off[3] = {lane % 3 - 1, (lane / 3) % 3 - 1, lane / 9 - 1};
                int q[3];
                bool ok = true;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    q[a] = hk[a] + off[a];
                    if (per[a])
                        q[a] = q[a] < 0 ? q[a] + cd[a] : (q[a] >= cd[a] ? q[a] - cd[a] : q[a]);
                    else
                        ok &= q[a] >= 0 && q[a] < cd[a];
                }
                const int v = (q[2] * cd[1] + q[1]) * cd[0] + q[0];
                if (ok && v >= cell) key = (v << 5) | lane;
            }
            key = warp_sort(key);
            m = __popc(__ballot_sync(kAll, key != 0x7fffffff));
        }
        int cs = 0, cn = 0;
        if (lane < m) {
            const int v = key >> 5;
            cs = cellStart[v];
            cn = cellStart[v + 1] - cs;
        }
        int pre = cn;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kAll, pre, o);
            if (lane >= o) pre += t;
        }
        const int T = __shfl_sync(kAll, pre, 31);  // lanes >= m add nothing
        // lane t: candidate bb of its cell is bubble cbase + bb; the cell's
        // move into the home frame
        const int cbase = cs - (pre - cn);
        float mvx = 0.f, mvy = 0.f, mvz = 0.f;
        {
            const int o = key & 31;
            mvx = (float)(o % 3 - 1) * cw[0];
            mvy = (float)((o / 3) % 3 - 1) * cw[1];
            mvz = (float)(o / 9 - 1) * cw[2];
        }
        for (int h0 = s0; h0 < e0; h0 += 32) {
            const int nh = min(32, e0 - h0);
            __syncwarp();
            float4 ph = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < nh) {
                ph = pos[h0 + lane];
                home[w][lane] = ph;
            }
            // the box around the home bubbles (each centre +- its radius): a
            // candidate farther from the box than its own radius + skin + pad
            // is farther than r_i + r_j + skin + pad from every home centre,
            // pairs with none of them, and is dropped before the tests (pad
            // = 4 band covers the FP32 error of the tests, so the exact test
            // would refuse every dropped pair)
            const bool hv = lane < nh;
            float blo[3] = {hv ? ph.x - ph.w : 3.4e38f, hv ? ph.y - ph.w : 3.4e38f,
                            hv ? ph.z - ph.w : 3.4e38f};
            float bhi[3] = {hv ? ph.x + ph.w : -3.4e38f, hv ? ph.y + ph.w : -3.4e38f,
                            hv ? ph.z + ph.w : -3.4e38f};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    blo[a] = fminf(blo[a], __shfl_xor_sync(kAll, blo[a], o));
                    bhi[a] = fmaxf(bhi[a], __shfl_xor_sync(kAll, bhi[a], o));
                }
            }
            const float reach0 = skin + 4.f * band;
            __syncwarp();
            int mycnt = 0;  // partners of home bubble h0 + lane so far
            int *row = stash + (size_t)(h0 + min(lane, nh - 1)) * M;
            // kept candidates wait in a ring of 64 (in candidate order) until
            // 32 of them fill a chunk; tc chunks are tested in the window
            int ns = 0, head = 0, tc = 0;
            for (int r0 = 0; r0 < T; r0 += 32) {
                const int bb = r0 + lane;
                // the cell of candidate bb: the number of cells whose
                // inclusive prefix is <= bb (pre ascends over the lanes)
                int t = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(kAll, pre, t + step - 1) <= bb) t += step;
                const int bt = __shfl_sync(kAll, cbase, t);
                const float mx = __shfl_sync(kAll, mvx, t), my = __shfl_sync(kAll, mvy, t),
                            mz = __shfl_sync(kAll, mvz, t);
                int j = -1;
                float4 pj = make_float4(0.f, 0.f, 0.f, 0.f);
                bool keep = false;
                if (bb < T) {
                    j = bt + bb;
                    pj = pos[j];
                    pj.x += mx;
                    pj.y += my;
                    pj.z += mz;
                    const float ex = fmaxf(fmaxf(blo[0] - pj.x, pj.x - bhi[0]), 0.f);
                    const float ey = fmaxf(fmaxf(blo[1] - pj.y, pj.y - bhi[1]), 0.f);
                    const float ez = fmaxf(fmaxf(blo[2] - pj.z, pj.z - bhi[2]), 0.f);
                    const float reach = reach0 + pj.w;
                    keep = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) <= reach * reach;
                }
                const unsigned km = __ballot_sync(kAll, keep);
                if (keep) {
                    const int s = (head + ns + __popc(km & ((1u << lane) - 1u))) & 63;
                    stj[w][s] = j;
                    stp[w][s] = pj;
                }
                ns += __popc(km);
                const bool last = r0 + 32 >= T;
                while (ns >= 32 || (last && ns > 0)) {
                    __syncwarp();
                    const int s = (head + lane) & 63;
                    int jt = -1;
                    // an unused lane tests a point far outside the box
                    float4 pt4 = make_float4(1e18f, 1e18f, 1e18f, 0.f);
                    if (lane < ns) {
                        jt = stj[w][s];
                        pt4 = stp[w][s];
                    }
                    candj[w][(tc << 5) + lane] = jt;
                    const float wj = pt4.w + skin;
                    // home cell bubbles (only j > i) come first, and only they
                    // lie below e0
                    const bool amb = __shfl_sync(kAll, jt, 0) < e0
                                         ? tile_tests<true>(home[w], nh, h0, jt, pt4, wj, tb,
                                                            hitmask[w][tc])
                                         : tile_tests<false>(home[w], nh, h0, jt, pt4, wj, tb,
                                                             hitmask[w][tc]);
                    if (amb)
                        tile_exact<DIM>(k, home[w], nh, h0, jt, pt4, wj, tb, hitmask[w][tc], X,
                                        Y, Z, R);
                    head = (head + 32) & 63;
                    ns = max(ns - 32, 0);
                    if (++tc == kTileChunks) {
                        tile_rows<M>(hitmask[w], candj[w], tc, nh, row, mycnt);
                        tc = 0;
                    }
                }
                __syncwarp();
            }
            if (tc > 0)
                tile_rows<M>(hitmask[w], candj[w], tc, nh, row, mycnt);
            if (lane < nh) {
                const int i = h0 + lane;
                NN[i] = mycnt;
                rowCount[i] = mycnt;
                over |= mycnt > M;
            }
        }
    }
    if (__syncthreads_or(over) && threadIdx.x == 0) atomicOr(&c->stash_over, 1);
}
CB_KERNEL_PAIR((template <int DIM>), k_pair_tiles, (<DIM>), __launch_bounds__(kBlock, 4))

// The pair list from the counting pass's stash: row i's partners go to
// rowStart[i] .. rowStart[i] + rowCount[i] (pairs grouped by i, j ascending
// inside a row as the enumeration found them). Skipped when a row
// overflowed its stash (the WRITE pass then writes the list).
template <int DIM>
__device__ __forceinline__ void k_pair_compact_body(const Bufs &b, const int vb, const int vg) {
    Ctrl *c = b.ctrl;
    if (c->stash_over) return;
    constexpr int M = kStash(DIM);
    const int n = c->n;
    const int pcap = b.k->pcap;
    int *PI = b.ps[c->prole[PI0]];
    int *PJ = b.ps[c->prole[PJ0]];
    // A warp writes the contiguous output range of its 32 rows, 32 slots at
    // a time (coalesced); the row of a slot is the last of the 32 rows
    // starting at or before it (binary search over the lanes' row starts).
    // Every loop bound is uniform over the warp, so all lanes take part in
    // each shuffle.
    const int lane = threadIdx.x & 31;
    int *NN = b.is[c->irole[INN]];
    for (int i0 = vb * blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += vg * blockDim.x) {
        const int i = i0 + lane;
        const bool act = i < n;
        const int st = act ? b.rowStart[i] : 0;
        const int ct = act ? b.rowCount[i] : 0;
        const int last = min(31, n - 1 - i0);
        const int lo = __shfl_sync(0xffffffffu, st, 0);
        const int hi = __shfl_sync(0xffffffffu, st + ct, last);
        for (int o0 = lo; o0 < hi; o0 += 32) {
            const int o = o0 + lane;
            int r = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                const int cand = r + step;
                const int sc = __shfl_sync(0xffffffffu, st, cand & 31);
                if (cand <= last && sc <= o) r = cand;
            }
            const int sr = __shfl_sync(0xffffffffu, st, r);
            if (o < hi && o < pcap) {
                const int j = b.stash[(size_t)(i0 + r) * M + (o - sr)];
                PI[o] = i0 + r;
                PJ[o] = j;
                atomicAdd(NN + j, 1);  // j's degree (countNumNeighbors); i's came with the row
            }
        }
    }
    if (last_block(&c->done[DC_MISC], vg) && threadIdx.x == 0) {
        const int found = c->np_found;
        if (found > pcap) {
            c->status = CB_ERR_CAPACITY;
            c->np = 0;
        } else {
            c->np = found;
        }
        c->need_search = 0;
        c->done[DC_MISC] = 0;
    }
}
CB_KERNEL_PAIR((template <int DIM>), k_pair_compact, (<DIM>), __launch_bounds__(kBlock))


// j-side neighbour counts of a list the second enumeration wrote (the
// compaction counts them itself when it writes the list).
__device__ __forceinline__ void k_degree_body(const Bufs &b, const int vb, const int vg) {
    const Ctrl *c = b.ctrl;
    if (!c->stash_over) return;
    const int np = c->np;
    const int *PJ = b.ps[c->prole[PJ0]];
    int *NN = b.is[c->irole[INN]];
    for (int p = vb * blockDim.x + threadIdx.x; p < np; p += vg * blockDim.x)
        atomicAdd(NN + PJ[p], 1);
}
CB_KERNEL_PAIR((), k_degree, (), __launch_bounds__(kBlock))


}  // namespace

void launch_search(const Launch &l, const Bufs &b, int dim) {
    const int G = l.grid;
    if (dim == 3) {
        CB_LAUNCH(l, k_wrap, (<3>), G, b);
        CB_LAUNCH(l, k_cell_count, (<3>), G, b);
    } else {
        CB_LAUNCH(l, k_wrap, (<2>), G, b);
        CB_LAUNCH(l, k_cell_count, (<2>), G, b);
    }
    launch_scan(l, b, SCAN_CELLS);
    CB_LAUNCH(l, k_cell_fill, (), G, b);
    CB_LAUNCH(l, k_cell_order, (), G, b);
    if (dim == 3) {
        CB_LAUNCH(l, k_permute, (<3>), G, b);
        CB_LAUNCH(l, k_pair_cells, (<3, false>), G, b);
        CB_LAUNCH(l, k_pair_tiles, (<3>), G, b);
        CB_LAUNCH(l, k_pair_rows, (<3>), G, b);
    } else {
        CB_LAUNCH(l, k_permute, (<2>), G, b);
        CB_LAUNCH(l, k_pair_cells, (<2, false>), G, b);
        CB_LAUNCH(l, k_pair_rows, (<2>), G, b);
    }
    launch_scan(l, b, SCAN_ROWS);
    if (dim == 3) {
        CB_LAUNCH(l, k_pair_compact, (<3>), G, b);
        CB_LAUNCH(l, k_pair_cells, (<3, true>), G, b);
    } else {
        CB_LAUNCH(l, k_pair_compact, (<2>), G, b);
        CB_LAUNCH(l, k_pair_cells, (<2, true>), G, b);
    }
    CB_LAUNCH(l, k_degree, (), G, b);
}

}  // namespace cbg
