// Neighbour search, searchNeighbors() (src/simulator.cu:60-178):
//   k_wrap        wrap positions into the box (wrapOverPeriodicBoundaries,
//                 src/kernels.cu:992-1011), exact maximum radius -> cell grid
//   k_cell_count  cell of every bubble (cellByPosition, src/kernels.cu:598-607)
//   scan          cell offsets
//   k_cell_fill   counting-sort scatter (indexByCell, src/kernels.cu:609-615)
//   k_cell_order  one warp per cell orders its bubbles by previous position,
//                 so the cell order is deterministic
//   k_permute_*   gather every persistent row into cell order and set
//                 saved := positions (reorganizeByIndex, src/kernels.cu:721-770);
//                 the pointer rotation of src/simulator.cu:99-146 becomes a
//                 role swap in the control block
//   k_pair_rows   per bubble, the pairs (i, j > i) within r_i + r_j + skin
//                 (neighborSearch / comparePair, src/kernels.cu:617-701):
//                 a count pass, a scan, a fill pass, so the list is ordered
//                 by (i, j) without atomics; candidates are screened in FP32
//                 with a conservative margin and accepted by the exact FP64
//                 test of the reference, so the pair set is bit-exact
//   k_degree      neighbour counts (countNumNeighbors, src/kernels.cu:713-719)
#include "common.cuh"

namespace cbg {
namespace {

__device__ __forceinline__ void swap_role(int *r, int a, int b) {
    const int t = r[a];
    r[a] = r[b];
    r[b] = t;
}

// Cell grid: cellDim_a = max(1, floor(interval_a / (2 maxR + skin))) on the
// used axes; while the product exceeds the cell capacity the largest
// dimension (lowest axis on ties) shrinks by one.
__device__ void cell_grid(const DevConst &k, double max_r, int cd[3]) {
    const double cutoff = __dadd_rn(__dmul_rn(2.0, max_r), k.skin);
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

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_wrap(Bufs b) {
    __shared__ double smem[32];
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    double *XR[3] = {drow(b, c, RX), drow(b, c, RY), drow(b, c, RZ)};
    int *WR[3] = {irow(b, c, IWX), irow(b, c, IWY), irow(b, c, IWZ)};
    const double *R = drow(b, c, RR);
    double mr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
#pragma unroll
        for (int a = 0; a < DIM; a++) {
            if (k.wall[a]) continue;
            const double lo = k.lbb[a], hi = k.tfr[a];
            const double x = XR[a][i];
            const int mult = x < lo ? 1 : (x > hi ? -1 : 0);
            if (mult) {
                XR[a][i] = x + (hi - lo) * (double)mult;
                WR[a][i] -= mult;
            }
        }
        mr = fmax(mr, R[i]);
    }
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= k.ccap; q += gridDim.x * blockDim.x) {
        b.cellCount[q] = 0;
        b.cellFill[q] = 0;
    }
    const double t = block_reduce(mr, OpMax(), smem);
    if (threadIdx.x == 0) b.part[7 * gridDim.x + blockIdx.x] = t;
    if (last_block(&c->done[DC_WRAP])) {
        const double f = fold_partials(b.part + 7 * gridDim.x, gridDim.x, true, smem);
        if (threadIdx.x == 0) {
            int cd[3];
            cell_grid(k, f, cd);
            c->cell_dims[0] = cd[0];
            c->cell_dims[1] = cd[1];
            c->cell_dims[2] = cd[2];
            c->ncell = cd[0] * cd[1] * cd[2];
            c->searches += 1;
            c->done[DC_WRAP] = 0;
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_cell_count(Bufs b) {
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const int cd0 = c->cell_dims[0], cd1 = c->cell_dims[1], cd2 = c->cell_dims[2];
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int kx = cell_coord(X[i], k.lbb[0], k.iv[0], cd0);
        const int ky = cell_coord(Y[i], k.lbb[1], k.iv[1], cd1);
        const int kz = DIM == 3 ? cell_coord(Z[i], k.lbb[2], k.iv[2], cd2) : 0;
        const int ci = (kz * cd1 + ky) * cd0 + kx;
        b.cellOf[i] = ci;
        atomicAdd(b.cellCount + ci, 1);
    }
}

__global__ void __launch_bounds__(kBlock) k_cell_fill(Bufs b) {
    const int n = b.ctrl->n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ci = b.cellOf[i];
        b.perm[b.cellStart[ci] + atomicAdd(b.cellFill + ci, 1)] = i;
    }
}

// One warp per cell: rank each member by its previous position (values are
// distinct), giving the stable counting-sort order.
__global__ void __launch_bounds__(kBlock) k_cell_order(Bufs b) {
    const int ncell = b.ctrl->ncell;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < ncell; q += warps) {
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

// Gather pass A: positions (+ saved), velocities, path, error, wrap counts
// and indices into their spare slots, then swap the roles.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_permute_a(Bufs b) {
    Ctrl *c = b.ctrl;
    const int n = c->n;
    const int *src = b.permSorted;
    const int roles[4][2] = {{RX, RXN}, {RY, RYN}, {RZ, RZN}, {RR, RRN}};
    double *pos[4];
    for (int a = 0; a < 4; a++) {
        const double *from = drow(b, c, roles[a][0]);
        double *to = drow(b, c, roles[a][1]);
        double *sv = drow(b, c, RS0 + a);
        pos[a] = to;
        if (DIM == 2 && a == 2) continue;
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
            const double v = from[src[q]];
            to[q] = v;
            sv[q] = v;
        }
    }
    for (int a = 0; a < 4; a++) {
        if (DIM == 2 && a == 2) continue;
        const double *from = drow(b, c, RV0 + a);
        double *to = drow(b, c, RVP0 + a);
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
            to[q] = from[src[q]];
    }
    {
        const double *f1 = drow(b, c, RPATH), *f2 = drow(b, c, RERR);
        double *t1 = drow(b, c, RPATHN), *t2 = drow(b, c, RERR2);
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
            const int s = src[q];
            t1[q] = f1[s];
            t2[q] = f2[s];
        }
    }
    {
        const int *f[4] = {irow(b, c, IWX), irow(b, c, IWY), irow(b, c, IWZ), irow(b, c, IIDX)};
        int *t[4] = {irow(b, c, IWX2), irow(b, c, IWY2), irow(b, c, IWZ2), irow(b, c, IIDX2)};
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
            const int s = src[q];
            t[0][q] = f[0][s];
            t[1][q] = f[1][s];
            t[2][q] = f[2][s];
            t[3][q] = f[3][s];
        }
    }
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        b.pos32[q] = make_float4((float)pos[0][q], (float)pos[1][q],
                                 DIM == 3 ? (float)pos[2][q] : 0.0f, (float)pos[3][q]);
    }
    if (last_block(&c->done[DC_PERMUTE]) && threadIdx.x == 0) {
        int *r = c->drole;
        for (int a = 0; a < 4; a++) {
            if (DIM == 2 && a == 2) continue;
            swap_role(r, roles[a][0], roles[a][1]);
            swap_role(r, RV0 + a, RVP0 + a);
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

// Gather pass B: previous velocities into the slot the old velocities left.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_permute_b(Bufs b) {
    Ctrl *c = b.ctrl;
    const int n = c->n;
    const int *src = b.permSorted;
    for (int a = 0; a < 4; a++) {
        if (DIM == 2 && a == 2) continue;
        const double *from = drow(b, c, RVO0 + a);
        double *to = drow(b, c, RVP0 + a);
        for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
            to[q] = from[src[q]];
    }
    if (last_block(&c->done[DC_PERMUTE]) && threadIdx.x == 0) {
        for (int a = 0; a < 4; a++) {
            if (DIM == 2 && a == 2) continue;
            swap_role(c->drole, RVO0 + a, RVP0 + a);
        }
        c->done[DC_PERMUTE] = 0;
    }
}

// Unique neighbour cells of `cell` with linear index >= cell, ascending.
template <int DIM>
__device__ __forceinline__ int upper_cells(const DevConst &k, const int cd[3], int cell,
                                           int out[27]) {
    const int kx = cell % cd[0], ky = (cell / cd[0]) % cd[1], kz = cell / (cd[0] * cd[1]);
    int nxs[3], nys[3], nzs[3];
    int mx = 0, my = 0, mz = 0;
    const int kk[3] = {kx, ky, kz};
    int *outs[3] = {nxs, nys, nzs};
    int *ms[3] = {&mx, &my, &mz};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int *o = outs[a];
        int &m = *ms[a];
        const int q = kk[a], d = cd[a];
        if (a >= DIM) {
            o[m++] = 0;
        } else if (!k.wall[a]) {
            if (d == 1) {
                o[m++] = q;
            } else if (d == 2) {
                o[m++] = q;
                o[m++] = (q + 1) % 2;
            } else {
                o[m++] = (q + d - 1) % d;
                o[m++] = q;
                o[m++] = (q + 1) % d;
            }
        } else {
            for (int t = -1; t <= 1; t++)
                if (q + t >= 0 && q + t < d) o[m++] = q + t;
        }
    }
    int m = 0;
    for (int az = 0; az < mz; az++)
        for (int ay = 0; ay < my; ay++)
            for (int ax = 0; ax < mx; ax++) {
                const int v = (nzs[az] * cd[1] + nys[ay]) * cd[0] + nxs[ax];
                if (v < cell) continue;
                int p = m++;
                while (p > 0 && out[p - 1] > v) {
                    out[p] = out[p - 1];
                    p--;
                }
                out[p] = v;
            }
    return m;
}

// Pair rows of bubble i. WRITE=false counts, WRITE=true writes at `base`.
template <int DIM, bool WRITE>
__device__ __forceinline__ int pair_row(const Bufs &b, const DevConst &k, const Ctrl *c, int i,
                                        const double *X, const double *Y, const double *Z,
                                        const double *R, int *PI, int *PJ, int base, int pcap) {
    const int cd[3] = {c->cell_dims[0], c->cell_dims[1], c->cell_dims[2]};
    const int cell = b.cellSorted[i];
    int cells[27];
    const int m = upper_cells<DIM>(k, cd, cell, cells);
    const float4 pi = b.pos32[i];
    const float skin32 = (float)k.skin + k.pre_margin;
    const bool per[3] = {!k.wall[0], !k.wall[1], !k.wall[2]};
    int cnt = 0;
    for (int qi = 0; qi < m; qi++) {
        const int q = cells[qi];
        int s = b.cellStart[q];
        const int e = b.cellStart[q + 1];
        if (q == cell) s = i + 1;
        for (int j = s; j < e; j++) {
            const float4 pj = b.pos32[j];
            float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
            if (per[0] && fabsf(dx) > k.half_iv32[0]) dx = fabsf(dx) - k.iv32[0];
            if (per[1] && fabsf(dy) > k.half_iv32[1]) dy = fabsf(dy) - k.iv32[1];
            if (DIM == 3 && per[2] && fabsf(dz) > k.half_iv32[2]) dz = fabsf(dz) - k.iv32[2];
            const float cut = pi.w + pj.w + skin32;
            float d2 = dx * dx + dy * dy;
            if (DIM == 3) d2 += dz * dz;
            if (d2 >= cut * cut) continue;
            // exact test of comparePair, src/kernels.cu:619-623
            const double maxd = __dadd_rn(__dadd_rn(R[i], R[j]), k.skin);
            const double sq = exact_sqdist<DIM>(k, X[i], Y[i], DIM == 3 ? Z[i] : 0.0, X[j], Y[j],
                                                DIM == 3 ? Z[j] : 0.0);
            if (sq < __dmul_rn(maxd, maxd)) {
                if (WRITE && base + cnt < pcap) {
                    PI[base + cnt] = i;
                    PJ[base + cnt] = j;
                }
                cnt++;
            }
        }
    }
    return cnt;
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_pair_count(Bufs b) {
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        b.rowCount[i] = pair_row<DIM, false>(b, k, c, i, X, Y, Z, R, nullptr, nullptr, 0, 0);
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) k_pair_fill(Bufs b) {
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    const double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ),
                 *R = drow(b, c, RR);
    int *PI = b.ps[c->prole[PI0]];
    int *PJ = b.ps[c->prole[PJ0]];
    int *NN = irow(b, c, INN);
    const int pcap = k.pcap;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int cnt = b.rowCount[i];
        NN[i] = cnt;
        if (cnt) pair_row<DIM, true>(b, k, c, i, X, Y, Z, R, PI, PJ, b.rowStart[i], pcap);
    }
    if (last_block(&c->done[DC_MISC]) && threadIdx.x == 0) {
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

__global__ void __launch_bounds__(kBlock) k_degree(Bufs b) {
    const Ctrl *c = b.ctrl;
    const int np = c->np;
    const int *PJ = b.ps[c->prole[PJ0]];
    int *NN = b.is[c->irole[INN]];
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
        atomicAdd(NN + PJ[p], 1);
}

}  // namespace

void launch_search(const Launch &l, const Bufs &b, int dim) {
    const int G = l.grid;
    cudaStream_t s = l.stream;
    Ctrl *c = b.ctrl;
    if (dim == 3) {
        k_wrap<3><<<G, kBlock, 0, s>>>(b);
        k_cell_count<3><<<G, kBlock, 0, s>>>(b);
    } else {
        k_wrap<2><<<G, kBlock, 0, s>>>(b);
        k_cell_count<2><<<G, kBlock, 0, s>>>(b);
    }
    *l.launches += 2;
    launch_scan(l, b, b.cellCount, b.cellStart, &c->ncell, 0, nullptr);
    k_cell_fill<<<G, kBlock, 0, s>>>(b);
    k_cell_order<<<G, kBlock, 0, s>>>(b);
    *l.launches += 2;
    if (dim == 3) {
        k_permute_a<3><<<G, kBlock, 0, s>>>(b);
        k_permute_b<3><<<G, kBlock, 0, s>>>(b);
        k_pair_count<3><<<G, kBlock, 0, s>>>(b);
    } else {
        k_permute_a<2><<<G, kBlock, 0, s>>>(b);
        k_permute_b<2><<<G, kBlock, 0, s>>>(b);
        k_pair_count<2><<<G, kBlock, 0, s>>>(b);
    }
    *l.launches += 3;
    launch_scan(l, b, b.rowCount, b.rowStart, &c->n, 0, &c->np_found);
    if (dim == 3)
        k_pair_fill<3><<<G, kBlock, 0, s>>>(b);
    else
        k_pair_fill<2><<<G, kBlock, 0, s>>>(b);
    k_degree<<<G, kBlock, 0, s>>>(b);
    *l.launches += 2;
}

}  // namespace cbg
