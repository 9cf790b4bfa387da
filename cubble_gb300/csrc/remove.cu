// Deletion of bubbles that fell below min_rad, removeBubbles()
// (src/simulator.cu:180-190 -> swapDataCountPairs and addVolumeFixPairs,
// src/kernels.cu:775-936), as parallel stream compaction:
//   * the survivors at or above nNew = n - D fill the deleted slots below
//     nNew: the k-th hole in ascending order takes the k-th survivor counted
//     from the back — the assignment the reference makes when its
//     toBeDeleted list is in ascending order — found with one exclusive scan
//     of the deletion marks instead of the reference's O(D^2) serial search;
//   * pairs touching a deleted bubble are dropped by a stable compaction and
//     the endpoints of moved bubbles are remapped;
//   * the volume fix r *= M / (sum r^D)^(1/D) restores the gas fraction.
#include "common.cuh"

namespace cbg {
namespace {

// holes[k] = k-th deleted index below nNew; keep flags of the pairs.
__device__ __forceinline__ void k_remove_a_body(const Bufs &b, const int vb, const int vg) {
    const Ctrl *c = b.ctrl;
    const int n = c->n, D = c->ndel, nNew = n - D, np = c->np;
    const int *PI = b.ps[c->prole[PI0]];
    const int *PJ = b.ps[c->prole[PJ0]];
    const int stride = vg * blockDim.x;
    for (int i = vb * blockDim.x + threadIdx.x; i < nNew; i += stride)
        if (b.delflag[i]) b.holes[b.iscan[i]] = i;
    for (int p = vb * blockDim.x + threadIdx.x; p < np; p += stride)
        b.keep[p] = !(b.delflag[PI[p]] | b.delflag[PJ[p]]);
}
CB_KERNEL_PAIR((), k_remove_a, (), __launch_bounds__(kBlock))


// Survivors at or above nNew move into the holes.
template <int DIM>
__device__ __forceinline__ void k_remove_b_body(const Bufs &b, const int vb, const int vg) {
    const Ctrl *c = b.ctrl;
    const int n = c->n, D = c->ndel, nNew = n - D;
    static constexpr int kRoles[] = {RX, RY, RZ, RR, RV0, RV1, RV2, RV3, RVO0, RVO1, RVO2, RVO3,
                                     RS0, RS1, RS2, RS3, RPATH, RERR};
    static constexpr int kIRoles[] = {IWX, IWY, IWZ, IIDX, INN};
    for (int i = nNew + vb * blockDim.x + threadIdx.x; i < n;
         i += vg * blockDim.x) {
        if (b.delflag[i]) continue;
        // survivors after i: (n - 1 - i) - (deleted after i)
        const int rank = (n - 1 - i) - (D - b.iscan[i]);
        const int dst = b.holes[rank];
        b.moveDst[i] = dst;
#pragma unroll
        for (int q = 0; q < (int)(sizeof(kRoles) / sizeof(int)); q++) {
            const int role = kRoles[q];
            if (DIM == 2 && (role == RZ || role == RV2 || role == RVO2 || role == RS2)) continue;
            double *row = drow(b, c, role);
            if (b.k->mixed && role >= RV0 && role <= RVO3)  // FP32 rate rows
                reinterpret_cast<float *>(row)[dst] = reinterpret_cast<float *>(row)[i];
            else
                row[dst] = row[i];
        }
#pragma unroll
        for (int q = 0; q < (int)(sizeof(kIRoles) / sizeof(int)); q++) {
            int *row = irow(b, c, kIRoles[q]);
            row[dst] = row[i];
        }
    }
}
CB_KERNEL_PAIR((template <int DIM>), k_remove_b, (<DIM>), __launch_bounds__(kBlock))


// Pair compaction + remap, the volume fix and the bookkeeping.
template <int DIM>
__device__ __forceinline__ void k_remove_c_body(const Bufs &b, const int vb, const int vg) {
    Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n, D = c->ndel, nNew = n - D, np = c->np;
    const int *PI = b.ps[c->prole[PI0]];
    const int *PJ = b.ps[c->prole[PJ0]];
    int *QI = b.ps[c->prole[PI1]];
    int *QJ = b.ps[c->prole[PJ1]];
    const int stride = vg * blockDim.x;
    for (int p = vb * blockDim.x + threadIdx.x; p < np; p += stride) {
        if (!b.keep[p]) continue;
        int e1 = PI[p], e2 = PJ[p];
        if (e1 >= nNew) e1 = b.moveDst[e1];
        if (e2 >= nNew) e2 = b.moveDst[e2];
        const int o = b.keepScan[p];
        QI[o] = e1;
        QJ[o] = e2;
    }
    // src/kernels.cu:861-867 and :932-934
    double volMul = c->vol_new;
    volMul = DIM == 3 ? rcbrt(volMul) : rsqrt(volMul);
    volMul *= k.vol_mul_const;
    double *R = drow(b, c, RR);
    for (int i = vb * blockDim.x + threadIdx.x; i < nNew; i += stride)
        R[i] = R[i] * volMul;
    if (last_block(&c->done[DC_REMOVE], vg) && threadIdx.x == 0) {
        swap_role(c->prole, PI0, PI1);
        swap_role(c->prole, PJ0, PJ1);
        c->np = b.keepScan[np];
        c->n = nNew;
        c->deleted += D;
        c->delete_events += 1;
        c->ndel = 0;
        c->need_delete = 0;
        c->pred_ready = 0;  // bubbles moved and radii rescaled
        c->pred_slot = 0;
        c->done[DC_REMOVE] = 0;
    }
}
CB_KERNEL_PAIR((template <int DIM>), k_remove_c, (<DIM>), __launch_bounds__(kBlock))


}  // namespace

void launch_remove(const Launch &l, const Bufs &b, int dim) {
    const int G = l.grid;
    launch_scan(l, b, SCAN_DEL);
    CB_LAUNCH(l, k_remove_a, (), G, b);
    if (dim == 3)
        CB_LAUNCH(l, k_remove_b, (<3>), G, b);
    else
        CB_LAUNCH(l, k_remove_b, (<2>), G, b);
    launch_scan(l, b, SCAN_KEEP);
    if (dim == 3)
        CB_LAUNCH(l, k_remove_c, (<3>), G, b);
    else
        CB_LAUNCH(l, k_remove_c, (<2>), G, b);
}

}  // namespace cbg
