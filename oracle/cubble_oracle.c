/*
 * TEST INFRASTRUCTURE — CPU FP64 oracle of the reference Durian wet-foam step.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline /
 * reference arm load this file's library, and only as the checker or as the
 * timed CPU baseline. The product (cubble_gb300) never calls it.
 *
 * It restates, line by line, the arithmetic of KJLankinen/cubble:
 *   preIntegrate           src/kernels.cu:40-170
 *   pairwiseInteraction    src/kernels.cu:172-337
 *   postIntegrate/correct  src/kernels.cu:339-495
 *   addFlowVelocity        src/kernels.cu:497-544
 *   addWallVelocity        src/kernels.cu:546-593
 *   cellByPosition..       src/kernels.cu:598-770, 1094-1220
 *   swapDataCountPairs     src/kernels.cu:775-857
 *   addVolumeFixPairs      src/kernels.cu:859-936
 *   potentialEnergy        src/kernels.cu:941-957
 *   euler                  src/kernels.cu:959-969
 *   wrapOverPeriodic..     src/kernels.cu:992-1011
 *   calculateVolumes       src/kernels.cu:1013-1024
 *   step/integrate         src/simulator.cu:192-337
 *   searchNeighbors        src/simulator.cu:60-178
 *   init bootstrap         src/simulator.cu:727-787
 * with the reference's nondeterministic orders replaced by deterministic
 * ones that are one of the orders the reference can produce:
 *   - bubbles within a cell are ordered by their previous position
 *     (the reference's indexByCell, src/kernels.cu:609-615, uses atomics);
 *   - pairs are ordered by (i, j) (src/kernels.cu:630, :707 use atomics);
 *   - deleted bubbles are processed in ascending index order
 *     (src/kernels.cu:425 appends with an atomic);
 *   - pairs that survive a deletion keep their relative order.
 * Two deliberate differences, documented in the design notes:
 *   - the cell grid is sized from the exact maximum radius and the pair
 *     cutoff 2*maxR + skin (the reference uses 2*(maxR + skin), :69-75);
 *     cells only decide which candidates are tested, so the pair set is the
 *     same, and for cellDim < 3 on a periodic axis no pair is double counted
 *     (the reference double counts there, src/kernels.cu:1167-1186);
 *   - the per-bubble error row takes the per-bubble maximum; the reference
 *     takes a per-thread running maximum (src/kernels.cu:455), identical for
 *     N <= 5120*384.
 * Build with -ffp-contract=off so that x86-64 and aarch64 give the same
 * bits (no fused multiply-add is formed).
 */
#include "cubble_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CBO_PI 3.1415926535897932384626433832795028841971693993

static _Thread_local char g_err[512];

static int fail(int code, const char *msg) {
    snprintf(g_err, sizeof(g_err), "%s", msg);
    return code;
}

const char *cbo_last_error(void) { return g_err; }

struct cbo_ctx {
    cb_config cfg;
    int dim, cap, pcap, ccap, n, np, nthreads;
    int use_gas, use_flow, inc_path, status, loaded;
    double lbb[3], tfr[3], iv[3];
    double vol_mul_const;
    double flow_lbb[3], flow_tfr[3];
    /* rows (roles rotate by pointer swaps like the reference's Params) */
    double *x[4], *xp[4], *v[4], *vo[4], *vp[4], *saved[4];
    double *path, *pathn, *err, *fv[3], *ov;
    int32_t *wrap[3], *index, *nn, *del;
    int32_t *pi, *pj;
    /* scratch */
    double *tmpd;
    int32_t *tmpi, *cell, *perm, *cstart, *cfill, *holes, *movers, *remap,
        *rowcnt;
    /* control */
    double dt, tfrac;
    uint64_t tint;
    int64_t steps, attempts, searches, deleted, bubble_steps;
    double max_err, max_exp, max_rad, max_bubble_radius;
    double sumA, sumAr, sumAo, sumAor, vol_new;
    int ndel;
    int cell_dims[3];
};

/* ------------------------------------------------------------- helpers */
static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s);
    return p;
}

static void swapp(double **a, double **b) {
    double *t = *a;
    *a = *b;
    *b = t;
}

/* wrappedDifference, src/kernels.cu:1094-1114 */
static inline void wrapped_diff(const cbo_ctx *c, double x1, double y1,
                                double z1, double x2, double y2, double z2,
                                double d[3]) {
    double d1[3] = {x1 - x2, y1 - y2, 0.0};
    if (3 == c->dim) d1[2] = z1 - z2;
    d[0] = d1[0];
    d[1] = d1[1];
    d[2] = d1[2];
    double t[3];
    for (int a = 0; a < 3; a++) t[a] = c->iv[a] - (d1[a] < 0 ? -d1[a] : d1[a]);
    if (!c->cfg.wall[0] && t[0] * t[0] < d1[0] * d1[0])
        d[0] = t[0] * (d1[0] < 0 ? 1.0 : -1.0);
    if (!c->cfg.wall[1] && t[1] * t[1] < d1[1] * d1[1])
        d[1] = t[1] * (d1[1] < 0 ? 1.0 : -1.0);
    if (3 == c->dim && !c->cfg.wall[2] && t[2] * t[2] < d1[2] * d1[2])
        d[2] = t[2] * (d1[2] < 0 ? 1.0 : -1.0);
}

/* vec::getSquaredLength, src/vec.h:41-49 */
static inline double sqlen(const double d[3]) {
    double t = 0.0;
    t += d[0] * d[0];
    t += d[1] * d[1];
    t += d[2] * d[2];
    return t;
}

/* Deterministic blocked sum: fixed 4096-element blocks summed in order, then
 * the block sums in order. Independent of the thread count. */
#define CBO_RBLK 4096
static double blocked_sum(const double *a, int n, int nthreads) {
    int nb = (n + CBO_RBLK - 1) / CBO_RBLK;
    double *bs = (double *)xcalloc((size_t)nb, sizeof(double));
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
    for (int b = 0; b < nb; b++) {
        double s = 0.0;
        int e = (b + 1) * CBO_RBLK < n ? (b + 1) * CBO_RBLK : n;
        for (int i = b * CBO_RBLK; i < e; i++) s += a[i];
        bs[b] = s;
    }
    (void)nthreads;
    double s = 0.0;
    for (int b = 0; b < nb; b++) s += bs[b];
    free(bs);
    return s;
}

/* --------------------------------------------------------------- create */
int cbo_create(const cb_config *cfg, cbo_ctx **out) {
    if (!cfg || !out) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    if (cfg->dimensionality != 2 && cfg->dimensionality != 3)
        return fail(CB_ERR_INVALID_ARGUMENT, "dimensionality must be 2 or 3");
    if (cfg->capacity <= 0)
        return fail(CB_ERR_INVALID_ARGUMENT, "capacity must be positive");
    cbo_ctx *c = (cbo_ctx *)xcalloc(1, sizeof(cbo_ctx));
    c->cfg = *cfg;
    c->dim = cfg->dimensionality;
    c->cap = cfg->capacity;
    c->pcap = cfg->pair_capacity > 0 ? cfg->pair_capacity
                                     : (c->dim == 3 ? 16 : 8) * c->cap;
    c->ccap = 2 * c->cap + 64;
    if (c->cfg.max_attempts <= 0) c->cfg.max_attempts = 64;
    c->nthreads = 1;
    c->use_gas = cfg->use_gas_exchange;
    c->use_flow = cfg->use_flow;
    c->inc_path = cfg->increment_path;
    for (int a = 0; a < 3; a++) {
        c->lbb[a] = cfg->lbb[a];
        c->tfr[a] = cfg->tfr[a];
        c->iv[a] = cfg->tfr[a] - cfg->lbb[a];
        c->flow_lbb[a] = cfg->flow_lbb[a];
        c->flow_tfr[a] = cfg->flow_tfr[a];
    }
    c->vol_mul_const = cfg->bubble_volume_multiplier;
    c->dt = cfg->time_step;
    size_t n = (size_t)c->cap;
    for (int a = 0; a < 4; a++) {
        c->x[a] = xcalloc(n, 8);
        c->xp[a] = xcalloc(n, 8);
        c->v[a] = xcalloc(n, 8);
        c->vo[a] = xcalloc(n, 8);
        c->vp[a] = xcalloc(n, 8);
        c->saved[a] = xcalloc(n, 8);
    }
    for (int a = 0; a < 3; a++) {
        c->fv[a] = xcalloc(n, 8);
        c->wrap[a] = xcalloc(n, 4);
    }
    c->path = xcalloc(n, 8);
    c->pathn = xcalloc(n, 8);
    c->err = xcalloc(n, 8);
    c->ov = xcalloc(n, 8);
    c->tmpd = xcalloc(n, 8);
    c->index = xcalloc(n, 4);
    c->nn = xcalloc(n, 4);
    c->del = xcalloc(n, 4);
    c->tmpi = xcalloc(n, 4);
    c->cell = xcalloc(n, 4);
    c->perm = xcalloc(n, 4);
    c->holes = xcalloc(n, 4);
    c->movers = xcalloc(n, 4);
    c->remap = xcalloc(n, 4);
    c->rowcnt = xcalloc(n + 1, 4);
    c->cstart = xcalloc((size_t)c->ccap + 1, 4);
    c->cfill = xcalloc((size_t)c->ccap + 1, 4);
    c->pi = xcalloc((size_t)c->pcap, 4);
    c->pj = xcalloc((size_t)c->pcap, 4);
    *out = c;
    return CB_OK;
}

int cbo_destroy(cbo_ctx *c) {
    if (!c) return CB_OK;
    for (int a = 0; a < 4; a++) {
        free(c->x[a]);
        free(c->xp[a]);
        free(c->v[a]);
        free(c->vo[a]);
        free(c->vp[a]);
        free(c->saved[a]);
    }
    for (int a = 0; a < 3; a++) {
        free(c->fv[a]);
        free(c->wrap[a]);
    }
    free(c->path);
    free(c->pathn);
    free(c->err);
    free(c->ov);
    free(c->tmpd);
    free(c->index);
    free(c->nn);
    free(c->del);
    free(c->tmpi);
    free(c->cell);
    free(c->perm);
    free(c->holes);
    free(c->movers);
    free(c->remap);
    free(c->rowcnt);
    free(c->cstart);
    free(c->cfill);
    free(c->pi);
    free(c->pj);
    free(c);
    return CB_OK;
}

int cbo_set_threads(cbo_ctx *c, int32_t nthreads) {
    if (!c || nthreads < 1) return fail(CB_ERR_INVALID_ARGUMENT, "threads");
    c->nthreads = nthreads;
    return CB_OK;
}

/* ------------------------------------------------------------ state io */
static void load_row_d(double *dst, const double *src, int n, double fill) {
    if (src)
        memcpy(dst, src, (size_t)n * 8);
    else
        for (int i = 0; i < n; i++) dst[i] = fill;
}

int cbo_load_state(cbo_ctx *c, const cb_state_view *s) {
    if (!c || !s) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    if (s->count < 0 || s->count > c->cap)
        return fail(CB_ERR_CAPACITY, "count exceeds capacity");
    if (!s->x || !s->y || !s->r || (c->dim == 3 && !s->z))
        return fail(CB_ERR_INVALID_ARGUMENT, "positions and radii required");
    int n = s->count;
    c->n = n;
    load_row_d(c->x[0], s->x, n, 0);
    load_row_d(c->x[1], s->y, n, 0);
    load_row_d(c->x[2], s->z, n, 0);
    load_row_d(c->x[3], s->r, n, 0);
    load_row_d(c->v[0], s->dxdt, n, 0);
    load_row_d(c->v[1], s->dydt, n, 0);
    load_row_d(c->v[2], s->dzdt, n, 0);
    load_row_d(c->v[3], s->drdt, n, 0);
    load_row_d(c->vo[0], s->dxdto, n, 0);
    load_row_d(c->vo[1], s->dydto, n, 0);
    load_row_d(c->vo[2], s->dzdto, n, 0);
    load_row_d(c->vo[3], s->drdto, n, 0);
    load_row_d(c->path, s->path, n, 0);
    load_row_d(c->err, s->error, n, 0);
    load_row_d(c->saved[0], s->saved_x ? s->saved_x : s->x, n, 0);
    load_row_d(c->saved[1], s->saved_y ? s->saved_y : s->y, n, 0);
    load_row_d(c->saved[2], s->saved_z ? s->saved_z : s->z, n, 0);
    load_row_d(c->saved[3], s->saved_r ? s->saved_r : s->r, n, 0);
    int32_t *wr[3] = {s->wrap_count_x, s->wrap_count_y, s->wrap_count_z};
    for (int a = 0; a < 3; a++) {
        if (wr[a])
            memcpy(c->wrap[a], wr[a], (size_t)n * 4);
        else
            memset(c->wrap[a], 0, (size_t)n * 4);
    }
    for (int i = 0; i < n; i++) c->index[i] = s->index ? s->index[i] : i;
    if (s->num_neighbors)
        memcpy(c->nn, s->num_neighbors, (size_t)n * 4);
    else
        memset(c->nn, 0, (size_t)n * 4);
    /* rp == r while gas exchange is off (src/simulator.cu:329-333) */
    memcpy(c->xp[3], c->x[3], (size_t)n * 8);
    double mr = 0.0;
    for (int i = 0; i < n; i++) mr = c->x[3][i] > mr ? c->x[3][i] : mr;
    c->max_bubble_radius = mr;
    c->np = 0;
    c->loaded = 1;
    c->status = CB_OK;
    return CB_OK;
}

static void get_row_d(double *dst, const double *src, int n) {
    if (dst) memcpy(dst, src, (size_t)n * 8);
}
static void get_row_i(int32_t *dst, const int32_t *src, int n) {
    if (dst) memcpy(dst, src, (size_t)n * 4);
}

int cbo_get_state(cbo_ctx *c, cb_state_view *s) {
    if (!c || !s) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    int n = c->n;
    s->count = n;
    get_row_d(s->x, c->x[0], n);
    get_row_d(s->y, c->x[1], n);
    get_row_d(s->z, c->x[2], n);
    get_row_d(s->r, c->x[3], n);
    get_row_d(s->dxdt, c->v[0], n);
    get_row_d(s->dydt, c->v[1], n);
    get_row_d(s->dzdt, c->v[2], n);
    get_row_d(s->drdt, c->v[3], n);
    get_row_d(s->dxdto, c->vo[0], n);
    get_row_d(s->dydto, c->vo[1], n);
    get_row_d(s->dzdto, c->vo[2], n);
    get_row_d(s->drdto, c->vo[3], n);
    get_row_d(s->path, c->path, n);
    get_row_d(s->error, c->err, n);
    get_row_d(s->saved_x, c->saved[0], n);
    get_row_d(s->saved_y, c->saved[1], n);
    get_row_d(s->saved_z, c->saved[2], n);
    get_row_d(s->saved_r, c->saved[3], n);
    get_row_i(s->wrap_count_x, c->wrap[0], n);
    get_row_i(s->wrap_count_y, c->wrap[1], n);
    get_row_i(s->wrap_count_z, c->wrap[2], n);
    get_row_i(s->index, c->index, n);
    get_row_i(s->num_neighbors, c->nn, n);
    return CB_OK;
}

int cbo_set_options(cbo_ctx *c, int32_t g, int32_t f, int32_t p) {
    if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    if (c->use_gas && !g) /* rp := r, as after a search with gas off */
        memcpy(c->xp[3], c->x[3], (size_t)c->n * 8);
    c->use_gas = g;
    c->use_flow = f;
    c->inc_path = p;
    return CB_OK;
}

int cbo_set_time(cbo_ctx *c, double dt, uint64_t ti, double tf) {
    if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    c->dt = dt;
    c->tint = ti;
    c->tfrac = tf;
    return CB_OK;
}

int cbo_set_box(cbo_ctx *c, const double lbb[3], const double tfr[3],
                double m, const double flbb[3], const double ftfr[3]) {
    if (!c) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    for (int a = 0; a < 3; a++) {
        c->lbb[a] = lbb[a];
        c->tfr[a] = tfr[a];
        c->iv[a] = tfr[a] - lbb[a];
        if (flbb) c->flow_lbb[a] = flbb[a];
        if (ftfr) c->flow_tfr[a] = ftfr[a];
    }
    c->vol_mul_const = m;
    return CB_OK;
}

/* ----------------------------------------------------- neighbour search */
/* Cell grid: cellDim_a = max(1, floor(interval_a / (2 maxR + skin))) on the
 * used axes, then while prod(cellDim) > 2*capacity + 64 the largest
 * dimension (lowest axis on ties) shrinks by one. */
static void cell_grid(const cbo_ctx *c, double max_r, int cd[3]) {
    double cutoff = 2.0 * max_r + c->cfg.skin_radius;
    for (int a = 0; a < 3; a++) {
        cd[a] = 1;
        if (a < c->dim) {
            double q = floor(c->iv[a] / cutoff);
            if (q > 1048576.0) q = 1048576.0;
            cd[a] = q >= 1.0 ? (int)q : 1;
        }
    }
    for (;;) {
        long long tot = (long long)cd[0] * cd[1] * cd[2];
        if (tot <= (long long)c->ccap) break;
        int m = 0;
        for (int a = 1; a < 3; a++)
            if (cd[a] > cd[m]) m = a;
        cd[m] -= 1;
    }
}

/* getCellIdxFromPos, src/kernels.cu:1191-1203 (clamped to the grid) */
static inline int cell_coord(double x, double lbb, double iv, int cd) {
    double q = floor((double)cd * (x - lbb) / iv);
    int k = q < 0.0 ? 0 : (q >= (double)cd ? cd - 1 : (int)q);
    return k;
}

/* Unique neighbour offsets of one axis: {0} for an unused axis or a
 * single-cell periodic axis, {0,+1} for a two-cell periodic axis, else
 * {-1,0,+1} (wall axes drop out-of-range cells). */
static int axis_neighbors(int k, int cd, int periodic, int used, int out[3]) {
    int m = 0;
    if (!used) {
        out[m++] = 0;
        return m;
    }
    if (periodic) {
        if (cd == 1) {
            out[m++] = 0;
        } else if (cd == 2) {
            out[m++] = k;
            out[m++] = (k + 1) % 2;
        } else {
            out[m++] = (k + cd - 1) % cd;
            out[m++] = k;
            out[m++] = (k + 1) % cd;
        }
        if (cd == 1) out[0] = k;
        return m;
    }
    for (int o = -1; o <= 1; o++)
        if (k + o >= 0 && k + o < cd) out[m++] = k + o;
    return m;
}

static int neighbor_cells(const cbo_ctx *c, int cell, int out[27]) {
    const int *cd = c->cell_dims;
    int kx = cell % cd[0], ky = (cell / cd[0]) % cd[1], kz = cell / (cd[0] * cd[1]);
    int nx[3], ny[3], nz[3];
    int mx = axis_neighbors(kx, cd[0], !c->cfg.wall[0], 1, nx);
    int my = axis_neighbors(ky, cd[1], !c->cfg.wall[1], 1, ny);
    int mz = axis_neighbors(kz, cd[2], !c->cfg.wall[2], c->dim == 3, nz);
    int m = 0;
    for (int a = 0; a < mz; a++)
        for (int b = 0; b < my; b++)
            for (int d = 0; d < mx; d++)
                out[m++] = (nz[a] * cd[1] + ny[b]) * cd[0] + nx[d];
    /* ascending linear order */
    for (int a = 1; a < m; a++) {
        int v = out[a], b = a - 1;
        while (b >= 0 && out[b] > v) {
            out[b + 1] = out[b];
            b--;
        }
        out[b + 1] = v;
    }
    return m;
}

/* comparePair's acceptance test, src/kernels.cu:617-623 */
static inline int pair_accept(const cbo_ctx *c, int i, int j) {
    double maxd = c->x[3][i] + c->x[3][j] + c->cfg.skin_radius;
    double d[3];
    wrapped_diff(c, c->x[0][i], c->x[1][i], c->x[2][i], c->x[0][j],
                 c->x[1][j], c->x[2][j], d);
    return sqlen(d) < maxd * maxd;
}

static void permute_d(cbo_ctx *c, double *row) {
    for (int k = 0; k < c->n; k++) c->tmpd[k] = row[c->perm[k]];
    memcpy(row, c->tmpd, (size_t)c->n * 8);
}
static void permute_i(cbo_ctx *c, int32_t *row) {
    for (int k = 0; k < c->n; k++) c->tmpi[k] = row[c->perm[k]];
    memcpy(row, c->tmpi, (size_t)c->n * 4);
}

int cbo_search_neighbors(cbo_ctx *c) {
    if (!c || !c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    const int n = c->n, dim = c->dim;
    c->searches++;
    /* wrapOverPeriodicBoundaries, src/kernels.cu:992-1011 */
    for (int a = 0; a < dim; a++) {
        if (c->cfg.wall[a]) continue;
        double lo = c->lbb[a], hi = c->tfr[a];
        for (int i = 0; i < n; i++) {
            double x = c->x[a][i];
            int mult = x < lo ? 1 : (x > hi ? -1 : 0);
            c->x[a][i] = x + (hi - lo) * (double)mult;
            c->wrap[a][i] -= mult;
        }
    }
    /* cell grid from the exact maximum radius */
    double mr = 0.0;
    for (int i = 0; i < n; i++) mr = c->x[3][i] > mr ? c->x[3][i] : mr;
    cell_grid(c, mr, c->cell_dims);
    const int *cd = c->cell_dims;
    const int ncell = cd[0] * cd[1] * cd[2];
    /* cellByPosition + stable counting sort (indexByCell, :598-615) */
    memset(c->cfill, 0, (size_t)(ncell + 1) * 4);
    for (int i = 0; i < n; i++) {
        int kx = cell_coord(c->x[0][i], c->lbb[0], c->iv[0], cd[0]);
        int ky = cell_coord(c->x[1][i], c->lbb[1], c->iv[1], cd[1]);
        int kz = dim == 3 ? cell_coord(c->x[2][i], c->lbb[2], c->iv[2], cd[2]) : 0;
        int ci = (kz * cd[1] + ky) * cd[0] + kx;
        c->cell[i] = ci;
        c->cfill[ci]++;
    }
    c->cstart[0] = 0;
    for (int k = 0; k < ncell; k++) c->cstart[k + 1] = c->cstart[k] + c->cfill[k];
    memset(c->cfill, 0, (size_t)(ncell + 1) * 4);
    for (int i = 0; i < n; i++) {
        int ci = c->cell[i];
        c->perm[c->cstart[ci] + c->cfill[ci]++] = i;
    }
    /* reorganizeByIndex, src/kernels.cu:721-770: permute every row, saved := x */
    for (int a = 0; a < 4; a++) {
        permute_d(c, c->x[a]);
        permute_d(c, c->v[a]);
        permute_d(c, c->vo[a]);
        memcpy(c->saved[a], c->x[a], (size_t)n * 8);
    }
    permute_d(c, c->path);
    permute_d(c, c->err);
    for (int a = 0; a < 3; a++) permute_i(c, c->wrap[a]);
    permute_i(c, c->index);
    for (int k = 0; k < n; k++) c->tmpi[k] = c->cell[c->perm[k]];
    memcpy(c->cell, c->tmpi, (size_t)n * 4);
    /* rp := r (src/simulator.cu:329-333; with gas on preIntegrate rewrites it) */
    memcpy(c->xp[3], c->x[3], (size_t)n * 8);

    /* neighborSearch, src/kernels.cu:636-701: pairs (i<j) in (i, j) order.
     * Two passes: count per row, then fill. */
#ifdef _OPENMP
#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic, 256)
#endif
    for (int i = 0; i < n; i++) {
        int nb[27];
        int m = neighbor_cells(c, c->cell[i], nb);
        int cnt = 0;
        for (int q = 0; q < m; q++) {
            if (nb[q] < c->cell[i]) continue;
            int s = c->cstart[nb[q]], e = c->cstart[nb[q] + 1];
            for (int j = s; j < e; j++)
                if (j > i && pair_accept(c, i, j)) cnt++;
        }
        c->rowcnt[i] = cnt;
    }
    long long tot = 0;
    for (int i = 0; i < n; i++) {
        int t = c->rowcnt[i];
        c->rowcnt[i] = (int)tot;
        tot += t;
    }
    if (tot > c->pcap) {
        c->np = 0;
        c->status = CB_ERR_CAPACITY;
        return fail(CB_ERR_CAPACITY, "pair capacity exceeded");
    }
#ifdef _OPENMP
#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic, 256)
#endif
    for (int i = 0; i < n; i++) {
        int nb[27];
        int m = neighbor_cells(c, c->cell[i], nb);
        int o = c->rowcnt[i];
        for (int q = 0; q < m; q++) {
            if (nb[q] < c->cell[i]) continue;
            int s = c->cstart[nb[q]], e = c->cstart[nb[q] + 1];
            for (int j = s; j < e; j++)
                if (j > i && pair_accept(c, i, j)) {
                    c->pi[o] = i;
                    c->pj[o] = j;
                    o++;
                }
        }
    }
    c->np = (int)tot;
    /* countNumNeighbors, src/kernels.cu:713-719 */
    memset(c->nn, 0, (size_t)n * 4);
    for (int p = 0; p < c->np; p++) {
        c->nn[c->pi[p]]++;
        c->nn[c->pj[p]]++;
    }
    return CB_OK;
}

int cbo_cell_dims(cbo_ctx *c, int32_t dims[3]) {
    if (!c || !dims) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    for (int a = 0; a < 3; a++) dims[a] = c->cell_dims[a];
    return CB_OK;
}

int cbo_get_pairs(cbo_ctx *c, int32_t *i, int32_t *j, int32_t capacity,
                  int32_t *count) {
    if (!c || !count) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    *count = c->np;
    if (!i || !j) return CB_OK;
    if (capacity < c->np) return fail(CB_ERR_CAPACITY, "buffer too small");
    memcpy(i, c->pi, (size_t)c->np * 4);
    memcpy(j, c->pj, (size_t)c->np * 4);
    return CB_OK;
}

int cbo_set_pairs(cbo_ctx *c, const int32_t *i, const int32_t *j,
                  int32_t count) {
    if (!c || count < 0 || (count && (!i || !j)))
        return fail(CB_ERR_INVALID_ARGUMENT, "bad pairs");
    if (count > c->pcap) return fail(CB_ERR_CAPACITY, "pair capacity exceeded");
    for (int p = 0; p < count; p++)
        if (i[p] < 0 || j[p] < 0 || i[p] >= c->n || j[p] >= c->n || i[p] == j[p])
            return fail(CB_ERR_INVALID_ARGUMENT, "pair index out of range");
    memcpy(c->pi, i, (size_t)count * 4);
    memcpy(c->pj, j, (size_t)count * 4);
    c->np = count;
    memset(c->nn, 0, (size_t)c->n * 4);
    for (int p = 0; p < count; p++) {
        c->nn[i[p]]++;
        c->nn[j[p]]++;
    }
    return CB_OK;
}

/* ---------------------------------------------------------------- step */
/* preIntegrate, src/kernels.cu:40-170 */
static void pre_integrate(cbo_ctx *c, double ts) {
    const int n = c->n, dim = c->dim, gas = c->use_gas;
    double *A = c->tmpd;
    double *Ar = c->ov; /* borrowed, zeroed below */
#ifdef _OPENMP
#pragma omp parallel for num_threads(c->nthreads) schedule(static)
#endif
    for (int i = 0; i < n; i++) {
        for (int a = 0; a < dim; a++)
            c->xp[a][i] = c->x[a][i] + 0.5 * ts * (3.0 * c->v[a][i] - c->vo[a][i]);
        A[i] = 0.0;
        Ar[i] = 0.0;
        if (gas) {
            double rp = c->x[3][i] + 0.5 * ts * (3.0 * c->v[3][i] - c->vo[3][i]);
            c->xp[3][i] = rp;
            double apr = 2.0 * CBO_PI;
            if (3 == dim) apr *= 2.0 * rp;
            A[i] = apr * rp;
            Ar[i] = apr;
        }
    }
    if (gas) {
        c->sumA = blocked_sum(A, n, c->nthreads);
        c->sumAr = blocked_sum(Ar, n, c->nthreads);
    } else {
        c->sumA = c->sumAr = 0.0;
    }
#ifdef _OPENMP
#pragma omp parallel for num_threads(c->nthreads) schedule(static)
#endif
    for (int i = 0; i < n; i++) {
        c->ov[i] = 0.0;
        for (int a = 0; a < 3; a++) {
            c->fv[a][i] = 0.0;
            c->vp[a][i] = 0.0;
        }
        if (gas) c->vp[3][i] = 0.0;
    }
}

/* pairwiseInteraction, src/kernels.cu:172-337, one pair */
static inline void pair_terms(const cbo_ctx *c, int i, int j, int gas,
                              int flow, double out[8], int *overlapping) {
    (void)flow;
    double r1 = c->xp[3][i];
    double r2 = c->xp[3][j];
    const double radii = r1 + r2;
    double d[3];
    wrapped_diff(c, c->xp[0][i], c->xp[1][i], c->xp[2][i], c->xp[0][j],
                 c->xp[1][j], c->xp[2][j], d);
    const double m = sqlen(d);
    *overlapping = radii * radii >= m;
    if (!*overlapping) return;
    const double f0 = c->cfg.f0_per_mu0;
    const double s = 1.0 / sqrt(m) - 1.0 / radii;
    out[0] = d[0] * f0 * s;
    out[1] = d[1] * f0 * s;
    out[2] = d[2] * f0 * s;
    out[3] = out[4] = out[5] = out[6] = 0.0;
    if (gas) {
        const double r1sq = r1 * r1;
        const double r2sq = r2 * r2;
        double oa = 0;
        if (m < r1sq || m < r2sq) {
            oa = r1sq < r2sq ? r1sq : r2sq;
        } else {
            oa = 0.5 * (r2sq - r1sq + m);
            oa *= oa;
            oa /= m;
            oa = r2sq - oa;
            oa = oa < 0 ? -oa : oa;
        }
        if (3 == c->dim)
            oa *= CBO_PI;
        else
            oa = 2.0 * sqrt(oa);
        r1 = 1.0 / r1;
        r2 = 1.0 / r2;
        out[4] = oa;                 /* overlap area         */
        out[5] = 2.0 * oa;           /* total overlap area   */
        out[6] = oa * (r1 + r2);     /* total overlap / r    */
        out[3] = oa * (r2 - r1);     /* drdtp                */
    }
}

static void pairwise(cbo_ctx *c, int gas, int flow) {
    const int np = c->np, dim = c->dim;
    double sAo = 0.0, sAor = 0.0;
    if (c->nthreads <= 1) {
        for (int p = 0; p < np; p++) {
            const int i = c->pi[p], j = c->pj[p];
            if (flow) {
                c->fv[0][j] += c->v[0][i];
                c->fv[1][j] += c->v[1][i];
                if (3 == dim) c->fv[2][j] += c->v[2][i];
            }
            double t[8];
            int ov;
            pair_terms(c, i, j, gas, flow, t, &ov);
            if (!ov) continue;
            c->vp[0][i] += t[0];
            c->vp[0][j] -= t[0];
            c->vp[1][i] += t[1];
            c->vp[1][j] -= t[1];
            if (3 == dim) {
                c->vp[2][i] += t[2];
                c->vp[2][j] -= t[2];
            }
            if (gas) {
                c->ov[i] += t[4];
                c->ov[j] += t[4];
                sAo += t[5];
                sAor += t[6];
                c->vp[3][i] += t[3];
                c->vp[3][j] -= t[3];
            }
            if (flow) {
                c->fv[0][i] += c->v[0][j];
                c->fv[1][i] += c->v[1][j];
                if (3 == dim) c->fv[2][i] += c->v[2][j];
            }
        }
    } else {
#ifdef _OPENMP
#pragma omp parallel for num_threads(c->nthreads) schedule(static) reduction(+ : sAo, sAor)
#endif
        for (int p = 0; p < np; p++) {
            const int i = c->pi[p], j = c->pj[p];
            if (flow) {
                for (int a = 0; a < dim; a++) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                    c->fv[a][j] += c->v[a][i];
                }
            }
            double t[8];
            int ov;
            pair_terms(c, i, j, gas, flow, t, &ov);
            if (!ov) continue;
            for (int a = 0; a < dim; a++) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                c->vp[a][i] += t[a];
#ifdef _OPENMP
#pragma omp atomic
#endif
                c->vp[a][j] -= t[a];
            }
            if (gas) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                c->ov[i] += t[4];
#ifdef _OPENMP
#pragma omp atomic
#endif
                c->ov[j] += t[4];
                sAo += t[5];
                sAor += t[6];
#ifdef _OPENMP
#pragma omp atomic
#endif
                c->vp[3][i] += t[3];
#ifdef _OPENMP
#pragma omp atomic
#endif
                c->vp[3][j] -= t[3];
            }
            if (flow) {
                for (int a = 0; a < dim; a++) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                    c->fv[a][i] += c->v[a][j];
                }
            }
        }
    }
    c->sumAo = sAo;
    c->sumAor = sAor;
}

/* addFlowVelocity, src/kernels.cu:497-544 */
static void add_flow_velocity(cbo_ctx *c, int i) {
    double multiplier = c->nn[i];
    multiplier = (multiplier > 0 ? 1.0 / multiplier : 0.0);
    const double xi = c->xp[0][i];
    const double yi = c->xp[1][i];
    double riSq = c->xp[3][i];
    riSq *= riSq;
    const double *fl = c->flow_lbb, *ft = c->flow_tfr, *fvel = c->cfg.flow_vel;
    int inside = (int)((xi < ft[0] && xi > fl[0]) ||
                       ((fl[0] - xi) * (fl[0] - xi) <= riSq) ||
                       ((ft[0] - xi) * (ft[0] - xi) <= riSq));
    inside *= (int)((yi < ft[1] && yi > fl[1]) ||
                    ((fl[1] - yi) * (fl[1] - yi) <= riSq) ||
                    ((ft[1] - yi) * (ft[1] - yi) <= riSq));
    if (c->dim == 3) {
        const double zi = c->xp[2][i];
        inside *= (int)((zi < ft[2] && zi > fl[2]) ||
                        ((fl[2] - zi) * (fl[2] - zi) <= riSq) ||
                        ((ft[2] - zi) * (ft[2] - zi) <= riSq));
        c->vp[2][i] += !inside * multiplier * c->fv[2][i] + fvel[2] * inside;
    }
    c->vp[0][i] += !inside * multiplier * c->fv[0][i] + fvel[0] * inside;
    c->vp[1][i] += !inside * multiplier * c->fv[1][i] + fvel[1] * inside;
}

/* Linear shear along x over the last axis (cb_config.shear_speed, an
 * extension of this library; the reference has only the box-region flow). */
static void add_shear_velocity(cbo_ctx *c, int i) {
    const int q = c->dim - 1;
    const double len = c->tfr[q] - c->lbb[q];
    const double pos = c->xp[q][i];
    c->vp[0][i] += c->cfg.shear_speed * ((pos - c->lbb[q]) * (2.0 / len) - 1.0);
}

/* touchesWall lambda of addWallVelocity, src/kernels.cu:553-566 */
static inline int touches_wall(double f0, double rad, double x, double low,
                               double high, double *velocity) {
    double d1 = x - low;
    double d2 = x - high;
    d1 = d1 * d1 < d2 * d2 ? d1 : d2;
    if (rad * rad >= d1 * d1) {
        d2 = d1 < 0.0 ? -1.0 : 1.0;
        d1 *= d2;
        *velocity = d2 * f0 * (1.0 - d1 / rad);
        return 1;
    }
    return 0;
}

/* addWallVelocity, src/kernels.cu:546-593 */
static void add_wall_velocity(cbo_ctx *c, int i) {
    const double drag = 1.0 - c->cfg.wall_drag;
    const double rad = c->xp[3][i];
    const double f0 = c->cfg.f0_per_mu0;
    double xDrag = 1.0, yDrag = 1.0, velocity = 0.0;
    velocity = 0.0;
    if (c->cfg.wall[0] &&
        touches_wall(f0, rad, c->xp[0][i], c->lbb[0], c->tfr[0], &velocity)) {
        c->vp[0][i] += velocity;
        c->vp[1][i] *= drag;
        c->vp[2][i] *= drag;
        xDrag = drag;
    }
    velocity = 0.0;
    if (c->cfg.wall[1] &&
        touches_wall(f0, rad, c->xp[1][i], c->lbb[1], c->tfr[1], &velocity)) {
        c->vp[0][i] *= drag;
        c->vp[1][i] += velocity * xDrag;
        c->vp[2][i] *= drag;
        yDrag = drag;
    }
    velocity = 0.0;
    if (c->cfg.wall[2] &&
        touches_wall(f0, rad, c->xp[2][i], c->lbb[2], c->tfr[2], &velocity)) {
        c->vp[0][i] *= drag;
        c->vp[1][i] *= drag;
        c->vp[2][i] += velocity * xDrag * yDrag;
    }
}

/* correct, src/kernels.cu:487-495 */
static inline double correct1(double ts, double *pp, const double *p,
                              const double *v, const double *vp,
                              const double *old, int i, double *maxErr) {
    const double predicted = pp[i];
    const double corrected = p[i] + 0.5 * ts * (v[i] + vp[i]);
    pp[i] = corrected;
    double e = predicted - corrected;
    e = e < 0 ? -e : e;
    *maxErr = fmax(*maxErr, e);
    return corrected - old[i];
}

/* postIntegrate, src/kernels.cu:339-485 */
static void post_integrate(cbo_ctx *c, double ts) {
    const int n = c->n, dim = c->dim, gas = c->use_gas, flow = c->use_flow,
              path = c->inc_path;
    const int walls = c->cfg.wall[0] || c->cfg.wall[1] || c->cfg.wall[2];
    const int shear = c->cfg.shear_speed != 0.0;
    double *vol = c->tmpd;
    double merr = 0.0, mrad = 0.0, mexp = 0.0;
    int nonfinite = 0;
    /* the mean-field numbers are per step constants */
    const double sA = c->sumA, sAr = c->sumAr, sAo = c->sumAo,
                 sAor = c->sumAor;
#ifdef _OPENMP
#pragma omp parallel for num_threads(c->nthreads) schedule(static) reduction(max : merr, mrad, mexp) reduction(| : nonfinite)
#endif
    for (int i = 0; i < n; i++) {
        if (flow && !shear) add_flow_velocity(c, i);
        if (flow && shear) add_shear_velocity(c, i);
        if (walls) add_wall_velocity(c, i);
        double e = 0.0, temp = 0.0, dist = 0.0;
        temp = correct1(ts, c->xp[0], c->x[0], c->v[0], c->vp[0], c->saved[0], i, &e);
        dist += temp * temp;
        temp = correct1(ts, c->xp[1], c->x[1], c->v[1], c->vp[1], c->saved[1], i, &e);
        dist += temp * temp;
        if (3 == dim) {
            temp = correct1(ts, c->xp[2], c->x[2], c->v[2], c->vp[2], c->saved[2], i, &e);
            dist += temp * temp;
        }
        dist = sqrt(dist);
        vol[i] = 0.0;
        c->del[i] = 0;
        if (gas) {
            double r = c->xp[3][i];
            temp = 2.0 * CBO_PI * r;
            if (dim == 3) temp *= 2.0 * r;
            double vr = (sAr - sAor) / (sA - sAo) - 1.0 / r;
            vr *= c->cfg.kappa * c->cfg.average_surface_area_in * (double)n / sA *
                  (temp - c->ov[i]);
            vr += c->vp[3][i];
            vr *= c->cfg.k_parameter / temp;
            c->vp[3][i] = vr;
            dist += correct1(ts, c->xp[3], c->x[3], c->v[3], c->vp[3], c->saved[3], i, &e);
            r = c->xp[3][i];
            if (r > c->cfg.min_rad) {
                vr = r * r;
                if (3 == dim) vr *= r;
                vol[i] = vr;
            } else {
                c->del[i] = 1;
            }
            mrad = fmax(mrad, r);
            if (!isfinite(r)) nonfinite = 1;
        }
        mexp = fmax(mexp, dist);
        if (path) {
            temp = c->x[0][i] - c->xp[0][i];
            dist = temp * temp;
            temp = c->x[1][i] - c->xp[1][i];
            dist += temp * temp;
            if (dim == 3) {
                temp = c->x[2][i] - c->xp[2][i];
                dist += temp * temp;
            }
            c->pathn[i] = c->path[i] + sqrt(dist);
        }
        c->err[i] = fmax(e, c->err[i]);
        merr = fmax(merr, e);
        for (int a = 0; a < dim; a++)
            if (!isfinite(c->xp[a][i])) nonfinite = 1;
    }
    c->max_err = merr;
    c->max_rad = mrad;
    c->max_exp = mexp;
    c->vol_new = gas ? blocked_sum(vol, n, c->nthreads) : 0.0;
    int nd = 0;
    for (int i = 0; i < n; i++) nd += c->del[i];
    c->ndel = nd;
    if (nonfinite) c->status = CB_ERR_NONFINITE;
}

/* step(), src/simulator.cu:192-249. Returns 1 if the error was too large. */
static int step_once(cbo_ctx *c) {
    const double ts = c->dt;
    c->attempts++;
    pre_integrate(c, ts);
    pairwise(c, c->use_gas, c->use_flow && c->cfg.shear_speed == 0.0);
    post_integrate(c, ts);
    const double tol = c->cfg.error_tolerance;
    const int too_large = c->max_err > tol;
    const int increase = c->max_err < 0.45 * tol && c->dt < 10;
    if (too_large)
        c->dt *= 0.37;
    else if (increase)
        c->dt *= 1.269;
    return too_large;
}

int cbo_attempt(cbo_ctx *c, cb_attempt_view *o) {
    if (!c || !c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    step_once(c);
    if (o) {
        int n = c->n;
        get_row_d(o->xp, c->xp[0], n);
        get_row_d(o->yp, c->xp[1], n);
        get_row_d(o->zp, c->xp[2], n);
        get_row_d(o->rp, c->xp[3], n);
        get_row_d(o->dxdtp, c->vp[0], n);
        get_row_d(o->dydtp, c->vp[1], n);
        get_row_d(o->dzdtp, c->vp[2], n);
        get_row_d(o->drdtp, c->vp[3], n);
        get_row_d(o->error, c->err, n);
        get_row_d(o->path_new, c->pathn, n);
        get_row_d(o->overlap, c->ov, n);
        get_row_i(o->delete_flags, c->del, n);
        o->total_area = c->sumA;
        o->total_area_per_radius = c->sumAr;
        o->total_overlap_area = c->sumAo;
        o->total_overlap_area_per_radius = c->sumAor;
        o->total_volume_new = c->vol_new;
        o->max_error = c->max_err;
        o->max_radius = c->max_rad;
        o->max_expansion = c->max_exp;
        o->num_to_be_deleted = c->use_gas ? c->ndel : 0;
    }
    /* restore rp == r when gas exchange is off */
    if (!c->use_gas) memcpy(c->xp[3], c->x[3], (size_t)c->n * 8);
    if (c->status != CB_OK) return fail(c->status, "non-finite value in step");
    return CB_OK;
}

/* removeBubbles(), src/simulator.cu:180-190 -> swapDataCountPairs and
 * addVolumeFixPairs (src/kernels.cu:775-936), deterministic order. */
static void remove_bubbles(cbo_ctx *c) {
    const int n = c->n, D = c->ndel, nNew = n - D;
    int h = 0, m = 0;
    for (int i = 0; i < nNew; i++)
        if (c->del[i]) c->holes[h++] = i;
    for (int i = n - 1; i >= nNew; i--)
        if (!c->del[i]) c->movers[m++] = i;
    /* h == m: the holes below nNew equal the survivors at or above it */
    for (int i = 0; i < n; i++) c->remap[i] = i;
    for (int k = 0; k < h; k++) {
        const int from = c->movers[k], to = c->holes[k];
        c->remap[from] = to;
        for (int a = 0; a < 4; a++) {
            c->x[a][to] = c->x[a][from];
            c->v[a][to] = c->v[a][from];
            c->vo[a][to] = c->vo[a][from];
            c->saved[a][to] = c->saved[a][from];
        }
        c->path[to] = c->path[from];
        c->err[to] = c->err[from];
        for (int a = 0; a < 3; a++) c->wrap[a][to] = c->wrap[a][from];
        c->index[to] = c->index[from];
        c->nn[to] = c->nn[from];
    }
    /* pairs touching a deleted bubble go; survivors keep their order and
     * endpoints of moved bubbles are remapped */
    int q = 0;
    for (int p = 0; p < c->np; p++) {
        const int i = c->pi[p], j = c->pj[p];
        if (c->del[i] || c->del[j]) continue;
        c->pi[q] = c->remap[i];
        c->pj[q] = c->remap[j];
        q++;
    }
    c->np = q;
    /* volume fix, src/kernels.cu:861-867 and :932-934 */
    double volMul = c->vol_new;
    if (c->dim == 3)
        volMul = 1.0 / cbrt(volMul);
    else
        volMul = 1.0 / sqrt(volMul);
    volMul *= c->vol_mul_const;
    for (int i = 0; i < nNew; i++) c->x[3][i] = c->x[3][i] * volMul;
    c->n = nNew;
    c->deleted += D;
}

/* integrate(), src/simulator.cu:251-337 */
static int integrate_once(cbo_ctx *c) {
    int attempts = 0;
    for (;;) {
        const int too_large = step_once(c);
        attempts++;
        if (c->status != CB_OK) return fail(c->status, "non-finite value in step");
        if (!too_large) break;
        if (attempts >= c->cfg.max_attempts) {
            c->status = CB_ERR_MAX_ATTEMPTS;
            return fail(CB_ERR_MAX_ATTEMPTS, "reject loop exceeded max_attempts");
        }
        if (c->dt < 1e-300) {
            c->status = CB_ERR_DT_UNDERFLOW;
            return fail(CB_ERR_DT_UNDERFLOW, "time step underflow");
        }
    }
    /* buffer rotation */
    for (int a = 0; a < 3; a++) {
        double *t = c->vo[a];
        c->vo[a] = c->v[a];
        c->v[a] = c->vp[a];
        c->vp[a] = t;
        swapp(&c->x[a], &c->xp[a]);
    }
    if (c->use_gas) {
        swapp(&c->x[3], &c->xp[3]);
        double *t = c->vo[3];
        c->vo[3] = c->v[3];
        c->v[3] = c->vp[3];
        c->vp[3] = t;
    }
    if (c->inc_path) swapp(&c->path, &c->pathn);
    c->steps++;
    c->bubble_steps += c->n;
    c->tfrac += c->dt;
    c->tint += (uint64_t)c->tfrac;
    c->tfrac = c->tfrac - (double)(uint64_t)c->tfrac;
    if (c->use_gas) {
        c->max_bubble_radius = c->max_rad;
        if (c->ndel > 0) remove_bubbles(c);
    }
    if (c->max_exp >= 0.5 * c->cfg.skin_radius) {
        int rc = cbo_search_neighbors(c);
        if (rc != CB_OK) return rc;
    } else if (!c->use_gas) {
        /* keep rp == r */
    }
    if (!c->use_gas) memcpy(c->xp[3], c->x[3], (size_t)c->n * 8);
    return CB_OK;
}

int cbo_integrate(cbo_ctx *c, int64_t n_steps, cb_report *rep) {
    if (!c || !c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    int rc = CB_OK;
    for (int64_t s = 0; s < n_steps; s++) {
        rc = integrate_once(c);
        if (rc != CB_OK) break;
    }
    if (rep) cbo_get_report(c, rep);
    return rc;
}

int cbo_get_report(cbo_ctx *c, cb_report *r) {
    if (!c || !r) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    memset(r, 0, sizeof(*r));
    r->steps = c->steps;
    r->attempts = c->attempts;
    r->searches = c->searches;
    r->deleted = c->deleted;
    r->bubble_steps = c->bubble_steps;
    r->time_integer = c->tint;
    r->time_fraction = c->tfrac;
    r->time_step = c->dt;
    r->max_error = c->max_err;
    r->max_radius = c->max_bubble_radius;
    r->max_expansion = c->max_exp;
    r->count = c->n;
    r->num_pairs = c->np;
    r->status = c->status;
    return CB_OK;
}

/* init()'s Euler bootstrap of the AB2 history, src/simulator.cu:727-787 */
int cbo_bootstrap(cbo_ctx *c) {
    if (!c || !c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    const int n = c->n, dim = c->dim;
    const double ts = c->dt;
    for (int a = 0; a < 4; a++) {
        memcpy(c->xp[a], c->x[a], (size_t)n * 8);
        memset(c->vo[a], 0, (size_t)n * 8);
        memset(c->vp[a], 0, (size_t)n * 8);
    }
    memset(c->path, 0, (size_t)n * 8);
    pairwise(c, 0, 0);
    for (int i = 0; i < n; i++) /* euler, src/kernels.cu:959-969 */
        for (int a = 0; a < dim; a++) c->xp[a][i] += c->vp[a][i] * ts;
    for (int a = 0; a < 3; a++) {
        double *t = c->vo[a];
        c->vo[a] = c->vp[a];
        c->vp[a] = t;
    }
    pairwise(c, 0, 0);
    for (int a = 0; a < 3; a++) {
        double *t = c->vo[a];
        c->vo[a] = c->vp[a];
        c->vp[a] = t;
    }
    memcpy(c->xp[3], c->x[3], (size_t)n * 8);
    return CB_OK;
}

/* potentialEnergy, src/kernels.cu:941-957 */
int cbo_bubble_energies(cbo_ctx *c, double *energy, int32_t capacity) {
    if (!c || !energy || capacity < c->n)
        return fail(CB_ERR_INVALID_ARGUMENT, "bad energy buffer");
    memset(energy, 0, (size_t)c->n * 8);
    for (int p = 0; p < c->np; p++) {
        const int i = c->pi[p], j = c->pj[p];
        double d[3];
        wrapped_diff(c, c->x[0][i], c->x[1][i], c->x[2][i], c->x[0][j],
                     c->x[1][j], c->x[2][j], d);
        double e = c->x[3][i] + c->x[3][j] - sqrt(sqlen(d));
        if (e > 0) {
            e *= e;
            energy[i] += e;
            energy[j] += e;
        }
    }
    return CB_OK;
}

int cbo_energy(cbo_ctx *c, double *out) {
    if (!c || !out) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    double *e = (double *)xcalloc((size_t)c->n, 8);
    cbo_bubble_energies(c, e, c->n);
    *out = blocked_sum(e, c->n, c->nthreads);
    free(e);
    return CB_OK;
}

/* calculateVolumes, src/kernels.cu:1013-1024 */
int cbo_total_volume(cbo_ctx *c, double *out) {
    if (!c || !out) return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    for (int i = 0; i < c->n; i++) {
        const double radius = c->x[3][i];
        double volume = radius * radius * CBO_PI;
        if (c->dim == 3) volume *= radius * 1.33333333333333333333333333;
        c->tmpd[i] = volume;
    }
    *out = blocked_sum(c->tmpd, c->n, c->nthreads);
    return CB_OK;
}
