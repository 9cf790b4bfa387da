// Entry points of the drop-in driver around the step (init()'s lattice and
// box rescale, simulate()'s averages): small kernels that run a few times
// per simulation, not per step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.cuh"

using namespace cbg;

namespace {

// transformPositions, src/kernels.cu:971-990.
__global__ void __launch_bounds__(kBlock) k_transform(Bufs b, int normalize) {
    const Ctrl *c = b.ctrl;
    const DevConst &k = *b.k;
    const int n = c->n;
    double *X = drow(b, c, RX), *Y = drow(b, c, RY), *Z = drow(b, c, RZ);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (normalize) {
            X[i] = (X[i] - k.lbb[0]) / k.iv[0];
            Y[i] = (Y[i] - k.lbb[1]) / k.iv[1];
            if (k.dim == 3) Z[i] = (Z[i] - k.lbb[2]) / k.iv[2];
        } else {
            X[i] = k.iv[0] * X[i] + k.lbb[0];
            Y[i] = k.iv[1] * Y[i] + k.lbb[1];
            if (k.dim == 3) Z[i] = k.iv[2] * Z[i] + k.lbb[2];
        }
    }
}

// Sums of r, the four rates and path (last block folds in block order).
__global__ void __launch_bounds__(kBlock) k_averages(Bufs b) {
    __shared__ double smem[32];
    Ctrl *c = b.ctrl;
    const int n = c->n;
    const bool f32 = b.k->mixed;
    const int roles[6] = {RR, RV0, RV1, RV2, RV3, RPATH};
    for (int q = 0; q < 6; q++) {
        const double *row = drow(b, c, roles[q]);
        const bool rate = q >= 1 && q <= 4;
        double s = 0.0;
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            s += (f32 && rate) ? (double)reinterpret_cast<const float *>(row)[i] : row[i];
        s = block_reduce(s, OpSum(), smem);
        if (threadIdx.x == 0) b.part[q * gridDim.x + blockIdx.x] = s;
    }
    if (last_block(&c->done[DC_MISC], gridDim.x)) {
        for (int q = 0; q < 6; q++) {
            const double t = fold_partials(b.part + q * gridDim.x, gridDim.x, false, smem);
            if (threadIdx.x == 0) b.energy[q] = t;
        }
        if (threadIdx.x == 0) c->done[DC_MISC] = 0;
    }
}

// assignDataToBubbles, src/kernels.cu:1026-1071: lattice point of bubble i
// plus a random offset of length avg_rad * w in the direction of (ux, uy,
// uz); |r| lifted by minRad when below it; w := initial area / count.
__global__ void __launch_bounds__(kBlock) k_assign(const DevConst *kp, int3 bpd, double avg_rad,
                                                  double *x, double *y, double *z, double *w,
                                                  double *r, int *index, int count) {
    const DevConst &k = *kp;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        index[i] = i;
        double px = (i % bpd.x) / (double)bpd.x;
        double py = ((i / bpd.x) % bpd.y) / (double)bpd.y;
        double pz = 0.0;
        double ox = x[i], oy = y[i], oz = 0.0;
        if (k.dim == 3) {
            oz = z[i];
            pz = (i / (bpd.x * bpd.y)) / (double)bpd.z;
        }
        px *= k.iv[0];
        py *= k.iv[1];
        pz *= k.iv[2];
        double len2 = 0.0;
        len2 += ox * ox;
        len2 += oy * oy;
        len2 += oz * oz;
        const double len = sqrt(len2);
        ox = ox / len * avg_rad * w[i];
        oy = oy / len * avg_rad * w[i];
        oz = oz / len * avg_rad * w[i];
        px += ox;
        py += oy;
        pz += oz;
        double rad = fabs(r[i]);
        rad = rad > k.min_rad ? rad : rad + k.min_rad;
        r[i] = rad;
        x[i] = px > k.lbb[0] ? (px < k.tfr[0] ? px : px - k.iv[0]) : px + k.iv[0];
        y[i] = py > k.lbb[1] ? (py < k.tfr[1] ? py : py - k.iv[1]) : py + k.iv[1];
        z[i] = pz > k.lbb[2] ? (pz < k.tfr[2] ? pz : pz - k.iv[2]) : pz + k.iv[2];
        double area = 2.0 * kPi * rad;
        if (k.dim == 3) area *= 2.0 * rad;
        w[i] = area / count;
    }
}

}  // namespace

#define CB_ENTER(c)                                                          \
    do {                                                                     \
        if (!(c)) return fail(CB_ERR_INVALID_ARGUMENT, "null context");      \
        cbg::note_call();                                                    \
        CB_CUDA(cudaSetDevice((c)->dev));                                    \
    } while (0)

extern "C" {

int cb_transform_positions(cb_context *c, int32_t normalize) {
    CB_ENTER(c);
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    int rc0 = invalidate_prediction(c);
    if (rc0) return rc0;
    k_transform<<<c->launch.grid, kBlock, 0, c->stream>>>(c->bufs, normalize ? 1 : 0);
    c->launches += 1;
    CB_CUDA(cudaGetLastError());
    CB_CUDA(cudaStreamSynchronize(c->stream));
    return CB_OK;
}

int cb_averages(cb_context *c, double means[6]) {
    CB_ENTER(c);
    if (!means) return fail(CB_ERR_INVALID_ARGUMENT, "null output");
    if (!c->loaded) return fail(CB_ERR_STATE, "state not loaded");
    int rc = c->pull();
    if (rc) return rc;
    const int n = c->hctrl->n;
    k_averages<<<c->launch.grid, kBlock, 0, c->stream>>>(c->bufs);
    c->launches += 1;
    CB_CUDA(cudaGetLastError());
    double sums[6];
    CB_CUDA(cudaMemcpyAsync(sums, c->bufs.energy, sizeof(sums), cudaMemcpyDeviceToHost,
                            c->stream));
    CB_CUDA(cudaStreamSynchronize(c->stream));
    for (int q = 0; q < 6; q++) means[q] = n > 0 ? sums[q] / n : 0.0;
    return CB_OK;
}

int cb_reset_rows(cb_context *c, int32_t which) {
    CB_ENTER(c);
    int rc = c->pull();
    if (rc) return rc;
    Ctrl &h = *c->hctrl;
    const size_t cap = (size_t)c->hk.cap;
    if (which & CB_RESET_ERROR)
        CB_CUDA(cudaMemsetAsync(c->dslot[h.drole[RERR]], 0, cap * 8, c->stream));
    if (which & CB_RESET_WRAP) {
        CB_CUDA(cudaMemsetAsync(c->islot[h.irole[IWX]], 0, cap * 4, c->stream));
        CB_CUDA(cudaMemsetAsync(c->islot[h.irole[IWY]], 0, cap * 4, c->stream));
        CB_CUDA(cudaMemsetAsync(c->islot[h.irole[IWZ]], 0, cap * 4, c->stream));
    }
    if (which & CB_RESET_DT_STATS) {
        h.dt_min = 9999999.9;  // simulate()'s starting values, src/simulator.cu:979-981
        h.dt_max = -1.0;
        h.dt_sum = 0.0;
        return c->push();
    }
    CB_CUDA(cudaStreamSynchronize(c->stream));
    return CB_OK;
}

int cb_set_average_area(cb_context *c, double ain) {
    CB_ENTER(c);
    c->cfg.average_surface_area_in = ain;
    c->hk.ain = ain;
    return c->upload_const();
}

int cb_assign_lattice(cb_context *c, const int32_t bpd[3], double avg_rad, const double *ux,
                      const double *uy, const double *uz, const double *uw, const double *nr,
                      int32_t count, double *avg_area, double *max_radius) {
    CB_ENTER(c);
    if (!bpd || !ux || !uy || !uw || !nr || (c->hk.dim == 3 && !uz))
        return fail(CB_ERR_INVALID_ARGUMENT, "null argument");
    if (count < 1 || count > c->hk.cap) return fail(CB_ERR_CAPACITY, "count exceeds capacity");
    const long long lattice = (long long)bpd[0] * bpd[1] * (c->hk.dim == 3 ? bpd[2] : 1);
    if (bpd[0] < 1 || bpd[1] < 1 || (c->hk.dim == 3 && bpd[2] < 1) || lattice < count)
        return fail(CB_ERR_INVALID_ARGUMENT, "lattice smaller than the bubble count");
    const size_t n = (size_t)count;
    double *d = nullptr;
    int *di = nullptr;
    CB_CUDA(cudaMalloc(&d, 5 * n * sizeof(double)));
    if (cudaMalloc(&di, n * sizeof(int)) != cudaSuccess) {
        cudaFree(d);
        return fail(CB_ERR_CUDA, "cudaMalloc");
    }
    double *x = d, *y = d + n, *z = d + 2 * n, *w = d + 3 * n, *r = d + 4 * n;
    std::vector<double> hx(n), hy(n), hz(n, 0.0), hw(n), hr(n);
    std::vector<int32_t> hi(n);
    int rc = CB_OK;
    auto run = [&]() -> int {
        CB_CUDA(cudaMemcpyAsync(x, ux, n * 8, cudaMemcpyHostToDevice, c->stream));
        CB_CUDA(cudaMemcpyAsync(y, uy, n * 8, cudaMemcpyHostToDevice, c->stream));
        if (c->hk.dim == 3)
            CB_CUDA(cudaMemcpyAsync(z, uz, n * 8, cudaMemcpyHostToDevice, c->stream));
        else
            CB_CUDA(cudaMemsetAsync(z, 0, n * 8, c->stream));
        CB_CUDA(cudaMemcpyAsync(w, uw, n * 8, cudaMemcpyHostToDevice, c->stream));
        CB_CUDA(cudaMemcpyAsync(r, nr, n * 8, cudaMemcpyHostToDevice, c->stream));
        k_assign<<<c->launch.grid, kBlock, 0, c->stream>>>(
            c->dk, make_int3(bpd[0], bpd[1], c->hk.dim == 3 ? bpd[2] : 1), avg_rad, x, y, z, w,
            r, di, count);
        c->launches += 1;
        CB_CUDA(cudaGetLastError());
        CB_CUDA(cudaMemcpyAsync(hx.data(), x, n * 8, cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaMemcpyAsync(hy.data(), y, n * 8, cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaMemcpyAsync(hz.data(), z, n * 8, cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaMemcpyAsync(hw.data(), w, n * 8, cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaMemcpyAsync(hr.data(), r, n * 8, cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaMemcpyAsync(hi.data(), di, n * 4, cudaMemcpyDeviceToHost, c->stream));
        CB_CUDA(cudaStreamSynchronize(c->stream));
        return CB_OK;
    };
    rc = run();
    cudaFree(d);
    cudaFree(di);
    if (rc) return rc;
    double area = 0.0, mr = 0.0;
    for (size_t i = 0; i < n; i++) {
        area += hw[i];
        mr = std::max(mr, hr[i]);
    }
    cb_state_view v;
    std::memset(&v, 0, sizeof(v));
    v.count = count;
    v.x = hx.data();
    v.y = hy.data();
    v.z = hz.data();
    v.r = hr.data();
    v.index = hi.data();
    rc = cb_load_state(c, &v);
    if (rc) return rc;
    if (avg_area) *avg_area = area;
    if (max_radius) *max_radius = mr;
    return CB_OK;
}

}  // extern "C"
