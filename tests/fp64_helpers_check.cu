// Test harness: evaluates the FP64 helpers of the step kernels (rcp_hn,
// rsqrt_hn, and rcp_d / rsqrt_d with their float-float estimates, min_image)
// next to CUDA's IEEE division and rsqrt() on the same inputs. Built by
// tests/test_gpu_math.py.
#include "../cubble_gb300/csrc/common.cuh"

__global__ void k_check(const double *in, int n, double *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double a = in[i];
        out[8 * i + 0] = cbg::rcp_hn(a);
        out[8 * i + 1] = 1.0 / a;
        out[8 * i + 2] = cbg::rsqrt_hn(a);
        out[8 * i + 3] = rsqrt(a);
        out[8 * i + 4] = cbg::rcp_d(a);
        out[8 * i + 5] = cbg::rsqrt_d(a);
        out[8 * i + 6] = cbg::min_image(a - 50.0, 40.0, 80.0);
        const double d = a - 50.0, t = 80.0 - fabs(d);
        out[8 * i + 7] = t * t < d * d ? t * (d < 0 ? 1.0 : -1.0) : d;
    }
}

extern "C" int fp64_check(const double *host_in, int n, double *host_out) {
    double *din = nullptr, *dout = nullptr;
    if (cudaMalloc(&din, n * sizeof(double)) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, 8 * n * sizeof(double)) != cudaSuccess) return 1;
    cudaMemcpy(din, host_in, n * sizeof(double), cudaMemcpyHostToDevice);
    k_check<<<256, 256>>>(din, n, dout);
    cudaError_t e = cudaMemcpy(host_out, dout, 8 * n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : 2;
}

// The float-float helpers of the FP64 pair kernel (ff.cuh) on the device,
// where the FP32 estimates come from the hardware approximations: split and
// back, reciprocal, rsqrt and sqrt, each rounded back to double.
__global__ void k_ff_check(const double *in, int n, double *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const cbg::ff a = cbg::ff_of(in[i]);
        out[4 * i + 0] = cbg::ff_to_double(cbg::fast_two_sum(a.h, a.l));
        out[4 * i + 1] = cbg::ff_to_double(cbg::ff_rcp(a));
        out[4 * i + 2] = cbg::ff_to_double(cbg::ff_rsqrt(a));
        out[4 * i + 3] = cbg::ff_to_double(cbg::ff_sqrt(a));
    }
}

extern "C" int ff_check(const double *host_in, int n, double *host_out) {
    double *din = nullptr, *dout = nullptr;
    if (cudaMalloc(&din, n * sizeof(double)) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, 4 * n * sizeof(double)) != cudaSuccess) return 1;
    cudaMemcpy(din, host_in, n * sizeof(double), cudaMemcpyHostToDevice);
    k_ff_check<<<256, 256>>>(din, n, dout);
    cudaError_t e = cudaMemcpy(host_out, dout, 4 * n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(din);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : 2;
}

// The exact subtraction of the FP64 pair kernel (ff.cuh sub_exact) next to
// the FP64 subtraction on the same operand pairs.
__global__ void k_sub_check(const double *a, const double *b, int n, double *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        out[2 * i + 0] = cbg::sub_exact(a[i], b[i]);
        out[2 * i + 1] = __dsub_rn(a[i], b[i]);
    }
}

extern "C" int sub_check(const double *ha, const double *hb, int n, double *host_out) {
    double *da = nullptr, *db = nullptr, *dout = nullptr;
    if (cudaMalloc(&da, n * sizeof(double)) != cudaSuccess) return 1;
    if (cudaMalloc(&db, n * sizeof(double)) != cudaSuccess) return 1;
    if (cudaMalloc(&dout, 2 * n * sizeof(double)) != cudaSuccess) return 1;
    cudaMemcpy(da, ha, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(db, hb, n * sizeof(double), cudaMemcpyHostToDevice);
    k_sub_check<<<256, 256>>>(da, db, n, dout);
    cudaError_t e = cudaMemcpy(host_out, dout, 2 * n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(da);
    cudaFree(db);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : 2;
}
