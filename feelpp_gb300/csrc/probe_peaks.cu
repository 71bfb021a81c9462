// Arithmetic-throughput probe used for the roofline denominators that the pool's
// measured peaks do not cover: FP64 FMA, FP32 FMA and f64<->f32 conversions.
// Grid 152*8 blocks x 256 threads; each thread writes one value (out sized accordingly).
// Built by feelpp_gb300/build.py as _lib/probe_peaks; prints one line per rate.
#include <cstdio>
#include <cuda_runtime.h>
#define ITERS 2048
template <typename T>
__global__ void fma_kernel(T* out, T a, T b) {
    T x0 = threadIdx.x * (T)1e-7, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3, x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < ITERS; ++i) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
__global__ void cvt_d2f_kernel(float* out, double a) {
    double d0 = threadIdx.x * 1e-7, d1 = d0 + 1, d2 = d0 + 2, d3 = d0 + 3;
    float s = 0.f;
    for (int i = 0; i < ITERS; ++i) {
        s += (float)d0 + (float)d1 + (float)d2 + (float)d3;
        d0 += a; d1 += a; d2 += a; d3 += a;  // 4 FP64 adds per 4 conversions
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void cvt_f2d_kernel(double* out, float a) {
    float f0 = threadIdx.x * 1e-7f, f1 = f0 + 1, f2 = f0 + 2, f3 = f0 + 3;
    double s0 = 0, s1 = 0;
    for (int i = 0; i < ITERS; ++i) {
        s0 += (double)f0; s1 += (double)f1; s0 += (double)f2; s1 += (double)f3;
        f0 += a; f1 += a; f2 += a; f3 += a;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = s0 + s1;
}
int main() {
    int blocks = 152 * 8, threads = 256;
    size_t n = (size_t)blocks * threads;
    double* dd; float* df;
    cudaMalloc(&dd, n * sizeof(double)); cudaMalloc(&df, n * sizeof(float));
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    float ms;
    for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(e0); fma_kernel<double><<<blocks, threads>>>(dd, 0.999999, 1e-9); cudaEventRecord(e1); cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) printf("fp64 fma: %.3f ms  %.2f TFLOP/s\n", ms, 2.0 * 8 * ITERS * n / (ms * 1e-3) / 1e12);
        cudaEventRecord(e0); fma_kernel<float><<<blocks, threads>>>(df, 0.999999f, 1e-9f); cudaEventRecord(e1); cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) printf("fp32 fma: %.3f ms  %.2f TFLOP/s\n", ms, 2.0 * 8 * ITERS * n / (ms * 1e-3) / 1e12);
        cudaEventRecord(e0); cvt_d2f_kernel<<<blocks, threads>>>(df, 1e-9); cudaEventRecord(e1); cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) printf("d2f cvt (+1 dadd each): %.3f ms  %.2f Gcvt/s\n", ms, 4.0 * ITERS * n / (ms * 1e-3) / 1e9);
        cudaEventRecord(e0); cvt_f2d_kernel<<<blocks, threads>>>(dd, 1e-9f); cudaEventRecord(e1); cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) printf("f2d cvt (+1 dadd each): %.3f ms  %.2f Gcvt/s\n", ms, 4.0 * ITERS * n / (ms * 1e-3) / 1e9);
    }
    cudaError_t e = cudaDeviceSynchronize();
    printf("status: %s\n", cudaGetErrorString(e));
    return e == cudaSuccess ? 0 : 1;
}
