// fp64_probe.cu -- measures the GPU's FP64 FMA issue rate, the roofline denominator of the
// chemistry kernels (which are bound by FP64 throughput, not by HBM).
#include <cuda_runtime.h>

#include "../../include/gdtk_chem.h"
#include "fast_exp.h"

namespace {

// Eight independent DFMA chains per thread; 2 FLOP per DFMA.
__global__ void dfma_loop(double* out, int iters, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
            x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void div_pairs(int n, const double* a, const double* b, double* q_fast, double* q_nr, double* q_ieee) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    q_fast[i] = gdtk::gdtk_div(a[i], b[i]);
    q_nr[i] = gdtk::gdtk_div_nr(a[i], b[i]);
    q_ieee[i] = a[i] / b[i];
}

}  // namespace

extern "C" int gdtk_div_device(int n, const double* a, const double* b, double* q_fast, double* q_nr,
                               double* q_ieee) {
    if (n < 0 || (n > 0 && (!a || !b || !q_fast || !q_nr || !q_ieee))) return -1;
    if (n == 0) return 0;
    div_pairs<<<(n + 255) / 256, 256>>>(n, a, b, q_fast, q_nr, q_ieee);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1;
}

extern "C" int gdtk_measure_fp64_peak(double* tflops) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    const int block = 256, grid = sms * 4, iters = 1000;
    double* buf = nullptr;
    if (cudaMalloc(&buf, (size_t)grid * block * sizeof(double)) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    dfma_loop<<<grid, block>>>(buf, 10, 0.999, 1e-3);   // warm-up
    cudaEventRecord(e0);
    dfma_loop<<<grid, block>>>(buf, iters, 0.999, 1e-3);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess || ms <= 0.f) return -1;
    const double flops = 2.0 * 8 * 16 * (double)iters * grid * block;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return 0;
}
