// qr_probe.cu -- measurement kernels for the benchmark (libqrusty_probe.so),
// not part of the product ABI.
//
// qr_probe_fp64_peak: the FP64 fused multiply-add rate of this GPU, the
// ceiling of the complex128 kernels (4 DFMA per complex multiply-add).  Every
// thread runs kChains independent DFMA chains for `iters` steps (enough
// chains per warp, and warps per SM, to keep the FP64 pipe busy); the grid
// is 8 CTAs of 256 threads per SM.  The result of every chain is stored, so
// no chain can be dropped.  Timed with CUDA events around the launch.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) dfma_chains(int iters, double a, double b,
                                                        double *out) {
    double x[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = (double)(threadIdx.x + k) * 1e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += x[k];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int qr_probe_fp64_peak(int iters, double *tflops, float *ms_out) {
    if (iters < 1 || !tflops || !ms_out) return -1;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -2;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -2;
    const int grid = nsm * 8;
    double *out = nullptr;
    if (cudaMalloc(&out, (size_t)grid * kThreads * sizeof(double)) != cudaSuccess) return -3;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // a = 1 - 2^-30, b = 2^-40: the chains neither overflow nor settle to a
    // value the compiler could know
    const double a = 1.0 - 9.313225746154785e-10, b = 9.094947017729282e-13;
    dfma_chains<<<grid, kThreads>>>(iters / 10 + 1, a, b, out);  // warm-up
    cudaEventRecord(e0);
    dfma_chains<<<grid, kThreads>>>(iters, a, b, out);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return -4;
    *ms_out = ms;
    *tflops = 2.0 * (double)grid * kThreads * kChains * (double)iters / (ms * 1e-3) / 1e12;
    return 0;
}
