/* Device-rate probe behind sh_probe_fp64_fma_rate: the issue rate of
 * dependent FP64 fused multiply-adds on this GPU, the denominator of the
 * FP64 roofline that the stage kernels are reported against (GB300 issues
 * far fewer FP64 than FP32 instructions per clock, so the plain FP64 path is
 * bound there before it reaches HBM bandwidth). */
#include <cuda_runtime.h>

#include "sledgehamr_gb300.h"

namespace {

constexpr int kChains = 8;   /* independent FMA chains per thread */
constexpr int kThreads = 256;

/* kChains chains of `iters` dependent FMAs per thread; a and b keep the
 * values bounded (|x| stays below 2 for |a| < 1/2, |b| < 1). */
__global__ void __launch_bounds__(kThreads) fp64_fma_chain_kernel(double *out, int iters,
                                                                  double a, double b) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 0.001 * (threadIdx.x + c);
    for (int q = 0; q < iters; ++q) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace

extern "C" int sh_probe_fp64_fma_rate(int device, double *fma_per_s) {
    if (!fma_per_s) return SH_ERR_ARG;
    *fma_per_s = 0.;
    if (cudaSetDevice(device) != cudaSuccess) return SH_ERR_CUDA;
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return SH_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp64_fma_chain_kernel, kThreads,
                                                      0) != cudaSuccess)
        return SH_ERR_CUDA;
    const int blocks = sms * per_sm;
    const int iters = 4096;
    double *out = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = SH_OK;
    if (cudaMalloc(&out, (size_t)blocks * kThreads * sizeof(double)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = SH_ERR_CUDA;
    } else {
        /* one warm-up launch, then the best of five timed launches */
        fp64_fma_chain_kernel<<<blocks, kThreads, 0, s>>>(out, iters, 0.4999, 0.25);
        float best = 0.f;
        for (int t = 0; t < 5 && rc == SH_OK; ++t) {
            cudaEventRecord(e0, s);
            fp64_fma_chain_kernel<<<blocks, kThreads, 0, s>>>(out, iters, 0.4999, 0.25);
            cudaEventRecord(e1, s);
            float ms = 0.f;
            if (cudaEventSynchronize(e1) != cudaSuccess ||
                cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                rc = SH_ERR_CUDA;
            else if (best == 0.f || ms < best)
                best = ms;
        }
        if (rc == SH_OK && best > 0.f)
            *fma_per_s = (double)blocks * kThreads * kChains * iters / (best * 1e-3);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    if (out) cudaFree(out);
    return rc;
}
