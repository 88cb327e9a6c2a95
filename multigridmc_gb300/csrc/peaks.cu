// peaks.cu -- measured FMA throughput of the current GPU in FP64 and FP32.
//
// The roofline of a kernel that does a few floating-point operations per
// byte depends on which limit it meets first: HBM bandwidth or the FMA pipe
// of its precision.  GB300 has few FP64 units per SM, so an FP64 stencil
// sweep can be bound by FP64 issue rather than by memory; this entry point
// measures the rate it is bound by, on the GPU it runs on, with CUDA events.
// It changes no clock or other setting of the GPU.
#include <algorithm>
#include <string>

#include <cuda_runtime.h>

#include "../../include/mgmc_gb300.h"

namespace mgmc {
void set_last_error(const std::string &msg);  // api.cu
}

namespace {

constexpr int kChains = 8;   // independent FMA chains per thread (covers the pipe latency)
constexpr int kUnroll = 16;  // FMAs per chain per loop iteration

__device__ __forceinline__ float fma_step(float v, float a, float b) { return __fmaf_rn(v, a, b); }
__device__ __forceinline__ double fma_step(double v, double a, double b) { return __fma_rn(v, a, b); }

// Every thread runs kChains independent chains v <- v a + b for
// iters * kUnroll steps; the sum of the chains is stored only when it equals
// an impossible value, which keeps every FMA live without memory traffic.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_rate(T *__restrict__ out, int iters, T a, T b) {
    T v[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) v[i] = T(threadIdx.x + i) * T(1e-3);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int i = 0; i < kChains; ++i) v[i] = fma_step(v[i], a, b);
    }
    T s = T(0);
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += v[i];
    if (s == T(-1.25e30)) out[blockIdx.x] = s;
}

template <typename T>
double fma_tflops(cudaStream_t st, int nblock, T *out) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const T a = T(0.999), b = T(1e-3);
    // size the run to about 20 ms from a short probe
    int iters = 16;
    float ms = 0.f;
    for (int attempt = 0; attempt < 8; ++attempt) {
        cudaEventRecord(e0, st);
        k_fma_rate<T><<<nblock, 256, 0, st>>>(out, iters, a, b);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms >= 10.f) break;
        const double scale = ms > 0.05f ? 20.0 / ms : 64.0;
        iters = (int)std::min<double>(iters * scale, 1 << 24);
    }
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, st);
        k_fma_rate<T><<<nblock, 256, 0, st>>>(out, iters, a, b);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flop = 2.0 * (double)nblock * 256.0 * (double)iters * kUnroll * kChains;
    return flop / (best * 1e-3) / 1e12;
}

}  // namespace

extern "C" mgmc_status mgmc_device_fma_rate(int precision, double *tflops) {
    if (!tflops || (precision != MGMC_FP64 && precision != MGMC_FP32_MIXED)) {
        mgmc::set_last_error("mgmc_device_fma_rate: precision must be MGMC_FP64 or MGMC_FP32_MIXED");
        return MGMC_ERR_INVALID_ARGUMENT;
    }
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t st = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    void *out = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&out, (size_t)nsm * 8 * sizeof(double));
    if (e == cudaSuccess) {
        const int nblock = nsm * 8;  // 8 CTAs of 256 threads per SM: 64 warps, full occupancy
        *tflops = precision == MGMC_FP64 ? fma_tflops<double>(st, nblock, static_cast<double *>(out))
                                         : fma_tflops<float>(st, nblock, static_cast<float *>(out));
        e = cudaGetLastError();
    }
    if (out) cudaFree(out);
    if (st) cudaStreamDestroy(st);
    if (e != cudaSuccess) {
        mgmc::set_last_error(std::string("mgmc_device_fma_rate: ") + cudaGetErrorString(e));
        return MGMC_ERR_CUDA;
    }
    return MGMC_OK;
}
