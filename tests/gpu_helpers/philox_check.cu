// Test helper (built by tests/test_gpu_stats.py): evaluates the library's
// Philox4x32-10 and Box-Muller device functions next to cuRAND's
// curand_Philox4x32_10 on the same counters and keys.
#include <curand_philox4x32_x.h>

#include "../../multigridmc_gb300/csrc/kernels.cuh"

__global__ void k_check(const uint4 *ctr, const uint2 *key, uint4 *mine, uint4 *ref, float4 *nrm, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint4 a = mgmc::philox4x32_10(ctr[i], key[i]);
    mine[i] = a;
    ref[i] = curand_Philox4x32_10(ctr[i], key[i]);
    nrm[i] = mgmc::normals4(a);
}

extern "C" int philox_check(const unsigned *ctr, const unsigned *key, unsigned *mine, unsigned *ref, float *nrm, int n) {
    uint4 *dc, *dm, *dr;
    uint2 *dk;
    float4 *dn;
    if (cudaMalloc(&dc, n * sizeof(uint4)) || cudaMalloc(&dk, n * sizeof(uint2)) || cudaMalloc(&dm, n * sizeof(uint4)) ||
        cudaMalloc(&dr, n * sizeof(uint4)) || cudaMalloc(&dn, n * sizeof(float4)))
        return 1;
    cudaMemcpy(dc, ctr, n * sizeof(uint4), cudaMemcpyHostToDevice);
    cudaMemcpy(dk, key, n * sizeof(uint2), cudaMemcpyHostToDevice);
    k_check<<<(n + 255) / 256, 256>>>(dc, dk, dm, dr, dn, n);
    cudaMemcpy(mine, dm, n * sizeof(uint4), cudaMemcpyDeviceToHost);
    cudaMemcpy(ref, dr, n * sizeof(uint4), cudaMemcpyDeviceToHost);
    cudaMemcpy(nrm, dn, n * sizeof(float4), cudaMemcpyDeviceToHost);
    int err = cudaGetLastError() != cudaSuccess;
    cudaFree(dc); cudaFree(dk); cudaFree(dm); cudaFree(dr); cudaFree(dn);
    return err;
}
