// noalloc.cu -- y = A x for the measured operator A = A_0 + B Sigma^{-1} B^T
// without allocating any device memory.
//
// Some callers cannot call cudaMalloc: a step that is being captured into a
// CUDA graph in global capture mode (allocation is not permitted while the
// stream captures), an application whose device memory is entirely owned by
// its own pool or arena and hands the library only the buffers it should
// touch, or a latency-critical loop where cudaMalloc's implicit device-wide
// synchronisation would stall other streams.  mgmc_measured_apply_noalloc
// serves them: the caller passes every input and output, and the only
// scratch -- the m-vector B^T x -- lives in the file-scope device array
// below, whose size is fixed when the library is loaded.
//
// Sharing rules: every call on a device uses the same array and leaves the
// last call's B^T x in it.  Calls whose kernels overlap on the GPU (for
// example issued on two streams without ordering between them) race on it;
// order them on one stream or with events.
#include <cstdio>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/mgmc_gb300.h"

namespace mgmc {
void set_last_error(const std::string &msg);  // api.cu
}

namespace {

// B^T x of the most recent call, one entry per measurement column.  Every
// GPU that loads the library holds these MGMC_NOALLOC_MAX_M doubles (32 KiB)
// until the process exits.
static __device__ __align__(256) double g_noalloc_btx[MGMC_NOALLOC_MAX_M];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_btx_addr[kMaxDevices] = {};  // device address of g_noalloc_btx, per device

struct Stencil27 {
    double w[27];
};

// y = A_0 x in the compact (reference) vertex order; neighbours outside the
// interior are omitted (homogeneous Dirichlet), terms summed in ascending
// index order as in the sparse rows of the reference.
__global__ void k_noalloc_stencil(const double *__restrict__ x, double *__restrict__ y, int N0, int N1, int N2,
                                  Stencil27 st) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y, c = blockIdx.z;
    if (a >= N0) return;
    double acc = 0.0;
    for (int dz = -1; dz <= 1; ++dz) {
        const int cc = c + dz;
        if (cc < 0 || cc >= N2) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int bb = b + dy;
            if (bb < 0 || bb >= N1) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int aa = a + dx;
                const double w = st.w[(dz + 1) * 9 + (dy + 1) * 3 + (dx + 1)];
                if (aa < 0 || aa >= N0 || w == 0.0) continue;
                acc += w * x[((long long)cc * N1 + bb) * N0 + aa];
            }
        }
    }
    y[((long long)c * N1 + b) * N0 + a] = acc;
}

// btx[j] = sum_i B_ij x_i, one block per column (every entry of btx[0..m)
// is written, so nothing has to start at zero).
__global__ void __launch_bounds__(256) k_noalloc_btx(const double *__restrict__ x, const int64_t *__restrict__ ptr,
                                                     const int64_t *__restrict__ idx, const double *__restrict__ val,
                                                     double *__restrict__ btx) {
    __shared__ double sh[8];
    const int j = blockIdx.x;
    double acc = 0.0;
    for (int64_t e = ptr[j] + threadIdx.x; e < ptr[j + 1]; e += blockDim.x) acc += val[e] * x[idx[e]];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += sh[w];
        btx[j] = t;
    }
}

// y += B (Sigma^{-1} btx): columns may share rows, so the adds are atomic,
// and the order in which the columns' terms reach a row depends on block
// timing -- the last bits of y may differ from run to run (mgmc_level_apply
// sums in a fixed order).
__global__ void __launch_bounds__(256) k_noalloc_add_B(double *__restrict__ y, const int64_t *__restrict__ ptr,
                                                       const int64_t *__restrict__ idx, const double *__restrict__ val,
                                                       const double *__restrict__ Sigma, const double *__restrict__ btx) {
    const int j = blockIdx.x;
    const double q = btx[j] / Sigma[j];
    for (int64_t e = ptr[j] + threadIdx.x; e < ptr[j + 1]; e += blockDim.x) atomicAdd(&y[idx[e]], val[e] * q);
}

mgmc_status fail(mgmc_status st, const std::string &msg) {
    mgmc::set_last_error(msg);
    return st;
}

}  // namespace

extern "C" mgmc_status mgmc_measured_apply_noalloc(int dim, int nx, int ny, int nz, const double stencil[27], int m,
                                                   const int64_t *B_colptr, const int64_t *B_rowidx,
                                                   const double *B_val, const double *Sigma, const double *x,
                                                   double *y, void *cuda_stream) {
    if (dim < 1 || dim > 3 || !stencil || !x || !y) return fail(MGMC_ERR_INVALID_ARGUMENT, "bad arguments");
    if (m < 0 || (m > 0 && (!B_colptr || !B_rowidx || !B_val || !Sigma)))
        return fail(MGMC_ERR_INVALID_ARGUMENT, "m > 0 needs B_colptr, B_rowidx, B_val and Sigma");
    if (m > MGMC_NOALLOC_MAX_M)
        return fail(MGMC_ERR_INVALID_ARGUMENT, "m = " + std::to_string(m) + " exceeds the no-allocation limit of " +
                                                   std::to_string(MGMC_NOALLOC_MAX_M) + " measurement columns");
    int cells[3] = {nx, dim > 1 ? ny : 2, dim > 2 ? nz : 2};
    for (int d = 0; d < 3; ++d)
        if (cells[d] < 2 || cells[d] - 1 > 65535) return fail(MGMC_ERR_LATTICE, "lattice extent out of range");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(MGMC_ERR_CUDA, "no current CUDA device");
    // Set-up, once per device with that device current: the device address
    // of the scratch array.  The first call on a device does this; make that
    // first call before any stream capture.
    double *btx = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_btx_addr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_btx);
            if (e != cudaSuccess)
                return fail(MGMC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            // Load all three kernels now, whatever m is: with lazy module
            // loading a kernel is otherwise loaded at its first launch, which
            // may come inside a later captured call (a first call with m = 0
            // never launches the two low-rank kernels).
            cudaFuncAttributes fa;
            const void *kernels[3] = {reinterpret_cast<const void *>(k_noalloc_stencil),
                                      reinterpret_cast<const void *>(k_noalloc_btx),
                                      reinterpret_cast<const void *>(k_noalloc_add_B)};
            for (const void *k : kernels) {
                e = cudaFuncGetAttributes(&fa, k);
                if (e != cudaSuccess)
                    return fail(MGMC_ERR_CUDA, std::string("cudaFuncGetAttributes: ") + cudaGetErrorString(e));
            }
            g_btx_addr[dev] = static_cast<double *>(p);
        }
        btx = g_btx_addr[dev];
    }
    // An error left by earlier work on this thread is reported, not cleared:
    // it is not this call's, and clearing it would hide it from its owner.
    e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return fail(MGMC_ERR_CUDA, std::string("a CUDA error from earlier work is pending (left in place): ") +
                                       cudaGetErrorString(e));
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    Stencil27 w;
    for (int k = 0; k < 27; ++k) w.w[k] = stencil[k];
    const int N0 = cells[0] - 1, N1 = cells[1] - 1, N2 = cells[2] - 1;
    dim3 grid((N0 + 127) / 128, N1, N2);
    k_noalloc_stencil<<<grid, 128, 0, st>>>(x, y, N0, N1, N2, w);
    if (m > 0) {
        k_noalloc_btx<<<m, 256, 0, st>>>(x, B_colptr, B_rowidx, B_val, btx);
        k_noalloc_add_B<<<m, 256, 0, st>>>(y, B_colptr, B_rowidx, B_val, Sigma, btx);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MGMC_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    return MGMC_OK;
}
