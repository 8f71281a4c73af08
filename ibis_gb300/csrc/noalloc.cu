// Residual L2 norms computed without allocating device memory.
//
// Some callers cannot allocate: code whose device memory belongs entirely to a
// caching allocator (PyTorch's pool can hold nearly all of HBM, so a raw
// cudaMalloc next to it can fail), and time loops that must not stall, since
// cudaMalloc/cudaFree synchronize the device.  For them this file provides
// ibisgb_l2_norms_noalloc: a deterministic two-pass reduction (a fixed
// summation order per call, so equal inputs give equal bits; equal to
// ibisgb_l2_norms to rounding, since that one sums in another order), with
// its per-block partial sums in a fixed file-scope __device__ array instead
// of a context buffer.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/ibisgb.h"
#include "engine.hpp"

namespace {

constexpr int kBlock = 256;
constexpr int kCellsPerThread = 16;
constexpr int kCellsPerBlock = kBlock * kCellsPerThread;  // 4096
constexpr int kMaxBlocks = IBISGB_NOALLOC_MAX_CELLS / kCellsPerBlock;
static_assert(kMaxBlocks * kCellsPerBlock == IBISGB_NOALLOC_MAX_CELLS, "max cells must fill whole blocks");

// Six partial sums of squares (global, mass, momentum x/y/z, energy) per block:
// 4096 x 6 doubles = 192 KiB, held by every GPU that loads the library until exit.
static __device__ __align__(256) double g_norm_partials[kMaxBlocks * 6];

// Block b sums the squares of cells [b*4096, (b+1)*4096) and writes all six of
// its partial sums, so no slot is read before the current call has written it.
__global__ void __launch_bounds__(kBlock) k_norm_partials(const double* rows, long long n, int nc,
                                                          double* partials) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    const long long base = (long long)blockIdx.x * kCellsPerBlock;
    for (int k = 0; k < kCellsPerThread; k++) {
        long long i = base + (long long)k * kBlock + threadIdx.x;
        if (i >= n) break;
        for (int q = 0; q < nc; q++) {
            double x = rows[i * nc + q];
            int slot = q == 0 ? 1 : (q == nc - 1 ? 5 : 1 + q);  // mass, mx, my, [mz], energy
            s[slot] += x * x;
            s[0] += x * x;
        }
    }
    __shared__ double sh[6][kBlock];
    for (int j = 0; j < 6; j++) sh[j][threadIdx.x] = s[j];
    __syncthreads();
    for (int w = kBlock / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int j = 0; j < 6; j++) sh[j][threadIdx.x] += sh[j][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int j = 0; j < 6; j++) partials[blockIdx.x * 6 + j] = sh[j][0];
}

// One thread adds the partials of the blocks of this call in block order.
__global__ void k_norm_final(const double* partials, int nblocks, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nblocks; b++)
        for (int j = 0; j < 6; j++) s[j] += partials[b * 6 + j];
    for (int j = 0; j < 6; j++) out[j] = sqrt(s[j]);
}

// Device address of g_norm_partials, looked up with the device current, once
// per device and context: after a cudaDeviceReset (or any other end of the
// primary context) the module is loaded again, possibly at another address, so
// the cached address is keyed on the context it was looked up in.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct Scratch {
    void* ctx;
    double* addr;
};
Scratch g_scratch[kMaxDevices] = {};

typedef int (*CtxGetCurrentFn)(void**);  // cuCtxGetCurrent(CUcontext*), CUresult 0 = success

cudaError_t current_context(void** ctx) {
    static CtxGetCurrentFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
        fn = (CtxGetCurrentFn)p;
    }
    *ctx = nullptr;
    return fn(ctx) == 0 ? cudaSuccess : cudaErrorDeviceUninitialized;
}

cudaError_t scratch_for_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    void* ctx = nullptr;
    e = current_context(&ctx);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!ctx || !g_scratch[dev].addr || g_scratch[dev].ctx != ctx) {
        // the lookup also makes the device's primary context current when no
        // context is yet, so the context is read again after it
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_norm_partials);
        if (e != cudaSuccess) return e;
        e = current_context(&ctx);
        if (e != cudaSuccess) return e;
        g_scratch[dev] = Scratch{ctx, (double*)p};
    }
    *out = g_scratch[dev].addr;
    return cudaSuccess;
}

}  // namespace

extern "C" int ibisgb_l2_norms_noalloc(const double* dudt_device, int64_t num_cells,
                                       int32_t n_conserved, double* norms_device, void* stream) {
    if (!dudt_device || !norms_device) {
        ibisgb::set_thread_error("ibisgb_l2_norms_noalloc: null device pointer");
        return IBISGB_ERR_ARG;
    }
    if (n_conserved != 4 && n_conserved != 5) {
        ibisgb::set_thread_error("ibisgb_l2_norms_noalloc: n_conserved must be 4 (2-D) or 5 (3-D)");
        return IBISGB_ERR_ARG;
    }
    if (num_cells < 1 || num_cells > IBISGB_NOALLOC_MAX_CELLS) {
        ibisgb::set_thread_error("ibisgb_l2_norms_noalloc: num_cells must be in 1.." +
                                 std::to_string(IBISGB_NOALLOC_MAX_CELLS) + ", got " +
                                 std::to_string(num_cells));
        return IBISGB_ERR_ARG;
    }
    double* scratch = nullptr;
    cudaError_t e = scratch_for_current_device(&scratch);
    if (e != cudaSuccess) {
        ibisgb::set_thread_error(std::string("ibisgb_l2_norms_noalloc: ") + cudaGetErrorString(e));
        return IBISGB_ERR_CUDA;
    }
    const int nblocks = (int)((num_cells + kCellsPerBlock - 1) / kCellsPerBlock);
    cudaStream_t s = (cudaStream_t)stream;
    k_norm_partials<<<nblocks, kBlock, 0, s>>>(dudt_device, (long long)num_cells, n_conserved, scratch);
    k_norm_final<<<1, 32, 0, s>>>(scratch, nblocks, norms_device);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        ibisgb::set_thread_error(std::string("ibisgb_l2_norms_noalloc: ") + cudaGetErrorString(e));
        return IBISGB_ERR_CUDA;
    }
    return IBISGB_OK;
}
