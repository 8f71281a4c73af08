// Mixed-precision residual kernels: reconstruction, gradients, limiters and
// fluxes in float with float primitives and geometry; surface integral, stage
// combination and conserved->primitive inversion in double.
#define IBISGB_KNS k_mixed
#include "kernels.cuh"

namespace ibisgb {
KernelOps kernels_mixed() { return k_mixed::Launch<float, float, float, false>::ops(); }
}  // namespace ibisgb

#include "kernels_fused.cuh"

namespace ibisgb {
void launch_fused_stage(const DevView& v, const SbView& sb, const FvParams& prm, int mode, int stage, int with_dt,
                        cudaStream_t s) {
    k_mixed::launch_fused(v, sb, prm, mode, stage, with_dt, s);
}
cudaError_t prepare_fused_stage() { return k_mixed::prepare_fused(); }
}  // namespace ibisgb

#include <cudaTypedefs.h>

#include "kernels_march.cuh"

namespace ibisgb {
static_assert(sizeof(TmaMap) == sizeof(CUtensorMap) && alignof(TmaMap) >= alignof(CUtensorMap),
              "TmaMap must hold a CUtensorMap");
static_assert(k_mixed::March::TX == kMarchTileX && k_mixed::March::TY == kMarchTileY, "march tile shape");

void launch_march_stage(const DevView& v, const SbView& sb, const SBlock& hb, const FvParams& prm,
                        const TmaMap& prim, const TmaMap& cc, int mode, int stage, int with_dt, int kc,
                        cudaStream_t s) {
    k_mixed::launch_march(v, sb, hb, prm, &prim, &cc, mode, stage, with_dt, kc, s);
}
cudaError_t prepare_march_stage() { return k_mixed::prepare_march(); }

int march_encode_map(TmaMap* out, const float* base, int ni, int nj, int nk, int nvar, long long var_stride,
                     std::string* why) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            if (why) *why = "the driver has no cuTensorMapEncodeTiled";
            return -1;
        }
        encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    const cuuint64_t dims[4] = {(cuuint64_t)ni, (cuuint64_t)nj, (cuuint64_t)nk, (cuuint64_t)nvar};
    const cuuint64_t strides[3] = {(cuuint64_t)ni * 4, (cuuint64_t)ni * nj * 4, (cuuint64_t)var_stride * 4};
    const cuuint32_t box[4] = {(cuuint32_t)k_mixed::March::BW, (cuuint32_t)k_mixed::March::BH, 1, 1};
    const cuuint32_t elem[4] = {1, 1, 1, 1};
    const CUresult r = encode((CUtensorMap*)out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, (void*)base, dims, strides, box,
                              elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        if (why) *why = "cuTensorMapEncodeTiled failed (error " + std::to_string((int)r) + ")";
        return -1;
    }
    return 0;
}
// Self-check of the integer-pipe float -> double conversion against the
// conversion instruction, compiled with the same flags as the kernels that use
// it: n pseudo-random float bit patterns (splitmix64 from seed).
namespace {
__device__ unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__global__ void k_check_conversions(long long n, unsigned long long seed, unsigned long long* bad) {
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long r = splitmix64(seed + (unsigned long long)t);
        const float x = __uint_as_float((unsigned)r);
        const double c = k_mixed::f2d(x), e = (double)x;
        const bool same_d = __double_as_longlong(c) == __double_as_longlong(e) || (c != c && e != e);
        if (!same_d) atomicAdd(bad, 1ull);
        // double -> float on doubles of three kinds: any bit pattern; exponents around
        // the float range (subnormal results, overflow); exact ties between two floats
        const unsigned long long r2 = splitmix64(r ^ 0x5DEECE66Dull);
        unsigned long long bits = r2;
        if (t % 3 == 1) bits = (r2 & 0x800FFFFFFFFFFFFFull) | ((unsigned long long)(860 + (r % 330)) << 52);
        if (t % 3 == 2)
            bits = (r2 & 0x800FFFFFE0000000ull) | 0x10000000ull | ((unsigned long long)(897 + (r % 254)) << 52);
        const double d = __longlong_as_double((long long)bits);
        const float g = k_mixed::d2f(d), h = __double2float_rn(d);
        if (!(__float_as_uint(g) == __float_as_uint(h) || (g != g && h != h))) atomicAdd(bad, 1ull);
    }
}
}  // namespace

int check_float_conversions(long long n, unsigned long long seed, unsigned long long* mismatches) {
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return -1;
    cudaMemset(d, 0, sizeof(unsigned long long));
    k_check_conversions<<<1216, 256>>>(n, seed, d);
    cudaError_t e = cudaMemcpy(mismatches, d, sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : -1;
}

void fused_tile_shape(int dim, int* tx, int* ty, int* tz) {
    if (dim == 3) {
        *tx = k_mixed::FusedTile<3>::X; *ty = k_mixed::FusedTile<3>::Y; *tz = k_mixed::FusedTile<3>::Z;
    } else {
        *tx = k_mixed::FusedTile<2>::X; *ty = k_mixed::FusedTile<2>::Y; *tz = k_mixed::FusedTile<2>::Z;
    }
}
}  // namespace ibisgb
