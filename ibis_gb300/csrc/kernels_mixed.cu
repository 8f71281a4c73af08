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
void fused_tile_shape(int dim, int* tx, int* ty, int* tz) {
    if (dim == 3) {
        *tx = k_mixed::FusedTile<3>::X; *ty = k_mixed::FusedTile<3>::Y; *tz = k_mixed::FusedTile<3>::Z;
    } else {
        *tx = k_mixed::FusedTile<2>::X; *ty = k_mixed::FusedTile<2>::Y; *tz = k_mixed::FusedTile<2>::Z;
    }
}
}  // namespace ibisgb
