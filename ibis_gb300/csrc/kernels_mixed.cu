// Mixed-precision residual kernels: reconstruction, gradients, limiters and
// fluxes in float with float primitives and geometry; surface integral, stage
// combination and conserved->primitive inversion in double.
#define IBISGB_KNS k_mixed
#include "kernels.cuh"

namespace ibisgb {
KernelOps kernels_mixed() { return k_mixed::Launch<float, float, float, false>::ops(); }
}  // namespace ibisgb
