// MIXED_FF residual kernels: the float state and geometry arrays of the mixed
// build plus their lo companions (each double held as float + lo, about 48
// bits).  Gradients and limiters (on cell-relative values), the packed
// limiter-scaled gradients, face states, thermo closure, flux calculators and
// viscous terms in float-float arithmetic on the FP32 pipe; fluxes stored as
// float + lo and summed as float pairs; Runge-Kutta update and
// conserved->primitive inversion in double.
#define IBISGB_KNS k_ff
#define IBISGB_FLOAT_FLOAT 1
#include "kernels.cuh"

namespace ibisgb {
KernelOps kernels_mixed_ff() { return k_ff::Launch<FF, float, float, false, FF>::ops(); }
}  // namespace ibisgb
