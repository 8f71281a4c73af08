// MIXED_GRAD residual kernels: least-squares gradients and Barth-Jespersen
// limiters in float (each neighbour value and face offset taken relative to
// the cell's own in double first, so float rounds only the increments), stored
// as packed limiter-scaled float gradients; face states (cell value in double
// plus the float increment), thermo closure, flux calculators, surface
// integral, Runge-Kutta update and conserved->primitive inversion in double.
#define IBISGB_KNS k_mgrad
#define IBISGB_FLOAT_GRADIENTS 1
#include "kernels.cuh"

namespace ibisgb {
KernelOps kernels_mixed_grad() { return k_mgrad::Launch<double, double, double, false, float>::ops(); }
}  // namespace ibisgb
