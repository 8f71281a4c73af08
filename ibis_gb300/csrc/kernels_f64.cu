// Double-precision residual kernels (FMA contraction allowed).
#define IBISGB_KNS k_f64
#include "kernels.cuh"

namespace ibisgb {
KernelOps kernels_f64() { return k_f64::Launch<double, double, double, false>::ops(); }
}  // namespace ibisgb
