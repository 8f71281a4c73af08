// Double-precision residual kernels with the reference's operation order and
// no FMA contraction (this file is compiled with -fmad=false): bitwise parity
// with ibis's FP64 arithmetic except where pow() is involved.
#define IBISGB_KNS k_exact
#include "kernels.cuh"

namespace ibisgb {
KernelOps kernels_f64_exact() { return k_exact::Launch<double, double, double, true>::ops(); }
}  // namespace ibisgb
