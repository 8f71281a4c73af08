// Tangent of the residual: (I/dt* - dR/dU) v, the Jacobian-vector product of
// ibis's steady solver (SteadyStateLinearisation::matrix_vector_product,
// src/solvers/solvers/steady_state.cpp:52-128).  The reference evaluates it by
// running the whole residual in its Dual<double> type; here the same kernels
// (k_recon, k_face) are instantiated on a device dual type with the
// reference's semantics (dual.cuh), so branch choices, limiter selections and
// flux splittings follow the real part exactly as in ibis.  Compiled with
// -fmad=false like the exact real path.
#include "numerics.cuh"
#include "dual.cuh"

#define IBISGB_KNS k_tan
#include "kernels.cuh"

namespace ibisgb {
namespace k_tan {

// Dual primitives of U + eps v (real part from the context state U, tangent
// from v, rows of N x nc) and the ghosts they feed: conserved_to_primatives in
// Dual (primative_conserved_conversion.cpp:4-23) followed by the
// pre-reconstruction / pre-viscous actions, as compute_dudt applies them.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_tan_prims(DevView v, FvParams prm, const double* vt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    constexpr int NC = DIM + 2;
    const int N = v.N;
    Dual u[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) u[q] = Dual(v.U[q * N + i], vt ? vt[(size_t)i * NC + q] : 0.0);
    Dual rho = u[0];
    Dual vx = u[1] / rho;
    Dual vy = u[2] / rho;
    Dual vz = DIM == 3 ? u[3] / rho : Dual(0.0);
    Dual ke = Dual(0.5) * (vx * vx + vy * vy + vz * vz);
    Dual e = u[DIM + 1] / rho - ke;
    Dual T = e / Dual(prm.Cv);
    Dual p = rho * Dual(prm.R) * T;
    Dual* pr = (Dual*)v.prim;
    const int NT = v.NT;
    pr[i] = rho; pr[NT + i] = p; pr[2 * NT + i] = T; pr[3 * NT + i] = e;
    pr[4 * NT + i] = vx; pr[5 * NT + i] = vy; pr[6 * NT + i] = vz;
    const StateT<Dual> s{rho, p, T, e, vx, vy, vz};
    for (int k = v.feed_off[i]; k < v.feed_off[i + 1]; k++)
        fill_ghost<Dual, double, Dual>(v, prm, v.feed_ghost[k], s);
}

// Dual surface integral (flux_surface_integral, finite_volume.cpp:220-255) and
// out = inv_dt * v - dual(dU/dt), the vector steady_state.cpp:102-110 builds.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_tan_update(DevView v, FvParams prm, const double* vt,
                                                       double inv_dt, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    constexpr int NC = DIM + 2;
    const int N = v.N, F = v.F;
    const double* area = (const double*)v.face + 12 * F;
    const Dual* fl = (const Dual*)v.flux;
    Dual acc[NC];
    const int nf = v.nfaces[i];
    for (int s = 0; s < nf; s++) {
        const int f = v.cell_face[s * N + i];
        const Dual a = -Dual(area[f]) * Dual((double)v.outsign[s * N + i]);
#pragma unroll
        for (int q = 0; q < NC; q++) acc[q] += fl[q * F + f] * a;
    }
    const Dual vol(v.vol[i]);
#pragma unroll
    for (int q = 0; q < NC; q++) {
        const Dual d = acc[q] / vol;
        const size_t idx = (size_t)i * NC + q;
        out[idx] = inv_dt * (vt ? vt[idx] : 0.0) - d.du;
    }
}

}  // namespace k_tan

void launch_tangent(const DevView& v, const FvParams& p, const double* vt, double inv_dt,
                    bool reconstruct, double* out, cudaStream_t s) {
    using namespace k_tan;
    const unsigned bn = blocks_for(v.N), bf = blocks_for(v.F);
    if (v.dim == 3) {
        k_tan_prims<3><<<bn, kBlock, 0, s>>>(v, p, vt);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, double, 3, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_face<Dual, Dual, double, 3, true><<<bf, kBlock, 0, s>>>(v, p, reconstruct);
        k_tan_update<3><<<bn, kBlock, 0, s>>>(v, p, vt, inv_dt, out);
    } else {
        k_tan_prims<2><<<bn, kBlock, 0, s>>>(v, p, vt);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, double, 2, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_face<Dual, Dual, double, 2, true><<<bf, kBlock, 0, s>>>(v, p, reconstruct);
        k_tan_update<2><<<bn, kBlock, 0, s>>>(v, p, vt, inv_dt, out);
    }
}

}  // namespace ibisgb
