// Tangent of the residual: (I/dt* - dR/dU) v, the Jacobian-vector product of
// ibis's steady solver (SteadyStateLinearisation::matrix_vector_product,
// src/solvers/solvers/steady_state.cpp:52-128).  The reference evaluates it by
// running the whole residual in its Dual<double> type; here the same kernels
// (k_recon, k_face) are instantiated on a device dual type with the
// reference's semantics (dual.cuh), so branch choices, limiter selections and
// flux splittings follow the real part exactly as in ibis.  Compiled with
// -fmad=false like the exact real path.
#include <algorithm>

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
// Gm = Dual: the geometry is dual too (the geometry tangent's ghost reflection).
template <int DIM, class Gm = double>
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
        fill_ghost<Dual, Gm, Dual>(v, prm, v.feed_ghost[k], s);
}

// ---------------------------------------------------------------------------
// Geometry tangent: dR/dgeometry . d at the current state, the residual kernels
// run on dual geometry (the face frame, centres and areas, the centroids --
// ghosts included -- and volumes, seeded with d) and a state of zero tangent; the
// least-squares factors are formed again from the dual centroids.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_geo_seed(const double* fg, const double* cc, const double* vol,
                                                     const double* dface, const double* dcell, int F, int NT, int N,
                                                     Dual* gface, Dual* gcc, Dual* gvol) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < 13LL * F) gface[t] = Dual(fg[t], dface[t]);
    if (t < 3LL * NT) gcc[t] = Dual(cc[t], dcell[t]);
    if (t < N) gvol[t] = Dual(vol[t], dcell[3LL * NT + t]);
}

// WLSGradient::compute_weights (gradient.h:119-162) on the dual centroids, in the
// mesh builder's form (r11 r12 r22 [r13 r23 r33], one array each)
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_geo_r(DevView v, const Dual* gcc, Dual* gr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    const int N = v.N, NT = v.NT;
    const Dual xi = gcc[i], yi = gcc[NT + i], zi = DIM == 3 ? gcc[2 * NT + i] : Dual(0.0);
    Dual sxx(0.0), sxy(0.0), sxz(0.0), syy(0.0), syz(0.0), szz(0.0);
    for (int s = 0; s < v.nfaces[i]; s++) {
        const int nb = v.cell_nbr[s * N + i];
        const Dual dx = gcc[nb] - xi, dy = gcc[NT + nb] - yi, dz = DIM == 3 ? gcc[2 * NT + nb] - zi : Dual(0.0);
        sxx += dx * dx; sxy += dx * dy; sxz += dx * dz;
        syy += dy * dy; syz += dy * dz; szz += dz * dz;
    }
    const Dual one(1.0);
    const Dual r11 = dual_sqrt(sxx);
    const Dual r12 = one / r11 * sxy;
    const Dual r22 = dual_sqrt(syy - r12 * r12);
    gr[i] = r11; gr[N + i] = r12; gr[2 * N + i] = r22;
    if (DIM == 3) {
        const Dual r13 = one / r11 * sxz;
        const Dual r23 = one / r22 * (syz - r12 / r11 * sxz);
        gr[3 * N + i] = r13; gr[4 * N + i] = r23; gr[5 * N + i] = dual_sqrt(szz - (r13 * r13 + r23 * r23));
    }
}

// out = -(dual part of dU/dt): the surface integral with dual areas and volumes
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_geo_tan_update(DevView v, const Dual* gface, const Dual* gvol,
                                                           double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    constexpr int NC = DIM + 2;
    const int N = v.N, F = v.F;
    const Dual* fl = (const Dual*)v.flux;
    Dual acc[NC];
    const int nf = v.nfaces[i];
    for (int s = 0; s < nf; s++) {
        const int f = v.cell_face[s * N + i];
        const Dual a = -gface[12 * F + f] * Dual((double)v.outsign[s * N + i]);
#pragma unroll
        for (int q = 0; q < NC; q++) acc[q] += fl[q * F + f] * a;
    }
#pragma unroll
    for (int q = 0; q < NC; q++) out[(size_t)i * NC + q] = (acc[q] / gvol[i]).du;
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

// ---------------------------------------------------------------------------
// Adjoint: (dR/dU)^T w, the transpose of the tangent above, in three passes
// that walk the residual backwards.  The forward state (primitives, ghosts,
// gradients, limiters) is recomputed by the tangent's own kernels with a zero
// tangent, and every branch (limiter winner, min/max arguments, flux
// splittings) is taken again from those real values with the Dual rules, so
// <w, J v> = <J^T w, v> to rounding.  Local derivatives of the face flux and
// the ghost actions come from dual evaluations seeded one input at a time, in
// DualA (the derivative of floor is zero; see dual.cuh), which differs from the
// tangent only for LDFSS2.
// ---------------------------------------------------------------------------

// inputs of the face flux on each side: the reconstructed pair and velocities
// when reconstructing (the closure rebuilds the rest), else rho, p, T, v
template <int DIM>
__device__ __forceinline__ int face_inputs(int thermo, bool reconstruct, int (&in)[6]) {
    if (reconstruct) {
        int ia, ib;
        thermo_vars(thermo, ia, ib);
        in[0] = ia; in[1] = ib; in[2] = 4; in[3] = 5; in[4] = 6; in[5] = -1;
        return DIM == 3 ? 5 : 4;
    }
    in[0] = 0; in[1] = 1; in[2] = 2; in[3] = 4; in[4] = 5; in[5] = 6;
    return DIM == 3 ? 6 : 5;
}

// Real reconstructed primitives of side cell c of face f (k_face's arithmetic).
template <int DIM>
__device__ void side_values(const DevView& v, const FvParams& prm, bool reconstruct, int c, int f, double (&q)[7]) {
    const Dual* pr = (const Dual*)v.prim;
    const Dual* gr = (const Dual*)v.grad;
    const Dual* ph = (const Dual*)v.phi;
    const double* fg = (const double*)v.face;
    const double* cc = (const double*)v.cc;
    const int NT = v.NT, N = v.N, F = v.F;
    for (int k = 0; k < 7; k++) q[k] = (DIM == 2 && k == 6) ? 0.0 : pr[k * NT + c].re;
    if (!reconstruct || c >= N) return;
    const double dx = fg[9 * F + f] - cc[c], dy = fg[10 * F + f] - cc[NT + c];
    const double dz = DIM == 3 ? fg[11 * F + f] - cc[2 * NT + c] : 0.0;
    int in[6];
    const int K = face_inputs<DIM>(prm.thermo, true, in);
    for (int k = 0; k < K; k++) {
        const double lim = prm.limiter ? ph[k * N + c].re : 1.0;
        const double sgr = DIM == 3 ? gr[(3 * k) * N + c].re * dx + gr[(3 * k + 1) * N + c].re * dy +
                                          gr[(3 * k + 2) * N + c].re * dz
                                    : gr[(3 * k) * N + c].re * dx + gr[(3 * k + 1) * N + c].re * dy;
        q[in[k]] = q[in[k]] + lim * sgr;
    }
}

// Pass 1, per face: adjoint of the face flux, wbar_F = sum over its valid cells of
// -outsign A / V w, pulled back to the reconstructed inputs of both sides.
// Valid sides go to qf[(side * 6 + k) * F + f]; ghost sides to ga[m * G + g].
// Viscous: also to the sides' p, T, v (qv, or the ghost's gav) and viscous
// gradients (qg), through viscous_face.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_adj_face(DevView v, FvParams prm, const double* w, int reconstruct,
                                                     AdjScratch a) {
    double* qf = a.qf;
    double* ga = a.ga;
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.F) return;
    constexpr int NC = DIM + 2;
    const int N = v.N, F = v.F, G = v.G;
    const double* fg = (const double*)v.face;
    const int cells[2] = {v.left[f], v.right[f]};
    const double A = fg[12 * F + f];
    double fb[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int side = 0; side < 2; side++) {
        const int c = cells[side];
        if (c >= N) continue;
        const double sc = (side == 0 ? -A : A) / v.vol[c];
        for (int q = 0; q < NC; q++) fb[q == NC - 1 ? 4 : q] += sc * w[(size_t)c * NC + q];
    }
    double qv[2][7];
    side_values<DIM>(v, prm, reconstruct, cells[0], f, qv[0]);
    side_values<DIM>(v, prm, reconstruct, cells[1], f, qv[1]);
    const DualA nx(fg[f]), ny(fg[F + f]), nz(DIM == 3 ? fg[2 * F + f] : 0.0);
    const DualA t1x(fg[3 * F + f]), t1y(fg[4 * F + f]), t1z(DIM == 3 ? fg[5 * F + f] : 0.0);
    const DualA t2x(DIM == 3 ? fg[6 * F + f] : 0.0), t2y(DIM == 3 ? fg[7 * F + f] : 0.0), t2z(fg[8 * F + f]);
    const Gas<DualA> gm(prm);
    int in[6];
    // a constant-flux face's convective flux does not depend on the state
    const int K = prm.cflux && constant_flux_bound(v, cells[0], cells[1]) ? 0
                                                                           : face_inputs<DIM>(prm.thermo, reconstruct, in);
    if (K == 0)  // nothing flows back to the valid side's inputs (k_adj_cell reads every slot of every face)
        for (int side = 0; side < 2; side++)
            if (cells[side] < N)
                for (int k = 0; k < 6; k++) qf[(size_t)(side * 6 + k) * F + f] = 0.0;
    for (int side = 0; side < 2; side++) {
        for (int k = 0; k < K; k++) {
            DualA qd[2][7];
            for (int s2 = 0; s2 < 2; s2++)
                for (int m = 0; m < 7; m++) qd[s2][m] = DualA(qv[s2][m], (s2 == side && m == in[k]) ? 1.0 : 0.0);
            FaceSide<DualA> S[2];
            side_state<DualA, DIM, true>(prm.thermo, gm, reconstruct, qd[0], nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z,
                                         S[0]);
            side_state<DualA, DIM, true>(prm.thermo, gm, reconstruct, qd[1], nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z,
                                         S[1]);
            DualA Fd[5];
            convective_flux<DualA, DIM, true>(prm, gm, S[0], S[1], nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z, Fd);
            double acc = 0.0;
            for (int q = 0; q < 5; q++) acc += fb[q] * Fd[q].du;
            const int c = cells[side];
            if (c < N) qf[(size_t)(side * 6 + k) * F + f] = acc;
            else ga[(size_t)in[k] * G + (c - N)] = acc;
        }
    }
    if (a.fs_ghost && prm.cflux)  // a constant-flux face: the flux of its boundary's fixed state
        if (const BoundDev* B = constant_flux_bound(v, cells[0], cells[1])) {
            const int g = (cells[1] >= N ? cells[1] : cells[0]) - N;
            for (int j = 0; j < 7; j++) {
                DualA fsd[7];
                for (int k = 0; k < 7; k++) fsd[k] = DualA(B->cfs[k], k == j ? 1.0 : 0.0);
                DualA Fd[5];
                constant_flux<DualA, DIM>(fsd, prm.Cv, nx, ny, nz, Fd);
                double acc = 0.0;
                for (int q = 0; q < 5; q++) acc += fb[q] * Fd[q].du;
                a.fs_ghost[(size_t)g * 7 + j] += acc;
            }
        }
    // the face's total flux (convective less viscous), for the area and volume adjoints
    double Ft[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    auto finish_geo = [&]() {
        double ab = 0.0;
        for (int q = 0; q < 5; q++) ab += fb[q] * Ft[q];
        a.geo_face[(size_t)12 * F + f] = ab / A;
        for (int side = 0; side < 2; side++) {
            const int c = cells[side];
            if (c >= N) continue;
            const double V = v.vol[c], sc = (side == 0 ? -A : A) / V;
            double wf = 0.0;
            for (int q = 0; q < NC; q++) wf += w[(size_t)c * NC + q] * Ft[q == NC - 1 ? 4 : q];
            a.geo_vb[(size_t)side * F + f] = -sc / V * wf;
        }
    };
    if (a.geo_face) {
        // geometry: each normal / tangent component read by the flux (one dual seed
        // each, 2-D reads n_x, n_y, t1_x, t1_y, t2_z), the area (R is linear in it) and
        // the volume of each valid side (R_c = -(1/V_c) sum outsign A F)
        constexpr int kRead[9] = {0, 1, 3, 4, 8, 2, 5, 6, 7};
        constexpr int NG = DIM == 3 ? 9 : 5;
        double gbar[9] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, Fr[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        for (int jj = 0; jj < NG; jj++) {
            const int j = kRead[jj];
            DualA gd[9];
            for (int k = 0; k < 9; k++) {
                const bool unread = DIM == 2 && (k == 2 || k == 5 || k == 6 || k == 7);
                gd[k] = DualA(unread ? 0.0 : fg[k * F + f], k == j ? 1.0 : 0.0);
            }
            DualA qd[2][7];
            for (int s2 = 0; s2 < 2; s2++)
                for (int m = 0; m < 7; m++) qd[s2][m] = DualA(qv[s2][m]);
            FaceSide<DualA> S[2];
            for (int s2 = 0; s2 < 2; s2++)
                side_state<DualA, DIM, true>(prm.thermo, gm, reconstruct, qd[s2], gd[0], gd[1], gd[2], gd[3], gd[4],
                                             gd[5], gd[6], gd[7], gd[8], S[s2]);
            DualA Fd[5];
            convective_flux<DualA, DIM, true>(prm, gm, S[0], S[1], gd[0], gd[1], gd[2], gd[3], gd[4], gd[5], gd[6],
                                              gd[7], gd[8], Fd);
            if (prm.cflux)  // a constant-flux face: the fixed state's flux through the face's normal
                if (const BoundDev* B = constant_flux_bound(v, cells[0], cells[1]))
                    constant_flux<DualA, DIM>(B->cfs, prm.Cv, gd[0], gd[1], gd[2], Fd);
            double acc = 0.0;
            for (int q = 0; q < 5; q++) acc += fb[q] * Fd[q].du;
            gbar[j] = acc;
            if (jj == 0)
                for (int q = 0; q < 5; q++) Fr[q] = Fd[q].re;
        }
        for (int k = 0; k < 9; k++) a.geo_face[(size_t)k * F + f] = gbar[k];
        for (int q = 0; q < 5; q++) Ft[q] = Fr[q];
    }
    if (!prm.viscous) {
        if (a.geo_face) finish_geo();
        return;
    }
    // viscous terms (subtracted from the flux): states p, T, v of both sides and
    // the viscous gradients of the valid cells, one dual seed each
    const Dual* pr = (const Dual*)v.prim;
    const Dual* vgd = (const Dual*)v.vgrad;
    const Dual* vgh = (const Dual*)v.vghost;
    const double* cc = (const double*)v.cc;
    const int NT = v.NT;
    const int l = cells[0], r = cells[1];
    const bool interior = l < N && r < N;
    const int gsrc[2] = {interior ? l : (l < N ? l : r), interior ? r : (l < N ? l : r)};
    double sv[2][5], gv[2][12];
    for (int side = 0; side < 2; side++) {
        const int c = cells[side];
        for (int k = 0; k < 5; k++)
            sv[side][k] = c >= N ? vgh[k * G + (c - N)].re : pr[(k == 0 ? 1 : visc_prim(k - 1)) * NT + c].re;
        for (int k = 0; k < 12; k++) gv[side][k] = vgd[k * N + gsrc[side]].re;
    }
    DualA ex(0.0), ey(0.0), ez(0.0);
    if (interior) {
        ex = DualA(cc[r] - cc[l]);
        ey = DualA(cc[NT + r] - cc[NT + l]);
        ez = DualA(DIM == 3 ? cc[2 * NT + r] - cc[2 * NT + l] : 0.0);
    }
    // the terms are subtracted from the momentum and energy fluxes
    const double tb[4] = {-fb[1], -fb[2], -fb[3], -fb[4]};
    auto eval = [&](int which, int side, int k) {
        DualA sl[5], sr[5], gl[12], gr[12];
        for (int q = 0; q < 5; q++) {
            sl[q] = DualA(sv[0][q], which == 0 && side == 0 && q == k ? 1.0 : 0.0);
            sr[q] = DualA(sv[1][q], which == 0 && side == 1 && q == k ? 1.0 : 0.0);
        }
        for (int q = 0; q < 12; q++) {
            // a boundary face uses its interior cell's gradients on both sides: one seed for both
            const bool seed_l = which == 1 && q == k && (side == 0 || !interior);
            const bool seed_r = which == 1 && q == k && (side == 1 || !interior);
            gl[q] = DualA(gv[0][q], seed_l ? 1.0 : 0.0);
            gr[q] = DualA(gv[1][q], seed_r ? 1.0 : 0.0);
        }
        DualA out[4], rho, mu, kk;
        viscous_face<DualA, DIM, true>(prm, gm, interior, sl, sr, gl, gr, ex, ey, ez, nx, ny, nz, out, rho, mu, kk);
        return tb[0] * out[0].du + tb[1] * out[1].du + tb[2] * out[2].du + tb[3] * out[3].du;
    };
    for (int side = 0; side < 2; side++) {
        const int c = cells[side];
        for (int k = 0; k < 5; k++) {
            const double b = eval(0, side, k);
            if (c < N) a.qv[(size_t)(side * 5 + k) * F + f] = b;
            else a.gav[(size_t)k * G + (c - N)] = b;
        }
    }
    // gradients: per valid side; a boundary face's one set of gradients is seeded once
    for (int side = 0; side < 2; side++) {
        const int c = cells[side];
        for (int k = 0; k < 12; k++) {
            double b = 0.0;
            if (c < N && (interior || side == (l < N ? 0 : 1))) b = eval(1, side, k);
            a.qg[(size_t)(side * 12 + k) * F + f] = b;
        }
    }
    if (!a.geo_face) return;
    // geometry of the viscous terms: the normal, the centroid offset e = x_r - x_l
    // (interior faces) and the terms' own values for the area and volume adjoints
    auto evalg = [&](int j, double (&re)[4]) {
        DualA sl[5], sr[5], gl[12], gr[12];
        for (int q = 0; q < 5; q++) { sl[q] = DualA(sv[0][q]); sr[q] = DualA(sv[1][q]); }
        for (int q = 0; q < 12; q++) { gl[q] = DualA(gv[0][q]); gr[q] = DualA(gv[1][q]); }
        const DualA gnx(fg[f], j == 0 ? 1.0 : 0.0), gny(fg[F + f], j == 1 ? 1.0 : 0.0);
        const DualA gnz(DIM == 3 ? fg[2 * F + f] : 0.0, j == 2 ? 1.0 : 0.0);
        const DualA gex(ex.re, j == 3 ? 1.0 : 0.0), gey(ey.re, j == 4 ? 1.0 : 0.0), gez(ez.re, j == 5 ? 1.0 : 0.0);
        DualA out[4], rho, mu, kk;
        viscous_face<DualA, DIM, true>(prm, gm, interior, sl, sr, gl, gr, gex, gey, gez, gnx, gny, gnz, out, rho, mu,
                                       kk);
        for (int m = 0; m < 4; m++) re[m] = out[m].re;
        return tb[0] * out[0].du + tb[1] * out[1].du + tb[2] * out[2].du + tb[3] * out[3].du;
    };
    double vr[4];
    for (int j = 0; j < (DIM == 3 ? 3 : 2); j++) a.geo_face[(size_t)j * F + f] += evalg(j, vr);
    for (int d = 0; d < 3; d++)
        a.geo_ceb[(size_t)d * F + f] = (interior && (DIM == 3 || d < 2)) ? evalg(3 + d, vr) : 0.0;
    for (int m = 0; m < 4; m++) Ft[1 + m] -= vr[m];  // the terms are subtracted from momentum and energy
    finish_geo();
}

// Least-squares weights of every face slot of a cell from its neighbours'
// centroid offsets d[s] = x_nb(s) - x_i, on a dual scalar: the factors r of
// WLSGradient::compute_weights (gradient.h:119-162) and the per-neighbour weights
// of compute_gradients (gradient.h:89-107), as the mesh builder forms them.
template <int DIM>
__device__ void lsq_weights(const DualA (&d)[6][3], int nf, DualA (&w)[6][3]) {
    const DualA one(1.0);
    DualA sxx(0.0), sxy(0.0), sxz(0.0), syy(0.0), syz(0.0), szz(0.0);
    for (int s = 0; s < nf; s++) {
        sxx += d[s][0] * d[s][0]; sxy += d[s][0] * d[s][1]; syy += d[s][1] * d[s][1];
        if (DIM == 3) { sxz += d[s][0] * d[s][2]; syz += d[s][1] * d[s][2]; szz += d[s][2] * d[s][2]; }
    }
    const DualA r11 = dual_sqrt(sxx);
    const DualA r12 = one / r11 * sxy;
    const DualA r22 = dual_sqrt(syy - r12 * r12);
    DualA r13(0.0), r23(0.0), r33(1.0);
    if (DIM == 3) {
        r13 = one / r11 * sxz;
        r23 = one / r22 * (syz - r12 / r11 * sxz);
        r33 = dual_sqrt(szz - (r13 * r13 + r23 * r23));
    }
    const DualA beta = (r12 * r23 - r13 * r23) / (r11 * r22);
    for (int s = 0; s < nf; s++) {
        const DualA a1 = d[s][0] / (r11 * r11);
        const DualA a2 = one / (r22 * r22) * (d[s][1] - r12 / r11 * d[s][0]);
        const DualA a3 = DIM == 3 ? one / (r33 * r33) * (d[s][2] - r23 / r22 * d[s][1] + beta * d[s][0]) : DualA(0.0);
        w[s][0] = a1 - r12 / r11 * a2 + beta * a3;
        w[s][1] = a2 - r23 / r22 * a3;
        w[s][2] = a3;
    }
}

// The least-squares weights' adjoint wb (per slot) of valid cell i taken through the
// centroid offsets: what each valid neighbour's centroid receives goes to
// a.geo_nbc per slot, a ghost's centroid receives it directly (its only valid
// cell), and the cell's own centroid adjoint is returned in own[].
template <int DIM>
__device__ void lsq_geometry_adjoint(const DevView& v, const AdjScratch& a, int i, int nf, const double (&wb)[6][3],
                                     double (&own)[3]) {
    const int N = v.N, NT = v.NT, MF = v.MF;
    const double* cc = (const double*)v.cc;
    const double xi = cc[i], yi = cc[NT + i], zi = DIM == 3 ? cc[2 * NT + i] : 0.0;
    DualA dd[6][3];
    for (int s = 0; s < nf; s++) {
        const int nb = v.cell_nbr[s * N + i];
        dd[s][0] = DualA(cc[nb] - xi);
        dd[s][1] = DualA(cc[NT + nb] - yi);
        dd[s][2] = DualA(DIM == 3 ? cc[2 * NT + nb] - zi : 0.0);
    }
    for (int sj = 0; sj < nf; sj++) {
        const int nb = v.cell_nbr[sj * N + i];
        for (int sd = 0; sd < DIM; sd++) {
            dd[sj][sd].du = 1.0;
            DualA wd[6][3];
            lsq_weights<DIM>(dd, nf, wd);
            dd[sj][sd].du = 0.0;
            double acc = 0.0;
            for (int s = 0; s < nf; s++)
                for (int d = 0; d < DIM; d++) acc += wb[s][d] * wd[s][d].du;
            own[sd] -= acc;
            if (nb < N) a.geo_nbc[((size_t)sd * MF + sj) * N + i] = acc;
            else a.geo_cell[(size_t)sd * NT + nb] += acc;
        }
    }
}

// Pass 2, per valid cell: gathers its faces' input adjoints, reverses the
// reconstruction, the Barth-Jespersen limiter (its winning face and the min/max
// neighbours chosen with the Dual rules) and the least-squares gradient.
// Viscous: also the faces' adjoints of the cell's p, T, v and viscous gradients,
// and the viscous least squares reversed.  The cell's own primitive adjoint
// goes to self[m * N + i]; what its neighbours receive, by primitive m, goes to
// nba[(m * MF + s) * N + i] (valid neighbours, read back by pass 3) or into ga
// / gav (ghost neighbours, each of which has one cell).
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_adj_cell(DevView v, FvParams prm, int reconstruct, AdjScratch a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    const double* qf = a.qf;
    double* self = a.self;
    double* nba = a.nba;
    double* ga = a.ga;
    constexpr int NV = DIM == 3 ? 5 : 4;
    const int N = v.N, F = v.F, G = v.G, NT = v.NT, MF = v.MF;
    const Dual* pr = (const Dual*)v.prim;
    const Dual* gr = (const Dual*)v.grad;
    const Dual* ph = (const Dual*)v.phi;
    int in[6];
    const int K = face_inputs<DIM>(prm.thermo, reconstruct, in);
    double pb[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int nf = v.nfaces[i];
    for (int s = 0; s < MF; s++)
        for (int m = 0; m < 7; m++) nba[((size_t)m * MF + s) * N + i] = 0.0;
    if (a.geo_nbc)  // every slot and coordinate: pass 3 reads all three, a 2-D grid writes two
        for (int s = 0; s < MF; s++)
            for (int d = 0; d < 3; d++) a.geo_nbc[((size_t)d * MF + s) * N + i] = 0.0;
    const double* fg = (const double*)v.face;
    const double* cc = (const double*)v.cc;
    const double* rr = (const double*)v.r;
    const double xi = cc[i], yi = cc[NT + i], zi = DIM == 3 ? cc[2 * NT + i] : 0.0;
    // least-squares weights of slot s (k_recon's exact form)
    double r11 = rr[i], r12 = rr[N + i], r22 = rr[2 * N + i], r13 = 0.0, r23 = 0.0, r33 = 1.0;
    if (DIM == 3) { r13 = rr[3 * N + i]; r23 = rr[4 * N + i]; r33 = rr[5 * N + i]; }
    const double beta = (r12 * r23 - r13 * r23) / (r11 * r22);
    auto weights = [&](int nb, double& w1, double& w2, double& w3) {
        const double dx = cc[nb] - xi, dy = cc[NT + nb] - yi, dz = DIM == 3 ? cc[2 * NT + nb] - zi : 0.0;
        const double a1 = dx / (r11 * r11);
        const double a2 = 1.0 / (r22 * r22) * (dy - r12 / r11 * dx);
        const double a3 = DIM == 3 ? 1.0 / (r33 * r33) * (dz - r23 / r22 * dy + beta * dx) : 0.0;
        w1 = a1 - r12 / r11 * a2 + beta * a3;
        w2 = a2 - r23 / r22 * a3;
        w3 = a3;
    };
    constexpr int NW = DIM == 3 ? 4 : 3;
    double hb[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (prm.viscous) {
        // viscous: the faces' adjoints of this cell's p, T, v and of its viscous
        // gradients, then the gradients' least squares reversed onto the neighbours
        // (valid cells' T, v; ghosts' pre-viscous values)
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            const int side = v.outsign[s * N + i] > 0 ? 0 : 1;
            const double q5[5] = {a.qv[(size_t)(side * 5 + 0) * F + f], a.qv[(size_t)(side * 5 + 1) * F + f],
                                  a.qv[(size_t)(side * 5 + 2) * F + f], a.qv[(size_t)(side * 5 + 3) * F + f],
                                  a.qv[(size_t)(side * 5 + 4) * F + f]};
            pb[1] += q5[0]; pb[2] += q5[1]; pb[4] += q5[2]; pb[5] += q5[3]; pb[6] += q5[4];
            for (int q = 0; q < 4; q++)
                for (int d = 0; d < 3; d++) hb[q][d] += a.qg[(size_t)(side * 12 + 3 * q + d) * F + f];
        }
        for (int s = 0; s < nf; s++) {
            const int nb = v.cell_nbr[s * N + i];
            double w1, w2, w3;
            weights(nb, w1, w2, w3);
            for (int q = 0; q < NW; q++) {
                const double c = w1 * hb[q][0] + w2 * hb[q][1] + (DIM == 3 ? w3 * hb[q][2] : 0.0);
                pb[visc_prim(q)] -= c;
                if (nb < N) nba[((size_t)visc_prim(q) * MF + s) * N + i] += c;
                else a.gav[(size_t)(1 + q) * G + (nb - N)] += c;
            }
        }
    }
    const bool geo = a.geo_cell != nullptr;
    // the least-squares weights' adjoint per slot (viscous gradients here, the
    // reconstruction gradients below) and the cell's own centroid adjoint
    double wb[6][3], ccs[3] = {0.0, 0.0, 0.0};
    if (geo) {
        double vbar = 0.0;  // the cell's volume, from its faces
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            const int side = v.outsign[s * N + i] > 0 ? 0 : 1;
            vbar += a.geo_vb[(size_t)side * F + f];
            if (prm.viscous)  // the viscous centroid offset e = x_r - x_l of interior faces
                for (int d = 0; d < 3; d++) ccs[d] += (side == 0 ? -1.0 : 1.0) * a.geo_ceb[(size_t)d * F + f];
        }
        a.geo_cell[(size_t)3 * NT + i] = vbar;
        const Dual* vgh = (const Dual*)v.vghost;
        for (int s = 0; s < 6; s++) wb[s][0] = wb[s][1] = wb[s][2] = 0.0;
        if (prm.viscous)
            for (int s = 0; s < nf; s++) {
                const int nb = v.cell_nbr[s * N + i];
                for (int q = 0; q < NW; q++) {
                    const double wi = pr[visc_prim(q) * NT + i].re;
                    const double wn = nb >= N ? vgh[(size_t)(1 + q) * G + (nb - N)].re : pr[visc_prim(q) * NT + nb].re;
                    for (int d = 0; d < 3; d++) wb[s][d] += hb[q][d] * (wn - wi);
                }
            }
    }
    if (!reconstruct) {
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            const int side = v.outsign[s * N + i] > 0 ? 0 : 1;
            for (int k = 0; k < K; k++) pb[in[k]] += qf[(size_t)(side * 6 + k) * F + f];
        }
        if (geo) {
            if (prm.viscous) lsq_geometry_adjoint<DIM>(v, a, i, nf, wb, ccs);
            for (int d = 0; d < 3; d++) a.geo_cell[(size_t)d * NT + i] = ccs[d];
        }
        for (int m = 0; m < 7; m++) self[(size_t)m * N + i] = pb[m];
        return;
    }
    double ui[NV], g[NV][3], phi[NV], gb[NV][3], phib[NV];
    for (int k = 0; k < NV; k++) {
        ui[k] = pr[in[k] * NT + i].re;
        phi[k] = prm.limiter ? ph[k * N + i].re : 1.0;
        phib[k] = 0.0;
        for (int d = 0; d < 3; d++) {
            g[k][d] = (DIM == 2 && d == 2) ? 0.0 : gr[(3 * k + d) * N + i].re;
            gb[k][d] = 0.0;
        }
    }
    // face-centre adjoint by slot (dx = x_f - x_i enters the reconstruction and the limiter)
    double fcs[6][3];
    for (int s = 0; s < 6; s++) fcs[s][0] = fcs[s][1] = fcs[s][2] = 0.0;
    // reconstruction q_f = q + phi (g . dx) on every face of the cell
    for (int s = 0; s < nf; s++) {
        const int f = v.cell_face[s * N + i];
        const int side = v.outsign[s * N + i] > 0 ? 0 : 1;
        const double dx = fg[9 * F + f] - xi, dy = fg[10 * F + f] - yi, dz = DIM == 3 ? fg[11 * F + f] - zi : 0.0;
        for (int k = 0; k < NV; k++) {
            const double b = qf[(size_t)(side * 6 + k) * F + f];
            pb[in[k]] += b;
            const double sgr = DIM == 3 ? g[k][0] * dx + g[k][1] * dy + g[k][2] * dz : g[k][0] * dx + g[k][1] * dy;
            phib[k] += b * sgr;
            gb[k][0] += b * phi[k] * dx; gb[k][1] += b * phi[k] * dy;
            if (DIM == 3) gb[k][2] += b * phi[k] * dz;
            if (geo) {
                const double c = b * phi[k];
                fcs[s][0] += c * g[k][0]; fcs[s][1] += c * g[k][1];
                if (DIM == 3) fcs[s][2] += c * g[k][2];
            }
        }
    }
    // the min / max arguments
    double umin[NV], umax[NV];
    int amin[NV], amax[NV];
    for (int k = 0; k < NV; k++) { umin[k] = ui[k]; umax[k] = ui[k]; amin[k] = -1; amax[k] = -1; }
    for (int s = 0; s < nf; s++) {
        const int nb = v.cell_nbr[s * N + i];
        for (int k = 0; k < NV; k++) {
            const double un = pr[in[k] * NT + nb].re;
            if (!(umin[k] < un)) { umin[k] = un; amin[k] = s; }  // Dual min: ties take the second
            if (!(umax[k] > un)) { umax[k] = un; amax[k] = s; }
        }
    }
    double extb[NV];  // adjoint of the chosen extreme neighbour value
    int ext[NV];
    for (int k = 0; k < NV; k++) { extb[k] = 0.0; ext[k] = -1; }
    if (prm.limiter) {
        const double eps = prm.eps;
        for (int k = 0; k < NV; k++) {
            // the limiter loop of k_recon: winner = last face whose ratio was taken by min(phi, ratio)
            double ph_k = 1.0;
            int win = -1;
            for (int s = 0; s < nf; s++) {
                const int f = v.cell_face[s * N + i];
                const double dx = fg[9 * F + f] - xi, dy = fg[10 * F + f] - yi;
                const double dz = DIM == 3 ? fg[11 * F + f] - zi : 0.0;
                double t = DIM == 3 ? g[k][0] * dx + g[k][1] * dy + g[k][2] * dz : g[k][0] * dx + g[k][1] * dy;
                const int sg = (t > 0.0) - (t < 0.0);
                const double d2 = (double)sg * (fabs(t) + eps);
                if (sg != 0) {
                    const double ratio = sg > 0 ? (umax[k] - ui[k]) / d2 : (umin[k] - ui[k]) / d2;
                    if (!(ph_k < ratio)) { ph_k = ratio; win = s; }
                }
            }
            if (win < 0) continue;
            const int f = v.cell_face[win * N + i];
            const double dx = fg[9 * F + f] - xi, dy = fg[10 * F + f] - yi, dz = DIM == 3 ? fg[11 * F + f] - zi : 0.0;
            const double t = DIM == 3 ? g[k][0] * dx + g[k][1] * dy + g[k][2] * dz : g[k][0] * dx + g[k][1] * dy;
            const int sg = (t > 0.0) - (t < 0.0);
            const double d2 = (double)sg * (fabs(t) + eps);
            const double delta = sg > 0 ? umax[k] - ui[k] : umin[k] - ui[k];
            const double db = phib[k] / d2;
            const double d2b = -phib[k] * delta / (d2 * d2);
            const double tb = d2b * (double)sg * (t < 0.0 ? -1.0 : 1.0);
            gb[k][0] += tb * dx; gb[k][1] += tb * dy;
            if (DIM == 3) gb[k][2] += tb * dz;
            if (geo) {
                fcs[win][0] += tb * g[k][0]; fcs[win][1] += tb * g[k][1];
                if (DIM == 3) fcs[win][2] += tb * g[k][2];
            }
            // delta = u_ext - u_i: the extreme is the cell itself (no net term) or a neighbour
            ext[k] = sg > 0 ? amax[k] : amin[k];
            if (ext[k] >= 0) { extb[k] = db; pb[in[k]] -= db; }
        }
    }
    // gradient g = sum_s w_s (u_nb - u_i)
    for (int s = 0; s < nf; s++) {
        const int nb = v.cell_nbr[s * N + i];
        double w1, w2, w3;
        weights(nb, w1, w2, w3);
        for (int k = 0; k < NV; k++) {
            double c = w1 * gb[k][0] + w2 * gb[k][1] + (DIM == 3 ? w3 * gb[k][2] : 0.0);
            pb[in[k]] -= c;
            if (ext[k] == s) c += extb[k];
            if (nb < N) nba[((size_t)in[k] * MF + s) * N + i] += c;
            else ga[(size_t)in[k] * G + (nb - N)] += c;
        }
    }
    for (int m = 0; m < 7; m++) self[(size_t)m * N + i] = pb[m];
    if (!geo) return;
    // the reconstruction gradients' part of the least-squares weights' adjoint
    for (int s = 0; s < nf; s++) {
        const int nb = v.cell_nbr[s * N + i];
        for (int k = 0; k < NV; k++) {
            const double du = pr[in[k] * NT + nb].re - ui[k];
            for (int d = 0; d < 3; d++) wb[s][d] += gb[k][d] * du;
        }
    }
    lsq_geometry_adjoint<DIM>(v, a, i, nf, wb, ccs);
    for (int s = 0; s < nf; s++) {
        const int f = v.cell_face[s * N + i];
        const int side = v.outsign[s * N + i] > 0 ? 0 : 1;
        for (int d = 0; d < 3; d++) {
            a.geo_fcb[((size_t)side * 3 + d) * F + f] = fcs[s][d];
            ccs[d] -= fcs[s][d];
        }
    }
    for (int d = 0; d < 3; d++) a.geo_cell[(size_t)d * NT + i] = ccs[d];
}

// Pass 3, per valid cell: the primitive adjoint (own part, what its valid
// neighbours sent back through the same face, and the ghosts it fills, through
// the transposed ghost actions), then back through conserved_to_primatives to U.
template <int DIM>
__global__ void __launch_bounds__(kBlock) k_adj_final(DevView v, FvParams prm, int reconstruct, AdjScratch a,
                                                      double* out, double* gout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    const double* self = a.self;
    const double* nba = a.nba;
    const double* ga = a.ga;
    const signed char* back = a.back;
    constexpr int NC = DIM + 2, NV = DIM == 3 ? 5 : 4;
    const int N = v.N, G = v.G, NT = v.NT, MF = v.MF;
    const Dual* pr = (const Dual*)v.prim;
    double pb[7];
    for (int m = 0; m < 7; m++) pb[m] = self[(size_t)m * N + i];
    if (reconstruct || prm.viscous) {
        const int nf = v.nfaces[i];
        double cb[3] = {0.0, 0.0, 0.0};
        for (int s = 0; s < nf; s++) {
            const int nb = v.cell_nbr[s * N + i];
            if (nb >= N) continue;
            const int bs = back[s * N + i];
            if (bs < 0) continue;  // no face back to this cell (cannot happen on a conforming grid)
            for (int m = 0; m < 7; m++) pb[m] += nba[((size_t)m * MF + bs) * N + nb];
            if (a.geo_cell)
                for (int d = 0; d < 3; d++) cb[d] += a.geo_nbc[((size_t)d * MF + bs) * N + nb];
        }
        if (a.geo_cell)
            for (int d = 0; d < 3; d++) a.geo_cell[(size_t)d * NT + i] += cb[d];
    }
    // ghosts filled from this cell (fill_ghost's pre-reconstruction actions)
    const double* fg = (const double*)v.face;
    for (int e = v.feed_off[i]; e < v.feed_off[i + 1]; e++) {
        const int g = v.feed_ghost[e];
        double gb[7];
        for (int m = 0; m < 7; m++) gb[m] = ga[(size_t)m * G + g];
        if (gout)
            for (int m = 0; m < 7; m++) gout[(size_t)g * 7 + m] = gb[m];
        const BoundDev& B = v.bounds[v.ghost_bound[g]];
        const int f = v.ghost_face[g];
        double gvb[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        if (prm.viscous)
            for (int q = 0; q < 5; q++) gvb[q] = a.gav[(size_t)q * G + g];
        if (a.geo_face) {  // the ghost's dependence on its face's frame (slip-wall reflection)
            constexpr int kRead[9] = {0, 1, 3, 4, 8, 2, 5, 6, 7};
            constexpr int NG = DIM == 3 ? 9 : 5;
            StateT<DualA> src{DualA(pr[i].re), DualA(pr[NT + i].re), DualA(pr[2 * NT + i].re),
                              DualA(pr[3 * NT + i].re), DualA(pr[4 * NT + i].re), DualA(pr[5 * NT + i].re),
                              DualA(pr[6 * NT + i].re)};
            for (int jj = 0; jj < NG; jj++) {
                const int j = kRead[jj];
                DualA gl[9];
                for (int k = 0; k < 9; k++) {
                    const bool unread = DIM == 2 && (k == 2 || k == 5 || k == 6 || k == 7);
                    gl[k] = DualA(unread ? 0.0 : fg[k * v.F + f], k == j ? 1.0 : 0.0);
                }
                StateT<DualA> gh = src;
                apply_actions<DualA, DualA>(B.pre, B.n_pre, gh, src, gl, 1, 0, prm, v.gfix, G, g);
                double d = gb[0] * gh.rho.du + gb[1] * gh.p.du + gb[2] * gh.T.du + gb[3] * gh.e.du +
                           gb[4] * gh.vx.du + gb[5] * gh.vy.du + gb[6] * gh.vz.du;
                if (prm.viscous) {  // the pre-viscous actions continue from the pre-reconstruction ghost
                    apply_actions<DualA, DualA>(B.visc, B.n_visc, gh, src, gl, 1, 0, prm, v.gfix, G, g);
                    d += gvb[0] * gh.p.du + gvb[1] * gh.T.du + gvb[2] * gh.vx.du + gvb[3] * gh.vy.du +
                         gvb[4] * gh.vz.du;
                }
                a.geo_face[(size_t)j * v.F + f] += d;
            }
        }
        if (a.fs_ghost) {  // the ghost's dependence on its boundary's flow state, one seed per entry
            bool uses = false;
            for (int k = 0; k < B.n_pre; k++) uses |= B.pre[k].kind == aFlowStateCopy || B.pre[k].kind == aSubsonicInflow;
            if (prm.viscous)
                for (int k = 0; k < B.n_visc; k++)
                    uses |= B.visc[k].kind == aFlowStateCopy || B.visc[k].kind == aSubsonicInflow;
            if (uses) {
                StateT<DualA> src{DualA(pr[i].re), DualA(pr[NT + i].re), DualA(pr[2 * NT + i].re),
                                  DualA(pr[3 * NT + i].re), DualA(pr[4 * NT + i].re), DualA(pr[5 * NT + i].re),
                                  DualA(pr[6 * NT + i].re)};
                for (int j = 0; j < 7; j++) {
                    double dir[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
                    dir[j] = 1.0;
                    StateT<DualA> gh = src;
                    apply_actions<DualA, double>(B.pre, B.n_pre, gh, src, fg, v.F, f, prm, v.gfix, G, g, nullptr, dir);
                    double d = gb[0] * gh.rho.du + gb[1] * gh.p.du + gb[2] * gh.T.du + gb[3] * gh.e.du +
                               gb[4] * gh.vx.du + gb[5] * gh.vy.du + gb[6] * gh.vz.du;
                    if (prm.viscous) {
                        apply_actions<DualA, double>(B.visc, B.n_visc, gh, src, fg, v.F, f, prm, v.gfix, G, g, nullptr,
                                                     dir);
                        d += gvb[0] * gh.p.du + gvb[1] * gh.T.du + gvb[2] * gh.vx.du + gvb[3] * gh.vy.du +
                             gvb[4] * gh.vz.du;
                    }
                    a.fs_ghost[(size_t)g * 7 + j] += d;
                }
            }
        }
        for (int m = 0; m < 7; m++) {
            double sv[7];
            for (int q = 0; q < 7; q++) sv[q] = pr[q * NT + i].re;
            StateT<DualA> src{DualA(sv[0], m == 0), DualA(sv[1], m == 1), DualA(sv[2], m == 2),
                              DualA(sv[3], m == 3), DualA(sv[4], m == 4), DualA(sv[5], m == 5),
                              DualA(sv[6], m == 6)};
            StateT<DualA> gh = src;
            apply_actions<DualA, double>(B.pre, B.n_pre, gh, src, fg, v.F, f, prm, v.gfix, G, g);
            pb[m] += gb[0] * gh.rho.du + gb[1] * gh.p.du + gb[2] * gh.T.du + gb[3] * gh.e.du +
                     gb[4] * gh.vx.du + gb[5] * gh.vy.du + gb[6] * gh.vz.du;
            if (prm.viscous) {  // the pre-viscous actions continue from the pre-reconstruction ghost
                apply_actions<DualA, double>(B.visc, B.n_visc, gh, src, fg, v.F, f, prm, v.gfix, G, g);
                pb[m] += gvb[0] * gh.p.du + gvb[1] * gh.T.du + gvb[2] * gh.vx.du + gvb[3] * gh.vy.du +
                         gvb[4] * gh.vz.du;
            }
        }
    }
    if (!out) return;
    // conserved_to_primatives (primative_conserved_conversion.cpp:4-23), one seed per component
    for (int j = 0; j < NC; j++) {
        DualA u[NC];
        for (int q = 0; q < NC; q++) u[q] = DualA(v.U[q * N + i], q == j ? 1.0 : 0.0);
        DualA rho = u[0];
        DualA vx = u[1] / rho;
        DualA vy = u[2] / rho;
        DualA vz = DIM == 3 ? u[3] / rho : DualA(0.0);
        DualA ke = DualA(0.5) * (vx * vx + vy * vy + vz * vz);
        DualA e = u[DIM + 1] / rho - ke;
        DualA T = e / DualA(prm.Cv);
        DualA p = rho * DualA(prm.R) * T;
        out[(size_t)i * NC + j] = pb[0] * rho.du + pb[1] * p.du + pb[2] * T.du + pb[3] * e.du + pb[4] * vx.du +
                                  pb[5] * vy.du + pb[6] * vz.du;
    }
}

// Face centres: the two side cells' reconstruction / limiter terms.
__global__ void __launch_bounds__(kBlock) k_adj_geo_face(int F, AdjScratch a) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    for (int d = 0; d < 3; d++)
        a.geo_face[(size_t)(9 + d) * F + f] = a.geo_fcb[(size_t)d * F + f] + a.geo_fcb[(size_t)(3 + d) * F + f];
}

}  // namespace k_tan

void launch_adjoint_geometry(const DevView& v, const FvParams& p, const double* w, bool reconstruct,
                             const AdjScratch& a, cudaStream_t s) {
    using namespace k_tan;
    const unsigned bn = blocks_for(v.N), bf = blocks_for(v.F);
    if (v.G > 0) cudaMemsetAsync(a.ga, 0, sizeof(double) * 7 * v.G, s);
    if (v.G > 0 && p.viscous) cudaMemsetAsync(a.gav, 0, sizeof(double) * 5 * v.G, s);
    cudaMemsetAsync(a.geo_cell, 0, sizeof(double) * 4 * (size_t)v.NT, s);
    cudaMemsetAsync(a.geo_fcb, 0, sizeof(double) * 6 * (size_t)v.F, s);
    cudaMemsetAsync(a.geo_vb, 0, sizeof(double) * 2 * (size_t)v.F, s);
    if (v.dim == 3) {
        k_tan_prims<3><<<bn, kBlock, 0, s>>>(v, p, nullptr);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, double, 3, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_adj_face<3><<<bf, kBlock, 0, s>>>(v, p, w, reconstruct, a);
        k_adj_cell<3><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a);
        k_adj_final<3><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a, nullptr, nullptr);
    } else {
        k_tan_prims<2><<<bn, kBlock, 0, s>>>(v, p, nullptr);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, double, 2, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_adj_face<2><<<bf, kBlock, 0, s>>>(v, p, w, reconstruct, a);
        k_adj_cell<2><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a);
        k_adj_final<2><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a, nullptr, nullptr);
    }
    k_adj_geo_face<<<bf, kBlock, 0, s>>>(v.F, a);
}

void launch_adjoint(const DevView& v, const FvParams& p, const double* w, bool reconstruct, const AdjScratch& a,
                    double* out, double* ghost_out, cudaStream_t s) {
    using namespace k_tan;
    const unsigned bn = blocks_for(v.N), bf = blocks_for(v.F);
    if (v.G > 0) cudaMemsetAsync(a.ga, 0, sizeof(double) * 7 * v.G, s);
    if (v.G > 0 && p.viscous) cudaMemsetAsync(a.gav, 0, sizeof(double) * 5 * v.G, s);
    if (v.dim == 3) {
        k_tan_prims<3><<<bn, kBlock, 0, s>>>(v, p, nullptr);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, double, 3, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_adj_face<3><<<bf, kBlock, 0, s>>>(v, p, w, reconstruct, a);
        k_adj_cell<3><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a);
        k_adj_final<3><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a, out, ghost_out);
    } else {
        k_tan_prims<2><<<bn, kBlock, 0, s>>>(v, p, nullptr);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, double, 2, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_adj_face<2><<<bf, kBlock, 0, s>>>(v, p, w, reconstruct, a);
        k_adj_cell<2><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a);
        k_adj_final<2><<<bn, kBlock, 0, s>>>(v, p, reconstruct, a, out, ghost_out);
    }
}

void launch_tangent_geometry(const DevView& v0, const FvParams& p, const double* dface, const double* dcell,
                             bool reconstruct, const GeoTangent& g, double* out, cudaStream_t s) {
    using namespace k_tan;
    const int F = v0.F, NT = v0.NT, N = v0.N;
    const long long nseed = std::max<long long>(13LL * F, 3LL * NT);
    k_geo_seed<<<(unsigned)((nseed + kBlock - 1) / kBlock), kBlock, 0, s>>>(
        (const double*)v0.face, (const double*)v0.cc, v0.vol, dface, dcell, F, NT, N, (Dual*)g.face, (Dual*)g.cc,
        (Dual*)g.vol);
    DevView v = v0;
    v.face = g.face;
    v.cc = g.cc;
    v.r = g.r;
    const unsigned bn = blocks_for(N), bf = blocks_for(F);
    if (v.dim == 3) {
        if (reconstruct || p.viscous) k_geo_r<3><<<bn, kBlock, 0, s>>>(v, (const Dual*)g.cc, (Dual*)g.r);
        k_tan_prims<3, Dual><<<bn, kBlock, 0, s>>>(v, p, nullptr);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, Dual, 3, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_face<Dual, Dual, Dual, 3, true><<<bf, kBlock, 0, s>>>(v, p, reconstruct);
        k_geo_tan_update<3><<<bn, kBlock, 0, s>>>(v, (const Dual*)g.face, (const Dual*)g.vol, out);
    } else {
        if (reconstruct || p.viscous) k_geo_r<2><<<bn, kBlock, 0, s>>>(v, (const Dual*)g.cc, (Dual*)g.r);
        k_tan_prims<2, Dual><<<bn, kBlock, 0, s>>>(v, p, nullptr);
        if (reconstruct || p.viscous) k_recon<Dual, Dual, Dual, 2, true><<<bn, kBlock, 0, s>>>(v, p, reconstruct);
        k_face<Dual, Dual, Dual, 2, true><<<bf, kBlock, 0, s>>>(v, p, reconstruct);
        k_geo_tan_update<2><<<bn, kBlock, 0, s>>>(v, (const Dual*)g.face, (const Dual*)g.vol, out);
    }
}

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
