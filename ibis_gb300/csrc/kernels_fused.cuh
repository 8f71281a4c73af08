// Fused Runge-Kutta stage for structured blocks (mixed precision, inviscid,
// second order): one CTA per tile of cells does the whole stage in shared
// memory, so every primitive is read from HBM once per stage instead of once
// for the gradients, twice per face and again for the update.
//
//   1. load the reconstructed variables and centroids of the tile and a halo of
//      two cells (ghost cells on block sides) into shared memory;
//   2. least-squares gradients and Barth-Jespersen limiters of the tile's cells
//      and of the first halo layer that shares a face with them, kept in shared
//      memory as limiter-scaled gradients;
//   3. every face of the tile's cells: MUSCL reconstruction of both sides, thermo
//      closure, flux in the face frame, into shared memory;
//   4. per cell: surface integral as a float pair, then the same double-precision
//      stage combination, inversion and ghost refill as k_update, writing the new
//      primitives into the other primitive buffer (tiles still reading the old
//      state are not disturbed).
//
// The arithmetic is that of the generic mixed kernels (same formulas, float
// reconstruction and fluxes, double update); faces are evaluated along +i/+j/+k,
// so the flux of a face whose reference normal points the other way is the
// mirror evaluation F(-n; R, L) = -F(n; L, R), equal up to rounding.
#pragma once

#include "sblock.hpp"

namespace ibisgb {
namespace IBISGB_KNS {

template <int DIM>
struct FusedTile {
    static constexpr int X = DIM == 3 ? 8 : 16, Y = DIM == 3 ? 8 : 16, Z = DIM == 3 ? 4 : 1;
    static constexpr int HZ = DIM == 3 ? 2 : 0, HZ1 = DIM == 3 ? 1 : 0;  // halos along k
    static constexpr int RX = X + 4, RY = Y + 4, RZ = Z + 2 * HZ, R2 = RX * RY * RZ;  // cells + 2 halos
    static constexpr int QX = X + 2, QY = Y + 2, QZ = Z + 2 * HZ1, R1 = QX * QY * QZ;  // cells + 1 halo
    static constexpr int NV = DIM == 3 ? 5 : 4, NC = DIM + 2;
    static constexpr int FXN = (X + 1) * Y * Z, FYN = X * (Y + 1) * Z, FZN = DIM == 3 ? X * Y * (Z + 1) : 0;
    static constexpr int NF = FXN + FYN + FZN;
    static constexpr int kThreads = X * Y * Z;
    static constexpr size_t kFloats = (size_t)NV * R2 + (size_t)DIM * R2 + (size_t)NV * DIM * R1 +
                                      (size_t)NC * NF + NF;
    static constexpr size_t kSmem = kFloats * sizeof(float) + R2;
};

// lattice face of direction a at lattice position (i, j, k) (the face on the -a side of that cell)
IBISGB_HD int lattice_face(const SBlock& B, int a, int i, int j, int k) {
    if (a == 0) return B.f0[0] + i + (B.ni + 1) * (j + B.nj * k);
    if (a == 1) return B.f0[1] + i + B.ni * (j + (B.nj + 1) * k);
    return B.f0[2] + i + B.ni * (j + B.nj * k);
}

template <int DIM>
__global__ void __launch_bounds__(FusedTile<DIM>::kThreads, DIM == 3 ? 2 : 3)
    k_fused_stage(DevView v, SbView sb, FvParams prm, int mode, int stage, int with_dt) {
    using T = FusedTile<DIM>;
    constexpr int X = T::X, Y = T::Y, Z = T::Z, HZ = T::HZ, HZ1 = T::HZ1;
    constexpr int RX = T::RX, RY = T::RY, R2 = T::R2, QX = T::QX, QY = T::QY, R1 = T::R1;
    constexpr int NV = T::NV, NC = T::NC, NF = T::NF, FXN = T::FXN, FYN = T::FYN;
    extern __shared__ float smem[];
    float* Qs = smem;                    // [NV][R2] reconstructed variables
    float* Cs = Qs + NV * R2;            // [DIM][R2] centroids
    float* Gs = Cs + DIM * R2;           // [NV*DIM][R1] limiter-scaled gradients
    float* Fs = Gs + NV * DIM * R1;      // [NC][NF] face fluxes (per unit area)
    float* As = Fs + NC * NF;            // [NF] face areas
    signed char* Ks = (signed char*)(As + NF);  // [R2] 0 absent, 1 valid cell, 2 ghost

    const STile tile = sb.tiles[blockIdx.x];
    const SBlock B = sb.blocks[tile.block];
    const int NT = v.NT, N = v.N, SF = sb.SF;
    const float* pr = (const float*)v.prim;
    const float* cc = (const float*)v.cc;
    const float* rr = (const float*)v.r;
    const float* fg = sb.face;
    int ia, ib;
    thermo_vars(prm.thermo, ia, ib);
    const int vidx[5] = {ia, ib, 4, 5, 6};

    // ---- 1. tile + two halo layers
    for (int p = threadIdx.x; p < R2; p += blockDim.x) {
        const int x = p % RX, y = (p / RX) % RY, z = p / (RX * RY);
        const int gi = tile.i0 - 2 + x, gj = tile.j0 - 2 + y, gk = tile.k0 - HZ + z;
        const int oi = gi < 0 ? -1 : (gi >= B.ni ? 1 : 0);
        const int oj = gj < 0 ? -1 : (gj >= B.nj ? 1 : 0);
        const int ok = gk < 0 ? -1 : (gk >= B.nk ? 1 : 0);
        int id = -1;
        signed char kind = 0;
        if (!oi && !oj && !ok) {
            id = B.c0 + gi + B.ni * (gj + B.nj * gk);
            kind = 1;
        } else if ((oi != 0) + (oj != 0) + (ok != 0) == 1) {  // the ghost layer behind a block side
            if (oi && (gi == -1 || gi == B.ni)) id = sb.ghost_map[B.g0[oi < 0 ? 0 : 1] + gj + B.nj * gk];
            if (oj && (gj == -1 || gj == B.nj)) id = sb.ghost_map[B.g0[oj < 0 ? 2 : 3] + gi + B.ni * gk];
            if (ok && (gk == -1 || gk == B.nk)) id = sb.ghost_map[B.g0[ok < 0 ? 4 : 5] + gi + B.ni * gj];
            kind = id >= 0 ? 2 : 0;
        }
        Ks[p] = kind;
        if (kind) {
#pragma unroll
            for (int q = 0; q < NV; q++) Qs[q * R2 + p] = pr[vidx[q] * NT + id];
#pragma unroll
            for (int d = 0; d < DIM; d++) Cs[d * R2 + p] = cc[d * NT + id];
        }
    }
    __syncthreads();

    // ---- 2. gradients and limiters of the cells that share a face with the tile
    for (int p1 = threadIdx.x; p1 < R1; p1 += blockDim.x) {
        const int x1 = p1 % QX, y1 = (p1 / QX) % QY, z1 = p1 / (QX * QY);
        const int out = (x1 < 1 || x1 > X) + (y1 < 1 || y1 > Y) + (DIM == 3 && (z1 < 1 || z1 > Z));
        if (out > 1) continue;
        const int x = x1 + 1, y = y1 + 1, z = z1 + (HZ - HZ1);
        const int p = x + RX * (y + RY * z);
        if (Ks[p] != 1) continue;  // ghost sides are first order
        const int gi = tile.i0 - 2 + x, gj = tile.j0 - 2 + y, gk = tile.k0 - HZ + z;
        const int c = B.c0 + gi + B.ni * (gj + B.nj * gk);
        // WLSGradient weights from the QR factors (gradient.h:119-162)
        const float r11 = rr[c], r12 = rr[N + c], r22 = rr[2 * N + c];
        const float r13 = DIM == 3 ? rr[3 * N + c] : 0.f, r23 = DIM == 3 ? rr[4 * N + c] : 0.f;
        const float r33 = DIM == 3 ? rr[5 * N + c] : 1.f;
        const float q12 = r12 / r11, q23 = r23 / r22;
        const float i11 = 1.f / (r11 * r11), i22 = 1.f / (r22 * r22), i33 = 1.f / (r33 * r33);
        const float beta = DIM == 3 ? (r12 * r23 - r13 * r23) / (r11 * r22) : 0.f;
        const float xi = Cs[p], yi = Cs[R2 + p], zi = DIM == 3 ? Cs[2 * R2 + p] : 0.f;
        float ui[NV], gx[NV], gy[NV], gz[NV], umin[NV], umax[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) {
            ui[q] = Qs[q * R2 + p];
            gx[q] = 0.f; gy[q] = 0.f; gz[q] = 0.f;
            umin[q] = ui[q]; umax[q] = ui[q];
        }
        const int nbo[6] = {-1, 1, -RX, RX, -RX * RY, RX * RY};
#pragma unroll
        for (int d = 0; d < 2 * DIM; d++) {
            const int pn = p + nbo[d];
            const float dx = Cs[pn] - xi, dy = Cs[R2 + pn] - yi, dz = DIM == 3 ? Cs[2 * R2 + pn] - zi : 0.f;
            const float a1 = dx * i11;
            const float a2 = i22 * (dy - q12 * dx);
            const float a3 = DIM == 3 ? i33 * (dz - q23 * dy + beta * dx) : 0.f;
            const float w1 = a1 - q12 * a2 + beta * a3, w2 = a2 - q23 * a3, w3 = a3;
#pragma unroll
            for (int q = 0; q < NV; q++) {
                const float un = Qs[q * R2 + pn];
                const float du = un - ui[q];
                gx[q] += w1 * du; gy[q] += w2 * du;
                if (DIM == 3) gz[q] += w3 * du;
                umin[q] = fminf(umin[q], un);
                umax[q] = fmaxf(umax[q], un);
            }
        }
        float phi[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) phi[q] = 1.f;
        if (prm.limiter) {
            // Barth-Jespersen (limiter.cpp:23-63) in the two-division form of k_recon
            float tpos[NV], tneg[NV];
#pragma unroll
            for (int q = 0; q < NV; q++) { tpos[q] = 0.f; tneg[q] = 0.f; }
#pragma unroll
            for (int d = 0; d < 2 * DIM; d++) {
                const int a = d >> 1;
                const int s = lattice_face(B, a, gi + (a == 0 && (d & 1)), gj + (a == 1 && (d & 1)),
                                           gk + (a == 2 && (d & 1)));
                const float dx = fg[4 * SF + s] - xi, dy = fg[5 * SF + s] - yi;
                const float dz = DIM == 3 ? fg[6 * SF + s] - zi : 0.f;
#pragma unroll
                for (int q = 0; q < NV; q++) {
                    const float d2 = DIM == 3 ? gx[q] * dx + gy[q] * dy + gz[q] * dz : gx[q] * dx + gy[q] * dy;
                    tpos[q] = fmaxf(tpos[q], d2);
                    tneg[q] = fminf(tneg[q], d2);
                }
            }
            const float eps = prm.feps;
#pragma unroll
            for (int q = 0; q < NV; q++) {
                if (tpos[q] > 0.f) phi[q] = fminf(phi[q], (umax[q] - ui[q]) / (tpos[q] + eps));
                if (tneg[q] < 0.f) phi[q] = fminf(phi[q], (umin[q] - ui[q]) / (tneg[q] - eps));
            }
        }
#pragma unroll
        for (int q = 0; q < NV; q++) {
            Gs[(q * DIM) * R1 + p1] = gx[q] * phi[q];
            Gs[(q * DIM + 1) * R1 + p1] = gy[q] * phi[q];
            if (DIM == 3) Gs[(q * DIM + 2) * R1 + p1] = gz[q] * phi[q];
        }
    }
    __syncthreads();

    // ---- 3. face fluxes
    const Gas<float> gm(prm);
    for (int fl = threadIdx.x; fl < NF; fl += blockDim.x) {
        int a, fx, fy, fz;
        if (fl < FXN) { a = 0; fx = fl % (X + 1); fy = (fl / (X + 1)) % Y; fz = fl / ((X + 1) * Y); }
        else if (fl < FXN + FYN) { const int t = fl - FXN; a = 1; fx = t % X; fy = (t / X) % (Y + 1); fz = t / (X * (Y + 1)); }
        else { const int t = fl - FXN - FYN; a = 2; fx = t % X; fy = (t / X) % Y; fz = t / (X * Y); }
        const int gi = tile.i0 + fx, gj = tile.j0 + fy, gk = tile.k0 + fz;
        const bool exists = (gi < B.ni + (a == 0)) && (gj < B.nj + (a == 1)) && (gk < B.nk + (a == 2));
        if (!exists) {
            As[fl] = 0.f;
#pragma unroll
            for (int q = 0; q < NC; q++) Fs[q * NF + fl] = 0.f;
            continue;
        }
        const int s = lattice_face(B, a, gi, gj, gk);
        const float nx = fg[s], ny = fg[SF + s], nz = DIM == 3 ? fg[2 * SF + s] : 0.f;
        const float fcx = fg[4 * SF + s], fcy = fg[5 * SF + s], fcz = DIM == 3 ? fg[6 * SF + s] : 0.f;
        float t1x, t1y, t1z = 0.f, t2x = 0.f, t2y = 0.f, t2z = 0.f;
        if (DIM == 3) {
            const float ax = fabsf(nx), ay = fabsf(ny), az = fabsf(nz);
            const bool ex = ax <= ay && ax <= az, ey = !ex && ay <= az;
            t1x = ex ? 0.f : (ey ? -nz : ny);
            t1y = ex ? nz : (ey ? 0.f : -nx);
            t1z = ex ? -ny : (ey ? nx : 0.f);
            const float inv = rsqrtf(t1x * t1x + t1y * t1y + t1z * t1z);
            t1x *= inv; t1y *= inv; t1z *= inv;
            t2x = ny * t1z - nz * t1y;
            t2y = nz * t1x - nx * t1z;
            t2z = nx * t1y - ny * t1x;
        } else {
            t1x = -ny; t1y = nx;  // n = t1 x z in 2-D
        }
        // lower and upper cells in halo-2 coordinates
        const int xu = fx + 2, yu = fy + 2, zu = fz + HZ;
        const int pu = xu + RX * (yu + RY * zu);
        const int pl = pu - (a == 0 ? 1 : (a == 1 ? RX : RX * RY));
        FaceSide<float> S[2];
#pragma unroll
        for (int side = 0; side < 2; side++) {
            const int p = side ? pu : pl;
            float rv[NV];  // reconstructed variables: thermo pair, vx, vy[, vz]
#pragma unroll
            for (int w = 0; w < NV; w++) rv[w] = Qs[w * R2 + p];
            if (Ks[p] == 1) {
                const int x = p % RX, y = (p / RX) % RY, z = p / (RX * RY);
                const int p1 = (x - 1) + QX * ((y - 1) + QY * (z - (HZ - HZ1)));
                const float dx = fcx - Cs[p], dy = fcy - Cs[R2 + p], dz = DIM == 3 ? fcz - Cs[2 * R2 + p] : 0.f;
#pragma unroll
                for (int w = 0; w < NV; w++) {
                    float sgr = Gs[(w * DIM) * R1 + p1] * dx + Gs[(w * DIM + 1) * R1 + p1] * dy;
                    if (DIM == 3) sgr += Gs[(w * DIM + 2) * R1 + p1] * dz;
                    rv[w] = rv[w] + sgr;
                }
            }
            float q[7];
#pragma unroll
            for (int k = 0; k < 4; k++) q[k] = ia == k ? rv[0] : (ib == k ? rv[1] : 0.f);
            q[4] = rv[2]; q[5] = rv[3]; q[6] = DIM == 3 ? rv[4] : 0.f;
            thermo_close<float>(prm.thermo, gm, q[0], q[1], q[2], q[3]);
            S[side].r = q[0]; S[side].p = q[1]; S[side].T = q[2];
            if (DIM == 3) {
                S[side].u = q[4] * nx + q[5] * ny + q[6] * nz;
                S[side].v = q[4] * t1x + q[5] * t1y + q[6] * t1z;
                S[side].w = q[4] * t2x + q[5] * t2y + q[6] * t2z;
            } else {
                S[side].u = q[4] * nx + q[5] * ny;
                S[side].v = q[4] * t1x + q[5] * t1y;
                S[side].w = 0.f;
            }
        }
        float Fl[5];
        switch (prm.flux) {
            case kHanel: flux_hanel<float, DIM>(S[0], S[1], gm, Fl); break;
            case kAusmdv: flux_ausmdv<float, DIM>(S[0], S[1], gm, Fl); break;
            case kLdfss2: flux_ldfss2<float, DIM, false>(S[0], S[1], gm, prm.fdelta, Fl); break;
            default: flux_rusanov<float, DIM>(S[0], S[1], gm, Fl); break;
        }
        const float px = Fl[1], py = Fl[2], pz = DIM == 3 ? Fl[3] : 0.f;
        Fs[fl] = Fl[0];
        if (DIM == 3) {
            Fs[NF + fl] = px * nx + py * t1x + pz * t2x;
            Fs[2 * NF + fl] = px * ny + py * t1y + pz * t2y;
            Fs[3 * NF + fl] = px * nz + py * t1z + pz * t2z;
        } else {
            Fs[NF + fl] = px * nx + py * t1x;
            Fs[2 * NF + fl] = px * ny + py * t1y;
        }
        Fs[(DIM + 1) * NF + fl] = Fl[4];
        As[fl] = fg[3 * SF + s];
    }
    __syncthreads();

    // ---- 4. surface integral and update of the tile's cells
    const int t = threadIdx.x;
    const int tx = t % X, ty = (t / X) % Y, tz = t / (X * Y);
    const int gi = tile.i0 + tx, gj = tile.j0 + ty, gk = tile.k0 + tz;
    const bool active = gi < B.ni && gj < B.nj && gk < B.nk;
    const int i = active ? B.c0 + gi + B.ni * (gj + B.nj * gk) : N;
    double local = 1.0e308 * 10.0;
    if (active) {
        float hi[NC], lo[NC];
#pragma unroll
        for (int q = 0; q < NC; q++) { hi[q] = 0.f; lo[q] = 0.f; }
        // faces -i, +i, -j, +j[, -k, +k]: inflow through the lower face, outflow through the upper
        int fidx[6];
        fidx[0] = tx + (X + 1) * (ty + Y * tz);
        fidx[1] = fidx[0] + 1;
        fidx[2] = FXN + tx + X * (ty + (Y + 1) * tz);
        fidx[3] = fidx[2] + X;
        fidx[4] = FXN + FYN + tx + X * (ty + Y * tz);
        fidx[5] = fidx[4] + X * Y;
#pragma unroll
        for (int d = 0; d < 2 * DIM; d++) {
            const int f = fidx[d];
            const float sa = (d & 1) ? -As[f] : As[f];
#pragma unroll
            for (int q = 0; q < NC; q++) {
                const float x = Fs[q * NF + f];
                const float pp = __fmul_rn(x, sa);
                const float pe = __fmaf_rn(x, sa, -pp);
                two_sum_acc(hi[q], lo[q], pp);
                lo[q] = __fadd_rn(lo[q], pe);
            }
        }
        const bool fold = mode == 3 && stage > 0;
        const double iv = fold ? v.inv_vol[i] : 0.0;
        double ks[NC];
        if (!fold) {
            const float2 ivp = v.inv_vol2[i];
            double* kk = v.k + (size_t)kslot(v, stage) * NC * N;
#pragma unroll
            for (int q = 0; q < NC; q++) {
                ks[q] = pair_scale(hi[q], lo[q], ivp);
                kk[q * N + i] = ks[q];
            }
        }
        DevView vo = v;
        vo.prim = sb.prim_out;
        local = update_tail<float, float, DIM, false>(vo, prm, i, mode, stage, with_dt, ks, fold, hi, lo, iv);
        if (mode >= 2 && ctl_of(v, i)->halt) {
            // a halted case keeps its state: carry its primitives into the other buffer
            float* po = (float*)sb.prim_out;
            for (int q = 0; q < 7; q++) po[q * NT + i] = pr[q * NT + i];
            for (int k = v.feed_off[i]; k < v.feed_off[i + 1]; k++) {
                const int id = N + v.feed_ghost[k];
                for (int q = 0; q < 7; q++) po[q * NT + id] = pr[q * NT + id];
            }
        }
    }
    if (with_dt) reduce_local_dt(v, i, local);
}

inline void launch_fused(const DevView& v, const SbView& sb, const FvParams& prm, int mode, int stage,
                         int with_dt, cudaStream_t s) {
    if (v.dim == 3) {
        using T = FusedTile<3>;
        k_fused_stage<3><<<sb.num_tiles, T::kThreads, T::kSmem, s>>>(v, sb, prm, mode, stage, with_dt);
    } else {
        using T = FusedTile<2>;
        k_fused_stage<2><<<sb.num_tiles, T::kThreads, T::kSmem, s>>>(v, sb, prm, mode, stage, with_dt);
    }
}

inline cudaError_t prepare_fused() {
    cudaError_t e = cudaFuncSetAttribute(k_fused_stage<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)FusedTile<3>::kSmem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_fused_stage<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)FusedTile<2>::kSmem);
}

}  // namespace IBISGB_KNS
}  // namespace ibisgb
