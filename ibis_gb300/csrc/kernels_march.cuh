// Plane-marching fused Runge-Kutta stage for one 3-D structured block (mixed
// precision, inviscid, second order).
//
// One CTA of 256 threads owns a column of 32 x 8 cells in (i, j) and marches
// along k over a chunk of planes.  Each plane of the reconstructed variables and
// centroids (the column plus a halo of two cells) is staged into shared memory
// once, by TMA tensor copies (cp.async.bulk.tensor, completion on an mbarrier),
// into a ring of four plane slots; ghost cells behind the block sides are
// gathered into the same slots by plain loads.  Per plane k the CTA
//   1. issues the copy of plane k+3 into the slot of plane k-1;
//   2. evaluates the fluxes of plane k's i- and j-faces into shared memory, from
//      plane k's limiter-scaled gradients (one gradient slot);
//   3. forms the gradients of plane k+1 (the cells that share a face with the
//      column) from planes k, k+1 and k+2 into the gradient slot; each thread
//      also reconstructs its own cell's states at the cell's -k and +k faces,
//      which stay in registers;
//   4. evaluates the k-face between planes k and k+1 from those registers (the
//      +k state of plane k was formed one plane earlier; the k-face below plane
//      k was evaluated one plane earlier too);
//   5. applies the surface integral (float pair) and the double-precision stage
//      update, inversion and ghost refill of its 256 cells, as k_update does.
// Every primitive then crosses HBM about once per stage (plus the halo columns,
// which neighbouring columns read from L2), the gradients and fluxes never
// leave the SM, and the double-precision update of one CTA overlaps the float
// flux work of the other CTA on the same SM.
//
// The arithmetic is that of the tile-fused stage (kernels_fused.cuh): the same
// formulas in the same order (faces along +i/+j/+k, surface integral over the
// faces -i, +i, -j, +j, -k, +k).
//
// Requirements checked on the host (march_eligible): one block whose first cell
// index, i-extent and total cell count N+G are multiples of 4, so that every
// TMA copy starts on a 16-byte boundary and every tensor stride is a multiple of
// 16 bytes.  Each copy's innermost start coordinate is i0 - 4 with i0 a multiple
// of 32, i.e. a multiple of 4 floats = 16 bytes; starts below zero or boxes
// beyond the block read zeros, which are never used (or are overwritten by the
// ghost gather).  Waits on an mbarrier give up after about one second of clock
// cycles, set *sb.fault and end the CTA after a second bounded wait.
#pragma once

#include <cuda.h>

#include "sblock.hpp"

namespace ibisgb {
namespace IBISGB_KNS {

struct March {
    static constexpr int TX = 32, TY = 8, kThreads = TX * TY;
    // TMA box of one variable of one plane: columns i0-4 .. i0+TX+3 (the x start
    // is rounded down to 16 bytes; the halo needs i0-2 .. i0+TX+1), rows j0-2 .. j0+TY+1
    static constexpr int BW = TX + 8, BH = TY + 4, SLAB = BW * BH;  // 480 floats = 1920 bytes
    static constexpr int NQ = 8;                                    // 5 reconstructed variables + 3 centroid coordinates
    static constexpr int PLANE = NQ * SLAB;                         // floats per plane slot
    static constexpr int NSLOT = 4;
    static constexpr unsigned kPlaneBytes = PLANE * 4u;
    // gradient region: the column and the cells that share a face with it
    static constexpr int GW = TX + 2, GH = TY + 2, GN = GW * GH, NG = 15;
    static constexpr int GHALO = 2 * TX + 2 * TY;  // halo part of the gradient region (corners excluded)
    static constexpr int FIN = (TX + 1) * TY, FJN = TX * (TY + 1);  // in-plane i- and j-faces
    static constexpr size_t kSlotBytes = (size_t)NSLOT * PLANE * 4;
    static constexpr size_t kGradBytes = (size_t)NG * GN * 4;
    static constexpr size_t kFaceBytes = (size_t)6 * (FIN + FJN) * 4;
    static constexpr size_t kSmem = kSlotBytes + kGradBytes + kFaceBytes + 64 + 1024;  // + mbarriers + alignment
};
static_assert(March::SLAB * 4 % 128 == 0, "TMA destinations must stay 128-byte aligned");

// ---- PTX helpers (mbarrier, TMA)
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred P1;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 P1, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, P1;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}
// Wait for the phase of `parity` to complete, for at most ~2^31 clock cycles.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > (1ll << 31)) return false;
    return true;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6}], "
        "[%2];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
        : "memory");
}

// Position in the gradient region of the idx-th gradient cell of a plane: the
// column's cells first (one per thread), then its halo ring without corners.
IBISGB_HD void march_grad_pos(int idx, int& x1, int& y1) {
    constexpr int TX = March::TX, TY = March::TY;
    if (idx < TX * TY) { x1 = 1 + idx % TX; y1 = 1 + idx / TX; return; }
    idx -= TX * TY;
    if (idx < TX) { x1 = 1 + idx; y1 = 0; return; }
    idx -= TX;
    if (idx < TX) { x1 = 1 + idx; y1 = TY + 1; return; }
    idx -= TX;
    if (idx < TY) { x1 = 0; y1 = 1 + idx; return; }
    x1 = TX + 1; y1 = 1 + idx - TY;
}

struct MarchCtx {
    SBlock B;
    int i0, j0;
    int ia, ib;
    float* slots;   // [NSLOT][NQ][BH][BW]
    float* grads;   // [NG][GN] limiter-scaled gradients of one plane
    float* fi;      // [6][FIN]: flux components per unit area, area
    float* fj;      // [6][FJN]
    unsigned bar0;  // shared address of the first of NSLOT mbarriers
};

// slot of plane k (k >= -2)
__device__ __forceinline__ int march_si(int k) { return (k + 4) & 3; }
__device__ __forceinline__ float* march_slot(const MarchCtx& m, int k) { return m.slots + march_si(k) * March::PLANE; }

// Thread 0: TMA copies of plane k (an interior plane of the block) into its slot.
__device__ __forceinline__ void march_issue(const MarchCtx& m, const CUtensorMap* tm_prim, const CUtensorMap* tm_cc,
                                            int k) {
    if (k < 0 || k >= m.B.nk) return;
    const int s = march_si(k);
    const unsigned bar = m.bar0 + 8u * s;
    const unsigned dst = smem_u32(m.slots + s * March::PLANE);
    fence_proxy_async();  // earlier generic accesses of the slot before the async writes
    mbar_expect_tx(bar, March::kPlaneBytes);
    const int vidx[5] = {m.ia, m.ib, 4, 5, 6};
#pragma unroll
    for (int q = 0; q < 5; q++) tma_load_4d(dst + q * March::SLAB * 4, tm_prim, m.i0 - 4, m.j0 - 2, k, vidx[q], bar);
#pragma unroll
    for (int d = 0; d < 3; d++) tma_load_4d(dst + (5 + d) * March::SLAB * 4, tm_cc, m.i0 - 4, m.j0 - 2, k, d, bar);
}

// All threads: wait for plane k's copies (if it has any), then gather the ghost
// cells of its halo (a whole plane of ghosts behind the -k / +k sides).
// Returns false, after the fault flag is set, when the copies did not complete.
__device__ __forceinline__ bool march_arrive(const MarchCtx& m, const DevView& v, const SbView& sb, int k, unsigned& phases) {
    const SBlock& B = m.B;
    if (k < -1 || k > B.nk) return true;  // no cell of this plane is ever read
    if (k >= 0 && k < B.nk) {
        const int s = march_si(k);
        const unsigned bar = m.bar0 + 8u * s;
        const unsigned par = (phases >> s) & 1u;
        const bool ok = mbar_wait_bounded(bar, par);
        phases ^= 1u << s;
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicOr(sb.fault, 1u);
            mbar_wait_bounded(bar, par);  // the copies may still be in flight into this CTA's memory
            return false;
        }
    }
    const bool ghost_plane = k == -1 || k == B.nk;
    const bool edge = m.i0 < 2 || m.i0 + March::TX + 2 > B.ni || m.j0 < 2 || m.j0 + March::TY + 2 > B.nj;
    if (!ghost_plane && !edge) return true;
    float* S = march_slot(m, k);
    const float* pr = (const float*)v.prim;
    const float* cc = (const float*)v.cc;
    const int NT = v.NT;
    const int vidx[5] = {m.ia, m.ib, 4, 5, 6};
    for (int p = threadIdx.x; p < March::SLAB; p += blockDim.x) {
        const int c = p % March::BW, r = p / March::BW;
        if (c < 2 || c > March::TX + 5) continue;  // columns the stage never reads
        const int gi = m.i0 - 4 + c, gj = m.j0 - 2 + r;
        const bool ii = gi >= 0 && gi < B.ni, jj = gj >= 0 && gj < B.nj;
        int id = -1;
        // (ghost-map offsets selected by value: a computed index into B.g0 would
        // place the block descriptor in local memory)
        if (ghost_plane) {
            if (ii && jj) id = sb.ghost_map[(k < 0 ? B.g0[4] : B.g0[5]) + gi + B.ni * gj];
        } else if (!ii && jj && (gi == -1 || gi == B.ni)) {
            id = sb.ghost_map[(gi < 0 ? B.g0[0] : B.g0[1]) + gj + B.nj * k];
        } else if (ii && !jj && (gj == -1 || gj == B.nj)) {
            id = sb.ghost_map[(gj < 0 ? B.g0[2] : B.g0[3]) + gi + B.ni * k];
        }
        if (id < 0) continue;
#pragma unroll
        for (int q = 0; q < 5; q++) S[q * March::SLAB + p] = pr[vidx[q] * NT + id];
#pragma unroll
        for (int d = 0; d < 3; d++) S[(5 + d) * March::SLAB + p] = cc[d * NT + id];
    }
    __syncthreads();
    return true;
}

// Least-squares gradients and Barth-Jespersen limiters of the valid cells of
// plane k (0 <= k < nk) in the gradient region, from planes k-1, k, k+1, stored
// limiter-scaled (as in kernels_fused.cuh) unless tile_only.  The thread's own
// column cell (the first item of every thread) also returns its reconstructed
// variables at its -k face (Rm) and +k face (Rp).  A ghost plane (k = -1 or nk)
// returns the ghost's own values (ghost sides are first order).
__device__ __forceinline__ void march_gradients(const MarchCtx& m, const DevView& v, const SbView& sb,
                                                const FvParams& prm, int k, bool tile_only, float (&Rm)[5],
                                                float (&Rp)[5]) {
    constexpr int BW = March::BW, SLAB = March::SLAB, GW = March::GW, GN = March::GN;
    const SBlock& B = m.B;
    const float* S0 = march_slot(m, k);
    if (k < 0 || k >= B.nk) {
        const int p = (threadIdx.x % March::TX + 4) + BW * (threadIdx.x / March::TX + 2);
#pragma unroll
        for (int q = 0; q < 5; q++) Rm[q] = Rp[q] = S0[q * SLAB + p];
        return;
    }
    const float* Sm = march_slot(m, k - 1);
    const float* Sp = march_slot(m, k + 1);
    float* G = m.grads;
    const int N = v.N, SF = sb.SF;
    const float* rr = (const float*)v.r;
    const float* fg = sb.face;
    const int nitems = tile_only ? March::kThreads : March::kThreads + March::GHALO;
    for (int idx = threadIdx.x; idx < nitems; idx += blockDim.x) {
        int x1, y1;
        march_grad_pos(idx, x1, y1);
        const int gi = m.i0 - 1 + x1, gj = m.j0 - 1 + y1;
        if (gi < 0 || gi >= B.ni || gj < 0 || gj >= B.nj) continue;  // ghost sides are first order
        const int p = (x1 + 3) + BW * (y1 + 1);
        const int c = B.c0 + gi + B.ni * (gj + B.nj * k);
        // WLSGradient weights from the QR factors (gradient.h:119-162)
        const float r11 = rr[c], r12 = rr[N + c], r22 = rr[2 * N + c];
        const float r13 = rr[3 * N + c], r23 = rr[4 * N + c], r33 = rr[5 * N + c];
        const float q12 = r12 / r11, q23 = r23 / r22;
        const float i11 = 1.f / (r11 * r11), i22 = 1.f / (r22 * r22), i33 = 1.f / (r33 * r33);
        const float beta = (r12 * r23 - r13 * r23) / (r11 * r22);
        const float xi = S0[5 * SLAB + p], yi = S0[6 * SLAB + p], zi = S0[7 * SLAB + p];
        float ui[5], gx[5], gy[5], gz[5], umin[5], umax[5];
#pragma unroll
        for (int q = 0; q < 5; q++) {
            ui[q] = S0[q * SLAB + p];
            gx[q] = 0.f; gy[q] = 0.f; gz[q] = 0.f;
            umin[q] = ui[q]; umax[q] = ui[q];
        }
#pragma unroll
        for (int d = 0; d < 6; d++) {
            const float* Sn = d < 4 ? S0 : (d == 4 ? Sm : Sp);
            const int pn = d == 0 ? p - 1 : d == 1 ? p + 1 : d == 2 ? p - BW : d == 3 ? p + BW : p;
            const float dx = Sn[5 * SLAB + pn] - xi, dy = Sn[6 * SLAB + pn] - yi, dz = Sn[7 * SLAB + pn] - zi;
            const float a1 = dx * i11;
            const float a2 = i22 * (dy - q12 * dx);
            const float a3 = i33 * (dz - q23 * dy + beta * dx);
            const float w1 = a1 - q12 * a2 + beta * a3, w2 = a2 - q23 * a3, w3 = a3;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                const float un = Sn[q * SLAB + pn];
                const float du = un - ui[q];
                gx[q] += w1 * du; gy[q] += w2 * du; gz[q] += w3 * du;
                umin[q] = fminf(umin[q], un);
                umax[q] = fmaxf(umax[q], un);
            }
        }
        float phi[5];
#pragma unroll
        for (int q = 0; q < 5; q++) phi[q] = 1.f;
        // offsets of the -k and +k face centres (the column cell's k-face states)
        const int skm = lattice_face(B, 2, gi, gj, k), skp = lattice_face(B, 2, gi, gj, k + 1);
        const float dxm = fg[4 * SF + skm] - xi, dym = fg[5 * SF + skm] - yi, dzm = fg[6 * SF + skm] - zi;
        const float dxp = fg[4 * SF + skp] - xi, dyp = fg[5 * SF + skp] - yi, dzp = fg[6 * SF + skp] - zi;
        if (prm.limiter) {
            // Barth-Jespersen (limiter.cpp:23-63) in the two-division form of k_recon
            float tpos[5], tneg[5];
#pragma unroll
            for (int q = 0; q < 5; q++) { tpos[q] = 0.f; tneg[q] = 0.f; }
#pragma unroll
            for (int d = 0; d < 6; d++) {
                const int a = d >> 1;
                float dx, dy, dz;
                if (a < 2) {
                    const int s = lattice_face(B, a, gi + (a == 0 && (d & 1)), gj + (a == 1 && (d & 1)), k);
                    dx = fg[4 * SF + s] - xi; dy = fg[5 * SF + s] - yi; dz = fg[6 * SF + s] - zi;
                } else {
                    dx = d == 4 ? dxm : dxp; dy = d == 4 ? dym : dyp; dz = d == 4 ? dzm : dzp;
                }
#pragma unroll
                for (int q = 0; q < 5; q++) {
                    const float d2 = gx[q] * dx + gy[q] * dy + gz[q] * dz;
                    tpos[q] = fmaxf(tpos[q], d2);
                    tneg[q] = fminf(tneg[q], d2);
                }
            }
            const float eps = prm.feps;
#pragma unroll
            for (int q = 0; q < 5; q++) {
                if (tpos[q] > 0.f) phi[q] = fminf(phi[q], (umax[q] - ui[q]) / (tpos[q] + eps));
                if (tneg[q] < 0.f) phi[q] = fminf(phi[q], (umin[q] - ui[q]) / (tneg[q] - eps));
            }
        }
        const int p1 = x1 + GW * y1;
#pragma unroll
        for (int q = 0; q < 5; q++) {
            const float sx = gx[q] * phi[q], sy = gy[q] * phi[q], sz = gz[q] * phi[q];
            if (!tile_only) {
                G[(q * 3) * GN + p1] = sx;
                G[(q * 3 + 1) * GN + p1] = sy;
                G[(q * 3 + 2) * GN + p1] = sz;
            }
            if (idx < March::kThreads) {  // the thread's own column cell: its k-face states
                float sm = sx * dxm + sy * dym;
                sm += sz * dzm;
                float sp = sx * dxp + sy * dyp;
                sp += sz * dzp;
                Rm[q] = ui[q] + sm;
                Rp[q] = ui[q] + sp;
            }
        }
    }
}

// Flux (per unit area, momentum rotated back to x, y, z) of lattice face s from
// the reconstructed variables of its lower and upper sides (thermo pair, vx,
// vy, vz): thermo closure, rotation into the face frame, flux calculator.
__device__ __forceinline__ void march_flux(const FvParams& prm, const Gas<float>& gm, const float* fg, int SF, int s,
                                           const float (&rl)[5], const float (&ru)[5], int ia, int ib,
                                           float (&out)[5], float& area) {
    const float nx = fg[s], ny = fg[SF + s], nz = fg[2 * SF + s];
    area = fg[3 * SF + s];
    float t1x, t1y, t1z, t2x, t2y, t2z;
    {
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
    }
    FaceSide<float> S[2];
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const float(&rv)[5] = side ? ru : rl;
        float q[7];
#pragma unroll
        for (int k = 0; k < 4; k++) q[k] = ia == k ? rv[0] : (ib == k ? rv[1] : 0.f);
        q[4] = rv[2]; q[5] = rv[3]; q[6] = rv[4];
        thermo_close<float>(prm.thermo, gm, q[0], q[1], q[2], q[3]);
        S[side].r = q[0]; S[side].p = q[1]; S[side].T = q[2];
        S[side].u = q[4] * nx + q[5] * ny + q[6] * nz;
        S[side].v = q[4] * t1x + q[5] * t1y + q[6] * t1z;
        S[side].w = q[4] * t2x + q[5] * t2y + q[6] * t2z;
    }
    float Fl[5];
    switch (prm.flux) {
        case kHanel: flux_hanel<float, 3>(S[0], S[1], gm, Fl); break;
        case kAusmdv: flux_ausmdv<float, 3>(S[0], S[1], gm, Fl); break;
        case kLdfss2: flux_ldfss2<float, 3, false>(S[0], S[1], gm, prm.fdelta, Fl); break;
        default: flux_rusanov<float, 3>(S[0], S[1], gm, Fl); break;
    }
    const float px = Fl[1], py = Fl[2], pz = Fl[3];
    out[0] = Fl[0];
    out[1] = px * nx + py * t1x + pz * t2x;
    out[2] = px * ny + py * t1y + pz * t2y;
    out[3] = px * nz + py * t1z + pz * t2z;
    out[4] = Fl[4];
}

// Reconstructed variables of one side of an in-plane face: the slot values at
// position p, plus (a valid cell) its limiter-scaled gradient at gradient
// position g dotted with the face centre's offset from the cell centroid.
__device__ __forceinline__ void march_side(const float* S, int p, const float* G, int g, bool valid, float fcx,
                                           float fcy, float fcz, float (&rv)[5]) {
    constexpr int SLAB = March::SLAB, GN = March::GN;
#pragma unroll
    for (int w = 0; w < 5; w++) rv[w] = S[w * SLAB + p];
    if (valid) {
        const float dx = fcx - S[5 * SLAB + p], dy = fcy - S[6 * SLAB + p], dz = fcz - S[7 * SLAB + p];
#pragma unroll
        for (int w = 0; w < 5; w++) {
            float sgr = G[(w * 3) * GN + g] * dx + G[(w * 3 + 1) * GN + g] * dy;
            sgr += G[(w * 3 + 2) * GN + g] * dz;
            rv[w] = rv[w] + sgr;
        }
    }
}

// The k-face between planes k and k+1 of the thread's column, from the lower
// cell's +k state and the upper cell's -k state (zero flux and area outside the block).
__device__ __forceinline__ void march_kface(const MarchCtx& m, const FvParams& prm, const Gas<float>& gm,
                                            const SbView& sb, int k, const float (&rl)[5], const float (&ru)[5],
                                            float (&out)[5], float& area) {
    const int gi = m.i0 + threadIdx.x % March::TX, gj = m.j0 + threadIdx.x / March::TX;
    if (gi >= m.B.ni || gj >= m.B.nj) {
#pragma unroll
        for (int q = 0; q < 5; q++) out[q] = 0.f;
        area = 0.f;
        return;
    }
    march_flux(prm, gm, sb.face, sb.SF, lattice_face(m.B, 2, gi, gj, k + 1), rl, ru, m.ia, m.ib, out, area);
}

// i- and j-faces of plane k, into shared memory (gradients of plane k in the slot).
__device__ __forceinline__ void march_plane_faces(const MarchCtx& m, const FvParams& prm, const Gas<float>& gm,
                                                  const SbView& sb, int k) {
    constexpr int TX = March::TX, TY = March::TY, BW = March::BW, GW = March::GW;
    constexpr int FIN = March::FIN, FJN = March::FJN;
    const SBlock& B = m.B;
    const float* S = march_slot(m, k);
    const float* G = m.grads;
    const float* fg = sb.face;
    const int SF = sb.SF;
    // 2 x 256 faces (the -i and -j face of every cell of the column) + the +i faces of
    // the last column and the +j faces of the last row
    for (int idx = threadIdx.x; idx < 2 * TX * TY + TY + TX; idx += blockDim.x) {
        int a, x, y;
        if (idx < TX * TY) { a = 0; x = idx % TX; y = idx / TX; }
        else if (idx < 2 * TX * TY) { a = 1; x = (idx - TX * TY) % TX; y = (idx - TX * TY) / TX; }
        else if (idx < 2 * TX * TY + TY) { a = 0; x = TX; y = idx - 2 * TX * TY; }
        else { a = 1; x = idx - 2 * TX * TY - TY; y = TY; }
        float F[5], A;
        const int gi = m.i0 + x, gj = m.j0 + y;  // the upper cell
        const bool exists = a == 0 ? (gi <= B.ni && gj < B.nj) : (gi < B.ni && gj <= B.nj);
        if (exists) {
            const int s = lattice_face(B, a, gi, gj, k);
            const int pu = (x + 4) + BW * (y + 2), gu = (x + 1) + GW * (y + 1);
            const int pl = a == 0 ? pu - 1 : pu - BW, gl = a == 0 ? gu - 1 : gu - GW;
            const bool vl = a == 0 ? gi - 1 >= 0 : gj - 1 >= 0;
            const bool vu = a == 0 ? gi < B.ni : gj < B.nj;
            const float fcx = fg[4 * SF + s], fcy = fg[5 * SF + s], fcz = fg[6 * SF + s];
            float rl[5], ru[5];
            march_side(S, pl, G, gl, vl, fcx, fcy, fcz, rl);
            march_side(S, pu, G, gu, vu, fcx, fcy, fcz, ru);
            march_flux(prm, gm, fg, SF, s, rl, ru, m.ia, m.ib, F, A);
        } else {
#pragma unroll
            for (int q = 0; q < 5; q++) F[q] = 0.f;
            A = 0.f;
        }
        if (a == 0) {
            const int f = x + (TX + 1) * y;
#pragma unroll
            for (int q = 0; q < 5; q++) m.fi[q * FIN + f] = F[q];
            m.fi[5 * FIN + f] = A;
        } else {
            const int f = x + TX * y;
#pragma unroll
            for (int q = 0; q < 5; q++) m.fj[q * FJN + f] = F[q];
            m.fj[5 * FJN + f] = A;
        }
    }
}

// Surface integral and double-precision update of the thread's cell of plane k;
// returns the new state's local time step (with_dt) or +inf.
template <int MODE>
__device__ __forceinline__ double march_update(const MarchCtx& m, const DevView& v, const SbView& sb,
                                               const FvParams& prm, int mode_arg, int stage, int with_dt, int k,
                                               const float (&Fb)[5], float Ab, const float (&Ft)[5], float At) {
    constexpr int TX = March::TX, FIN = March::FIN, FJN = March::FJN, NC = 5;
    const int mode = MODE >= 0 ? MODE : mode_arg;
    const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
    const int gi = m.i0 + tx, gj = m.j0 + ty;
    if (gi >= m.B.ni || gj >= m.B.nj) return 1.0e308 * 10.0;
    const int N = v.N;
    const int i = m.B.c0 + gi + m.B.ni * (gj + m.B.nj * k);
    float hi[NC], lo[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) { hi[q] = 0.f; lo[q] = 0.f; }
    // faces -i, +i, -j, +j, -k, +k: inflow through the lower face, outflow through the upper
#pragma unroll
    for (int d = 0; d < 6; d++) {
        float x[5], A;
        if (d < 2) {
            const int f = tx + d + (TX + 1) * ty;
#pragma unroll
            for (int q = 0; q < NC; q++) x[q] = m.fi[q * FIN + f];
            A = m.fi[5 * FIN + f];
        } else if (d < 4) {
            const int f = tx + TX * (ty + (d - 2));
#pragma unroll
            for (int q = 0; q < NC; q++) x[q] = m.fj[q * FJN + f];
            A = m.fj[5 * FJN + f];
        } else {
#pragma unroll
            for (int q = 0; q < NC; q++) x[q] = d == 4 ? Fb[q] : Ft[q];
            A = d == 4 ? Ab : At;
        }
        const float sa = (d & 1) ? -A : A;
#pragma unroll
        for (int q = 0; q < NC; q++) {
            const float pp = __fmul_rn(x[q], sa);
            const float pe = __fmaf_rn(x[q], sa, -pp);
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
    const double local = update_tail<float, float, 3, false, MODE>(vo, prm, i, mode, stage, with_dt, ks, fold, hi,
                                                                  lo, iv);
    if (mode >= 2 && ctl_of(v, i)->halt) {
        // a halted case keeps its state: carry its primitives into the other buffer
        const float* pr = (const float*)v.prim;
        float* po = (float*)sb.prim_out;
        const int NT = v.NT;
        for (int q = 0; q < 7; q++) po[q * NT + i] = pr[q * NT + i];
        for (int kk = v.feed_off[i]; kk < v.feed_off[i + 1]; kk++) {
            const int id = N + v.feed_ghost[kk];
            for (int q = 0; q < 7; q++) po[q * NT + id] = pr[q * NT + id];
        }
    }
    return local;
}

// grid: columns x chunks (blockIdx.x = column + ncol * chunk); kc planes per chunk.
template <int MODE>
__global__ void __launch_bounds__(March::kThreads, 2)
    k_march_stage(DevView v, SbView sb, FvParams prm, const SBlock Bp, const __grid_constant__ CUtensorMap tm_prim,
                  const __grid_constant__ CUtensorMap tm_cc, int mode, int stage, int with_dt, int kc) {
    extern __shared__ unsigned char msm_raw[];
    unsigned char* base = msm_raw + ((1024u - (smem_u32(msm_raw) & 1023u)) & 1023u);  // 1024-byte aligned
    MarchCtx m;
    m.B = Bp;
    const int ncx = (m.B.ni + March::TX - 1) / March::TX, ncy = (m.B.nj + March::TY - 1) / March::TY;
    const int col = blockIdx.x % (ncx * ncy), chunk = blockIdx.x / (ncx * ncy);
    m.i0 = (col % ncx) * March::TX;
    m.j0 = (col / ncx) * March::TY;
    thermo_vars(prm.thermo, m.ia, m.ib);
    m.slots = (float*)base;
    m.grads = (float*)(base + March::kSlotBytes);
    m.fi = (float*)(base + March::kSlotBytes + March::kGradBytes);
    m.fj = m.fi + 6 * March::FIN;
    m.bar0 = smem_u32(base + March::kSlotBytes + March::kGradBytes + March::kFaceBytes);
    const int kb = chunk * kc, ke = min(kb + kc, m.B.nk);
    double local = 1.0e308 * 10.0;
    unsigned phases = 0u;   // parity of the next completion of each slot's mbarrier
    unsigned pending = 0u;  // slots with copies issued and not yet waited for (the same in every thread)
    const Gas<float> gm(prm);
    const int t = threadIdx.x;
    // copies of plane k (an interior plane) into its slot, issued by thread 0
#define MARCH_ISSUE(k_)                                                   \
    do {                                                                  \
        const int kq_ = (k_);                                             \
        if (kq_ >= 0 && kq_ < m.B.nk) {                                   \
            if (t == 0) march_issue(m, &tm_prim, &tm_cc, kq_);            \
            pending |= 1u << march_si(kq_);                             \
        }                                                                 \
    } while (0)
#define MARCH_ARRIVE(ok_, k_)                                             \
    do {                                                                  \
        const int kq_ = (k_);                                             \
        ok_ = march_arrive(m, v, sb, kq_, phases);                        \
        if (kq_ >= 0 && kq_ < m.B.nk) pending &= ~(1u << march_si(kq_)); \
    } while (0)

    if (t == 0) {
        for (int s = 0; s < March::NSLOT; s++) mbar_init(m.bar0 + 8u * s, 1u);
        fence_mbar_init();
    }
    __syncthreads();
    bool ok = true;
    if (kb < ke) {
        // prologue: planes kb-2 .. kb+1; the +k states of plane kb-1 (its column cells'
        // gradients); plane kb+2 (into the slot of kb-2); the gradients of plane kb and
        // its -k / +k states; the k-face below plane kb
        for (int k = kb - 2; k <= kb + 1; k++) MARCH_ISSUE(k);
        for (int k = kb - 2; k <= kb + 1 && ok; k++) MARCH_ARRIVE(ok, k);
        float Rp[5], Rm[5], Fb[5], Ab = 0.f;
        if (ok) {
            float Rx[5];
            march_gradients(m, v, sb, prm, kb - 1, true, Rx, Rp);
            __syncthreads();
            MARCH_ISSUE(kb + 2);
            float Rn[5];
            march_gradients(m, v, sb, prm, kb, false, Rm, Rn);
            march_kface(m, prm, gm, sb, kb - 1, Rp, Rm, Fb, Ab);
#pragma unroll
            for (int q = 0; q < 5; q++) Rp[q] = Rn[q];
            __syncthreads();
        }
        for (int k = kb; k < ke && ok; k++) {
            // planes k, k+1 resident and k+2 arriving; gradients of plane k in the slot;
            // Rp: the +k states of plane k; Fb: the k-face below plane k
            if (k + 1 < ke) MARCH_ISSUE(k + 3);  // into the slot of plane k-1
            march_plane_faces(m, prm, gm, sb, k);
            MARCH_ARRIVE(ok, k + 2);
            if (!ok) break;
            __syncthreads();
            float Rn[5];
            march_gradients(m, v, sb, prm, k + 1, false, Rm, Rn);
            float Ft[5], At;
            march_kface(m, prm, gm, sb, k, Rp, Rm, Ft, At);
            const double lk = march_update<MODE>(m, v, sb, prm, mode, stage, with_dt, k, Fb, Ab, Ft, At);
            local = fmin(local, lk);
#pragma unroll
            for (int q = 0; q < 5; q++) { Fb[q] = Ft[q]; Rp[q] = Rn[q]; }
            Ab = At;
            __syncthreads();
        }
    }
    if (!ok) {
        // a copy did not complete: wait (bounded) for the others still in flight
        // into this CTA's memory, and leave
        for (int s = 0; s < March::NSLOT; s++)
            if ((pending >> s) & 1u) mbar_wait_bounded(m.bar0 + 8u * s, (phases >> s) & 1u);
        return;
    }
    if (with_dt) reduce_local_dt(v, 0, local);
#undef MARCH_ISSUE
#undef MARCH_ARRIVE
}

// Host side: one block (hb, its host copy), columns of March::TX x March::TY
// cells, kc planes per CTA; tm_prim / tm_cc: the CUtensorMaps of the
// primitive buffer the stage reads and of the centroids.
inline void launch_march(const DevView& v, const SbView& sb, const SBlock& hb, const FvParams& prm,
                         const void* tm_prim, const void* tm_cc, int mode, int stage, int with_dt, int kc,
                         cudaStream_t s) {
    const int ncx = (hb.ni + March::TX - 1) / March::TX, ncy = (hb.nj + March::TY - 1) / March::TY;
    const int nch = (hb.nk + kc - 1) / kc;
    const CUtensorMap& mp = *(const CUtensorMap*)tm_prim;
    const CUtensorMap& mc = *(const CUtensorMap*)tm_cc;
    const unsigned grid = (unsigned)(ncx * ncy * nch);
    if (mode == 2)
        k_march_stage<2><<<grid, March::kThreads, March::kSmem, s>>>(v, sb, prm, hb, mp, mc, mode, stage, with_dt, kc);
    else if (mode == 3)
        k_march_stage<3><<<grid, March::kThreads, March::kSmem, s>>>(v, sb, prm, hb, mp, mc, mode, stage, with_dt, kc);
    else
        k_march_stage<-1><<<grid, March::kThreads, March::kSmem, s>>>(v, sb, prm, hb, mp, mc, mode, stage, with_dt, kc);
}

inline cudaError_t prepare_march() {
    for (cudaError_t e : {cudaFuncSetAttribute(k_march_stage<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)March::kSmem),
                          cudaFuncSetAttribute(k_march_stage<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)March::kSmem),
                          cudaFuncSetAttribute(k_march_stage<-1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)March::kSmem)})
        if (e != cudaSuccess) return e;
    return cudaSuccess;
}

}  // namespace IBISGB_KNS
}  // namespace ibisgb
