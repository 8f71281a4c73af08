// Residual and Runge-Kutta kernels for sm_103a, templated on
//   R  arithmetic of reconstruction, limiting and fluxes (double or float),
//   P  storage type of primitives and per-cell/face intermediates,
//   Gm storage type of geometry,
//   DIM 2 or 3, EXACT (reference operation order, pow in Sutherland, used by the
//   no-FMA build that reproduces ibis bit for bit).
// One translation unit instantiates one (R, P, Gm, EXACT) family; see kernels_*.cu.
//
// Pipeline of one residual evaluation (FiniteVolume::compute_dudt,
// finite_volume.cpp:56-85), all cell arrays SoA and slot-major:
//   k_recon   per valid cell: least-squares gradients of the reconstructed
//             variables and Barth-Jespersen limiters in one pass over the
//             neighbours (+ the viscous gradients of T, v with the
//             pre-viscous ghost values)              [gradient.h, limiter.cpp]
//   k_face    per face: MUSCL reconstruction of both sides, thermo closure,
//             rotation to the face frame, flux calculator, rotation back,
//             viscous stress / heat flux             [convective_flux.cpp, viscous_flux.cpp]
//   k_update  per valid cell: surface integral in double, then the Runge-Kutta
//             stage combination, conserved->primitive inversion and the
//             ghost cells this cell feeds (the next evaluation's
//             pre-reconstruction boundary actions)    [finite_volume.cpp:220-255,
//                                                      runge_kutta.cpp:131-203]
#pragma once

#include <type_traits>

#include "numerics.cuh"

namespace ibisgb {
namespace IBISGB_KNS {

constexpr int kBlock = 256;

inline unsigned blocks_for(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

// thermo variable pair in the reference's call order (compute_convective_gradient,
// convective_flux.cpp:180-209): prim indices 0 rho, 1 p, 2 T, 3 e
IBISGB_HD void thermo_vars(int kind, int& a, int& b) {
    switch (kind) {
        case kRhoP: a = 1; b = 0; break;
        case kRhoU: a = 0; b = 3; break;
        case kRhoT: a = 0; b = 2; break;
        default: a = 1; b = 2; break;  // p_T
    }
}

template <class S>
struct StateT {
    S rho, p, T, e, vx, vy, vz;
};
using State64 = StateT<double>;

IBISGB_HD double real_of(double x) { return x; }
IBISGB_HD double real_of(float x) { return (double)x; }
IBISGB_HD double real_of(const FF& x) { return ff_to_double(x); }
IBISGB_HD float to_float(double x) { return (float)x; }
IBISGB_HD float to_float(float x) { return x; }
IBISGB_HD float to_float(const FF& x) { return x.hi; }
// a value of arithmetic R stored as P (a float-float value keeps its hi part)
template <class P, class R>
IBISGB_HD P narrow(const R& x) {
    if constexpr (std::is_same_v<R, FF>) return (P)x.hi;
    else return (P)x;
}

// A translation unit that defines IBISGB_FLOAT_FLOAT to 1 builds the MIXED_FF
// family: the float state and geometry arrays plus their lo companions
// (DevView::prim_lo ...), face states and fluxes in float-float arithmetic.
#ifndef IBISGB_FLOAT_FLOAT
#define IBISGB_FLOAT_FLOAT 0
#endif
constexpr bool kFFBuild = IBISGB_FLOAT_FLOAT != 0;

// primitive index of viscous variable q (0 T, 1 vx, 2 vy, 3 vz)
IBISGB_HD int visc_prim(int q) { return q == 0 ? 2 : 3 + q; }

// float -> double and double -> float (round to nearest even) by assembling the
// bit patterns on the integer pipe.  The conversion instructions run on GB300's
// narrow FP64 pipe, the mixed update's bottleneck.  Only the rare inputs --
// subnormal floats; doubles outside the normal float range, infinities, NaN --
// take the instruction, in a function that is called, not inlined, so that no
// predicated conversion is issued for the common case.  Results are bit for bit
// the instructions' under the translation unit's compiler flags (checked by ibisgb_check_conversions).
__device__ __noinline__ double f2d_by_instruction(float x) { return (double)x; }
__device__ __noinline__ float d2f_by_instruction(double x) { return __double2float_rn(x); }

__device__ __forceinline__ double f2d(float x) {
    const unsigned u = __float_as_uint(x);
    const unsigned ex = (u >> 23) & 0xFFu;
    const unsigned man = u & 0x7FFFFFu;
    if (ex == 0u && man != 0u) return f2d_by_instruction(x);
    const unsigned e11 = ex == 0xFFu ? 0x7FFu : (ex == 0u ? 0u : ex + 896u);
    return __hiloint2double((int)((u & 0x80000000u) | (e11 << 20) | (man >> 3)), (int)(man << 29));
}

__device__ __forceinline__ float d2f(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned ex = (hi >> 20) & 0x7FFu;
    if (ex - 897u > 253u) return d2f_by_instruction(x);  // float exponent outside 1..254
    const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);  // the 23 kept significand bits
    const unsigned rem = lo & 0x1FFFFFFFu;                   // the 29 dropped ones
    const unsigned up = (rem > 0x10000000u) | ((rem == 0x10000000u) & m);
    // a carry out of the significand moves to the next binade (to infinity above the largest float)
    return __uint_as_float(((hi & 0x80000000u) | ((ex - 896u) << 23)) + m + up);
}

// A double as a float-float pair on the integer pipe: hi as d2f, lo the exact
// remainder x - hi (the 29 dropped significand bits less the rounding carry,
// at most 28 bits) rounded to float by an int->float conversion and moved to
// its binade by an exponent addition.  Zero takes a bit test; tiny and
// non-finite inputs take the conversion instructions, in a call.
__device__ __noinline__ FF d2ff_by_instruction(double x) {
    const float h = __double2float_rn(x);
    return FF(h, __double2float_rn(x - (double)h));
}
__device__ __forceinline__ FF d2ff(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned ex = (hi >> 20) & 0x7FFu;
    if (ex == 0u && (hi & 0xFFFFFu) == 0u && lo == 0u) return FF(__uint_as_float(hi & 0x80000000u), 0.f);  // +-0
    // |x| outside [2^-74, 2^128): hi out of float range, or lo possibly subnormal
    if (ex - 949u > 201u) return d2ff_by_instruction(x);
    const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1FFFFFFFu;
    const unsigned up = (rem > 0x10000000u) | ((rem == 0x10000000u) & m);
    const float h = __uint_as_float(((hi & 0x80000000u) | ((ex - 896u) << 23)) + m + up);
    int d = (int)rem - (int)(up << 29);
    if (d == 0) return FF(h, 0.f);
    if (hi >> 31) d = -d;
    // d * 2^(ex - 1075): the conversion is exact to 24 bits, the scaling exact (normal result)
    const int fb = __float_as_int(__int2float_rn(d));
    return FF(h, __int_as_float(fb + ((int)ex - 1075) * (1 << 23)));
}

// (ah + al) - (bh + bl) as a float-float value: the float difference exactly
// (TwoSum), then the difference of the remainders
__device__ __forceinline__ FF ff_diff(float ah, float al, float bh, float bl) {
    const FF d = ff_two_sum(ah, -bh);
    return ff_fast_two_sum(d.hi, __fadd_rn(d.lo, __fsub_rn(al, bl)));
}

// A value in the storage type P of the state arrays: for the float build the
// integer-pipe conversion (bit for bit the instruction's), else a cast.
template <class P, class S>
__device__ __forceinline__ P to_storage(S x) {
    if constexpr (sizeof(P) == sizeof(float) && sizeof(S) == sizeof(double) && !kIsDual<S>) return d2f(x);
    else return (P)x;
}

// ---------------------------------------------------------------------------
// Ghost-cell actions on one ghost (boundary.cpp:9-400), in double.
// ---------------------------------------------------------------------------
// face_lo (float-float build, else null): what the float geometry leaves out,
// so that the normal and tangents the actions use are hi + lo in double.
// fs_dir (dual S only, else null): a tangent direction of the actions' flow
// state (T, p, rho, energy, vx, vy, vz), for the derivative with respect to it.
template <class S, class Gm>
__device__ void apply_actions(const Action* acts, int n, StateT<S>& gh, const StateT<S>& src,
                              const Gm* face, int F, int f, const FvParams& prm, const double* gfix, int G,
                              int g, const float* face_lo = nullptr, const double* fs_dir = nullptr) {
    auto geo = [&](int k) -> S {
        if constexpr (std::is_arithmetic<Gm>::value)  // (a dual geometry, for its adjoint, has no lo part)
            if (face_lo) return S((double)face[k * F + f] + (double)face_lo[k * F + f]);
        return S(face[k * F + f]);
    };
    auto fsv = [&](const Action& A, int k) -> S {
        if constexpr (kIsDual<S>)
            if (fs_dir) return S(A.fs[k], fs_dir[k]);
        return S(A.fs[k]);
    };
    for (int a = 0; a < n; a++) {
        const Action& A = acts[a];
        switch (A.kind) {
            case aFlowStateCopy:
                gh.T = fsv(A, 0); gh.p = fsv(A, 1); gh.rho = fsv(A, 2); gh.e = fsv(A, 3);
                gh.vx = fsv(A, 4); gh.vy = fsv(A, 5); gh.vz = fsv(A, 6);
                break;
            case aInternalCopy:
            case aPeriodicCopy:
                gh = src;
                break;
            case aReflectNormal: {
                gh.T = src.T; gh.p = src.p; gh.rho = src.rho; gh.e = src.e;
                S x = src.vx, y = src.vy, z = src.vz;
                S nx = geo(0), ny = geo(1), nz = geo(2);
                S t1x = geo(3), t1y = geo(4), t1z = geo(5);
                S t2x = geo(6), t2y = geo(7), t2z = geo(8);
                S xs = -(x * nx + y * ny + z * nz);
                S ys = x * t1x + y * t1y + z * t1z;
                S zs = x * t2x + y * t2y + z * t2z;
                gh.vx = xs * nx + ys * t1x + zs * t2x;
                gh.vy = xs * ny + ys * t1y + zs * t2y;
                gh.vz = xs * nz + ys * t1z + zs * t2z;
                break;
            }
            case aVelReflect:
                gh.vx = -src.vx; gh.vy = -src.vy; gh.vz = -src.vz;
                break;
            case aFixTemperature:
                gh.T = S(2.0) * S(A.value) - src.T;
                break;
            case aBoundaryLayer: {  // boundary.cpp:59-94, evaluated on the host at the ghost's height
                const double* t = gfix + (size_t)A.table * 5 * G;
                gh.T = S(t[g]); gh.p = S(t[G + g]); gh.rho = S(t[2 * G + g]); gh.e = S(t[3 * G + g]);
                gh.vx = S(t[4 * G + g]); gh.vy = S(0.0); gh.vz = S(0.0);
                break;
            }
            case aSubsonicInflow: {
                S nx = geo(0), ny = geo(1), nz = geo(2);
                S vc = nx * (fsv(A, 4) - src.vx) + ny * (fsv(A, 5) - src.vy) + nz * (fsv(A, 6) - src.vz);
                S sos = d_sqrt<S>(S(prm.gamma) * S(prm.R) * src.T);
                S rho_ref = src.rho;
                S p_in = fsv(A, 1);
                S p_face = S(0.5) * (p_in + src.p - rho_ref * sos * vc);
                S rho_face = fsv(A, 2) + (p_face - p_in) / sos / sos;
                S vxf = fsv(A, 4) - nx * (p_in - p_face) / (rho_ref * sos);
                S vyf = fsv(A, 5) - ny * (p_in - p_face) / (rho_ref * sos);
                S vzf = fsv(A, 6) - nz * (p_in - p_face) / (rho_ref * sos);
                gh.p = S(2.0) * p_face - src.p;
                gh.rho = S(2.0) * rho_face - src.rho;
                gh.T = gh.p / (gh.rho * S(prm.R));
                gh.e = S(prm.Cv) * gh.T;
                gh.vx = S(2.0) * vxf - src.vx; gh.vy = S(2.0) * vyf - src.vy; gh.vz = S(2.0) * vzf - src.vz;
                break;
            }
            case aSubsonicOutflow: {
                S nx = geo(0), ny = geo(1), nz = geo(2);
                S p_face = S(A.value);
                S rho_ref = src.rho, p_ref = src.p;
                S sos = d_sqrt<S>(S(prm.gamma) * S(prm.R) * src.T);
                S rho_face = src.rho + (p_face - p_ref) / sos / sos;
                S vxf = src.vx + nx * (p_ref - p_face) / (rho_ref * sos);
                S vyf = src.vy + ny * (p_ref - p_face) / (rho_ref * sos);
                S vzf = src.vz + nz * (p_ref - p_face) / (rho_ref * sos);
                gh.p = S(2.0) * p_face - src.p;
                gh.rho = S(2.0) * rho_face - src.rho;
                gh.T = gh.p / (gh.rho * S(prm.R));
                gh.e = S(prm.Cv) * gh.T;
                gh.vx = S(2.0) * vxf - src.vx; gh.vy = S(2.0) * vyf - src.vy; gh.vz = S(2.0) * vzf - src.vz;
                break;
            }
        }
    }
}

// Fill ghost g from the state of its source cell: pre-reconstruction actions
// into the primitive arrays, then the pre-viscous-gradient actions on top of
// them into the viscous ghost arrays (p, T, vx, vy, vz).
template <class P, class Gm, class S = double>
__device__ void fill_ghost(const DevView& v, const FvParams& prm, int g, const StateT<S>& src) {
    const BoundDev& B = v.bounds[v.ghost_bound[g]];
    const Gm* face = (const Gm*)v.face;
    int f = v.ghost_face[g];
    StateT<S> gh = src;
    const double* fs_dir = nullptr;  // the flow-state tangent's direction for this boundary
    if constexpr (kIsDual<S>)
        if (v.fs_tan) fs_dir = v.fs_tan + 7 * (size_t)v.ghost_bound[g];
    apply_actions<S, Gm>(B.pre, B.n_pre, gh, src, face, v.F, f, prm, v.gfix, v.G, g, v.face_lo, fs_dir);
    P* pr = (P*)v.prim;
    const int NT = v.NT, id = v.N + g;
    if constexpr (kFFBuild && sizeof(P) == sizeof(float) && !kIsDual<S>) {
        const double w[7] = {gh.rho, gh.p, gh.T, gh.e, gh.vx, gh.vy, gh.vz};
#pragma unroll
        for (int k = 0; k < 7; k++) {
            const FF x = d2ff(w[k]);
            pr[k * NT + id] = x.hi;
            v.prim_lo[k * NT + id] = x.lo;
        }
    } else {
        pr[id] = to_storage<P>(gh.rho); pr[NT + id] = to_storage<P>(gh.p); pr[2 * NT + id] = to_storage<P>(gh.T);
        pr[3 * NT + id] = to_storage<P>(gh.e); pr[4 * NT + id] = to_storage<P>(gh.vx);
        pr[5 * NT + id] = to_storage<P>(gh.vy); pr[6 * NT + id] = to_storage<P>(gh.vz);
    }
    if (prm.viscous) {
        apply_actions<S, Gm>(B.visc, B.n_visc, gh, src, face, v.F, f, prm, v.gfix, v.G, g, v.face_lo, fs_dir);
        P* vg = (P*)v.vghost;
        if constexpr (kFFBuild && sizeof(P) == sizeof(float) && !kIsDual<S>) {
            const double w[5] = {gh.p, gh.T, gh.vx, gh.vy, gh.vz};
#pragma unroll
            for (int k = 0; k < 5; k++) {
                const FF x = d2ff(w[k]);
                vg[k * v.G + g] = x.hi;
                v.vghost_lo[k * v.G + g] = x.lo;
            }
        } else {
            vg[g] = to_storage<P>(gh.p); vg[v.G + g] = to_storage<P>(gh.T); vg[2 * v.G + g] = to_storage<P>(gh.vx);
            vg[3 * v.G + g] = to_storage<P>(gh.vy); vg[4 * v.G + g] = to_storage<P>(gh.vz);
        }
    }
}

template <class P, class S>
__device__ StateT<S> load_state(const DevView& v, int c) {
    const P* pr = (const P*)v.prim;
    const int NT = v.NT;
    if constexpr (kFFBuild && sizeof(P) == sizeof(float) && !kIsDual<S>) {
        const float* lo = v.prim_lo;
        auto g = [&](int k) { return S((double)pr[k * NT + c] + (double)lo[k * NT + c]); };
        return StateT<S>{g(0), g(1), g(2), g(3), g(4), g(5), g(6)};
    }
    return StateT<S>{S(pr[c]), S(pr[NT + c]), S(pr[2 * NT + c]), S(pr[3 * NT + c]),
                     S(pr[4 * NT + c]), S(pr[5 * NT + c]), S(pr[6 * NT + c])};
}

template <class P, class Gm, class S = double>
__global__ void __launch_bounds__(kBlock) k_ghost_fill(DevView v, FvParams prm) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= v.G) return;
    fill_ghost<P, Gm, S>(v, prm, g, load_state<P, S>(v, v.ghost_src[g]));
}

// ---------------------------------------------------------------------------
// k_recon: gradients (WLSGradient::compute_gradients, gradient.h:65-116) and
// Barth-Jespersen limiters (limiter.cpp:23-63) of every valid cell.
// ---------------------------------------------------------------------------
// The float build stores limiter-scaled gradients (phi * grad) instead of
// gradients and limiters, packed per cell: the DIM components of each
// reconstructed variable in turn (15 floats in 3-D, 8 in 2-D) in a 16-float
// slot that the face kernel reads as four (two) 128-bit loads per side, instead
// of 20 (12) scattered values.
// A translation unit that defines IBISGB_FLOAT_GRADIENTS to 1 builds the
// MIXED_GRAD family: float gradients and limiters (packed as above) over double
// primitives, geometry, face states and fluxes.
#ifndef IBISGB_FLOAT_GRADIENTS
#define IBISGB_FLOAT_GRADIENTS 0
#endif
template <class P, bool EXACT>
constexpr bool prescaled_gradients() { return !EXACT && (sizeof(P) == sizeof(float) || IBISGB_FLOAT_GRADIENTS); }
// float gradient arithmetic over double primitives and geometry (MIXED_GRAD):
// every neighbour value and face offset enters the float arithmetic relative to
// the cell's own value and centroid, formed in double, so that float rounds
// the increments, not the values they are added to
template <class R, class P, bool EXACT>
constexpr bool relative_float_gradients() {
    return !EXACT && sizeof(R) == sizeof(float) && sizeof(P) == sizeof(double);
}
// the same for the float-float build: the differences are (hi - hi) + (lo - lo)
// of the float arrays and their lo companions
template <class R, class P, bool EXACT>
constexpr bool relative_ff_gradients() {
    return kFFBuild && !EXACT && sizeof(P) == sizeof(float) && (sizeof(R) == sizeof(float) || std::is_same_v<R, FF>);
}
constexpr int kPackedGrad = 16;  // floats per cell of the packed gradients

template <class R, class P, class Gm, int DIM, bool EXACT, int BS = kBlock, int MINB = 1>
__global__ void __launch_bounds__(BS, MINB) k_recon(DevView v, FvParams prm, int reconstruct) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    constexpr int NV = DIM == 3 ? 5 : 4;  // reconstructed variables (vz only in 3-D)
    const int N = v.N, NT = v.NT, G = v.G, F = v.F;
    const Gm* cc = (const Gm*)v.cc;
    const Gm* rr = (const Gm*)v.r;
    const Gm* fcen = (const Gm*)v.face + 9 * F;
    const P* pr = (const P*)v.prim;
    const P* vg = (const P*)v.vghost;
    int ia, ib;
    thermo_vars(prm.thermo, ia, ib);
    const int vidx[5] = {ia, ib, 4, 5, 6};
    const bool visc = prm.viscous != 0;
    const bool lim = reconstruct && prm.limiter;

    constexpr bool REL = relative_float_gradients<R, P, EXACT>();
    constexpr bool RELF = relative_ff_gradients<R, P, EXACT>();
    // float-float gradients and limiters (MIXED_FF): weights, offsets and the
    // packed output carry their lo companions too
    constexpr bool FFG = RELF && std::is_same_v<R, FF>;
    const float* plo = v.prim_lo;
    R xi = (R)cc[i], yi = (R)cc[NT + i], zi = DIM == 3 ? (R)cc[2 * NT + i] : R(0.0);
    double xid = 0.0, yid = 0.0, zid = 0.0;
    if constexpr (REL) { xid = (double)cc[i]; yid = (double)cc[NT + i]; zid = DIM == 3 ? (double)cc[2 * NT + i] : 0.0; }
    R r11 = R(1.0), r12 = R(0.0), r22 = R(1.0), r13 = R(0.0), r23 = R(0.0), r33 = R(1.0), beta = R(0.0);
    if (EXACT) {
        r11 = (R)rr[i]; r12 = (R)rr[N + i]; r22 = (R)rr[2 * N + i];
        if (DIM == 3) { r13 = (R)rr[3 * N + i]; r23 = (R)rr[4 * N + i]; r33 = (R)rr[5 * N + i]; }
        beta = (r12 * r23 - r13 * r23) / (r11 * r22);
    }

    // REL: ui = 0 and every neighbour value is taken relative to the cell's (uid)
    R ui[NV], gx[NV], gy[NV], gz[NV], umin[NV], umax[NV];
    double uid[NV];
    float uhi[NV], ulo[NV];  // RELF: the cell's own value as hi + lo
#pragma unroll
    for (int q = 0; q < NV; q++) {
        uhi[q] = 0.f; ulo[q] = 0.f;
        if constexpr (REL) {
            uid[q] = (double)pr[vidx[q] * NT + i];
            ui[q] = R(0.0);
        } else if constexpr (RELF) {
            uid[q] = 0.0;
            uhi[q] = (float)pr[vidx[q] * NT + i];
            ulo[q] = plo[vidx[q] * NT + i];
            ui[q] = R(0.0);
        } else {
            uid[q] = 0.0;
            ui[q] = (R)pr[vidx[q] * NT + i];
        }
        gx[q] = R(0.0); gy[q] = R(0.0); gz[q] = R(0.0);
        umin[q] = ui[q]; umax[q] = ui[q];
    }
    constexpr int NW = DIM == 3 ? 4 : 3;  // viscous: T, vx, vy[, vz]
    R wi[NW], hx[NW], hy[NW], hz[NW];
    double wid[NW];
    float whi[NW], wlo[NW];
#pragma unroll
    for (int q = 0; q < NW; q++) {
        whi[q] = 0.f; wlo[q] = 0.f;
        if constexpr (REL) {
            wid[q] = (double)pr[visc_prim(q) * NT + i];
            wi[q] = R(0.0);
        } else if constexpr (RELF) {
            wid[q] = 0.0;
            whi[q] = (float)pr[visc_prim(q) * NT + i];
            wlo[q] = plo[visc_prim(q) * NT + i];
            wi[q] = R(0.0);
        } else {
            wid[q] = 0.0;
            wi[q] = (R)pr[visc_prim(q) * NT + i];
        }
        hx[q] = R(0.0); hy[q] = R(0.0); hz[q] = R(0.0);
    }

    const int nf = v.nfaces[i];
    const Gm* W = (const Gm*)v.lsqw;
    const int MF = v.MF;
    // the weight and offset tables: per cell, or one row per slot shared by every cell
    const int sN = v.lsq_shared ? 1 : N, si = v.lsq_shared ? 0 : i;
    auto slot = [&](int s, int nb) {
        R w1, w2, w3;
        if constexpr (FFG) {
            const float* Wl = v.lsqw_lo;
            w1 = FF((float)W[s * sN + si], Wl[s * sN + si]);
            w2 = FF((float)W[(MF + s) * sN + si], Wl[(MF + s) * sN + si]);
            w3 = DIM == 3 ? FF((float)W[(2 * MF + s) * sN + si], Wl[(2 * MF + s) * sN + si]) : FF(0.f);
        } else if (!EXACT) {  // weights precomputed on the host from the same formulas
            w1 = (R)W[s * sN + si];
            w2 = (R)W[(MF + s) * sN + si];
            w3 = DIM == 3 ? (R)W[(2 * MF + s) * sN + si] : R(0.0);
        } else {
            R dx = (R)cc[nb] - xi, dy = (R)cc[NT + nb] - yi;
            R dz = DIM == 3 ? (R)cc[2 * NT + nb] - zi : R(0.0);
            R a1 = dx / (r11 * r11);
            R a2 = R(1.0) / (r22 * r22) * (dy - r12 / r11 * dx);
            R a3 = R(0.0);
            if (DIM == 3) a3 = R(1.0) / (r33 * r33) * (dz - r23 / r22 * dy + beta * dx);
            w1 = a1 - r12 / r11 * a2 + beta * a3;
            w2 = a2 - r23 / r22 * a3;
            w3 = a3;
        }
        if (reconstruct) {
#pragma unroll
            for (int q = 0; q < NV; q++) {
                R un;
                if constexpr (REL) un = (R)((double)pr[vidx[q] * NT + nb] - uid[q]);
                else if constexpr (FFG)
                    un = ff_diff((float)pr[vidx[q] * NT + nb], plo[vidx[q] * NT + nb], uhi[q], ulo[q]);
                else if constexpr (RELF)
                    un = ((float)pr[vidx[q] * NT + nb] - uhi[q]) + (plo[vidx[q] * NT + nb] - ulo[q]);
                else un = (R)pr[vidx[q] * NT + nb];
                R du = un - ui[q];
                gx[q] += w1 * du; gy[q] += w2 * du;
                if (DIM == 3) gz[q] += w3 * du;
                umin[q] = d_min(umin[q], un);
                umax[q] = d_max(umax[q], un);
            }
        }
        if (visc) {
            const bool ghost = nb >= N;
#pragma unroll
            for (int q = 0; q < NW; q++) {
                R un;
                if constexpr (REL)
                    un = (R)((ghost ? (double)vg[(1 + q) * G + (nb - N)] : (double)pr[visc_prim(q) * NT + nb]) - wid[q]);
                else if constexpr (FFG)  // the pre-viscous ghost values are floats
                    un = ghost ? ff_diff((float)vg[(1 + q) * G + (nb - N)], v.vghost_lo[(1 + q) * G + (nb - N)], whi[q], wlo[q])
                               : ff_diff((float)pr[visc_prim(q) * NT + nb], plo[visc_prim(q) * NT + nb], whi[q], wlo[q]);
                else if constexpr (RELF)  // the pre-viscous ghost values are floats
                    un = ghost ? ((float)vg[(1 + q) * G + (nb - N)] - whi[q]) - wlo[q]
                               : ((float)pr[visc_prim(q) * NT + nb] - whi[q]) + (plo[visc_prim(q) * NT + nb] - wlo[q]);
                else un = ghost ? (R)vg[(1 + q) * G + (nb - N)] : (R)pr[visc_prim(q) * NT + nb];
                R du = un - wi[q];
                hx[q] += w1 * du; hy[q] += w2 * du;
                if (DIM == 3) hz[q] += w3 * du;
            }
        }
    };
    // each slot's neighbour id is loaded while the previous slot's values are in
    // flight, so that the gathers do not wait for the id load in turn
    int nb_next = nf > 0 ? v.cell_nbr[i] : 0;
    for (int s = 0; s < nf; s++) {
        const int nb = nb_next;
        if (s + 1 < nf) nb_next = v.cell_nbr[(s + 1) * N + i];
        slot(s, nb);
    }

    if (reconstruct) {
        P* gout = (P*)v.grad;
        R phi[NV];
        unsigned code[NV];
#pragma unroll
        for (int q = 0; q < NV; q++) { phi[q] = R(1.0); code[q] = 0u; }
        if (lim) {
            const R eps = par<R>(prm.eps, prm.feps);
            if (EXACT || v.branches) {
                // face by face, as limiter.cpp:46-60, recording the branch taken; the
                // fast builds take the face offsets as their two-division form below
                // does (per slot where stored), so recording changes no value
                const Gm* D = (const Gm*)v.lsqd;
                for (int s = 0; s < nf; s++) {
                    const int f = v.cell_face[s * N + i];
                    R dx = (R)fcen[f] - xi, dy = (R)fcen[F + f] - yi;
                    R dz = DIM == 3 ? (R)fcen[2 * F + f] - zi : R(0.0);
                    if (!EXACT && D) {
                        if constexpr (FFG) {
                            const float* Dl = v.lsqd_lo;
                            dx = FF((float)D[s * sN + si], Dl[s * sN + si]);
                            dy = FF((float)D[(MF + s) * sN + si], Dl[(MF + s) * sN + si]);
                            dz = DIM == 3 ? FF((float)D[(2 * MF + s) * sN + si], Dl[(2 * MF + s) * sN + si]) : FF(0.f);
                        } else {
                            dx = (R)D[s * sN + si]; dy = (R)D[(MF + s) * sN + si];
                            dz = DIM == 3 ? (R)D[(2 * MF + s) * sN + si] : R(0.0);
                        }
                    } else if constexpr (REL) {
                        dx = (R)((double)fcen[f] - xid); dy = (R)((double)fcen[F + f] - yid);
                        dz = DIM == 3 ? (R)((double)fcen[2 * F + f] - zid) : R(0.0);
                    }
#pragma unroll
                    for (int q = 0; q < NV; q++) {
                        R d2 = DIM == 3 ? gx[q] * dx + gy[q] * dy + gz[q] * dz : gx[q] * dx + gy[q] * dy;
                        int sg = (d2 > R(0.0)) - (d2 < R(0.0));
                        d2 = (R)sg * (d_abs(d2) + eps);
                        if (sg != 0) {
                            R ratio = sg > 0 ? (umax[q] - ui[q]) / d2 : (umin[q] - ui[q]) / d2;
                            code[q] |= (unsigned)(sg > 0 ? 1 : 2) << (2 * s);
                            if (!(phi[q] < ratio)) code[q] = (code[q] & 0xFFFFu) | ((unsigned)(s + 1) << 16);
                            phi[q] = d_min(phi[q], ratio);
                        }
                    }
                }
            } else {
                // Same value with two divisions per variable: (U_max - U_i) / (d + eps)
                // decreases with d, and IEEE division and addition round monotonically,
                // so the minimum over faces is taken at the largest projection of each sign.
                R tpos[NV], tneg[NV];
#pragma unroll
                for (int q = 0; q < NV; q++) { tpos[q] = R(0.0); tneg[q] = R(0.0); }
                const Gm* D = (const Gm*)v.lsqd;
                for (int s = 0; s < nf; s++) {
                    R dx, dy, dz;
                    if (D) {  // face offsets stored per slot
                        if constexpr (FFG) {
                            const float* Dl = v.lsqd_lo;
                            dx = FF((float)D[s * sN + si], Dl[s * sN + si]);
                            dy = FF((float)D[(MF + s) * sN + si], Dl[(MF + s) * sN + si]);
                            dz = DIM == 3 ? FF((float)D[(2 * MF + s) * sN + si], Dl[(2 * MF + s) * sN + si]) : FF(0.f);
                        } else {
                            dx = (R)D[s * sN + si]; dy = (R)D[(MF + s) * sN + si];
                            dz = DIM == 3 ? (R)D[(2 * MF + s) * sN + si] : R(0.0);
                        }
                    } else {
                        const int f = v.cell_face[s * N + i];
                        if constexpr (REL) {
                            dx = (R)((double)fcen[f] - xid); dy = (R)((double)fcen[F + f] - yid);
                            dz = DIM == 3 ? (R)((double)fcen[2 * F + f] - zid) : R(0.0);
                        } else {
                            dx = (R)fcen[f] - xi; dy = (R)fcen[F + f] - yi;
                            dz = DIM == 3 ? (R)fcen[2 * F + f] - zi : R(0.0);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < NV; q++) {
                        R d2 = DIM == 3 ? gx[q] * dx + gy[q] * dy + gz[q] * dz : gx[q] * dx + gy[q] * dy;
                        tpos[q] = d_max(tpos[q], d2);
                        tneg[q] = d_min(tneg[q], d2);
                    }
                }
#pragma unroll
                for (int q = 0; q < NV; q++) {
                    if (tpos[q] > R(0.0)) phi[q] = d_min(phi[q], (umax[q] - ui[q]) / (tpos[q] + eps));
                    if (tneg[q] < R(0.0)) phi[q] = d_min(phi[q], (umin[q] - ui[q]) / (tneg[q] - eps));
                }
            }
            if constexpr (!prescaled_gradients<P, EXACT>()) {
                P* pout = (P*)v.phi;
#pragma unroll
                for (int q = 0; q < NV; q++) pout[q * N + i] = (P)phi[q];
            }
            if (v.branches) {
#pragma unroll
                for (int q = 0; q < 5; q++) v.branches[i * 5 + q] = q < NV ? code[q] : 0u;
            }
        }
        if constexpr (FFG) {
            float pk[kPackedGrad], pl[kPackedGrad];
#pragma unroll
            for (int k = 0; k < kPackedGrad; k++) { pk[k] = 0.f; pl[k] = 0.f; }
#pragma unroll
            for (int q = 0; q < NV; q++) {
                const FF a = gx[q] * phi[q], b = gy[q] * phi[q];
                pk[DIM * q] = a.hi; pl[DIM * q] = a.lo;
                pk[DIM * q + 1] = b.hi; pl[DIM * q + 1] = b.lo;
                if (DIM == 3) {
                    const FF c = gz[q] * phi[q];
                    pk[DIM * q + 2] = c.hi; pl[DIM * q + 2] = c.lo;
                }
            }
            float4* dst = (float4*)v.grad + (size_t)i * (kPackedGrad / 4);
            float4* dlo = (float4*)v.grad_lo + (size_t)i * (kPackedGrad / 4);
#pragma unroll
            for (int k = 0; k < (DIM == 3 ? 4 : 2); k++) {
                dst[k] = make_float4(pk[4 * k], pk[4 * k + 1], pk[4 * k + 2], pk[4 * k + 3]);
                dlo[k] = make_float4(pl[4 * k], pl[4 * k + 1], pl[4 * k + 2], pl[4 * k + 3]);
            }
        } else if constexpr (prescaled_gradients<P, EXACT>()) {
            float pk[kPackedGrad];
#pragma unroll
            for (int k = 0; k < kPackedGrad; k++) pk[k] = 0.f;
#pragma unroll
            for (int q = 0; q < NV; q++) {
                pk[DIM * q] = (float)(gx[q] * phi[q]);
                pk[DIM * q + 1] = (float)(gy[q] * phi[q]);
                if (DIM == 3) pk[DIM * q + 2] = (float)(gz[q] * phi[q]);
            }
            float4* dst = (float4*)v.grad + (size_t)i * (kPackedGrad / 4);
#pragma unroll
            for (int k = 0; k < (DIM == 3 ? 4 : 2); k++)
                dst[k] = make_float4(pk[4 * k], pk[4 * k + 1], pk[4 * k + 2], pk[4 * k + 3]);
        } else {
#pragma unroll
            for (int q = 0; q < NV; q++) {
                gout[(3 * q) * N + i] = (P)gx[q];
                gout[(3 * q + 1) * N + i] = (P)gy[q];
                gout[(3 * q + 2) * N + i] = (P)gz[q];
            }
        }
    }
    if (visc) {
        P* hout = (P*)v.vgrad;
#pragma unroll
        for (int q = 0; q < NW; q++) {
            hout[(3 * q) * N + i] = narrow<P>(hx[q]);
            hout[(3 * q + 1) * N + i] = narrow<P>(hy[q]);
            hout[(3 * q + 2) * N + i] = narrow<P>(hz[q]);
            if constexpr (FFG) {
                v.vgrad_lo[(3 * q) * N + i] = hx[q].lo;
                v.vgrad_lo[(3 * q + 1) * N + i] = hy[q].lo;
                v.vgrad_lo[(3 * q + 2) * N + i] = hz[q].lo;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// k_face: reconstruction + flux + viscous flux of every face.
// ---------------------------------------------------------------------------
template <class R, class P, int DIM>
IBISGB_HD R lin_interp(R value, R lim, const P* g, int N, int q, int c, R dx, R dy, R dz) {
    // value + limiter * (grad . d)   (linear_interpolate, convective_flux.cpp:242-255)
    R s = DIM == 3 ? (R)g[(3 * q) * N + c] * dx + (R)g[(3 * q + 1) * N + c] * dy + (R)g[(3 * q + 2) * N + c] * dz
                   : (R)g[(3 * q) * N + c] * dx + (R)g[(3 * q + 1) * N + c] * dy;
    return value + lim * s;
}

// One side of a face from its (reconstructed) primitives q (rho, p, T, e, vx,
// vy, vz): the thermo closure of the interpolated pair when reconstructing, then
// the velocity in the face frame (transform_to_local_frame, vector3.cpp:141-153).
template <class R, int DIM, bool EXACT>
__device__ __forceinline__ void side_state(int thermo, const Gas<R>& gm, bool reconstruct, R (&q)[7], R nx, R ny,
                                           R nz, R t1x, R t1y, R t1z, R t2x, R t2y, R t2z, FaceSide<R>& S) {
    if (reconstruct) thermo_close<R>(thermo, gm, q[0], q[1], q[2], q[3]);
    S.r = q[0]; S.p = q[1]; S.T = q[2];
    if (DIM == 3) {
        S.u = q[4] * nx + q[5] * ny + q[6] * nz;
        S.v = q[4] * t1x + q[5] * t1y + q[6] * t1z;
        S.w = q[4] * t2x + q[5] * t2y + q[6] * t2z;
    } else if (EXACT) {
        S.u = q[4] * nx + q[5] * ny + q[6] * nz;
        S.v = q[4] * t1x + q[5] * t1y + q[6] * t1z;
        S.w = R(0.0);
    } else {
        S.u = q[4] * nx + q[5] * ny;
        S.v = q[4] * t1x + q[5] * t1y;
        S.w = R(0.0);
    }
}

// The selected flux calculator in the face frame, rotated back to the global
// frame (transform_to_global, convective_flux.cpp:145-177): out = mass,
// momentum x, y, z, energy.
template <class R, int DIM, bool EXACT>
__device__ __forceinline__ void convective_flux(const FvParams& prm, const Gas<R>& gm, const FaceSide<R>& L,
                                                const FaceSide<R>& Rt, R nx, R ny, R nz, R t1x, R t1y, R t1z,
                                                R t2x, R t2y, R t2z, R (&out)[5]) {
    R Fl[5];
    switch (prm.flux) {
        case kHanel: flux_hanel<R, DIM>(L, Rt, gm, Fl); break;
        case kAusmdv: flux_ausmdv<R, DIM>(L, Rt, gm, Fl); break;
        case kLdfss2: flux_ldfss2<R, DIM, EXACT>(L, Rt, gm, par<R>(prm.delta, prm.fdelta, prm.lodelta), Fl); break;
        default: flux_rusanov<R, DIM>(L, Rt, gm, Fl); break;
    }
    R px = Fl[1], py = Fl[2], pz = DIM == 3 ? Fl[3] : R(0.0);
    out[0] = Fl[0];
    out[3] = R(0.0);
    if (DIM == 3 || EXACT) {
        out[1] = px * nx + py * t1x + pz * t2x;
        out[2] = px * ny + py * t1y + pz * t2y;
        if (DIM == 3) out[3] = px * nz + py * t1z + pz * t2z;
    } else {
        out[1] = px * nx + py * t1x;
        out[2] = px * ny + py * t1y;
    }
    out[4] = Fl[4];
}

// ConstantFlux::apply (boundary.cpp:404-444) on a fixed grid: the flux of the
// state fs (T, p, rho, energy, vx, vy, vz) through a face of normal n, in the
// global frame.  The energy term keeps the reference's vy * n.x.
template <class R, int DIM, class E = double>
__device__ __forceinline__ void constant_flux(const E (&fs)[7], double Cv, R nx, R ny, R nz, R (&out)[5]) {
    const R vx = R(fs[4]), vy = R(fs[5]), vz = R(fs[6]), p = R(fs[1]);
    const R u = R(Cv) * R(fs[0]);  // internal_energy: Cv T
    const R mass = R(fs[2]) * (vx * nx + vy * ny + vz * nz);
    out[0] = mass;
    out[1] = p * nx + vx * mass;
    out[2] = p * ny + vy * mass;
    out[3] = DIM == 3 ? p * nz + vz * mass : R(0.0);
    out[4] = mass * (u + R(0.5) * (vx * vx + vy * vy + vz * vz)) + p * (vx * nx + vy * nx + vz * nz);
}

// The boundary of a face's ghost side when that boundary has a constant_flux
// action, else null.
IBISGB_HD const BoundDev* constant_flux_bound(const DevView& v, int l, int r) {
    const int gc = r >= v.N ? r : (l >= v.N ? l : -1);
    if (gc < 0) return nullptr;
    const BoundDev* B = &v.bounds[v.ghost_bound[gc - v.N]];
    return B->cflux ? B : nullptr;
}

// Viscous stress and heat flux through a face (viscous_flux.cpp:130-232) from
// the states of both sides (p, T, vx, vy, vz: the cells' primitives, or a ghost's
// pre-viscous values) and the viscous gradients (T, vx, vy, vz: 3 components
// each) of the two cells; a boundary face passes its interior cell's gradients
// for both and interior = false.  ex, ey, ez: centroid of the right cell minus
// the left (interior faces).  out: the x, y, z momentum and energy terms that
// the face flux loses; also the face density, viscosity and conductivity.
template <class R, int DIM, bool EXACT>
__device__ __forceinline__ void viscous_face(const FvParams& prm, const Gas<R>& gm, bool interior, const R (&sl)[5],
                                             const R (&sr)[5], const R (&gl)[12], const R (&gr)[12], R ex, R ey,
                                             R ez, R nx, R ny, R nz, R (&out)[4], R& rho, R& mu, R& k) {
    constexpr int NW = DIM == 3 ? 4 : 3;
    R g[4][3];
    if (!interior) {
#pragma unroll
        for (int q = 0; q < NW; q++)
            for (int d = 0; d < 3; d++) g[q][d] = gl[3 * q + d];
    } else {
        R len_e = d_sqrt(ex * ex + ey * ey + ez * ez);
        R ehx = ex / len_e, ehy = ey / len_e, ehz = ez / len_e;
        R edn = ehx * nx + ehy * ny + ehz * nz;
        // hasselbacher_average_ (viscous_flux.cpp:84-98), variable order T, vx, vy, vz
#pragma unroll
        for (int q = 0; q < NW; q++) {
            R ax = R(0.5) * (gl[3 * q] + gr[3 * q]);
            R ay = R(0.5) * (gl[3 * q + 1] + gr[3 * q + 1]);
            R az = R(0.5) * (gl[3 * q + 2] + gr[3 * q + 2]);
            R ade = ax * ehx + ay * ehy + az * ehz;
            R corr = ade - (sr[1 + q] - sl[1 + q]) / len_e;
            g[q][0] = ax - corr * nx / edn;
            g[q][1] = ay - corr * ny / edn;
            g[q][2] = az - corr * nz / edn;
        }
    }
    if (DIM == 2) { g[3][0] = R(0.0); g[3][1] = R(0.0); g[3][2] = R(0.0); }
    // face state: average of p, T, v (average_pT, gas_state.h:219-225) + update_thermo_from_pT
    R p = R(0.5) * (sl[0] + sr[0]);
    R T = R(0.5) * (sl[1] + sr[1]);
    rho = p / (gm.R_ * T);
    R vx = R(0.5) * (sl[2] + sr[2]);
    R vy = R(0.5) * (sl[3] + sr[3]);
    R vz = DIM == 3 ? R(0.5) * (sl[4] + sr[4]) : R(0.0);
    mu = sutherland<R, EXACT>(T, par<R>(prm.mu0, prm.fmu0, prm.lomu0), par<R>(prm.T0, prm.fT0, prm.loT0),
                             par<R>(prm.Ts, prm.fTs, prm.loTs));
    k = gm.Cp * mu / par<R>(prm.Pr, prm.fPr, prm.loPr);
    R lambda = R(-2.0 / 3.0) * mu;
    const R *gT = g[0], *gx = g[1], *gy = g[2], *gz = g[3];
    R bulk = lambda * (gx[0] + gy[1] + gz[2]);
    R txx = R(2.0) * mu * gx[0] + bulk;
    R tyy = R(2.0) * mu * gy[1] + bulk;
    R tzz = R(2.0) * mu * gz[2] + bulk;
    R txy = mu * (gx[1] + gy[0]);
    R txz = mu * (gx[2] + gz[0]);
    R tyz = mu * (gy[2] + gz[1]);
    R thx = vx * txx + vy * txy + vz * txz + k * gT[0];
    R thy = vx * txy + vy * tyy + vz * tyz + k * gT[1];
    R thz = vx * txz + vy * tyz + vz * tzz + k * gT[2];
    out[0] = nx * txx + ny * txy + nz * txz;
    out[1] = nx * txy + ny * tyy + nz * tyz;
    out[2] = nx * txz + ny * tyz + nz * tzz;
    out[3] = nx * thx + ny * thy + nz * thz;
}

// The convective flux of face f in the global frame (after the post-convective
// flux actions): reconstruction of both sides, thermo closure, flux calculator.
// Also returns the face normal.  Shared by k_face and the per-cell flux path,
// so that both produce the same bits.
template <class R, class P, class Gm, int DIM, bool EXACT>
__device__ __forceinline__ void face_convective(const DevView& v, const FvParams& prm, int f, int reconstruct,
                                                R (&Fg)[5], R& nx_out, R& ny_out, R& nz_out) {
    const int N = v.N, NT = v.NT, F = v.F;
    const Gm* fg = (const Gm*)v.face;
    const Gm* cc = (const Gm*)v.cc;
    const P* pr = (const P*)v.prim;
    const P* gr = (const P*)v.grad;
    const P* ph = (const P*)v.phi;
    const Gas<R> gm(prm);
    // float-float build: every geometry and state value as its float plus its lo companion
    constexpr bool FFR = kFFBuild && std::is_same_v<R, FF>;
    auto geo = [&](int k) -> R {
        if constexpr (FFR) return FF((float)fg[k * F + f], v.face_lo[k * F + f]);
        else return (R)fg[k * F + f];
    };
    auto cen = [&](int k, int c) -> R {
        if constexpr (FFR) return FF((float)cc[k * NT + c], v.cc_lo[k * NT + c]);
        else return (R)cc[k * NT + c];
    };
    auto prim = [&](int k, int c) -> R {
        if constexpr (FFR) return FF((float)pr[k * NT + c], v.prim_lo[k * NT + c]);
        else return (R)pr[k * NT + c];
    };
    // a uniform lattice's face class (float build): the normal, the 2-D tangents and
    // the sides' offsets from the class's row, the same values the arrays hold
    const float* ct = nullptr;
    if constexpr (!FFR && !EXACT && sizeof(R) == sizeof(float) && sizeof(Gm) == sizeof(float))
        if (v.face_class) ct = v.face_class_tab + kFaceClassRow * v.face_class[f];
    const R nx = ct ? (R)ct[0] : geo(0), ny = ct ? (R)ct[1] : geo(1);
    const R nz = DIM == 3 ? (ct ? (R)ct[2] : geo(2)) : R(0.0);
    R t1x, t1y, t1z, t2x, t2y, t2z;
    if constexpr (!EXACT && sizeof(R) == sizeof(float) && DIM == 3) {
        // The float build rotates into a frame built from n (any orthonormal
        // tangents give the same flux up to rounding): t1 = n x e / |n x e| for
        // the axis e of n's smallest component, t2 = n x t1.
        const R ax = d_abs(nx), ay = d_abs(ny), az = d_abs(nz);
        const bool ex = ax <= ay && ax <= az, ey = !ex && ay <= az;
        t1x = ex ? R(0.0) : (ey ? -nz : ny);
        t1y = ex ? nz : (ey ? R(0.0) : -nx);
        t1z = ex ? -ny : (ey ? nx : R(0.0));
        const R inv = rsqrtf(t1x * t1x + t1y * t1y + t1z * t1z);
        t1x *= inv; t1y *= inv; t1z *= inv;
        t2x = ny * t1z - nz * t1y;
        t2y = nz * t1x - nx * t1z;
        t2z = nx * t1y - ny * t1x;
    } else {
        t1x = ct ? (R)ct[3] : geo(3); t1y = ct ? (R)ct[4] : geo(4); t1z = DIM == 3 ? geo(5) : R(0.0);
        t2x = DIM == 3 ? geo(6) : R(0.0); t2y = DIM == 3 ? geo(7) : R(0.0);
        t2z = ct ? (R)ct[5] : geo(8);
    }
    const R fx = ct ? R(0.0) : geo(9), fy = ct ? R(0.0) : geo(10);
    const R fz = DIM == 3 && !ct ? geo(11) : R(0.0);
    int ia, ib;
    thermo_vars(prm.thermo, ia, ib);
    const int cells[2] = {v.left[f], v.right[f]};
    FaceSide<R> S[2];
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const int c = cells[side];
        R q[7];
        // with reconstruction both sides pass through the thermo closure, which
        // overwrites the two thermodynamic values that are not interpolated
#pragma unroll
        for (int k = 0; k < 7; k++)
            q[k] = (DIM == 2 && k == 6) || (reconstruct && k < 4 && k != ia && k != ib) ? R(0.0)
                                                                                    : prim(k, c);
        if (reconstruct && c < N) {
            R dx, dy, dz;
            if (ct) {
                dx = (R)ct[6 + 3 * side]; dy = (R)ct[7 + 3 * side]; dz = DIM == 3 ? (R)ct[8 + 3 * side] : R(0.0);
            } else {
                dx = fx - cen(0, c); dy = fy - cen(1, c); dz = DIM == 3 ? fz - cen(2, c) : R(0.0);
            }
            if constexpr (prescaled_gradients<P, EXACT>()) {
                // packed limiter-scaled gradients: q_f = q + (phi grad) . d
                const float4* src = (const float4*)v.grad + (size_t)c * (kPackedGrad / 4);
                float pk[kPackedGrad];
#pragma unroll
                for (int k = 0; k < (DIM == 3 ? 4 : 2); k++) {
                    const float4 t = src[k];
                    pk[4 * k] = t.x; pk[4 * k + 1] = t.y; pk[4 * k + 2] = t.z; pk[4 * k + 3] = t.w;
                }
                // the increment (phi grad) . d in float; with double face states
                // (MIXED_GRAD) it is added to the double cell value; the float-float
                // build forms it in float-float from the packed gradients' lo parts
                const float fdx = to_float(dx), fdy = to_float(dy), fdz = to_float(dz);
                float pl[kPackedGrad];
                if constexpr (FFR) {
                    const float4* slo = (const float4*)v.grad_lo + (size_t)c * (kPackedGrad / 4);
#pragma unroll
                    for (int k = 0; k < (DIM == 3 ? 4 : 2); k++) {
                        const float4 t = slo[k];
                        pl[4 * k] = t.x; pl[4 * k + 1] = t.y; pl[4 * k + 2] = t.z; pl[4 * k + 3] = t.w;
                    }
                }
                auto rec = [&](R val, int w) -> R {
                    if constexpr (FFR) {
                        auto g = [&](int k) { return FF(pk[k], pl[k]); };
                        const FF sgr = DIM == 3 ? g(3 * w) * dx + g(3 * w + 1) * dy + g(3 * w + 2) * dz
                                                : g(2 * w) * dx + g(2 * w + 1) * dy;
                        return val + sgr;
                    } else {
                        float sgr = DIM == 3 ? pk[3 * w] * fdx + pk[3 * w + 1] * fdy + pk[3 * w + 2] * fdz
                                             : pk[2 * w] * fdx + pk[2 * w + 1] * fdy;
                        return val + (R)sgr;
                    }
                };
                q[ia] = rec(q[ia], 0);
                q[ib] = rec(q[ib], 1);
                q[4] = rec(q[4], 2);
                q[5] = rec(q[5], 3);
                if (DIM == 3) q[6] = rec(q[6], 4);
            } else {
                const bool lim = prm.limiter != 0;
                auto L = [&](int k) { return lim ? (R)ph[k * N + c] : R(1.0); };
                q[ia] = lin_interp<R, P, DIM>(q[ia], L(0), gr, N, 0, c, dx, dy, dz);
                q[ib] = lin_interp<R, P, DIM>(q[ib], L(1), gr, N, 1, c, dx, dy, dz);
                q[4] = lin_interp<R, P, DIM>(q[4], L(2), gr, N, 2, c, dx, dy, dz);
                q[5] = lin_interp<R, P, DIM>(q[5], L(3), gr, N, 3, c, dx, dy, dz);
                if (DIM == 3) q[6] = lin_interp<R, P, DIM>(q[6], L(4), gr, N, 4, c, dx, dy, dz);
            }
        }
        // the ghost side is first order but passes through the same thermo closure
        side_state<R, DIM, EXACT>(prm.thermo, gm, reconstruct, q, nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z,
                                  S[side]);
    }
    convective_flux<R, DIM, EXACT>(prm, gm, S[0], S[1], nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z, Fg);
    if (prm.cflux) {  // apply_post_convective_flux_bc (finite_volume.cpp:71, 197-209)
        if (const BoundDev* B = constant_flux_bound(v, cells[0], cells[1])) {
            bool seeded = false;
            if constexpr (kIsDual<R>)
                if (v.fs_tan) {  // the flow-state tangent: the fixed state carries its direction
                    const double* d = v.fs_tan + 7 * (size_t)(B - v.bounds);
                    R fsd[7];
#pragma unroll
                    for (int k = 0; k < 7; k++) fsd[k] = R(B->cfs[k], d[k]);
                    constant_flux<R, DIM>(fsd, prm.Cv, nx, ny, nz, Fg);
                    seeded = true;
                }
            if (!seeded) constant_flux<R, DIM>(B->cfs, prm.Cv, nx, ny, nz, Fg);
        }
    }
    nx_out = nx;
    ny_out = ny;
    nz_out = nz;
}

template <class R, class P, class Gm, int DIM, bool EXACT, int BS = kBlock, int MINB = 1>
__global__ void __launch_bounds__(BS, MINB) k_face(DevView v, FvParams prm, int reconstruct) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.F) return;
    const int N = v.N, NT = v.NT, F = v.F, G = v.G;
    R Fg[5], nx, ny, nz;
    face_convective<R, P, Gm, DIM, EXACT>(v, prm, f, reconstruct, Fg, nx, ny, nz);
    R mx = Fg[1], my = Fg[2], mz = Fg[3];
    R en = Fg[4];

    if (prm.viscous) {
        // viscous_flux.cpp:130-232; the states and gradients of both sides, then viscous_face
        const Gm* cc = (const Gm*)v.cc;
        const P* pr = (const P*)v.prim;
        const Gas<R> gm(prm);
        const int l = v.left[f], r = v.right[f];
        const bool lv = l < N, rv = r < N;
        const P* vgd = (const P*)v.vgrad;
        const P* vgh = (const P*)v.vghost;
        // visc states of both sides (ghost: pre-viscous values): p, T, vx, vy, vz
        constexpr bool FFR = kFFBuild && std::is_same_v<R, FF>;
        auto vstate = [&](int c, int k) -> R {
            if (c >= N) {
                if constexpr (FFR) return FF((float)vgh[k * G + (c - N)], v.vghost_lo[k * G + (c - N)]);
                else return (R)vgh[k * G + (c - N)];
            }
            const int idx = (k == 0 ? 1 : visc_prim(k - 1)) * NT + c;
            if constexpr (FFR) return FF((float)pr[idx], v.prim_lo[idx]);
            else return (R)pr[idx];
        };
        auto cen = [&](int k, int c) -> R {
            if constexpr (FFR) return FF((float)cc[k * NT + c], v.cc_lo[k * NT + c]);
            else return (R)cc[k * NT + c];
        };
        R sl[5], sr[5], gl[12], grr[12];
#pragma unroll
        for (int k = 0; k < 5; k++) { sl[k] = vstate(l, k); sr[k] = vstate(r, k); }
        const bool interior = lv && rv;
        const int gl_c = interior ? l : (lv ? l : r), gr_c = interior ? r : gl_c;
#pragma unroll
        for (int k = 0; k < 12; k++) {
            if constexpr (FFR) {
                gl[k] = FF((float)vgd[k * N + gl_c], v.vgrad_lo[k * N + gl_c]);
                grr[k] = FF((float)vgd[k * N + gr_c], v.vgrad_lo[k * N + gr_c]);
            } else {
                gl[k] = (R)vgd[k * N + gl_c];
                grr[k] = (R)vgd[k * N + gr_c];
            }
        }
        R ex = R(0.0), ey = R(0.0), ez = R(0.0);
        if (interior) {
            ex = cen(0, r) - cen(0, l); ey = cen(1, r) - cen(1, l);
            ez = DIM == 3 ? cen(2, r) - cen(2, l) : R(0.0);
        }
        R vt[4], rho, mu, k;
        viscous_face<R, DIM, EXACT>(prm, gm, interior, sl, sr, gl, grr, ex, ey, ez, nx, ny, nz, vt, rho, mu, k);
        mx -= vt[0];
        my -= vt[1];
        if (DIM == 3) mz -= vt[2];
        en -= vt[3];
        // time-step signal (estimate_dt, finite_volume.cpp:167-175), in double
        double mud = real_of(mu), kd = real_of(k);
        double Prf = mud * prm.Cp / kd;
        v.vsig[f] = (prm.gamma / real_of(rho)) * (mud / Prf);
    }
    P* fo = (P*)v.flux;
    if constexpr (kFFBuild && std::is_same_v<R, FF>) {  // hi into the flux array, lo into its companion
        float* flo = v.flux_lo;
        fo[f] = Fg[0].hi; flo[f] = Fg[0].lo;
        fo[F + f] = mx.hi; flo[F + f] = mx.lo;
        fo[2 * F + f] = my.hi; flo[2 * F + f] = my.lo;
        if (DIM == 3) { fo[3 * F + f] = mz.hi; flo[3 * F + f] = mz.lo; }
        fo[(DIM + 1) * F + f] = en.hi; flo[(DIM + 1) * F + f] = en.lo;
    } else {
        fo[f] = (P)Fg[0];
        fo[F + f] = (P)mx;
        fo[2 * F + f] = (P)my;
        if (DIM == 3) fo[3 * F + f] = (P)mz;
        fo[(DIM + 1) * F + f] = (P)en;
    }
}

// ---------------------------------------------------------------------------
// k_update: surface integral (flux_surface_integral, finite_volume.cpp:220-255)
// in double, then (mode 2) the next stage state or (mode 3) the solution
// update, conserved->primitive inversion (primative_conserved_conversion.cpp:4-23)
// and the ghost cells fed by this cell.
// ---------------------------------------------------------------------------
// 1/x in double for x > 0 of normal range: the hardware's approximate reciprocal
// (PTX rcp.approx.ftz.f64) refined by two Newton-Raphson steps r <- r + r (1 - x r),
// each of which squares the relative error; the result is within an ulp or so
// of the correctly rounded reciprocal.
__device__ __forceinline__ double recip_newton(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    double e = fma(-x, r, 1.0);
    r = fma(r, e, r);
    e = fma(-x, r, 1.0);
    return fma(r, e, r);
}

// Inputs whose value or reciprocal is not a normal float take the double seed,
// in a call (not inlined, so that its instructions are not issued predicated
// for the common case).
__device__ __noinline__ double recip_by_double_seed(double x) { return recip_newton(x); }

// 1/x in double from a float reciprocal seed refined by one Newton step in
// double: the seed's relative error (below 2^-22) is squared, so the result is
// within 2^-44 of 1/x -- far below the float rounding of the primitives the
// mixed build stores, and it leaves the cancellation E/rho - |v|^2/2 in double.
// Two FP64 operations (one FMA for the residual, one for the step); inputs
// outside the normal float range take the double seed and two steps.
__device__ __forceinline__ double recip_newton1_fseed(double x) {
    const unsigned ex = ((unsigned)__double2hiint(x) >> 20) & 0x7FFu;
    if (ex - 897u > 251u) return recip_by_double_seed(x);  // |x| outside [2^-126, 2^126)
    float rf;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(d2f(x)));
    const double r = f2d(rf);
    return fma(r, fma(-x, r, 1.0), r);
}

// What the update needs of a committed state: rho (bad-cell test) and the
// stored temperature and velocity (local time step), at storage precision P.
template <class P>
struct Committed {
    double rho;
    P T, vx, vy, vz;
};

template <class P, class Gm, int DIM, bool EXACT>
__device__ Committed<P> commit_state(const DevView& v, const FvParams& prm, int i, const double* u) {
    // conserved_to_primatives in double (primative_conserved_conversion.cpp:4-23); the fast
    // paths replace the divisions by one reciprocal (the FP64 pipe is GB300's scarcest unit)
    double rho = u[0], vx, vy, vz, e, T;
    if constexpr (kFFBuild && sizeof(P) == sizeof(float)) {
        // float-float build: the inversion in double as the mixed build, T and p in
        // double too, each primitive stored as float + lo (integer-pipe split)
        const double ir = recip_newton1_fseed(rho);
        vx = u[1] * ir;
        vy = u[2] * ir;
        vz = DIM == 3 ? u[3] * ir : 0.0;
        double ke = 0.5 * (vx * vx + vy * vy + vz * vz);
        e = u[DIM + 1] * ir - ke;
        T = e * prm.inv_Cv;
        const double p = rho * prm.R * T;
        const double w[7] = {rho, p, T, e, vx, vy, vz};
        float* pr = (float*)v.prim;
        const int NT = v.NT;
        float hs[7];
#pragma unroll
        for (int k = 0; k < 7; k++) {
            const FF x = (DIM == 2 && k == 6) ? FF(0.f, 0.f) : d2ff(w[k]);
            hs[k] = x.hi;
            pr[k * NT + i] = x.hi;
            v.prim_lo[k * NT + i] = x.lo;
        }
        const State64 s{rho, p, T, e, vx, vy, vz};
        for (int k = v.feed_off[i]; k < v.feed_off[i + 1]; k++) fill_ghost<P, Gm>(v, prm, v.feed_ghost[k], s);
        return Committed<P>{rho, (P)hs[2], (P)hs[4], (P)hs[5], (P)hs[6]};
    }
    if (!EXACT && sizeof(P) == sizeof(float)) {
        // Mixed build: rho, v and e = E/rho - |v|^2/2 in double (the cancellation of
        // strong expansions happens there); T = e/Cv and p = rho R T are products of
        // values already rounded to float, so they are formed in float.
        const double ir = recip_newton1_fseed(rho);  // a state with rho <= 0 is a bad cell either way
        vx = u[1] * ir;
        vy = u[2] * ir;
        vz = DIM == 3 ? u[3] * ir : 0.0;
        double ke = 0.5 * (vx * vx + vy * vy + vz * vz);
        e = u[DIM + 1] * ir - ke;
        const float rf = d2f(rho), ef = d2f(e);
        const float Tf = ef * prm.finv_Cv;
        const float pf = rf * prm.fR * Tf;
        const float vxf = d2f(vx), vyf = d2f(vy), vzf = DIM == 3 ? d2f(vz) : 0.f;
        P* pr = (P*)v.prim;
        const int NT = v.NT;
        pr[i] = (P)rf; pr[NT + i] = (P)pf; pr[2 * NT + i] = (P)Tf; pr[3 * NT + i] = (P)ef;
        pr[4 * NT + i] = (P)vxf; pr[5 * NT + i] = (P)vyf; pr[6 * NT + i] = (P)vzf;
        const int k0 = v.feed_off[i], k1 = v.feed_off[i + 1];
        if (k0 < k1) {  // boundary cells: the ghost actions work on the double state
            const State64 s{rho, f2d(pf), f2d(Tf), e, vx, vy, vz};
            for (int k = k0; k < k1; k++) fill_ghost<P, Gm>(v, prm, v.feed_ghost[k], s);
        }
        return Committed<P>{rho, (P)Tf, (P)vxf, (P)vyf, (P)vzf};
    }
    if (EXACT) {
        vx = u[1] / rho;
        vy = u[2] / rho;
        vz = DIM == 3 ? u[3] / rho : 0.0;
        double ke = 0.5 * (vx * vx + vy * vy + vz * vz);
        e = u[DIM + 1] / rho - ke;
        T = e / prm.Cv;
    } else {
        const double ir = 1.0 / rho;
        vx = u[1] * ir;
        vy = u[2] * ir;
        vz = DIM == 3 ? u[3] * ir : 0.0;
        double ke = 0.5 * (vx * vx + vy * vy + vz * vz);
        e = u[DIM + 1] * ir - ke;
        T = e * prm.inv_Cv;
    }
    double p = rho * prm.R * T;
    P* pr = (P*)v.prim;
    const int NT = v.NT;
    pr[i] = (P)rho; pr[NT + i] = (P)p; pr[2 * NT + i] = (P)T; pr[3 * NT + i] = (P)e;
    pr[4 * NT + i] = (P)vx; pr[5 * NT + i] = (P)vy; pr[6 * NT + i] = (P)vz;
    const State64 s{rho, p, T, e, vx, vy, vz};
    for (int k = v.feed_off[i]; k < v.feed_off[i + 1]; k++) fill_ghost<P, Gm>(v, prm, v.feed_ghost[k], s);
    return Committed<P>{rho, (P)T, (P)vx, (P)vy, (P)vz};
}

// Storage slot of stage j's derivative: its own, or, when the stages alias
// (the reference's RungeKutta, whose stage derivatives share one array), slot 0
// for every stage, which then always holds the latest derivative.
IBISGB_HD int kslot(const DevView& v, int j) { return v.k_alias ? 0 : j; }

// control block of the case cell i belongs to
IBISGB_HD StepCtl* ctl_of(const DevView& v, int i) { return v.case_of ? v.ctl + v.case_of[i] : v.ctl; }

// count_bad_cells (finite_volume.cpp:257-270)
// T < 0, rho < 0, isnan(rho) or isinf(rho), tested on the bit patterns (the
// same predicates for IEEE doubles, without the FP64 pipe)
IBISGB_HD bool is_negative(double x) {  // x < 0.0: sign set, nonzero, not NaN
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long mag = b & 0x7FFFFFFFFFFFFFFFull;
    return (b >> 63) && mag != 0 && mag <= 0x7FF0000000000000ull;
}
IBISGB_HD bool is_negative(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned mag = b & 0x7FFFFFFFu;
    return (b >> 31) && mag != 0 && mag <= 0x7F800000u;
}
template <class P>
IBISGB_HD void count_bad(StepCtl* ctl, const Committed<P>& s) {
    const unsigned long long rb = (unsigned long long)__double_as_longlong(s.rho);
    if (is_negative(s.T) || is_negative(s.rho) || ((rb >> 52) & 0x7FFull) == 0x7FFull)
        atomicAdd(&ctl->bad_cells, 1ull);
}

// Error-free transformations for the float accumulation of the mixed build
// (Knuth's TwoSum, and the product error through an FMA).
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float p) {
    float s = __fadd_rn(hi, p);
    float bb = __fsub_rn(s, hi);
    float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, err);
}

// (hi + lo) * s as a double, for s given as the float pair s.x + s.y: the leading
// product hi * s.x, its exact rounding error (FMA) plus the cross terms hi * s.y
// and lo * s.x in float, formed in double by one addition (relative error about
// 2^-46, the precision of the float-pair sum itself).  One FP64 operation
// instead of the two of (f2d(hi) + f2d(lo)) * s.
__device__ __forceinline__ double pair_scale(float hi, float lo, float2 s) {
    const float p = __fmul_rn(hi, s.x);
    float e = __fmaf_rn(hi, s.x, -p);
    e = __fmaf_rn(hi, s.y, e);
    e = __fmaf_rn(lo, s.x, e);
    return f2d(p) + f2d(e);
}

// hi + lo += x * a, keeping the product's rounding error (an FMA gives it exactly)
// and the addition's (TwoSum).
__device__ __forceinline__ void pair_acc(float& hi, float& lo, float x, float a) {
    const float pr = __fmul_rn(x, a);
    const float pe = __fmaf_rn(x, a, -pr);
    two_sum_acc(hi, lo, pr);
    lo = __fadd_rn(lo, pe);
}

// Local CFL time step of valid cell i from its primitives (FiniteVolume::estimate_dt,
// finite_volume.cpp:130-184).  The float build evaluates the inviscid signal in
// float from its float state.
template <class P, class Gm, int DIM>
__device__ double cell_local_dt(const DevView& v, const FvParams& prm, int i, P pvx, P pvy, P pvz, P pT) {
    const int N = v.N, F = v.F;
    const Gm* fg = (const Gm*)v.face;
    const int nf = v.nfaces[i];
    double src = 0.0, srv = 0.0;
    const double vol = v.vol[i];
    if constexpr (kFFBuild && sizeof(P) == sizeof(float)) {
        // float-float build: the state this thread just committed (hi + lo) and the
        // geometry as hi + lo, the signal in float-float arithmetic
        const float* pr = (const float*)v.prim;
        const float* lo = v.prim_lo;
        const int NT = v.NT;
        const FF vx(pr[4 * NT + i], lo[4 * NT + i]), vy(pr[5 * NT + i], lo[5 * NT + i]);
        const FF vz = DIM == 3 ? FF(pr[6 * NT + i], lo[6 * NT + i]) : FF(0.f);
        const FF a = ff_sqrt(FF(prm.fgR, prm.logR) * FF(pr[2 * NT + i], lo[2 * NT + i]));
        FF sf(0.f);
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            const float* fl = v.face_lo;
            auto geo = [&](int k) { return FF((float)fg[k * F + f], fl[k * F + f]); };
            FF dot = vx * geo(0) + vy * geo(1);
            if (DIM == 3) dot = dot + vz * geo(2);
            const FF A = geo(12);
            sf = sf + (ff_abs(dot) + a) * A;
            if (prm.viscous) {
                const double Ad = ff_to_double(A);
                srv += v.vsig[f] * Ad * Ad / vol;
            }
        }
        if (!prm.viscous) {
            const FF lf = d2ff(vol) / sf;
            return lf.hi > 0.f ? ff_to_double(lf) : 1.0e308 * 10.0;
        }
        src = ff_to_double(sf);
    } else if (sizeof(P) == sizeof(float)) {
        const float vx = (float)pvx, vy = (float)pvy;
        const float vz = DIM == 3 ? (float)pvz : 0.f;
        const float a = sqrtf(prm.fgR * (float)pT);
        float sf = 0.f;
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            // a uniform lattice's face class holds the same normal and area
            const float* ct = v.face_class ? v.face_class_tab + kFaceClassRow * v.face_class[f] : nullptr;
            const float A = ct ? ct[12] : (float)fg[12 * F + f];
            float dot = vx * (ct ? ct[0] : (float)fg[f]) + vy * (ct ? ct[1] : (float)fg[F + f]);
            if (DIM == 3) dot += vz * (ct ? ct[2] : (float)fg[2 * F + f]);
            sf += (fabsf(dot) + a) * A;
            if (prm.viscous) srv += v.vsig[f] * (double)A * (double)A / vol;
        }
        if (!prm.viscous) {
            // the float build's inviscid signal is a float; so is its quotient
            const float lf = __fdiv_rn(d2f(vol), sf);
            return lf > 0.f ? f2d(lf) : 1.0e308 * 10.0;
        }
        src = f2d(sf);
    } else {
        const double vx = (double)pvx, vy = (double)pvy, vz = (double)pvz;
        const double a = sqrt(prm.gamma * prm.R * (double)pT);
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            const double A = (double)fg[12 * F + f];
            const double dot = vx * (double)fg[f] + vy * (double)fg[F + f] + vz * (double)fg[2 * F + f];
            src += (fabs(dot) + a) * A;
            if (prm.viscous) {
                double tmp = v.vsig[f] * A * A;
                srv += tmp / vol;
            }
        }
    }
    double local = vol / (src + prm.signal_factor * srv);
    if (!(local > 0.0)) local = 1.0e308 * 10.0;
    return local;
}

// Min-reduce the local time steps of a block into the control blocks' dt_bits
// (bits of a positive double order like the double).  Every thread of the
// block must call it; threads without a cell pass +inf.
__device__ void reduce_local_dt(const DevView& v, int i, double local) {
    if (v.case_of) {
        // batched ensemble: one min per case; a warp whose cells share a case
        // (the usual situation, cases are contiguous) reduces before its atomic
        const int cs = i < v.N ? v.case_of[i] : -1;
        const int c0 = __shfl_sync(0xffffffffu, cs, 0);
        if (__all_sync(0xffffffffu, cs == c0)) {
            for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_down_sync(0xffffffffu, local, o));
            if ((threadIdx.x & 31) == 0 && c0 >= 0)
                atomicMin(&v.ctl[c0].dt_bits, (unsigned long long)__double_as_longlong(local));
        } else if (cs >= 0) {
            atomicMin(&v.ctl[cs].dt_bits, (unsigned long long)__double_as_longlong(local));
        }
        return;
    }
    // warp-shuffle + block min, one atomic per block (blocks of up to 1024 threads)
    for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_down_sync(0xffffffffu, local, o));
    __shared__ double wmin[32];
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        double m = threadIdx.x < (blockDim.x >> 5) ? wmin[threadIdx.x] : 1.0e308 * 10.0;
        for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
        if (threadIdx.x == 0) atomicMin(&v.ctl->dt_bits, (unsigned long long)__double_as_longlong(m));
    }
}

// The part of k_update after the surface integral: the Runge-Kutta combination
// of `mode`, the primitives and ghosts of the new state (into v.prim) and, with
// with_dt, the new state's local time step.  ks holds the stage derivative, or,
// when fold, the mixed build's float pair (hi + lo) * iv stands for it.
// MODE >= 0 fixes the mode at compile time (the mixed build's Runge-Kutta
// launches), so that the other modes' double arithmetic is not issued,
// predicated off, to the FP64 pipe; MODE = -1 takes the `mode` argument.
template <class P, class Gm, int DIM, bool EXACT, int MODE = -1>
__device__ __forceinline__ double update_tail(const DevView& v, const FvParams& prm, int i, int mode_arg, int stage,
                                              int with_dt, const double* ks, bool fold, const float* hi,
                                              const float* lo, double iv) {
    constexpr double kInf = 1.0e308 * 10.0;
    constexpr int NC = DIM + 2;
    const int N = v.N;
    const int mode = MODE >= 0 ? MODE : mode_arg;
    if (mode < 2) return kInf;
    StepCtl* ctl = ctl_of(v, i);
    if (ctl->halt) return kInf;
    double u[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) u[q] = v.U[q * N + i];
    if (mode == 2) {
        // state of stage s+1 (runge_kutta.cpp:151-181)
        const int ns = stage + 1;
#pragma unroll
        for (int q = 0; q < NC; q++) u[q] = u[q] + (stage == 0 ? ks[q] : v.k[q * N + i]) * ctl->ca[ns][0];
        for (int j = 1; j < ns; j++) {
            if (!((ctl->a_used[ns] >> j) & 1u)) continue;
            const double c = ctl->ca[ns][j];
#pragma unroll
            for (int q = 0; q < NC; q++) {
                double kj = j == stage ? ks[q] : v.k[((size_t)kslot(v, j) * NC + q) * N + i];
                u[q] += kj * c;
            }
        }
        commit_state<P, Gm, DIM, EXACT>(v, prm, i, u);
        return kInf;
    }
    // solution update (runge_kutta.cpp:185-193)
    if (fold) {
        for (int j = 0; j < ctl->stages; j++) {
            if (j == stage) continue;
            const double c = ctl->cb[j];
#pragma unroll
            for (int q = 0; q < NC; q++) u[q] += v.k[((size_t)kslot(v, j) * NC + q) * N + i] * c;
        }
        const double c = ctl->cb[stage] * iv;
#pragma unroll
        for (int q = 0; q < NC; q++) u[q] = fma(f2d(lo[q]), c, fma(f2d(hi[q]), c, u[q]));
    } else {
        for (int j = 0; j < ctl->stages; j++) {
            const double c = ctl->cb[j];
#pragma unroll
            for (int q = 0; q < NC; q++) {
                double kj = j == stage ? ks[q] : v.k[((size_t)kslot(v, j) * NC + q) * N + i];
                u[q] += kj * c;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < NC; q++) v.U[q * N + i] = u[q];
    const Committed<P> st = commit_state<P, Gm, DIM, EXACT>(v, prm, i, u);
    count_bad(ctl, st);
    if (!with_dt) return kInf;
    return cell_local_dt<P, Gm, DIM>(v, prm, i, st.vx, st.vy, st.vz, st.T);
}

// One valid cell of k_update; returns the local time step of the new state when
// with_dt (mode 3), else +inf.
template <class P, class Gm, int DIM, bool EXACT, int MODE = -1>
__device__ __forceinline__ double update_cell(const DevView& v, const FvParams& prm, int i, int mode_arg, int stage,
                                              double* out_rm, int with_dt) {
    constexpr int NC = DIM + 2;
    const int mode = MODE >= 0 ? MODE : mode_arg;
    const int N = v.N, F = v.F;
    const Gm* area = (const Gm*)v.face + 12 * F;
    const P* fl = (const P*)v.flux;
    const int nf = v.nfaces[i];
    double ks[NC];
    // Mixed, last stage of a multi-stage step: the stage derivative is never read
    // again, so it is not stored and its float pair goes straight into the update.
    const bool fold = sizeof(P) == sizeof(float) && mode == 3 && stage > 0 && !out_rm && !v.k_alias;
    float hi[NC], lo[NC];
    double iv = 0.0;
    if (sizeof(P) == sizeof(float)) {
        // Mixed: each face term (float flux x area) is summed as an unevaluated
        // float pair (hi + lo, ~48-bit significand: the exact products' rounding
        // errors and every addition error are kept), then formed in double once.
#pragma unroll
        for (int q = 0; q < NC; q++) { hi[q] = 0.f; lo[q] = 0.f; }
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            const float sg = (float)v.outsign[s * N + i];
            const float a = -(float)area[f] * sg;
            if constexpr (kFFBuild) {
                // float-float flux times float-float area: hi*a, lo*a and hi*a_lo
                const float alo = -v.face_lo[12 * F + f] * sg;
#pragma unroll
                for (int q = 0; q < NC; q++) {
                    const float x = (float)fl[q * F + f];
                    pair_acc(hi[q], lo[q], x, a);
                    pair_acc(hi[q], lo[q], v.flux_lo[q * F + f], a);
                    pair_acc(hi[q], lo[q], x, alo);
                }
            } else {
#pragma unroll
                for (int q = 0; q < NC; q++) pair_acc(hi[q], lo[q], (float)fl[q * F + f], a);
            }
        }
        if (fold) {
            iv = v.inv_vol[i];
        } else {
            const float2 ivp = v.inv_vol2[i];
#pragma unroll
            for (int q = 0; q < NC; q++) ks[q] = pair_scale(hi[q], lo[q], ivp);
        }
    } else {
        double acc[NC];
#pragma unroll
        for (int q = 0; q < NC; q++) acc[q] = 0.0;
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            const double a = -(double)area[f] * (double)v.outsign[s * N + i];
#pragma unroll
            for (int q = 0; q < NC; q++) acc[q] += (double)fl[q * F + f] * a;
        }
        if (EXACT) {
            const double vol = v.vol[i];
#pragma unroll
            for (int q = 0; q < NC; q++) ks[q] = acc[q] / vol;
        } else {
            const double iv = v.inv_vol[i];
#pragma unroll
            for (int q = 0; q < NC; q++) ks[q] = acc[q] * iv;
        }
    }
    if (!fold) {
        double* kk = v.k + (size_t)kslot(v, stage) * NC * N;
#pragma unroll
        for (int q = 0; q < NC; q++) {
            kk[q * N + i] = ks[q];
            if (out_rm) out_rm[(size_t)i * NC + q] = ks[q];
        }
    }
    return update_tail<P, Gm, DIM, EXACT, MODE>(v, prm, i, mode, stage, with_dt, ks, fold, hi, lo, iv);
}

template <class P, class Gm, int DIM, bool EXACT, int BS = kBlock, int MINB = 1, int MODE = -1>
__global__ void __launch_bounds__(BS, MINB) k_update(DevView v, FvParams prm, int mode, int stage,
                                                   double* out_rm, int with_dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 1.0e308 * 10.0;
    if (i < v.N) local = update_cell<P, Gm, DIM, EXACT, MODE>(v, prm, i, mode, stage, out_rm, with_dt);
    if (with_dt) reduce_local_dt(v, i, local);
}

// Mixed build, inviscid Runge-Kutta stages: the face fluxes are recomputed by
// each cell that needs them (an interior face twice) and summed straight into
// the update, instead of being written by k_face and gathered by k_update.  The
// flux of every face is formed by the same function as k_face's, so the result
// is the same bits as k_face + k_update.  Trades the flux array's write and
// gather and one launch for twice the flux arithmetic, which runs on the FP32
// pipe beside the update's FP64 work.  Cells read their neighbours' primitives
// while others commit new ones, so the new primitives (and ghosts) go to the
// other buffer, prim_out.
template <int DIM, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_cell_update(DevView v, FvParams prm, int reconstruct, int mode,
                                                        int stage, int with_dt, float* prim_out) {
    constexpr int NC = DIM + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 1.0e308 * 10.0;
    if (i < v.N) {
        const int N = v.N, F = v.F;
        const float* area = (const float*)v.face + 12 * F;
        const int nf = v.nfaces[i];
        float hi[NC], lo[NC];
#pragma unroll
        for (int q = 0; q < NC; q++) { hi[q] = 0.f; lo[q] = 0.f; }
        for (int s = 0; s < nf; s++) {
            const int f = v.cell_face[s * N + i];
            float Fg[5], nx, ny, nz;
            face_convective<float, float, float, DIM, false>(v, prm, f, reconstruct, Fg, nx, ny, nz);
            const float a = -area[f] * (float)v.outsign[s * N + i];
#pragma unroll
            for (int q = 0; q < NC; q++) pair_acc(hi[q], lo[q], Fg[q < DIM + 1 ? q : 4], a);
        }
        double ks[NC];
        const bool fold = mode == 3 && stage > 0;
        const double iv = fold ? v.inv_vol[i] : 0.0;
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
        vo.prim = prim_out;
        local = update_tail<float, float, DIM, false>(vo, prm, i, mode, stage, with_dt, ks, fold, hi, lo, iv);
        if (ctl_of(v, i)->halt) {
            // a halted case keeps its state: carry its primitives into the other buffer
            const float* pr = (const float*)v.prim;
            const int NT = v.NT;
            for (int q = 0; q < 7; q++) prim_out[q * NT + i] = pr[q * NT + i];
            for (int k = v.feed_off[i]; k < v.feed_off[i + 1]; k++) {
                const int id = N + v.feed_ghost[k];
                for (int q = 0; q < 7; q++) prim_out[q * NT + id] = pr[q * NT + id];
            }
        }
    }
    if (with_dt) reduce_local_dt(v, i, local);
}

// Solution update from stored stage derivatives (single-stage tableaus, where
// dt is only known after the one residual evaluation).
template <class P, class Gm, int DIM, bool EXACT>
__global__ void __launch_bounds__(kBlock) k_finalize(DevView v, FvParams prm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    StepCtl* ctl = ctl_of(v, i);
    if (ctl->halt) return;
    constexpr int NC = DIM + 2;
    const int N = v.N;
    double u[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) u[q] = v.U[q * N + i];
    for (int j = 0; j < ctl->stages; j++) {
        const double c = ctl->cb[j];
#pragma unroll
        for (int q = 0; q < NC; q++) u[q] += v.k[((size_t)kslot(v, j) * NC + q) * N + i] * c;
    }
#pragma unroll
    for (int q = 0; q < NC; q++) v.U[q * N + i] = u[q];
    count_bad(ctl, commit_state<P, Gm, DIM, EXACT>(v, prm, i, u));
}

// State of stage `stage` from U and k_0..k_{stage-1} (after dt is known), then primitives and ghosts.
template <class P, class Gm, int DIM, bool EXACT>
__global__ void __launch_bounds__(kBlock) k_combine(DevView v, FvParams prm, int stage) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    const StepCtl* ctl = ctl_of(v, i);
    if (ctl->halt) return;
    constexpr int NC = DIM + 2;
    const int N = v.N;
    double u[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) u[q] = v.U[q * N + i] + v.k[q * N + i] * ctl->ca[stage][0];
    for (int j = 1; j < stage; j++) {
        if (!((ctl->a_used[stage] >> j) & 1u)) continue;
        const double c = ctl->ca[stage][j];
#pragma unroll
        for (int q = 0; q < NC; q++) u[q] += v.k[((size_t)kslot(v, j) * NC + q) * N + i] * c;
    }
    commit_state<P, Gm, DIM, EXACT>(v, prm, i, u);
}

template <class P, class Gm, int DIM, bool EXACT>
__global__ void __launch_bounds__(kBlock) k_prims_from_U(DevView v, FvParams prm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.N) return;
    constexpr int NC = DIM + 2;
    double u[NC];
#pragma unroll
    for (int q = 0; q < NC; q++) u[q] = v.U[q * v.N + i];
    commit_state<P, Gm, DIM, EXACT>(v, prm, i, u);
}

// U of valid cell i from its row (row map[i] of the rows when map is set), then
// what k_prims_from_U and (with_dt) k_local_dt do for it, in one pass.
template <class P, class Gm, int DIM, bool EXACT>
__global__ void __launch_bounds__(kBlock) k_load_state(DevView v, FvParams prm, const double* rows, const int32_t* map,
                                                     int with_dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 1.0e308 * 10.0;
    if (i < v.N) {
        constexpr int NC = DIM + 2;
        const long long r = map ? (long long)map[i] : (long long)i;
        double u[NC];
#pragma unroll
        for (int q = 0; q < NC; q++) {
            u[q] = rows[r * NC + q];
            v.U[q * v.N + i] = u[q];
        }
        const Committed<P> st = commit_state<P, Gm, DIM, EXACT>(v, prm, i, u);
        if (with_dt) local = cell_local_dt<P, Gm, DIM>(v, prm, i, st.vx, st.vy, st.vz, st.T);
    }
    if (with_dt) reduce_local_dt(v, i, local);
}

// Local CFL time step of each valid cell, min-reduced into ctl->dt_bits.
template <class P, class Gm, int DIM>
__global__ void __launch_bounds__(kBlock) k_local_dt(DevView v, FvParams prm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double local = 1.0e308 * 10.0;
    if (i < v.N) {
        const P* pr = (const P*)v.prim;
        const int NT = v.NT;
        local = cell_local_dt<P, Gm, DIM>(v, prm, i, pr[4 * NT + i], pr[5 * NT + i], pr[6 * NT + i], pr[2 * NT + i]);
    }
    reduce_local_dt(v, i, local);
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
// RR: arithmetic of the gradient/limiter kernel when it differs from the face
// kernel's R (the MIXED_GRAD family: float gradients, double fluxes).
template <class R, class P, class Gm, bool EXACT, class RR = R>
struct Launch {
    static void ghost_fill(const DevView& v, const FvParams& p, cudaStream_t s) {
        if (v.G > 0) k_ghost_fill<P, Gm><<<blocks_for(v.G), kBlock, 0, s>>>(v, p);
    }
    // Launch variants of the stage kernels (threads per block, minimum resident
    // blocks per SM, which caps registers per thread), chosen per context by the
    // autotuner; every variant computes bit-identical results.
    template <int V>
    static void recon_v(const DevView& v, const FvParams& p, bool reco, cudaStream_t s) {
        constexpr int BS = kVariantThreads[V], MB = kVariantMinBlocks[V];
        const unsigned g = (unsigned)((v.N + BS - 1) / BS);
        if (v.dim == 3) k_recon<RR, P, Gm, 3, EXACT, BS, MB><<<g, BS, 0, s>>>(v, p, reco);
        else k_recon<RR, P, Gm, 2, EXACT, BS, MB><<<g, BS, 0, s>>>(v, p, reco);
    }
    template <int V>
    static void face_v(const DevView& v, const FvParams& p, bool reco, cudaStream_t s) {
        constexpr int BS = kVariantThreads[V], MB = kVariantMinBlocks[V];
        const unsigned g = (unsigned)((v.F + BS - 1) / BS);
        if (v.dim == 3) k_face<R, P, Gm, 3, EXACT, BS, MB><<<g, BS, 0, s>>>(v, p, reco);
        else k_face<R, P, Gm, 2, EXACT, BS, MB><<<g, BS, 0, s>>>(v, p, reco);
    }
    template <int V, int MODE>
    static void update_vm(const DevView& v, const FvParams& p, int mode, int stage, double* out, int with_dt,
                          cudaStream_t s) {
        constexpr int BS = kVariantThreads[V], MB = kVariantMinBlocks[V];
        const unsigned g = (unsigned)((v.N + BS - 1) / BS);
        if (v.dim == 3) k_update<P, Gm, 3, EXACT, BS, MB, MODE><<<g, BS, 0, s>>>(v, p, mode, stage, out, with_dt);
        else k_update<P, Gm, 2, EXACT, BS, MB, MODE><<<g, BS, 0, s>>>(v, p, mode, stage, out, with_dt);
    }
    template <int V>
    static void update_v(const DevView& v, const FvParams& p, int mode, int stage, double* out, int with_dt,
                         cudaStream_t s) {
        // the mixed build's Runge-Kutta modes get their own instances (see update_tail)
        constexpr bool kModes = sizeof(P) == sizeof(float) && !EXACT;
        if (kModes && mode == 2) update_vm<V, kModes ? 2 : -1>(v, p, mode, stage, out, with_dt, s);
        else if (kModes && mode == 3) update_vm<V, kModes ? 3 : -1>(v, p, mode, stage, out, with_dt, s);
        else update_vm<V, -1>(v, p, mode, stage, out, with_dt, s);
    }
    static void recon(const DevView& v, const FvParams& p, bool reco, int var, cudaStream_t s) {
        if (!reco && !p.viscous) return;
        if constexpr (EXACT) {
            recon_v<0>(v, p, reco, s);
        } else {
            switch (var) {
                case 1: recon_v<1>(v, p, reco, s); break;
                case 2: recon_v<2>(v, p, reco, s); break;
                case 3: recon_v<3>(v, p, reco, s); break;
                case 4: recon_v<4>(v, p, reco, s); break;
                default: recon_v<0>(v, p, reco, s); break;
            }
        }
    }
    static void face_flux(const DevView& v, const FvParams& p, bool reco, int var, cudaStream_t s) {
        if constexpr (EXACT) {
            face_v<0>(v, p, reco, s);
        } else {
            switch (var) {
                case 1: face_v<1>(v, p, reco, s); break;
                case 2: face_v<2>(v, p, reco, s); break;
                case 3: face_v<3>(v, p, reco, s); break;
                case 4: face_v<4>(v, p, reco, s); break;
                default: face_v<0>(v, p, reco, s); break;
            }
        }
    }
    static void update(const DevView& v, const FvParams& p, int mode, int stage, double* out, int with_dt,
                       int var, cudaStream_t s) {
        if constexpr (EXACT) {
            update_v<0>(v, p, mode, stage, out, with_dt, s);
        } else {
            switch (var) {
                case 1: update_v<1>(v, p, mode, stage, out, with_dt, s); break;
                case 2: update_v<2>(v, p, mode, stage, out, with_dt, s); break;
                case 3: update_v<3>(v, p, mode, stage, out, with_dt, s); break;
                case 4: update_v<4>(v, p, mode, stage, out, with_dt, s); break;
                default: update_v<0>(v, p, mode, stage, out, with_dt, s); break;
            }
        }
    }
    template <int V>
    static void cell_update_v(const DevView& v, const FvParams& p, bool reco, int mode, int stage, int with_dt,
                              void* po, cudaStream_t s) {
        constexpr int BS = kVariantThreads[V], MB = kVariantMinBlocks[V];
        const unsigned g = (unsigned)((v.N + BS - 1) / BS);
        float* out = (float*)po;
        if (v.dim == 3) k_cell_update<3, BS, MB><<<g, BS, 0, s>>>(v, p, reco, mode, stage, with_dt, out);
        else k_cell_update<2, BS, MB><<<g, BS, 0, s>>>(v, p, reco, mode, stage, with_dt, out);
    }
    // the mixed build's per-cell flux + update (inviscid Runge-Kutta stages, mode 2 or 3)
    static void cell_update(const DevView& v, const FvParams& p, bool reco, int mode, int stage, int with_dt,
                            int var, void* prim_out, cudaStream_t s) {
        if constexpr (sizeof(P) == sizeof(float) && !EXACT) {
            switch (var) {
                case 1: cell_update_v<1>(v, p, reco, mode, stage, with_dt, prim_out, s); break;
                case 2: cell_update_v<2>(v, p, reco, mode, stage, with_dt, prim_out, s); break;
                case 3: cell_update_v<3>(v, p, reco, mode, stage, with_dt, prim_out, s); break;
                case 4: cell_update_v<4>(v, p, reco, mode, stage, with_dt, prim_out, s); break;
                default: cell_update_v<0>(v, p, reco, mode, stage, with_dt, prim_out, s); break;
            }
        }
    }
    static void combine(const DevView& v, const FvParams& p, int stage, cudaStream_t s) {
        if (v.dim == 3) k_combine<P, Gm, 3, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p, stage);
        else k_combine<P, Gm, 2, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p, stage);
    }
    static void prims_from_U(const DevView& v, const FvParams& p, cudaStream_t s) {
        if (v.dim == 3) k_prims_from_U<P, Gm, 3, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p);
        else k_prims_from_U<P, Gm, 2, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p);
    }
    static void load_state(const DevView& v, const FvParams& p, const double* rows, const int32_t* map, int with_dt,
                           cudaStream_t s) {
        if (v.dim == 3) k_load_state<P, Gm, 3, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p, rows, map, with_dt);
        else k_load_state<P, Gm, 2, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p, rows, map, with_dt);
    }
    static void local_dt(const DevView& v, const FvParams& p, cudaStream_t s) {
        if (v.dim == 3) k_local_dt<P, Gm, 3><<<blocks_for(v.N), kBlock, 0, s>>>(v, p);
        else k_local_dt<P, Gm, 2><<<blocks_for(v.N), kBlock, 0, s>>>(v, p);
    }
    static void finalize(const DevView& v, const FvParams& p, cudaStream_t s) {
        if (v.dim == 3) k_finalize<P, Gm, 3, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p);
        else k_finalize<P, Gm, 2, EXACT><<<blocks_for(v.N), kBlock, 0, s>>>(v, p);
    }
    static KernelOps ops() {
        return KernelOps{&ghost_fill, &recon, &face_flux, &update, &combine, &prims_from_U, &local_dt,
                         &finalize, sizeof(P) == sizeof(float) && !EXACT && !kFFBuild ? &cell_update : nullptr,
                         &load_state};
    }
};

}  // namespace IBISGB_KNS
}  // namespace ibisgb
