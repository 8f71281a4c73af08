// Device numerics of the residual: thermodynamic closures, the four flux
// calculators in the face-normal frame and Sutherland transport.  Templated on
// the arithmetic type R (double or float).  Expressions keep the reference's
// operation order (comments cite it) so that the double build compiled without
// FMA contraction reproduces ibis bit for bit.
#pragma once

#include <type_traits>

#include <cuda_runtime.h>

#include "engine.hpp"
#include "ff.cuh"

namespace ibisgb {

#define IBISGB_HD __device__ __forceinline__

template <bool RefFloor> struct DualT;  // dual.cuh
using Dual = DualT<true>;
using DualA = DualT<false>;
template <class R> constexpr bool kIsDual = false;
template <bool B> constexpr bool kIsDual<DualT<B>> = true;

template <class R> IBISGB_HD R d_sqrt(R x);
template <> IBISGB_HD double d_sqrt<double>(double x) { return sqrt(x); }
template <> IBISGB_HD float d_sqrt<float>(float x) { return sqrtf(x); }
template <class R> IBISGB_HD R d_abs(R x);
template <> IBISGB_HD double d_abs<double>(double x) { return fabs(x); }
template <> IBISGB_HD float d_abs<float>(float x) { return fabsf(x); }
template <class R> IBISGB_HD R d_pow(R b, R e);
template <> IBISGB_HD double d_pow<double>(double b, double e) { return pow(b, e); }
template <> IBISGB_HD float d_pow<float>(float b, float e) { return powf(b, e); }
template <class R> IBISGB_HD R d_floor(R x);
template <> IBISGB_HD double d_floor<double>(double x) { return floor(x); }
template <> IBISGB_HD float d_floor<float>(float x) { return floorf(x); }
template <class R> IBISGB_HD R d_copysign(R m, R s);
template <> IBISGB_HD double d_copysign<double>(double m, double s) { return copysign(m, s); }
template <> IBISGB_HD float d_copysign<float>(float m, float s) { return copysignf(m, s); }
template <> IBISGB_HD FF d_sqrt<FF>(FF x) { return ff_sqrt(x); }
template <> IBISGB_HD FF d_abs<FF>(FF x) { return ff_abs(x); }
template <> IBISGB_HD FF d_floor<FF>(FF x) { return ff_floor(x); }
template <> IBISGB_HD FF d_copysign<FF>(FF m, FF s) { return ff_copysign(m, s); }
// the powers the float-float kernels meet (b^2 in LDFSS2, b^1.5 in Sutherland's
// law) in float-float; any other power through double
template <> IBISGB_HD FF d_pow<FF>(FF b, FF e) {
    if (e.hi == 2.f && e.lo == 0.f) return b * b;
    if (e.hi == 1.5f && e.lo == 0.f) return b * ff_sqrt(b);
    const double r = pow(ff_to_double(b), ff_to_double(e));
    const float h = (float)r;
    return FF(h, (float)(r - (double)h));
}
// Kokkos::min / max semantics (ties keep the first operand)
template <class R> IBISGB_HD R d_min(R a, R b) { return (b < a) ? b : a; }
template <class R> IBISGB_HD R d_max(R a, R b) { return (a < b) ? b : a; }

// A parameter in the arithmetic of the kernel: the double value, or its float
// copy prepared on the host for float kernels.
// Float-float kernels take the float copy plus what it leaves out (lo).
template <class R> IBISGB_HD R par(double d, float, float = 0.f) { return R(d); }
template <> IBISGB_HD float par<float>(double, float f, float) { return f; }
template <> IBISGB_HD FF par<FF>(double, float f, float lo) { return FF(f, lo); }

// Gas constants in the arithmetic of the kernel.
template <class R>
struct Gas {
    R R_, Cv, Cp, gamma, gR;  // gR = gamma * R, as in speed_of_sound_ (gas_model.h:27-30)
    R iCv;                    // 1 / Cv: the float-float build multiplies by it instead of dividing
    IBISGB_HD explicit Gas(const FvParams& p)
        : R_(par<R>(p.R, p.fR, p.loR)), Cv(par<R>(p.Cv, p.fCv, p.loCv)), Cp(par<R>(p.Cp, p.fCp, p.loCp)),
          gamma(par<R>(p.gamma, p.fgamma, p.logamma)), gR(par<R>(p.gamma * p.R, p.fgR, p.logR)),
          iCv(par<R>(p.inv_Cv, p.finv_Cv, p.loinv_Cv)) {}
    IBISGB_HD R sound(R T) const { return d_sqrt<R>(gR * T); }
};

// One side of a face in the face frame (u normal, v/w tangential).
template <class R>
struct FaceSide {
    R r, p, T, u, v, w;
};

// Hanel flux (src/finite_volume/finite_volume/flux_calculators/hanel.cpp:7-65).
// F = (mass, normal momentum, t1 momentum, t2 momentum, energy).
template <class R, int DIM>
IBISGB_HD void flux_hanel(const FaceSide<R>& L, const FaceSide<R>& Rt, const Gas<R>& gm, R* F) {
    R rL = L.r, pL = L.p, eL = gm.Cv * L.T, aL = gm.sound(L.T);
    R uL = L.u, vL = L.v, wL = L.w;
    R keL = DIM == 3 ? R(0.5) * (uL * uL + vL * vL + wL * wL) : R(0.5) * (uL * uL + vL * vL);
    R pLrL = pL / rL;
    R HL = eL + pLrL + keL;
    R rR = Rt.r, pR = Rt.p, eR = gm.Cv * Rt.T, aR = gm.sound(Rt.T);
    R uR = Rt.u, vR = Rt.v, wR = Rt.w;
    R keR = DIM == 3 ? R(0.5) * (uR * uR + vR * vR + wR * wR) : R(0.5) * (uR * uR + vR * vR);
    R pRrR = pR / rR;
    R HR = eR + pRrR + keR;
    R pLplus, uLplus;
    if (d_abs(uL) <= aL) {
        if constexpr (std::is_same<R, FF>::value) {  // one reciprocal of a for its three uses
            const R ia = R(1.f) / aL;
            uLplus = ia * 0.25f * (uL + aL) * (uL + aL);
            pLplus = pL * uLplus * (ia * (R(2.0) - uL * ia));
        } else {
            uLplus = R(1.0) / (R(4.0) * aL) * (uL + aL) * (uL + aL);
            pLplus = pL * uLplus * (R(1.0) / aL * (R(2.0) - uL / aL));
        }
    } else {
        uLplus = R(0.5) * (uL + d_abs(uL));
        pLplus = pL * uLplus * (R(1.0) / uL);
    }
    R pRminus, uRminus;
    if (d_abs(uR) <= aR) {
        if constexpr (std::is_same<R, FF>::value) {
            const R ia = R(1.f) / aR;
            uRminus = -(ia * 0.25f * (uR - aR) * (uR - aR));
            pRminus = pR * uRminus * (ia * (R(-2.0) - uR * ia));
        } else {
            uRminus = R(-1.0) / (R(4.0) * aR) * (uR - aR) * (uR - aR);
            pRminus = pR * uRminus * (R(1.0) / aR * (R(-2.0) - uR / aR));
        }
    } else {
        uRminus = R(0.5) * (uR - d_abs(uR));
        pRminus = pR * uRminus * (R(1.0) / uR);
    }
    R p_half = pLplus + pRminus;
    F[0] = uLplus * rL + uRminus * rR;
    F[1] = uLplus * rL * uL + uRminus * rR * uR + p_half;
    F[2] = uLplus * rL * vL + uRminus * rR * vR;
    F[3] = DIM == 3 ? uLplus * rL * wL + uRminus * rR * wR : R(0.0);
    F[4] = uLplus * rL * HL + uRminus * rR * HR;
}

// AUSMDV flux (flux_calculators/ausmdv.cpp:8-132)
template <class R, int DIM>
IBISGB_HD void flux_ausmdv(const FaceSide<R>& L, const FaceSide<R>& Rt, const Gas<R>& gm, R* F) {
    R rL = L.r, pL = L.p, pLrL = pL / rL, uL = L.u, vL = L.v, wL = L.w;
    R eL = gm.Cv * L.T, aL = gm.sound(L.T);
    R keL = DIM == 3 ? R(0.5) * (uL * uL + vL * vL + wL * wL) : R(0.5) * (uL * uL + vL * vL);
    R HL = eL + pLrL + keL;
    R rR = Rt.r, pR = Rt.p, pRrR = pR / rR, uR = Rt.u, vR = Rt.v, wR = Rt.w;
    R eR = gm.Cv * Rt.T, aR = gm.sound(Rt.T);
    R keR = DIM == 3 ? R(0.5) * (uR * uR + vR * vR + wR * wR) : R(0.5) * (uR * uR + vR * vR);
    R HR = eR + pRrR + keR;
    R alphaL = R(2.0) * pLrL / (pLrL + pRrR);
    R alphaR = R(2.0) * pRrR / (pLrL + pRrR);
    R am = d_max(aL, aR);
    R ML = uL / am, MR = uR / am;
    R pLplus, uLplus;
    R duL = R(0.5) * (uL + d_abs(uL));
    if (d_abs(ML) <= R(1.0)) {
        pLplus = pL * (ML + R(1.0)) * (ML + R(1.0)) * (R(2.0) - ML) * R(0.25);
        uLplus = alphaL * ((uL + am) * (uL + am) / (R(4.0) * am) - duL) + duL;
    } else {
        pLplus = pL * duL / uL;
        uLplus = duL;
    }
    R pRminus, uRminus;
    R duR = R(0.5) * (uR - d_abs(uR));
    if (d_abs(MR) <= R(1.0)) {
        pRminus = pR * (MR - R(1.0)) * (MR - R(1.0)) * (R(2.0) + MR) * R(0.25);
        uRminus = alphaR * (-(uR - am) * (uR - am) / (R(4.0) * am) - duR) + duR;
    } else {
        pRminus = pR * duR / uR;
        uRminus = duR;
    }
    R ru_half = uLplus * rL + uRminus * rR;
    R p_half = pLplus + pRminus;
    R dp = pL - pR;
    dp = R(10.0) * d_abs(dp) / d_min(pL, pR);
    R s = R(0.5) * d_min(R(1.0), dp);
    R ru2_AUSMV = uLplus * rL * uL + uRminus * rR * uR;
    R ru2_AUSMD = R(0.5) * (ru_half * (uL + uR) - d_abs(ru_half) * (uR - uL));
    R ru2_half = (R(0.5) + s) * ru2_AUSMV + (R(0.5) - s) * ru2_AUSMD;
    F[0] = ru_half;
    F[1] = ru2_half + p_half;
    if (ru_half >= R(0.0)) {
        F[2] = ru_half * vL;
        F[3] = DIM == 3 ? ru_half * wL : R(0.0);
        F[4] = ru_half * HL;
    } else {
        F[2] = ru_half * vR;
        F[3] = DIM == 3 ? ru_half * wR : R(0.0);
        F[4] = ru_half * HR;
    }
    bool caseA = ((uL - aL) < R(0.0)) && ((uR - aR) > R(0.0));
    bool caseB = ((uL + aL) < R(0.0)) && ((uR + aR) > R(0.0));
    R d_ua = R(0.0);
    if (caseA && !caseB) d_ua = R(0.125) * ((uR - aR) - (uL - aL));
    if (caseB && !caseA) d_ua = R(0.125) * ((uR + aR) - (uL + aL));
    if (d_ua != R(0.0)) {
        F[0] -= d_ua * (rR - rL);
        F[1] -= d_ua * (rR * uR - rL * uL);
        F[2] -= d_ua * (rR * vR - rL * vL);
        if (DIM == 3) F[3] -= d_ua * (rR * wR - rL * wL);
        F[4] -= d_ua * (rR * HR - rL * HL);
    }
}

// LDFSS(2) flux (flux_calculators/ldfss2.cpp:9-90); EXACT keeps the
// reference's pow(x, 2.0), the fast paths square instead.  The tangent squares
// too: the reference's dual pow adds 0*log(x), which is NaN for x < 0.
template <class R, int DIM, bool EXACT>
IBISGB_HD void flux_ldfss2(const FaceSide<R>& L, const FaceSide<R>& Rt, const Gas<R>& gm, R delta,
                           R* F) {
    R rL = L.r, pL = L.p, pLrL = pL / rL, uL = L.u, vL = L.v, wL = L.w;
    R eL = gm.Cv * L.T, aL = gm.sound(L.T);
    R keL = DIM == 3 ? R(0.5) * (uL * uL + vL * vL + wL * wL) : R(0.5) * (uL * uL + vL * vL);
    R HL = eL + pLrL + keL;
    R rR = Rt.r, pR = Rt.p, pRrR = pR / rR, uR = Rt.u, vR = Rt.v, wR = Rt.w;
    R eR = gm.Cv * Rt.T, aR = gm.sound(Rt.T);
    R keR = DIM == 3 ? R(0.5) * (uR * uR + vR * vR + wR * wR) : R(0.5) * (uR * uR + vR * vR);
    R HR = eR + pRrR + keR;
    R am = R(0.5) * (aL + aR);
    R ML = uL / am, MR = uR / am;
    R MpL = R(0.25) * (ML + R(1.0)) * (ML + R(1.0));
    R MmR = R(-0.25) * (MR - R(1.0)) * (MR - R(1.0));
    R alphaL = R(0.5) * (R(1.0) + d_copysign(R(1.0), ML));
    R alphaR = R(0.5) * (R(1.0) - d_copysign(R(1.0), MR));
    R betaL = -d_max(R(0.0), R(1.0) - d_floor(d_abs(ML)));
    R betaR = -d_max(R(0.0), R(1.0) - d_floor(d_abs(MR)));
    R PL = R(0.25) * (ML + R(1.0)) * (ML + R(1.0)) * (R(2.0) - ML);
    R PR = R(0.25) * (MR - R(1.0)) * (MR - R(1.0)) * (R(2.0) + MR);
    R DL = alphaL * (R(1.0) + betaL) - betaL * PL;
    R DR = alphaR * (R(1.0) + betaR) - betaR * PR;
    R mb = d_sqrt(R(0.5) * (ML * ML + MR * MR)) - R(1.0);
    R Mhalf = R(0.25) * betaL * betaR * ((EXACT && !kIsDual<R>) ? d_pow(mb, R(2.0)) : mb * mb);
    R MhalfL = Mhalf * (R(1.0) - ((pL - pR) / (pL + pR) + delta * (d_abs(pL - pR) / pL)));
    R MhalfR = Mhalf * (R(1.0) + ((pL - pR) / (pL + pR) - delta * (d_abs(pL - pR) / pR)));
    R CL = alphaL * (R(1.0) + betaL) * ML - betaL * MpL - MhalfL;
    R CR = alphaR * (R(1.0) + betaR) * MR - betaR * MmR + MhalfR;
    R ru_half = am * rL * CL + am * rR * CR;
    R ru2_half = am * rL * CL * uL + am * rR * CR * uR;
    R p_half = DL * pL + DR * pR;
    F[0] = ru_half;
    F[1] = ru2_half + p_half;
    F[2] = am * rL * CL * vL + am * rR * CR * vR;
    F[3] = DIM == 3 ? am * rL * CL * wL + am * rR * CR * wR : R(0.0);
    F[4] = am * rL * CL * HL + am * rR * CR * HR;
}

// Rusanov flux (flux_calculators/rusanov.cpp:9-53)
template <class R, int DIM>
IBISGB_HD void flux_rusanov(const FaceSide<R>& L, const FaceSide<R>& Rt, const Gas<R>& gm, R* F) {
    R rL = L.r, eL = gm.Cv * L.T, pL = L.p, uL = L.u, vL = L.v, wL = L.w;
    R ruL = rL * uL;
    R keL = DIM == 3 ? R(0.5) * (uL * uL + vL * vL + wL * wL) : R(0.5) * (uL * uL + vL * vL);
    R HL = eL + pL / rL + keL;
    R aL = gm.sound(L.T);
    R rR = Rt.r, eR = gm.Cv * Rt.T, pR = Rt.p, uR = Rt.u, vR = Rt.v, wR = Rt.w;
    R ruR = rR * uR;
    R keR = DIM == 3 ? R(0.5) * (uR * uR + vR * vR + wR * wR) : R(0.5) * (uR * uR + vR * vR);
    R HR = eR + pR / rR + keR;
    R aR = gm.sound(Rt.T);
    R S = d_max(d_abs(uL - aL), d_abs(uR - aR));
    S = d_max(S, d_abs(uL + aL));
    S = d_max(S, d_abs(uR + aR));
    F[0] = R(0.5) * (ruL + ruR) - R(0.5) * S * (rR - rL);
    F[1] = R(0.5) * (ruL * uL + pL + ruR * uR + pR) - R(0.5) * S * (rR * uR - rL * uL);
    F[2] = R(0.5) * (ruL * vL + ruR * vR) - R(0.5) * S * (rR * vR - rL * vL);
    F[3] = DIM == 3 ? R(0.5) * (ruL * wL + ruR * wR) - R(0.5) * S * (rR * wR - rL * wL) : R(0.0);
    F[4] = R(0.5) * (ruL * HL + ruR * HR) - R(0.5) * S * (rR * HR - rL * HL);
}

// Thermodynamic closure after reconstructing one of the four variable pairs
// (IdealGas::update_thermo_from_{rhop,rhoT,rhou,pT}, gas_model.h:77-116).
template <class R>
IBISGB_HD void thermo_close(int kind, const Gas<R>& gm, R& rho, R& p, R& T, R& e) {
    switch (kind) {
        case kRhoP: T = p / (rho * gm.R_); e = gm.Cv * T; break;
        case kRhoU:
            if constexpr (std::is_same<R, FF>::value) T = e * gm.iCv;
            else T = e / gm.Cv;
            p = rho * gm.R_ * T;
            break;
        case kRhoT: p = rho * gm.R_ * T; e = gm.Cv * T; break;
        default: rho = p / (gm.R_ * T); e = gm.Cv * T; break;  // p_T
    }
}

// Sutherland viscosity (transport_properties.h:28-42); EXACT selects pow as in
// the reference, otherwise T^1.5 = T*sqrt(T).
template <class R, bool EXACT>
IBISGB_HD R sutherland(R T, R mu0, R T0, R Ts) {
    R x = T / T0;
    R p15 = EXACT ? d_pow(x, R(3.0 / 2.0)) : x * d_sqrt(x);
    return mu0 * p15 * (T0 + Ts) / (T + Ts);
}

}  // namespace ibisgb
