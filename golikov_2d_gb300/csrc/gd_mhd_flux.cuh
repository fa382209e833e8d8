// gd_mhd_flux.cuh -- the fast path's HLLD / HLLC-MHD flux in a face's local frame, field in
// Heaviside-Lorentz units (b = B / sqrt(4 pi)), templated on the scalar type (double, or
// Dual for the tangent).  Used by the fast MHD step (gd_fast_mhd.cu) and the fast
// MUSCL-Hancock step (gd_fast_hancock.cu).
//
// Reference semantics kept (Gas_Dinamic.cu:964-1510): wave speeds SL = min(u) - max(cf),
// SR = max(u) + max(cf), SM and p_T* (:1062-1075); HLL-averaged field; HLLD star and
// double-star states with the |tt| >= 1e-5 and |bn| > 1e-6 guards (:1306-1430) and the
// six-region selection (:1434-1484), or the HLLC-MHD states (:1137-1302); normal-field flux
// -max(|SL|,|SR|) (bn_R - bn_L) (:1488-1490).
#pragma once

#include "gd_dual.cuh"
#include "gd_internal.cuh"

namespace gd {
namespace {

template <class T>
__device__ __forceinline__ T cst(double x);
template <>
__device__ __forceinline__ double cst<double>(double x) { return x; }
template <>
__device__ __forceinline__ Dual cst<Dual>(double x) { return Dual{x, 0.0}; }

template <class T>
struct FluxM {
    T m, mn, mt, e, bn, bt, bz;  // mass, normal / tangential momentum, energy, field
};

// The per-side products (side, side_flux) form on the integer pipes (mulx, general case out
// of line); the HLLD core keeps its products on the FP64 unit: the MHD and Hancock tiles run
// two CTAs per SM, too few warps to cover the integer product's latency on that chain
// (measured slower).

// One side of the face in the local frame (un normal, ut in-plane tangential, uz = 0): what
// the wave speeds and the star states need from both sides.
template <class T>
struct Side {
    T r, p, un, ut, bn, bt, bz, bb, pT, cf;
};

template <class T>
__device__ __forceinline__ void side(Side<T>& S, T r, T p, T un, T ut, T bn, T bt, T bz,
                                     const Params& P) {
    S.r = r; S.p = p; S.un = un; S.ut = ut; S.bn = bn; S.bt = bt; S.bz = bz;
    const T bn2 = mulx<true>(bn, bn);
    S.bb = fma(bz, bz, fma(bt, bt, bn2));
    S.pT = fma(0.5, S.bb, p);
    const T gp = mulx<true>(P.gamma, p);
    const T a = gp + S.bb;
    T disc = fma(a, a, mulx<true>(mulx<true>(-4.0, gp), bn2));
    disc = le_zero(disc) ? cst<T>(0.0) : disc;
    const T X = mulx<true>(0.5, a + sqrt_fast_im<true>(disc));  // rho cf^2
    S.cf = sqrt_over_im<true>(X, r);                             // sqrt(X / r)
}

// a side's total energy and physical flux (mass, normal / tangential momentum, energy,
// tangential and z field); HLLD needs them for the upwind side only
template <class T>
struct SideF {
    T E, F0, F1, F2, F4, F6, F7;
};

template <class T>
__device__ __forceinline__ void side_flux(SideF<T>& F, const Side<T>& S, const Params& P) {
    F.E = fma(S.p, P.inv_gm1,
              mulx<true>(0.5, fma(S.r, fma(S.un, S.un, mulx<true>(S.ut, S.ut)), S.bb)));
    F.F0 = mulx<true>(S.r, S.un);
    F.F1 = fma(F.F0, S.un, fma(-S.bn, S.bn, S.pT));
    F.F2 = fma(F.F0, S.ut, -mulx<true>(S.bn, S.bt));
    F.F4 = fma(F.E + S.pT, S.un,
               -mulx<true>(S.bn, fma(S.ut, S.bt, mulx<true>(S.un, S.bn))));
    F.F6 = fma(S.un, S.bt, -mulx<true>(S.ut, S.bn));
    F.F7 = mulx<true>(S.un, S.bz);
}

// field-by-field select of one side (selects, no arithmetic)
template <class T>
__device__ __forceinline__ Side<T> pick(bool first, const Side<T>& A, const Side<T>& B) {
    Side<T> K;
    K.r = first ? A.r : B.r;
    K.p = first ? A.p : B.p;
    K.un = first ? A.un : B.un;
    K.ut = first ? A.ut : B.ut;
    K.bn = first ? A.bn : B.bn;
    K.bt = first ? A.bt : B.bt;
    K.bz = first ? A.bz : B.bz;
    K.bb = first ? A.bb : B.bb;
    K.pT = first ? A.pT : B.pT;
    K.cf = first ? A.cf : B.cf;
    return K;
}

__device__ __forceinline__ double sgn_select(double v, int idbn) {
    // idbn * v for idbn in {-1, 0, 1}, on the integer pipe (sign-bit flip, select)
    const double w = idbn < 0 ? from_bits(bits(v) ^ (long long)0x8000000000000000ULL) : v;
    return idbn == 0 ? 0.0 : w;
}
__device__ __forceinline__ Dual sgn_select(Dual v, int idbn) {
    return idbn == 0 ? Dual{0.0, 0.0} : (idbn < 0 ? -v : v);
}

// HLLD (method 3) or HLLC-MHD (method 2) flux.  UU = SL or SR, the one of larger magnitude
// (signed; the dt reduction takes |UU|).  The energy and the
// physical flux are formed for the sides that use them: both for HLLC-MHD (its HLL state of
// the fan), the upwind side K alone for HLLD, whose star energy is likewise K's alone.
template <class T>
__device__ __forceinline__ FluxM<T> hlld_local(const Side<T>& A, const Side<T>& B, int method,
                                               const Params& P, T& UU) {
    const T uminN = dmin(A.un, B.un);
    const T umaxN = dmax(A.un, B.un);
    const T cmax = max_nonneg(A.cf, B.cf);
    const T SL = uminN - cmax, SR = umaxN + cmax;
    const T suL = SL - A.un, suR = SR - B.un;
    const T mL = A.r * suL, mR = B.r * suR;
    const T iden = rcp_fast(mR - mL);
    const T SM = ((fma(mR, B.un, -mL * A.un) - B.pT) + A.pT) * iden;
    const T PTT = fma(mL * mR, B.un - A.un, fma(mR, A.pT, -mL * B.pT)) * iden;
    UU = max_nonneg(SL, SR);  // signed: the block reduction takes the magnitude
    const T iS = rcp_fast(SR - SL);
    const T bn = fma(SR, B.bn, -SL * A.bn) * iS;
    const T iL = rcp_fast(SL - SM), iR = rcp_fast(SR - SM);
    const T rLL = mL * iL, rRR = mR * iR;

    FluxM<T> F;
    if (method == GD_METHOD_HLLC_MHD) {
        SideF<T> FA, FB;
        side_flux(FA, A, P);
        side_flux(FB, B, P);
        const T bt = (fma(SR, B.bt, -SL * A.bt) + (FA.F6 - FB.F6)) * iS;
        const T bz = (fma(SR, B.bz, -SL * A.bz) + (FA.F7 - FB.F7)) * iS;
        const bool takeL = ge_zero(SL) || ge_zero(SM);
        const Side<T> K = pick(takeL, A, B);
        const T KE = takeL ? FA.E : FB.E;
        const T S = takeL ? SL : SR;
        const bool star = takeL ? lt_zero(SL) : gt_zero(SR);
        F.m = takeL ? FA.F0 : FB.F0;
        F.mn = takeL ? FA.F1 : FB.F1;
        F.mt = takeL ? FA.F2 : FB.F2;
        F.e = takeL ? FA.F4 : FB.F4;
        F.bt = takeL ? FA.F6 : FB.F6;
        F.bz = takeL ? FA.F7 : FB.F7;
        if (star) {
            // HLL state of the fan (Gas_Dinamic.cu:1145-1149); mom_z: U = 0, F = -bn bz
            const T UZ0 = (fma(SR, B.r, -SL * A.r) + (FA.F0 - FB.F0)) * iS;
            const T UZ1 = (fma(SR, B.r * B.un, -SL * A.r * A.un) + (FA.F1 - FB.F1)) * iS;
            const T UZ2 = (fma(SR, B.r * B.ut, -SL * A.r * A.ut) + (FA.F2 - FB.F2)) * iS;
            const T UZ3 = (B.bn * B.bz - A.bn * A.bz) * iS;
            const T iU0 = rcp_fast(UZ0);
            const T vS = UZ2 * iU0;
            const T ptz = 0.5 * (fma(mR, SM - B.un, B.pT) + fma(mL, SM - A.un, A.pT));
            const T sbvz = fma(bn, UZ1, fma(bt, UZ2, bz * UZ3)) * iU0;
            const T sbvK = fma(K.un, K.bn, K.ut * K.bt);
            const T iK = takeL ? iL : iR;
            const T suK = takeL ? suL : suR;
            const T eK = (fma(KE, suK, fma(ptz, SM, -K.pT * K.un)) + bn * (sbvK - sbvz)) * iK;
            const T rK = takeL ? rLL : rRR;
            F.m = fma(S, rK - K.r, F.m);
            F.mn = fma(S, fma(rK, SM, -K.r * K.un), F.mn);
            F.mt = fma(S, fma(rK, vS, -K.r * K.ut), F.mt);
            F.e = fma(S, eK - KE, F.e);
            F.bt = fma(S, bt - K.bt, F.bt);
            F.bz = fma(S, bz - K.bz, F.bz);
        }
    } else {
        const T bbn = bn * bn;
        // star states of both sides (Gas_Dinamic.cu:1306-1350)
        T vLL, wLL, btL, bzL, vRR, wRR, btR, bzR;
        {
            const T tt = fma(mL, SL - SM, -bbn);
            if (mag_ge(tt, kMag1em5)) {  // |tt| >= 1e-5
                const T it = rcp_fast(tt);
                const T c = bn * (SM - A.un) * it;
                const T d = fma(mL, suL, -bbn) * it;
                vLL = fma(-c, A.bt, A.ut);
                wLL = -c * A.bz;
                btL = A.bt * d;
                bzL = A.bz * d;
            } else {
                vLL = A.ut; wLL = cst<T>(0.0); btL = cst<T>(0.0); bzL = cst<T>(0.0);
            }
        }
        {
            const T tt = fma(mR, SR - SM, -bbn);
            if (mag_ge(tt, kMag1em5)) {
                const T it = rcp_fast(tt);
                const T c = bn * (SM - B.un) * it;
                const T d = fma(mR, suR, -bbn) * it;
                vRR = fma(-c, B.bt, B.ut);
                wRR = -c * B.bz;
                btR = B.bt * d;
                bzR = B.bz * d;
            } else {
                vRR = B.ut; wRR = cst<T>(0.0); btR = cst<T>(0.0); bzR = cst<T>(0.0);
            }
        }
        const T SMbn = SM * bn;
        T isLL, isRR, sLL, sRR;
        rsqrt_and_sqrt(rLL, isLL, sLL);
        rsqrt_and_sqrt(rRR, isRR, sRR);
        const bool bnz = mag_ge(bn, kMag1em6 + 1);  // |bn| > 1e-6
        const T abn = dabs(bn);
        const T SLL = bnz ? fma(-abn, isLL, SM) : SM;
        const T SRR = bnz ? fma(abn, isRR, SM) : SM;
        const int idbn = bnz ? (gt_zero(bn) ? 1 : -1) : 0;

        const bool takeL = ge_zero(SL) || ge_zero(SM);
        int level;
        if (takeL) level = ge_zero(SL) ? 0 : (ge_zero(SLL) ? 1 : 2);
        else level = gt_zero(SRR) ? 2 : (gt_zero(SR) ? 1 : 0);
        const Side<T> K = pick(takeL, A, B);
        SideF<T> KF;
        side_flux(KF, K, P);
        F.m = KF.F0; F.mn = KF.F1; F.mt = KF.F2; F.e = KF.F4; F.bt = KF.F6; F.bz = KF.F7;
        if (level >= 1) {
            const T S = takeL ? SL : SR;
            const T su = takeL ? suL : suR;
            const T iK = takeL ? iL : iR;
            const T rK = takeL ? rLL : rRR;
            const T vK = takeL ? vLL : vRR;
            const T wK = takeL ? wLL : wRR;
            const T btK = takeL ? btL : btR;
            const T bzK = takeL ? bzL : bzR;
            const T sbK = fma(wK, bzK, fma(vK, btK, SMbn));
            const T eK = (fma(KF.E, su, fma(PTT, SM, -K.pT * K.un)) +
                          bn * (fma(K.un, K.bn, K.ut * K.bt) - sbK)) * iK;
            F.m = fma(S, rK - K.r, F.m);
            F.mn = fma(S, fma(rK, SM, -K.r * K.un), F.mn);
            F.mt = fma(S, fma(rK, vK, -K.r * K.ut), F.mt);
            F.e = fma(S, eK - KF.E, F.e);
            F.bt = fma(S, btK - K.bt, F.bt);
            F.bz = fma(S, bzK - K.bz, F.bz);
            if (level == 2) {
                // double-star states (Gas_Dinamic.cu:1371-1430)
                const T is = rcp_fast(sLL + sRR);
                const T vL3 = (fma(sLL, vLL, sRR * vRR) + sgn_select(btR - btL, idbn)) * is;
                const T wL3 = (fma(sLL, wLL, sRR * wRR) + sgn_select(bzR - bzL, idbn)) * is;
                const T s2 = sgn_select(sLL * sRR, idbn);
                const T bt3 = fma(s2, vRR - vLL, fma(sLL, btR, sRR * btL)) * is;
                const T bz3 = fma(s2, wRR - wLL, fma(sLL, bzR, sRR * bzL)) * is;
                const T sb3 = fma(wL3, bz3, fma(vL3, bt3, SMbn));
                const T sK = takeL ? -sLL : sRR;
                const T e3 = fma(sgn_select(sK, idbn), sbK - sb3, eK);
                const T S2 = takeL ? SLL : SRR;
                F.mt = fma(S2, rK * (vL3 - vK), F.mt);
                F.e = fma(S2, e3 - eK, F.e);
                F.bt = fma(S2, bt3 - btK, F.bt);
                F.bz = fma(S2, bz3 - bzK, F.bz);
            }
        }
    }
    // normal-field flux replaced by the diffusive term (Gas_Dinamic.cu:1488-1490)
    F.bn = -dabs(UU) * (B.bn - A.bn);
    return F;
}

}  // namespace
}  // namespace gd
