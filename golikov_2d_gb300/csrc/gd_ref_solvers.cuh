// gd_ref_solvers.cuh -- the reference's Riemann solvers in its own arithmetic order, for the
// parity kernels.  Included only by translation units built with --fmad=false: with IEEE
// division and square root, and no contraction of multiply-adds, each function returns
// bit for bit what the reference's solver returns for the same face states.
//   hll_ref   HLL          kernel.cu:1485-1609
//   hllc_ref  Euler HLLC   kernel.cu:853-1165
//   hlld_ref  HLLD / HLLC-MHD  Gas_Dinamic.cu:964-1510
// The expressions follow the reference term by term because bit-identity requires it; the
// local-frame structure (MSide) is this library's own.
#pragma once

#include "gd_internal.cuh"

namespace gd {
namespace {

__device__ __forceinline__ double ref_min(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double ref_max(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ int sgn(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }

// the reference's my_min / my_max (kernel.cu:102-124), which HLL uses
__device__ __forceinline__ double my_min(double a, double b) { return a <= b ? a : b; }
__device__ __forceinline__ double my_max(double a, double b) { return a >= b ? a : b; }

// Euler HLL of kernel.cu:1485-1609, term by term in the reference's order: sound speeds 0
// for rho <= 0, speeds min/max of the normal velocities -+ the larger sound speed, the
// upwind flux when the fan does not straddle the face (Omega = 0, kernel.cu:11), else the
// HLL average.  out = {F_rho, F_E, F_mx, F_my}; returns krit rad / max(|D_L|, |D_R|).
__device__ double hll_ref(const double* L, const double* R, double n1, double n2, double rad,
                          const Params& P, double* out) {
    const double g = P.gamma;
    const double ro_L = L[0], p_L = L[1], v1_L = L[2], v2_L = L[3];
    const double ro_R = R[0], p_R = R[1], v1_R = R[2], v2_R = R[3];
    const double Vkv_L = v1_L * v1_L + v2_L * v2_L;
    const double Vkv_R = v1_R * v1_R + v2_R * v2_R;
    const double c_L = ro_L <= 0 ? 0.0 : sqrt(g * p_L / ro_L);
    const double c_R = ro_R <= 0 ? 0.0 : sqrt(g * p_R / ro_R);
    const double e_L = p_L / (g - 1.0) + ro_L * Vkv_L / 2.0;
    const double e_R = p_R / (g - 1.0) + ro_R * Vkv_R / 2.0;
    const double Vn_L = v1_L * n1 + v2_L * n2;
    const double Vn_R = v1_R * n1 + v2_R * n2;
    const double D_L = my_min(Vn_L, Vn_R) - my_max(c_L, c_R);
    const double D_R = my_max(Vn_L, Vn_R) + my_max(c_L, c_R);
    double t = 10000000;
    t = my_min(t, P.krit * rad / my_max(fabs(D_L), fabs(D_R)));
    const double fl_1 = (ro_L * v1_L) * n1 + (ro_L * v2_L) * n2;
    const double fl_2 = (ro_L * v1_L * v1_L + p_L) * n1 + (ro_L * v1_L * v2_L) * n2;
    const double fl_3 = (ro_L * v1_L * v2_L) * n1 + (ro_L * v2_L * v2_L + p_L) * n2;
    const double fl_5 = ((e_L + p_L) * v1_L) * n1 + ((e_L + p_L) * v2_L) * n2;
    if (D_L > 0.0) {
        out[0] = fl_1;
        out[1] = fl_5;
        out[2] = fl_2;
        out[3] = fl_3;
        return t;
    }
    const double fr_1 = (ro_R * v1_R) * n1 + (ro_R * v2_R) * n2;
    const double fr_2 = (ro_R * v1_R * v1_R + p_R) * n1 + (ro_R * v1_R * v2_R) * n2;
    const double fr_3 = (ro_R * v1_R * v2_R) * n1 + (ro_R * v2_R * v2_R + p_R) * n2;
    const double fr_5 = ((e_R + p_R) * v1_R) * n1 + ((e_R + p_R) * v2_R) * n2;
    if (D_R < 0.0) {
        out[0] = fr_1;
        out[1] = fr_5;
        out[2] = fr_2;
        out[3] = fr_3;
        return t;
    }
    const double dq1 = ro_R - ro_L;
    const double dq2 = ro_R * v1_R - ro_L * v1_L;
    const double dq3 = ro_R * v2_R - ro_L * v2_L;
    const double dq5 = e_R - e_L;
    out[0] = (D_R * fl_1 - D_L * fr_1 + D_L * D_R * dq1) / (D_R - D_L);
    out[2] = (D_R * fl_2 - D_L * fr_2 + D_L * D_R * dq2) / (D_R - D_L);
    out[3] = (D_R * fl_3 - D_L * fr_3 + D_L * D_R * dq3) / (D_R - D_L);
    out[1] = (D_R * fl_5 - D_L * fr_5 + D_L * D_R * dq5) / (D_R - D_L);
    return t;
}

// Euler HLLC of kernel.cu:853-1165 for B = 0: basis (n, e_z, (-n2, n1, 0)).
// L, R = {rho, p, vx, vy}; out = {F_rho, F_E, F_mx, F_my}; returns krit*rad/UU.
__device__ double hllc_ref(const double* L, const double* R, double n1, double n2, double rad,
                           const Params& P, double* out) {
    const double g = P.gamma, g1 = P.gamma - 1.0;
    const double m0 = -n2, m1 = n1;
    const double r1 = L[0], p1 = L[1], u1 = L[2], v1 = L[3];
    const double r2 = R[0], p2 = R[1], u2 = R[2], v2 = R[3];
    const double a1 = n1 * u1 + n2 * v1, t1 = m0 * u1 + m1 * v1;
    const double a2 = n1 * u2 + n2 * v2, t2 = m0 * u2 + m1 * v2;
    const double cL = sqrt(g * p1 / r1);
    const double qL = sqrt(cL * cL);
    const double cfL = (qL + qL) / 2.0;
    const double cR = sqrt(g * p2 / r2);
    const double qR = sqrt(cR * cR);
    const double cfR = (qR + qR) / 2.0;
    const double SL = ref_min(a1 - cfL, a2 - cfR);
    const double SR = ref_max(a1 + cfL, a2 + cfR);
    const double suR = SR - a2, suL = SL - a1;
    const double SM = (suR * r2 * a2 - p2 + p1 - suL * r1 * a1) / (suR * r2 - suL * r1);
    const double UU = ref_max(fabs(SL), fabs(SR));
    const double time = P.krit * rad / UU;
    const double e1 = p1 / g1 + r1 * ((u1 * u1 + v1 * v1) / 2.0);
    const double e2 = p2 / g1 + r2 * ((u2 * u2 + v2 * v2) / 2.0);
    const double FL0 = r1 * a1, FL1 = r1 * a1 * a1 + p1, FL3 = r1 * a1 * t1, FL4 = (e1 + p1) * a1;
    const double FR0 = r2 * a2, FR1 = r2 * a2 * a2 + p2, FR3 = r2 * a2 * t2, FR4 = (e2 + p2) * a2;
    const double suRm = suR / (SR - SM), suLm = suL / (SL - SM);
    const double rzR = r2 * suRm, rzL = r1 * suLm;
    const double ptzR = p2 + r2 * suR * (SM - a2);
    const double ptzL = p1 + r1 * suL * (SM - a1);
    const double ptz = (ptzR + ptzL) / 2.0;
    const double ezR = e2 * suRm + (ptz * SM - p2 * a2) / (SR - SM);
    const double ezL = e1 * suLm + (ptz * SM - p1 * a1) / (SL - SM);
    double fm = 0.0, fe = 0.0, q0 = 0.0, q2 = 0.0;
    if (SL > 0.0) {
        fm = FL0; fe = FL4; q0 = FL1; q2 = FL3;
    } else if (SL <= 0.0 && SM >= 0.0) {
        fm = FL0 + SL * (rzL - r1);
        fe = FL4 + SL * (ezL - e1);
        q0 = FL1 + SL * (SM * rzL - r1 * a1);
        q2 = FL3 + SL * (t1 * rzL - r1 * t1);
    } else if (SM <= 0.0 && SR >= 0.0) {
        fm = FR0 + SR * (rzR - r2);
        fe = FR4 + SR * (ezR - e2);
        q0 = FR1 + SR * (SM * rzR - r2 * a2);
        q2 = FR3 + SR * (t2 * rzR - r2 * t2);
    } else if (SR < 0.0) {
        fm = FR0; fe = FR4; q0 = FR1; q2 = FR3;
    }
    out[0] = fm;
    out[1] = fe;
    out[2] = n1 * q0 + m0 * q2;
    out[3] = n2 * q0 + m1 * q2;
    return time;
}

// One side of the MHD Riemann problem in the (n, t, m) frame, B in Heaviside-Lorentz units.
struct MSide {
    double r, p, vn, vt, vm, bn, bt, bm, bb, e, pt;
    double F[8], U[8];
};

__device__ __forceinline__ void mside(MSide& S, const double* Q, const double* n, const double* t,
                                      const double* m, double g) {
    const double bx = Q[5] / kSpi4, by = Q[6] / kSpi4, bz = Q[7] / kSpi4;
    S.r = Q[0];
    S.p = Q[1];
    S.vn = Q[2] * n[0] + Q[3] * n[1] + Q[4] * n[2];
    S.vt = Q[2] * t[0] + Q[3] * t[1] + Q[4] * t[2];
    S.vm = Q[2] * m[0] + Q[3] * m[1] + Q[4] * m[2];
    S.bn = bx * n[0] + by * n[1] + bz * n[2];
    S.bt = bx * t[0] + by * t[1] + bz * t[2];
    S.bm = bx * m[0] + by * m[1] + bz * m[2];
    S.bb = bx * bx + by * by + bz * bz;
    const double uu = (Q[2] * Q[2] + Q[3] * Q[3] + Q[4] * Q[4]) / 2.0;
    S.pt = S.p + S.bb / 2.0;
    S.e = S.p / (g - 1.0) + S.r * uu + S.bb / 2.0;
    S.F[0] = S.r * S.vn;
    S.F[1] = S.r * S.vn * S.vn + S.pt - S.bn * S.bn;
    S.F[2] = S.r * S.vn * S.vt - S.bn * S.bt;
    S.F[3] = S.r * S.vn * S.vm - S.bn * S.bm;
    S.F[4] = (S.e + S.pt) * S.vn - S.bn * (S.vn * S.bn + S.vt * S.bt + S.vm * S.bm);
    S.F[5] = 0.0;
    S.F[6] = S.vn * S.bt - S.vt * S.bn;
    S.F[7] = S.vn * S.bm - S.vm * S.bn;
    S.U[0] = S.r;
    S.U[1] = S.r * S.vn;
    S.U[2] = S.r * S.vt;
    S.U[3] = S.r * S.vm;
    S.U[4] = S.e;
    S.U[5] = S.bn;
    S.U[6] = S.bt;
    S.U[7] = S.bm;
}

// HLLD (method 3) / HLLC-MHD (method 2) of Gas_Dinamic.cu:964-1510.
// L, R = {rho, p, vx, vy, vz, Bx, By, Bz} (Gaussian B).
// P8 = {F_rho, F_mx, F_my, F_mz, F_Bx, F_By, F_Bz, F_E}; returns krit*rad/UU.
__device__ double hlld_ref(const double* L, const double* R, double n1, double n2, double rad,
                           int method, const Params& Pp, double* P8) {
    const double g = Pp.gamma;
    double n[3] = {n1, n2, 0.0}, t[3] = {0.0, 0.0, 0.0}, m[3] = {0.0, 0.0, 0.0};
    if (n1 > 0.1) {
        t[1] = 1.0; m[2] = 1.0;
    } else if (n2 > 0.1) {
        t[2] = 1.0; m[0] = 1.0;
    } else if (n1 < -0.1) {
        t[2] = -1.0; m[1] = -1.0;
    } else {
        t[0] = -1.0; m[2] = -1.0;
    }
    MSide A, B;
    mside(A, L, n, t, m, g);
    mside(B, R, n, t, m, g);
    const double cfL = sqrt((g * A.p + A.bb + sqrt((g * A.p + A.bb) * (g * A.p + A.bb) -
                                                    4.0 * g * A.p * (A.bn * A.bn))) /
                            (2.0 * A.r));
    const double cfR = sqrt((g * B.p + B.bb + sqrt((g * B.p + B.bb) * (g * B.p + B.bb) -
                                                    4.0 * g * B.p * (B.bn * B.bn))) /
                            (2.0 * B.r));
    const double SL = ref_min(A.vn, B.vn) - ref_max(cfL, cfR);
    const double SR = ref_max(A.vn, B.vn) + ref_max(cfL, cfR);
    const double suR = SR - B.vn, suL = SL - A.vn;
    const double SM = (suR * B.r * B.vn - suL * A.r * A.vn - B.pt + A.pt) / (suR * B.r - suL * A.r);
    const double PTT = (suR * B.r * A.pt - suL * A.r * B.pt + A.r * B.r * suR * suL * (B.vn - A.vn)) /
                       (suR * B.r - suL * A.r);
    const double UU = ref_max(fabs(SL), fabs(SR));
    const double time = Pp.krit * rad / UU;
    const double bn = (SR * B.U[5] - SL * A.U[5] + A.F[5] - B.F[5]) / (SR - SL);
    const double bt = (SR * B.U[6] - SL * A.U[6] + A.F[6] - B.F[6]) / (SR - SL);
    const double bm = (SR * B.U[7] - SL * A.U[7] + A.F[7] - B.F[7]) / (SR - SL);
    const double bbn = bn * bn;
    const double ro_LL = A.r * (SL - A.vn) / (SL - SM);
    const double ro_RR = B.r * (SR - B.vn) / (SR - SM);
    double PO[8];
    if (method == GD_METHOD_HLLC_MHD) {
        const double sbv1 = A.vn * A.bn + A.vt * A.bt + A.vm * A.bm;
        const double sbv2 = B.vn * B.bn + B.vt * B.bt + B.vm * B.bm;
        double UZ[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) UZ[k] = (SR * B.U[k] - SL * A.U[k] + A.F[k] - B.F[k]) / (SR - SL);
        const double suRm = suR / (SR - SM), suLm = suL / (SL - SM);
        const double ptzR = B.pt + B.r * suR * (SM - B.vn);
        const double ptzL = A.pt + A.r * suL * (SM - A.vn);
        const double ptz = (ptzR + ptzL) / 2.0;
        const double vS = UZ[2] / UZ[0], wS = UZ[3] / UZ[0];
        const double sbvz = (bn * UZ[1] + bt * UZ[2] + bm * UZ[3]) / UZ[0];
        const double ee2 = B.e * suRm + (ptz * SM - B.pt * B.vn + bn * (sbv2 - sbvz)) / (SR - SM);
        const double ee1 = A.e * suLm + (ptz * SM - A.pt * A.vn + bn * (sbv1 - sbvz)) / (SL - SM);
        const double ULL[8] = {ro_LL, ro_LL * SM, ro_LL * vS, ro_LL * wS, ee1, bn, bt, bm};
        const double URR[8] = {ro_RR, ro_RR * SM, ro_RR * vS, ro_RR * wS, ee2, bn, bt, bm};
        if (SL >= 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = A.F[k];
        } else if (SL < 0.0 && SM >= 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = A.F[k] + SL * ULL[k] - SL * A.U[k];
        } else if (SR > 0.0 && SM < 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = B.F[k] + SR * URR[k] - SR * B.U[k];
        } else if (SR <= 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = B.F[k];
        } else {
            for (int k = 0; k < 8; ++k) PO[k] = __longlong_as_double(0x7ff8000000000000LL);
        }
    } else {
        const double ttL = A.r * suL * (SL - SM) - bbn;
        const double ttR = B.r * suR * (SR - SM) - bbn;
        double vLL, wLL, vRR, wRR, btt1, bmm1, btt2, bmm2;
        if (fabs(ttL) >= 0.00001) {
            vLL = A.vt - bn * A.bt * (SM - A.vn) / ttL;
            wLL = A.vm - bn * A.bm * (SM - A.vn) / ttL;
            btt1 = A.bt * (A.r * suL * suL - bbn) / ttL;
            bmm1 = A.bm * (A.r * suL * suL - bbn) / ttL;
        } else {
            vLL = A.vt; wLL = A.vm; btt1 = 0.0; bmm1 = 0.0;
        }
        if (fabs(ttR) >= 0.00001) {
            vRR = B.vt - bn * B.bt * (SM - B.vn) / ttR;
            wRR = B.vm - bn * B.bm * (SM - B.vn) / ttR;
            btt2 = B.bt * (B.r * suR * suR - bbn) / ttR;
            bmm2 = B.bm * (B.r * suR * suR - bbn) / ttR;
        } else {
            vRR = B.vt; wRR = B.vm; btt2 = 0.0; bmm2 = 0.0;
        }
        const double eLL = (A.e * suL + PTT * SM - A.pt * A.vn +
                            bn * ((A.vn * A.bn + A.vt * A.bt + A.vm * A.bm) -
                                  (SM * bn + vLL * btt1 + wLL * bmm1))) / (SL - SM);
        const double eRR = (B.e * suR + PTT * SM - B.pt * B.vn +
                            bn * ((B.vn * B.bn + B.vt * B.bt + B.vm * B.bm) -
                                  (SM * bn + vRR * btt2 + wRR * bmm2))) / (SR - SM);
        const double sLL = sqrt(ro_LL), sRR = sqrt(ro_RR);
        double SLL = SM - fabs(bn) / sLL;
        double SRR = SM + fabs(bn) / sRR;
        double idbn;
        if (fabs(bn) > 0.000001) {
            idbn = 1.0 * sgn(bn);
        } else {
            idbn = 0.0;
            SLL = SM;
            SRR = SM;
        }
        const double vLLL = (sLL * vLL + sRR * vRR + idbn * (btt2 - btt1)) / (sLL + sRR);
        const double wLLL = (sLL * wLL + sRR * wRR + idbn * (bmm2 - bmm1)) / (sLL + sRR);
        const double bttt = (sLL * btt2 + sRR * btt1 + idbn * sLL * sRR * (vRR - vLL)) / (sLL + sRR);
        const double bmmm = (sLL * bmm2 + sRR * bmm1 + idbn * sLL * sRR * (wRR - wLL)) / (sLL + sRR);
        const double eLLL = eLL - idbn * sLL * ((SM * bn + vLL * btt1 + wLL * bmm1) -
                                                (SM * bn + vLLL * bttt + wLLL * bmmm));
        const double eRRR = eRR + idbn * sRR * ((SM * bn + vRR * btt2 + wRR * bmm2) -
                                                (SM * bn + vLLL * bttt + wLLL * bmmm));
        const double ULL[8] = {ro_LL, ro_LL * SM, ro_LL * vLL, ro_LL * wLL, eLL, bn, btt1, bmm1};
        const double URR[8] = {ro_RR, ro_RR * SM, ro_RR * vRR, ro_RR * wRR, eRR, bn, btt2, bmm2};
        const double ULLL[8] = {ro_LL, ro_LL * SM, ro_LL * vLLL, ro_LL * wLLL, eLLL, bn, bttt, bmmm};
        const double URRR[8] = {ro_RR, ro_RR * SM, ro_RR * vLLL, ro_RR * wLLL, eRRR, bn, bttt, bmmm};
        if (SL >= 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = A.F[k];
        } else if (SL < 0.0 && SLL >= 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = A.F[k] + SL * ULL[k] - SL * A.U[k];
        } else if (SLL <= 0.0 && SM >= 0.0) {
            for (int k = 0; k < 8; ++k)
                PO[k] = A.F[k] + SLL * ULLL[k] - (SLL - SL) * ULL[k] - SL * A.U[k];
        } else if (SM < 0.0 && SRR > 0.0) {
            for (int k = 0; k < 8; ++k)
                PO[k] = B.F[k] + SRR * URRR[k] - (SRR - SR) * URR[k] - SR * B.U[k];
        } else if (SR > 0.0 && SRR <= 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = B.F[k] + SR * URR[k] - SR * B.U[k];
        } else if (SR <= 0.0) {
            for (int k = 0; k < 8; ++k) PO[k] = B.F[k];
        } else {
            for (int k = 0; k < 8; ++k) PO[k] = __longlong_as_double(0x7ff8000000000000LL);
        }
    }
    const double SN = ref_max(fabs(SL), fabs(SR));
    PO[5] = -SN * (B.bn - A.bn);
    P8[0] = PO[0];
    P8[1] = n[0] * PO[1] + t[0] * PO[2] + m[0] * PO[3];
    P8[2] = n[1] * PO[1] + t[1] * PO[2] + m[1] * PO[3];
    P8[3] = n[2] * PO[1] + t[2] * PO[2] + m[2] * PO[3];
    P8[4] = kSpi4 * (n[0] * PO[5] + t[0] * PO[6] + m[0] * PO[7]);
    P8[5] = kSpi4 * (n[1] * PO[5] + t[1] * PO[6] + m[1] * PO[7]);
    P8[6] = kSpi4 * (n[2] * PO[5] + t[2] * PO[6] + m[2] * PO[7]);
    P8[7] = PO[4];
    return time;
}

}  // namespace
}  // namespace gd
