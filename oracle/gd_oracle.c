/*
 * gd_oracle.c -- CPU restatement of the reference's explicit finite-volume step.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle.  Loaded by tests/, __graft_entry__.smoke() and
 * bench.py (CPU-baseline leg) as the oracle or the timed CPU baseline, never by the product.
 *
 * Each routine restates the reference routine named beside it, keeping the reference's
 * arithmetic order (compile with -ffp-contract=off) so that results are bit-identical; the
 * structure around the arithmetic is this project's own:
 *   - the reference's per-cell rotated-frame code is written as a local (normal, tangent)
 *     frame with explicit basis vectors;
 *   - the reference's per-cell boundary branches (kernel.cu:2226-2405) are written as two
 *     ghost layers per side, which yields exactly the same stencil values (derivation in
 *     stencil_value below);
 *   - Cartesian geometry is the reference's axisymmetric update with the 1/y source terms
 *     removed; periodic and transmissive ghosts are added for the benchmark problems.
 * Terms that the reference evaluates as exact zeros (B = 0 in the Euler solver, v_z = 0)
 * are dropped; dropping an exact zero from a sum changes at most the sign of a zero result.
 */
#include "gd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Header.h:18-21 */
#define GDO_CPI4 12.56637061435917295384
#define GDO_CPI8 25.13274122871834590768
#define GDO_SPI4 3.544907701811032

/* ------------------------------------------------------------------------------------- */
/* Reconstruction: kernel.cu:51-100                                                      */
/* ------------------------------------------------------------------------------------- */

static int sign_of(double v) { return v > 0 ? 1 : (v < 0 ? -1 : 0); }
/* std::min / std::max as the reference calls them (first argument wins ties). */
static double mn(double a, double b) { return (b < a) ? b : a; }
static double mx(double a, double b) { return (a < b) ? b : a; }

double gdo_minmod(double a, double b) {
    int s = sign_of(a) + sign_of(b);
    if (s == 0) return 0.0;
    return (s / 2.0) * mn(fabs(a), fabs(b));
}

double gdo_linear(double x1, double t1, double x2, double t2, double x3, double t3, double y) {
    double d = gdo_minmod((t1 - t2) / (x1 - x2), (t2 - t3) / (x2 - x3));
    return d * (y - x2) + t2;
}

void gdo_linear2(double x1, double t1, double x2, double t2, double x3, double t3, double y1,
                 double y2, double* A, double* B) {
    double d = gdo_minmod((t1 - t2) / (x1 - x2), (t2 - t3) / (x2 - x3));
    *A = d * (y1 - x2) + t2;
    *B = d * (y2 - x2) + t2;
}

/* ------------------------------------------------------------------------------------- */
/* Euler HLL: kernel.cu:1485-1609.  my_min / my_max as kernel.cu:102-124; Omega = 0          */
/* (kernel.cu:11).  out = {F_rho, F_E, F_mx, F_my}.                                         */
/* ------------------------------------------------------------------------------------- */

static double my_min(double a, double b) { return a <= b ? a : b; }
static double my_max(double a, double b) { return a >= b ? a : b; }

double gdo_hll(const double* L, const double* R, double n1, double n2, double rad,
               double gamma, double krit, double* out) {
    const double ro_L = L[0], p_L = L[1], v1_L = L[2], v2_L = L[3];
    const double ro_R = R[0], p_R = R[1], v1_R = R[2], v2_R = R[3];
    const double Vkv_L = v1_L * v1_L + v2_L * v2_L;
    const double Vkv_R = v1_R * v1_R + v2_R * v2_R;
    const double c_L = ro_L <= 0 ? 0.0 : sqrt(gamma * p_L / ro_L);
    const double c_R = ro_R <= 0 ? 0.0 : sqrt(gamma * p_R / ro_R);
    const double e_L = p_L / (gamma - 1.0) + ro_L * Vkv_L / 2.0;
    const double e_R = p_R / (gamma - 1.0) + ro_R * Vkv_R / 2.0;
    const double Vn_L = v1_L * n1 + v2_L * n2;
    const double Vn_R = v1_R * n1 + v2_R * n2;
    const double D_L = my_min(Vn_L, Vn_R) - my_max(c_L, c_R);
    const double D_R = my_max(Vn_L, Vn_R) + my_max(c_L, c_R);
    double t = 10000000;
    t = my_min(t, krit * rad / my_max(fabs(D_L), fabs(D_R)));
    const double fl_1 = (ro_L * v1_L) * n1 + (ro_L * v2_L) * n2;
    const double fl_2 = (ro_L * v1_L * v1_L + p_L) * n1 + (ro_L * v1_L * v2_L) * n2;
    const double fl_3 = (ro_L * v1_L * v2_L) * n1 + (ro_L * v2_L * v2_L + p_L) * n2;
    const double fl_5 = ((e_L + p_L) * v1_L) * n1 + ((e_L + p_L) * v2_L) * n2;
    if (D_L > 0.0) {
        out[0] = fl_1; out[1] = fl_5; out[2] = fl_2; out[3] = fl_3;
        return t;
    }
    const double fr_1 = (ro_R * v1_R) * n1 + (ro_R * v2_R) * n2;
    const double fr_2 = (ro_R * v1_R * v1_R + p_R) * n1 + (ro_R * v1_R * v2_R) * n2;
    const double fr_3 = (ro_R * v1_R * v2_R) * n1 + (ro_R * v2_R * v2_R + p_R) * n2;
    const double fr_5 = ((e_R + p_R) * v1_R) * n1 + ((e_R + p_R) * v2_R) * n2;
    if (D_R < 0.0) {
        out[0] = fr_1; out[1] = fr_5; out[2] = fr_2; out[3] = fr_3;
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

/* ------------------------------------------------------------------------------------- */
/* Euler HLLC: HLLC_Aleksashov, kernel.cu:853-1165, with B = 0 and v_z = 0.               */
/* ------------------------------------------------------------------------------------- */

double gdo_hllc(const double* L, const double* R, double n1, double n2, double rad,
                double gamma, double krit, double* out) {
    const double g1 = gamma - 1.0;
    /* Basis for B = 0 (the d <= eps branch, kernel.cu:915-945): normal n, first tangent
     * e_z, second tangent (-n2, n1, 0). */
    const double mvec0 = -n2, mvec1 = n1;
    const double r1 = L[0], p1 = L[1], u1 = L[2], v1 = L[3];
    const double r2 = R[0], p2 = R[1], u2 = R[2], v2 = R[3];

    /* local-frame velocities: normal and second tangent (the first tangent is 0) */
    const double vn1 = n1 * u1 + n2 * v1, vm1 = mvec0 * u1 + mvec1 * v1;
    const double vn2 = n1 * u2 + n2 * v2, vm2 = mvec0 * u2 + mvec1 * v2;

    /* fast speeds with zero field: (sqrt(c*c) + sqrt(c*c)) / 2 (kernel.cu:948-964) */
    const double cL = sqrt(gamma * p1 / r1);
    const double qL = sqrt(cL * cL);
    const double cfL = (qL + qL) / 2.0;
    const double cR = sqrt(gamma * p2 / r2);
    const double qR = sqrt(cR * cR);
    const double cfR = (qR + qR) / 2.0;

    /* Davis speeds and contact speed (kernel.cu:981-986) */
    const double SL = mn(vn1 - cfL, vn2 - cfR);
    const double SR = mx(vn1 + cfL, vn2 + cfR);
    const double suR = SR - vn2;
    const double suL = SL - vn1;
    const double SM = (suR * r2 * vn2 - p2 + p1 - suL * r1 * vn1) / (suR * r2 - suL * r1);

    const double UU = mx(fabs(SL), fabs(SR));
    const double t = krit * rad / UU;

    /* total energies with the global-frame kinetic term (kernel.cu:1020-1029) */
    const double e1 = p1 / g1 + r1 * ((u1 * u1 + v1 * v1) / 2.0);
    const double e2 = p2 / g1 + r2 * ((u2 * u2 + v2 * v2) / 2.0);

    /* physical fluxes in the local frame: mass, normal mom., tangent-2 mom., energy */
    const double FL0 = r1 * vn1, FL1 = r1 * vn1 * vn1 + p1, FL3 = r1 * vn1 * vm1,
                 FL4 = (e1 + p1) * vn1;
    const double FR0 = r2 * vn2, FR1 = r2 * vn2 * vn2 + p2, FR3 = r2 * vn2 * vm2,
                 FR4 = (e2 + p2) * vn2;

    /* star states (kernel.cu:1059-1117; the |UZ[5]| < eps branch holds for B = 0) */
    const double suRm = suR / (SR - SM);
    const double suLm = suL / (SL - SM);
    const double rzR = r2 * suRm;
    const double rzL = r1 * suLm;
    const double ptzR = p2 + r2 * suR * (SM - vn2);
    const double ptzL = p1 + r1 * suL * (SM - vn1);
    const double ptz = (ptzR + ptzL) / 2.0;
    const double ezR = e2 * suRm + (ptz * SM - p2 * vn2) / (SR - SM);
    const double ezL = e1 * suLm + (ptz * SM - p1 * vn1) / (SL - SM);

    double f_mass = 0.0, f_en = 0.0, q0 = 0.0, q2 = 0.0;
    if (SL > 0.0) {
        f_mass = FL0;
        f_en = FL4;
        q0 = FL1;
        q2 = FL3;
    } else if (SL <= 0.0 && SM >= 0.0) {
        f_mass = FL0 + SL * (rzL - r1);
        f_en = FL4 + SL * (ezL - e1);
        q0 = FL1 + SL * (SM * rzL - r1 * vn1);
        q2 = FL3 + SL * (vm1 * rzL - r1 * vm1);
    } else if (SM <= 0.0 && SR >= 0.0) {
        f_mass = FR0 + SR * (rzR - r2);
        f_en = FR4 + SR * (ezR - e2);
        q0 = FR1 + SR * (SM * rzR - r2 * vn2);
        q2 = FR3 + SR * (vm2 * rzR - r2 * vm2);
    } else if (SR < 0.0) {
        f_mass = FR0;
        f_en = FR4;
        q0 = FR1;
        q2 = FR3;
    }
    out[0] = f_mass;
    out[1] = f_en;
    /* back to global axes (kernel.cu:1161-1162) */
    out[2] = n1 * q0 + mvec0 * q2;
    out[3] = n2 * q0 + mvec1 * q2;
    return t;
}

/* ------------------------------------------------------------------------------------- */
/* MHD HLLD / HLLC-MHD: HLLDQ_Korolkov, Gas_Dinamic.cu:964-1510 (v_z = 0 at call sites).  */
/* ------------------------------------------------------------------------------------- */

typedef struct {
    double r, p, vn, vt, vm, bn, bt, bm, bb, e, pt;
    double F[8]; /* mass, mom n, mom t, mom m, energy, (Bn), Bt, Bm */
    double U[8];
} mhd_side;

static void mhd_side_fill(mhd_side* S, const double* Q, const double* n, const double* t,
                          const double* m, double gamma) {
    const double bx = Q[5] / GDO_SPI4, by = Q[6] / GDO_SPI4, bz = Q[7] / GDO_SPI4;
    S->r = Q[0];
    S->p = Q[1];
    S->vn = Q[2] * n[0] + Q[3] * n[1] + Q[4] * n[2];
    S->vt = Q[2] * t[0] + Q[3] * t[1] + Q[4] * t[2];
    S->vm = Q[2] * m[0] + Q[3] * m[1] + Q[4] * m[2];
    S->bn = bx * n[0] + by * n[1] + bz * n[2];
    S->bt = bx * t[0] + by * t[1] + bz * t[2];
    S->bm = bx * m[0] + by * m[1] + bz * m[2];
    S->bb = bx * bx + by * by + bz * bz;
    const double uu = (Q[2] * Q[2] + Q[3] * Q[3] + Q[4] * Q[4]) / 2.0;
    S->pt = S->p + S->bb / 2.0;
    S->e = S->p / (gamma - 1.0) + S->r * uu + S->bb / 2.0;
    S->F[0] = S->r * S->vn;
    S->F[1] = S->r * S->vn * S->vn + S->pt - S->bn * S->bn;
    S->F[2] = S->r * S->vn * S->vt - S->bn * S->bt;
    S->F[3] = S->r * S->vn * S->vm - S->bn * S->bm;
    S->F[4] = (S->e + S->pt) * S->vn - S->bn * (S->vn * S->bn + S->vt * S->bt + S->vm * S->bm);
    S->F[5] = 0.0;
    S->F[6] = S->vn * S->bt - S->vt * S->bn;
    S->F[7] = S->vn * S->bm - S->vm * S->bn;
    S->U[0] = S->r;
    S->U[1] = S->r * S->vn;
    S->U[2] = S->r * S->vt;
    S->U[3] = S->r * S->vm;
    S->U[4] = S->e;
    S->U[5] = S->bn;
    S->U[6] = S->bt;
    S->U[7] = S->bm;
}

/* fast magnetosonic speed, Gas_Dinamic.cu:1056-1059 */
static double fast_speed(double r, double p, double bb, double bn, double gamma) {
    return sqrt((gamma * p + bb + sqrt((gamma * p + bb) * (gamma * p + bb) -
                                       4.0 * gamma * p * (bn * bn))) /
                (2.0 * r));
}

double gdo_hlld(const double* L, const double* R, double n1, double n2, double n3, double rad,
                int method, double gamma, double krit, double* P) {
    /* tangent basis chosen by the sign of the normal (Gas_Dinamic.cu:986-1019) */
    double n[3] = {n1, n2, n3}, t[3] = {0.0, 0.0, 0.0}, m[3] = {0.0, 0.0, 0.0};
    if (n1 > 0.1) {
        t[1] = 1.0; m[2] = 1.0;
    } else if (n2 > 0.1) {
        t[2] = 1.0; m[0] = 1.0;
    } else if (n3 > 0.1) {
        t[0] = 1.0; m[1] = 1.0;
    } else if (n1 < -0.1) {
        t[2] = -1.0; m[1] = -1.0;
    } else if (n2 < -0.1) {
        t[0] = -1.0; m[2] = -1.0;
    } else if (n3 < -0.1) {
        t[0] = -1.0; m[1] = -1.0;
    }
    mhd_side A, B;
    mhd_side_fill(&A, L, n, t, m, gamma);
    mhd_side_fill(&B, R, n, t, m, gamma);

    const double cfL = fast_speed(A.r, A.p, A.bb, A.bn, gamma);
    const double cfR = fast_speed(B.r, B.p, B.bb, B.bn, gamma);

    /* wave speeds (Gas_Dinamic.cu:1062-1075) */
    const double SL = mn(A.vn, B.vn) - mx(cfL, cfR);
    const double SR = mx(A.vn, B.vn) + mx(cfL, cfR);
    const double suR = SR - B.vn;
    const double suL = SL - A.vn;
    const double SM = (suR * B.r * B.vn - suL * A.r * A.vn - B.pt + A.pt) / (suR * B.r - suL * A.r);
    const double PTT = (suR * B.r * A.pt - suL * A.r * B.pt + A.r * B.r * suR * suL * (B.vn - A.vn)) /
                       (suR * B.r - suL * A.r);
    const double UU = mx(fabs(SL), fabs(SR));
    const double time = krit * rad / UU;

    /* HLL average of the field (Gas_Dinamic.cu:1127-1130) */
    const double bn = (SR * B.U[5] - SL * A.U[5] + A.F[5] - B.F[5]) / (SR - SL);
    const double bt = (SR * B.U[6] - SL * A.U[6] + A.F[6] - B.F[6]) / (SR - SL);
    const double bm = (SR * B.U[7] - SL * A.U[7] + A.F[7] - B.F[7]) / (SR - SL);
    const double bbn = bn * bn;
    const double ro_LL = A.r * (SL - A.vn) / (SL - SM);
    const double ro_RR = B.r * (SR - B.vn) / (SR - SM);

    double PO[8];
    int k;
    if (method == 2) {
        /* HLLC-MHD, Gas_Dinamic.cu:1137-1302 */
        const double sbv1 = A.vn * A.bn + A.vt * A.bt + A.vm * A.bm;
        const double sbv2 = B.vn * B.bn + B.vt * B.bt + B.vm * B.bm;
        double UZ[5];
        for (k = 0; k < 5; ++k)
            UZ[k] = (SR * B.U[k] - SL * A.U[k] + A.F[k] - B.F[k]) / (SR - SL);
        const double suRm = suR / (SR - SM);
        const double suLm = suL / (SL - SM);
        const double ptzR = B.pt + B.r * suR * (SM - B.vn);
        const double ptzL = A.pt + A.r * suL * (SM - A.vn);
        const double ptz = (ptzR + ptzL) / 2.0;
        const double vS = UZ[2] / UZ[0];
        const double wS = UZ[3] / UZ[0];
        const double sbvz = (bn * UZ[1] + bt * UZ[2] + bm * UZ[3]) / UZ[0];
        const double ee2 = B.e * suRm + (ptz * SM - B.pt * B.vn + bn * (sbv2 - sbvz)) / (SR - SM);
        const double ee1 = A.e * suLm + (ptz * SM - A.pt * A.vn + bn * (sbv1 - sbvz)) / (SL - SM);
        const double ULL[8] = {ro_LL, ro_LL * SM, ro_LL * vS, ro_LL * wS, ee1, bn, bt, bm};
        const double URR[8] = {ro_RR, ro_RR * SM, ro_RR * vS, ro_RR * wS, ee2, bn, bt, bm};
        if (SL >= 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = A.F[k];
        } else if (SL < 0.0 && SM >= 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = A.F[k] + SL * ULL[k] - SL * A.U[k];
        } else if (SR > 0.0 && SM < 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = B.F[k] + SR * URR[k] - SR * B.U[k];
        } else if (SR <= 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = B.F[k];
        } else {
            for (k = 0; k < 8; ++k) PO[k] = NAN;
        }
    } else {
        /* HLLD, Gas_Dinamic.cu:1303-1490 */
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
                                  (SM * bn + vLL * btt1 + wLL * bmm1))) /
                           (SL - SM);
        const double eRR = (B.e * suR + PTT * SM - B.pt * B.vn +
                            bn * ((B.vn * B.bn + B.vt * B.bt + B.vm * B.bm) -
                                  (SM * bn + vRR * btt2 + wRR * bmm2))) /
                           (SR - SM);
        const double sqrtroLL = sqrt(ro_LL);
        const double sqrtroRR = sqrt(ro_RR);
        double SLL = SM - fabs(bn) / sqrtroLL;
        double SRR = SM + fabs(bn) / sqrtroRR;
        double idbn;
        if (fabs(bn) > 0.000001) {
            idbn = 1.0 * sign_of(bn);
        } else {
            idbn = 0.0;
            SLL = SM;
            SRR = SM;
        }
        const double vLLL = (sqrtroLL * vLL + sqrtroRR * vRR + idbn * (btt2 - btt1)) /
                            (sqrtroLL + sqrtroRR);
        const double wLLL = (sqrtroLL * wLL + sqrtroRR * wRR + idbn * (bmm2 - bmm1)) /
                            (sqrtroLL + sqrtroRR);
        const double bttt = (sqrtroLL * btt2 + sqrtroRR * btt1 +
                             idbn * sqrtroLL * sqrtroRR * (vRR - vLL)) /
                            (sqrtroLL + sqrtroRR);
        const double bmmm = (sqrtroLL * bmm2 + sqrtroRR * bmm1 +
                             idbn * sqrtroLL * sqrtroRR * (wRR - wLL)) /
                            (sqrtroLL + sqrtroRR);
        const double eLLL = eLL - idbn * sqrtroLL *
                                      ((SM * bn + vLL * btt1 + wLL * bmm1) -
                                       (SM * bn + vLLL * bttt + wLLL * bmmm));
        const double eRRR = eRR + idbn * sqrtroRR *
                                      ((SM * bn + vRR * btt2 + wRR * bmm2) -
                                       (SM * bn + vLLL * bttt + wLLL * bmmm));
        const double ULL[8] = {ro_LL, ro_LL * SM, ro_LL * vLL, ro_LL * wLL, eLL, bn, btt1, bmm1};
        const double URR[8] = {ro_RR, ro_RR * SM, ro_RR * vRR, ro_RR * wRR, eRR, bn, btt2, bmm2};
        const double ULLL[8] = {ro_LL, ro_LL * SM, ro_LL * vLLL, ro_LL * wLLL, eLLL, bn, bttt, bmmm};
        const double URRR[8] = {ro_RR, ro_RR * SM, ro_RR * vLLL, ro_RR * wLLL, eRRR, bn, bttt, bmmm};
        if (SL >= 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = A.F[k];
        } else if (SL < 0.0 && SLL >= 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = A.F[k] + SL * ULL[k] - SL * A.U[k];
        } else if (SLL <= 0.0 && SM >= 0.0) {
            for (k = 0; k < 8; ++k)
                PO[k] = A.F[k] + SLL * ULLL[k] - (SLL - SL) * ULL[k] - SL * A.U[k];
        } else if (SM < 0.0 && SRR > 0.0) {
            for (k = 0; k < 8; ++k)
                PO[k] = B.F[k] + SRR * URRR[k] - (SRR - SR) * URR[k] - SR * B.U[k];
        } else if (SR > 0.0 && SRR <= 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = B.F[k] + SR * URR[k] - SR * B.U[k];
        } else if (SR <= 0.0) {
            for (k = 0; k < 8; ++k) PO[k] = B.F[k];
        } else {
            for (k = 0; k < 8; ++k) PO[k] = NAN;
        }
    }

    /* normal-field flux replaced by the diffusive term (Gas_Dinamic.cu:1488-1490) */
    const double SN = mx(fabs(SL), fabs(SR));
    PO[5] = -SN * (B.bn - A.bn);

    /* back to global axes, field flux to Gaussian units, energy moved last (:1492-1506) */
    P[0] = PO[0];
    P[1] = n[0] * PO[1] + t[0] * PO[2] + m[0] * PO[3];
    P[2] = n[1] * PO[1] + t[1] * PO[2] + m[1] * PO[3];
    P[3] = n[2] * PO[1] + t[2] * PO[2] + m[2] * PO[3];
    P[4] = GDO_SPI4 * (n[0] * PO[5] + t[0] * PO[6] + m[0] * PO[7]);
    P[5] = GDO_SPI4 * (n[1] * PO[5] + t[1] * PO[6] + m[1] * PO[7]);
    P[6] = GDO_SPI4 * (n[2] * PO[5] + t[2] * PO[6] + m[2] * PO[7]);
    P[7] = PO[4];
    return time;
}

/* ------------------------------------------------------------------------------------- */
/* Step: the per-cell structure of Kernel_TVD (kernel.cu:2198-2661), add2 (:1877-2196),   */
/* Ker_Dekard (:1736-1875) and the reconstruction of Kernel_TVD_old (:3436-3544).         */
/* ------------------------------------------------------------------------------------- */

typedef struct {
    double r, p, u, v, bx, by, bz;
} prim;

static prim load_cell(const gdo_config* c, const double* s, const double* u, const double* b,
                      int n, int m) {
    const long k = (long)m * c->N + n;
    prim q;
    q.r = s[2 * k];
    q.p = s[2 * k + 1];
    q.u = u[2 * k];
    q.v = u[2 * k + 1];
    if (b) {
        q.bx = b[3 * k];
        q.by = b[3 * k + 1];
        q.bz = b[3 * k + 2];
    } else {
        q.bx = q.by = q.bz = 0.0;
    }
    return q;
}

/* Ghost value `depth` (1 or 2) cells beyond the edge cell `edge` of a row/column.
 * `inner` is the interior cell at the same distance from the edge (depth 1 -> edge cell,
 * depth 2 -> its neighbour); the reference's mirror conditions reflect that cell:
 *   left  n==0: s_4 = mirror(s_1), n==0: s41 = mirror(s_2), n==1: s41 = mirror(s_4)
 *   bottom m==0: s_3 = axis(s_1), m==0: s31 = axis(s_5), m==1: s31 = axis(s_3)
 * while the outflow and ambient conditions give the same value at both depths:
 *   right n==N-1: s_2 = clamp(s_1); n>=N-2: s21 = clamp(s_2)
 *   top m==M-1: s_5 = ambient; m>=M-2: s51 = ambient. */
static prim ghost(const gdo_config* c, int bc, prim edge, prim inner) {
    prim g;
    switch (bc) {
        case GDO_BC_MIRROR_X:
            g = inner;
            g.u = -inner.u;
            g.bx = -inner.bx;
            g.by = -inner.by;
            return g;
        case GDO_BC_AXIS:
            g = inner;
            g.v = -inner.v;
            g.bz = -inner.bz;
            return g;
        case GDO_BC_AMBIENT:
        case GDO_BC_AMBIENT_KEEPB:
            g.r = 1.0;
            g.p = 1.0 / c->gamma;
            g.u = 0.0;
            g.v = 0.0;
            if (bc == GDO_BC_AMBIENT_KEEPB) {
                g.bx = edge.bx; g.by = edge.by; g.bz = edge.bz;
            } else {
                g.bx = 0.0; g.by = 0.0; g.bz = 0.0;
            }
            return g;
        case GDO_BC_OUTFLOW:
            g = edge;
            if (g.u < 0) g.u = 0.01;
            return g;
        case GDO_BC_TRANSMISSIVE:
        default:
            return edge;
    }
}

/* Value of the cell at (n, m) where exactly one of n, m may lie outside the grid by <= 2. */
static prim stencil_value(const gdo_config* c, const double* s, const double* u, const double* b,
                          int n, int m) {
    const int N = c->N, M = c->M;
    if (n < 0 || n >= N) {
        const int left = n < 0;
        const int bc = left ? c->bc[0] : c->bc[1];
        const int depth = left ? -n : n - N + 1;
        if (bc == GDO_BC_PERIODIC) return load_cell(c, s, u, b, (n + N) % N, m);
        const int e = left ? 0 : N - 1;
        const int in = left ? depth - 1 : N - depth;
        return ghost(c, bc, load_cell(c, s, u, b, e, m), load_cell(c, s, u, b, in, m));
    }
    if (m < 0 || m >= M) {
        const int bottom = m < 0;
        const int bc = bottom ? c->bc[2] : c->bc[3];
        const int depth = bottom ? -m : m - M + 1;
        if (bc == GDO_BC_PERIODIC) return load_cell(c, s, u, b, n, (m + M) % M);
        const int e = bottom ? 0 : M - 1;
        const int in = bottom ? depth - 1 : M - depth;
        return ghost(c, bc, load_cell(c, s, u, b, n, e), load_cell(c, s, u, b, n, in));
    }
    return load_cell(c, s, u, b, n, m);
}

/* field accessors so the 7 reconstructions can loop */
static double* fld(prim* q, int f) {
    switch (f) {
        case 0: return &q->r;
        case 1: return &q->p;
        case 2: return &q->u;
        case 3: return &q->v;
        case 4: return &q->bx;
        case 5: return &q->by;
        default: return &q->bz;
    }
}

typedef struct {
    prim c1, own[4], nbr[4]; /* own face states 12,13,14,15 and neighbour face states 21,31,41,51 */
    prim s2, s3, s4, s5;     /* first neighbours E, S, W, N (cell values, used by Pdiv) */
} cell_faces;

/* Face states of one cell, kernel.cu:2226-2548 (order 2) or the raw neighbours (order 1). */
static void build_faces(const gdo_config* c, const double* s, const double* u, const double* b,
                        int n, int m, double x, double y, cell_faces* F) {
    const double dx = c->dx, dy = c->dy;
    const int nf = c->physics == GDO_MHD ? 7 : 4;
    prim q1 = load_cell(c, s, u, b, n, m);
    prim q2 = stencil_value(c, s, u, b, n + 1, m);
    prim q4 = stencil_value(c, s, u, b, n - 1, m);
    prim q3 = stencil_value(c, s, u, b, n, m - 1);
    prim q5 = stencil_value(c, s, u, b, n, m + 1);
    F->c1 = q1;
    F->s2 = q2; F->s3 = q3; F->s4 = q4; F->s5 = q5;
    if (c->order == 1) {
        F->own[0] = F->own[1] = F->own[2] = F->own[3] = q1;
        F->nbr[0] = q2; F->nbr[1] = q3; F->nbr[2] = q4; F->nbr[3] = q5;
        return;
    }
    prim q21 = stencil_value(c, s, u, b, n + 2, m);
    prim q41 = stencil_value(c, s, u, b, n - 2, m);
    prim q31 = stencil_value(c, s, u, b, n, m - 2);
    prim q51 = stencil_value(c, s, u, b, n, m + 2);
    prim f12 = q1, f13 = q1, f14 = q1, f15 = q1, f21 = q2, f31 = q3, f41 = q4, f51 = q5;
    for (int f = 0; f < nf; ++f) {
        const int positive = (f == 0 || f == 1); /* rho and p fall back when <= 0 */
        const double v1 = *fld(&q1, f), v2 = *fld(&q2, f), v3 = *fld(&q3, f), v4 = *fld(&q4, f),
                     v5 = *fld(&q5, f);
        double A, B;
        /* own x faces: linear2 over (x-dx, x, x+dx) evaluated at x -/+ dx/2 (:2407-2458) */
        gdo_linear2(x - dx, v4, x, v1, x + dx, v2, x - dx / 2.0, x + dx / 2.0, &A, &B);
        *fld(&f12, f) = (positive && B <= 0) ? v1 : B;
        *fld(&f14, f) = (positive && A <= 0) ? v1 : A;
        /* own y faces (:2461-2508) */
        gdo_linear2(y - dy, v3, y, v1, y + dy, v5, y - dy / 2.0, y + dy / 2.0, &A, &B);
        *fld(&f15, f) = (positive && B <= 0) ? v1 : B;
        *fld(&f13, f) = (positive && A <= 0) ? v1 : A;
        /* neighbours' facing states with their own stencils (:2510-2548) */
        double w;
        w = gdo_linear(x, v1, x + dx, v2, x + 2.0 * dx, *fld(&q21, f), x + dx / 2.0);
        *fld(&f21, f) = (positive && w <= 0) ? v2 : w;
        w = gdo_linear(x, v1, x - dx, v4, x - 2.0 * dx, *fld(&q41, f), x - dx / 2.0);
        *fld(&f41, f) = (positive && w <= 0) ? v4 : w;
        w = gdo_linear(y, v1, y - dy, v3, y - 2.0 * dy, *fld(&q31, f), y - dy / 2.0);
        *fld(&f31, f) = (positive && w <= 0) ? v3 : w;
        w = gdo_linear(y, v1, y + dy, v5, y + 2.0 * dy, *fld(&q51, f), y + dy / 2.0);
        *fld(&f51, f) = (positive && w <= 0) ? v5 : w;
    }
    F->own[0] = f12; F->own[1] = f13; F->own[2] = f14; F->own[3] = f15;
    F->nbr[0] = f21; F->nbr[1] = f31; F->nbr[2] = f41; F->nbr[3] = f51;
}

/* outward normals of faces 12 (E), 13 (S), 14 (W), 15 (N) */
static const double FACE_N1[4] = {1.0, 0.0, -1.0, 0.0};
static const double FACE_N2[4] = {0.0, -1.0, 0.0, 1.0};

/* Euler cell: fluxes as Kernel_TVD_old :3560-3586, update as Ker_Dekard :1849-1874
 * (Cartesian) or Kernel_TVD_old :3636-3665 (axisymmetric).  Returns the cell's dt. */
static double euler_cell(const gdo_config* c, const cell_faces* F, double y, double T_do,
                         double* out) {
    const double dx = c->dx, dy = c->dy, gamma = c->gamma;
    double tmin = 1000;
    double Ps[4][2], Pu[4][2];
    for (int f = 0; f < 4; ++f) {
        const prim* a = &F->own[f];
        const prim* z = &F->nbr[f];
        const double L[4] = {a->r, a->p, a->u, a->v};
        const double R[4] = {z->r, z->p, z->u, z->v};
        const double rad = (f == 0 || f == 2) ? dy : dx; /* kernel.cu:3562-3586 */
        double o[4];
        /* method 0 = HLL everywhere (Ker_Dekard / Kernel_TVD_old, kernel.cu:1796, 3547) */
        tmin = mn(tmin, c->method == 0
                            ? gdo_hll(L, R, FACE_N1[f], FACE_N2[f], rad, gamma, c->krit, o)
                            : gdo_hllc(L, R, FACE_N1[f], FACE_N2[f], rad, gamma, c->krit, o));
        Ps[f][0] = o[0]; Ps[f][1] = o[1]; Pu[f][0] = o[2]; Pu[f][1] = o[3];
    }
    const double PSx = Ps[0][0] * dy + Ps[1][0] * dx + Ps[2][0] * dy + Ps[3][0] * dx;
    const double PSy = Ps[0][1] * dy + Ps[1][1] * dx + Ps[2][1] * dy + Ps[3][1] * dx;
    const double PUx = Pu[0][0] * dy + Pu[1][0] * dx + Pu[2][0] * dy + Pu[3][0] * dx;
    const double PUy = Pu[0][1] * dy + Pu[1][1] * dx + Pu[2][1] * dy + Pu[3][1] * dx;
    const double dV = dx * dy;
    const prim* q = &F->c1;
    double r2, ux2, uy2, p2;
    if (c->geometry == GDO_AXISYM) {
        r2 = q->r - (T_do / dV) * PSx - T_do * q->r * q->v / y;
        if (r2 <= 0) r2 = 0.0001;
        ux2 = (q->r * q->u - (T_do / dV) * PUx - T_do * q->r * q->v * q->u / y) / r2;
        uy2 = (q->r * q->v - (T_do / dV) * PUy - T_do * q->r * q->v * q->v / y) / r2;
        p2 = (((q->p / (gamma - 1) + q->r * (q->u * q->u + q->v * q->v) * 0.5) -
               (T_do / dV) * PSy -
               T_do * q->v * (gamma * q->p / (gamma - 1) + q->r * (q->u * q->u + q->v * q->v) * 0.5) /
                   y) -
              0.5 * r2 * (ux2 * ux2 + uy2 * uy2)) *
             (gamma - 1);
    } else {
        r2 = q->r - (T_do / dV) * PSx;
        if (r2 <= 0) r2 = 0.0001;
        ux2 = (q->r * q->u - (T_do / dV) * PUx) / r2;
        uy2 = (q->r * q->v - (T_do / dV) * PUy) / r2;
        p2 = (((q->p / (gamma - 1) + q->r * (q->u * q->u + q->v * q->v) * 0.5) - (T_do / dV) * PSy) -
              0.5 * r2 * (ux2 * ux2 + uy2 * uy2)) *
             (gamma - 1);
    }
    if (p2 <= 0) p2 = 0.000001;
    out[0] = r2; out[1] = p2; out[2] = ux2; out[3] = uy2;
    return tmin;
}

/* MHD cell: Kernel_TVD :2550-2660 (add2 :2064-2192 has the same flux and update). */
static double mhd_cell(const gdo_config* c, const cell_faces* F, double y, double T_do,
                       double* out) {
    const double dx = c->dx, dy = c->dy, gamma = c->gamma;
    const int axi = c->geometry == GDO_AXISYM;
    double tmin = 1000;
    double PSx = 0.0, PSy = 0.0, PUx = 0.0, PUy = 0.0, PBx = 0.0, PBy = 0.0, PBz = 0.0;
    double Pdiv = 0.0;
    const prim* q = &F->c1;
    for (int f = 0; f < 4; ++f) {
        const prim* a = &F->own[f];
        const prim* z = &F->nbr[f];
        const double L[8] = {a->r, a->p, a->u, a->v, 0.0, a->bx, a->by, a->bz};
        const double R[8] = {z->r, z->p, z->u, z->v, 0.0, z->bx, z->by, z->bz};
        const int xface = (f == 0 || f == 2);
        const double rad = xface ? dx : dy;  /* kernel.cu:2559-2604 */
        const double len = xface ? dy : dx;  /* face length */
        double P[8];
        tmin = mn(tmin, gdo_hlld(L, R, FACE_N1[f], FACE_N2[f], 0.0, rad, c->method, gamma, c->krit, P));
        PSx = PSx + P[0] * len;
        PSy = PSy + P[7] * len;
        PUx = PUx + P[1] * len;
        PUy = PUy + P[2] * len;
        PBx = PBx + P[4] * len;
        PBy = PBy + P[5] * len;
        PBz = PBz + P[6] * len;
        /* Powell divergence from cell-centred B (kernel.cu:2568, 2580, 2592, 2604) */
        switch (f) {
            case 0: Pdiv = Pdiv + dy * (q->bx + F->s2.bx) / 2.0; break;
            case 1: Pdiv = Pdiv - dx * (q->by + F->s3.by) / 2.0; break;
            case 2: Pdiv = Pdiv - dy * (q->bx + F->s4.bx) / 2.0; break;
            default: Pdiv = Pdiv + dx * (q->by + F->s5.by) / 2.0; break;
        }
    }
    const double dV = dx * dy;
    if (axi) Pdiv = Pdiv + dV * q->by / y; /* kernel.cu:2615 */

    /* update, kernel.cu:2619-2660 (Cartesian: the 1/y source terms removed) */
    const double kvu = q->u * q->u + q->v * q->v + 0.0 * 0.0;
    const double kvb = q->bx * q->bx + q->by * q->by + q->bz * q->bz;
    const double U8 = q->p / (gamma - 1.0) + 0.5 * q->r * kvu + kvb / 25.13274122871834590768;
    const double skk = q->u * q->bx + q->v * q->by + 0.0 * q->bz;
    double r2 = q->r - T_do * PSx / dV;
    if (axi) r2 = r2 - T_do * q->r * q->v / y;
    if (r2 <= 0) r2 = q->r;
    double ux2 = q->r * q->u - T_do * (PUx + (q->bx / GDO_CPI4) * Pdiv) / dV;
    double uy2 = q->r * q->v - T_do * (PUy + (q->by / GDO_CPI4) * Pdiv) / dV;
    double bx2 = q->bx - T_do * (PBx + q->u * Pdiv) / dV;
    if (axi) {
        ux2 = ux2 - T_do * (q->r * q->u * q->v - q->bx * q->by / GDO_CPI4) / y;
        uy2 = uy2 - T_do * (q->r * q->v * q->v + (q->bz * q->bz - q->by * q->by) / GDO_CPI4) / y;
        bx2 = bx2 - T_do * (q->v * q->bx - q->by * q->u) / y;
    }
    ux2 = ux2 / r2;
    uy2 = uy2 / r2;
    const double by2 = q->by - T_do * (PBy + q->v * Pdiv) / dV;
    const double bz2 = q->bz - T_do * (PBz) / dV;
    double e = U8 - T_do * (PSy + (skk / GDO_CPI4) * Pdiv) / dV;
    if (axi) e = e - T_do * (((U8 + q->p + kvb / GDO_CPI8) * q->v - q->by * skk / GDO_CPI4) / y);
    double p2 = (e - 0.5 * r2 * (ux2 * ux2 + uy2 * uy2 + 0.0 * 0.0) -
                 (bx2 * bx2 + by2 * by2 + bz2 * bz2) / GDO_CPI8) *
                (gamma - 1.0);
    if (p2 <= 0) p2 = 0.000001;
    out[0] = r2; out[1] = p2; out[2] = ux2; out[3] = uy2;
    out[4] = bx2; out[5] = by2; out[6] = bz2;
    return tmin;
}

/* ------------------------------------------------------------------------------------- */
/* MUSCL-Hancock step of Kernel_GKR (kernel.cu:2663-3284), term by term.                   */
/* ------------------------------------------------------------------------------------- */

#define GK_CPI4 12.56637061435917295384 /* Header.h:20-22 */
#define GK_CPI8 25.13274122871834590768
#define GK_SPI4 (3.544907701811032)

typedef struct {
    double sx, sy, ux, uy, bx, by, bz; /* s = (rho, p), u = (vx, vy), b = (Bx, By, Bz) */
} gk_cell;

static gk_cell gk_load(const double* s, const double* u, const double* b, long k) {
    gk_cell c = {s[2 * k], s[2 * k + 1], u[2 * k], u[2 * k + 1], b[3 * k], b[3 * k + 1],
                 b[3 * k + 2]};
    return c;
}

/* U8 (Header.h:16): p/(ggg-1) + 0.5 rho |v|^2 + |B|^2 / (8 pi) */
static double gk_u8(double g, double ro, double p, double u, double v, double w, double bx,
                    double by, double bz) {
    return p / (g - 1.0) + 0.5 * ro * ((u * u + v * v) + w * w) +
           ((bx * bx + by * by) + bz * bz) / 25.13274122871834590768;
}
static double gk_kvv(double x, double y, double z) { return (x * x + y * y) + z * z; }
static double gk_skk(double u, double v, double w, double bx, double by, double bz) {
    return u * bx + v * by + w * bz;
}

/* POTOK_Korolkov (Gas_Dinamic.cu:70-180): the physical MHD flux through a face with normal
 * n = (n1, n2, n3), rotated back to (x, y, z); P = {F_rho, F_mx, F_my, F_mz, F_Bx, F_By,
 * F_Bz, F_E} with the field fluxes in Gaussian units. */
static void gk_potok(double g, double ro_L, double Q_L, double p_L, double v1_L, double v2_L,
                     double v3_L, double Bx_L, double By_L, double Bz_L, double* P, double n1,
                     double n2, double n3) {
    const double bx_L = Bx_L / GK_SPI4, by_L = By_L / GK_SPI4, bz_L = Bz_L / GK_SPI4;
    double t1 = 0.0, t2 = 0.0, t3 = 0.0, m1 = 0.0, m2 = 0.0, m3 = 0.0;
    if (n1 > 0.1) { t2 = 1.0; m3 = 1.0; }
    else if (n2 > 0.1) { t3 = 1.0; m1 = 1.0; }
    else if (n3 > 0.1) { t1 = 1.0; m2 = 1.0; }
    else if (n1 < -0.1) { t3 = -1.0; m2 = -1.0; }
    else if (n2 < -0.1) { t1 = -1.0; m3 = -1.0; }
    else if (n3 < -0.1) { t1 = -1.0; m2 = -1.0; }
    const double u1 = v1_L * n1 + v2_L * n2 + v3_L * n3;
    const double v1 = v1_L * t1 + v2_L * t2 + v3_L * t3;
    const double w1 = v1_L * m1 + v2_L * m2 + v3_L * m3;
    const double bn1 = bx_L * n1 + by_L * n2 + bz_L * n3;
    const double bt1 = bx_L * t1 + by_L * t2 + bz_L * t3;
    const double bm1 = bx_L * m1 + by_L * m2 + bz_L * m3;
    const double bb_L = bx_L * bx_L + by_L * by_L + bz_L * bz_L;
    const double uu_L = (v1_L * v1_L + v2_L * v2_L + v3_L * v3_L) / 2.0;
    const double pTL = p_L + bb_L / 2.0;
    const double e1 = p_L / (g - 1.0) + ro_L * uu_L + bb_L / 2.0;
    double PO[9];
    PO[0] = ro_L * u1;
    PO[1] = ro_L * u1 * u1 + pTL - bn1 * bn1;
    PO[2] = ro_L * u1 * v1 - bn1 * bt1;
    PO[3] = ro_L * u1 * w1 - bn1 * bm1;
    PO[4] = (e1 + pTL) * u1 - bn1 * (u1 * bn1 + v1 * bt1 + w1 * bm1);
    PO[5] = 0.0;
    PO[6] = u1 * bt1 - v1 * bn1;
    PO[7] = u1 * bm1 - w1 * bn1;
    PO[8] = Q_L * u1;
    P[1] = n1 * PO[1] + t1 * PO[2] + m1 * PO[3];
    P[2] = n2 * PO[1] + t2 * PO[2] + m2 * PO[3];
    P[3] = n3 * PO[1] + t3 * PO[2] + m3 * PO[3];
    P[5] = GK_SPI4 * (n1 * PO[5] + t1 * PO[6] + m1 * PO[7]);
    P[6] = GK_SPI4 * (n2 * PO[5] + t2 * PO[6] + m2 * PO[7]);
    P[7] = GK_SPI4 * (n3 * PO[5] + t3 * PO[6] + m3 * PO[7]);
    P[0] = PO[0];
    P[4] = PO[4];
    const double SWAP = P[4];
    P[4] = P[5];
    P[5] = P[6];
    P[6] = P[7];
    P[7] = SWAP;
}

/* predictor (kernel.cu:1612-1720): half step of a cell from its own slopes.  Q, DX, DY,
 * QQ in the order rho, p, vx, vy, Bx, By, Bz. */
static void gk_predictor(const gdo_config* c, const double* Q, const double* DX,
                         const double* DY, double* QQ, double st, double y) {
    const double g = c->gamma, dx = c->dx, dy = c->dy;
    double P[8];
    double PSx = 0.0, PSy = 0.0, PUx = 0.0, PUy = 0.0, PBx = 0.0, PBy = 0.0, PBz = 0.0;
    /* faces -x, +x (times dy), +y, -y (times dx) */
    const double sg[4] = {-1.0, 1.0, 1.0, -1.0};
    for (int f = 0; f < 4; ++f) {
        const double* D = f < 2 ? DX : DY;
        const double h = f < 2 ? dy : dx;
        double ro_, p_, a[7];
        if (sg[f] < 0) {
            ro_ = Q[0] - D[0] / 2.0;
            p_ = Q[1] - D[1] / 2.0;
            for (int i = 2; i < 7; ++i) a[i] = Q[i] - D[i] / 2.0;
        } else {
            ro_ = Q[0] + D[0] / 2.0;
            p_ = Q[1] + D[1] / 2.0;
            for (int i = 2; i < 7; ++i) a[i] = Q[i] + D[i] / 2.0;
        }
        if (ro_ <= 0.0) ro_ = Q[0];
        if (p_ <= 0.0) p_ = Q[1];
        const double n1 = f < 2 ? sg[f] : 0.0, n2 = f < 2 ? 0.0 : sg[f];
        gk_potok(g, ro_, 0.0, p_, a[2], a[3], 0.0, a[4], a[5], a[6], P, n1, n2, 0.0);
        PSx = PSx + P[0] * h;
        PSy = PSy + P[7] * h;
        PUx = PUx + P[1] * h;
        PUy = PUy + P[2] * h;
        PBx = PBx + P[4] * h;
        PBy = PBy + P[5] * h;
        PBz = PBz + P[6] * h;
    }
    const double dV = dx * dy;
    QQ[0] = Q[0] - st * PSx / dV - st * Q[0] * Q[3] / y;
    if (QQ[0] <= 0) QQ[0] = Q[0];
    QQ[2] = (Q[0] * Q[2] - st * (PUx) / dV - st * (Q[0] * Q[2] * Q[3] - Q[4] * Q[5] / GK_CPI4) / y) /
            QQ[0];
    QQ[3] = (Q[0] * Q[3] - st * (PUy) / dV -
             st * (Q[0] * Q[3] * Q[3] + (Q[6] * Q[6] - Q[5] * Q[5]) / GK_CPI4) / y) / QQ[0];
    QQ[4] = (Q[4] - st * (PBx) / dV - st * (Q[3] * Q[4] - Q[5] * Q[2]) / y);
    QQ[5] = (Q[5] - st * (PBy) / dV);
    QQ[6] = (Q[6] - st * (PBz) / dV);
    const double U = gk_u8(g, Q[0], Q[1], Q[2], Q[3], 0.0, Q[4], Q[5], Q[6]);
    QQ[1] = (U - st * (PSy) / dV -
             st * (((U + Q[1] + gk_kvv(Q[4], Q[5], Q[6]) / GK_CPI8) * Q[3] -
                    Q[5] * gk_skk(Q[2], Q[3], 0.0, Q[4], Q[5], Q[6]) / GK_CPI4) / y) -
             0.5 * QQ[0] * gk_kvv(QQ[2], QQ[3], 0.0) - gk_kvv(QQ[4], QQ[5], QQ[6]) / GK_CPI8) *
            (g - 1.0);
    if (QQ[1] <= 0) QQ[1] = 0.000001;
}

static void gk_to_q(const gk_cell* c, double* q) {
    q[0] = c->sx; q[1] = c->sy; q[2] = c->ux; q[3] = c->uy;
    q[4] = c->bx; q[5] = c->by; q[6] = c->bz;
}

/* dx * minmod((a - b)/dx, (b - c)/dx) for every component; component 3 (vy) from the
 * pressures as written (kernel.cu:2966 ...) unless fixed */
static void gk_slopes(const gk_cell* a, const gk_cell* b, const gk_cell* c, double h, int fixed,
                      double* D) {
    double qa[7], qb[7], qc[7];
    gk_to_q(a, qa);
    gk_to_q(b, qb);
    gk_to_q(c, qc);
    for (int i = 0; i < 7; ++i) {
        const int j = (i == 3 && !fixed) ? 1 : i;
        D[i] = h * gdo_minmod((qa[j] - qb[j]) / h, (qb[j] - qc[j]) / h);
    }
}

static gk_cell gk_flip(gk_cell c, double fux, double fuy, double fbx, double fby, double fbz) {
    gk_cell r = c;
    r.ux = fux * c.ux; r.uy = fuy * c.uy;
    r.bx = fbx * c.bx; r.by = fby * c.by; r.bz = fbz * c.bz;
    return r;
}

/* mirrors as the reference writes them: vx, Bx, By odd (x); vy, Bz odd (y) */
static gk_cell gk_mx(gk_cell c) {
    gk_cell r = c;
    r.ux = -c.ux; r.bx = -c.bx; r.by = -c.by;
    return r;
}
static gk_cell gk_my(gk_cell c) {
    gk_cell r = c;
    r.uy = -c.uy; r.bz = -c.bz;
    return r;
}
static gk_cell gk_clamp_vx(gk_cell c) {
    if (c.ux < 0) c.ux = 0.01;
    return c;
}

static double gk_cell_step(const gdo_config* c, const double* s, const double* u, const double* b,
                           int n, int m, double T_do, double* out, int* frozen) {
    const int N = c->N, M = c->M;
    const double g = c->gamma, dx = c->dx, dy = c->dy;
    const double x_min = c->x0, y_min = c->y0;
    const double y = y_min + m * (c->y_max) / (M);
    const double x = x_min + n * (c->x_max - x_min) / (N - 1);
    const double dist = sqrt(x * x + y * y);
    const int fixed = c->scheme == 2;
    const gk_cell c1 = gk_load(s, u, b, (long)m * N + n);
    *frozen = 0;
    if (dist < c->frozen_radius) {
        *frozen = 1;
        return 1000.0;
    }
#define AT(nn, mm) gk_load(s, u, b, (long)(mm) * N + (nn))
    const gk_cell amb = {1.0, 1.0 / g, 0.0, 0.0, 0.0, 0.0, 0.0};
    gk_cell c2, c3, c4, c5, c6, c7, c8, c9, c10, c11, c12, c13;
    if (m == M - 1) { c5 = amb; c5.bx = c1.bx; c5.by = c1.by; c5.bz = c1.bz; }
    else c5 = AT(n, m + 1);
    if (n == N - 1) c2 = gk_clamp_vx(c1);
    else c2 = AT(n + 1, m);
    if (n == 0) c4 = gk_mx(c1);
    else c4 = AT(n - 1, m);
    if (m == 0) c3 = gk_my(c1);
    else c3 = AT(n, m - 1);
    if (n == N - 1) c10 = c5;
    else if (m == M - 1) { c10 = amb; c10.bx = c2.bx; c10.by = c2.by; c10.bz = c2.bz; }
    else c10 = AT(n + 1, m + 1);
    if (m == 0) {
        c12 = gk_my(c4);
        c11 = gk_my(c2);
    } else {
        if (n == 0) c12 = gk_mx(c3);
        else c12 = AT(n - 1, m - 1);
        if (n == N - 1) c11 = gk_clamp_vx(c3);
        else c11 = AT(n + 1, m - 1);
    }
    if (n == 0) c13 = gk_mx(c5);
    else if (m == M - 1) { c13 = amb; c13.bx = c4.bx; c13.by = c4.by; c13.bz = c4.bz; }
    else c13 = AT(n - 1, m + 1);
    if (n >= N - 2) c6 = gk_clamp_vx(c2);
    else c6 = AT(n + 2, m);
    if (m >= M - 2) c9 = c5;
    else c9 = AT(n, m + 2);
    if (n == 0 || n == 1) c8 = gk_mx(c2);
    else c8 = AT(n - 2, m);
    if (m == 1) c7 = gk_my(c5);
    else if (m == 0) c7 = gk_my(c3);
    else c7 = AT(n, m - 2);
#undef AT
    (void)gk_flip;
    double DX1[7], DY1[7], DX2[7], DY2[7], DX3[7], DY3[7], DX4[7], DY4[7], DX5[7], DY5[7];
    gk_slopes(&c2, &c1, &c4, dx, fixed, DX1);
    gk_slopes(&c6, &c2, &c1, dx, fixed, DX2);
    gk_slopes(&c1, &c4, &c8, dx, fixed, DX4);
    gk_slopes(&c10, &c5, &c13, dx, fixed, DX5);
    gk_slopes(&c11, &c3, &c12, dx, fixed, DX3);
    gk_slopes(&c5, &c1, &c3, dy, fixed, DY1);
    gk_slopes(&c9, &c5, &c1, dy, fixed, DY5);
    gk_slopes(&c13, &c4, &c12, dy, fixed, DY4);
    gk_slopes(&c10, &c2, &c11, dy, fixed, DY2);
    gk_slopes(&c1, &c3, &c7, dy, fixed, DY3);
    double Q1[7], Q2[7], Q3[7], Q4[7], Q5[7];
    gk_to_q(&c1, Q1); gk_to_q(&c2, Q2); gk_to_q(&c3, Q3); gk_to_q(&c4, Q4); gk_to_q(&c5, Q5);
    double QQ1[7], QQ2[7], QQ3[7], QQ4[7], QQ5[7];
    const double st = T_do / 2.0;
    gk_predictor(c, Q1, DX1, DY1, QQ1, st, y);
    gk_predictor(c, Q2, DX2, DY2, QQ2, st, y);
    gk_predictor(c, Q3, DX3, DY3, QQ3, st, y - dy);
    gk_predictor(c, Q4, DX4, DY4, QQ4, st, y);
    gk_predictor(c, Q5, DX5, DY5, QQ5, st, y + dy);
    /* faces E (own +DX1, nbr Q2 -DX2), S (own -DY1, nbr Q3 +DY3), W (own -DX1, nbr Q4 +DX4),
     * N (own +DY1, nbr Q5 -DY5) */
    const double* nbrQ[4] = {Q2, Q3, Q4, Q5};
    const double* nbrQQ[4] = {QQ2, QQ3, QQ4, QQ5};
    const double* ownD[4] = {DX1, DY1, DX1, DY1};
    const double* nbrD[4] = {DX2, DY3, DX4, DY5};
    const double ownS[4] = {1.0, -1.0, -1.0, 1.0};
    const double fn1[4] = {1.0, 0.0, -1.0, 0.0}, fn2[4] = {0.0, -1.0, 0.0, 1.0};
    double tmin = 1000;
    double PSx = 0.0, PSy = 0.0, PUx = 0.0, PUy = 0.0, PBx = 0.0, PBy = 0.0, PBz = 0.0;
    for (int f = 0; f < 4; ++f) {
        const double* A = nbrQ[f];
        const double* AA = nbrQQ[f];
        double L[8], R[8];
        double ro_1, p_1, ro_2, p_2;
        if (ownS[f] > 0) {
            ro_1 = (Q1[0] + QQ1[0]) / 2.0 + ownD[f][0] / 2.0;
            p_1 = (Q1[1] + QQ1[1]) / 2.0 + ownD[f][1] / 2.0;
        } else {
            ro_1 = (Q1[0] + QQ1[0]) / 2.0 - ownD[f][0] / 2.0;
            p_1 = (Q1[1] + QQ1[1]) / 2.0 - ownD[f][1] / 2.0;
        }
        if (ro_1 <= 0.0) ro_1 = (Q1[0] + QQ1[0]) / 2.0;
        if (p_1 <= 0.0) p_1 = (Q1[1] + QQ1[1]) / 2.0;
        if (ownS[f] > 0) {
            ro_2 = (A[0] + AA[0]) / 2.0 - nbrD[f][0] / 2.0;
            p_2 = (A[1] + AA[1]) / 2.0 - nbrD[f][1] / 2.0;
        } else {
            ro_2 = (A[0] + AA[0]) / 2.0 + nbrD[f][0] / 2.0;
            p_2 = (A[1] + AA[1]) / 2.0 + nbrD[f][1] / 2.0;
        }
        if (ro_2 <= 0.0) ro_2 = (A[0] + AA[0]) / 2.0;
        if (p_2 <= 0.0) p_2 = (A[1] + AA[1]) / 2.0;
        L[0] = ro_1; L[1] = p_1; L[4] = 0.0;
        R[0] = ro_2; R[1] = p_2; R[4] = 0.0;
        const int qi[5] = {2, 3, 4, 5, 6}, li[5] = {2, 3, 5, 6, 7};
        for (int t = 0; t < 5; ++t) {
            const int i = qi[t];
            L[li[t]] = ownS[f] > 0 ? (Q1[i] + QQ1[i]) / 2.0 + ownD[f][i] / 2.0
                                   : (Q1[i] + QQ1[i]) / 2.0 - ownD[f][i] / 2.0;
            R[li[t]] = ownS[f] > 0 ? (A[i] + AA[i]) / 2.0 - nbrD[f][i] / 2.0
                                   : (A[i] + AA[i]) / 2.0 + nbrD[f][i] / 2.0;
        }
        double P[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const double rad = (f == 0 || f == 2) ? dx : dy;
        const double t = gdo_hlld(L, R, fn1[f], fn2[f], 0.0, rad, 3, g, c->krit, P);
        tmin = my_min(tmin, t);
        const double h = (f == 0 || f == 2) ? dy : dx;
        PSx = PSx + P[0] * h;
        PSy = PSy + P[7] * h;
        PUx = PUx + P[1] * h;
        PUy = PUy + P[2] * h;
        PBx = PBx + P[4] * h;
        PBy = PBy + P[5] * h;
        PBz = PBz + P[6] * h;
    }
    const double dV = dx * dy;
    const double Pdiv = 0.0;
    const double hT = T_do / 2.0;
    double A[7];
    for (int i = 0; i < 7; ++i) A[i] = (Q1[i] + QQ1[i]) / 2.0;
    double r2 = A[0] - hT * PSx / dV - hT * A[0] * A[3] / y;
    if (r2 <= 0) r2 = A[0];
    const double ux2 = (A[0] * A[2] - hT * (PUx + (A[4] / GK_CPI4) * Pdiv) / dV -
                        hT * (A[0] * A[2] * A[3] - A[4] * A[5] / GK_CPI4) / y) / r2;
    const double uy2 = (A[0] * A[3] - hT * (PUy + (A[5] / GK_CPI4) * Pdiv) / dV -
                        hT * (A[0] * A[3] * A[3] + (A[6] * A[6] - A[5] * A[5]) / GK_CPI4) / y) / r2;
    const double bx2 = (A[4] - hT * (PBx + A[2] * Pdiv) / dV - hT * (A[3] * A[4] - A[5] * A[2]) / y);
    const double by2 = (A[5] - hT * (PBy + A[3] * Pdiv) / dV);
    const double bz2 = (A[6] - hT * (PBz) / dV);
    const double U = gk_u8(g, A[0], A[1], A[2], A[3], 0.0, A[4], A[5], A[6]);
    const double sk = gk_skk(A[2], A[3], 0.0, A[4], A[5], A[6]);
    double p2 = (U - hT * (PSy + (sk / GK_CPI4) * Pdiv) / dV -
                 hT * (((U + A[1] + gk_kvv(A[4], A[5], A[6]) / GK_CPI8) * A[3] -
                        A[5] * sk / GK_CPI4) / y) -
                 0.5 * r2 * gk_kvv(ux2, uy2, 0.0) - gk_kvv(bx2, by2, bz2) / GK_CPI8) * (g - 1.0);
    if (p2 <= 0) p2 = 0.000001;
    out[0] = r2; out[1] = p2; out[2] = ux2; out[3] = uy2;
    out[4] = bx2; out[5] = by2; out[6] = bz2;
    return tmin;
}

static double gdo_step_hancock(const gdo_config* c, const double* s, const double* u,
                               const double* b, double* s2, double* u2, double* b2, double T_do,
                               double T_in, int dt_only) {
    const int N = c->N, M = c->M;
    double T = T_in;
#pragma omp parallel
    {
        double tloc = T_in;
#pragma omp for schedule(static)
        for (int m = 0; m < M; ++m) {
            for (int n = 0; n < N; ++n) {
                const long k = (long)m * N + n;
                double out[7];
                int frozen = 0;
                const double t = gk_cell_step(c, s, u, b, n, m, T_do, out, &frozen);
                if (frozen) {
                    if (!dt_only) {
                        s2[2 * k] = s[2 * k]; s2[2 * k + 1] = s[2 * k + 1];
                        u2[2 * k] = u[2 * k]; u2[2 * k + 1] = u[2 * k + 1];
                        b2[3 * k] = b[3 * k]; b2[3 * k + 1] = b[3 * k + 1];
                        b2[3 * k + 2] = b[3 * k + 2];
                    }
                    continue;
                }
                if (tloc > t) tloc = t;
                if (!dt_only) {
                    s2[2 * k] = out[0]; s2[2 * k + 1] = out[1];
                    u2[2 * k] = out[2]; u2[2 * k + 1] = out[3];
                    b2[3 * k] = out[4]; b2[3 * k + 1] = out[5]; b2[3 * k + 2] = out[6];
                }
            }
        }
#pragma omp critical
        {
            if (tloc < T) T = tloc;
        }
    }
    return T;
}

double gdo_step(const gdo_config* c, const double* s, const double* u, const double* b,
                double* s2, double* u2, double* b2, double T_do, double T_in, int dt_only) {
    if (c->scheme == 1 || c->scheme == 2)
        return gdo_step_hancock(c, s, u, b, s2, u2, b2, T_do, T_in, dt_only);
    const int N = c->N, M = c->M;
    double T = T_in;
#pragma omp parallel
    {
        double tloc = T_in;
#pragma omp for schedule(static)
        for (int m = 0; m < M; ++m) {
            for (int n = 0; n < N; ++n) {
                const long k = (long)m * N + n;
                const double y = c->y0 + m * c->dy;
                const double x = c->x0 + n * c->dx;
                if (c->frozen_radius > 0.0) {
                    const double dist = sqrt(x * x + y * y);
                    if (dist < c->frozen_radius) {
                        if (!dt_only) {
                            s2[2 * k] = s[2 * k]; s2[2 * k + 1] = s[2 * k + 1];
                            u2[2 * k] = u[2 * k]; u2[2 * k + 1] = u[2 * k + 1];
                            if (b && b2) {
                                b2[3 * k] = b[3 * k]; b2[3 * k + 1] = b[3 * k + 1];
                                b2[3 * k + 2] = b[3 * k + 2];
                            }
                        }
                        continue;
                    }
                }
                cell_faces F;
                build_faces(c, s, u, b, n, m, x, y, &F);
                double out[7] = {0, 0, 0, 0, 0, 0, 0};
                double tcell = (c->physics == GDO_MHD) ? mhd_cell(c, &F, y, T_do, out)
                                                       : euler_cell(c, &F, y, T_do, out);
                if (tloc > tcell) tloc = tcell;
                if (!dt_only) {
                    s2[2 * k] = out[0]; s2[2 * k + 1] = out[1];
                    u2[2 * k] = out[2]; u2[2 * k + 1] = out[3];
                    if (c->physics == GDO_MHD) {
                        b2[3 * k] = out[4]; b2[3 * k + 1] = out[5]; b2[3 * k + 2] = out[6];
                    }
                }
            }
        }
#pragma omp critical
        {
            if (tloc < T) T = tloc;
        }
    }
    return T;
}

int gdo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

void gdo_funk_time(double* T, double* T_do, double* TT, int* i) {
    *T_do = *T;
    *TT = *TT + *T_do;
    *T = 10000000;
    *i = *i + 1;
}

/* ---- state files ------------------------------------------------------------------------
 * Restart text: the stream of kernel.cu:4245-4254, one line per cell, x = x_min + n dx,
 * y = y_min + m dy; an Euler state (b == NULL) writes 0 for B. */
int gdo_write_restart(const gdo_config* c, const double* s, const double* u, const double* b,
                      const char* path) {
    FILE* f = fopen(path, "w");
    if (!f) return 1;
    const long K = (long)c->N * c->M;
    for (long k = 0; k < K; ++k) {
        const int n = (int)(k % c->N), m = (int)(k / c->N);
        const double y = c->y0 + m * c->dy;
        const double x = c->x0 + n * c->dx;
        fprintf(f, "%g %g %g %g %g %g %g %g %g\n", x, y, s[2 * k], s[2 * k + 1], u[2 * k],
                u[2 * k + 1], b ? b[3 * k] : 0.0, b ? b[3 * k + 1] : 0.0, b ? b[3 * k + 2] : 0.0);
    }
    return fclose(f) != 0;
}

/* Restart reader: `fin >> c1 >> c2 >> a1 ... >> a7` per cell, restated with fscanf("%lf")
 * (both are correctly rounded decimal conversions). */
int gdo_read_restart(const gdo_config* c, const char* path, double* s, double* u, double* b) {
    FILE* f = fopen(path, "r");
    if (!f) return 1;
    const long K = (long)c->N * c->M;
    for (long k = 0; k < K; ++k) {
        double v[9];
        for (int i = 0; i < 9; ++i)
            if (fscanf(f, "%lf", &v[i]) != 1) {
                fclose(f);
                return 1;
            }
        s[2 * k] = v[2];
        s[2 * k + 1] = v[3];
        u[2 * k] = v[4];
        u[2 * k + 1] = v[5];
        if (b) {
            b[3 * k] = v[6];
            b[3 * k + 1] = v[7];
            b[3 * k + 2] = v[8];
        }
    }
    fclose(f);
    return 0;
}

/* save_b3.dat (kernel.cu:4255-4261): x, y, rho, p, vx, vy, Bz as raw doubles. */
int gdo_write_binary(const gdo_config* c, const double* s, const double* u, const double* b,
                     const char* path) {
    FILE* f = fopen(path, "wb");
    if (!f) return 1;
    const long K = (long)c->N * c->M;
    for (long k = 0; k < K; ++k) {
        const int n = (int)(k % c->N), m = (int)(k / c->N);
        const double rec[7] = {c->x0 + n * c->dx, c->y0 + m * c->dy, s[2 * k], s[2 * k + 1],
                               u[2 * k], u[2 * k + 1], b ? b[3 * k + 2] : 0.0};
        if (fwrite(rec, sizeof(double), 7, f) != 7) {
            fclose(f);
            return 1;
        }
    }
    return fclose(f) != 0;
}

/* print_file_mini (b == NULL, kernel.cu:3682-3722) and print_file_mini2 (kernel.cu:3724-3808,
 * with_time adds SOLUTIONTIME): every nmin-th point, Max and T per point, then the
 * quadrilateral connectivity. */
int gdo_write_tecplot(const gdo_config* c, const double* s, const double* u, const double* b,
                      int nmin, double x_min, double x_max, double y_min, double y_max,
                      int with_time, double time, const char* path) {
    FILE* f = fopen(path, "w");
    if (!f) return 1;
    const int N = c->N, M = c->M;
    const int nn = (N + nmin - 1) / nmin, mm = (M + nmin - 1) / nmin;
    if (b)
        fprintf(f, "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", \"Vx\", "
                   "\"Vy\", \"Bx\", \"By\", \"Bz\", \"Max\", \"T\", ZONE T = \"HP\", N = %d , "
                   "E = %d, F = FEPOINT, ET = quadrilateral",
                nn * mm, (nn - 1) * (mm - 1));
    else
        fprintf(f, "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", \"Vx\", "
                   "\"Vy\", \"Max\", \"T\", ZONE T = \"HP\", N = %d , E = %d, F = FEPOINT, "
                   "ET = quadrilateral",
                nn * mm, (nn - 1) * (mm - 1));
    if (with_time) fprintf(f, ", SOLUTIONTIME = %g", time);
    fprintf(f, "\n");
    const long K = (long)N * M;
    for (long k = 0; k < K; ++k) {
        const int n = (int)(k % N), m = (int)((k - n) / N);
        if (n % nmin != 0 || m % nmin != 0) continue;
        const double y = y_min + m * (y_max - y_min) / (M - 1);
        const double x = x_min + n * (x_max - x_min) / (N - 1);
        double Max = 0.0, Temp = 0.0;
        const double r = s[2 * k], p = s[2 * k + 1], vx = u[2 * k], vy = u[2 * k + 1];
        if (r > 0.0) {
            Max = sqrt((vx * vx + vy * vy) / (c->gamma * p / r));
            Temp = p / r;
        }
        if (b)
            fprintf(f, "%g %g %g %g %g %g %g %g %g %g %g\n", x, y, r, p, vx, vy, b[3 * k],
                    b[3 * k + 1], b[3 * k + 2], Max, Temp);
        else
            fprintf(f, "%g %g %g %g %g %g %g %g\n", x, y, r, p, vx, vy, Max, Temp);
    }
    for (long k = 0; k < (long)nn * mm; ++k) {
        const int n = (int)(k % nn), m = (int)((k - n) / nn);
        if (m < mm - 1 && n < nn - 1)
            fprintf(f, "%d %d %d %d\n", m * nn + n + 1, m * nn + n + 2, (m + 1) * nn + n + 2,
                    (m + 1) * nn + n + 1);
    }
    return fclose(f) != 0;
}
