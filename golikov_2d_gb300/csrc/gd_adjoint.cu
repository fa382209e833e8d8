// gd_adjoint.cu -- hand-written discrete adjoint (reverse mode, VJP) of the fast MHD step.
//
// The step U' = S(U; dt) of gd_fast_mhd.cu (HLLD, minmod TVD, Powell source, Cartesian,
// periodic) is differentiated with dt held fixed and every non-smooth choice (minmod
// selection, wave-speed min/max, region selection, guards, floors) frozen at the branch
// the forward values take.  Given lambda' = dL/dU', one reverse step returns
// lambda = dL/dU = S'(U)^T lambda' in two passes:
//
//   A  per cell (adj_update_kernel): the transpose of the cell update.  Inputs: U, the
//      forward flux differences d[7] and the Powell term divb of that cell (stored by the
//      recompute pass), lambda'.  Outputs: the direct adjoint of the cell state, the adjoint
//      of d[7] and of divb.
//   B  per face, then per cell (adj_face_kernel, adj_gather_kernel): every face recomputes
//      its forward states and HLLD flux once and runs the flux's reverse sweep on
//      Fbar = k (dbar_low - dbar_high); the adjoints of the two face states are gathered
//      into the cells through the reconstruction (c +- slope/2, minmod choice, rho/p
//      fallback) and the Powell central difference, in a fixed order (deterministic).
//
// All internal arithmetic is in Heaviside-Lorentz field units (b = B / sqrt(4 pi)), as in
// the forward kernel; adjoints w.r.t. the stored Gaussian field are converted at the ends.
#include "gd_internal.cuh"
#include "gd_kernels.h"
#include "gd_mhd_flux.cuh"

namespace gd {
namespace {

constexpr int NF = 7;
constexpr int NT = 256;

// ---------------------------------------------------------------------------------------
// Pass A: transpose of the cell update (Cartesian).
// aux layout per cell: d[0..6] (slot order m, e, mx, my, bx, by, bz), divb.  Adjoint
// scratch per cell: qbar[0..6] (field order rho, p, vx, vy, bx, by, bz, field in b units),
// dbar[0..6] (slot order), divbbar.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) adj_update_kernel(Params P, CPlanes U, const double* aux,
                                                        CPlanes lam_out, double* scratch) {
    const long long K = (long long)P.N * P.M;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K;
         k += (long long)gridDim.x * blockDim.x) {
        const double r = U.f[0][k], p = U.f[1][k], u = U.f[2][k], v = U.f[3][k];
        // rounded products, as the forward update has them (see ld_b)
        const double bx = imul(U.f[4][k], kInvSpi4), by = imul(U.f[5][k], kInvSpi4);
        const double bz = imul(U.f[6][k], kInvSpi4);
        double d[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) d[f] = aux[(size_t)f * K + k];
        const double divb = aux[(size_t)7 * K + k];
        // forward (same operations as the tile update)
        const double ub = fma(u, bx, imul(v, by));
        const double bb = fma(bz, bz, fma(by, by, imul(bx, bx)));
        const double E = fma(p, P.inv_gm1, half_exact(fma(r, fma(u, u, imul(v, v)), bb)));
        double r2 = r - d[0];
        const bool rfl = le_zero(r2);
        if (rfl) r2 = r;
        const double mx2 = fma(r, u, -fma(bx, divb, d[2]));
        const double my2 = fma(r, v, -fma(by, divb, d[3]));
        const double bx2 = bx - fma(u, divb, d[4]);
        const double by2 = by - fma(v, divb, d[5]);
        const double bz2 = bz - d[6];
        const double E2 = E - fma(ub, divb, d[1]);
        const double inv = rcp_fast(r2);
        const double u2 = imul(mx2, inv), v2 = imul(my2, inv);
        const double p2 = (E2 - 0.5 * fma(r2, fma(u2, u2, imul(v2, v2)),
                                          fma(bz2, bz2, fma(by2, by2, imul(bx2, bx2))))) * P.gm1;
        const bool pfl = le_zero(p2);
        // reverse
        double r2b = lam_out.f[0][k], p2b = lam_out.f[1][k];
        double u2b = lam_out.f[2][k], v2b = lam_out.f[3][k];
        double bx2b = imul(lam_out.f[4][k], kSpi4), by2b = imul(lam_out.f[5][k], kSpi4);
        double bz2b = imul(lam_out.f[6][k], kSpi4);
        double E2b = 0.0;
        if (!pfl) {
            E2b = p2b * P.gm1;
            const double Xb = -0.5 * p2b * P.gm1;
            r2b += Xb * fma(u2, u2, v2 * v2);
            u2b += Xb * 2.0 * r2 * u2;
            v2b += Xb * 2.0 * r2 * v2;
            bx2b += Xb * 2.0 * bx2;
            by2b += Xb * 2.0 * by2;
            bz2b += Xb * 2.0 * bz2;
        }
        const double mx2b = imul(u2b, inv), my2b = imul(v2b, inv);
        const double invb = u2b * mx2 + v2b * my2;
        r2b += -invb * inv * inv;
        double rb = 0.0, pb = 0.0, ub_ = 0.0, vb = 0.0, bxb = 0.0, byb = 0.0, bzb = 0.0;
        double db[NF] = {0, 0, 0, 0, 0, 0, 0};
        double divbb = 0.0, Eb = 0.0, ubb = 0.0;
        rb += r2b;
        if (!rfl) db[0] -= r2b;
        Eb += E2b;
        ubb -= E2b * divb;
        divbb -= E2b * ub;
        db[1] -= E2b;
        bzb += bz2b;
        db[6] -= bz2b;
        byb += by2b;
        vb -= by2b * divb;
        divbb -= by2b * v;
        db[5] -= by2b;
        bxb += bx2b;
        ub_ -= bx2b * divb;
        divbb -= bx2b * u;
        db[4] -= bx2b;
        rb += my2b * v;
        vb += my2b * r;
        byb -= my2b * divb;
        divbb -= my2b * by;
        db[3] -= my2b;
        rb += mx2b * u;
        ub_ += mx2b * r;
        bxb -= mx2b * divb;
        divbb -= mx2b * bx;
        db[2] -= mx2b;
        pb += Eb * P.inv_gm1;
        rb += 0.5 * Eb * fma(u, u, v * v);
        ub_ += Eb * r * u;
        vb += Eb * r * v;
        const double bbb = 0.5 * Eb;
        bxb += 2.0 * bbb * bx + ubb * u;
        byb += 2.0 * bbb * by + ubb * v;
        bzb += 2.0 * bbb * bz;
        ub_ += ubb * bx;
        vb += ubb * by;
        double* s = scratch;
        s[0 * K + k] = rb;
        s[1 * K + k] = pb;
        s[2 * K + k] = ub_;
        s[3 * K + k] = vb;
        s[4 * K + k] = bxb;
        s[5 * K + k] = byb;
        s[6 * K + k] = bzb;
#pragma unroll
        for (int f = 0; f < NF; ++f) s[(size_t)(7 + f) * K + k] = db[f];
        s[(size_t)14 * K + k] = divbb;
    }
}

// ---------------------------------------------------------------------------------------
// Reverse sweep of one HLLD face flux (method 3) in the local frame.
// Inputs: the two face states A (low) and B (high) as (r, p, un, ut, bn, bt, bz) and the
// adjoint of the flux (m, mn, mt, e, bn, bt, bz).  Writes the adjoints of A and B to Ab, Bb.
// The forward part repeats hlld_local<double> of gd_fast_mhd.cu operation for operation.
// The reverse does per-side work only where the adjoint can be non-zero: the flux's base
// terms and the energy enter through the upwind side K alone (the side whose state or star
// state gives the flux), the fast speed through the side of max(cf) alone, and only K's
// star energy and its sb term reach the flux; those chains run once, on the selected
// side's values, and their results are added to that side.
// ---------------------------------------------------------------------------------------
struct SideV {
    double r, p, un, ut, bn, bt, bz;
    double bn2, bb, pT, gp, a, disc, rq, rs, cf;  // rq = 1 / sqrt(disc), rs = 1 / sqrt(X r)
    bool disc0;
};

__device__ __forceinline__ void side_fwd(SideV& S, const double* q, const Params& P) {
    S.r = q[0]; S.p = q[1]; S.un = q[2]; S.ut = q[3]; S.bn = q[4]; S.bt = q[5]; S.bz = q[6];
    S.bn2 = imul<true>(S.bn, S.bn);
    S.bb = fma(S.bz, S.bz, fma(S.bt, S.bt, S.bn2));
    S.pT = fma(0.5, S.bb, S.p);
    S.gp = imul<true>(P.gamma, S.p);
    S.a = S.gp + S.bb;
    double disc = fma(S.a, S.a, imul<true>(imul<true>(-4.0, S.gp), S.bn2));
    S.disc0 = le_zero(disc);
    S.disc = S.disc0 ? 0.0 : disc;
    // sqrt_fast(disc) of the forward, keeping 1/sqrt(disc) for the reverse
    double sq;
    sqrt_and_rs_im<true>(S.disc, sq, S.rq);
    const double X = imul<true>(0.5, S.a + sq);
    // cf = sqrt_over(X, r) of the forward, keeping its 1/sqrt(X r) for the reverse
    sqrt_over_rs_im<true>(X, S.r, S.cf, S.rs);
}

// per-side adjoint accumulators of the face state and of two derived quantities
struct SideB {
    double r, p, un, ut, bn, bt, bz, pT, bb, bn2;
};

// adds k to the side the select names with one FP64 add (the other side is untouched)
__device__ __forceinline__ void add_to(bool first, double& a, double& b, double k) {
    const double s = (first ? a : b) + k;
    a = first ? s : a;
    b = first ? b : s;
}

// the side-generic tail: pT = 0.5 bb + p, bb = bz^2 + bt^2 + bn2, bn2 = bn^2
__device__ __forceinline__ void side_tail(const SideV& S, SideB& b, double* qb) {
    const double bbb = fma(0.5, b.pT, b.bb);
    const double bn2b = b.bn2 + bbb;
    qb[0] = b.r;
    qb[1] = b.p + b.pT;
    qb[2] = b.un;
    qb[3] = b.ut;
    qb[4] = fma(2.0 * bn2b, S.bn, b.bn);
    qb[5] = fma(2.0 * bbb, S.bt, b.bt);
    qb[6] = fma(2.0 * bbb, S.bz, b.bz);
}

// Fb = (m, mn, mt, e, bn, bt, bz); qa_b, qb_b receive (r, p, un, ut, bn, bt, bz).
__device__ __forceinline__ void hlld_vjp(const double* qa, const double* qb, const double* Fb,
                                         const Params& P, double* qa_b, double* qb_b) {
    SideV A, B;
    side_fwd(A, qa, P);
    side_fwd(B, qb, P);
    // ---- forward, shared part
    const bool minA = !dlt(B.un, A.un);              // uminN = A.un (else B.un)
    const bool maxB = dlt(A.un, B.un);               // umaxN = B.un (else A.un)
    const double uminN = minA ? A.un : B.un;
    const double umaxN = maxB ? B.un : A.un;
    const bool cfB = mag_lt(A.cf, B.cf);
    const double cmax = cfB ? B.cf : A.cf;
    const double SL = uminN - cmax, SR = umaxN + cmax;
    const double suL = SL - A.un, suR = SR - B.un;
    const double mL = A.r * suL, mR = B.r * suR;
    const double iden = rcp_fast(mR - mL);
    const double SMn = (fma(mR, B.un, -mL * A.un) - B.pT) + A.pT;
    const double SM = SMn * iden;
    const double PTTn = fma(mL * mR, B.un - A.un, fma(mR, A.pT, -mL * B.pT));
    const double PTT = PTTn * iden;
    const bool UUR = mag_lt(SL, SR);
    const double UU = dabs(UUR ? SR : SL);
    const double iS = rcp_fast(SR - SL);
    const double bnn = fma(SR, B.bn, -SL * A.bn);
    const double bn = bnn * iS;
    const double iL = rcp_fast(SL - SM), iR = rcp_fast(SR - SM);
    const double rLL = mL * iL, rRR = mR * iR;
    const double bbn = bn * bn;
    // star states
    const double ttL = fma(mL, SL - SM, -bbn);
    const bool gL = mag_ge(ttL, kMag1em5);
    double itL = 0, cL = 0, dL = 0, vLL, wLL, btL, bzL;
    if (gL) {
        itL = rcp_fast(ttL);
        cL = bn * (SM - A.un) * itL;
        dL = fma(mL, suL, -bbn) * itL;
        vLL = fma(-cL, A.bt, A.ut);
        wLL = -cL * A.bz;
        btL = A.bt * dL;
        bzL = A.bz * dL;
    } else {
        vLL = A.ut; wLL = 0.0; btL = 0.0; bzL = 0.0;
    }
    const double ttR = fma(mR, SR - SM, -bbn);
    const bool gR = mag_ge(ttR, kMag1em5);
    double itR = 0, cR = 0, dR = 0, vRR, wRR, btR, bzR;
    if (gR) {
        itR = rcp_fast(ttR);
        cR = bn * (SM - B.un) * itR;
        dR = fma(mR, suR, -bbn) * itR;
        vRR = fma(-cR, B.bt, B.ut);
        wRR = -cR * B.bz;
        btR = B.bt * dR;
        bzR = B.bz * dR;
    } else {
        vRR = B.ut; wRR = 0.0; btR = 0.0; bzR = 0.0;
    }
    const double SMbn = SM * bn;
    double isLL, isRR, sLL, sRR;
    rsqrt_and_sqrt(rLL, isLL, sLL);
    rsqrt_and_sqrt(rRR, isRR, sRR);
    const bool bnz = mag_ge(bn, kMag1em6 + 1);
    const double abn = dabs(bn);
    const double SLL = bnz ? fma(-abn, isLL, SM) : SM;
    const double SRR = bnz ? fma(abn, isRR, SM) : SM;
    const int idbn = bnz ? (gt_zero(bn) ? 1 : -1) : 0;
    const bool takeL = ge_zero(SL) || ge_zero(SM);
    int level;
    if (takeL) level = ge_zero(SL) ? 0 : (ge_zero(SLL) ? 1 : 2);
    else level = gt_zero(SRR) ? 2 : (gt_zero(SR) ? 1 : 0);
    // the upwind side K: its state, star state and energies
    const double Kr = takeL ? A.r : B.r, Kp = takeL ? A.p : B.p;
    const double Kun = takeL ? A.un : B.un, Kut = takeL ? A.ut : B.ut;
    const double Kbn = takeL ? A.bn : B.bn, Kbt = takeL ? A.bt : B.bt;
    const double Kbz = takeL ? A.bz : B.bz, KpT = takeL ? A.pT : B.pT;
    const double Kbb = takeL ? A.bb : B.bb;
    const double S = takeL ? SL : SR;
    const double su = takeL ? suL : suR;
    const double iK = takeL ? iL : iR;
    const double rK = takeL ? rLL : rRR;
    const double vK = takeL ? vLL : vRR;
    const double wK = takeL ? wLL : wRR;
    const double btK = takeL ? btL : btR;
    const double bzK = takeL ? bzL : bzR;
    const double vsq = fma(Kun, Kun, Kut * Kut);
    const double KE = fma(Kp, P.inv_gm1, 0.5 * fma(Kr, vsq, Kbb));
    const double sbK = fma(wK, bzK, fma(vK, btK, SMbn));
    const double wKf = fma(Kun, Kbn, Kut * Kbt);
    const double eKn = fma(KE, su, fma(PTT, SM, -KpT * Kun)) + bn * (wKf - sbK);
    const double eK = eKn * iK;
    // double-star (only needed for level 2)
    double is = 0, vL3 = 0, wL3 = 0, s2 = 0, bt3 = 0, bz3 = 0, sb3 = 0, sK = 0, e3 = 0, S2 = 0;
    if (level == 2) {
        is = rcp_fast(sLL + sRR);
        vL3 = (fma(sLL, vLL, sRR * vRR) + sgn_select(btR - btL, idbn)) * is;
        wL3 = (fma(sLL, wLL, sRR * wRR) + sgn_select(bzR - bzL, idbn)) * is;
        s2 = sgn_select(sLL * sRR, idbn);
        bt3 = fma(s2, vRR - vLL, fma(sLL, btR, sRR * btL)) * is;
        bz3 = fma(s2, wRR - wLL, fma(sLL, bzR, sRR * bzL)) * is;
        sb3 = fma(wL3, bz3, fma(vL3, bt3, SMbn));
        sK = takeL ? -sLL : sRR;
        e3 = fma(sgn_select(sK, idbn), sbK - sb3, eK);
        S2 = takeL ? SLL : SRR;
    }

    // ---- reverse ------------------------------------------------------------------------
    SideB Ab = {}, Bb = {};
    // adjoints of the K side's state and energy (added to its side at the end)
    double kr = 0, kun = 0, kut = 0, kE = 0, kbt = 0, kbz = 0, kbn = 0, kpT = 0;
    // adjoints of intermediates
    double SLb = 0, SRb = 0, SMb = 0, PTTb = 0, UUb = 0, bnb = 0;
    double rLLb = 0, rRRb = 0, iLb = 0, iRb = 0;
    double vLLb = 0, wLLb = 0, btLb = 0, bzLb = 0, vRRb = 0, wRRb = 0, btRb = 0, bzRb = 0;
    double sLLb = 0, sRRb = 0, SLLb = 0, SRRb = 0, SMbnb = 0;
    const double Fm = Fb[0], Fmn = Fb[1], Fmt = Fb[2], Fe = Fb[3], Fbn = Fb[4], Fbt = Fb[5],
                 Fbz = Fb[6];
    // F.bn = -UU (B.bn - A.bn)
    UUb = -Fbn * (B.bn - A.bn);
    Bb.bn = -Fbn * UU;
    Ab.bn = Fbn * UU;
    double Sb = 0, rKb = 0, vKb = 0, wKb = 0, eKb = 0, btKb = 0, bzKb = 0, sbKb = 0;
    if (level >= 1) {
        if (level == 2) {
            // F.mt += S2 rK (vL3 - vK); F.e += S2 (e3 - eK); F.bt += S2 (bt3 - btK);
            // F.bz += S2 (bz3 - bzK)
            const double S2b = Fmt * rK * (vL3 - vK) + Fe * (e3 - eK) + Fbt * (bt3 - btK) +
                               Fbz * (bz3 - bzK);
            rKb += Fmt * S2 * (vL3 - vK);
            double vL3b = Fmt * S2 * rK;
            vKb -= Fmt * S2 * rK;
            double e3b = Fe * S2;
            eKb -= Fe * S2;
            double bt3b = Fbt * S2;
            btKb -= Fbt * S2;
            double bz3b = Fbz * S2;
            bzKb -= Fbz * S2;
            if (takeL) SLLb += S2b; else SRRb += S2b;
            // e3 = eK + sgn(sK) (sbK - sb3)
            eKb += e3b;
            const double sKv = sgn_select(sK, idbn);
            const double sKvb = e3b * (sbK - sb3);
            sbKb += e3b * sKv;
            double sb3b = -e3b * sKv;
            const double sKb = sgn_select(sKvb, idbn);
            if (takeL) sLLb -= sKb; else sRRb += sKb;
            // sb3 = wL3 bz3 + vL3 bt3 + SMbn
            double wL3b = sb3b * bz3;
            bz3b += sb3b * wL3;
            vL3b += sb3b * bt3;
            bt3b += sb3b * vL3;
            SMbnb += sb3b;
            // bz3 = (s2 (wRR - wLL) + sLL bzR + sRR bzL) is
            double isb = bz3b * (bz3 * (sLL + sRR));  // bz3 / is = numerator
            {
                const double nb = bz3b * is;
                double s2b = nb * (wRR - wLL);
                wRRb += nb * s2;
                wLLb -= nb * s2;
                sLLb += nb * bzR;
                bzRb += nb * sLL;
                sRRb += nb * bzL;
                bzLb += nb * sRR;
                // bt3 = (s2 (vRR - vLL) + sLL btR + sRR btL) is
                isb += bt3b * (bt3 * (sLL + sRR));
                const double mb = bt3b * is;
                s2b += mb * (vRR - vLL);
                vRRb += mb * s2;
                vLLb -= mb * s2;
                sLLb += mb * btR;
                btRb += mb * sLL;
                sRRb += mb * btL;
                btLb += mb * sRR;
                // s2 = sgn(sLL sRR)
                const double pb = sgn_select(s2b, idbn);
                sLLb += pb * sRR;
                sRRb += pb * sLL;
            }
            // wL3 = (sLL wLL + sRR wRR + sgn(bzR - bzL)) is
            {
                isb += wL3b * (wL3 * (sLL + sRR));
                const double nb = wL3b * is;
                sLLb += nb * wLL;
                wLLb += nb * sLL;
                sRRb += nb * wRR;
                wRRb += nb * sRR;
                const double tb = sgn_select(nb, idbn);
                bzRb += tb;
                bzLb -= tb;
            }
            // vL3 = (sLL vLL + sRR vRR + sgn(btR - btL)) is
            {
                isb += vL3b * (vL3 * (sLL + sRR));
                const double nb = vL3b * is;
                sLLb += nb * vLL;
                vLLb += nb * sLL;
                sRRb += nb * vRR;
                vRRb += nb * sRR;
                const double tb = sgn_select(nb, idbn);
                btRb += tb;
                btLb -= tb;
            }
            // is = 1 / (sLL + sRR)
            const double db = -isb * is * is;
            sLLb += db;
            sRRb += db;
        }
        // level-1 terms: F.m += S (rK - K.r); F.mn += S (rK SM - K.r K.un);
        // F.mt += S (rK vK - K.r K.ut); F.e += S (eK - K.E); F.bt += S (btK - K.bt);
        // F.bz += S (bzK - K.bz)
        Sb += Fm * (rK - Kr) + Fmn * fma(rK, SM, -Kr * Kun) + Fmt * fma(rK, vK, -Kr * Kut) +
              Fe * (eK - KE) + Fbt * (btK - Kbt) + Fbz * (bzK - Kbz);
        rKb += S * (Fm + Fmn * SM + Fmt * vK);
        SMb += S * Fmn * rK;
        vKb += S * Fmt * rK;
        eKb += S * Fe;
        btKb += S * Fbt;
        bzKb += S * Fbz;
        kr = -S * (Fm + Fmn * Kun + Fmt * Kut);
        kun = -S * Fmn * Kr;
        kut = -S * Fmt * Kr;
        kE = -S * Fe;
        kbt = -S * Fbt;
        kbz = -S * Fbz;
    }
    // eK = eKn iK, eKn = K.E su + PTT SM - K.pT K.un + bn (wKf - sbK)
    const double iKb = eKb * eKn;
    {
        const double nb = eKb * iK;
        kE += nb * su;
        const double sub = nb * KE;
        PTTb += nb * SM;
        SMb += nb * PTT;
        kpT -= nb * Kun;
        kun -= nb * KpT;
        bnb += nb * (wKf - sbK);
        const double wKfb = nb * bn;
        sbKb -= nb * bn;
        // wKf = K.un K.bn + K.ut K.bt
        kun += wKfb * Kbn;
        kbn += wKfb * Kun;
        kut += wKfb * Kbt;
        kbt += wKfb * Kut;
        // su = S - K.un
        Sb += sub;
        kun -= sub;
    }
    // sbK = wK bzK + vK btK + SMbn
    wKb += sbKb * bzK;
    bzKb += sbKb * wK;
    vKb += sbKb * btK;
    btKb += sbKb * vK;
    SMbnb += sbKb;
    // distribute the K-selected adjoints
    if (takeL) {
        SLb += Sb; rLLb += rKb; vLLb += vKb; wLLb += wKb; btLb += btKb; bzLb += bzKb;
        iLb += iKb;
    } else {
        SRb += Sb; rRRb += rKb; vRRb += vKb; wRRb += wKb; btRb += btKb; bzRb += bzKb;
        iRb += iKb;
    }
    // SLL = SM - abn isLL ; SRR = SM + abn isRR  (if bnz, else = SM)
    double isLLb = 0, isRRb = 0;
    SMb += SLLb + SRRb;
    if (bnz) {
        const double abnb = fma(SRRb, isRR, -SLLb * isLL);
        isLLb = -SLLb * abn;
        isRRb = SRRb * abn;
        bnb += sgn_select(abnb, idbn);
    }
    // sLL = rLL isLL, isLL = rsqrt(rLL)  =>  d sLL / d rLL = 0.5 isLL
    rLLb += sLLb * 0.5 * isLL;
    rRRb += sRRb * 0.5 * isRR;
    rLLb += isLLb * (-0.5) * isLL * isLL * isLL;
    rRRb += isRRb * (-0.5) * isRR * isRR * isRR;
    // SMbn = SM bn
    SMb += SMbnb * bn;
    bnb += SMbnb * SM;
    // star states L
    double bbnb = 0;
    if (gL) {
        // vLL = A.ut - cL A.bt ; wLL = -cL A.bz ; btL = A.bt dL ; bzL = A.bz dL
        Ab.ut += vLLb;
        const double cLb = -vLLb * A.bt - wLLb * A.bz;
        Ab.bt += -vLLb * cL + btLb * dL;
        Ab.bz += -wLLb * cL + bzLb * dL;
        const double dLb = btLb * A.bt + bzLb * A.bz;
        // dL = (mL suL - bbn) itL ; cL = bn (SM - A.un) itL
        const double itLb = dLb * fma(mL, suL, -bbn) + cLb * bn * (SM - A.un);
        const double dnb = dLb * itL;
        double mLb_s = dnb * suL;
        double suLb_s = dnb * mL;
        bbnb -= dnb;
        const double cnb = cLb * itL;
        bnb += cnb * (SM - A.un);
        SMb += cnb * bn;
        Ab.un -= cnb * bn;
        // itL = 1 / ttL ; ttL = mL (SL - SM) - bbn
        const double ttLb = -itLb * itL * itL;
        mLb_s += ttLb * (SL - SM);
        SLb += ttLb * mL;
        SMb -= ttLb * mL;
        bbnb -= ttLb;
        // mL and suL adjoints
        Ab.r += mLb_s * suL;
        suLb_s += mLb_s * A.r;
        SLb += suLb_s;
        Ab.un -= suLb_s;
    } else {
        Ab.ut += vLLb;
    }
    if (gR) {
        Bb.ut += vRRb;
        const double cRb = -vRRb * B.bt - wRRb * B.bz;
        Bb.bt += -vRRb * cR + btRb * dR;
        Bb.bz += -wRRb * cR + bzRb * dR;
        const double dRb = btRb * B.bt + bzRb * B.bz;
        const double itRb = dRb * fma(mR, suR, -bbn) + cRb * bn * (SM - B.un);
        const double dnb = dRb * itR;
        double mRb_s = dnb * suR;
        double suRb_s = dnb * mR;
        bbnb -= dnb;
        const double cnb = cRb * itR;
        bnb += cnb * (SM - B.un);
        SMb += cnb * bn;
        Bb.un -= cnb * bn;
        const double ttRb = -itRb * itR * itR;
        mRb_s += ttRb * (SR - SM);
        SRb += ttRb * mR;
        SMb -= ttRb * mR;
        bbnb -= ttRb;
        Bb.r += mRb_s * suR;
        suRb_s += mRb_s * B.r;
        SRb += suRb_s;
        Bb.un -= suRb_s;
    } else {
        Bb.ut += vRRb;
    }
    // bbn = bn^2
    bnb += 2.0 * bbnb * bn;
    // rLL = mL iL ; rRR = mR iR ; iL = 1 / (SL - SM) ; iR = 1 / (SR - SM)
    double mLb = rLLb * iL, mRb = rRRb * iR;
    iLb += rLLb * mL;
    iRb += rRRb * mR;
    {
        const double dLb = -iLb * iL * iL;
        SLb += dLb;
        SMb -= dLb;
        const double dRb = -iRb * iR * iR;
        SRb += dRb;
        SMb -= dRb;
    }
    // bn = bnn iS (the star bt, bz of the HLLC-MHD branch are not used by HLLD)
    const double iSb = bnb * bnn;
    {
        const double nb = bnb * iS;  // bnn = SR B.bn - SL A.bn
        SRb += nb * B.bn;
        Bb.bn += nb * SR;
        SLb -= nb * A.bn;
        Ab.bn -= nb * SL;
    }
    // iS = 1 / (SR - SL)
    {
        const double db = -iSb * iS * iS;
        SRb += db;
        SLb -= db;
    }
    // UU = max(|SL|, |SR|)
    {
        const double Sx = UUR ? SR : SL;
        const double t = lt_zero(Sx) ? from_bits(bits(UUb) ^ (long long)0x8000000000000000ULL)
                                     : UUb;  // sign(Sx) UUb on the integer pipe
        add_to(UUR, SRb, SLb, t);
    }
    // PTT = PTTn iden ; SM = SMn iden
    const double idenb = PTTb * PTTn + SMb * SMn;
    {
        const double nb = PTTb * iden;  // PTTn = mL mR (B.un - A.un) + mR A.pT - mL B.pT
        mLb += nb * (mR * (B.un - A.un) - B.pT);
        mRb += nb * (mL * (B.un - A.un) + A.pT);
        Bb.un += nb * mL * mR;
        Ab.un -= nb * mL * mR;
        Ab.pT += nb * mR;
        Bb.pT -= nb * mL;
    }
    {
        const double nb = SMb * iden;  // SMn = mR B.un - mL A.un - B.pT + A.pT
        mRb += nb * B.un;
        Bb.un += nb * mR;
        mLb -= nb * A.un;
        Ab.un -= nb * mL;
        Bb.pT -= nb;
        Ab.pT += nb;
    }
    // iden = 1 / (mR - mL)
    {
        const double db = -idenb * iden * iden;
        mRb += db;
        mLb -= db;
    }
    // mL = A.r suL, mR = B.r suR ; suL = SL - A.un ; suR = SR - B.un
    Ab.r += mLb * suL;
    const double suLb = mLb * A.r;
    Bb.r += mRb * suR;
    const double suRb = mRb * B.r;
    SLb += suLb;
    Ab.un -= suLb;
    SRb += suRb;
    Bb.un -= suRb;
    // SL = uminN - cmax ; SR = umaxN + cmax
    const double cmaxb = SRb - SLb;
    if (minA) Ab.un += SLb; else Bb.un += SLb;
    if (maxB) Bb.un += SRb; else Ab.un += SRb;

    // ---- the K side's base flux and energy ----------------------------------------------
    {
        // F7 = un bz ; F6 = un bt - ut bn
        kun += Fbz * Kbz;
        kbz += Fbz * Kun;
        kun += Fbt * Kbt;
        kbt += Fbt * Kun;
        kut -= Fbt * Kbn;
        kbn -= Fbt * Kut;
        // F4 = (E + pT) un - bn (ut bt + un bn)
        const double w = fma(Kut, Kbt, Kun * Kbn);
        kE += Fe * Kun;
        kpT += Fe * Kun;
        kun += Fe * (KE + KpT);
        kbn -= Fe * w;
        const double wb = -Fe * Kbn;
        kut += wb * Kbt;
        kbt += wb * Kut;
        kun += wb * Kbn;
        kbn += wb * Kun;
        // F0 = r un ; F1 = F0 un + pT - bn^2 ; F2 = F0 ut - bn bt
        const double F0 = Kr * Kun;
        const double F0b = fma(Fmt, Kut, fma(Fmn, Kun, Fm));
        kut += Fmt * F0;
        kbn -= Fmt * Kbt;
        kbt -= Fmt * Kbn;
        kun += Fmn * F0;
        kpT += Fmn;
        kbn -= 2.0 * Fmn * Kbn;
        kr += F0b * Kun;
        kun += F0b * Kr;
        // E = p inv_gm1 + 0.5 (r (un^2 + ut^2) + bb)
        const double kinb = 0.5 * kE;
        kr += kinb * vsq;
        kun += kinb * 2.0 * Kr * Kun;
        kut += kinb * 2.0 * Kr * Kut;
        add_to(takeL, Ab.r, Bb.r, kr);
        add_to(takeL, Ab.un, Bb.un, kun);
        add_to(takeL, Ab.ut, Bb.ut, kut);
        add_to(takeL, Ab.bn, Bb.bn, kbn);
        add_to(takeL, Ab.bt, Bb.bt, kbt);
        add_to(takeL, Ab.bz, Bb.bz, kbz);
        add_to(takeL, Ab.pT, Bb.pT, kpT);
        // the side's p and bb adjoints are still zero: assign
        const double kp = kE * P.inv_gm1;
        Ab.p = takeL ? kp : 0.0;
        Bb.p = takeL ? 0.0 : kp;
        Ab.bb = takeL ? kinb : 0.0;
        Bb.bb = takeL ? 0.0 : kinb;
    }
    // ---- the fast speed of the side of max(cf) ------------------------------------------
    {
        const double Ccf = cfB ? B.cf : A.cf, Crs = cfB ? B.rs : A.rs;
        const double Crq = cfB ? B.rq : A.rq, Ca = cfB ? B.a : A.a, Cgp = cfB ? B.gp : A.gp;
        const double Cbn2 = cfB ? B.bn2 : A.bn2, Cdisc = cfB ? B.disc : A.disc;
        // cf = X rsqrt(X r) = sqrt(X / r): d/dX = 0.5 rs, d/dr = -0.5 cf / r = -0.5 cf^2 rs
        const double Xb = cmaxb * 0.5 * Crs;
        const double rb = -0.5 * cmaxb * (Ccf * Ccf) * Crs;
        // X = 0.5 (a + sq), sq = sqrt(disc), disc = a^2 - 4 gp bn2 (clamped at 0)
        double ab = 0.5 * Xb, gpb = 0.0, bn2b = 0.0;
        if ((bits(Cdisc) << 1) != 0) {
            const double discb = (0.5 * Xb) * 0.5 * Crq;
            ab = fma(discb * 2.0, Ca, ab);
            gpb = -discb * 4.0 * Cbn2;
            bn2b = -discb * 4.0 * Cgp;
        }
        gpb += ab;  // a = gp + bb
        add_to(!cfB, Ab.r, Bb.r, rb);
        add_to(!cfB, Ab.p, Bb.p, gpb * P.gamma);
        add_to(!cfB, Ab.bb, Bb.bb, ab);
        Ab.bn2 = cfB ? 0.0 : bn2b;
        Bb.bn2 = cfB ? bn2b : 0.0;
    }
    side_tail(A, Ab, qa_b);
    side_tail(B, Bb, qb_b);
}

// ---------------------------------------------------------------------------------------
// Pass B: face adjoints (each face once), then the gather into cells.
//
// B1 adj_face_kernel: one thread per face.  It reconstructs the face's two states from the
// four cells along its normal, recomputes the HLLD flux and runs its reverse sweep on
// Fbar = k (dbar_low - dbar_high).  The adjoint of the low-side state (the upper face state
// of the low cell) goes to that cell's "up" plane, the adjoint of the high-side state (the
// lower face state of the high cell) to that cell's "dn" plane: every entry has exactly one
// writer.  The face thread also records, before its reverse sweep, the reconstruction
// choices of its two cells in bytes: for the low cell the minmod choice of its slope and
// whether its upper face state fell back to the cell value (rho, p), for the high cell
// whether its lower face state fell back (a fallback face state does not depend on the slope).
// Scratch layout after the 15 pass-A planes:
//   kFaceAdj + (dir * 2 + side) * 7 + f         face-state adjoints, side 0 = up, 1 = dn
//   kSel bytes, (dir * 7 + f) * K + cell        (choice + 1) | upper fallback << 2,
//                                               choice -1 left, +1 right, 0 none
//   kSel bytes, 14 K + (dir * 2 + f) * K + cell lower fallback (f < 2)
// dir 0 = x, 1 = y.
// B2 adj_gather_kernel: one thread per cell.  The cell's state adjoint collects the value
// parts of its two face states per direction, its own slope adjoint through its minmod
// choice, its neighbours' slope adjoints where their minmod choice used it, and the Powell
// terms of its neighbours, in a fixed order (deterministic).
// ---------------------------------------------------------------------------------------
constexpr int kFaceAdj = 15;
constexpr int kSel = kFaceAdj + 4 * NF;
constexpr int kScratchPlanes = kSel + 3;  // 18 bytes per cell fit in three planes of doubles
constexpr int FBX = 32, FBY = 4;  // 128-thread blocks of both kernels

// periodic index for any i
__device__ __forceinline__ int wrap(int i, int n) {
    const int r = i % n;
    return r < 0 ? r + n : r;
}

// state value in b units (the field is stored in Gaussian units).  The product is rounded
// on its own (__dmul_rn: never fused into a later add), as the forward kernel rounds it when
// it stages the tile: equal neighbours then give an exact zero difference, and the minmod
// choices here are the forward's.
__device__ __forceinline__ double ld_b(const CPlanes& U, int f, long long k) {
    const double v = __ldg(U.f[f] + k);
    return f >= 4 ? __dmul_rn(v, kInvSpi4) : v;
}

// minmod slope and which difference it took: +1 right (c_{+1} - c), -1 left (c - c_{-1}), 0
__device__ __forceinline__ double slope_sel(double cm, double c, double cp, int& sel) {
    const double l = c - cm, r = cp - c;
    const double s = minmod(l, r);
    sel = mag(s) == 0 ? 0 : (mag_lt(r, l) ? 1 : -1);
    return s;
}

__global__ void __launch_bounds__(FBX * FBY) adj_face_kernel(Params P, CPlanes U, double* scratch,
                                                             const double* __restrict__ T_do_ptr) {
    const int N = P.N, M = P.M;
    const long long K = (long long)N * M;
    const bool isx = blockIdx.z == 0;
    const int ix = blockIdx.x * FBX + threadIdx.x;  // x-face index (x) or column (y)
    const int iy = blockIdx.y * FBY + threadIdx.y;  // row (x) or y-face index (y)
    if (ix >= N || iy >= M) return;
    const double T_do = *T_do_ptr;
    const double kk = T_do * (isx ? P.inv_dx : P.inv_dy);  // the forward's scaling
    // the face lies between cells a-1 and a along its normal; cells a-2 .. a+1
    long long kc[4];
#pragma unroll
    for (int t = 0; t < 4; ++t)
        kc[t] = isx ? (long long)iy * N + wrap(ix - 2 + t, N)
                    : (long long)wrap(iy - 2 + t, M) * N + ix;
    double c[4][NF];
#pragma unroll
    for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int f = 0; f < NF; ++f) c[t][f] = ld_b(U, f, kc[t]);
    // face states: low cell (t=1) + its slope / 2, high cell (t=2) - its slope / 2
    double qa[NF], qb[NF];
    unsigned char* rec = reinterpret_cast<unsigned char*>(scratch + (size_t)kSel * K);
    unsigned char* sel = rec + (size_t)(isx ? 0 : NF) * K;
    unsigned char* fbl = rec + (size_t)(2 * NF + (isx ? 0 : 2)) * K;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        int sa, sb_;
        const double da = slope_sel(c[0][f], c[1][f], c[2][f], sa);
        const double db = slope_sel(c[1][f], c[2][f], c[3][f], sb_);
        const double va = fma(0.5, da, c[1][f]), vb = fma(-0.5, db, c[2][f]);
        const bool fu = f < 2 && le_zero(va), fd = f < 2 && le_zero(vb);
        qa[f] = fu ? c[1][f] : va;
        qb[f] = fd ? c[2][f] : vb;
        sel[(size_t)f * K + kc[1]] = (unsigned char)((sa + 1) | (fu ? 4 : 0));  // low cell
        if (f < 2) fbl[(size_t)f * K + kc[2]] = fd ? 1 : 0;                   // high cell
    }
    // flux adjoint: d_low += k F, d_high -= k F
    double Fslot[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f)
        Fslot[f] = kk * (scratch[(size_t)(7 + f) * K + kc[1]] - scratch[(size_t)(7 + f) * K + kc[2]]);
    // slots: 0 m, 1 e, 2 mx, 3 my, 4 bx, 5 by, 6 bz -> local (m, mn, mt, e, bn, bt, bz)
    const double Fb[7] = {Fslot[0], isx ? Fslot[2] : Fslot[3], isx ? Fslot[3] : Fslot[2],
                          Fslot[1], isx ? Fslot[4] : Fslot[5], isx ? Fslot[5] : Fslot[4],
                          Fslot[6]};
    const double la[7] = {qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2],
                          isx ? qa[4] : qa[5], isx ? qa[5] : qa[4], qa[6]};
    const double lb[7] = {qb[0], qb[1], isx ? qb[2] : qb[3], isx ? qb[3] : qb[2],
                          isx ? qb[4] : qb[5], isx ? qb[5] : qb[4], qb[6]};
    double lab[7], lbb[7];
    hlld_vjp(la, lb, Fb, P, lab, lbb);
    // back to field order (rho, p, vx, vy, bx, by, bz)
    const double gab[7] = {lab[0], lab[1], isx ? lab[2] : lab[3], isx ? lab[3] : lab[2],
                           isx ? lab[4] : lab[5], isx ? lab[5] : lab[4], lab[6]};
    const double gbb[7] = {lbb[0], lbb[1], isx ? lbb[2] : lbb[3], isx ? lbb[3] : lbb[2],
                           isx ? lbb[4] : lbb[5], isx ? lbb[5] : lbb[4], lbb[6]};
    double* up = scratch + (size_t)(kFaceAdj + (isx ? 0 : 2) * NF) * K;
    double* dn = up + (size_t)NF * K;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        up[(size_t)f * K + kc[1]] = gab[f];
        dn[(size_t)f * K + kc[2]] = gbb[f];
    }
}

__global__ void __launch_bounds__(FBX * FBY) adj_gather_kernel(Params P,
                                                               const double* __restrict__ scratch,
                                                               Planes lam_in,
                                                               const double* __restrict__ T_do_ptr) {
    const int N = P.N, M = P.M;
    const long long K = (long long)N * M;
    const int gx = blockIdx.x * FBX + threadIdx.x, gy = blockIdx.y * FBY + threadIdx.y;
    if (gx >= N || gy >= M) return;
    const long long k = (long long)gy * N + gx;
    const double T_do = *T_do_ptr;
    const double kx = T_do * P.inv_dx, ky = T_do * P.inv_dy;
    double lam[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) lam[f] = scratch[(size_t)f * K + k];
    const unsigned char* rec = reinterpret_cast<const unsigned char*>(scratch + (size_t)kSel * K);
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const bool isx = dir == 0;
        // the cells at positions -1, 0, +1 along the direction
        long long kc[3];
#pragma unroll
        for (int t = 0; t < 3; ++t)
            kc[t] = isx ? (long long)gy * N + wrap(gx - 1 + t, N)
                        : (long long)wrap(gy - 1 + t, M) * N + gx;
        const double* up = scratch + (size_t)(kFaceAdj + 2 * dir * NF) * K;
        const double* dn = up + (size_t)NF * K;
        const unsigned char* sel = rec + (size_t)dir * NF * K;
        const unsigned char* fbl = rec + (size_t)(2 * NF + 2 * dir) * K;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const double* upf = up + (size_t)f * K;
            const double* dnf = dn + (size_t)f * K;
            // twice the slope adjoint of cell t: up - dn of that cell, a fallback face state
            // dropping its term; 0.5 a - 0.5 b rounds as 0.5 (a - b) (scaling by 2^-1 is
            // exact), so the factor goes last
            double sb2[3];
            int s[3];
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const int b = sel[(size_t)f * K + kc[t]];
                s[t] = (b & 3) - 1;
                const bool fu = (b & 4) != 0;
                const bool fd = f < 2 && fbl[(size_t)f * K + kc[t]] != 0;
                sb2[t] = (fu ? 0.0 : upf[kc[t]]) - (fd ? 0.0 : dnf[kc[t]]);
            }
            // value parts of the cell's two face states
            double acc = upf[k] + dnf[k];
            // own slope: left difference (c - c_{-1}) -> +1, right (c_{+1} - c) -> -1
            if (s[1] != 0) acc = fma(s[1] == -1 ? 0.5 : -0.5, sb2[1], acc);
            // neighbour -1 took its right difference (c - c_{-1})
            if (s[0] == 1) acc = fma(0.5, sb2[0], acc);
            // neighbour +1 took its left difference (c_{+1} - c)
            if (s[2] == -1) acc = fma(-0.5, sb2[2], acc);
            lam[f] += acc;
        }
    }
    // Powell: divb_c' = 0.5 kx (bx_{c'+1} - bx_{c'-1}) + 0.5 ky (by_{c'+N} - by_{c'-N})
    {
        const long long kW = (long long)gy * N + wrap(gx - 1, N);
        const long long kE = (long long)gy * N + wrap(gx + 1, N);
        const long long kS = (long long)wrap(gy - 1, M) * N + gx;
        const long long kN = (long long)wrap(gy + 1, M) * N + gx;
        const double* dvb = scratch + (size_t)14 * K;
        lam[4] += 0.5 * kx * (dvb[kW] - dvb[kE]);
        lam[5] += 0.5 * ky * (dvb[kS] - dvb[kN]);
    }
    // field adjoint back to the stored Gaussian units: b = B / sqrt(4 pi)
    lam[4] *= kInvSpi4;
    lam[5] *= kInvSpi4;
    lam[6] *= kInvSpi4;
#pragma unroll
    for (int f = 0; f < NF; ++f) lam_in.f[f][k] = lam[f];
}

int grid_cells(long long K) {
    long long g = (K + NT - 1) / NT;
    return (int)(g > 152 * 16 ? 152 * 16 : (g < 1 ? 1 : g));
}

// ---------------------------------------------------------------------------------------
// Branch switches between two runs (gd_adj_switches).  A central difference of runs from
// U0 + eps v and U0 - eps v is the derivative of the branch both take only where every
// non-smooth choice comes out the same in both.  Per face, the choices its flux depends on,
// computed with the forward's own operations (as adj_face_kernel repeats them): the minmod
// pick of its low cell's slope (every cell's slope is counted at exactly one face per
// direction), the rho / p fallbacks of its two face states, and the HLLD choices: which
// side gives min(u), max(u), max(cf) and max(|S|) (speeds), the upwind side and the region
// of the fan (region), and the guards disc <= 0, |tt| >= 1e-5 on both sides, |bn| > 1e-6
// and sign(bn) (guards).  Per cell, the update's floors rho <= 0 and p <= 0.  Counters
// (kSw*): (step, face) pairs per face category, (step, cell) pairs for floors and for
// cells touched by any switch, and, at the end, the cells switched at any step.
// ---------------------------------------------------------------------------------------
struct FaceCode {
    unsigned int minmod, fallback, speeds, region, guards;
};

__device__ __forceinline__ FaceCode face_code(const Params& P, const CPlanes& U, bool isx,
                                              const long long* kc) {
    FaceCode code{0u, 0u, 0u, 0u, 0u};
    double c[4][NF];
#pragma unroll
    for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int f = 0; f < NF; ++f) c[t][f] = ld_b(U, f, kc[t]);
    double qa[NF], qb[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        int sa, sb_;
        const double da = slope_sel(c[0][f], c[1][f], c[2][f], sa);
        const double db = slope_sel(c[1][f], c[2][f], c[3][f], sb_);
        const double va = fma(0.5, da, c[1][f]), vb = fma(-0.5, db, c[2][f]);
        const bool fu = f < 2 && le_zero(va), fd = f < 2 && le_zero(vb);
        qa[f] = fu ? c[1][f] : va;
        qb[f] = fd ? c[2][f] : vb;
        code.minmod |= (unsigned int)(sa + 1) << (2 * f);
        if (f < 2) code.fallback |= (fu ? 1u : 0u) << (2 * f) | (fd ? 2u : 0u) << (2 * f);
    }
    const double la[7] = {qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2],
                          isx ? qa[4] : qa[5], isx ? qa[5] : qa[4], qa[6]};
    const double lb[7] = {qb[0], qb[1], isx ? qb[2] : qb[3], isx ? qb[3] : qb[2],
                          isx ? qb[4] : qb[5], isx ? qb[5] : qb[4], qb[6]};
    SideV A, B;
    side_fwd(A, la, P);
    side_fwd(B, lb, P);
    // the forward part of hlld_vjp up to the region, operation for operation
    const bool minA = !dlt(B.un, A.un);
    const bool maxB = dlt(A.un, B.un);
    const double uminN = minA ? A.un : B.un;
    const double umaxN = maxB ? B.un : A.un;
    const bool cfB = mag_lt(A.cf, B.cf);
    const double cmax = cfB ? B.cf : A.cf;
    const double SL = uminN - cmax, SR = umaxN + cmax;
    const double suL = SL - A.un, suR = SR - B.un;
    const double mL = A.r * suL, mR = B.r * suR;
    const double iden = rcp_fast(mR - mL);
    const double SM = ((fma(mR, B.un, -mL * A.un) - B.pT) + A.pT) * iden;
    const bool UUR = mag_lt(SL, SR);
    const double iS = rcp_fast(SR - SL);
    const double bn = fma(SR, B.bn, -SL * A.bn) * iS;
    const double iL = rcp_fast(SL - SM), iR = rcp_fast(SR - SM);
    const double rLL = mL * iL, rRR = mR * iR;
    const double bbn = bn * bn;
    const double ttL = fma(mL, SL - SM, -bbn);
    const bool gL = mag_ge(ttL, kMag1em5);
    const double ttR = fma(mR, SR - SM, -bbn);
    const bool gR = mag_ge(ttR, kMag1em5);
    double isLL, isRR, sLL, sRR;
    rsqrt_and_sqrt(rLL, isLL, sLL);
    rsqrt_and_sqrt(rRR, isRR, sRR);
    const bool bnz = mag_ge(bn, kMag1em6 + 1);
    const double abn = dabs(bn);
    const double SLL = bnz ? fma(-abn, isLL, SM) : SM;
    const double SRR = bnz ? fma(abn, isRR, SM) : SM;
    const bool takeL = ge_zero(SL) || ge_zero(SM);
    int level;
    if (takeL) level = ge_zero(SL) ? 0 : (ge_zero(SLL) ? 1 : 2);
    else level = gt_zero(SRR) ? 2 : (gt_zero(SR) ? 1 : 0);
    code.speeds = (minA ? 1u : 0u) | (maxB ? 2u : 0u) | (cfB ? 4u : 0u) | (UUR ? 8u : 0u);
    code.region = (takeL ? 1u : 0u) | ((unsigned int)level << 1);
    code.guards = (A.disc0 ? 1u : 0u) | (B.disc0 ? 2u : 0u) | (gL ? 4u : 0u) | (gR ? 8u : 0u) |
                  (bnz ? 16u : 0u) | (bnz && lt_zero(bn) ? 32u : 0u);
    return code;
}

// warp-aggregated counter increment: one atomic per warp and kind
__device__ __forceinline__ void count_if(unsigned long long* ctr, bool hit) {
    const unsigned int m = __ballot_sync(0xffffffffu, hit);
    if (m != 0u && (threadIdx.x & 31) == (unsigned)(__ffs((int)m) - 1))
        atomicAdd(ctr, (unsigned long long)__popc(m));
}

__global__ void __launch_bounds__(FBX * FBY) switch_face_kernel(Params P, CPlanes Ua, CPlanes Ub,
                                                                unsigned long long* ctr,
                                                                unsigned char* step_mark) {
    const int N = P.N, M = P.M;
    const bool isx = blockIdx.z == 0;
    const int ix = blockIdx.x * FBX + threadIdx.x;
    const int iy = blockIdx.y * FBY + threadIdx.y;
    const bool in = ix < N && iy < M;
    FaceCode a{0u, 0u, 0u, 0u, 0u}, b{0u, 0u, 0u, 0u, 0u};
    long long kc[4] = {0, 0, 0, 0};
    if (in) {
#pragma unroll
        for (int t = 0; t < 4; ++t)
            kc[t] = isx ? (long long)iy * N + wrap(ix - 2 + t, N)
                        : (long long)wrap(iy - 2 + t, M) * N + ix;
        a = face_code(P, Ua, isx, kc);
        b = face_code(P, Ub, isx, kc);
    }
    const bool sm = a.minmod != b.minmod, sf = a.fallback != b.fallback;
    const bool ss = a.speeds != b.speeds, sr = a.region != b.region, sg = a.guards != b.guards;
    // counted per warp: threadIdx is 32 x 4, so each warp is one threadIdx.y row
    count_if(ctr + 0, sm);
    count_if(ctr + 1, sf);
    count_if(ctr + 2, ss);
    count_if(ctr + 3, sr);
    count_if(ctr + 4, sg);
    if (sm || sf || ss || sr || sg) {
        // the slope of the low cell, both face states and the flux between them
        step_mark[kc[1]] = 1;
        step_mark[kc[2]] = 1;
    }
}

// Floors of the update of U (with the forward's flux differences and Powell term aux), as
// adj_update_kernel recomputes them: bit 0 rho <= 0, bit 1 p <= 0.
__device__ __forceinline__ unsigned int floor_code(const Params& P, const CPlanes& U,
                                                   const double* aux, long long K, long long k) {
    const double r = U.f[0][k], p = U.f[1][k], u = U.f[2][k], v = U.f[3][k];
    const double bx = __dmul_rn(U.f[4][k], kInvSpi4), by = __dmul_rn(U.f[5][k], kInvSpi4);
    const double bz = __dmul_rn(U.f[6][k], kInvSpi4);
    double d[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) d[f] = aux[(size_t)f * K + k];
    const double divb = aux[(size_t)7 * K + k];
    const double ub = fma(u, bx, v * by);
    const double bb = fma(bz, bz, fma(by, by, bx * bx));
    const double E = fma(p, P.inv_gm1, 0.5 * fma(r, fma(u, u, v * v), bb));
    double r2 = r - d[0];
    const bool rfl = le_zero(r2);
    if (rfl) r2 = r;
    const double mx2 = fma(r, u, -fma(bx, divb, d[2]));
    const double my2 = fma(r, v, -fma(by, divb, d[3]));
    const double bx2 = bx - fma(u, divb, d[4]);
    const double by2 = by - fma(v, divb, d[5]);
    const double bz2 = bz - d[6];
    const double E2 = E - fma(ub, divb, d[1]);
    const double inv = rcp_fast(r2);
    const double u2 = mx2 * inv, v2 = my2 * inv;
    const double p2 = (E2 - 0.5 * fma(r2, fma(u2, u2, v2 * v2),
                                      fma(bz2, bz2, fma(by2, by2, bx2 * bx2)))) * P.gm1;
    return (rfl ? 1u : 0u) | (le_zero(p2) ? 2u : 0u);
}

__global__ void __launch_bounds__(NT) switch_cell_kernel(Params P, CPlanes Ua, const double* auxa,
                                                         CPlanes Ub, const double* auxb,
                                                         unsigned long long* ctr,
                                                         unsigned char* step_mark,
                                                         unsigned char* ever_mark) {
    const long long K = (long long)P.N * P.M;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long K_up = (K + 31) / 32 * 32;  // whole warps through the loop (ballots)
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K_up; k += stride) {
        bool fl = false, any = false;
        if (k < K) {
            fl = floor_code(P, Ua, auxa, K, k) != floor_code(P, Ub, auxb, K, k);
            any = fl || step_mark[k] != 0;
            if (any) {
                ever_mark[k] = 1;
                step_mark[k] = 0;
            }
        }
        count_if(ctr + 5, fl);
        count_if(ctr + 6, any);
    }
}

__global__ void __launch_bounds__(NT) switch_total_kernel(long long K,
                                                          const unsigned char* ever_mark,
                                                          unsigned long long* ctr) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long K_up = (K + 31) / 32 * 32;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K_up; k += stride)
        count_if(ctr + 7, k < K && ever_mark[k] != 0);
}

}  // namespace

int switch_kinds() { return 8; }

cudaError_t launch_switch_faces(const Params& P, const CPlanes& Ua, const CPlanes& Ub,
                                unsigned long long* ctr, unsigned char* step_mark,
                                cudaStream_t st) {
    const unsigned gxb = (unsigned)((P.N + FBX - 1) / FBX), gyb = (unsigned)((P.M + FBY - 1) / FBY);
    if (gyb > 65535u) return cudaErrorInvalidConfiguration;
    switch_face_kernel<<<dim3(gxb, gyb, 2), dim3(FBX, FBY), 0, st>>>(P, Ua, Ub, ctr, step_mark);
    return cudaGetLastError();
}

cudaError_t launch_switch_cells(const Params& P, const CPlanes& Ua, const double* auxa,
                                const CPlanes& Ub, const double* auxb, unsigned long long* ctr,
                                unsigned char* step_mark, unsigned char* ever_mark,
                                cudaStream_t st) {
    const long long K = (long long)P.N * P.M;
    switch_cell_kernel<<<grid_cells(K), NT, 0, st>>>(P, Ua, auxa, Ub, auxb, ctr, step_mark,
                                                     ever_mark);
    return cudaGetLastError();
}

cudaError_t launch_switch_total(long long K, const unsigned char* ever_mark,
                                unsigned long long* ctr, cudaStream_t st) {
    switch_total_kernel<<<grid_cells(K), NT, 0, st>>>(K, ever_mark, ctr);
    return cudaGetLastError();
}

int adjoint_scratch_planes() { return kScratchPlanes; }

cudaError_t prepare_adjoint() { return cudaSuccess; }

cudaError_t launch_adjoint_step(const Params& P, const CPlanes& U, const double* aux,
                                const CPlanes& lam_out, const Planes& lam_in, double* scratch,
                                const double* T_do, cudaStream_t st) {
    const long long K = (long long)P.N * P.M;
    const dim3 blk(FBX, FBY);
    const unsigned gxb = (unsigned)((P.N + FBX - 1) / FBX), gyb = (unsigned)((P.M + FBY - 1) / FBY);
    if (gyb > 65535u) return cudaErrorInvalidConfiguration;
    adj_update_kernel<<<grid_cells(K), NT, 0, st>>>(P, U, aux, lam_out, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    adj_face_kernel<<<dim3(gxb, gyb, 2), blk, 0, st>>>(P, U, scratch, T_do);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    adj_gather_kernel<<<dim3(gxb, gyb, 1), blk, 0, st>>>(P, scratch, lam_in, T_do);
    return cudaGetLastError();
}

}  // namespace gd
