// gd_adjoint_euler.cu -- hand-written discrete adjoint (reverse mode, VJP) of the fast Euler
// step, the counterpart of gd_adjoint.cu for the tile of gd_fast_euler.cu.
//
// The step U' = S(U; dt) (HLLC, minmod TVD, Cartesian, periodic) is differentiated with dt
// held fixed and every non-smooth choice (minmod selection, the Davis wave-speed min / max,
// the side and star-region selection, the rho / p face fallback, the floors) frozen at the
// branch the forward values take.  Given lambda' = dL/dU', one reverse step returns
// lambda = dL/dU in the three passes of the MHD adjoint:
//
//   A  per cell (eadj_update_kernel): the transpose of the cell update.  Inputs: U, the
//      forward flux differences d[4] of that cell (stored by the recording), lambda'.
//      Outputs: the direct adjoint of the cell state and the adjoint of d[4].
//   B1 per face (eadj_face_kernel): the face recomputes its two reconstructed states and its
//      HLLC flux (hllc_local of gd_fast_euler.cu, operation for operation) and runs the
//      flux's reverse sweep on Fbar = k (dbar_low - dbar_high); the two face-state adjoints
//      go to one writer each, with the reconstruction choices of both cells as bytes.
//   B2 per cell (eadj_gather_kernel): the cell's adjoint collects its face states' value
//      parts, its own slope through its minmod choice and its neighbours' slopes where their
//      choice used it, in a fixed order (deterministic).
#include "gd_internal.cuh"
#include "gd_kernels.h"

namespace gd {
namespace {

constexpr int NF = 4;
constexpr int NT = 256;

// ---------------------------------------------------------------------------------------
// Pass A: transpose of the cell update.  aux per cell: d[0..3] (slot order m, e, mx, my).
// Scratch per cell: qbar[0..3] (rho, p, vx, vy), dbar[0..3] (slot order).
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NT) eadj_update_kernel(Params P, CPlanes U, const double* aux,
                                                         CPlanes lam_out, double* scratch) {
    const long long K = (long long)P.N * P.M;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < K;
         k += (long long)gridDim.x * blockDim.x) {
        const double r = U.f[0][k], p = U.f[1][k], u = U.f[2][k], v = U.f[3][k];
        double d[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) d[f] = aux[(size_t)f * K + k];
        // forward, the same operations as the tile update
        double r2 = r - d[0];
        const bool rfl = le_zero(r2);
        if (rfl) r2 = 0.0001;
        const double inv = rcp_2op(r2);
        const double mx2 = fma(r, u, -d[2]), my2 = fma(r, v, -d[3]);
        const double u2 = imul(mx2, inv), v2 = imul(my2, inv);
        const double w = fma(u, u, imul(v, v));
        const double K1 = r * w;
        const double K2 = fma(mx2, u2, imul(my2, v2));
        const double p2 = fma(P.hgm1, K1 - K2, fma(-P.gm1, d[1], p));
        const bool pfl = le_zero(p2);
        // reverse; a floored value is a constant
        double r2b = lam_out.f[0][k], u2b = lam_out.f[2][k], v2b = lam_out.f[3][k];
        const double p2b = lam_out.f[1][k];
        double db[NF] = {0, 0, 0, 0};
        double rb = 0.0, pb = 0.0, ub = 0.0, vb = 0.0, mx2b = 0.0, my2b = 0.0;
        if (!pfl) {
            // p2 = p - gm1 d1 + hgm1 (K1 - K2), K1 = r (u^2 + v^2), K2 = mx2 u2 + my2 v2
            pb = p2b;
            db[1] = -p2b * P.gm1;
            const double Kb = p2b * P.hgm1;
            rb = Kb * w;
            ub = 2.0 * Kb * r * u;
            vb = 2.0 * Kb * r * v;
            mx2b = -Kb * u2;
            my2b = -Kb * v2;
            u2b -= Kb * mx2;
            v2b -= Kb * my2;
        }
        // u2 = mx2 / r2, v2 = my2 / r2
        mx2b += u2b * inv;
        my2b += v2b * inv;
        const double invb = u2b * mx2 + v2b * my2;
        r2b -= invb * inv * inv;
        if (!rfl) {
            rb += r2b;
            db[0] = -r2b;
        }
        // mx2 = r u - d2, my2 = r v - d3
        rb += mx2b * u + my2b * v;
        ub += mx2b * r;
        vb += my2b * r;
        db[2] = -mx2b;
        db[3] = -my2b;
        double* s = scratch;
        s[0 * K + k] = rb;
        s[1 * K + k] = pb;
        s[2 * K + k] = ub;
        s[3 * K + k] = vb;
#pragma unroll
        for (int f = 0; f < NF; ++f) s[(size_t)(4 + f) * K + k] = db[f];
    }
}

// ---------------------------------------------------------------------------------------
// Reverse sweep of one HLLC face flux in the local frame.  Inputs: the face states a (low)
// and b (high) as (r, p, un, ut) and the flux adjoint (m, mn, mt, e).  Writes the adjoints of
// a and b to ab, bb.  The forward part repeats hllc_local of gd_fast_euler.cu operation for
// operation (products on the integer pipes where it has them there: the same bits).
//   Nm = mR unR - mL unL + pL - pR, D = mR - mL, m = rho (S - un); K the side that gives
//   the flux.  Star: X = S D - Nm, R = 1 / (D X), S_M = Nm R X (= Nm / D), q = Nm R D
//   (= Nm / X), F.m = r qs with qs = q su, F.mn = F.m S_M + p*, p* = mm (S_M - un) + p,
//   F.mt = F.m ut, F.e = qs (p G + r (|v|^2 / 2 + S (S_M - un))).  Otherwise F.m = r un,
//   F.mn = F.m un + p, F.mt = F.m ut, F.e = un (p G + r |v|^2 / 2).  G = gamma / (gamma - 1).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void hllc_vjp(const double* a, const double* b, const double* Fb,
                                         const Params& P, double* ab, double* bb) {
    const double g = P.gamma, G = P.g_gm1;
    const double rL = a[0], pL = a[1], unL = a[2], utL = a[3];
    const double rR = b[0], pR = b[1], unR = b[2], utR = b[3];
    // ---- forward
    const double gpL = imul(g, pL), gpR = imul(g, pR);
    double cL, cR, rsL, rsR;  // sqrt_over(g p, rho) of the forward and 1/sqrt(g p rho)
    cL = sqrt_over_2op(gpL, rL, &rsL);
    cR = sqrt_over_2op(gpR, rR, &rsR);
    const double aL = unL - cL, aR = unR - cR;
    const double bL = unL + cL, bR = unR + cR;
    const bool slR = dlt(aR, aL);  // SL = dmin(aL, aR)
    const bool srR = dlt(bL, bR);  // SR = dmax(bL, bR)
    const double SL = slR ? aR : aL, SR = srR ? bR : bL;
    const double suL = SL - unL, suR = SR - unR;
    const double mL = imul(rL, suL), mR = imul(rR, suR);
    const double Nm = fma(mR, unR, fma(-mL, unL, pL - pR));
    const double D = mR - mL;
    const bool takeL = gt_zero(SL) || !quotient_neg(Nm, D);
    const double r = takeL ? rL : rR, p = takeL ? pL : pR;
    const double un = takeL ? unL : unR, ut = takeL ? utL : utR;
    const double S = takeL ? SL : SR, su = takeL ? suL : suR, mm = takeL ? mL : mR;
    const bool star = takeL ? !gt_zero(SL) : ge_zero(SR);
    const double V2 = fma(un, un, imul(ut, ut));
    // ---- reverse
    const double Fmb = Fb[0], Fmnb = Fb[1], Fmtb = Fb[2], Feb = Fb[3];
    double rb, pb, unb, utb, V2b, Sb = 0.0, sub = 0.0, mmb = 0.0, Nmb = 0.0, Db = 0.0;
    if (star) {
        const double X = fma(S, D, -Nm);
        const double R = rcp_2op(imul(D, X));
        const double NR = imul(Nm, R);
        const double SM = imul(NR, X);
        const double q = imul(NR, D);
        const double SMu = SM - un;
        const double qs = imul(q, su);
        const double Fm = imul(r, qs);
        const double t2 = fma(0.5, V2, imul(S, SMu));
        const double inner = fma(p, G, imul(r, t2));
        // F.e = qs inner, inner = p G + r t2, t2 = V2 / 2 + S SMu
        double qsb = imul(Feb, inner);
        const double innerb = imul(Feb, qs);
        pb = imul(innerb, G);
        rb = imul(innerb, t2);
        const double t2b = imul(innerb, r);
        V2b = imul(0.5, t2b);
        Sb = imul(t2b, SMu);
        double SMub = imul(t2b, S);
        // F.m = r qs, with all of F.m's adjoint (F.mn = F.m SM + p*, F.mt = F.m ut)
        const double Fmbt = fma(Fmnb, SM, fma(Fmtb, ut, Fmb));
        rb = fma(Fmbt, qs, rb);
        qsb = fma(Fmbt, r, qsb);
        utb = imul(Fmtb, Fm);
        double SMb = imul(Fmnb, Fm);
        // qs = q su
        const double qb = imul(qsb, su);
        sub = imul(qsb, q);
        // p* = mm SMu + p (its adjoint is Fmnb)
        mmb = imul(Fmnb, SMu);
        SMub = fma(Fmnb, mm, SMub);
        pb += Fmnb;
        // SMu = SM - un
        SMb += SMub;
        unb = -SMub;
        // q = Nm / X, SM = Nm / D, X = S D - Nm, with 1 / X = D R and 1 / D = X R
        const double DR = imul(D, R), XR = imul(X, R);
        const double Xb = -imul(imul(qb, q), DR);
        Nmb = fma(qb, DR, imul(SMb, XR)) - Xb;
        Db = fma(Xb, S, -imul(imul(SMb, SM), XR));
        Sb = fma(Xb, D, Sb);
    } else {
        // F.e = un H, H = p G + hr V2 with hr = r / 2
        const double hr = imul(0.5, r);
        const double H = fma(p, G, imul(hr, V2));
        const double Fm = imul(r, un);
        const double Hb = imul(Feb, un);
        const double Fm0b = fma(Fmnb, un, fma(Fmtb, ut, Fmb));  // all of F.m's adjoint
        unb = fma(Feb, H, fma(Fm0b, r, imul(Fmnb, Fm)));
        pb = fma(Hb, G, Fmnb);
        rb = fma(imul(0.5, Hb), V2, imul(Fm0b, un));
        V2b = imul(Hb, hr);
        utb = imul(Fmtb, Fm);
    }
    // V2 = un^2 + ut^2
    const double V2b2 = V2b + V2b;
    unb = fma(V2b2, un, unb);
    utb = fma(V2b2, ut, utb);
    // the K side's adjoints to its side
    double rLb = 0, pLb = 0, unLb = 0, utLb = 0, rRb = 0, pRb = 0, unRb = 0, utRb = 0;
    double SLb = 0, SRb = 0, suLb = 0, suRb = 0, mLb = 0, mRb = 0;
    if (takeL) {
        rLb = rb; pLb = pb; unLb = unb; utLb = utb; SLb = Sb; suLb = sub; mLb = mmb;
    } else {
        rRb = rb; pRb = pb; unRb = unb; utRb = utb; SRb = Sb; suRb = sub; mRb = mmb;
    }
    // Nm = mR unR - mL unL + pL - pR, D = mR - mL
    mRb = fma(Nmb, unR, mRb + Db);
    unRb = fma(Nmb, mR, unRb);
    mLb = fma(-Nmb, unL, mLb - Db);
    unLb = fma(-Nmb, mL, unLb);
    pLb += Nmb;
    pRb -= Nmb;
    // mL = rL suL, mR = rR suR; suL = SL - unL, suR = SR - unR
    rLb = fma(mLb, suL, rLb);
    suLb = fma(mLb, rL, suLb);
    rRb = fma(mRb, suR, rRb);
    suRb = fma(mRb, rR, suRb);
    SLb += suLb;
    unLb -= suLb;
    SRb += suRb;
    unRb -= suRb;
    // SL = min(unL - cL, unR - cR), SR = max(unL + cL, unR + cR)
    double cLb = 0.0, cRb = 0.0;
    if (slR) { unRb += SLb; cRb -= SLb; } else { unLb += SLb; cLb -= SLb; }
    if (srR) { unRb += SRb; cRb += SRb; } else { unLb += SRb; cLb += SRb; }
    // c = sqrt(g p / r): d/d(g p) = 0.5 / sqrt(g p r), d/dr = -0.5 c / r (0 where p = 0)
    if ((bits(gpL) << 1) != 0) {
        pLb = fma(imul(imul(0.5, cLb), rsL), g, pLb);
        rLb -= imul(imul(imul(0.5, cLb), cL), rcp_fast(rL));
    }
    if ((bits(gpR) << 1) != 0) {
        pRb = fma(imul(imul(0.5, cRb), rsR), g, pRb);
        rRb -= imul(imul(imul(0.5, cRb), cR), rcp_fast(rR));
    }
    ab[0] = rLb; ab[1] = pLb; ab[2] = unLb; ab[3] = utLb;
    bb[0] = rRb; bb[1] = pRb; bb[2] = unRb; bb[3] = utRb;
}

// ---------------------------------------------------------------------------------------
// Pass B: face adjoints (each face once), then the gather into cells; the layout of
// gd_adjoint.cu with four fields.  Scratch after the 8 pass-A planes:
//   kFaceAdj + (dir * 2 + side) * 4 + f       face-state adjoints, side 0 = up, 1 = dn
//   kSel bytes, (dir * 4 + f) * K + cell      (choice + 1) | upper fallback << 2
//   kSel bytes, 8 K + (dir * 2 + f) * K + cell  lower fallback (f < 2)
// ---------------------------------------------------------------------------------------
constexpr int kFaceAdj = 8;
constexpr int kSel = kFaceAdj + 4 * NF;
constexpr int kScratchPlanes = kSel + 2;  // 12 bytes per cell fit in two planes of doubles
constexpr int FBX = 32, FBY = 4;

__device__ __forceinline__ int wrap(int i, int n) {
    const int r = i % n;
    return r < 0 ? r + n : r;
}

// minmod slope and which difference it took: +1 right (c_{+1} - c), -1 left (c - c_{-1}), 0
__device__ __forceinline__ double slope_sel(double cm, double c, double cp, int& sel) {
    const double l = c - cm, r = cp - c;
    const double s = minmod(l, r);
    sel = mag(s) == 0 ? 0 : (mag_lt(r, l) ? 1 : -1);
    return s;
}

// at most 128 registers a thread (four blocks per SM): uncapped, the integer products of the
// sweep took 146 and three blocks, slower
__global__ void __launch_bounds__(FBX * FBY, 4)
    eadj_face_kernel(Params P, CPlanes U, double* scratch, const double* __restrict__ T_do_ptr) {
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
        for (int f = 0; f < NF; ++f) c[t][f] = __ldg(U.f[f] + kc[t]);
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
    // flux adjoint: d_low += k F, d_high -= k F; slots 0 m, 1 e, 2 mx, 3 my
    double Fslot[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f)
        Fslot[f] = kk * (scratch[(size_t)(4 + f) * K + kc[1]] - scratch[(size_t)(4 + f) * K + kc[2]]);
    const double Fb[4] = {Fslot[0], isx ? Fslot[2] : Fslot[3], isx ? Fslot[3] : Fslot[2],
                          Fslot[1]};
    const double la[4] = {qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2]};
    const double lb[4] = {qb[0], qb[1], isx ? qb[2] : qb[3], isx ? qb[3] : qb[2]};
    double lab[4], lbb[4];
    hllc_vjp(la, lb, Fb, P, lab, lbb);
    const double gab[4] = {lab[0], lab[1], isx ? lab[2] : lab[3], isx ? lab[3] : lab[2]};
    const double gbb[4] = {lbb[0], lbb[1], isx ? lbb[2] : lbb[3], isx ? lbb[3] : lbb[2]};
    double* up = scratch + (size_t)(kFaceAdj + (isx ? 0 : 2) * NF) * K;
    double* dn = up + (size_t)NF * K;
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        up[(size_t)f * K + kc[1]] = gab[f];
        dn[(size_t)f * K + kc[2]] = gbb[f];
    }
}

__global__ void __launch_bounds__(FBX * FBY) eadj_gather_kernel(Params P,
                                                                const double* __restrict__ scratch,
                                                                Planes lam_in) {
    const int N = P.N, M = P.M;
    const long long K = (long long)N * M;
    const int gx = blockIdx.x * FBX + threadIdx.x, gy = blockIdx.y * FBY + threadIdx.y;
    if (gx >= N || gy >= M) return;
    const long long k = (long long)gy * N + gx;
    double lam[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f) lam[f] = scratch[(size_t)f * K + k];
    const unsigned char* rec = reinterpret_cast<const unsigned char*>(scratch + (size_t)kSel * K);
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const bool isx = dir == 0;
        long long kc[3];  // the cells at positions -1, 0, +1 along the direction
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
            // dropping its term (the factor 1/2 goes last, an exact scaling)
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
#pragma unroll
    for (int f = 0; f < NF; ++f) lam_in.f[f][k] = lam[f];
}

int grid_cells(long long K) {
    long long g = (K + NT - 1) / NT;
    return (int)(g > 152 * 16 ? 152 * 16 : (g < 1 ? 1 : g));
}

}  // namespace

int adjoint_euler_scratch_planes() { return kScratchPlanes; }

cudaError_t launch_adjoint_step_euler(const Params& P, const CPlanes& U, const double* aux,
                                      const CPlanes& lam_out, const Planes& lam_in,
                                      double* scratch, const double* T_do, cudaStream_t st) {
    const long long K = (long long)P.N * P.M;
    const dim3 blk(FBX, FBY);
    const unsigned gxb = (unsigned)((P.N + FBX - 1) / FBX), gyb = (unsigned)((P.M + FBY - 1) / FBY);
    if (gyb > 65535u) return cudaErrorInvalidConfiguration;
    eadj_update_kernel<<<grid_cells(K), NT, 0, st>>>(P, U, aux, lam_out, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    eadj_face_kernel<<<dim3(gxb, gyb, 2), blk, 0, st>>>(P, U, scratch, T_do);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    eadj_gather_kernel<<<dim3(gxb, gyb, 1), blk, 0, st>>>(P, scratch, lam_in);
    return cudaGetLastError();
}

}  // namespace gd
