// gd_fast_mhd.cu -- fused minmod-TVD + HLLD / HLLC-MHD + Powell-source update for 2-D ideal
// MHD, face-once tiles (same phase structure as gd_fast_euler.cu: load, slopes, faces,
// update).
//
// Field units.  The reference stores Gaussian B and divides by sqrt(4 pi) inside every flux
// call (Gas_Dinamic.cu:970-976), multiplying the field fluxes back (:1497-1499).  Here the
// field is converted once per cell when the tile is loaded, b = B / sqrt(4 pi), the whole
// step runs in these units, and B = b * sqrt(4 pi) is stored.  In these units the Powell
// terms of the reference update (kernel.cu:2641-2648), (B/4pi) Pdiv_B, (v.B/4pi) Pdiv_B and
// v Pdiv_B, become b Pdiv_b, (v.b) Pdiv_b and v Pdiv_b, and |B|^2/8pi becomes |b|^2/2.
//
// Reference semantics kept: primitive reconstruction of all seven fields with the rho/p
// fallback (kernel.cu:2407-2548); wave speeds SL = min(u) - max(cf), SR = max(u) + max(cf),
// SM and p_T* (Gas_Dinamic.cu:1062-1075); HLL-averaged field; HLLD star and double-star
// states with the |tt| >= 1e-5 and |bn| > 1e-6 guards (:1306-1430) and the six-region
// selection (:1434-1484), or the HLLC-MHD states (:1137-1302); normal-field flux
// -max(|SL|,|SR|) (bn_R - bn_L) (:1488-1490); Powell divergence from cell-centred B
// (kernel.cu:2568-2604); axisymmetric sources (kernel.cu:2615-2648); floors rho <= 0 ->
// old rho, p <= 0 -> 1e-6; dt = min over faces of krit*rad/max(|SL|,|SR|), rad = dx on
// x-faces (kernel.cu:2560).
#include "gd_internal.cuh"
#include "gd_kernels.h"

namespace gd {
namespace {

constexpr int TX = 32;
constexpr int NT = 256;
constexpr int NF = 7;  // rho, p, vx, vy, bx, by, bz

struct FluxM {
    double m, mn, mt, e, bn, bt, bz;  // mass, normal / tangential momentum, energy, field
};

// One side of the face in the local frame (un normal, ut in-plane tangential, uz = 0).
struct Side {
    double r, p, un, ut, bn, bt, bz, bb, pT, E, cf;
    double F0, F1, F2, F4, F6, F7;
};

__device__ __forceinline__ void side(Side& S, double r, double p, double un, double ut, double bn,
                                     double bt, double bz, const Params& P) {
    S.r = r; S.p = p; S.un = un; S.ut = ut; S.bn = bn; S.bt = bt; S.bz = bz;
    const double bn2 = bn * bn;
    S.bb = fma(bz, bz, fma(bt, bt, bn2));
    S.pT = fma(0.5, S.bb, p);
    S.E = fma(p, P.inv_gm1, 0.5 * fma(r, fma(un, un, ut * ut), S.bb));
    const double gp = P.gamma * p;
    const double a = gp + S.bb;
    double disc = fma(a, a, -4.0 * gp * bn2);
    disc = le_zero(disc) ? 0.0 : disc;
    const double X = 0.5 * (a + sqrt_fast(disc));  // rho cf^2
    S.cf = X * rsqrt_fast(X * r);                   // sqrt(X / r)
    S.F0 = r * un;
    S.F1 = fma(S.F0, un, S.pT - bn2);
    S.F2 = fma(S.F0, ut, -bn * bt);
    S.F4 = fma(S.E + S.pT, un, -bn * fma(ut, bt, un * bn));
    S.F6 = fma(un, bt, -ut * bn);
    S.F7 = un * bz;
}

__device__ __forceinline__ double sgn_select(double v, int idbn) {
    // idbn * v for idbn in {-1, 0, 1}, on the integer pipe (sign-bit flip, select)
    const double w = idbn < 0 ? from_bits(bits(v) ^ (long long)0x8000000000000000ULL) : v;
    return idbn == 0 ? 0.0 : w;
}

// HLLD (method 3) or HLLC-MHD (method 2) flux.  UU = max(|SL|, |SR|).
__device__ __forceinline__ FluxM hlld_local(const Side& A, const Side& B, int method,
                                            double& UU) {
    const double uminN = dmin(A.un, B.un);
    const double umaxN = dmax(A.un, B.un);
    const double cmax = max_nonneg(A.cf, B.cf);
    const double SL = uminN - cmax, SR = umaxN + cmax;
    const double suL = SL - A.un, suR = SR - B.un;
    const double mL = A.r * suL, mR = B.r * suR;
    const double iden = rcp_fast(mR - mL);
    const double SM = ((fma(mR, B.un, -mL * A.un) - B.pT) + A.pT) * iden;
    const double PTT = fma(mL * mR, B.un - A.un, fma(mR, A.pT, -mL * B.pT)) * iden;
    UU = max_nonneg(dabs(SL), dabs(SR));
    const double iS = rcp_fast(SR - SL);
    const double bn = fma(SR, B.bn, -SL * A.bn) * iS;
    const double bt = (fma(SR, B.bt, -SL * A.bt) + (A.F6 - B.F6)) * iS;
    const double bz = (fma(SR, B.bz, -SL * A.bz) + (A.F7 - B.F7)) * iS;
    const double iL = rcp_fast(SL - SM), iR = rcp_fast(SR - SM);
    const double rLL = mL * iL, rRR = mR * iR;

    // region: takeL, level 0 (F), 1 (star), 2 (double star)
    FluxM F;
    if (method == GD_METHOD_HLLC_MHD) {
        const bool takeL = ge_zero(SL) || ge_zero(SM);
        const Side& K = takeL ? A : B;
        const double S = takeL ? SL : SR;
        const bool star = takeL ? lt_zero(SL) : gt_zero(SR);
        F.m = K.F0; F.mn = K.F1; F.mt = K.F2; F.e = K.F4; F.bt = K.F6; F.bz = K.F7;
        if (star) {
            // HLL state of the fan (Gas_Dinamic.cu:1145-1149); mom_z: U = 0, F = -bn bz
            const double UZ0 = (fma(SR, B.r, -SL * A.r) + (A.F0 - B.F0)) * iS;
            const double UZ1 = (fma(SR, B.r * B.un, -SL * A.r * A.un) + (A.F1 - B.F1)) * iS;
            const double UZ2 = (fma(SR, B.r * B.ut, -SL * A.r * A.ut) + (A.F2 - B.F2)) * iS;
            const double UZ3 = (B.bn * B.bz - A.bn * A.bz) * iS;
            const double iU0 = rcp_fast(UZ0);
            const double vS = UZ2 * iU0, wS = UZ3 * iU0;
            const double ptz = 0.5 * (fma(mR, SM - B.un, B.pT) + fma(mL, SM - A.un, A.pT));
            const double sbvz = fma(bn, UZ1, fma(bt, UZ2, bz * UZ3)) * iU0;
            const double sbvK = fma(K.un, K.bn, K.ut * K.bt);
            const double iK = takeL ? iL : iR;
            const double suK = takeL ? suL : suR;
            const double eK = (fma(K.E, suK, fma(ptz, SM, -K.pT * K.un)) + bn * (sbvK - sbvz)) * iK;
            const double rK = takeL ? rLL : rRR;
            F.m = fma(S, rK - K.r, F.m);
            F.mn = fma(S, fma(rK, SM, -K.r * K.un), F.mn);
            F.mt = fma(S, fma(rK, vS, -K.r * K.ut), F.mt);
            F.e = fma(S, eK - K.E, F.e);
            F.bt = fma(S, bt - K.bt, F.bt);
            F.bz = fma(S, bz - K.bz, F.bz);
            (void)wS;
        }
    } else {
        const double bbn = bn * bn;
        // star states of both sides (Gas_Dinamic.cu:1306-1350)
        double vLL, wLL, btL, bzL, vRR, wRR, btR, bzR;
        {
            const double tt = fma(mL, SL - SM, -bbn);
            if (abs_bits(tt) >= 0x3EE4F8B588E368F1ULL) {  // |tt| >= 1e-5
                const double it = rcp_fast(tt);
                const double c = bn * (SM - A.un) * it;
                const double d = fma(mL, suL, -bbn) * it;
                vLL = fma(-c, A.bt, A.ut);
                wLL = -c * A.bz;
                btL = A.bt * d;
                bzL = A.bz * d;
            } else {
                vLL = A.ut; wLL = 0.0; btL = 0.0; bzL = 0.0;
            }
        }
        {
            const double tt = fma(mR, SR - SM, -bbn);
            if (abs_bits(tt) >= 0x3EE4F8B588E368F1ULL) {
                const double it = rcp_fast(tt);
                const double c = bn * (SM - B.un) * it;
                const double d = fma(mR, suR, -bbn) * it;
                vRR = fma(-c, B.bt, B.ut);
                wRR = -c * B.bz;
                btR = B.bt * d;
                bzR = B.bz * d;
            } else {
                vRR = B.ut; wRR = 0.0; btR = 0.0; bzR = 0.0;
            }
        }
        const double SMbn = SM * bn;
        const double sbLL = fma(wLL, bzL, fma(vLL, btL, SMbn));
        const double sbRR = fma(wRR, bzR, fma(vRR, btR, SMbn));
        const double eLL = (fma(A.E, suL, fma(PTT, SM, -A.pT * A.un)) +
                            bn * (fma(A.un, A.bn, A.ut * A.bt) - sbLL)) * iL;
        const double eRR = (fma(B.E, suR, fma(PTT, SM, -B.pT * B.un)) +
                            bn * (fma(B.un, B.bn, B.ut * B.bt) - sbRR)) * iR;
        const double isLL = rsqrt_fast(rLL), isRR = rsqrt_fast(rRR);
        const double sLL = rLL * isLL, sRR = rRR * isRR;
        const bool bnz = abs_bits(bn) > 0x3EB0C6F7A0B5ED8DULL;  // |bn| > 1e-6
        const double abn = dabs(bn);
        const double SLL = bnz ? fma(-abn, isLL, SM) : SM;
        const double SRR = bnz ? fma(abn, isRR, SM) : SM;
        const int idbn = bnz ? (gt_zero(bn) ? 1 : -1) : 0;

        const bool takeL = ge_zero(SL) || ge_zero(SM);
        int level;
        if (takeL) level = ge_zero(SL) ? 0 : (ge_zero(SLL) ? 1 : 2);
        else level = gt_zero(SRR) ? 2 : (gt_zero(SR) ? 1 : 0);
        const Side& K = takeL ? A : B;
        F.m = K.F0; F.mn = K.F1; F.mt = K.F2; F.e = K.F4; F.bt = K.F6; F.bz = K.F7;
        if (level >= 1) {
            const double S = takeL ? SL : SR;
            const double rK = takeL ? rLL : rRR;
            const double vK = takeL ? vLL : vRR;
            const double eK = takeL ? eLL : eRR;
            const double btK = takeL ? btL : btR;
            const double bzK = takeL ? bzL : bzR;
            F.m = fma(S, rK - K.r, F.m);
            F.mn = fma(S, fma(rK, SM, -K.r * K.un), F.mn);
            F.mt = fma(S, fma(rK, vK, -K.r * K.ut), F.mt);
            F.e = fma(S, eK - K.E, F.e);
            F.bt = fma(S, btK - K.bt, F.bt);
            F.bz = fma(S, bzK - K.bz, F.bz);
            if (level == 2) {
                // double-star states (Gas_Dinamic.cu:1371-1430)
                const double is = rcp_fast(sLL + sRR);
                const double vL3 = (fma(sLL, vLL, sRR * vRR) + sgn_select(btR - btL, idbn)) * is;
                const double wL3 = (fma(sLL, wLL, sRR * wRR) + sgn_select(bzR - bzL, idbn)) * is;
                const double s2 = sgn_select(sLL * sRR, idbn);
                const double bt3 = fma(s2, vRR - vLL, fma(sLL, btR, sRR * btL)) * is;
                const double bz3 = fma(s2, wRR - wLL, fma(sLL, bzR, sRR * bzL)) * is;
                const double sb3 = fma(wL3, bz3, fma(vL3, bt3, SMbn));
                const double sK = takeL ? -sLL : sRR;
                const double e3 = fma(sgn_select(sK, idbn), (takeL ? sbLL : sbRR) - sb3, eK);
                const double S2 = takeL ? SLL : SRR;
                F.mt = fma(S2, rK * (vL3 - vK), F.mt);
                F.e = fma(S2, e3 - eK, F.e);
                F.bt = fma(S2, bt3 - btK, F.bt);
                F.bz = fma(S2, bz3 - bzK, F.bz);
            }
        }
    }
    // normal-field flux replaced by the diffusive term (Gas_Dinamic.cu:1488-1490)
    F.bn = -UU * (B.bn - A.bn);
    return F;
}

template <int ORDER, int TY>
struct SmemM {
    static constexpr int H = ORDER == 2 ? 2 : 1;
    static constexpr int SX = TX + 2 * H;
    static constexpr int SY = TY + 2 * H;
    static constexpr int kPrim = NF * SY * SX;
    static constexpr int kSlx = ORDER == 2 ? NF * TY * (TX + 2) : 0;
    static constexpr int kSly = ORDER == 2 ? NF * (TY + 2) * TX : 0;
    static constexpr int kFx = NF * TY * (TX + 1);
    static constexpr int kFy = NF * (TY + 1) * TX;
    static constexpr size_t bytes = sizeof(double) * (kPrim + kSlx + kSly + kFx + kFy);
};

// flux component slots in smem: 0 mass, 1 energy, 2 mom x, 3 mom y, 4 bx, 5 by, 6 bz
template <int ORDER, int TY>
__global__ void __launch_bounds__(NT) mhd_fast_kernel(Params P, CPlanes in, Planes out,
                                                      const double* __restrict__ T_do_ptr,
                                                      unsigned long long* T_bits, Scalars* rot,
                                                      Scalars* ctr, int dt_only) {
    using S = SmemM<ORDER, TY>;
    constexpr int H = S::H, SX = S::SX, SY = S::SY;
    extern __shared__ double smem[];
    double* prim = smem;
    double* slx = prim + S::kPrim;
    double* sly = slx + S::kSlx;
    double* fx = sly + S::kSly;
    double* fy = fx + S::kFx;

    const int tid = threadIdx.x;
    const int tx0 = blockIdx.x * TX, ty0 = blockIdx.y * TY;
    const int N = P.N, M = P.M;

    // ---- L: tile + cross halo, field to Heaviside-Lorentz units --------------------------
    for (int i = tid; i < SY * SX; i += NT) {
        const int ly = i / SX, lx = i - ly * SX;
        const bool xh = lx < H || lx >= TX + H, yh = ly < H || ly >= TY + H;
        if (xh && yh) continue;
        const int gx = tx0 + lx - H, gy = ty0 + ly - H;
        double v[NF];
        if (gx >= -2 && gx < N + 2 && gy >= -2 && gy < M + 2 &&
            !((gx < 0 || gx >= N) && (gy < 0 || gy >= M))) {
            fetch_cell<NF>(P, in, gx, gy, v);
        } else {
#pragma unroll
            for (int f = 0; f < NF; ++f) v[f] = f < 2 ? 1.0 : 0.0;  // never used
        }
        v[4] *= kInvSpi4;
        v[5] *= kInvSpi4;
        v[6] *= kInvSpi4;
#pragma unroll
        for (int f = 0; f < NF; ++f) prim[(f * SY + ly) * SX + lx] = v[f];
    }
    __syncthreads();

    // ---- S: slopes ---------------------------------------------------------------------------
    if (ORDER == 2) {
        for (int i = tid; i < TY * (TX + 2); i += NT) {
            const int ly = i / (TX + 2), c = i - ly * (TX + 2);
            const double* row = prim + (ly + H) * SX + (c - 1 + H);
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const double* q = row + f * SY * SX;
                slx[(f * TY + ly) * (TX + 2) + c] = minmod(q[0] - q[-1], q[1] - q[0]);
            }
        }
        for (int i = tid; i < (TY + 2) * TX; i += NT) {
            const int r = i / TX, lx = i - r * TX;
            const double* col = prim + (r - 1 + H) * SX + (lx + H);
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const double* q = col + f * SY * SX;
                sly[(f * (TY + 2) + r) * TX + lx] = minmod(q[0] - q[-SX], q[SX] - q[0]);
            }
        }
        __syncthreads();
    }

    // ---- F: faces ----------------------------------------------------------------------------
    double umax_x = 0.0, umax_y = 0.0;
    constexpr int NFX = (TX + 1) * TY, NFY = TX * (TY + 1);
    for (int i = tid; i < NFX + NFY; i += NT) {
        const bool isx = i < NFX;
        int lx, ly;
        if (isx) {
            ly = i / (TX + 1);
            lx = i - ly * (TX + 1);
            if (tx0 + lx > N || ty0 + ly >= M) continue;
        } else {
            const int j = i - NFX;
            ly = j / TX;
            lx = j - ly * TX;
            if (tx0 + lx >= N || ty0 + ly > M) continue;
        }
        const int ax = isx ? lx - 1 : lx, ay = isx ? ly : ly - 1;
        if (P.frozen_radius > 0.0 && !cell_active(P, tx0 + ax, ty0 + ay) &&
            !cell_active(P, tx0 + lx, ty0 + ly))
            continue;
        const double* pa = prim + (ay + H) * SX + (ax + H);
        const double* pb = pa + (isx ? 1 : SX);
        double qa[NF], qb[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const double ca = pa[f * SY * SX], cb = pb[f * SY * SX];
            if (ORDER == 2) {
                double da, db;
                if (isx) {
                    da = slx[(f * TY + ly) * (TX + 2) + lx];
                    db = slx[(f * TY + ly) * (TX + 2) + lx + 1];
                } else {
                    da = sly[(f * (TY + 2) + ly) * TX + lx];
                    db = sly[(f * (TY + 2) + ly + 1) * TX + lx];
                }
                double a = fma(0.5, da, ca), b = fma(-0.5, db, cb);
                if (f < 2) {
                    a = le_zero(a) ? ca : a;
                    b = le_zero(b) ? cb : b;
                }
                qa[f] = a;
                qb[f] = b;
            } else {
                qa[f] = ca;
                qb[f] = cb;
            }
        }
        // local frame: x-face (n, t) = (x, y); y-face (n, t) = (y, x); z stays z
        Side A, B;
        side(A, qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2], isx ? qa[4] : qa[5],
             isx ? qa[5] : qa[4], qa[6], P);
        side(B, qb[0], qb[1], isx ? qb[2] : qb[3], isx ? qb[3] : qb[2], isx ? qb[4] : qb[5],
             isx ? qb[5] : qb[4], qb[6], P);
        double UU;
        const FluxM F = hlld_local(A, B, P.method, UU);
        if (isx) {
            double* fo = fx + ly * (TX + 1) + lx;
            constexpr int st = TY * (TX + 1);
            fo[0 * st] = F.m;
            fo[1 * st] = F.e;
            fo[2 * st] = F.mn;
            fo[3 * st] = F.mt;
            fo[4 * st] = F.bn;
            fo[5 * st] = F.bt;
            fo[6 * st] = F.bz;
            umax_x = max_nonneg(umax_x, UU);
        } else {
            double* fo = fy + ly * TX + lx;
            constexpr int st = (TY + 1) * TX;
            fo[0 * st] = F.m;
            fo[1 * st] = F.e;
            fo[2 * st] = F.mt;
            fo[3 * st] = F.mn;
            fo[4 * st] = F.bt;
            fo[5 * st] = F.bn;
            fo[6 * st] = F.bz;
            umax_y = max_nonneg(umax_y, UU);
        }
    }
    __syncthreads();

    // ---- U: update (kernel.cu:2606-2660 in Heaviside-Lorentz field units) ----------------------
    const double T_do = *T_do_ptr;
    const double kx = T_do / P.dx, ky = T_do / P.dy;
    const bool axi = P.geometry == GD_AXISYM;
    bool any_active = false;
    unsigned int nfl_r = 0, nfl_p = 0, nbad = 0;
    for (int i = tid; i < TX * TY; i += NT) {
        const int ly = i / TX, lx = i - ly * TX;
        const int gx = tx0 + lx, gy = ty0 + ly;
        if (gx >= N || gy >= M) continue;
        const double* c = prim + (ly + H) * SX + (lx + H);
        constexpr int PS = SY * SX;
        const double r = c[0], p = c[PS], u = c[2 * PS], v = c[3 * PS];
        const double bx = c[4 * PS], by = c[5 * PS], bz = c[6 * PS];
        const long long k = (long long)gy * N + gx;
        const double y = P.y0 + gy * P.dy;
        if (P.frozen_radius > 0.0) {
            const double x = P.x0 + gx * P.dx;
            if (sqrt(x * x + y * y) < P.frozen_radius) {
                if (!dt_only) {
#pragma unroll
                    for (int f = 0; f < NF; ++f) out.f[f][k] = in.f[f][k];
                }
                continue;
            }
        }
        any_active = true;
        if (dt_only) continue;
        const double* fxc = fx + ly * (TX + 1) + lx;
        const double* fyc = fy + ly * TX + lx;
        double d[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const double* a = fxc + f * TY * (TX + 1);
            const double* b = fyc + f * (TY + 1) * TX;
            d[f] = fma(kx, a[1] - a[0], ky * (b[TX] - b[0]));
        }
        // Powell divergence from cell-centred field: dx dy div b (kernel.cu:2568-2604)
        const double bxE = c[4 * PS + 1], bxW = c[4 * PS - 1];
        const double byN = c[5 * PS + SX], byS = c[5 * PS - SX];
        double divb = fma(0.5 * kx, bxE - bxW, 0.5 * ky * (byN - byS));  // T_do * div b
        const double iy = axi ? rcp_fast(y) : 0.0;
        if (axi) divb = fma(T_do * by, iy, divb);                      // kernel.cu:2615
        const double ub = fma(u, bx, v * by);
        const double bb = fma(bz, bz, fma(by, by, bx * bx));
        const double E = fma(p, P.inv_gm1, 0.5 * fma(r, fma(u, u, v * v), bb));
        double r2 = r - d[0];
        double mx2 = fma(r, u, -fma(bx, divb, d[2]));
        double my2 = fma(r, v, -fma(by, divb, d[3]));
        double bx2 = bx - fma(u, divb, d[4]);
        const double by2 = by - fma(v, divb, d[5]);
        const double bz2 = bz - d[6];
        double E2 = E - fma(ub, divb, d[1]);
        if (axi) {
            // geometric sources / y (kernel.cu:2619-2648) in field units b
            const double ty = T_do * iy;
            r2 = fma(-ty * r, v, r2);
            mx2 = fma(-ty, fma(r * u, v, -bx * by), mx2);
            my2 = fma(-ty, fma(r * v, v, fma(bz, bz, -by * by)), my2);
            bx2 = fma(-ty, fma(v, bx, -by * u), bx2);
            E2 = fma(-ty, fma(E + p + 0.5 * bb, v, -by * ub), E2);
        }
        if (le_zero(r2)) { r2 = r; ++nfl_r; }
        const double inv = rcp_fast(r2);
        const double u2 = mx2 * inv, v2 = my2 * inv;
        double p2 = (E2 - 0.5 * fma(r2, fma(u2, u2, v2 * v2), fma(bz2, bz2, fma(by2, by2, bx2 * bx2)))) * P.gm1;
        if (le_zero(p2)) { p2 = 0.000001; ++nfl_p; }
        if (!isfinite(r2) || !isfinite(p2) || !isfinite(u2) || !isfinite(v2) || !isfinite(bx2) ||
            !isfinite(by2) || !isfinite(bz2))
            ++nbad;
        out.f[0][k] = r2;
        out.f[1][k] = p2;
        out.f[2][k] = u2;
        out.f[3][k] = v2;
        out.f[4][k] = bx2 * kSpi4;
        out.f[5][k] = by2 * kSpi4;
        out.f[6][k] = bz2 * kSpi4;
    }
    if (ctr != nullptr && (nfl_r | nfl_p | nbad)) {
        if (nfl_r) atomicAdd(&ctr->rho_floor, (unsigned long long)nfl_r);
        if (nfl_p) atomicAdd(&ctr->p_floor, (unsigned long long)nfl_p);
        if (nbad) atomicAdd(&ctr->nonfinite, (unsigned long long)nbad);
    }
    block_dt_and_rotate<NT>(P, umax_x, umax_y, any_active, T_bits, rot);
}

constexpr int kTY = 16;

template <int ORDER>
cudaError_t launch_t(const Params& P, const CPlanes& in, const Planes& out, const double* T_do,
                     unsigned long long* T_bits, Scalars* rot, Scalars* ctr, int dt_only,
                     cudaStream_t st) {
    dim3 grid((P.N + TX - 1) / TX, (P.M + kTY - 1) / kTY);
    mhd_fast_kernel<ORDER, kTY><<<grid, NT, SmemM<ORDER, kTY>::bytes, st>>>(
        P, in, out, T_do, T_bits, rot, ctr, dt_only);
    return cudaGetLastError();
}

}  // namespace

cudaError_t prepare_mhd_fast() {
    cudaError_t e = cudaFuncSetAttribute(mhd_fast_kernel<1, kTY>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SmemM<1, kTY>::bytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(mhd_fast_kernel<2, kTY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)SmemM<2, kTY>::bytes);
}

cudaError_t launch_mhd_fast(const Params& P, const CPlanes& in, const Planes& out,
                            const double* T_do, unsigned long long* T_bits, Scalars* rot,
                            Scalars* ctr, int dt_only, cudaStream_t st) {
    if (P.order == 1) return launch_t<1>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
    return launch_t<2>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
}

}  // namespace gd
