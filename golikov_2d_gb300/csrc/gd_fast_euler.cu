// gd_fast_euler.cu -- fused minmod-TVD + HLLC/HLL + update step for 2-D Euler, face-once tiles.
//
// One CTA owns a TX x TY tile.  Phases, separated by __syncthreads():
//   L  load the tile plus a 2-cell cross-shaped halo (boundary ghosts applied) into smem;
//   S  per-cell minmod slopes along x and y (integer-pipe minmod, one FP64 sub per edge);
//   F  every face of the tile once: left/right face states from the slopes, the HLLC (or,
//      for method 0, HLL) flux in the face's local (normal, tangent) frame, and the face's
//      wave-speed maximum;
//   U  conservative update of each cell from its four face fluxes, positivity floors,
//      primitive recovery; store; block dt minimum and the fused funk_time rotation.
// The reference computes every face twice, once from each neighbour (kernel.cu:3560-3586);
// here each face is computed once and used with opposite signs by its two cells.  The
// standalone products run on the integer pipes (mulx: the FP64 multiply's bits), the sound
// speeds and reciprocals take two FP64 operations each (sqrt_over_2op, rcp_2op), and the
// HLLC star state takes S_M and q from one reciprocal.
//
// Each tile shape is a separate template instantiation; the compiler may fuse multiply-adds
// differently in each, so shapes agree to rounding (~1e-14 relative per step), not bit for
// bit.  A given shape is deterministic.
//
// Two kernels share the tile body: euler_fast_kernel (one grid, one CTA per tile) and
// euler_batch_kernel (a persistent launch that walks the tiles of many independent grids,
// each grid with its own parameters, state, dt reduction and funk_time rotation).  Tile
// shapes 16x16, 32x8, 32x16 and 64x8 are compiled; the autotuner picks one for a batch, and
// the single-grid step uses 16x16 (49 KB of shared memory and 64 registers a thread: four
// CTAs, 32 warps, per SM; at 32x16, 93 KB, two CTAs left the FP64 pipe waiting on its own
// results once the flux took fewer operations: 7.01 against 6.49 ms per step at 4096^2).
//
// Reference semantics kept: primitive reconstruction of (rho, p, vx, vy) with the rho/p
// face fallback to the cell value (kernel.cu:3436-3544), Davis wave speeds and the HLLC
// star states of HLLC_Aleksashov (kernel.cu:853-1165), the HLL flux (kernel.cu:1485-1609)
// for method 0, the Ker_Dekard update and floors
// rho <= 0 -> 1e-4, p <= 0 -> 1e-6 (kernel.cu:1849-1874), dt = min over faces of
// krit*rad/max(|SL|,|SR|) with rad = dy on x-faces (kernel.cu:1811).
#include <type_traits>

#include "gd_dual.cuh"
#include "gd_internal.cuh"
#include "gd_kernels.h"
#include "gd_mhd_flux.cuh"  // cst<T>

namespace gd {
namespace {

constexpr int NT = 256;
constexpr int NF = 4;

template <class T>
struct FluxE {
    T m, mn, mt, e;
};

// HLLC flux in a local frame: un = normal velocity, ut = in-plane tangential velocity.
// Returns the flux (mass, normal momentum, tangential momentum, energy) and, in UU, SL or
// SR, the one of larger magnitude (signed; the dt reduction takes |UU|).  T is double, or
// Dual for the tangent (value and derivative, the branch choices taken on the value).
// Products go through mulx (on the integer pipes for double), sums and fused
// multiply-adds through the FP64 unit.
template <class T>
__device__ __forceinline__ FluxE<T> hllc_local(T rL, T pL, T unL, T utL, T rR, T pR, T unR,
                                               T utR, const Params& P, T& UU) {
    const double g = P.gamma;
    const T cL = sqrt_over_2op(mulx(g, pL), rL);  // sqrt(g p / rho)
    const T cR = sqrt_over_2op(mulx(g, pR), rR);
    const T aL = unL - cL, aR = unR - cR;
    const T bL = unL + cL, bR = unR + cR;
    const T SL = dmin(aL, aR);  // Davis estimates (kernel.cu:981-982)
    const T SR = dmax(bL, bR);
    const T suL = SL - unL, suR = SR - unR;
    const T mL = mulx(rL, suL), mR = mulx(rR, suR);
    // S_M = Nm / D (kernel.cu:1001-1003): its sign is the sign of Nm times that of D
    const T Nm = fma(mR, unR, fma(-mL, unL, pL - pR));
    const T D = mR - mL;
    UU = max_nonneg(SL, SR);  // signed: the block reduction takes the magnitude

    // Side whose state (or star state) gives the flux at x/t = 0 (kernel.cu:1119-1158).
    const bool takeL = gt_zero(SL) || !quotient_neg(Nm, D);
    const T r = takeL ? rL : rR;
    const T p = takeL ? pL : pR;
    const T un = takeL ? unL : unR;
    const T ut = takeL ? utL : utR;
    const T S = takeL ? SL : SR;
    const T su = takeL ? suL : suR;
    const T mm = takeL ? mL : mR;
    const bool star = takeL ? !gt_zero(SL) : ge_zero(SR);

    const T V2 = fma(un, un, mulx(ut, ut));
    FluxE<T> F;
    if (star) {
        // F_K + S_K (U*_K - U_K) is the physical flux of the star state, F(U*_K) with the
        // star pressure: the jump conditions across S_K are what define rho*, p* and E*
        // (kernel.cu:1119-1158).  With q = S_M / (S_K - S_M), p* = p + rho su (S_M - un),
        // su = S_K - un and G = gamma / (gamma - 1):
        //   mass rho* S_M = rho su q,  momentum rho* S_M^2 + p*,  tangential rho* S_M ut,
        //   energy (E* + p*) S_M = q su (p G + rho (|v|^2 / 2 + S_K (S_M - un))).
        // S_M and q from one reciprocal: with X = S_K D - Nm = D (S_K - S_M),
        //   S_M = Nm X / (D X),  q = Nm D / (D X).
        const T X = fma(S, D, -Nm);
        const T R = rcp_2op(mulx(D, X));
        const T NR = mulx(Nm, R);
        const T SM = mulx(NR, X);
        const T q = mulx(NR, D);
        const T SMu = SM - un;
        const T pst = fma(mm, SMu, p);
        const T qs = mulx(q, su);
        F.m = mulx(r, qs);
        F.mn = fma(F.m, SM, pst);
        F.mt = mulx(F.m, ut);
        F.e = mulx(qs, fma(p, P.g_gm1, mulx(r, fma(0.5, V2, mulx(S, SMu)))));
    } else {
        F.m = mulx(r, un);
        F.mn = fma(F.m, un, p);
        F.mt = mulx(F.m, ut);
        F.e = mulx(un, fma(p, P.g_gm1, mulx(mulx(0.5, r), V2)));  // (E + p) un
    }
    return F;
}

// HLL flux of kernel.cu:1485-1609 in a local frame (same arguments and results as
// hllc_local): sound speed 0 where rho <= 0, D_L = min(un) - max(c), D_R = max(un) + max(c),
// the upwind physical flux when the fan lies on one side of the face (strict tests against
// Omega = 0, kernel.cu:11), else (D_R F_L - D_L F_R + D_L D_R (U_R - U_L)) / (D_R - D_L).
// Its products stay on the FP64 unit: the tile function holds both fluxes, and registers
// are allocated for its heavier path -- integer-pipe products here took the tile to about
// 110 registers a thread, two CTAs per SM for the HLLC step as well.
template <class T>
__device__ __forceinline__ FluxE<T> hll_local(T rL, T pL, T unL, T utL, T rR, T pR, T unR,
                                              T utR, const Params& P, T& UU) {
    const double g = P.gamma;
    const T gpL = g * pL, gpR = g * pR;
    const T cL = le_zero(rL) ? cst<T>(0.0) : sqrt_over(gpL, rL);  // sqrt(g p / rho)
    const T cR = le_zero(rR) ? cst<T>(0.0) : sqrt_over(gpR, rR);
    const T cm = max_nonneg(cL, cR);
    const T DL = dmin(unL, unR) - cm;
    const T DR = dmax(unL, unR) + cm;
    UU = max_nonneg(DL, DR);  // signed: the block reduction takes the magnitude
    const bool left = gt_zero(DL), right = !left && lt_zero(DR);
    FluxE<T> F;
    if (left || right) {  // one side's physical flux
        const T r = left ? rL : rR, p = left ? pL : pR;
        const T un = left ? unL : unR, ut = left ? utL : utR;
        F.m = r * un;
        F.mn = fma(F.m, un, p);
        F.mt = F.m * ut;
        const T E = fma(p, P.inv_gm1, 0.5 * r * fma(un, un, ut * ut));
        F.e = (E + p) * un;
        return F;
    }
    const T mL = rL * unL, mR = rR * unR;
    const T EL = fma(pL, P.inv_gm1, 0.5 * rL * fma(unL, unL, utL * utL));
    const T ER = fma(pR, P.inv_gm1, 0.5 * rR * fma(unR, unR, utR * utR));
    const T inv = rcp_fast(DR - DL);
    const T dd = DL * DR;
    // (D_R F_L - D_L F_R + D_L D_R dU) / (D_R - D_L), component by component
    F.m = fma(dd, rR - rL, fma(DR, mL, -DL * mR)) * inv;
    F.mn = fma(dd, mR - mL, fma(DR, fma(mL, unL, pL), -DL * fma(mR, unR, pR))) * inv;
    F.mt = fma(dd, fma(rR, utR, -rL * utL), fma(DR, mL * utL, -DL * (mR * utR))) * inv;
    F.e = fma(dd, ER - EL, fma(DR, (EL + pL) * unL, -DL * ((ER + pR) * unR))) * inv;
    return F;
}

template <int ORDER, int TX, int TY>
struct Shape {
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

// Value and tangent planes (the tangent step of the adjoint checks).
struct DualIn {
    CPlanes v, d;
};
struct DualOut {
    Planes v, d;
};

__device__ __forceinline__ void load_cell(const Params& P, const CPlanes& in, int gx, int gy,
                                          double* v) {
    fetch_cell<NF>(P, in, gx, gy, v);
}
// The tangent of a ghost value: the same copy (the tangent runs on periodic grids only, where
// a ghost is a copy of a cell).
__device__ __forceinline__ void load_cell(const Params& P, const DualIn& in, int gx, int gy,
                                          Dual* v) {
    double a[NF], b[NF];
    fetch_cell<NF>(P, in.v, gx, gy, a);
    fetch_cell<NF>(P, in.d, gx, gy, b);
#pragma unroll
    for (int f = 0; f < NF; ++f) v[f] = Dual{a[f], b[f]};
}
__device__ __forceinline__ void store_cell(const Planes& out, long long k, int f, double x) {
    store_f(out, f, k, x);
}
__device__ __forceinline__ void store_cell2(const Planes& out, long long k, int f0, double a,
                                            double b) {
    store_pair(out, f0, k, a, b);
}
__device__ __forceinline__ void store_cell(const DualOut& out, long long k, int f, Dual x);
__device__ __forceinline__ void store_cell2(const DualOut& out, long long k, int f0, Dual a,
                                            Dual b) {
    store_cell(out, k, f0, a);
    store_cell(out, k, f0 + 1, b);
}
__device__ __forceinline__ void store_cell(const DualOut& out, long long k, int f, Dual x) {
    out.v.f[f][k] = x.v;
    out.d.f[f][k] = x.d;
}

struct TileResult {
    double umax_x, umax_y;
    bool any_active;
    unsigned int nfl_r, nfl_p, nbad;
};

// One TX x TY tile whose lower-left cell is (tx0, ty0).  Reads `in`, writes `out`, returns
// the per-thread wave-speed maxima and counters.  Every thread of the block must call it.
// `aux` (may be null): per cell, the flux differences d[0..3] of the update, planes of N*M
// (the adjoint's recording).
// Not inlined: the single-grid kernel and the persistent batch kernel call one compiled
// function per tile shape, so a grid's arithmetic, and its bits, do not depend on which
// schedule advanced it (inlined into each, the compiler may fuse the two differently).
template <class T, int ORDER, int TX, int TY, class IN, class OUT>
__device__ __noinline__ void euler_tile(const Params& P, const IN& in, const OUT& out, int tx0,
                                        int ty0, double T_do, int dt_only, T* smem,
                                        TileResult& res, double* aux) {
    using S = Shape<ORDER, TX, TY>;
    constexpr int H = S::H, SX = S::SX, SY = S::SY;
    T* prim = smem;                 // [NF][SY][SX]
    T* slx = prim + S::kPrim;       // [NF][TY][TX+2]   cells x in [-1, TX]
    T* sly = slx + S::kSlx;         // [NF][TY+2][TX]   cells y in [-1, TY]
    T* fx = sly + S::kSly;          // [NF][TY][TX+1]   face between x-1 and x
    T* fy = fx + S::kFx;            // [NF][TY+1][TX]   face between y-1 and y

    const int tid = threadIdx.x;
    const int N = P.N, M = P.M;

    // ---- L: tile + cross halo ------------------------------------------------------------
    for (int i = tid; i < SY * SX; i += NT) {
        const int ly = i / SX, lx = i - ly * SX;
        const bool xh = lx < H || lx >= TX + H, yh = ly < H || ly >= TY + H;
        if (xh && yh) continue;  // corners are never read
        const int gx = tx0 + lx - H, gy = ty0 + ly - H;
        T v[NF];
        if (gx >= -2 && gx < N + 2 && gy >= -2 && gy < M + 2 &&
            !((gx < 0 || gx >= N) && (gy < 0 || gy >= M))) {
            load_cell(P, in, gx, gy, v);
        } else {
#pragma unroll
            for (int f = 0; f < NF; ++f) v[f] = cst<T>(1.0);  // outside the grid, never used
        }
#pragma unroll
        for (int f = 0; f < NF; ++f) prim[(f * SY + ly) * SX + lx] = v[f];
    }
    __syncthreads();

    // ---- S: slopes --------------------------------------------------------------------------
    // A thread takes a run of G cells along the direction, so neighbouring slopes share their
    // difference: G + 1 FP64 subtractions per G cells instead of 2 G.
    if (ORDER == 2) {
        constexpr int GX = (TX + 2) % 3 == 0 ? 3 : 2, GY = (TY + 2) % 3 == 0 ? 3 : 2;
        constexpr int NGX = (TX + 2) / GX, NGY = (TY + 2) / GY;
        static_assert((TX + 2) % GX == 0 && (TY + 2) % GY == 0, "slope runs tile the rows");
        for (int i = tid; i < TY * NGX; i += NT) {
            const int ly = i / NGX, c0 = (i - ly * NGX) * GX;  // cells x = c0 - 1 ...
            const T* row = prim + (ly + H) * SX + (c0 - 1 + H);
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const T* q = row + f * SY * SX;
                T* o = slx + (f * TY + ly) * (TX + 2) + c0;
                T dl = q[0] - q[-1];
#pragma unroll
                for (int j = 0; j < GX; ++j) {
                    const T dr = q[j + 1] - q[j];
                    o[j] = minmod(dl, dr);
                    dl = dr;
                }
            }
        }
        for (int i = tid; i < NGY * TX; i += NT) {
            const int g = i / TX, lx = i - g * TX, r0 = g * GY;  // cells y = r0 - 1 ...
            const T* col = prim + (r0 - 1 + H) * SX + (lx + H);
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const T* q = col + f * SY * SX;
                T* o = sly + (f * (TY + 2) + r0) * TX + lx;
                T dl = q[0] - q[-SX];
#pragma unroll
                for (int j = 0; j < GY; ++j) {
                    const T dr = q[(j + 1) * SX] - q[j * SX];
                    o[j * TX] = minmod(dl, dr);
                    dl = dr;
                }
            }
        }
        __syncthreads();
    }

    // ---- F: faces ---------------------------------------------------------------------------
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
        // cells on either side: A (low) and B (high)
        const int ax = isx ? lx - 1 : lx, ay = isx ? ly : ly - 1;
        if (P.frozen && !cell_active(P, tx0 + ax, ty0 + ay) &&
            !cell_active(P, tx0 + lx, ty0 + ly))
            continue;  // no updated cell uses this face
        const T* pa = prim + (ay + H) * SX + (ax + H);
        const T* pb = pa + (isx ? 1 : SX);
        T qa[NF], qb[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const T ca = pa[f * SY * SX], cb = pb[f * SY * SX];
            if (ORDER == 2) {
                T da, db;
                if (isx) {
                    da = slx[(f * TY + ly) * (TX + 2) + lx];
                    db = slx[(f * TY + ly) * (TX + 2) + lx + 1];
                } else {
                    da = sly[(f * (TY + 2) + ly) * TX + lx];
                    db = sly[(f * (TY + 2) + ly + 1) * TX + lx];
                }
                T a = fma(0.5, da, ca), b = fma(-0.5, db, cb);
                if (f < 2) {  // rho, p fall back to the cell value (kernel.cu:3436-3470)
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
        T UU;
        const FluxE<T> F =
            P.method == GD_METHOD_HLL
                ? hll_local(qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2], qb[0], qb[1],
                            isx ? qb[2] : qb[3], isx ? qb[3] : qb[2], P, UU)
                : hllc_local(qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2], qb[0], qb[1],
                             isx ? qb[2] : qb[3], isx ? qb[3] : qb[2], P, UU);
        if (isx) {
            T* fo = fx + ly * (TX + 1) + lx;
            fo[0 * TY * (TX + 1)] = F.m;
            fo[1 * TY * (TX + 1)] = F.e;
            fo[2 * TY * (TX + 1)] = F.mn;  // x momentum
            fo[3 * TY * (TX + 1)] = F.mt;  // y momentum
            umax_x = max_nonneg(umax_x, value_of(UU));
        } else {
            T* fo = fy + ly * TX + lx;
            fo[0 * (TY + 1) * TX] = F.m;
            fo[1 * (TY + 1) * TX] = F.e;
            fo[2 * (TY + 1) * TX] = F.mt;  // x momentum
            fo[3 * (TY + 1) * TX] = F.mn;  // y momentum
            umax_y = max_nonneg(umax_y, value_of(UU));
        }
    }
    __syncthreads();

    // ---- U: update --------------------------------------------------------------------------
    const double kx = T_do * P.inv_dx, ky = T_do * P.inv_dy;
    bool any_active = false;
    unsigned int nfl_r = 0, nfl_p = 0, nbad = 0;
    for (int i = tid; i < TX * TY; i += NT) {
        const int ly = i / TX, lx = i - ly * TX;
        const int gx = tx0 + lx, gy = ty0 + ly;
        if (gx >= N || gy >= M) continue;
        const T* c = prim + (ly + H) * SX + (lx + H);
        const T r = c[0], p = c[SY * SX], u = c[2 * SY * SX], v = c[3 * SY * SX];
        const long long k = (long long)gy * N + gx;
        if (P.frozen && !cell_active(P, gx, gy)) {  // the faces' own test
            if (!dt_only) {
                store_cell2(out, k, 0, r, p);
                store_cell2(out, k, 2, u, v);
            }
            continue;
        }
        any_active = true;
        if (dt_only) continue;
        const T* fxc = fx + ly * (TX + 1) + lx;
        const T* fyc = fy + ly * TX + lx;
        T d[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const T* a = fxc + f * TY * (TX + 1);
            const T* b = fyc + f * (TY + 1) * TX;
            d[f] = fma(kx, a[1] - a[0], mulx(ky, b[TX] - b[0]));
        }
        if constexpr (std::is_same<T, double>::value) {
            if (aux != nullptr) {  // the recording of the adjoint: the flux differences used
                const long long KK = (long long)N * M;
#pragma unroll
                for (int f = 0; f < NF; ++f) aux[f * KK + k] = d[f];
            }
        }
        T r2 = r - d[0];
        if (le_zero(r2)) { r2 = cst<T>(0.0001); ++nfl_r; }
        const T inv = rcp_2op(r2);
        const T mx2 = fma(r, u, -d[2]), my2 = fma(r, v, -d[3]);
        const T u2 = mulx(mx2, inv);
        const T v2 = mulx(my2, inv);
        // p' = (gamma - 1) (E - d_E - K'/2) with E = p / (gamma - 1) + K / 2, K = rho |v|^2,
        // K' = rho' |v'|^2 = m' . v' (kernel.cu:1861-1870)
        const T K1 = r * fma(u, u, mulx(v, v));
        const T K2 = fma(mx2, u2, mulx(my2, v2));
        T p2 = fma(P.hgm1, K1 - K2, fma(-P.gm1, d[1], p));
        if (le_zero(p2)) { p2 = cst<T>(0.000001); ++nfl_p; }
        if (!finite_bits(r2) || !finite_bits(p2) || !finite_bits(u2) || !finite_bits(v2)) ++nbad;
        store_cell2(out, k, 0, r2, p2);
        store_cell2(out, k, 2, u2, v2);
    }
    res.umax_x = umax_x;
    res.umax_y = umax_y;
    res.any_active = any_active;
    res.nfl_r = nfl_r;
    res.nfl_p = nfl_p;
    res.nbad = nbad;
}

__device__ __forceinline__ void add_counters(Scalars* ctr, const TileResult& r) {
    if (ctr != nullptr && (r.nfl_r | r.nfl_p | r.nbad)) {
        if (r.nfl_r) atomicAdd(&ctr->rho_floor, (unsigned long long)r.nfl_r);
        if (r.nfl_p) atomicAdd(&ctr->p_floor, (unsigned long long)r.nfl_p);
        if (r.nbad) atomicAdd(&ctr->nonfinite, (unsigned long long)r.nbad);
    }
}

template <int ORDER, int TX, int TY>
__global__ void __launch_bounds__(NT) euler_fast_kernel(Params P, CPlanes in, Planes out,
                                                        const double* __restrict__ T_do_ptr,
                                                        unsigned long long* T_bits, Scalars* rot,
                                                        Scalars* ctr, int dt_only,
                                                        double* aux) {
    extern __shared__ double smem[];
    TileResult r;
    euler_tile<double, ORDER, TX, TY>(P, in, out, blockIdx.x * TX,
                                      (blockIdx.y + P.tile_row0) * TY, *T_do_ptr, dt_only, smem,
                                      r, aux);
    add_counters(ctr, r);
    block_dt_and_rotate<NT>(P, r.umax_x, r.umax_y, r.any_active, T_bits, rot, P.tile_nblocks);
}

// Tangent of one step: (U, dU) -> (U', dU') with the dt read from *T_do_ptr (held fixed):
// the same tile instantiated with Dual values.  32 x 8 tiles: a Dual tile holds twice the
// bytes of a double one (101 KB at second order), so two CTAs fit on an SM (at 32 x 16, 186 KB,
// one).
constexpr int kTanTX = 32, kTanTY = 8;
template <int ORDER>
__global__ void __launch_bounds__(NT) euler_tangent_kernel(Params P, CPlanes in, CPlanes din,
                                                           Planes out, Planes dout,
                                                           const double* __restrict__ T_do_ptr) {
    extern __shared__ __align__(16) double smem[];
    TileResult r;
    const DualIn I{in, din};
    const DualOut O{out, dout};
    euler_tile<Dual, ORDER, kTanTX, kTanTY>(P, I, O, blockIdx.x * kTanTX, blockIdx.y * kTanTY,
                                            *T_do_ptr, 0, reinterpret_cast<Dual*>(smem), r,
                                            nullptr);
}

// Persistent batched step: CTAs stride over the flattened (grid, tile) work list; each tile
// reports its dt to its own grid, and the last tile of a grid rotates that grid's dt.
// With dt_only, tiles only min-combine their dt (no state write, no rotation).
// `sc_override` (may be null) replaces every grid's scalars (the autotuner times steps
// without touching the real dt and time).
template <int ORDER, int TX, int TY>
__global__ void __launch_bounds__(NT) euler_batch_kernel(const BatchGrid* __restrict__ grids,
                                                         const int2* __restrict__ items,
                                                         int nitems, int cur, int dt_only,
                                                         Scalars* sc_override) {
    extern __shared__ double smem[];
    __shared__ BatchGrid g;
    __shared__ int tile;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        __syncthreads();  // the previous tile is done with smem and g
        if (threadIdx.x == 0) {
            const int2 w = items[it];
            g = grids[w.x];
            if (sc_override != nullptr) g.sc = sc_override + w.x;
            tile = w.y;
        }
        __syncthreads();
        const long long K = g.K;
        CPlanes in{};
        Planes out{};
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            in.f[f] = g.state[cur] + f * K;
            out.f[f] = g.state[cur ^ 1] + f * K;
        }
        const int tx0 = (tile % g.tiles_x) * TX, ty0 = (tile / g.tiles_x) * TY;
        const double T_do = g.sc->T_do;
        TileResult r;
        euler_tile<double, ORDER, TX, TY>(g.P, in, out, tx0, ty0, T_do, dt_only, smem, r,
                                          nullptr);
        add_counters(dt_only ? nullptr : g.sc, r);
        block_dt_and_rotate<NT>(g.P, r.umax_x, r.umax_y, r.any_active, &g.sc->T_bits,
                                dt_only ? nullptr : g.sc, (unsigned int)g.ntiles);
    }
}

template <int ORDER, int TX, int TY>
cudaError_t set_attrs() {
    cudaError_t e = cudaFuncSetAttribute(euler_fast_kernel<ORDER, TX, TY>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)Shape<ORDER, TX, TY>::bytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(euler_batch_kernel<ORDER, TX, TY>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)Shape<ORDER, TX, TY>::bytes);
}

template <int ORDER, int TX, int TY>
cudaError_t launch_single(const Params& P, const CPlanes& in, const Planes& out,
                          const double* T_do, unsigned long long* T_bits, Scalars* rot,
                          Scalars* ctr, int dt_only, cudaStream_t st, double* aux = nullptr) {
    dim3 grid((P.N + TX - 1) / TX, P.tile_rows ? P.tile_rows : (P.M + TY - 1) / TY);
    euler_fast_kernel<ORDER, TX, TY><<<grid, NT, Shape<ORDER, TX, TY>::bytes, st>>>(
        P, in, out, T_do, T_bits, rot, ctr, dt_only, aux);
    return cudaGetLastError();
}

template <int ORDER, int TX, int TY>
cudaError_t launch_batch(const BatchGrid* grids, const int2* items, int nitems, int cur,
                         int dt_only, Scalars* sc_override, int ctas, cudaStream_t st) {
    euler_batch_kernel<ORDER, TX, TY><<<ctas, NT, Shape<ORDER, TX, TY>::bytes, st>>>(
        grids, items, nitems, cur, dt_only, sc_override);
    return cudaGetLastError();
}

// tile shapes of the variants: 0: 16x16 (the single-grid step's), 1: 32x8, 2: 32x16, 3: 64x8
#define GD_EULER_DISPATCH(ORDER, VAR, CALL, ARGS) \
    switch (VAR) {                                \
        case 1: return CALL<ORDER, 32, 8> ARGS;   \
        case 2: return CALL<ORDER, 32, 16> ARGS;  \
        case 3: return CALL<ORDER, 64, 8> ARGS;   \
        default: return CALL<ORDER, 16, 16> ARGS; \
    }

}  // namespace

void euler_tile_shape(int variant, int* tx, int* ty) {
    static const int shapes[kEulerVariants][2] = {{16, 16}, {32, 8}, {32, 16}, {64, 8}};
    const int v = (variant >= 0 && variant < kEulerVariants) ? variant : 0;
    *tx = shapes[v][0];
    *ty = shapes[v][1];
}

size_t euler_smem_bytes(int order, int variant) {
    switch (variant) {
        case 1: return order == 1 ? Shape<1, 32, 8>::bytes : Shape<2, 32, 8>::bytes;
        case 2: return order == 1 ? Shape<1, 32, 16>::bytes : Shape<2, 32, 16>::bytes;
        case 3: return order == 1 ? Shape<1, 64, 8>::bytes : Shape<2, 64, 8>::bytes;
        default: return order == 1 ? Shape<1, 16, 16>::bytes : Shape<2, 16, 16>::bytes;
    }
}

namespace {
template <int ORDER, int TX, int TY>
int blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, euler_batch_kernel<ORDER, TX, TY>, NT,
                                                      Shape<ORDER, TX, TY>::bytes) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}
}  // namespace

int euler_batch_blocks_per_sm(int order, int variant) {
    if (order == 1) {
        switch (variant) {
            case 1: return blocks_per_sm<1, 32, 8>();
            case 2: return blocks_per_sm<1, 32, 16>();
            case 3: return blocks_per_sm<1, 64, 8>();
            default: return blocks_per_sm<1, 16, 16>();
        }
    }
    switch (variant) {
        case 1: return blocks_per_sm<2, 32, 8>();
        case 2: return blocks_per_sm<2, 32, 16>();
        case 3: return blocks_per_sm<2, 64, 8>();
        default: return blocks_per_sm<2, 16, 16>();
    }
}

cudaError_t prepare_euler_fast() {
    cudaError_t e = set_attrs<1, 32, 16>();
    if (e == cudaSuccess)  // Dual tiles: twice the bytes of the double ones
        e = cudaFuncSetAttribute(euler_tangent_kernel<1>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(2 * Shape<1, kTanTX, kTanTY>::bytes));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(euler_tangent_kernel<2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(2 * Shape<2, kTanTX, kTanTY>::bytes));
    if (e == cudaSuccess) e = set_attrs<2, 32, 16>();
    if (e == cudaSuccess) e = set_attrs<1, 32, 8>();
    if (e == cudaSuccess) e = set_attrs<2, 32, 8>();
    if (e == cudaSuccess) e = set_attrs<1, 16, 16>();
    if (e == cudaSuccess) e = set_attrs<2, 16, 16>();
    if (e == cudaSuccess) e = set_attrs<1, 64, 8>();
    if (e == cudaSuccess) e = set_attrs<2, 64, 8>();
    return e;
}

cudaError_t launch_euler_fast_v(int variant, const Params& P, const CPlanes& in,
                                const Planes& out, const double* T_do,
                                unsigned long long* T_bits, Scalars* rot, Scalars* ctr,
                                int dt_only, cudaStream_t st) {
    if (P.order == 1) {
        GD_EULER_DISPATCH(1, variant, launch_single,
                          (P, in, out, T_do, T_bits, rot, ctr, dt_only, st));
    }
    GD_EULER_DISPATCH(2, variant, launch_single, (P, in, out, T_do, T_bits, rot, ctr, dt_only, st));
}

cudaError_t launch_euler_fast(const Params& P, const CPlanes& in, const Planes& out,
                              const double* T_do, unsigned long long* T_bits, Scalars* rot,
                              Scalars* ctr, int dt_only, cudaStream_t st) {
    return launch_euler_fast_v(0, P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
}

cudaError_t launch_euler_tangent(const Params& P, const CPlanes& in, const CPlanes& din,
                                 const Planes& out, const Planes& dout, const double* T_do,
                                 cudaStream_t st) {
    const dim3 grid((P.N + kTanTX - 1) / kTanTX, (P.M + kTanTY - 1) / kTanTY);
    if (P.order == 1)
        euler_tangent_kernel<1><<<grid, NT, 2 * Shape<1, kTanTX, kTanTY>::bytes, st>>>(
            P, in, din, out, dout, T_do);
    else
        euler_tangent_kernel<2><<<grid, NT, 2 * Shape<2, kTanTX, kTanTY>::bytes, st>>>(
            P, in, din, out, dout, T_do);
    return cudaGetLastError();
}

cudaError_t launch_euler_fast_aux(const Params& P, const CPlanes& in, const Planes& out,
                                  const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                  Scalars* ctr, double* aux, cudaStream_t st) {
    // variant 0, the launch gd_advance makes: the recorded step is the plain step
    if (P.order == 1)
        return launch_single<1, 16, 16>(P, in, out, T_do, T_bits, rot, ctr, 0, st, aux);
    return launch_single<2, 16, 16>(P, in, out, T_do, T_bits, rot, ctr, 0, st, aux);
}

cudaError_t launch_euler_batch(int variant, int order, const BatchGrid* grids, const int2* items,
                               int nitems, int cur, int dt_only, Scalars* sc_override, int ctas,
                               cudaStream_t st) {
    if (order == 1) {
        GD_EULER_DISPATCH(1, variant, launch_batch,
                          (grids, items, nitems, cur, dt_only, sc_override, ctas, st));
    }
    GD_EULER_DISPATCH(2, variant, launch_batch,
                      (grids, items, nitems, cur, dt_only, sc_override, ctas, st));
}


namespace {
// One face per thread through the step's own face solver (hllc_local / hll_local): L, R are
// n x 4 (rho, p, vx, vy); flux n x 4 (mass, energy, x momentum, y momentum), the reference's
// HLLC_Aleksashov output order; speed n values max(|S_L|, |S_R|).  axis 0: normal +x.
__global__ void euler_face_probe_kernel(Params P, long long n, int axis,
                                        const double* __restrict__ L,
                                        const double* __restrict__ R, double* flux,
                                        double* speed) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* a = L + 4 * i;
    const double* b = R + 4 * i;
    const bool isx = axis == 0;
    double UU;
    const FluxE<double> F =
        P.method == GD_METHOD_HLL
            ? hll_local(a[0], a[1], isx ? a[2] : a[3], isx ? a[3] : a[2], b[0], b[1],
                        isx ? b[2] : b[3], isx ? b[3] : b[2], P, UU)
            : hllc_local(a[0], a[1], isx ? a[2] : a[3], isx ? a[3] : a[2], b[0], b[1],
                         isx ? b[2] : b[3], isx ? b[3] : b[2], P, UU);
    double* o = flux + 4 * i;
    o[0] = F.m;
    o[1] = F.e;
    o[2] = isx ? F.mn : F.mt;
    o[3] = isx ? F.mt : F.mn;
    speed[i] = dabs(UU);
}
}  // namespace

cudaError_t launch_euler_face_probe(const Params& P, long long n, int axis, const double* L,
                                    const double* R, double* flux, double* speed,
                                    cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const long long blocks = (n + 255) / 256;
    euler_face_probe_kernel<<<(unsigned int)blocks, 256, 0, st>>>(P, n, axis, L, R, flux, speed);
    return cudaGetLastError();
}

}  // namespace gd
