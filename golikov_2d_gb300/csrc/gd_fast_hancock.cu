// gd_fast_hancock.cu -- fast MUSCL-Hancock step (Kernel_GKR, kernel.cu:2663-3284): the
// predictor-corrector with HLLD faces, face-once on tiles, FMA contraction, field in
// Heaviside-Lorentz units (b = B / sqrt(4 pi)).
//
// The reference evaluates, for every cell, the half-step predictions of itself and of its
// four neighbours, so each prediction is computed five times and each face twice.  Away
// from the edges a cell's view of a neighbour's prediction is the neighbour's own (same
// stencil points), so here every prediction is computed once per tile and every face once.
// That holds for the cells with 2 <= n < N-2 and 2 <= m < M-2 (the "interior"); along the
// edges the reference's substitutes depend on the asking cell (see gd_hancock_cell.cuh), and
// the two-cell band is computed cell by cell exactly as the reference does.  Two launches:
//   hancock_band_kernel   the band cells, per cell (hancock_cell of gd_hancock_cell.cuh)
//   hancock_tile_kernel   32 x 8 interior tiles:
//     L  state of the tile + 2 halo (cross-shaped), B -> b
//     P  per cell of the tile + 1 halo: minmod slopes, the predictor's four physical fluxes
//        (POTOK_Korolkov, Gas_Dinamic.cu:70-180, written in x / y components) and
//        sources, the half-step mean A = (Q + QQ)/2
//     F  each face once: HLLD between A_L + D_L/2 and A_R - D_R/2 (gd_mhd_flux.cuh)
//     U  the corrector of kernel.cu:3256-3281 (Pdiv = 0) from A and the four faces
// Given a side stream, the band kernel runs on it concurrently with the tile kernel (they
// write disjoint cells); the blocks of both share one ticket, and the last block of either to
// finish performs the funk_time rotation.
//
// Differences from the parity step are rounding only: contraction, reciprocals instead of
// divisions, slopes minmod(a - b, b - c) instead of h minmod((a - b)/h, (b - c)/h), the
// neighbour's prediction at its own radius y_{m+-1} instead of y -+ dy, and the face solved
// once (its two sides see the same flux up to rounding of the solver's symmetry).
#include "gd_hancock_cell.cuh"
#include "gd_internal.cuh"
#include "gd_kernels.h"
#include "gd_mhd_flux.cuh"

namespace gd {
namespace {

constexpr int TX = 32, TY = 8, NT = TX * TY;  // one interior cell per thread in U
constexpr int NF = 7;                          // rho, p, vx, vy, bx, by, bz
constexpr int RX = TX + 4, RY = TY + 4;        // state: tile + 2
constexpr int PX = TX + 2, PY = TY + 2;        // predictions: tile + 1
constexpr int kRaw = NF * RY * RX;
constexpr int kPred = NF * PY * PX;            // one array each of A, DX, DY
constexpr int NFX = (TX + 1) * TY, NFY = TX * (TY + 1);
constexpr int kFx = NF * NFX, kFy = NF * NFY;
constexpr int kUnion = kRaw > kFx + kFy ? kRaw : kFx + kFy;  // state, later the fluxes
constexpr size_t kSmemBytes = sizeof(double) * (kUnion + 3 * kPred + 2 * PY + TX) + TX * TY;

constexpr int BNT = 128;  // band kernel

// Half the jump F(m + h) - F(m - h) of the physical flux through a face, in its local frame
// (normal velocity u, tangential v, no z velocity; field bn, bt, bz in b units), by the product
// rule: the predictor's flux differences of kernel.cu:1611-1720 without forming the two
// fluxes (no cancellation between them).  For a product, (a + x)(b + y) - (a - x)(b - y) =
// 2 (a y + x b); the cubic and quartic terms expand the same way.  G = gamma / (gamma - 1).
// Components: mass, energy, normal and tangential momentum, tangential and z field (the normal
// field's flux is 0).
struct FluxJump {
    double m, e, mn, mt, bt, bz;
};
__device__ __forceinline__ FluxJump flux_jump(double r, double p, double u, double v, double bn,
                                              double bt, double bz, double rh, double ph,
                                              double uh, double vh, double bnh, double bth,
                                              double bzh, double G) {
    FluxJump J;
    const double ru = r * u;
    const double A0 = fma(r, uh, rh * u);  // half the jump of r u
    const double rhuh = rh * uh;
    const double u2 = fma(u, u, uh * uh);
    J.m = A0;
    // r u^2 + p + (bt^2 + bz^2 - bn^2) / 2
    J.mn = fma(bt, bth, fma(bz, bzh, fma(-bn, bnh, fma(rh, u2, fma(twice_exact(ru), uh, ph)))));
    // r u v - bn bt
    const double X = fma(bn, bth, bnh * bt);
    J.mt = fma(ru, vh, fma(A0, v, fma(rhuh, vh, -X)));
    // u bt - v bn; u bz
    J.bt = fma(u, bth, fma(uh, bt, -fma(v, bnh, vh * bn)));
    J.bz = fma(u, bzh, uh * bz);
    // energy: G p u + r u (u^2 + v^2) / 2 + u (bt^2 + bz^2) - v bn bt
    const double S = u2 + fma(v, v, vh * vh);
    const double kin = fma(half_exact(A0), S, (ru + rhuh) * fma(u, uh, v * vh));
    const double Tb = fma(bt, bth, bz * bzh);
    const double Sb = fma(bt, bt, fma(bth, bth, fma(bz, bz, bzh * bzh)));
    const double Y = fma(bn, bt, bnh * bth);
    J.e = fma(G, fma(p, uh, ph * u),
              fma(twice_exact(u), Tb, fma(uh, Sb, fma(-v, X, fma(-vh, Y, kin)))));
    return J;
}

// The predictor's face states Q +- D/2 as mean m and half-difference h: rho and p from the
// two states with the reference's fallback to Q where <= 0 (kernel.cu:1640-1680); the other
// fields m = Q, h = D/2 exactly.
__device__ __forceinline__ void mean_half(const double* Q, const double* D, double* m,
                                          double* h) {
#pragma unroll
    for (int f = 0; f < 2; ++f) {
        double a = fma(0.5, D[f], Q[f]), b = fma(-0.5, D[f], Q[f]);
        a = le_zero(a) ? Q[f] : a;
        b = le_zero(b) ? Q[f] : b;
        m[f] = half_exact(a + b);
        h[f] = half_exact(a - b);
    }
#pragma unroll
    for (int f = 2; f < NF; ++f) {
        m[f] = Q[f];
        h[f] = half_exact(D[f]);
    }
}

template <bool VYP>
__global__ void __launch_bounds__(NT) hancock_tile_kernel(Params P, CPlanes in, Planes out,
                                                          const double* __restrict__ T_do_ptr,
                                                          unsigned long long* T_bits,
                                                          Scalars* rot, Scalars* ctr,
                                                          int dt_only, unsigned int nblocks) {
    extern __shared__ __align__(16) double smem[];
    double* raw = smem;            // [NF][RY][RX], then fx [NF][TY][TX+1], fy [NF][TY+1][TX]
    double* fx = smem;
    double* fy = smem + kFx;
    double* pA = smem + kUnion;    // [NF][PY][PX]
    double* pDX = pA + kPred;
    double* pDY = pDX + kPred;
    double* rowy = pDY + kPred;    // radius of prediction rows
    double* rowiy = rowy + PY;     // its reciprocal
    double* colx = rowiy + PY;     // x of the tile's columns
    unsigned char* flag = reinterpret_cast<unsigned char*>(colx + TX);  // [TY][TX]

    const int tid = threadIdx.x;
    const int N = P.N, M = P.M;
    const int tx0 = 2 + blockIdx.x * TX, ty0 = 2 + (blockIdx.y + P.tile_row0) * TY;
    const double ig = P.inv_gm1;

    // ---- L: state of the tile + 2 halo; corner blocks the stencils never reach are skipped
    for (int i = tid; i < RY * RX; i += NT) {
        const int ly = i / RX, lx = i - ly * RX;
        if ((lx == 0 || lx == RX - 1) && (ly < 2 || ly >= TY + 2)) continue;
        if ((ly == 0 || ly == RY - 1) && (lx < 2 || lx >= TX + 2)) continue;
        const int gx = tx0 + lx - 2, gy = ty0 + ly - 2;
        double v[NF];
        if (gx >= 0 && gx < N && gy >= 0 && gy < M) {
            const long long k = (long long)gy * N + gx;
#pragma unroll
            for (int f = 0; f < NF; ++f) v[f] = load_f(in, f, k);
            v[4] *= kInvSpi4;
            v[5] *= kInvSpi4;
            v[6] *= kInvSpi4;
        } else {
            // outside the grid: only predictions that no interior face uses read these
#pragma unroll
            for (int f = 0; f < NF; ++f) v[f] = f < 2 ? 1.0 : 0.0;
        }
#pragma unroll
        for (int f = 0; f < NF; ++f) raw[(f * RY + ly) * RX + lx] = v[f];
    }
    if (tid < PY) {
        const double y = hancock_y(P, ty0 + tid - 1);
        rowy[tid] = y;
        rowiy[tid] = 1.0 / y;
    } else if (tid >= 32 && tid < 32 + TX) {
        colx[tid - 32] = hancock_x(P, tx0 + tid - 32);
    }
    __syncthreads();
    // this thread's cell: 0 outside the interior, 1 interior and frozen, 2 interior, updated
    const int cx = tid % TX, cy = tid / TX;
    const int gx = tx0 + cx, gy = ty0 + cy;
    int my_flag = 0;
    if (gx < N - 2 && gy < M - 2) my_flag = hancock_frozen_fast(P, colx[cx], rowy[cy + 1]) ? 1 : 2;
    flag[tid] = (unsigned char)my_flag;

    // ---- P: predictions of the tile + 1 halo (not its corners) ---------------------------
    const double T_do = *T_do_ptr;
    const double st = 0.5 * T_do;
    const double sx = st * P.inv_dx, sy = st * P.inv_dy;
    const double sx2 = twice_exact(sx), sy2 = twice_exact(sy);
    for (int i = tid; i < PY * PX; i += NT) {
        const int py = i / PX, px = i - py * PX;
        if ((px == 0 || px == PX - 1) && (py == 0 || py == PY - 1)) continue;
        const double* c = raw + (py + 1) * RX + (px + 1);
        constexpr int PS = RY * RX;
        double Q[NF], DX[NF], DY[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const double* q = c + f * PS;
            Q[f] = q[0];
            DX[f] = minmod(q[1] - q[0], q[0] - q[-1]);
            DY[f] = minmod(q[RX] - q[0], q[0] - q[-RX]);
        }
        if (VYP) {
            DX[3] = DX[1];
            DY[3] = DY[1];
        }
        // predictor (kernel.cu:1611-1720): the flux differences of the face states Q +- D/2,
        // 2 sx J_x + 2 sy J_y with J the half jumps (x: normal u, field bx; y: normal v, by)
        double d[NF];
        {
            double m[NF], h[NF];
            mean_half(Q, DX, m, h);
            const FluxJump Jx = flux_jump(m[0], m[1], m[2], m[3], m[4], m[5], m[6], h[0], h[1],
                                          h[2], h[3], h[4], h[5], h[6], P.g_gm1);
            mean_half(Q, DY, m, h);
            const FluxJump Jy = flux_jump(m[0], m[1], m[3], m[2], m[5], m[4], m[6], h[0], h[1],
                                          h[3], h[2], h[5], h[4], h[6], P.g_gm1);
            d[0] = fma(sy2, Jy.m, sx2 * Jx.m);
            d[1] = fma(sy2, Jy.e, sx2 * Jx.e);
            d[2] = fma(sy2, Jy.mt, sx2 * Jx.mn);
            d[3] = fma(sy2, Jy.mn, sx2 * Jx.mt);
            d[4] = sy2 * Jy.bt;
            d[5] = sx2 * Jx.bt;
            d[6] = fma(sy2, Jy.bz, sx2 * Jx.bz);
        }
        const double sty = st * rowiy[py];
        const double r = Q[0], p = Q[1], u = Q[2], v = Q[3], bx = Q[4], by = Q[5], bz = Q[6];
        const double bb = fma(bz, bz, fma(by, by, bx * bx));
        const double U = fma(p, ig, 0.5 * fma(r, fma(u, u, v * v), bb));
        double r2 = fma(-sty * r, v, r - d[0]);
        r2 = le_zero(r2) ? r : r2;
        const double ir2 = rcp_fast(r2);
        const double u2 = fma(-sty, fma(r * u, v, -bx * by), fma(r, u, -d[2])) * ir2;
        const double v2 = fma(-sty, fma(r * v, v, fma(bz, bz, -by * by)), fma(r, v, -d[3])) * ir2;
        const double bx2 = fma(-sty, fma(v, bx, -by * u), bx - d[4]);
        const double by2 = by - d[5];
        const double bz2 = bz - d[6];
        const double E2 =
            fma(-sty, fma(U + p + 0.5 * bb, v, -by * fma(u, bx, v * by)), U - d[1]);
        double p2 = (E2 - 0.5 * fma(r2, fma(u2, u2, v2 * v2),
                                    fma(bz2, bz2, fma(by2, by2, bx2 * bx2)))) * P.gm1;
        p2 = le_zero(p2) ? 0.000001 : p2;
        const double QQ[NF] = {r2, p2, u2, v2, bx2, by2, bz2};
        const int o = py * PX + px;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            pA[f * PY * PX + o] = 0.5 * (Q[f] + QQ[f]);
            pDX[f * PY * PX + o] = DX[f];
            pDY[f * PY * PX + o] = DY[f];
        }
    }
    __syncthreads();

    // ---- F: each face of an updated cell once -------------------------------------------
    double umax_x = 0.0, umax_y = 0.0;
    for (int i = tid; i < NFX + NFY; i += NT) {
        const bool isx = i < NFX;
        int lx, ly, pa, pb;
        if (isx) {
            ly = i / (TX + 1);
            lx = i - ly * (TX + 1);
            const bool need = (lx > 0 && flag[ly * TX + lx - 1] == 2) ||
                              (lx < TX && flag[ly * TX + lx] == 2);
            if (!need) continue;
            pa = (ly + 1) * PX + lx;  // cell lx-1 of the tile
            pb = pa + 1;
        } else {
            const int j = i - NFX;
            ly = j / TX;
            lx = j - ly * TX;
            const bool need = (ly > 0 && flag[(ly - 1) * TX + lx] == 2) ||
                              (ly < TY && flag[ly * TX + lx] == 2);
            if (!need) continue;
            pa = ly * PX + lx + 1;  // cell (lx, ly-1) of the tile
            pb = pa + PX;
        }
        const double* D = isx ? pDX : pDY;
        double qa[NF], qb[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            const double Aa = pA[f * PY * PX + pa], Ab = pA[f * PY * PX + pb];
            qa[f] = fma(0.5, D[f * PY * PX + pa], Aa);
            qb[f] = fma(-0.5, D[f * PY * PX + pb], Ab);
            if (f < 2) {
                qa[f] = le_zero(qa[f]) ? Aa : qa[f];
                qb[f] = le_zero(qb[f]) ? Ab : qb[f];
            }
        }
        // local frame: x-face (n, t) = (x, y); y-face (n, t) = (y, x); z stays z
        Side<double> A, B;
        side(A, qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2], isx ? qa[4] : qa[5],
             isx ? qa[5] : qa[4], qa[6], P);
        side(B, qb[0], qb[1], isx ? qb[2] : qb[3], isx ? qb[3] : qb[2], isx ? qb[4] : qb[5],
             isx ? qb[5] : qb[4], qb[6], P);
        double UU;
        const FluxM<double> F = hlld_local(A, B, GD_METHOD_HLLD, P, UU);
        if (isx) {
            double* fo = fx + ly * (TX + 1) + lx;
            fo[0 * NFX] = F.m;
            fo[1 * NFX] = F.e;
            fo[2 * NFX] = F.mn;
            fo[3 * NFX] = F.mt;
            fo[4 * NFX] = F.bn;
            fo[5 * NFX] = F.bt;
            fo[6 * NFX] = F.bz;
            umax_x = max_nonneg(umax_x, UU);
        } else {
            double* fo = fy + ly * TX + lx;
            fo[0 * NFY] = F.m;
            fo[1 * NFY] = F.e;
            fo[2 * NFY] = F.mt;
            fo[3 * NFY] = F.mn;
            fo[4 * NFY] = F.bt;
            fo[5 * NFY] = F.bn;
            fo[6 * NFY] = F.bz;
            umax_y = max_nonneg(umax_y, UU);
        }
    }
    __syncthreads();

    // ---- U: corrector (kernel.cu:3256-3281, Pdiv = 0) --------------------------------------
    unsigned int nfl_r = 0, nfl_p = 0, nbad = 0;
    if (my_flag == 1 && !dt_only) {
        const long long k = (long long)gy * N + gx;
#pragma unroll
        for (int f = 0; f < NF; ++f) store_f(out, f, k, load_f(in, f, k));
    } else if (my_flag == 2 && !dt_only) {
        const double hT = 0.5 * T_do;
        const double kx = hT * P.inv_dx, ky = hT * P.inv_dy;
        const double hTy = hT * rowiy[cy + 1];
        const int o = (cy + 1) * PX + (cx + 1);
        double A[NF], d[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            A[f] = pA[f * PY * PX + o];
            const double* a = fx + f * NFX + cy * (TX + 1) + cx;
            const double* b = fy + f * NFY + cy * TX + cx;
            d[f] = fma(kx, a[1] - a[0], ky * (b[TX] - b[0]));
        }
        const double r = A[0], p = A[1], u = A[2], v = A[3], bx = A[4], by = A[5], bz = A[6];
        const double bb = fma(bz, bz, fma(by, by, bx * bx));
        const double U = fma(p, ig, 0.5 * fma(r, fma(u, u, v * v), bb));
        double r2 = fma(-hTy * r, v, r - d[0]);
        if (le_zero(r2)) {
            r2 = r;
            ++nfl_r;
        }
        const double ir2 = rcp_fast(r2);
        const double u2 = fma(-hTy, fma(r * u, v, -bx * by), fma(r, u, -d[2])) * ir2;
        const double v2 = fma(-hTy, fma(r * v, v, fma(bz, bz, -by * by)), fma(r, v, -d[3])) * ir2;
        const double bx2 = fma(-hTy, fma(v, bx, -by * u), bx - d[4]);
        const double by2 = by - d[5];
        const double bz2 = bz - d[6];
        const double E2 =
            fma(-hTy, fma(U + p + 0.5 * bb, v, -by * fma(u, bx, v * by)), U - d[1]);
        double p2 = (E2 - 0.5 * fma(r2, fma(u2, u2, v2 * v2),
                                    fma(bz2, bz2, fma(by2, by2, bx2 * bx2)))) * P.gm1;
        if (le_zero(p2)) {
            p2 = 0.000001;
            ++nfl_p;
        }
        if (!finite_bits(r2) || !finite_bits(p2) || !finite_bits(u2) || !finite_bits(v2) ||
            !finite_bits(bx2) || !finite_bits(by2) || !finite_bits(bz2))
            ++nbad;
        const long long k = (long long)gy * N + gx;
        store_f(out, 0, k, r2);
        store_f(out, 1, k, p2);
        store_f(out, 2, k, u2);
        store_f(out, 3, k, v2);
        store_f(out, 4, k, bx2 * kSpi4);
        store_f(out, 5, k, by2 * kSpi4);
        store_f(out, 6, k, bz2 * kSpi4);
    }
    if (ctr != nullptr && (nfl_r | nfl_p | nbad)) {
        if (nfl_r) atomicAdd(&ctr->rho_floor, (unsigned long long)nfl_r);
        if (nfl_p) atomicAdd(&ctr->p_floor, (unsigned long long)nfl_p);
        if (nbad) atomicAdd(&ctr->nonfinite, (unsigned long long)nbad);
    }
    const bool any_active = __syncthreads_or(my_flag == 2) != 0;
    block_dt_and_rotate<NT>(P, umax_x, umax_y, any_active, T_bits, rot, nblocks);
}

// The edge cells of rows [r0, r1): rows m < 2 and m >= M-2 whole, and the columns n < 2 and
// n >= N-2 of the rows between.
struct Band {
    int lo0, nlo;    // whole rows [lo0, lo0 + nlo) at the bottom
    int hi0, nhi;    // whole rows [hi0, hi0 + nhi) at the top
    int mid0, nmid;  // rows [mid0, mid0 + nmid) between, their edge columns only
    int cols_lo, cols_hi0, ncols;
    int total;
};

int clamp_count(int a, int b) { return b > a ? b - a : 0; }

Band make_band(int N, int M, int r0, int r1) {
    Band b;
    const int bot = M < 2 ? M : 2;           // rows [0, bot) are whole
    const int top = M - 2 > 2 ? M - 2 : 2;   // rows [top, M) are whole
    b.lo0 = r0;
    b.nlo = clamp_count(r0, r1 < bot ? r1 : bot);
    b.hi0 = r0 > top ? r0 : top;
    b.nhi = clamp_count(b.hi0, r1 < M ? r1 : M);
    b.mid0 = r0 > bot ? r0 : bot;
    b.nmid = clamp_count(b.mid0, r1 < top ? r1 : top);
    b.cols_lo = N < 2 ? N : 2;
    b.cols_hi0 = N - 2 > 2 ? N - 2 : 2;
    b.ncols = b.cols_lo + (N - b.cols_hi0);
    b.total = (b.nlo + b.nhi) * N + b.nmid * b.ncols;
    return b;
}

template <bool VYP>
__global__ void __launch_bounds__(BNT) hancock_band_kernel(Params P, CPlanes in, Planes out,
                                                           const double* __restrict__ T_do_ptr,
                                                           unsigned long long* T_bits,
                                                           Scalars* rot, Scalars* ctr,
                                                           int dt_only, Band b,
                                                           unsigned int nblocks) {
    const int i = blockIdx.x * BNT + threadIdx.x;
    double tmin = kCellTmin0;
    bool active = false;
    unsigned int nfl_r = 0, nfl_p = 0, nbad = 0;
    if (i < b.total) {
        int n, m;
        if (i < (b.nlo + b.nhi) * P.N) {
            const int r = i / P.N;
            n = i - r * P.N;
            m = r < b.nlo ? b.lo0 + r : b.hi0 + (r - b.nlo);
        } else {
            const int j = i - (b.nlo + b.nhi) * P.N;
            const int r = j / b.ncols, c = j - r * b.ncols;
            m = b.mid0 + r;
            n = c < b.cols_lo ? c : b.cols_hi0 + (c - b.cols_lo);
        }
        const long long k = (long long)m * P.N + n;
        const double y = hancock_y(P, m);
        if (hancock_frozen(P, n, y)) {
            if (!dt_only)
                for (int f = 0; f < NF; ++f) store_f(out, f, k, load_f(in, f, k));
        } else {
            active = true;
            double res[NF];
            tmin = hancock_cell<VYP>(P, in, n, m, y, *T_do_ptr, res, nfl_r, nfl_p);
            if (!dt_only) {
                for (int f = 0; f < NF; ++f) {
                    if (!finite_bits(res[f])) {
                        ++nbad;
                        break;
                    }
                }
                for (int f = 0; f < NF; ++f) store_f(out, f, k, res[f]);
            }
        }
    }
    if (ctr != nullptr && !dt_only && (nfl_r | nfl_p | nbad)) {
        if (nfl_r) atomicAdd(&ctr->rho_floor, (unsigned long long)nfl_r);
        if (nfl_p) atomicAdd(&ctr->p_floor, (unsigned long long)nfl_p);
        if (nbad) atomicAdd(&ctr->nonfinite, (unsigned long long)nbad);
    }
    block_tmin_and_rotate<BNT>(tmin, active, T_bits, rot, nblocks);
}

// Interior tile rows (at least one launch row, so a step always has a tile block) and the
// tile rows [t0, t1) of the rows [r0, r1), whose ends are 0, M or 2 + a multiple of TY.
int tile_rows_all(const Params& P) { return P.M - 4 > 0 ? (P.M - 4 + TY - 1) / TY : 1; }
void tile_range(const Params& P, int r0, int r1, int* t0, int* t1) {
    *t0 = r0 <= 2 ? 0 : (r0 - 2) / TY;
    *t1 = r1 >= P.M ? tile_rows_all(P) : (r1 - 2) / TY;
}
int tile_cols(const Params& P) { return P.N - 4 > 0 ? (P.N - 4 + TX - 1) / TX : 1; }

template <bool VYP>
cudaError_t launch_rows(const Params& P0, const CPlanes& in, const Planes& out,
                        const double* T_do, unsigned long long* T_bits, Scalars* rot,
                        Scalars* ctr, int r0, int r1, unsigned int nblocks, int parts,
                        cudaStream_t st) {
    const Band b = make_band(P0.N, P0.M, r0, r1);
    int t0, t1;
    tile_range(P0, r0, r1, &t0, &t1);
    Params P = P0;
    P.tile_row0 = t0;
    if ((parts & 1) && b.total > 0)
        hancock_band_kernel<VYP><<<(b.total + BNT - 1) / BNT, BNT, 0, st>>>(
            P, in, out, T_do, T_bits, rot, ctr, 0, b, nblocks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !(parts & 2) || t1 <= t0) return e;
    hancock_tile_kernel<VYP><<<dim3(tile_cols(P), t1 - t0), NT, kSmemBytes, st>>>(
        P, in, out, T_do, T_bits, rot, ctr, 0, nblocks);
    return cudaGetLastError();
}

template <bool VYP>
cudaError_t launch_v(const Params& P, const CPlanes& in, const Planes& out, const double* T_do,
                     unsigned long long* T_bits, Scalars* rot, Scalars* ctr, int dt_only,
                     cudaStream_t st, const HancockStreams* side) {
    const Band b = make_band(P.N, P.M, 0, P.M);
    const unsigned int band_blocks = (b.total + BNT - 1) / BNT;
    const int nx = tile_cols(P), ny = tile_rows_all(P);
    const unsigned int total = band_blocks + (unsigned int)(nx * ny);
    cudaStream_t bs = st;
    cudaError_t e;
    if (side != nullptr) {
        e = cudaEventRecord(side->fork, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side->stream, side->fork, 0);
        if (e != cudaSuccess) return e;
        bs = side->stream;
    }
    hancock_band_kernel<VYP><<<band_blocks, BNT, 0, bs>>>(P, in, out, T_do, T_bits, rot, ctr,
                                                          dt_only, b, total);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hancock_tile_kernel<VYP><<<dim3(nx, ny), NT, kSmemBytes, st>>>(P, in, out, T_do, T_bits, rot,
                                                                   ctr, dt_only, total);
    e = cudaGetLastError();
    if (e != cudaSuccess || side == nullptr) return e;
    e = cudaEventRecord(side->join, side->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, side->join, 0);
    return e;
}

}  // namespace

cudaError_t prepare_hancock_fast() {
    cudaError_t e = cudaFuncSetAttribute(hancock_tile_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSmemBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(hancock_tile_kernel<false>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
    return e;
}

int hancock_tile_height() { return TY; }

unsigned int hancock_fast_blocks(const Params& P, int r0, int r1, int parts) {
    const Band b = make_band(P.N, P.M, r0, r1);
    int t0, t1;
    tile_range(P, r0, r1, &t0, &t1);
    return ((parts & 1) ? (unsigned int)((b.total + BNT - 1) / BNT) : 0u) +
           ((parts & 2) && t1 > t0 ? (unsigned int)((t1 - t0) * tile_cols(P)) : 0u);
}

cudaError_t launch_hancock_fast_rows(const Params& P, const CPlanes& in, const Planes& out,
                                     const double* T_do, unsigned long long* T_bits,
                                     Scalars* rot, Scalars* ctr, int r0, int r1,
                                     unsigned int nblocks, int parts, cudaStream_t st) {
    if (P.scheme == GD_SCHEME_HANCOCK_REF)
        return launch_rows<true>(P, in, out, T_do, T_bits, rot, ctr, r0, r1, nblocks, parts,
                                 st);
    return launch_rows<false>(P, in, out, T_do, T_bits, rot, ctr, r0, r1, nblocks, parts, st);
}

cudaError_t launch_hancock_fast(const Params& P, const CPlanes& in, const Planes& out,
                                const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                Scalars* ctr, int dt_only, cudaStream_t st,
                                const HancockStreams* side) {
    if (P.scheme == GD_SCHEME_HANCOCK_REF)
        return launch_v<true>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st, side);
    return launch_v<false>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st, side);
}

}  // namespace gd
