// gd_hancock_cell.cuh -- one cell of the MUSCL-Hancock step of Kernel_GKR
// (kernel.cu:2663-3284) as the reference computes it: its 13-point stencil, the half-step
// predictions of itself and of its four neighbours (predictor, kernel.cu:1611-1720, with the
// physical flux of POTOK_Korolkov, Gas_Dinamic.cu:70-180), its four HLLD faces
// (kernel.cu:3123-3245) and the corrector (kernel.cu:3256-3281), term by term in the
// reference's order.  Included by gd_hancock.cu (built with --fmad=false: bit-identical to
// the reference) and by gd_fast_hancock.cu (built with contraction, for the cells near the
// edges).
//
// Near the edges the reference does not use a ghost layer: where a stencil point lies
// outside the grid it substitutes a transformed copy of a point inside, chosen from the
// position of the cell being updated (kernel.cu:2701-2960).  A neighbour's predicted state
// near an edge therefore depends on which cell asks for it, and two cells sharing a face
// may see different fluxes there.  stencil<ID>() reproduces those substitutions.
//
// VYP (GD_SCHEME_HANCOCK_REF) keeps the reference's v_y slopes, which it takes from the
// pressures (kernel.cu:2966, 2974, ...); without it (GD_SCHEME_HANCOCK) they come from v_y.
#pragma once

#include "gd_internal.cuh"
#include "gd_ref_solvers.cuh"

namespace gd {
namespace {

// One stencil point, components in the planes' order: rho, p, vx, vy, Bx, By, Bz.
struct HC {
    double q[7];
};

__device__ __forceinline__ HC hload(const CPlanes& in, int N, int n, int m) {
    HC c;
    const long long k = (long long)m * N + n;
#pragma unroll
    for (int f = 0; f < 7; ++f) c.q[f] = load_f(in, f, k);
    return c;
}

// the reference's substitutes: mirror in x (vx, Bx, By odd), mirror in y (vy, Bz odd),
// outflow (vx < 0 -> 0.01), ambient (rho 1, p 1/gamma, v 0) keeping a cell's B
__device__ __forceinline__ HC mir_x(HC c) {
    c.q[2] = -c.q[2];
    c.q[4] = -c.q[4];
    c.q[5] = -c.q[5];
    return c;
}
__device__ __forceinline__ HC mir_y(HC c) {
    c.q[3] = -c.q[3];
    c.q[6] = -c.q[6];
    return c;
}
__device__ __forceinline__ HC clamp_vx(HC c) {
    if (c.q[2] < 0) c.q[2] = 0.01;
    return c;
}
__device__ __forceinline__ HC ambient_b(const Params& P, const HC& b) {
    HC c;
    c.q[0] = 1.0;
    c.q[1] = P.ambient_p;
    c.q[2] = 0.0;
    c.q[3] = 0.0;
    c.q[4] = b.q[4];
    c.q[5] = b.q[5];
    c.q[6] = b.q[6];
    return c;
}

// Stencil point ID of cell (n, m) in the reference's numbering: 1 the cell, 2 / 4 its
// +x / -x neighbours, 5 / 3 its +y / -y neighbours, 6, 8, 9, 7 the points two away
// (+x, -x, +y, -y), 10 (+x,+y), 11 (+x,-y), 12 (-x,-y), 13 (-x,+y).
template <int ID>
__device__ __forceinline__ HC stencil(const Params& P, const CPlanes& in, int n, int m) {
    const int N = P.N, M = P.M;
    if constexpr (ID == 1) {
        return hload(in, N, n, m);
    } else if constexpr (ID == 2) {
        return n == N - 1 ? clamp_vx(stencil<1>(P, in, n, m)) : hload(in, N, n + 1, m);
    } else if constexpr (ID == 3) {
        return m == 0 ? mir_y(stencil<1>(P, in, n, m)) : hload(in, N, n, m - 1);
    } else if constexpr (ID == 4) {
        return n == 0 ? mir_x(stencil<1>(P, in, n, m)) : hload(in, N, n - 1, m);
    } else if constexpr (ID == 5) {
        return m == M - 1 ? ambient_b(P, stencil<1>(P, in, n, m)) : hload(in, N, n, m + 1);
    } else if constexpr (ID == 6) {
        return n >= N - 2 ? clamp_vx(stencil<2>(P, in, n, m)) : hload(in, N, n + 2, m);
    } else if constexpr (ID == 7) {
        if (m == 1) return mir_y(stencil<5>(P, in, n, m));
        if (m == 0) return mir_y(stencil<3>(P, in, n, m));
        return hload(in, N, n, m - 2);
    } else if constexpr (ID == 8) {
        return n <= 1 ? mir_x(stencil<2>(P, in, n, m)) : hload(in, N, n - 2, m);
    } else if constexpr (ID == 9) {
        return m >= M - 2 ? stencil<5>(P, in, n, m) : hload(in, N, n, m + 2);
    } else if constexpr (ID == 10) {
        if (n == N - 1) return stencil<5>(P, in, n, m);
        if (m == M - 1) return ambient_b(P, stencil<2>(P, in, n, m));
        return hload(in, N, n + 1, m + 1);
    } else if constexpr (ID == 11) {
        if (m == 0) return mir_y(stencil<2>(P, in, n, m));
        if (n == N - 1) return clamp_vx(stencil<3>(P, in, n, m));
        return hload(in, N, n + 1, m - 1);
    } else if constexpr (ID == 12) {
        if (m == 0) return mir_y(stencil<4>(P, in, n, m));
        if (n == 0) return mir_x(stencil<3>(P, in, n, m));
        return hload(in, N, n - 1, m - 1);
    } else {
        static_assert(ID == 13, "stencil points are 1..13");
        if (n == 0) return mir_x(stencil<5>(P, in, n, m));
        if (m == M - 1) return ambient_b(P, stencil<4>(P, in, n, m));
        return hload(in, N, n - 1, m + 1);
    }
}

// h * minmod((a - b)/h, (b - c)/h) for every component (kernel.cu:2963-3081); with VYP the
// v_y component is computed from the pressures, as the reference writes it.
template <bool VYP>
__device__ __forceinline__ void slopes(const HC& a, const HC& b, const HC& c, double h,
                                       double* D) {
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        const int j = (i == 3 && VYP) ? 1 : i;
        D[i] = h * minmod((a.q[j] - b.q[j]) / h, (b.q[j] - c.q[j]) / h);
    }
}

// U8, kvv, skk (Header.h:16, kernel.cu:33-48)
__device__ __forceinline__ double u8_ref(double g, double ro, double p, double u, double v,
                                         double w, double bx, double by, double bz) {
    return p / (g - 1.0) + 0.5 * ro * ((u * u + v * v) + w * w) +
           ((bx * bx + by * by) + bz * bz) / 25.13274122871834590768;
}
__device__ __forceinline__ double kvv_ref(double x, double y, double z) {
    return (x * x + y * y) + z * z;
}
__device__ __forceinline__ double skk_ref(double u, double v, double w, double bx, double by,
                                          double bz) {
    return u * bx + v * by + w * bz;
}

// POTOK_Korolkov (Gas_Dinamic.cu:70-180) for v_z = 0 through a face of normal (n1, n2, 0):
// the physical flux of one state in the face's frame (n, t, m), rotated back.
// P8 = {F_rho, F_mx, F_my, F_mz, F_Bx, F_By, F_Bz, F_E}, the field fluxes Gaussian.
__device__ __forceinline__ void potok_ref(double g, double ro_L, double p_L, double v1_L,
                                          double v2_L, double Bx_L, double By_L, double Bz_L,
                                          double n1, double n2, double* P8) {
    const double v3_L = 0.0, n3 = 0.0;
    const double bx_L = Bx_L / kSpi4, by_L = By_L / kSpi4, bz_L = Bz_L / kSpi4;
    double t1 = 0.0, t2 = 0.0, t3 = 0.0, m1 = 0.0, m2 = 0.0, m3 = 0.0;
    if (n1 > 0.1) {
        t2 = 1.0; m3 = 1.0;
    } else if (n2 > 0.1) {
        t3 = 1.0; m1 = 1.0;
    } else if (n1 < -0.1) {
        t3 = -1.0; m2 = -1.0;
    } else if (n2 < -0.1) {
        t1 = -1.0; m3 = -1.0;
    }
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
    const double F0 = ro_L * u1;
    const double F1 = ro_L * u1 * u1 + pTL - bn1 * bn1;
    const double F2 = ro_L * u1 * v1 - bn1 * bt1;
    const double F3 = ro_L * u1 * w1 - bn1 * bm1;
    const double F4 = (e1 + pTL) * u1 - bn1 * (u1 * bn1 + v1 * bt1 + w1 * bm1);
    const double F5 = 0.0;
    const double F6 = u1 * bt1 - v1 * bn1;
    const double F7 = u1 * bm1 - w1 * bn1;
    P8[0] = F0;
    P8[1] = n1 * F1 + t1 * F2 + m1 * F3;
    P8[2] = n2 * F1 + t2 * F2 + m2 * F3;
    P8[3] = n3 * F1 + t3 * F2 + m3 * F3;
    P8[4] = kSpi4 * (n1 * F5 + t1 * F6 + m1 * F7);
    P8[5] = kSpi4 * (n2 * F5 + t2 * F6 + m2 * F7);
    P8[6] = kSpi4 * (n3 * F5 + t3 * F6 + m3 * F7);
    P8[7] = F4;
}

// predictor (kernel.cu:1611-1720): the state of a cell after half a step (st = T_do/2) of
// its own reconstructed face fluxes and axisymmetric sources at radius y.  Faces in the
// reference's order -x, +x, +y, -y; the face states Q -+ D/2 fall back to Q for rho, p <= 0.
__device__ __forceinline__ void predictor_ref(const Params& P, const double* Q, const double* DX,
                                              const double* DY, double st, double y,
                                              double* QQ) {
    const double g = P.gamma, dx = P.dx, dy = P.dy;
    double PSx = 0.0, PSy = 0.0, PUx = 0.0, PUy = 0.0, PBx = 0.0, PBy = 0.0, PBz = 0.0;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const double* D = f < 2 ? DX : DY;
        const double h = f < 2 ? dy : dx;
        const bool minus = (f == 0 || f == 3);
        double a[7];
#pragma unroll
        for (int i = 0; i < 7; ++i) a[i] = minus ? Q[i] - D[i] / 2.0 : Q[i] + D[i] / 2.0;
        if (a[0] <= 0.0) a[0] = Q[0];
        if (a[1] <= 0.0) a[1] = Q[1];
        const double s = minus ? -1.0 : 1.0;
        const double n1 = f < 2 ? s : 0.0, n2 = f < 2 ? 0.0 : s;
        double F[8];
        potok_ref(g, a[0], a[1], a[2], a[3], a[4], a[5], a[6], n1, n2, F);
        PSx = PSx + F[0] * h;
        PSy = PSy + F[7] * h;
        PUx = PUx + F[1] * h;
        PUy = PUy + F[2] * h;
        PBx = PBx + F[4] * h;
        PBy = PBy + F[5] * h;
        PBz = PBz + F[6] * h;
    }
    const double dV = dx * dy;
    QQ[0] = Q[0] - st * PSx / dV - st * Q[0] * Q[3] / y;
    if (QQ[0] <= 0) QQ[0] = Q[0];
    QQ[2] = (Q[0] * Q[2] - st * (PUx) / dV - st * (Q[0] * Q[2] * Q[3] - Q[4] * Q[5] / kCpi4) / y) /
            QQ[0];
    QQ[3] = (Q[0] * Q[3] - st * (PUy) / dV -
             st * (Q[0] * Q[3] * Q[3] + (Q[6] * Q[6] - Q[5] * Q[5]) / kCpi4) / y) / QQ[0];
    QQ[4] = (Q[4] - st * (PBx) / dV - st * (Q[3] * Q[4] - Q[5] * Q[2]) / y);
    QQ[5] = (Q[5] - st * (PBy) / dV);
    QQ[6] = (Q[6] - st * (PBz) / dV);
    const double U = u8_ref(g, Q[0], Q[1], Q[2], Q[3], 0.0, Q[4], Q[5], Q[6]);
    QQ[1] = (U - st * (PSy) / dV -
             st * (((U + Q[1] + kvv_ref(Q[4], Q[5], Q[6]) / kCpi8) * Q[3] -
                    Q[5] * skk_ref(Q[2], Q[3], 0.0, Q[4], Q[5], Q[6]) / kCpi4) / y) -
             0.5 * QQ[0] * kvv_ref(QQ[2], QQ[3], 0.0) - kvv_ref(QQ[4], QQ[5], QQ[6]) / kCpi8) *
            (g - 1.0);
    if (QQ[1] <= 0) QQ[1] = 0.000001;
}

// The face-centred state of a cell from its half-step mean A = (Q + QQ)/2 and slope D:
// A + D/2 (sgn > 0) or A - D/2, with rho, p falling back to A's when <= 0
// (kernel.cu:3100-3122), in the solver's order {rho, p, vx, vy, vz = 0, Bx, By, Bz}.
__device__ __forceinline__ void face_state(const double* A, const double* D, bool plus,
                                           double* S) {
    double ro = plus ? A[0] + D[0] / 2.0 : A[0] - D[0] / 2.0;
    double p = plus ? A[1] + D[1] / 2.0 : A[1] - D[1] / 2.0;
    if (ro <= 0.0) ro = A[0];
    if (p <= 0.0) p = A[1];
    S[0] = ro;
    S[1] = p;
    S[2] = plus ? A[2] + D[2] / 2.0 : A[2] - D[2] / 2.0;
    S[3] = plus ? A[3] + D[3] / 2.0 : A[3] - D[3] / 2.0;
    S[4] = 0.0;
    S[5] = plus ? A[4] + D[4] / 2.0 : A[4] - D[4] / 2.0;
    S[6] = plus ? A[5] + D[5] / 2.0 : A[5] - D[5] / 2.0;
    S[7] = plus ? A[6] + D[6] / 2.0 : A[6] - D[6] / 2.0;
}

// Face F of cell (n, m): 0 = +x (E), 1 = -y (S), 2 = -x (W), 3 = +y (N), in the reference's
// order.  Predicts the neighbour across the face from its own slopes as seen from (n, m),
// solves HLLD between the two face states, and adds the flux times the face length to
// acc = {PSx, PSy, PUx, PUy, PBx, PBy, PBz}.  Returns the face's krit*rad/UU.
template <int F, bool VYP>
__device__ __forceinline__ double hancock_face(const Params& P, const CPlanes& in, int n, int m,
                                               double y, double st, const double* A1,
                                               const double* DX1, const double* DY1,
                                               double* acc) {
    const double dx = P.dx, dy = P.dy;
    HC q;
    double DXn[7], DYn[7];
    double yn = y;
    if constexpr (F == 0) {
        q = stencil<2>(P, in, n, m);
        slopes<VYP>(stencil<6>(P, in, n, m), q, stencil<1>(P, in, n, m), dx, DXn);
        slopes<VYP>(stencil<10>(P, in, n, m), q, stencil<11>(P, in, n, m), dy, DYn);
    } else if constexpr (F == 1) {
        q = stencil<3>(P, in, n, m);
        slopes<VYP>(stencil<11>(P, in, n, m), q, stencil<12>(P, in, n, m), dx, DXn);
        slopes<VYP>(stencil<1>(P, in, n, m), q, stencil<7>(P, in, n, m), dy, DYn);
        yn = y - dy;
    } else if constexpr (F == 2) {
        q = stencil<4>(P, in, n, m);
        slopes<VYP>(stencil<1>(P, in, n, m), q, stencil<8>(P, in, n, m), dx, DXn);
        slopes<VYP>(stencil<13>(P, in, n, m), q, stencil<12>(P, in, n, m), dy, DYn);
    } else {
        q = stencil<5>(P, in, n, m);
        slopes<VYP>(stencil<10>(P, in, n, m), q, stencil<13>(P, in, n, m), dx, DXn);
        slopes<VYP>(stencil<9>(P, in, n, m), q, stencil<1>(P, in, n, m), dy, DYn);
        yn = y + dy;
    }
    double QQn[7], An[7];
    predictor_ref(P, q.q, DXn, DYn, st, yn, QQn);
#pragma unroll
    for (int i = 0; i < 7; ++i) An[i] = (q.q[i] + QQn[i]) / 2.0;
    // own side: +D for the + faces (E, N); neighbour side: the opposite sign
    constexpr bool own_plus = (F == 0 || F == 3);
    const double* Down = (F == 0 || F == 2) ? DX1 : DY1;
    const double* Dnbr = (F == 0 || F == 2) ? DXn : DYn;
    double L[8], R[8], Pf[8];
    face_state(A1, Down, own_plus, L);
    face_state(An, Dnbr, !own_plus, R);
    constexpr double n1 = F == 0 ? 1.0 : (F == 2 ? -1.0 : 0.0);
    constexpr double n2 = F == 3 ? 1.0 : (F == 1 ? -1.0 : 0.0);
    const bool xf = (F == 0 || F == 2);
    const double t = hlld_ref(L, R, n1, n2, xf ? dx : dy, GD_METHOD_HLLD, P, Pf);
    const double h = xf ? dy : dx;
    acc[0] = acc[0] + Pf[0] * h;
    acc[1] = acc[1] + Pf[7] * h;
    acc[2] = acc[2] + Pf[1] * h;
    acc[3] = acc[3] + Pf[2] * h;
    acc[4] = acc[4] + Pf[4] * h;
    acc[5] = acc[5] + Pf[5] * h;
    acc[6] = acc[6] + Pf[6] * h;
    return t;
}

// the reference's cell coordinates and frozen test (kernel.cu:2669-2692); the sum of squares
// is written with explicit roundings so that no build contracts it and every build freezes
// the same cells
__device__ __forceinline__ double hancock_y(const Params& P, int m) {
    return P.y0 + m * (P.y_max) / (P.M);
}
__device__ __forceinline__ double hancock_x(const Params& P, int n) {
    return P.x0 + n * (P.x_max - P.x0) / (P.N - 1);
}
__device__ __forceinline__ bool hancock_frozen_xy(const Params& P, double x, double y) {
    return P.frozen_radius > 0.0 &&
           sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))) < P.frozen_radius;
}
__device__ __forceinline__ bool hancock_frozen(const Params& P, int n, double y) {
    return hancock_frozen_xy(P, hancock_x(P, n), y);
}
// The same decision without the square root away from the sphere: sqrt is correctly
// rounded and monotone, so for x^2 + y^2 outside R^2 (1 -+ 1e-12) its comparison with R is
// decided by the squares; only the thin shell in between takes the square root.
__device__ __forceinline__ bool hancock_frozen_fast(const Params& P, double x, double y) {
    if (!(P.frozen_radius > 0.0)) return false;
    const double s = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    const double R2 = P.frozen_radius * P.frozen_radius;
    if (dlt(s, R2 * (1.0 - 1e-12))) return true;
    if (dlt(R2 * (1.0 + 1e-12), s)) return false;
    return sqrt(s) < P.frozen_radius;
}

// Kernel_GKR's update of the non-frozen cell (n, m) at radius y with step T_do: res gets
// the new {rho, p, vx, vy, Bx, By, Bz}; returns the cell's dt (min over its four faces of
// krit*rad/UU); fl_r / fl_p count the density / pressure floors.
template <bool VYP>
__device__ __forceinline__ double hancock_cell(const Params& P, const CPlanes& in, int n, int m,
                                               double y, double T_do, double* res,
                                               unsigned int& fl_r, unsigned int& fl_p) {
    const double st = T_do / 2.0;
    double DX1[7], DY1[7], A1[7];
    {
        const HC c1 = stencil<1>(P, in, n, m);
        slopes<VYP>(stencil<2>(P, in, n, m), c1, stencil<4>(P, in, n, m), P.dx, DX1);
        slopes<VYP>(stencil<5>(P, in, n, m), c1, stencil<3>(P, in, n, m), P.dy, DY1);
        double QQ1[7];
        predictor_ref(P, c1.q, DX1, DY1, st, y, QQ1);
#pragma unroll
        for (int i = 0; i < 7; ++i) A1[i] = (c1.q[i] + QQ1[i]) / 2.0;
    }
    double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double tmin = kCellTmin0;
    tmin = my_min(tmin, hancock_face<0, VYP>(P, in, n, m, y, st, A1, DX1, DY1, acc));
    tmin = my_min(tmin, hancock_face<1, VYP>(P, in, n, m, y, st, A1, DX1, DY1, acc));
    tmin = my_min(tmin, hancock_face<2, VYP>(P, in, n, m, y, st, A1, DX1, DY1, acc));
    tmin = my_min(tmin, hancock_face<3, VYP>(P, in, n, m, y, st, A1, DX1, DY1, acc));
    const double PSx = acc[0], PSy = acc[1], PUx = acc[2], PUy = acc[3];
    const double PBx = acc[4], PBy = acc[5], PBz = acc[6];
    // corrector (kernel.cu:3256-3281), Pdiv = 0
    const double g = P.gamma;
    const double dV = P.dx * P.dy;
    const double Pdiv = 0.0;
    const double hT = T_do / 2.0;
    const double* A = A1;
    double r2 = A[0] - hT * PSx / dV - hT * A[0] * A[3] / y;
    if (r2 <= 0) {
        r2 = A[0];
        ++fl_r;
    }
    const double ux2 = (A[0] * A[2] - hT * (PUx + (A[4] / kCpi4) * Pdiv) / dV -
                        hT * (A[0] * A[2] * A[3] - A[4] * A[5] / kCpi4) / y) / r2;
    const double uy2 = (A[0] * A[3] - hT * (PUy + (A[5] / kCpi4) * Pdiv) / dV -
                        hT * (A[0] * A[3] * A[3] + (A[6] * A[6] - A[5] * A[5]) / kCpi4) / y) /
                       r2;
    const double bx2 =
        (A[4] - hT * (PBx + A[2] * Pdiv) / dV - hT * (A[3] * A[4] - A[5] * A[2]) / y);
    const double by2 = (A[5] - hT * (PBy + A[3] * Pdiv) / dV);
    const double bz2 = (A[6] - hT * (PBz) / dV);
    const double U = u8_ref(g, A[0], A[1], A[2], A[3], 0.0, A[4], A[5], A[6]);
    const double sk = skk_ref(A[2], A[3], 0.0, A[4], A[5], A[6]);
    double p2 = (U - hT * (PSy + (sk / kCpi4) * Pdiv) / dV -
                 hT * (((U + A[1] + kvv_ref(A[4], A[5], A[6]) / kCpi8) * A[3] -
                        A[5] * sk / kCpi4) / y) -
                 0.5 * r2 * kvv_ref(ux2, uy2, 0.0) - kvv_ref(bx2, by2, bz2) / kCpi8) *
                (g - 1.0);
    if (p2 <= 0) {
        p2 = 0.000001;
        ++fl_p;
    }
    res[0] = r2; res[1] = p2; res[2] = ux2; res[3] = uy2;
    res[4] = bx2; res[5] = by2; res[6] = bz2;
    return tmin;
}

}  // namespace
}  // namespace gd
