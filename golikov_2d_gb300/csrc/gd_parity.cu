// gd_parity.cu -- the reference-parity step: one thread per cell, each cell computing its
// own four face fluxes from its own 9-point cross stencil, in the reference's arithmetic
// order, with the solvers of gd_ref_solvers.cuh.  This translation unit is compiled with
// --fmad=false, so with IEEE division and square root the results are bit-identical to the
// reference's step (Kernel_TVD kernel.cu:2198-2661, add2 :1877-2196, Ker_Dekard
// :1736-1875).  The expressions below follow the reference's evaluation order term by term
// because bit-identity requires it; the structure (local-frame solvers, ghost layers, SoA
// planes, block dt reduction) is this library's own.
//
// Used for GD_MODE_PARITY; the fast path (gd_fast_*.cu) is checked against it and against
// the oracle to 1e-12 per step.
#include "gd_internal.cuh"
#include "gd_kernels.h"
#include "gd_ref_solvers.cuh"

namespace gd {
namespace {

constexpr int PTX = 32, PTY = 4, PNT = PTX * PTY;

// kernel.cu:69-84: slope through three points, value at y
__device__ __forceinline__ double lin(double x1, double t1, double x2, double t2, double x3,
                                      double t3, double y) {
    const double d = minmod((t1 - t2) / (x1 - x2), (t2 - t3) / (x2 - x3));
    return d * (y - x2) + t2;
}
__device__ __forceinline__ void lin2(double x1, double t1, double x2, double t2, double x3,
                                     double t3, double y1, double y2, double& A, double& B) {
    const double d = minmod((t1 - t2) / (x1 - x2), (t2 - t3) / (x2 - x3));
    A = d * (y1 - x2) + t2;
    B = d * (y2 - x2) + t2;
}

// outward normals of the reference's faces 12 (E), 13 (S), 14 (W), 15 (N)
__constant__ double kFaceN1[4] = {1.0, 0.0, -1.0, 0.0};
__constant__ double kFaceN2[4] = {0.0, -1.0, 0.0, 1.0};

template <int NF, int ORDER>
__global__ void __launch_bounds__(PNT) parity_kernel(Params P, CPlanes in, Planes out,
                                                     const double* __restrict__ T_do_ptr,
                                                     unsigned long long* T_bits, Scalars* rot,
                                                     Scalars* ctr, int dt_only) {
    const int n = blockIdx.x * PTX + (threadIdx.x % PTX);
    const int mm = (blockIdx.y + P.tile_row0) * PTY + (threadIdx.x / PTX);
    const bool inside = n < P.N && mm < P.M;
    double tmin = kCellTmin0;
    bool active = false;
    unsigned int nfl_r = 0, nfl_p = 0, nbad = 0;
    if (inside) {
        const long long k = (long long)mm * P.N + n;
        const double y = P.y0 + mm * P.dy;
        const double x = P.x0 + n * P.dx;
        bool frozen = false;
        if (P.frozen_radius > 0.0) frozen = sqrt(x * x + y * y) < P.frozen_radius;
        if (frozen) {
            if (!dt_only)
                for (int f = 0; f < NF; ++f) store_f(out, f, k, load_f(in, f, k));
        } else {
            active = true;
            const double dx = P.dx, dy = P.dy;
            // stencil: c1, E(2), S(3), W(4), N(5), and the +-2 cells 21, 31, 41, 51
            double c1[NF], c2[NF], c3[NF], c4[NF], c5[NF];
            fetch_cell<NF>(P, in, n, mm, c1);
            fetch_cell<NF>(P, in, n + 1, mm, c2);
            fetch_cell<NF>(P, in, n, mm - 1, c3);
            fetch_cell<NF>(P, in, n - 1, mm, c4);
            fetch_cell<NF>(P, in, n, mm + 1, c5);
            // face states: own[face][f], nbr[face][f] for faces 12, 13, 14, 15
            double own[4][NF], nbr[4][NF];
            if (ORDER == 1) {
                for (int f = 0; f < NF; ++f) {
                    own[0][f] = own[1][f] = own[2][f] = own[3][f] = c1[f];
                    nbr[0][f] = c2[f]; nbr[1][f] = c3[f]; nbr[2][f] = c4[f]; nbr[3][f] = c5[f];
                }
            } else {
                double c21[NF], c31[NF], c41[NF], c51[NF];
                fetch_cell<NF>(P, in, n + 2, mm, c21);
                fetch_cell<NF>(P, in, n, mm - 2, c31);
                fetch_cell<NF>(P, in, n - 2, mm, c41);
                fetch_cell<NF>(P, in, n, mm + 2, c51);
                for (int f = 0; f < NF; ++f) {
                    const bool pos = f < 2;  // rho, p fall back when <= 0 (kernel.cu:2407-2508)
                    double A, B, w;
                    lin2(x - dx, c4[f], x, c1[f], x + dx, c2[f], x - dx / 2.0, x + dx / 2.0, A, B);
                    own[0][f] = (pos && B <= 0) ? c1[f] : B;
                    own[2][f] = (pos && A <= 0) ? c1[f] : A;
                    lin2(y - dy, c3[f], y, c1[f], y + dy, c5[f], y - dy / 2.0, y + dy / 2.0, A, B);
                    own[3][f] = (pos && B <= 0) ? c1[f] : B;
                    own[1][f] = (pos && A <= 0) ? c1[f] : A;
                    w = lin(x, c1[f], x + dx, c2[f], x + 2.0 * dx, c21[f], x + dx / 2.0);
                    nbr[0][f] = (pos && w <= 0) ? c2[f] : w;
                    w = lin(x, c1[f], x - dx, c4[f], x - 2.0 * dx, c41[f], x - dx / 2.0);
                    nbr[2][f] = (pos && w <= 0) ? c4[f] : w;
                    w = lin(y, c1[f], y - dy, c3[f], y - 2.0 * dy, c31[f], y - dy / 2.0);
                    nbr[1][f] = (pos && w <= 0) ? c3[f] : w;
                    w = lin(y, c1[f], y + dy, c5[f], y + 2.0 * dy, c51[f], y + dy / 2.0);
                    nbr[3][f] = (pos && w <= 0) ? c5[f] : w;
                }
            }
            const double T_do = *T_do_ptr;
            const double dV = dx * dy;
            double res[NF];
            if constexpr (NF == 4) {
                // Euler: fluxes as Kernel_TVD_old :3560-3586, update as Ker_Dekard :1849-1874
                double Ps[4][2], Pu[4][2];
                for (int fc = 0; fc < 4; ++fc) {
                    const double rad = (fc == 0 || fc == 2) ? dy : dx;
                    double o[4];
                    const double tf =
                        P.method == GD_METHOD_HLL
                            ? hll_ref(own[fc], nbr[fc], kFaceN1[fc], kFaceN2[fc], rad, P, o)
                            : hllc_ref(own[fc], nbr[fc], kFaceN1[fc], kFaceN2[fc], rad, P, o);
                    tmin = ref_min(tmin, tf);
                    Ps[fc][0] = o[0]; Ps[fc][1] = o[1]; Pu[fc][0] = o[2]; Pu[fc][1] = o[3];
                }
                const double PSx = Ps[0][0] * dy + Ps[1][0] * dx + Ps[2][0] * dy + Ps[3][0] * dx;
                const double PSy = Ps[0][1] * dy + Ps[1][1] * dx + Ps[2][1] * dy + Ps[3][1] * dx;
                const double PUx = Pu[0][0] * dy + Pu[1][0] * dx + Pu[2][0] * dy + Pu[3][0] * dx;
                const double PUy = Pu[0][1] * dy + Pu[1][1] * dx + Pu[2][1] * dy + Pu[3][1] * dx;
                const double g = P.gamma;
                const double r = c1[0], p = c1[1], u = c1[2], v = c1[3];
                double r2, u2, v2, p2;
                if (P.geometry == GD_AXISYM) {
                    r2 = r - (T_do / dV) * PSx - T_do * r * v / y;
                    if (r2 <= 0) { r2 = 0.0001; ++nfl_r; }
                    u2 = (r * u - (T_do / dV) * PUx - T_do * r * v * u / y) / r2;
                    v2 = (r * v - (T_do / dV) * PUy - T_do * r * v * v / y) / r2;
                    p2 = (((p / (g - 1) + r * (u * u + v * v) * 0.5) - (T_do / dV) * PSy -
                           T_do * v * (g * p / (g - 1) + r * (u * u + v * v) * 0.5) / y) -
                          0.5 * r2 * (u2 * u2 + v2 * v2)) * (g - 1);
                } else {
                    r2 = r - (T_do / dV) * PSx;
                    if (r2 <= 0) { r2 = 0.0001; ++nfl_r; }
                    u2 = (r * u - (T_do / dV) * PUx) / r2;
                    v2 = (r * v - (T_do / dV) * PUy) / r2;
                    p2 = (((p / (g - 1) + r * (u * u + v * v) * 0.5) - (T_do / dV) * PSy) -
                          0.5 * r2 * (u2 * u2 + v2 * v2)) * (g - 1);
                }
                if (p2 <= 0) { p2 = 0.000001; ++nfl_p; }
                res[0] = r2; res[1] = p2; res[2] = u2; res[3] = v2;
            } else {
                // MHD: Kernel_TVD :2550-2660
                double PSx = 0.0, PSy = 0.0, PUx = 0.0, PUy = 0.0, PBx = 0.0, PBy = 0.0, PBz = 0.0;
                double Pdiv = 0.0;
                for (int fc = 0; fc < 4; ++fc) {
                    const bool xf = (fc == 0 || fc == 2);
                    const double rad = xf ? dx : dy;
                    const double len = xf ? dy : dx;
                    const double Lq[8] = {own[fc][0], own[fc][1], own[fc][2], own[fc][3], 0.0,
                                          own[fc][4], own[fc][5], own[fc][6]};
                    const double Rq[8] = {nbr[fc][0], nbr[fc][1], nbr[fc][2], nbr[fc][3], 0.0,
                                          nbr[fc][4], nbr[fc][5], nbr[fc][6]};
                    double Pf[8];
                    const double tf = hlld_ref(Lq, Rq, kFaceN1[fc], kFaceN2[fc], rad, P.method, P, Pf);
                    tmin = ref_min(tmin, tf);
                    PSx = PSx + Pf[0] * len;
                    PSy = PSy + Pf[7] * len;
                    PUx = PUx + Pf[1] * len;
                    PUy = PUy + Pf[2] * len;
                    PBx = PBx + Pf[4] * len;
                    PBy = PBy + Pf[5] * len;
                    PBz = PBz + Pf[6] * len;
                    if (fc == 0) Pdiv = Pdiv + dy * (c1[4] + c2[4]) / 2.0;
                    else if (fc == 1) Pdiv = Pdiv - dx * (c1[5] + c3[5]) / 2.0;
                    else if (fc == 2) Pdiv = Pdiv - dy * (c1[4] + c4[4]) / 2.0;
                    else Pdiv = Pdiv + dx * (c1[5] + c5[5]) / 2.0;
                }
                const bool axi = P.geometry == GD_AXISYM;
                const double g = P.gamma;
                const double r = c1[0], p = c1[1], u = c1[2], v = c1[3];
                const double bx = c1[4], by = c1[5], bz = c1[6];
                if (axi) Pdiv = Pdiv + dV * by / y;
                const double kvu = u * u + v * v + 0.0 * 0.0;
                const double kvb = bx * bx + by * by + bz * bz;
                const double U8 = p / (g - 1.0) + 0.5 * r * kvu + kvb / 25.13274122871834590768;
                const double skk = u * bx + v * by + 0.0 * bz;
                double r2 = r - T_do * PSx / dV;
                if (axi) r2 = r2 - T_do * r * v / y;
                if (r2 <= 0) { r2 = r; ++nfl_r; }
                double u2 = r * u - T_do * (PUx + (bx / kCpi4) * Pdiv) / dV;
                double v2 = r * v - T_do * (PUy + (by / kCpi4) * Pdiv) / dV;
                double bx2 = bx - T_do * (PBx + u * Pdiv) / dV;
                if (axi) {
                    u2 = u2 - T_do * (r * u * v - bx * by / kCpi4) / y;
                    v2 = v2 - T_do * (r * v * v + (bz * bz - by * by) / kCpi4) / y;
                    bx2 = bx2 - T_do * (v * bx - by * u) / y;
                }
                u2 = u2 / r2;
                v2 = v2 / r2;
                const double by2 = by - T_do * (PBy + v * Pdiv) / dV;
                const double bz2 = bz - T_do * (PBz) / dV;
                double e = U8 - T_do * (PSy + (skk / kCpi4) * Pdiv) / dV;
                if (axi) e = e - T_do * (((U8 + p + kvb / kCpi8) * v - by * skk / kCpi4) / y);
                double p2 = (e - 0.5 * r2 * (u2 * u2 + v2 * v2 + 0.0 * 0.0) -
                             (bx2 * bx2 + by2 * by2 + bz2 * bz2) / kCpi8) * (g - 1.0);
                if (p2 <= 0) { p2 = 0.000001; ++nfl_p; }
                res[0] = r2; res[1] = p2; res[2] = u2; res[3] = v2;
                res[4] = bx2; res[5] = by2; res[6] = bz2;
            }
            if (!dt_only) {
                for (int f = 0; f < NF; ++f) {
                    if (!isfinite(res[f])) { ++nbad; break; }
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
    block_tmin_and_rotate<PNT>(tmin, active, T_bits, rot, P.tile_nblocks);
}

template <int NF, int ORDER>
cudaError_t launch_t(const Params& P, const CPlanes& in, const Planes& out, const double* T_do,
                     unsigned long long* T_bits, Scalars* rot, Scalars* ctr, int dt_only,
                     cudaStream_t st) {
    dim3 grid((P.N + PTX - 1) / PTX, P.tile_rows ? P.tile_rows : (P.M + PTY - 1) / PTY);
    parity_kernel<NF, ORDER><<<grid, PNT, 0, st>>>(P, in, out, T_do, T_bits, rot, ctr, dt_only);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_parity(const Params& P, const CPlanes& in, const Planes& out,
                          const double* T_do, unsigned long long* T_bits, Scalars* rot,
                          Scalars* ctr, int dt_only, cudaStream_t st) {
    if (P.physics == GD_EULER) {
        return P.order == 1 ? launch_t<4, 1>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st)
                            : launch_t<4, 2>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
    }
    return P.order == 1 ? launch_t<7, 1>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st)
                        : launch_t<7, 2>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
}

}  // namespace gd
