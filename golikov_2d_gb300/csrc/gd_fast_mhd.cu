// gd_fast_mhd.cu -- fused minmod-TVD + HLLD / HLLC-MHD + Powell-source update for 2-D ideal
// MHD, face-once tiles (same phase structure as gd_fast_euler.cu: load, slopes, faces,
// update), and its forward-mode tangent.
//
// The flux and the tile body are templates on the scalar type: `double` gives the step,
// `Dual` (gd_dual.cuh) gives the tangent (JVP) of exactly the same arithmetic, with the dt
// held fixed and derivatives taken along the branches the values take.
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
#include <type_traits>

#include "gd_dual.cuh"
#include "gd_internal.cuh"
#include "gd_kernels.h"
#include "gd_mhd_flux.cuh"

namespace gd {
namespace {

constexpr int TX = 32;
constexpr int NT = 256;
constexpr int NF = 7;  // rho, p, vx, vy, bx, by, bz

// ---- state access: planes of doubles for the step, value + tangent planes for the JVP ----

struct DualCPlanes {
    CPlanes v, d;
};
struct DualPlanes {
    Planes v, d;
};

__device__ __forceinline__ void load_state(const Params& P, const CPlanes& in, int gx, int gy,
                                           double* v) {
    fetch_cell<NF>(P, in, gx, gy, v);
}

// Tangent of a ghost value: the linear part of the boundary condition.  Copies and sign
// flips carry the derivative; constants (ambient) and the active outflow clamp have none.
__device__ __forceinline__ void load_state(const Params& P, const DualCPlanes& in, int gx,
                                           int gy, Dual* v) {
    double a[NF], b[NF];
    fetch_cell<NF>(P, in.v, gx, gy, a);
    fetch_cell<NF>(P, in.d, gx, gy, b);
    int bc = -1;
    if (gx < 0 || gx >= P.N) bc = gx < 0 ? P.bc[0] : P.bc[1];
    else if (gy < 0 || gy >= P.M) bc = gy < 0 ? P.bc[2] : P.bc[3];
    if (bc == GD_BC_AMBIENT || bc == GD_BC_AMBIENT_KEEPB) {
        for (int f = 0; f < (bc == GD_BC_AMBIENT ? NF : 4); ++f) b[f] = 0.0;
    } else if (bc == GD_BC_OUTFLOW) {
        double raw[NF];
        CPlanes plain = in.v;
        int sx = gx < 0 ? 0 : (gx >= P.N ? P.N - 1 : gx);
        int sy = gy < 0 ? 0 : (gy >= P.M ? P.M - 1 : gy);
        raw[2] = plain.f[2][(long long)sy * P.N + sx];
        if (raw[2] < 0) b[2] = 0.0;
    }
#pragma unroll
    for (int f = 0; f < NF; ++f) v[f] = Dual{a[f], b[f]};
}

__device__ __forceinline__ void store_state(const Planes& out, long long k, int f, double x) {
    store_f(out, f, k, x);
}
__device__ __forceinline__ void store_state2(const Planes& out, long long k, int f0, double a,
                                             double b) {
    store_pair(out, f0, k, a, b);
}
__device__ __forceinline__ void store_state(const DualPlanes& out, long long k, int f, Dual x);
__device__ __forceinline__ void store_state2(const DualPlanes& out, long long k, int f0, Dual a,
                                             Dual b) {
    store_state(out, k, f0, a);
    store_state(out, k, f0 + 1, b);
}
__device__ __forceinline__ void store_state(const DualPlanes& out, long long k, int f, Dual x) {
    out.v.f[f][k] = x.v;
    out.d.f[f][k] = x.d;
}
__device__ __forceinline__ void copy_cell(const CPlanes& in, const Planes& out, long long k) {
#pragma unroll
    for (int f = 0; f < NF; ++f) store_f(out, f, k, load_f(in, f, k));
}
__device__ __forceinline__ void copy_cell(const DualCPlanes& in, const DualPlanes& out,
                                          long long k) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        out.v.f[f][k] = in.v.f[f][k];
        out.d.f[f][k] = in.d.f[f][k];
    }
}

template <class T, int ORDER, int TY>
struct SmemM {
    static constexpr int H = ORDER == 2 ? 2 : 1;
    static constexpr int SX = TX + 2 * H;
    static constexpr int SY = TY + 2 * H;
    static constexpr int kPrim = NF * SY * SX;
    static constexpr int kSlx = ORDER == 2 ? NF * TY * (TX + 2) : 0;
    static constexpr int kSly = ORDER == 2 ? NF * (TY + 2) * TX : 0;
    static constexpr int kFx = NF * TY * (TX + 1);
    static constexpr int kFy = NF * (TY + 1) * TX;
    static constexpr size_t bytes = sizeof(T) * (kPrim + kSlx + kSly + kFx + kFy);
};

struct MhdTileResult {
    double umax_x, umax_y;
    bool any_active;
    unsigned int nfl_r, nfl_p, nbad;
};

// One TX x TY tile at (tx0, ty0): load, slopes, faces, update.  IN/OUT are CPlanes/Planes
// for T = double and DualCPlanes/DualPlanes for T = Dual.
// flux component slots in smem: 0 mass, 1 energy, 2 mom x, 3 mom y, 4 bx, 5 by, 6 bz
// `aux` (T = double only; may be null) receives, per cell, the flux differences d[0..6]
// and the Powell term divb that the update used (planes of N*M), for the adjoint.
template <class T, int ORDER, int TY, class IN, class OUT>
__device__ __forceinline__ void mhd_tile(const Params& P, const IN& in, const OUT& out, int tx0,
                                         int ty0, double T_do, int dt_only, T* smem,
                                         MhdTileResult& res, double* aux = nullptr) {
    using S = SmemM<T, ORDER, TY>;
    constexpr int H = S::H, SX = S::SX, SY = S::SY;
    T* prim = smem;
    T* slx = prim + S::kPrim;
    T* sly = slx + S::kSlx;
    T* fx = sly + S::kSly;
    T* fy = fx + S::kFx;

    const int tid = threadIdx.x;
    const int N = P.N, M = P.M;

    // ---- L: tile + cross halo, field to Heaviside-Lorentz units --------------------------
    for (int i = tid; i < SY * SX; i += NT) {
        const int ly = i / SX, lx = i - ly * SX;
        const bool xh = lx < H || lx >= TX + H, yh = ly < H || ly >= TY + H;
        if (xh && yh) continue;
        const int gx = tx0 + lx - H, gy = ty0 + ly - H;
        T v[NF];
        if (gx >= -2 && gx < N + 2 && gy >= -2 && gy < M + 2 &&
            !((gx < 0 || gx >= N) && (gy < 0 || gy >= M))) {
            load_state(P, in, gx, gy, v);
        } else {
#pragma unroll
            for (int f = 0; f < NF; ++f) v[f] = cst<T>(f < 2 ? 1.0 : 0.0);  // never used
        }
        v[4] = v[4] * kInvSpi4;
        v[5] = v[5] * kInvSpi4;
        v[6] = v[6] * kInvSpi4;
#pragma unroll
        for (int f = 0; f < NF; ++f) prim[(f * SY + ly) * SX + lx] = v[f];
    }
    __syncthreads();

    // ---- S: slopes ---------------------------------------------------------------------------
    // a thread takes a run of G cells, so neighbouring slopes share their difference
    if (ORDER == 2) {
        constexpr int GX = (TX + 2) % 3 == 0 ? 3 : 2, GY = (TY + 2) % 3 == 0 ? 3 : 2;
        constexpr int NGX = (TX + 2) / GX, NGY = (TY + 2) / GY;
        static_assert((TX + 2) % GX == 0 && (TY + 2) % GY == 0, "slope runs tile the rows");
        for (int i = tid; i < TY * NGX; i += NT) {
            const int ly = i / NGX, c0 = (i - ly * NGX) * GX;
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
            const int g = i / TX, lx = i - g * TX, r0 = g * GY;
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
        if (P.frozen && !cell_active(P, tx0 + ax, ty0 + ay) &&
            !cell_active(P, tx0 + lx, ty0 + ly))
            continue;
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
        Side<T> A, B;
        side(A, qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2], isx ? qa[4] : qa[5],
             isx ? qa[5] : qa[4], qa[6], P);
        side(B, qb[0], qb[1], isx ? qb[2] : qb[3], isx ? qb[3] : qb[2], isx ? qb[4] : qb[5],
             isx ? qb[5] : qb[4], qb[6], P);
        T UU;
        const FluxM<T> F = hlld_local(A, B, P.method, P, UU);
        if (isx) {
            T* fo = fx + ly * (TX + 1) + lx;
            constexpr int st = TY * (TX + 1);
            fo[0 * st] = F.m;
            fo[1 * st] = F.e;
            fo[2 * st] = F.mn;
            fo[3 * st] = F.mt;
            fo[4 * st] = F.bn;
            fo[5 * st] = F.bt;
            fo[6 * st] = F.bz;
            umax_x = max_nonneg(umax_x, value_of(UU));
        } else {
            T* fo = fy + ly * TX + lx;
            constexpr int st = (TY + 1) * TX;
            fo[0 * st] = F.m;
            fo[1 * st] = F.e;
            fo[2 * st] = F.mt;
            fo[3 * st] = F.mn;
            fo[4 * st] = F.bt;
            fo[5 * st] = F.bn;
            fo[6 * st] = F.bz;
            umax_y = max_nonneg(umax_y, value_of(UU));
        }
    }
    __syncthreads();

    // ---- U: update (kernel.cu:2606-2660 in Heaviside-Lorentz field units) ----------------------
    const double kx = imul<true>(T_do, P.inv_dx), ky = imul<true>(T_do, P.inv_dy);
    const double hkx = half_exact(kx), hky = half_exact(ky);  // 0.5 kx, 0.5 ky
    const bool axi = P.geometry == GD_AXISYM;
    bool any_active = false;
    unsigned int nfl_r = 0, nfl_p = 0, nbad = 0;
    for (int i = tid; i < TX * TY; i += NT) {
        const int ly = i / TX, lx = i - ly * TX;
        const int gx = tx0 + lx, gy = ty0 + ly;
        if (gx >= N || gy >= M) continue;
        const T* c = prim + (ly + H) * SX + (lx + H);
        constexpr int PS = SY * SX;
        const T r = c[0], p = c[PS], u = c[2 * PS], v = c[3 * PS];
        const T bx = c[4 * PS], by = c[5 * PS], bz = c[6 * PS];
        const long long k = (long long)gy * N + gx;
        if (P.frozen && !cell_active(P, gx, gy)) {  // the faces' own test
            if (!dt_only) copy_cell(in, out, k);
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
            d[f] = fma(kx, a[1] - a[0], ky * (b[TX] - b[0]));
        }
        // Powell divergence from cell-centred field: dx dy div b (kernel.cu:2568-2604)
        const T bxE = c[4 * PS + 1], bxW = c[4 * PS - 1];
        const T byN = c[5 * PS + SX], byS = c[5 * PS - SX];
        T divb = fma(hkx, bxE - bxW, mulx<true>(hky, byN - byS));  // T_do * div b
        const double iy = axi ? rcp_fast(P.y0 + gy * P.dy) : 0.0;
        if (axi) divb = fma(T_do * by, iy, divb);                 // kernel.cu:2615
        if constexpr (std::is_same<T, double>::value) {
            if (aux != nullptr) {
                const long long KK = (long long)N * M;
#pragma unroll
                for (int f = 0; f < NF; ++f) aux[f * KK + k] = d[f];
                aux[7 * KK + k] = divb;
            }
        }
        const T ub = fma(u, bx, v * by);
        const T bb = fma(bz, bz, fma(by, by, bx * bx));
        const T E = fma(p, P.inv_gm1, 0.5 * fma(r, fma(u, u, v * v), bb));
        T r2 = r - d[0];
        T mx2 = fma(r, u, -fma(bx, divb, d[2]));
        T my2 = fma(r, v, -fma(by, divb, d[3]));
        T bx2 = bx - fma(u, divb, d[4]);
        const T by2 = by - fma(v, divb, d[5]);
        const T bz2 = bz - d[6];
        T E2 = E - fma(ub, divb, d[1]);
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
        const T inv = rcp_fast(r2);
        const T u2 = mx2 * inv, v2 = my2 * inv;
        T p2 = (E2 - 0.5 * fma(r2, fma(u2, u2, v2 * v2), fma(bz2, bz2, fma(by2, by2, bx2 * bx2)))) * P.gm1;
        if (le_zero(p2)) { p2 = cst<T>(0.000001); ++nfl_p; }
        if (!finite_bits(r2) || !finite_bits(p2) || !finite_bits(u2) || !finite_bits(v2) ||
            !finite_bits(bx2) || !finite_bits(by2) || !finite_bits(bz2))
            ++nbad;
        store_state2(out, k, 0, r2, p2);
        store_state2(out, k, 2, u2, v2);
        store_state(out, k, 4, bx2 * kSpi4);
        store_state(out, k, 5, by2 * kSpi4);
        store_state(out, k, 6, bz2 * kSpi4);
    }
    res.umax_x = umax_x;
    res.umax_y = umax_y;
    res.any_active = any_active;
    res.nfl_r = nfl_r;
    res.nfl_p = nfl_p;
    res.nbad = nbad;
}

template <int ORDER, int TY>
__global__ void __launch_bounds__(NT, 2) mhd_fast_kernel(Params P, CPlanes in, Planes out,
                                                      const double* __restrict__ T_do_ptr,
                                                      unsigned long long* T_bits, Scalars* rot,
                                                      Scalars* ctr, int dt_only, double* aux) {
    extern __shared__ __align__(16) double smem[];
    MhdTileResult r;
    mhd_tile<double, ORDER, TY>(P, in, out, blockIdx.x * TX, (blockIdx.y + P.tile_row0) * TY,
                                *T_do_ptr, dt_only,
                                smem, r, aux);
    if (ctr != nullptr && (r.nfl_r | r.nfl_p | r.nbad)) {
        if (r.nfl_r) atomicAdd(&ctr->rho_floor, (unsigned long long)r.nfl_r);
        if (r.nfl_p) atomicAdd(&ctr->p_floor, (unsigned long long)r.nfl_p);
        if (r.nbad) atomicAdd(&ctr->nonfinite, (unsigned long long)r.nbad);
    }
    block_dt_and_rotate<NT>(P, r.umax_x, r.umax_y, r.any_active, T_bits, rot, P.tile_nblocks);
}

// Tangent of one step: (U, dU) -> (U', dU') with the dt read from *T_do_ptr (held fixed).
template <int ORDER, int TY>
__global__ void __launch_bounds__(NT) mhd_tangent_kernel(Params P, CPlanes in, CPlanes din,
                                                         Planes out, Planes dout,
                                                         const double* __restrict__ T_do_ptr) {
    extern __shared__ __align__(16) double smem[];
    MhdTileResult r;
    const DualCPlanes I{in, din};
    const DualPlanes O{out, dout};
    mhd_tile<Dual, ORDER, TY>(P, I, O, blockIdx.x * TX, blockIdx.y * TY, *T_do_ptr, 0,
                              reinterpret_cast<Dual*>(smem), r);
}

// 32 x 8 tiles: 88 KB of shared memory and at most 128 registers, so two CTAs (16 warps) are
// resident per SM; the halo costs 3 % more faces than 32 x 16 tiles at one CTA per SM.
constexpr int kTY = 8;
constexpr int kTYDual = 8;

template <int ORDER>
cudaError_t launch_t(const Params& P, const CPlanes& in, const Planes& out, const double* T_do,
                     unsigned long long* T_bits, Scalars* rot, Scalars* ctr, int dt_only,
                     cudaStream_t st, double* aux = nullptr) {
    dim3 grid((P.N + TX - 1) / TX, P.tile_rows ? P.tile_rows : (P.M + kTY - 1) / kTY);
    mhd_fast_kernel<ORDER, kTY><<<grid, NT, SmemM<double, ORDER, kTY>::bytes, st>>>(
        P, in, out, T_do, T_bits, rot, ctr, dt_only, aux);
    return cudaGetLastError();
}

template <int ORDER>
cudaError_t launch_tangent_t(const Params& P, const CPlanes& in, const CPlanes& din,
                             const Planes& out, const Planes& dout, const double* T_do,
                             cudaStream_t st) {
    dim3 grid((P.N + TX - 1) / TX, (P.M + kTYDual - 1) / kTYDual);
    mhd_tangent_kernel<ORDER, kTYDual><<<grid, NT, SmemM<Dual, ORDER, kTYDual>::bytes, st>>>(
        P, in, din, out, dout, T_do);
    return cudaGetLastError();
}

}  // namespace

int mhd_tile_height() { return kTY; }

cudaError_t prepare_mhd_fast() {
    cudaError_t e = cudaFuncSetAttribute(mhd_fast_kernel<1, kTY>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)SmemM<double, 1, kTY>::bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mhd_fast_kernel<2, kTY>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SmemM<double, 2, kTY>::bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mhd_tangent_kernel<1, kTYDual>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SmemM<Dual, 1, kTYDual>::bytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mhd_tangent_kernel<2, kTYDual>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)SmemM<Dual, 2, kTYDual>::bytes);
    return e;
}

cudaError_t launch_mhd_fast(const Params& P, const CPlanes& in, const Planes& out,
                            const double* T_do, unsigned long long* T_bits, Scalars* rot,
                            Scalars* ctr, int dt_only, cudaStream_t st) {
    if (P.order == 1) return launch_t<1>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
    return launch_t<2>(P, in, out, T_do, T_bits, rot, ctr, dt_only, st);
}

cudaError_t launch_mhd_fast_aux(const Params& P, const CPlanes& in, const Planes& out,
                                const double* T_do, unsigned long long* T_bits, Scalars* rot,
                                Scalars* ctr, double* aux, cudaStream_t st) {
    if (P.order == 1) return launch_t<1>(P, in, out, T_do, T_bits, rot, ctr, 0, st, aux);
    return launch_t<2>(P, in, out, T_do, T_bits, rot, ctr, 0, st, aux);
}

cudaError_t launch_mhd_tangent(const Params& P, const CPlanes& in, const CPlanes& din,
                               const Planes& out, const Planes& dout, const double* T_do,
                               cudaStream_t st) {
    if (P.order == 1) return launch_tangent_t<1>(P, in, din, out, dout, T_do, st);
    return launch_tangent_t<2>(P, in, din, out, dout, T_do, st);
}


namespace {
// One face per thread through the step's own face solver (side + hlld_local): L, R are n x 8
// in the reference's HLLDQ_Korolkov layout (rho, p, vx, vy, vz, Bx, By, Bz; Gaussian B, vz
// taken as 0 as the 2-D step does); flux n x 8 in its output order and units (mass, x, y, z
// momentum, Bx, By, Bz, energy; the z-momentum flux is not formed by the 2-D step: 0);
// speed n values max(|S_L|, |S_R|).  The field goes to Heaviside-Lorentz units by the
// rounded product the tile load uses.  axis 0: normal +x.
__global__ void mhd_face_probe_kernel(Params P, long long n, int axis,
                                      const double* __restrict__ L,
                                      const double* __restrict__ R, double* flux,
                                      double* speed) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* a = L + 8 * i;
    const double* b = R + 8 * i;
    const bool isx = axis == 0;
    double qa[NF], qb[NF];
    qa[0] = a[0]; qa[1] = a[1]; qa[2] = a[2]; qa[3] = a[3];
    qb[0] = b[0]; qb[1] = b[1]; qb[2] = b[2]; qb[3] = b[3];
#pragma unroll
    for (int f = 4; f < NF; ++f) {
        qa[f] = __dmul_rn(a[f + 1], kInvSpi4);
        qb[f] = __dmul_rn(b[f + 1], kInvSpi4);
    }
    Side<double> A, B;
    side(A, qa[0], qa[1], isx ? qa[2] : qa[3], isx ? qa[3] : qa[2], isx ? qa[4] : qa[5],
         isx ? qa[5] : qa[4], qa[6], P);
    side(B, qb[0], qb[1], isx ? qb[2] : qb[3], isx ? qb[3] : qb[2], isx ? qb[4] : qb[5],
         isx ? qb[5] : qb[4], qb[6], P);
    double UU;
    const FluxM<double> F = hlld_local(A, B, P.method, P, UU);
    double* o = flux + 8 * i;
    o[0] = F.m;
    o[1] = isx ? F.mn : F.mt;
    o[2] = isx ? F.mt : F.mn;
    o[3] = 0.0;
    o[4] = (isx ? F.bn : F.bt) * kSpi4;
    o[5] = (isx ? F.bt : F.bn) * kSpi4;
    o[6] = F.bz * kSpi4;
    o[7] = F.e;
    speed[i] = dabs(UU);
}
}  // namespace

cudaError_t launch_mhd_face_probe(const Params& P, long long n, int axis, const double* L,
                                  const double* R, double* flux, double* speed,
                                  cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const long long blocks = (n + 255) / 256;
    mhd_face_probe_kernel<<<(unsigned int)blocks, 256, 0, st>>>(P, n, axis, L, R, flux, speed);
    return cudaGetLastError();
}

}  // namespace gd
