// gd_internal.cuh -- device-side types and helpers shared by the step kernels.
//
// FP64 on GB300 issues at a small fraction of the FP32 rate, so the step is bound by the
// FP64 pipe, not by HBM.  Everything that does not need the FP64 unit is done on the
// integer pipe here: sign tests, absolute values, minmod selection and max-reductions
// work on the IEEE-754 bit patterns, binary64 products can be formed there bit for bit
// (imul, from gd_swfp.cuh), and the small second-order terms of the Newton corrections are
// added into bit patterns (grow_rel).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gd2d.h"
#include "gd_swfp.cuh"

namespace gd {

constexpr int kMaxFields = 7;  // rho, p, vx, vy, Bx, By, Bz
constexpr double kSpi4 = 3.544907701811032;                 // sqrt(4 pi), Header.h:21
constexpr double kInvSpi4 = 0.28209479177387814347;         // 1/sqrt(4 pi)
constexpr double kCpi4 = 12.56637061435917295384;           // 4 pi, Header.h:19
constexpr double kCpi8 = 25.13274122871834590768;           // 8 pi, Header.h:20
constexpr double kTReset = 10000000.0;                      // funk_time, kernel.cu:1726
constexpr double kCellTmin0 = 1000.0;                       // per-cell start, kernel.cu:2216

// Launch-invariant parameters, passed by value.
struct Params {
    int N, M;
    int physics, geometry, order, method;
    int bc[4];
    double dx, dy, x0, y0;
    double gamma, krit;
    double frozen_radius;
    int frozen;           // frozen_radius > 0 (tested on the integer pipe)
    int scheme;           // GD_SCHEME_*
    double x_max, y_max;  // domain extents of the Hancock schemes' cell coordinates
    // A launch of the fast step over a band of tile rows (gd_step_host): the band starts at
    // tile row tile_row0 and has tile_rows rows (0: the whole grid); the blocks of all the
    // band launches of one step share one rotation ticket, tile_nblocks (0: this grid's).
    int tile_row0, tile_rows;
    unsigned int tile_nblocks;
    // derived
    double gm1, inv_gm1, hgm1;  // gamma - 1, 1 / (gamma - 1), (gamma - 1) / 2
    double g_gm1;               // gamma / (gamma - 1)
    double inv_dx, inv_dy;  // 1/dx, 1/dy: the fast kernels scale fluxes by T_do * inv_dx
    double ambient_p;   // 1/gamma
    double krad_x;      // krit * rad used for faces with an x normal
    double krad_y;      // krit * rad used for faces with a y normal
};

// A state: SoA planes, f[k] + m*N + n; or, where s is set, the reference's AoS layout
// (kernel.cu:3814-3825: s = {rho, p}, u = {vx, vy}, b = {Bx, By, Bz} per cell), which the
// drop-in step (gd_step_ref) and the host-to-host step (gd_step_host) read and write without
// a conversion pass.  An output with both set is written in both layouts.  Step kernels
// access a field of a cell through load_f / store_f; the layout test is the same for every
// thread of a launch.
struct Planes {
    double* f[kMaxFields];
    double *s, *u, *b;
};
struct CPlanes {
    const double* f[kMaxFields];
    const double *s, *u, *b;
};
__device__ __forceinline__ double load_f(const CPlanes& p, int f, long long k) {
    if (p.s == nullptr) return p.f[f][k];
    return f < 2 ? p.s[2 * k + f] : (f < 4 ? p.u[2 * k + (f - 2)] : p.b[3 * k + (f - 4)]);
}
__device__ __forceinline__ void store_f(const Planes& p, int f, long long k, double x) {
    if (p.f[0] != nullptr) p.f[f][k] = x;
    if (p.s != nullptr) {
        if (f < 2) p.s[2 * k + f] = x;
        else if (f < 4) p.u[2 * k + (f - 2)] = x;
        else p.b[3 * k + (f - 4)] = x;
    }
}
// The AoS pairs {rho, p} and {vx, vy} move as single 16-byte accesses where the array is
// 16-byte aligned (a double2 array always is; the test is the same for every thread).
__device__ __forceinline__ bool aligned16(const void* p) {
    return ((unsigned long long)p & 15ULL) == 0;
}
// fields f0 and f0 + 1 (f0 = 0: rho, p; f0 = 2: vx, vy) of cell k
__device__ __forceinline__ void store_pair(const Planes& p, int f0, long long k, double a,
                                           double b) {
    if (p.f[0] != nullptr) {
        p.f[f0][k] = a;
        p.f[f0 + 1][k] = b;
    }
    if (p.s != nullptr) {
        double* d = f0 == 0 ? p.s : p.u;
        if (aligned16(d)) {
            reinterpret_cast<double2*>(d)[k] = make_double2(a, b);
        } else {
            d[2 * k] = a;
            d[2 * k + 1] = b;
        }
    }
}
// the NF fields of cell k
template <int NF>
__device__ __forceinline__ void load_cell_fields(const CPlanes& in, long long k, double* v) {
    if (in.s == nullptr) {
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] = in.f[f][k];
        return;
    }
    if (aligned16(in.s) && aligned16(in.u)) {
        const double2 a = reinterpret_cast<const double2*>(in.s)[k];
        const double2 c = reinterpret_cast<const double2*>(in.u)[k];
        v[0] = a.x; v[1] = a.y; v[2] = c.x; v[3] = c.y;
    } else {
        v[0] = in.s[2 * k]; v[1] = in.s[2 * k + 1];
        v[2] = in.u[2 * k]; v[3] = in.u[2 * k + 1];
    }
    if (NF > 4) {
        v[4] = in.b[3 * k];
        v[5] = in.b[3 * k + 1];
        v[6] = in.b[3 * k + 2];
    }
}

struct Scalars;

// A side stream and the two events that fork the fast Hancock step's edge-band launch onto it
// and join it back (null: both launches on the caller's stream, one after the other).
struct HancockStreams {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};

// One grid of a batch, device-resident: its parameters, its two state buffers (nf planes
// of K doubles each), its scalars, and its tiling for the kernel variant in use.
struct BatchGrid {
    Params P;
    double* state[2];
    long long K;
    Scalars* sc;
    int tiles_x;
    int ntiles;
};

// Device-resident time-step scalars of one grid (the reference's T, T_do, TT, i).
struct Scalars {
    unsigned long long T_bits;  // running min of the CFL dt, as the bits of a positive double
    double T_do;                // dt used by the current step
    double TT;                  // simulated time
    long long step;             // steps taken
    unsigned int done;          // blocks finished in the current launch (last-block rotation)
    unsigned int pad;
    unsigned long long rho_floor, p_floor, nonfinite;
    double t_state;  // simulated time of the current state: the sum of the dt each step used
    double t_end;    // > 0: no step is given a dt that carries t_state past it (gd_advance_to)
    double T_cfl;    // the last CFL dt before that limit
};

// The dt the next step will use: T, or what is left to t_end when that is set.
__device__ __forceinline__ double clamp_to_end(const Scalars* sc, double T) {
    if (sc->t_end > 0.0) {
        const double rem = sc->t_end - sc->t_state;
        const double r = rem > 0.0 ? rem : 0.0;
        return T < r ? T : r;
    }
    return T;
}

// ---------------------------------------------------------------------------------------
// Bit-pattern helpers (integer pipe).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ double from_bits(long long b) { return __longlong_as_double(b); }

// The magnitude of x as an order key: the bit pattern shifted left by one, which drops the
// sign.  For non-NaN a, b: mag(a) < mag(b) <=> |a| < |b|, and mag(x) >> 53 is the biased
// exponent.  Magnitude comparisons must stay integer operations, and the compiler is apt to
// turn them into FP64 ones: a mask of the sign bit becomes fabs, issued on the FP64 pipe
// where no FP64 instruction absorbs it as an operand modifier, and a test of the key against
// zero becomes an FP64 comparison (measured on sm_103a: two FP64 operations per minmod
// either way, 18 per Euler cell).  The comparisons the step kernels make per face or per
// cell (mag_lt, mag_ge, minmod) are therefore written in inline PTX, which the compiler keeps
// as integer operations.
__device__ __forceinline__ unsigned long long mag(double x) {
    return (unsigned long long)bits(x) << 1;
}
// |a| < |b| for non-NaN a, b
__device__ __forceinline__ bool mag_lt(double a, double b) {
    unsigned int r;
    asm("{\n\t.reg .b64 ma, mb;\n\t.reg .pred p;\n\t"
        "shl.b64 ma, %1, 1;\n\tshl.b64 mb, %2, 1;\n\t"
        "setp.lt.u64 p, ma, mb;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r) : "l"(bits(a)), "l"(bits(b)));
    return r != 0;
}
// mag(x) >= m (m a magnitude key)
__device__ __forceinline__ bool mag_ge(double x, unsigned long long m) {
    unsigned int r;
    asm("{\n\t.reg .b64 mx;\n\t.reg .pred p;\n\t"
        "shl.b64 mx, %1, 1;\n\tsetp.ge.u64 p, mx, %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r) : "l"(bits(x)), "l"(m));
    return r != 0;
}
// mag() of 1e-5 and 1e-6, the HLLD guards' thresholds (Gas_Dinamic.cu:1306-1369)
constexpr unsigned long long kMag1em5 = 0x3EE4F8B588E368F1ULL << 1;
constexpr unsigned long long kMag1em6 = 0x3EB0C6F7A0B5ED8DULL << 1;
// The bit pattern of |x|, masked in inline PTX so that it stays an integer operation.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    unsigned long long r;
    asm("and.b64 %0, %1, 0x7FFFFFFFFFFFFFFF;" : "=l"(r) : "l"(bits(x)));
    return r;
}
// |x| for use as an FP64 operand (free there as an operand modifier)
__device__ __forceinline__ double dabs(double x) { return fabs(x); }
// x <= 0 (for non-NaN x): sign bit set, or +0.
__device__ __forceinline__ bool le_zero(double x) { return bits(x) <= 0; }
// x > 0 (for non-NaN x)
__device__ __forceinline__ bool gt_zero(double x) { return bits(x) > 0; }

// Of two values, the one of larger magnitude (for non-negative values, the larger), by bit
// pattern.
__device__ __forceinline__ double max_nonneg(double a, double b) {
    return mag_lt(a, b) ? b : a;
}

// minmod(a, b): 0 unless a and b are non-zero with the same sign, else the one of smaller
// magnitude.  Equal, bit for bit, to the reference's (sign(a)+sign(b))/2 * min(|a|,|b|)
// (kernel.cu:51-62) for non-NaN inputs.  The sign, zero and magnitude tests and both
// selects are integer operations in inline PTX (see mag).
__device__ __forceinline__ double minmod(double a, double b) {
    long long r;
    asm("{\n\t.reg .b64 ma, mb, s;\n\t.reg .pred pz, pl;\n\t"
        "shl.b64 ma, %1, 1;\n\t"
        "shl.b64 mb, %2, 1;\n\t"
        "xor.b64 s, %1, %2;\n\t"
        "setp.lt.s64 pz, s, 0;\n\t"          // signs differ
        "setp.eq.or.u64 pz, ma, 0, pz;\n\t"  // or a is +-0
        "setp.eq.or.u64 pz, mb, 0, pz;\n\t"  // or b is +-0
        "setp.le.u64 pl, ma, mb;\n\t"
        "selp.b64 %0, %1, %2, pl;\n\t"
        "selp.b64 %0, 0, %0, pz;\n\t"
        "}"
        : "=l"(r) : "l"(bits(a)), "l"(bits(b)));
    return from_bits(r);
}

// Order-preserving integer key of a double (non-NaN): a < b  <=>  key(a) < key(b), with
// -0 ordered just below +0.  Comparisons on the integer pipe instead of DSETP / DMNMX,
// which issue on the FP64 pipe.
__device__ __forceinline__ long long okey(double x) {
    const long long b = bits(x);
    return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool dlt(double a, double b) { return okey(a) < okey(b); }
__device__ __forceinline__ double dmin(double a, double b) { return dlt(b, a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return dlt(a, b) ? b : a; }
// x < 0 strictly (-0 is not negative), x >= 0: the bit pattern, as unsigned, above -0's
__device__ __forceinline__ bool lt_zero(double x) {
    return (unsigned long long)bits(x) > 0x8000000000000000ULL;
}
__device__ __forceinline__ bool ge_zero(double x) { return !lt_zero(x); }
// n / d < 0 strictly, from the bit patterns (inline PTX, see mag): the signs differ and n is
// not +-0
__device__ __forceinline__ bool quotient_neg(double n, double d) {
    unsigned int r;
    asm("{\n\t.reg .b64 x, m;\n\t.reg .pred p;\n\t"
        "xor.b64 x, %1, %2;\n\t"
        "shl.b64 m, %1, 1;\n\t"
        "setp.lt.s64 p, x, 0;\n\t"
        "setp.ne.and.u64 p, m, 0, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t"
        "}"
        : "=r"(r) : "l"(bits(n)), "l"(bits(d)));
    return r != 0;
}

// ---------------------------------------------------------------------------------------
// FP64 reciprocal and reciprocal square root for the fast path.
//
// Seed: the double's high word is re-biased into an FP32 bit pattern on the integer pipe
// (no F2F conversion, which issues on the FP64 pipe), the FP32 special-function unit gives
// rcp / rsqrt of it (relative error ~2^-20 from the truncated mantissa), and the FP32
// result is re-biased back into a double.  One third-order Newton-Raphson step in FP64
// then brings the relative error from e ~ 2^-20 to O(e^3) ~ 2^-60, below double rounding:
//   reciprocal:  e = 1 - x y,    y <- y (1 + e + e^2)
//   rsqrt:       e = 1 - x y^2,  y <- y (1 + e/2 + 3 e^2 / 8)
// Valid for |x| in [2^-120, 2^120]; outside it the correctly rounded operation is used.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool in_f32_range(double x) {
    // biased exponent within [1023-120, 1023+120]
    const unsigned int e = (unsigned int)(mag(x) >> 53);
    return (e - 903u) <= 240u;
}

__device__ __forceinline__ float seed_f32(double x) {
    const int hi = __double2hiint(x);
    return __int_as_float((hi & (int)0x80000000) | (((hi & 0x7fffffff) - (896 << 20)) << 3));
}

__device__ __forceinline__ double widen_f32(float f) {
    const int b = __float_as_int(f);
    return __hiloint2double((b & (int)0x80000000) | (((b & 0x7fffffff) >> 3) + (896 << 20)),
                            (b & 7) << 29);
}

__device__ __forceinline__ double rcp_fast(double x) {
    if (!in_f32_range(x)) return 1.0 / x;
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(seed_f32(x)));
    const double y = widen_f32(r);
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// The fast reciprocal square root applies to x > 0 in the seeded range (tested on the
// integer pipe); NaN, +-0, negative and out-of-range values take the correctly rounded path.
__device__ __forceinline__ bool rsqrt_ok(double x) { return in_f32_range(x) && gt_zero(x); }

// the seeded FP32 estimate of 1/sqrt(x) and one third-order Newton step; x as rsqrt_ok
__device__ __forceinline__ double rsqrt_newton(double x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(seed_f32(x)));
    const double y = widen_f32(r);
    const double e = fma(-x * y, y, 1.0);
    return fma(y, e * fma(0.375, e, 0.5), y);
}

__device__ __forceinline__ double rsqrt_fast(double x) {
    if (!rsqrt_ok(x)) return 1.0 / sqrt(x);
    return rsqrt_newton(x);
}

// sqrt(x) and 1/sqrt(x) from one seed y ~ 1/sqrt(x): with w = x y and e = 1 - w y,
// sqrt(x) = w (1 + e/2 + 3 e^2 / 8) and 1/sqrt(x) = y (1 + e/2 + 3 e^2 / 8) to O(e^3): five
// FP64 operations for the root alone, where x * rsqrt(x) takes six.  Outside the fast range
// (rsqrt_ok), the correctly rounded pair, with sqrt(+-0) = 0 exactly.
__device__ __forceinline__ void sqrt_and_rs(double x, double& sx, double& ix) {
    if (!rsqrt_ok(x)) {
        sx = sqrt(x);
        ix = 1.0 / sx;
        return;
    }
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(seed_f32(x)));
    const double y = widen_f32(r);
    const double w = x * y;
    const double e = fma(-w, y, 1.0);
    const double et = e * fma(0.375, e, 0.5);
    sx = fma(w, et, w);
    ix = fma(y, et, y);
}
__device__ __forceinline__ double sqrt_fast(double x) {
    double sx, ix;
    sqrt_and_rs(x, sx, ix);
    return sx;
}

// 1/sqrt(x) and sqrt(x) = x / sqrt(x) together; where the fast path does not apply, the
// correctly rounded pair (x = 0: sqrt 0 and 1/sqrt inf, as the reference's sqrt(x))
__device__ __forceinline__ void rsqrt_and_sqrt(double x, double& ix, double& sx) {
    if (!rsqrt_ok(x)) {
        sx = sqrt(x);
        ix = 1.0 / sx;
        return;
    }
    ix = rsqrt_newton(x);
    sx = x * ix;
}

// 1/sqrt(a r), except 0 where a = +-0, for the product a * rsqrt(a r) = sqrt(a / r): the
// zero test sits in the slow branch only, so the fast path is rsqrt_fast's
__device__ __forceinline__ double rsqrt_times(double a, double r) {
    const double x = a * r;
    if (!rsqrt_ok(x)) return (bits(a) << 1) == 0 ? 0.0 : 1.0 / sqrt(x);
    return rsqrt_newton(x);
}

// The seed of 1/sqrt(a r) without the FP64 product: the leading 23 bits of each factor
// re-biased into FP32 (integer pipe), one FP32 product, the FP32 rsqrt; valid for a and r
// positive with exponents within +-60 of 1 (each factor's truncation 2^-23, the product's
// rounding 2^-24, the rsqrt's error ~2^-23: a relative seed error below 2^-21).
__device__ __forceinline__ bool in_half_range_pos(double x) {
    const unsigned int e = (unsigned int)(mag(x) >> 53);
    return gt_zero(x) && (e - 963u) <= 120u;
}
__device__ __forceinline__ float seed23_f32(double x) {
    const int hi = __double2hiint(x);
    const unsigned int lo = (unsigned int)__double2loint(x);
    return __int_as_float((hi & (int)0x80000000) |
                          (((hi & 0x7fffffff) - (896 << 20)) << 3) | (int)(lo >> 29));
}

// sqrt(a / r) (a sound or fast magnetosonic speed, a >= 0) and 1/sqrt(a r).  With y the seed
// of 1/sqrt(a r), w = a y and e = 1 - w r y: sqrt(a / r) = w (1 + e/2 + 3 e^2 / 8) to O(e^3),
// six FP64 operations where a * rsqrt(a r) takes seven.  Outside the seeded range: a = 0
// gives 0, as the reference's sqrt(a / r) (the plain product would be 0 * inf); r = 0 gives
// inf and r < 0 NaN, as there.
__device__ __forceinline__ void sqrt_over_rs(double a, double r, double& c, double& rs) {
    if (!(in_half_range_pos(a) && in_half_range_pos(r))) {
        rs = rsqrt_times(a, r);
        c = a * rs;
        return;
    }
    float f;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(f) : "f"(seed23_f32(a) * seed23_f32(r)));
    const double y = widen_f32(f);
    const double w = a * y;
    const double e = fma(-w, r * y, 1.0);
    const double et = e * fma(0.375, e, 0.5);
    c = fma(w, et, w);
    rs = fma(y, et, y);
}
__device__ __forceinline__ double sqrt_over(double a, double r) {
    double c, rs;
    sqrt_over_rs(a, r, c, rs);
    return c;
}

// a * b formed on the integer pipes (swfp::mul_rn: the bits of the FP64 multiply, NaN
// payloads aside), leaving the FP64 unit to the kernel's other operations
// (OUTLINE: the general case out of line, see swfp::mul_rn)
template <bool OUTLINE = false>
__device__ __forceinline__ double imul(double a, double b) {
    return swfp::mul_rn<OUTLINE>(a, b);
}
template <bool OUTLINE = false>
__device__ __forceinline__ double mulx(double a, double b) { return imul<OUTLINE>(a, b); }

// sqrt_fast with its products on the integer pipes
template <bool OUTLINE = false>
__device__ __forceinline__ double sqrt_fast_im(double x) {
    if (!rsqrt_ok(x)) return sqrt(x);
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(seed_f32(x)));
    const double y = widen_f32(r);
    const double w = imul<OUTLINE>(x, y);
    const double e = fma(-w, y, 1.0);
    return fma(w, imul<OUTLINE>(e, fma(0.375, e, 0.5)), w);
}
// sqrt_over with its three products on the integer pipes
template <bool OUTLINE = false>
__device__ __forceinline__ double sqrt_over_im(double a, double r) {
    if (!(in_half_range_pos(a) && in_half_range_pos(r))) return a * rsqrt_times(a, r);
    float f;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(f) : "f"(seed23_f32(a) * seed23_f32(r)));
    const double y = widen_f32(f);
    const double w = imul<OUTLINE>(a, y);
    const double e = fma(-w, imul<OUTLINE>(r, y), 1.0);
    const double et = imul<OUTLINE>(e, fma(0.375, e, 0.5));
    return fma(w, et, w);
}

// sqrt_and_rs with its products on the integer pipes: the same sx as sqrt_fast_im
template <bool OUTLINE = false>
__device__ __forceinline__ void sqrt_and_rs_im(double x, double& sx, double& ix) {
    if (!rsqrt_ok(x)) {
        sx = sqrt(x);
        ix = 1.0 / sx;
        return;
    }
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(seed_f32(x)));
    const double y = widen_f32(r);
    const double w = imul<OUTLINE>(x, y);
    const double e = fma(-w, y, 1.0);
    const double et = imul<OUTLINE>(e, fma(0.375, e, 0.5));
    sx = fma(w, et, w);
    ix = fma(y, et, y);
}
// sqrt_over_rs with its products on the integer pipes: the same c as sqrt_over_im
template <bool OUTLINE = false>
__device__ __forceinline__ void sqrt_over_rs_im(double a, double r, double& c, double& rs) {
    if (!(in_half_range_pos(a) && in_half_range_pos(r))) {
        rs = rsqrt_times(a, r);
        c = a * rs;
        return;
    }
    float f;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(f) : "f"(seed23_f32(a) * seed23_f32(r)));
    const double y = widen_f32(f);
    const double w = imul<OUTLINE>(a, y);
    const double e = fma(-w, imul<OUTLINE>(r, y), 1.0);
    const double et = imul<OUTLINE>(e, fma(0.375, e, 0.5));
    c = fma(w, et, w);
    rs = fma(y, et, y);
}
// ---------------------------------------------------------------------------------------
// Root and reciprocal in two FP64 operations.  The Newton corrections above,
//   sqrt(a / r) = w (1 + e/2 + 3 e^2 / 8),   1 / x = y (1 + e + e^2),
// take three: the residual e, the polynomial in e, the final multiply-add.  The quadratic
// term is 2^-40 or less of the result, so FP32 resolves it: w (3 e^2 / 8) (or y e^2) is formed
// in FP32 as a count of w's last place (at most 2^22) and added to w's bit pattern (integer
// pipe); the final multiply-add then takes w e/2 (or y e) on top.  An addition that carries
// into w's exponent field counts the places beyond the binade boundary at the doubled size
// (halved, rounded).  Measured on the device against IEEE results (gd_check_fast_roots,
// 67 M values): the reciprocal within 1 ulp of 1/x, the root within 2 ulp of the IEEE
// sqrt(a / r) -- which itself rounds twice -- where the three-operation root stays within 1.
// ---------------------------------------------------------------------------------------
// e as an FP32 value (high word), and w grown by t 2^-52 of itself on the integer pipe (swfp)
__device__ __forceinline__ float small_f32(double e) { return swfp::high_f32(e); }
__device__ __forceinline__ double grow_rel(double w, float t) { return swfp::grow_rel(w, t); }
// x / 2 and 2 x, exactly as the FP64 unit rounds them, on the integer pipe (swfp)
__device__ __forceinline__ double half_exact(double x) { return swfp::half_rn(x); }
__device__ __forceinline__ double twice_exact(double x) { return swfp::twice_rn(x); }
// sqrt(a / r) as sqrt_over_im, and (with rs) 1/sqrt(a r), the root in two FP64 operations
__device__ __forceinline__ double sqrt_over_2op(double a, double r, double* rs = nullptr) {
    if (!(in_half_range_pos(a) && in_half_range_pos(r))) {
        const double q = rsqrt_times(a, r);
        if (rs) *rs = q;
        return a * q;
    }
    float f;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(f) : "f"(seed23_f32(a) * seed23_f32(r)));
    const double y = widen_f32(f);
    const double w = imul(a, y);
    const double e = fma(-w, imul(r, y), 1.0);
    const float ef = small_f32(e);
    const double wq = grow_rel(w, (ef * ef) * 1688849860263936.0f);  // 3/8 2^52
    if (rs) *rs = fma(y, imul(e, fma(0.375, e, 0.5)), y);
    return fma(half_exact(w), e, wq);
}
// 1/x as rcp_fast, in two FP64 operations
__device__ __forceinline__ double rcp_2op(double x) {
    if (!in_f32_range(x)) return 1.0 / x;
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(seed_f32(x)));
    const double y = widen_f32(r);
    const double e = fma(-x, y, 1.0);
    const float ef = small_f32(e);
    return fma(y, e, grow_rel(y, (ef * ef) * 4503599627370496.0f));  // 2^52
}

// isfinite(x) on the integer pipe: the exponent field is not all ones
__device__ __forceinline__ bool finite_bits(double x) {
    return (mag(x) >> 53) != 0x7ffULL;
}

// ---------------------------------------------------------------------------------------
// Ghost values.  Two ghost layers per side; depth 1 is adjacent to the edge cell.  The
// reference's per-cell boundary branches (kernel.cu:2226-2405) produce exactly these values
// for every stencil position: mirror conditions reflect the cell at the same distance from
// the edge, the outflow and ambient conditions use the same value at both depths.
// ---------------------------------------------------------------------------------------

// Index of the interior cell that supplies ghost `g` (g < 0 or g >= n) for condition bc.
__device__ __forceinline__ int ghost_source(int g, int n, int bc) {
    if (bc == GD_BC_PERIODIC) return g < 0 ? g + n : g - n;
    const bool low = g < 0;
    const int depth = low ? -g : g - n + 1;  // 1 or 2
    if (bc == GD_BC_MIRROR_X || bc == GD_BC_AXIS) return low ? depth - 1 : n - depth;
    return low ? 0 : n - 1;
}

// Apply the value transformation of condition bc to a fetched state v[0..nf).
// Field order: rho, p, vx, vy, bx, by, bz.
template <int NF>
__device__ __forceinline__ void ghost_transform(double* v, int bc, double ambient_p) {
    switch (bc) {
        case GD_BC_MIRROR_X:
            v[2] = -v[2];
            if (NF > 4) { v[4] = -v[4]; v[5] = -v[5]; }
            break;
        case GD_BC_AXIS:
            v[3] = -v[3];
            if (NF > 4) v[6] = -v[6];
            break;
        case GD_BC_AMBIENT:
            v[0] = 1.0; v[1] = ambient_p; v[2] = 0.0; v[3] = 0.0;
            if (NF > 4) { v[4] = 0.0; v[5] = 0.0; v[6] = 0.0; }
            break;
        case GD_BC_AMBIENT_KEEPB:
            v[0] = 1.0; v[1] = ambient_p; v[2] = 0.0; v[3] = 0.0;
            break;
        case GD_BC_OUTFLOW:
            if (v[2] < 0) v[2] = 0.01;
            break;
        default:
            break;
    }
}

// State of cell (gx, gy); at most one coordinate may lie outside the grid, by 1 or 2.
template <int NF>
__device__ __forceinline__ void fetch_cell(const Params& P, const CPlanes& in, int gx, int gy,
                                           double* v) {
    int sx = gx, sy = gy, bc = -1;
    if (gx < 0 || gx >= P.N) {
        bc = gx < 0 ? P.bc[0] : P.bc[1];
        sx = ghost_source(gx, P.N, bc);
    } else if (gy < 0 || gy >= P.M) {
        bc = gy < 0 ? P.bc[2] : P.bc[3];
        sy = ghost_source(gy, P.M, bc);
    }
    const long long k = (long long)sy * P.N + sx;
    load_cell_fields<NF>(in, k, v);
    if (bc >= 0) ghost_transform<NF>(v, bc, P.ambient_p);
}

// Inside the grid and not frozen (kernel.cu:2205, 2218: dist = sqrt(x*x + y*y) < ddist).
__device__ __forceinline__ bool cell_active(const Params& P, int gx, int gy) {
    if (gx < 0 || gx >= P.N || gy < 0 || gy >= P.M) return false;
    if (!P.frozen) return true;
    const double x = P.x0 + gx * P.dx, y = P.y0 + gy * P.dy;
    // explicit roundings: every build and every call site decides alike (the parity build,
    // without contraction, computes the same sum)
    return !(sqrt(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y))) < P.frozen_radius);
}

// ---------------------------------------------------------------------------------------
// Block-level dt reduction and the fused funk_time rotation (kernel.cu:1722-1733).
// ---------------------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Called by one thread of each block after the block's dt is combined: the last block of
// the launch to arrive performs the funk_time rotation on `sc` (T_do <- T, TT += T_do,
// T <- 1e7, ++step).  `nblocks` blocks report per launch; 0 means every block of the grid.
__device__ __forceinline__ void rotate_if_last(Scalars* sc, unsigned int nblocks) {
    __threadfence();
    const unsigned int nb = nblocks ? nblocks : gridDim.x * gridDim.y * gridDim.z;
    const unsigned int ticket = atomicAdd(&sc->done, 1u);
    if (ticket == nb - 1) {
        __threadfence();
        sc->t_state = sc->t_state + sc->T_do;
        const double Tc = from_bits((long long)atomicAdd(&sc->T_bits, 0ULL));
        sc->T_cfl = Tc;
        const double T = clamp_to_end(sc, Tc);
        sc->T_do = T;
        sc->TT = sc->TT + T;
        sc->T_bits = (unsigned long long)bits(kTReset);
        sc->step = sc->step + 1;
        sc->done = 0;
        __threadfence();
    }
}

// Reduces the per-thread maximum wave speeds of x and y faces over the block, turns them
// into the block's dt (min over faces of krit*rad/UU, capped at 1000) and min-combines it
// into *T_bits.  `any_active` says whether the block contains a non-frozen cell.  Then,
// if `sc` is given, the last block to finish performs the funk_time rotation on it.
// Must be called by every thread of the block.
// `nblocks` is the number of blocks (tiles) that report to `sc` in this launch; 0 means
// every block of the grid.
template <int NTHREADS>
__device__ void block_dt_and_rotate(const Params& P, double umax_x, double umax_y,
                                    bool any_active, unsigned long long* T_bits,
                                    Scalars* sc, unsigned int nblocks = 0) {
    __shared__ unsigned long long red[2][NTHREADS / 32];
    __shared__ int act[NTHREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long ax = warp_max_u64(abs_bits(umax_x));
    unsigned long long ay = warp_max_u64(abs_bits(umax_y));
    int a = __any_sync(0xffffffffu, any_active);
    if (lane == 0) {
        red[0][warp] = ax;
        red[1][warp] = ay;
        act[warp] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long mx = 0, my = 0;
        int any = 0;
        for (int w = 0; w < NTHREADS / 32; ++w) {
            mx = red[0][w] > mx ? red[0][w] : mx;
            my = red[1][w] > my ? red[1][w] : my;
            any |= act[w];
        }
        if (any) {
            double t = kCellTmin0;
            const double ux = from_bits((long long)mx), uy = from_bits((long long)my);
            if (mx != 0) {
                const double tx = P.krad_x / ux;
                t = tx < t ? tx : t;
            }
            if (my != 0) {
                const double ty = P.krad_y / uy;
                t = ty < t ? ty : t;
            }
            atomicMin(T_bits, (unsigned long long)bits(t));
        }
        if (sc != nullptr) rotate_if_last(sc, nblocks);
    }
}

// Block minimum of per-thread dt values (positive doubles order like their bit patterns),
// min-combined into *T_bits when the block holds an active cell, then the funk_time
// rotation as in block_dt_and_rotate (`nblocks` as there).  Must be called by every thread
// of the block.
template <int NTHREADS>
__device__ void block_tmin_and_rotate(double tmin, bool active, unsigned long long* T_bits,
                                      Scalars* sc, unsigned int nblocks = 0) {
    __shared__ unsigned long long red[NTHREADS / 32];
    __shared__ int act[NTHREADS / 32];
    unsigned long long tb = active ? (unsigned long long)bits(tmin) : ~0ULL;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, tb, o);
        tb = w < tb ? w : tb;
    }
    const int a = __any_sync(0xffffffffu, active);
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = tb;
        act[threadIdx.x >> 5] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long mn = ~0ULL;
        int any = 0;
        for (int w = 0; w < NTHREADS / 32; ++w) {
            mn = red[w] < mn ? red[w] : mn;
            any |= act[w];
        }
        if (any) atomicMin(T_bits, mn);
        if (sc != nullptr) rotate_if_last(sc, nblocks);
    }
}

}  // namespace gd
