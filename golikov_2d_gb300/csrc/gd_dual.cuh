// gd_dual.cuh -- forward-mode dual numbers for the tangent (JVP) of the fast step.
//
// A Dual carries a value and one directional derivative.  The overloads mirror the double
// helpers of gd_internal.cuh, so the templated tile code (gd_mhd_tile.cuh) runs unchanged
// on either type: arithmetic propagates derivatives by the chain rule; comparisons,
// selections, guards and the minmod choice look at the value only, i.e. the derivative is
// taken along the branch the value takes (minmod, wave-speed min/max, region selection,
// floors).
#pragma once

#include "gd_internal.cuh"

namespace gd {

// keep the double overloads visible next to the Dual ones inside this namespace
using ::fma;
using ::isfinite;

struct Dual {
    double v, d;
};

__device__ __forceinline__ Dual make_dual(double v, double d = 0.0) { return Dual{v, d}; }

__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) {
    return {a.v * b.v, fma(a.v, b.d, a.d * b.v)};
}
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
__device__ __forceinline__ Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }

__device__ __forceinline__ Dual fma(Dual a, Dual b, Dual c) {
    return {::fma(a.v, b.v, c.v), ::fma(a.v, b.d, ::fma(a.d, b.v, c.d))};
}
__device__ __forceinline__ Dual fma(double a, Dual b, Dual c) {
    return {::fma(a, b.v, c.v), ::fma(a, b.d, c.d)};
}
__device__ __forceinline__ Dual fma(Dual a, double b, Dual c) {
    return {::fma(a.v, b, c.v), ::fma(a.d, b, c.d)};
}
__device__ __forceinline__ Dual fma(Dual a, Dual b, double c) {
    return {::fma(a.v, b.v, c), ::fma(a.v, b.d, a.d * b.v)};
}

__device__ __forceinline__ Dual rcp_fast(Dual x) {
    const double r = rcp_fast(x.v);
    return {r, -x.d * r * r};
}
__device__ __forceinline__ Dual rsqrt_fast(Dual x) {
    const double r = rsqrt_fast(x.v);
    return {r, -0.5 * x.d * r * r * r};
}
__device__ __forceinline__ Dual sqrt_fast(Dual x) {
    // the value as the double step computes it, so the tangent takes the step's branches
    double s, r;
    sqrt_and_rs(x.v, s, r);
    if (x.v == 0.0) return {0.0, 0.0};
    return {s, 0.5 * x.d * r};
}

// value-only predicates and selections (derivative follows the selected branch)
// values exactly as the double versions (the tangent takes the forward's branches)
__device__ __forceinline__ void rsqrt_and_sqrt(Dual x, Dual& ix, Dual& sx) {
    double i, s;
    rsqrt_and_sqrt(x.v, i, s);
    ix = {i, -0.5 * x.d * i * i * i};
    sx = {s, 0.5 * x.d * i};
}
__device__ __forceinline__ Dual sqrt_over(Dual a, Dual r) {
    // d sqrt(a / r) = sqrt(a / r) / 2 (da / a - dr / r); 0 at a = 0
    const double v = sqrt_over(a.v, r.v);
    if ((bits(a.v) << 1) == 0) return {v, 0.0};
    return {v, 0.5 * v * (a.d / a.v - r.d / r.v)};
}
// the values as the double versions compute them (the tangent takes the step's branches)
__device__ __forceinline__ Dual rcp_2op(Dual x) {
    const double r = rcp_2op(x.v);
    return {r, -x.d * r * r};
}
__device__ __forceinline__ Dual sqrt_over_2op(Dual a, Dual r) {
    const double v = sqrt_over_2op(a.v, r.v);
    if ((bits(a.v) << 1) == 0) return {v, 0.0};
    return {v, 0.5 * v * (a.d / a.v - r.d / r.v)};
}
__device__ __forceinline__ unsigned long long abs_bits(Dual x) { return abs_bits(x.v); }
__device__ __forceinline__ unsigned long long mag(Dual x) { return mag(x.v); }
__device__ __forceinline__ bool mag_lt(Dual a, Dual b) { return mag_lt(a.v, b.v); }
__device__ __forceinline__ bool mag_ge(Dual x, unsigned long long m) { return mag_ge(x.v, m); }
__device__ __forceinline__ bool le_zero(Dual x) { return le_zero(x.v); }
__device__ __forceinline__ bool gt_zero(Dual x) { return gt_zero(x.v); }
__device__ __forceinline__ bool lt_zero(Dual x) { return lt_zero(x.v); }
__device__ __forceinline__ bool ge_zero(Dual x) { return ge_zero(x.v); }
__device__ __forceinline__ bool isfinite(Dual x) { return ::isfinite(x.v); }
__device__ __forceinline__ bool finite_bits(Dual x) { return finite_bits(x.v); }
__device__ __forceinline__ bool quotient_neg(Dual n, Dual d) { return quotient_neg(n.v, d.v); }
template <bool OUTLINE = false>
__device__ __forceinline__ Dual mulx(Dual a, Dual b) { return a * b; }
template <bool OUTLINE = false>
__device__ __forceinline__ Dual mulx(double a, Dual b) { return a * b; }
template <bool OUTLINE = false>
__device__ __forceinline__ Dual mulx(Dual a, double b) { return a * b; }
template <bool OUTLINE = false>
__device__ __forceinline__ Dual sqrt_over_im(Dual a, Dual r) { return sqrt_over(a, r); }
template <bool OUTLINE = false>
__device__ __forceinline__ Dual sqrt_fast_im(Dual x) { return sqrt_fast(x); }
__device__ __forceinline__ Dual dabs(Dual x) { return lt_zero(x.v) ? -x : x; }
__device__ __forceinline__ Dual dmin(Dual a, Dual b) { return dlt(b.v, a.v) ? b : a; }
__device__ __forceinline__ Dual dmax(Dual a, Dual b) { return dlt(a.v, b.v) ? b : a; }
__device__ __forceinline__ Dual max_nonneg(Dual a, Dual b) {
    return mag_lt(a, b) ? b : a;
}
__device__ __forceinline__ Dual minmod(Dual a, Dual b) {
    const long long ba = bits(a.v), bb = bits(b.v);
    const bool zero = ((ba << 1) == 0) | ((bb << 1) == 0) | ((ba ^ bb) < 0);
    const Dual m = mag(a.v) <= mag(b.v) ? a : b;
    return zero ? Dual{0.0, 0.0} : m;
}
__device__ __forceinline__ double value_of(Dual x) { return x.v; }
__device__ __forceinline__ double value_of(double x) { return x; }

}  // namespace gd
