// gd_swfp.cuh -- IEEE-754 binary64 multiplication on the integer pipes.
//
// GB300 issues FP64 at 2 operations per clock per SM: one FP64 warp instruction holds an SM
// sub-partition's FP64 unit for 64 cycles, while the integer ALU and the IMAD path sit
// mostly idle in the step kernels.  mul_rn computes the binary64 product rounded to
// nearest even -- the bits of the hardware multiply -- with 32-bit integer instructions, so
// a kernel can move part of its multiplications off the FP64 pipe without changing a
// result bit.
//
//   dmul_fast: normal operands with a normal product (result exponent field in [1, 2045]
//              before rounding) and zero operands with a finite partner: four 32x32->64
//              multiply-adds for the 106-bit significand product, normalisation by one bit,
//              round-to-nearest-even, packing.  Reports !ok for everything else.
//   dmul_slow: every other case, still in integers: subnormal operands (normalised with a
//              count of leading zeros), subnormal and zero results (denormalised with the
//              shifted-out bits kept as sticky), overflow to infinity, infinities, and NaN
//              (every NaN result is the canonical quiet NaN 0x7fffffffffffffff; the payload is
//              the one thing that may differ from a hardware multiply).
//
// On the device the operands' 32-bit halves come out of inline PTX moves: the compiler then
// sees integers only, and cannot turn a bit test back into an FP64 compare (which would
// issue on the FP64 pipe).  Host-compilable (plain integer arithmetic) so the same code is
// checked against the host's IEEE multiplication on the CPU.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define GD_HD __host__ __device__ __forceinline__
#else
#define GD_HD inline
#endif

namespace gd {
namespace swfp {

constexpr uint64_t kQNaN = 0x7fffffffffffffffULL;
constexpr uint64_t kInf = 0x7ff0000000000000ULL;

GD_HD uint64_t to_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}
GD_HD double from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}
// the high and low 32-bit words of x, opaque to the compiler's floating-point reasoning
GD_HD void halves(double x, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
#else
    const uint64_t b = to_bits(x);
    hi = (uint32_t)(b >> 32);
    lo = (uint32_t)b;
#endif
}
GD_HD double from_halves(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
    double x;
    asm("mov.b64 %0, {%1, %2};" : "=d"(x) : "r"(lo), "r"(hi));
    return x;
#else
    return from_bits(((uint64_t)hi << 32) | lo);
#endif
}
GD_HD int clz64(uint64_t x) {  // x != 0
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

// a * b rounded to nearest even for the common case; ok = false where dmul_slow must be used.
GD_HD double dmul_fast(double a, double b, bool& ok) {
    uint32_t ah, al, bh, bl;
    halves(a, ah, al);
    halves(b, bh, bl);
    const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu;
    const uint32_t sign = (ah ^ bh) & 0x80000000u;
    // significands with the hidden bit, (m:lo) = 53 bits
    const uint32_t ma = (ah & 0xfffffu) | 0x100000u, mb = (bh & 0xfffffu) | 0x100000u;
    // P = ma mb in [2^104, 2^106) = t3 2^64 + lo(t2) 2^32 + lo(t0)
    const uint64_t t0 = (uint64_t)al * bl;
    const uint64_t t1 = (uint64_t)al * mb + (t0 >> 32);
    const uint64_t t2 = (uint64_t)ma * bl + t1;  // < 2^54
    const uint64_t t3 = (uint64_t)ma * mb + (t2 >> 32);
    const uint32_t n = (uint32_t)(t3 >> 41);  // 1 where P >= 2^105
    // P >> 51: the 53-bit significand of the result and its guard bit, one bit higher where n
    uint64_t g = (t3 << 13) | ((uint32_t)t2 >> 19);
    uint32_t sticky = ((uint32_t)t2 & 0x7ffffu) | (uint32_t)t0;
    sticky |= (uint32_t)g & n;
    g >>= n;
    // exponent field of the result minus one (the hidden bit of g >> 1 adds the one)
    const uint32_t e = ea + eb + n - 1024u;
    const uint32_t lsb_or_sticky = (uint32_t)(g >> 1) | (sticky != 0u ? 1u : 0u);
    const uint32_t rnd = (uint32_t)g & lsb_or_sticky & 1u;
    const uint64_t r = ((uint64_t)(sign | (e << 20)) << 32) + (g >> 1) + rnd;
    // zero operands (exponent and fraction fields zero): +-0 when the other one is finite
    const bool za = ((ah << 1) | al) == 0u, zb = ((bh << 1) | bl) == 0u;
    const bool zero = (za && eb != 0x7ffu) || (zb && ea != 0x7ffu);
    ok = zero || ((ea - 1u < 2046u) && (eb - 1u < 2046u) && (e < 2045u));
    return zero ? from_halves(sign, 0u) : from_halves((uint32_t)(r >> 32), (uint32_t)r);
}

// a * b rounded to nearest even, any operands (bit patterns in, bit pattern out)
GD_HD uint64_t dmul_slow(uint64_t A, uint64_t B) {
    const uint64_t S = (A ^ B) & 0x8000000000000000ULL;
    int ea = (int)((A >> 52) & 0x7ff), eb = (int)((B >> 52) & 0x7ff);
    uint64_t fa = A & 0xfffffffffffffULL, fb = B & 0xfffffffffffffULL;
    if ((ea == 0x7ff && fa != 0) || (eb == 0x7ff && fb != 0)) return kQNaN;
    const bool za = ea == 0 && fa == 0, zb = eb == 0 && fb == 0;
    if (ea == 0x7ff || eb == 0x7ff) return (za || zb) ? kQNaN : (S | kInf);
    if (za || zb) return S;
    if (ea == 0) {  // subnormal: normalise, the exponent goes to 1 - shift
        const int s = clz64(fa) - 11;
        fa <<= s;
        ea = 1 - s;
    } else {
        fa |= 1ULL << 52;
    }
    if (eb == 0) {
        const int s = clz64(fb) - 11;
        fb <<= s;
        eb = 1 - s;
    } else {
        fb |= 1ULL << 52;
    }
    const unsigned __int128 P = (unsigned __int128)fa * fb;  // [2^104, 2^106)
    const int n = (int)(P >> 105);
    int E = ea + eb - 1023 + n;  // exponent field where the significand is P >> (52 + n)
    if (E >= 2047) return S | kInf;
    int sh = 52 + n;
    if (E <= 0) {  // subnormal result: shift further, exponent field 0
        sh += 1 - E;
        E = 0;
        if (sh > 108) sh = 108;  // every bit below the rounding position
    }
    const uint64_t q = (uint64_t)(P >> sh);
    const bool guard = ((P >> (sh - 1)) & 1) != 0;
    const bool sticky = (P & ((((unsigned __int128)1) << (sh - 1)) - 1)) != 0;
    const uint64_t m = q + ((guard && (sticky || (q & 1))) ? 1 : 0);
    // normal: the hidden bit of m adds one to the field E - 1 (and a rounding carry to 2^53
    // adds one more); subnormal: m < 2^52 is the fraction, m = 2^52 is the smallest normal
    const uint64_t bits = E >= 1 ? ((uint64_t)(E - 1) << 52) + m : m;
    if ((bits >> 52) >= 0x7ff) return S | kInf;
    return S | bits;
}

// x / 2 and 2 x rounded to nearest even, every input, on the integer pipe: the exponent
// field moves by one; at the bottom of the range the magnitude shifts (a subnormal half
// rounds its dropped bit to even; a doubled subnormal may become normal, which the shifted
// pattern encodes as it is); 2 x above the range is infinity; infinities and NaN pass through.
GD_HD double half_rn(double x) {
    uint32_t hi, lo;
    halves(x, hi, lo);
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (e == 0x7ffu) return x;
    if (e >= 2u) return from_halves(hi - 0x100000u, lo);
    const uint32_t sign = hi & 0x80000000u, mh = hi & 0x7fffffffu;
    uint32_t nl = (lo >> 1) | (mh << 31), nh = mh >> 1;
    const uint32_t rnd = lo & nl & 1u;  // dropped bit set and the result odd: to even
    nl += rnd;
    nh += (nl < rnd) ? 1u : 0u;
    return from_halves(sign | nh, nl);
}
GD_HD double twice_rn(double x) {
    uint32_t hi, lo;
    halves(x, hi, lo);
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const uint32_t sign = hi & 0x80000000u;
    if (e == 0x7ffu) return x;
    if (e == 0x7feu) return from_halves(sign | 0x7ff00000u, 0u);
    if (e != 0u) return from_halves(hi + 0x100000u, lo);
    return from_halves(sign | ((hi << 1) & 0x7fffffffu) | (lo >> 31), lo << 1);
}

GD_HD float f32_from_bits(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
#endif
}
GD_HD uint32_t bits_of_f32(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t b;
    std::memcpy(&b, &f, sizeof b);
    return b;
#endif
}
// e as an FP32 value from its high word (20 bits of mantissa, truncated); 0 for |e| < 2^-126
GD_HD float high_f32(double e) {
    uint32_t hi, lo;
    halves(e, hi, lo);
    if (((hi >> 20) & 0x7ffu) <= 896u) return 0.0f;
    return f32_from_bits((hi & 0x80000000u) | (((hi & 0x7fffffffu) - (896u << 20)) << 3));
}
// w (1 + t 2^-52) for normal w and 0 <= t < 2^21 (the relative growth below 2^-31): the
// increment, w t 2^-52 in units of w's last place (at most 2^22), formed in FP32 and added to
// w's bit pattern; the magnitude grows (either sign of w).  An addition that carries into the
// exponent field counts the places beyond the binade boundary at the doubled size (halved,
// rounded half up).  Within one unit of the last place of the exact value.
GD_HD double grow_rel(double w, float t) {
    uint32_t hi, lo;
    halves(w, hi, lo);
    // w's significand in [1, 2) from its leading 23 bits
    const float mant = f32_from_bits(0x3f800000u | ((hi & 0xfffffu) << 3) | (lo >> 29));
#if defined(__CUDA_ARCH__)
    const float q = fmaf(mant, t, 12582912.0f);
#else
    const float q = std::fmaf(mant, t, 12582912.0f);
#endif
    const uint32_t m = bits_of_f32(q) - 0x4b400000u;  // round(mant t)
    uint32_t nlo = lo + m;
    const uint32_t c = nlo < lo ? 1u : 0u;
    if (c && (hi & 0xfffffu) == 0xfffffu) nlo = (nlo + 1u) >> 1;  // into the next binade
    return from_halves(hi + c, nlo);
}

#if defined(__CUDA_ARCH__)
static __device__ __noinline__ uint64_t dmul_slow_call(uint64_t A, uint64_t B) {
    return dmul_slow(A, B);
}
#endif

// a * b rounded to nearest even, any operands.  OUTLINE: on the device the rare general case
// is a call instead of an inlined copy, which keeps a kernel with many products smaller (the
// call's register conventions can cost more than that saves in a kernel tight on registers).
template <bool OUTLINE = false>
GD_HD double mul_rn(double a, double b) {
    bool ok;
    double r = dmul_fast(a, b, ok);
#if defined(__CUDA_ARCH__)
    if (!ok) r = from_bits(OUTLINE ? dmul_slow_call(to_bits(a), to_bits(b))
                                   : dmul_slow(to_bits(a), to_bits(b)));
#else
    if (!ok) r = from_bits(dmul_slow(to_bits(a), to_bits(b)));
#endif
    return r;
}

}  // namespace swfp
}  // namespace gd
