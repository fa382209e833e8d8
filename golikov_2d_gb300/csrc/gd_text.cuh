// gd_text.cuh -- exact decimal text conversion of doubles for the state I/O kernels.
//
// The reference writes its restart and Tecplot files with C++ streams at their default
// format (kernel.cu:3682-3808, 4253-4254): `os << double` is printf "%.6g" -- six significant
// digits, round-half-even on the exact binary value, %f or %e style by the decimal
// exponent, trailing zeros removed.  It reads restart files with `is >> double`
// (kernel.cu:3944-3996), i.e. a correctly rounded decimal-to-double conversion.
//
// Both directions are done here without a host library: a fast path in FP64 whose single
// rounding provably cannot change the answer, and an exact fallback on arbitrary-precision
// integers (m 2^e against c 10^s, compared as integers) for the cases near a rounding
// boundary and outside the range of exact powers of ten.  Everything is __host__ __device__
// so the same code serves every kernel.
#pragma once

#include <cmath>
#include <cstdint>

#include "gd_pow10.h"

#ifdef __CUDACC__
#define GD_HD __host__ __device__ __forceinline__
#else
#define GD_HD inline
#endif

namespace gd {
namespace text {

// ---- arbitrary-precision unsigned integers (little-endian 32-bit limbs) ------------------
// 48 limbs (1536 bits) hold every product formed below: at most a 53-bit mantissa or a
// 400-digit decimal significand times 5^400 times 2^1100.
struct Big {
    static constexpr int kLimbs = 48;
    uint32_t w[kLimbs];
    int n;  // limbs in use; w[n-1] != 0 unless n == 0 (the value 0)
};

GD_HD void big_set(Big& a, uint64_t v) {
    a.n = 0;
    while (v) {
        a.w[a.n++] = (uint32_t)v;
        v >>= 32;
    }
}

// a = a * m + add (m, add < 2^32); false on limb overflow
GD_HD bool big_muladd(Big& a, uint32_t m, uint32_t add) {
    uint64_t carry = add;
    for (int i = 0; i < a.n; ++i) {
        const uint64_t t = (uint64_t)a.w[i] * m + carry;
        a.w[i] = (uint32_t)t;
        carry = t >> 32;
    }
    if (carry) {
        if (a.n == Big::kLimbs) return false;
        a.w[a.n++] = (uint32_t)carry;
    }
    return true;
}

// a *= 5^k (k >= 0)
GD_HD bool big_mul_pow5(Big& a, int k) {
    while (k >= 13) {  // 5^13 = 1220703125 < 2^32
        if (!big_muladd(a, 1220703125u, 0u)) return false;
        k -= 13;
    }
    uint32_t p = 1;
    while (k-- > 0) p *= 5u;
    return p == 1 ? true : big_muladd(a, p, 0u);
}

// a <<= s (s >= 0)
GD_HD bool big_shl(Big& a, int s) {
    if (a.n == 0 || s == 0) return true;
    const int limbs = s >> 5, bits = s & 31;
    if (a.n + limbs + 1 > Big::kLimbs) return false;
    if (bits) {
        a.w[a.n] = 0;
        for (int i = a.n; i >= 0; --i) {
            const uint32_t hi = a.w[i] << bits;
            const uint32_t lo = i > 0 ? a.w[i - 1] >> (32 - bits) : 0u;
            a.w[i] = hi | lo;
        }
        a.n += 1;
    }
    if (limbs) {
        for (int i = a.n - 1; i >= 0; --i) a.w[i + limbs] = a.w[i];
        for (int i = 0; i < limbs; ++i) a.w[i] = 0;
        a.n += limbs;
    }
    while (a.n > 0 && a.w[a.n - 1] == 0) --a.n;
    return true;
}

GD_HD int big_cmp(const Big& a, const Big& b) {
    if (a.n != b.n) return a.n < b.n ? -1 : 1;
    for (int i = a.n - 1; i >= 0; --i)
        if (a.w[i] != b.w[i]) return a.w[i] < b.w[i] ? -1 : 1;
    return 0;
}

// ---- doubles as exact integer pairs --------------------------------------------------------

GD_HD uint64_t dbits(double x) {
    union {
        double d;
        uint64_t u;
    } c;
    c.d = x;
    return c.u;
}
GD_HD double from_dbits(uint64_t u) {
    union {
        double d;
        uint64_t u;
    } c;
    c.u = u;
    return c.d;
}

// |x| = m 2^e exactly (x finite, non-zero)
GD_HD void decompose(double x, uint64_t& m, int& e) {
    const uint64_t b = dbits(x) & 0x7fffffffffffffffULL;
    const int be = (int)(b >> 52);
    const uint64_t f = b & 0x000fffffffffffffULL;
    if (be == 0) {
        m = f;
        e = -1074;
    } else {
        m = f | (1ULL << 52);
        e = be - 1075;
    }
}

// kFail if the limbs overflow (not reachable for the operands formed here)
constexpr int kFail = 99;

// sign of (m 2^e) - (c 10^s), exact; m > 0, c >= 0
GD_HD int cmp_bin_dec(uint64_t m, int e, const Big& c, int s) {
    Big L, R;
    big_set(L, m);
    R = c;
    bool ok;
    // m 2^e  vs  c 5^s 2^s
    if (s >= 0) ok = big_mul_pow5(R, s);
    else ok = big_mul_pow5(L, -s);
    const int sh = e - s;
    if (ok) ok = sh >= 0 ? big_shl(L, sh) : big_shl(R, -sh);
    if (!ok) return kFail;
    return big_cmp(L, R);
}

// 10^k for 0 <= k <= 22, exact in binary64
GD_HD double pow10_exact(int k) {
    double p = 1.0, b = 10.0;
    while (k) {
        if (k & 1) p *= b;
        b *= b;
        k >>= 1;
    }
    return p;
}

// x 10^k by exact powers of ten (an estimate when |k| > 22)
GD_HD double scale10(double x, int k) {
    while (k > 22) {
        x *= 1e22;
        k -= 22;
    }
    while (k < -22) {
        x /= 1e22;
        k += 22;
    }
    return k >= 0 ? x * pow10_exact(k) : x / pow10_exact(-k);
}

// ---- double -> "%.6g" --------------------------------------------------------------------

constexpr int kPrec = 6;
constexpr uint32_t kLow = 100000u, kHigh = 1000000u;  // 10^(P-1), 10^P

// Digits D (kLow <= D < kHigh) and exponent X with |x| = D 10^(X-P+1) rounded half-even on
// the exact value, decided on integers where FP64 cannot decide.  ax finite, positive.
GD_HD bool round_sig_exact(double ax, int& X, uint32_t& D) {
    uint64_t m;
    int e;
    decompose(ax, m, e);
    Big one;
    big_set(one, 1);
    // X = floor(log10 ax): from log10 unless ax is within rounding of a power of ten
    const double lg = log10(ax);
    int X0 = (int)floor(lg);
    const double fr = lg - (double)X0;
    if (fr < 1e-9 || fr > 1.0 - 1e-9) {
        for (int it = 0; it < 4; ++it) {  // exact: 10^X0 <= ax < 10^(X0+1)
            const int lo = cmp_bin_dec(m, e, one, X0);
            if (lo == kFail) return false;
            if (lo < 0) {
                --X0;
                continue;
            }
            const int hi = cmp_bin_dec(m, e, one, X0 + 1);
            if (hi == kFail) return false;
            if (hi >= 0) {
                ++X0;
                continue;
            }
            break;
        }
    }
    X = X0;
    const int s = X - kPrec + 1;
    uint32_t c;
    // fast path: t = ax / 10^s with one correctly rounded operation
    if (s >= -22 && s <= 22) {
        const double t = s >= 0 ? ax / pow10_exact(s) : ax * pow10_exact(-s);
        const double fl = floor(t);
        const double f = t - fl;  // exact: t < 2^21
        c = (uint32_t)fl;
        // t is within half an ulp (< 6e-11 for t < 10^6) of ax / 10^s: outside this margin
        // around 1/2 the rounding decision is the exact one
        if (f < 0.5 - 1e-9) {
            D = c;
        } else if (f > 0.5 + 1e-9) {
            D = c + 1;
        } else {
            c = c == 0 ? 1 : c;
            goto exact;
        }
        goto done;
    }
    {
        const double t = scale10(ax, -s);
        c = t < 1.0 ? 1u : (t > 2.0e6 ? 2000000u : (uint32_t)(t + 0.5));
    }
exact:
    // exact: the c with (2c-1) 10^s <= 2 ax <= (2c+1) 10^s, ties to even
    for (int it = 0; it < 96; ++it) {
        Big b;
        big_set(b, 2ull * c + 1ull);
        const int up = cmp_bin_dec(m, e + 1, b, s);  // 2 ax vs (2c+1) 10^s
        if (up == kFail) return false;
        if (up > 0) {
            ++c;
            continue;
        }
        big_set(b, 2ull * c - 1ull);
        const int dn = cmp_bin_dec(m, e + 1, b, s);  // 2 ax vs (2c-1) 10^s
        if (dn == kFail) return false;
        if (dn < 0) {
            --c;
            continue;
        }
        if (up == 0 && (c & 1u)) ++c;
        else if (dn == 0 && (c & 1u)) --c;
        break;
    }
    D = c;
done:
    if (D >= kHigh) {  // rounded up to 10^P
        D = kLow;
        ++X;
    }
    return true;
}

// ---- the fast path ---------------------------------------------------------------------

#ifdef __CUDACC__
__device__ const double d_pow10[] = {GD_POW10_TABLE};
#endif
static const double h_pow10[] = {GD_POW10_TABLE};

// binary64 nearest to 10^k, GD_POW10_LO <= k <= GD_POW10_HI
GD_HD double pow10_near(int k) {
#ifdef __CUDA_ARCH__
    return d_pow10[k - GD_POW10_LO];
#else
    return h_pow10[k - GD_POW10_LO];
#endif
}

GD_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

// floor(e log10 2) for |e| <= 1650: (e 78913) >> 18, the approximation published with the
// Ryu conversion (Adams 2018) for e >= 0, mirrored for e < 0
GD_HD int floor_log10_pow2(int e) {
    return e >= 0 ? (int)(((uint32_t)e * 78913u) >> 18) : -(int)(((uint32_t)(-e) * 78913u) >> 18) - 1;
}

// round_sig with four FP64 operations on the common path: the decimal exponent from the
// binary one and one integer comparison with the nearest double to a power of ten, the
// scaled value t = ax 10^-s from one (rarely two) multiplications by table values, and
// its nearest integer and remainder by the 2^52 addition.  t carries at most three
// roundings, i.e. it is within 4e-10 of the exact ax / 10^s (t < 10^6); outside that
// margin around a half-integer the nearest integer of t is the exact rounding.  The
// remaining cases (a half-integer within the margin, ax within one ulp of a power of ten
// whose double is inexact) go to round_sig_exact.
GD_HD bool round_sig(double ax, int& X, uint32_t& D) {
    const uint64_t b = dbits(ax);
    const int be = (int)(b >> 52);
    const int e2 = be ? be - 1023 : -1011 - clz64(b);  // floor(log2 ax); subnormal: top bit
    const int X0 = floor_log10_pow2(e2);                // X is X0 or X0 + 1
    const int k = X0 + 1;
    const uint64_t tb = dbits(pow10_near(k));
    if (k >= 0 && k <= 22) {  // exact power of ten
        X = b >= tb ? k : X0;
    } else {
        if (b + 1 >= tb && b <= tb + 1) return round_sig_exact(ax, X, D);
        X = b > tb ? k : X0;
    }
    const int ms = kPrec - 1 - X;  // -s
    const double t = ms > 300 ? (ax * 1e30) * pow10_near(ms - 30) : ax * pow10_near(ms);
    const double y = t + 4503599627370496.0;  // 2^52: y - 2^52 is t rounded to an integer
    const uint32_t r = (uint32_t)(dbits(y) - 0x4330000000000000ULL);
    const double f = t - (y - 4503599627370496.0);
    if ((dbits(f) & 0x7fffffffffffffffULL) >= 0x3FDFFFFFFEED1F41ULL /* 0.5 - 1e-9 */ ||
        r < kLow || r > kHigh)
        return round_sig_exact(ax, X, D);
    D = r;
    if (D == kHigh) {  // rounded up to 10^P
        D = kLow;
        ++X;
    }
    return true;
}

GD_HD int put_uint(char* out, uint64_t v) {
    char tmp[20];
    int n = 0;
    do {
        tmp[n++] = (char)('0' + (int)(v % 10u));
        v /= 10u;
    } while (v);
    for (int i = 0; i < n; ++i) out[i] = tmp[n - 1 - i];
    return n;
}

GD_HD int put_int(char* out, long long v) {
    if (v < 0) {
        out[0] = '-';
        return 1 + put_uint(out + 1, (uint64_t)(-(v + 1)) + 1u);
    }
    return put_uint(out, (uint64_t)v);
}

// printf("%.6g", x); returns the length (at most 13: "-1.23456e-308")
GD_HD int format_g6(double x, char* out) {
    int n = 0;
    const uint64_t b = dbits(x);
    const uint64_t ab = b & 0x7fffffffffffffffULL;
    if (b >> 63) out[n++] = '-';
    if (ab >= 0x7ff0000000000000ULL) {  // as glibc prints them
        const char* w = ab == 0x7ff0000000000000ULL ? "inf" : "nan";
        for (int i = 0; i < 3; ++i) out[n++] = w[i];
        return n;
    }
    if (ab == 0) {
        out[n++] = '0';
        return n;
    }
    int X;
    uint32_t D;
    if (!round_sig(from_dbits(ab), X, D)) {
        out[n++] = '?';
        return n;
    }
    char dg[kPrec];
    for (int i = kPrec - 1; i >= 0; --i) {
        dg[i] = (char)('0' + (int)(D % 10u));
        D /= 10u;
    }
    int last = kPrec - 1;  // last non-zero digit
    while (last > 0 && dg[last] == '0') --last;
    if (X >= -4 && X < kPrec) {  // %f style with P-1-X fraction digits, zeros stripped
        if (X >= 0) {
            for (int i = 0; i <= X; ++i) out[n++] = dg[i];
            if (last > X) {
                out[n++] = '.';
                for (int i = X + 1; i <= last; ++i) out[n++] = dg[i];
            }
        } else {
            out[n++] = '0';
            out[n++] = '.';
            for (int i = 0; i < -X - 1; ++i) out[n++] = '0';
            for (int i = 0; i <= last; ++i) out[n++] = dg[i];
        }
    } else {  // %e style, exponent with at least two digits
        out[n++] = dg[0];
        if (last > 0) {
            out[n++] = '.';
            for (int i = 1; i <= last; ++i) out[n++] = dg[i];
        }
        out[n++] = 'e';
        int ex = X;
        out[n++] = ex < 0 ? '-' : '+';
        if (ex < 0) ex = -ex;
        if (ex < 10) out[n++] = '0';
        n += put_uint(out + n, (uint64_t)ex);
    }
    return n;
}

// ---- decimal text -> double (correctly rounded, ties to even) ----------------------------
// Accepts [+-]digits[.[digits]][(e|E)[+-]digits] and [+-].digits[...], `len` bytes at p.
// Returns false for anything else, for more than kMaxDigits significant digits and for
// values beyond the largest double (the stream extraction fails there too).

constexpr int kMaxDigits = 400;

GD_HD bool parse_double(const char* p, int len, double& out) {
    int i = 0;
    bool neg = false;
    if (i < len && (p[i] == '+' || p[i] == '-')) {
        neg = p[i] == '-';
        ++i;
    }
    int ndig = 0, nfrac = 0, nsig = 0, first_sig = -1;
    bool dot = false;
    uint64_t w = 0;  // the first min(nsig, 19) significant digits
    for (; i < len; ++i) {
        const char ch = p[i];
        if (ch == '.') {
            if (dot) return false;
            dot = true;
            continue;
        }
        if (ch < '0' || ch > '9') break;
        ++ndig;
        if (dot) ++nfrac;
        if (nsig == 0 && ch == '0') continue;
        if (nsig == 0) first_sig = i;
        if (nsig < 19) w = w * 10u + (uint64_t)(ch - '0');
        ++nsig;
    }
    const int mant_end = i;
    if (ndig == 0) return false;
    int ev = 0;
    if (i < len && (p[i] == 'e' || p[i] == 'E')) {
        ++i;
        bool eneg = false;
        if (i < len && (p[i] == '+' || p[i] == '-')) {
            eneg = p[i] == '-';
            ++i;
        }
        if (i >= len || p[i] < '0' || p[i] > '9') return false;
        for (; i < len && p[i] >= '0' && p[i] <= '9'; ++i)
            if (ev < 100000) ev = ev * 10 + (p[i] - '0');
        if (eneg) ev = -ev;
    }
    if (i != len) return false;
    if (nsig == 0) {
        out = neg ? -0.0 : 0.0;
        return true;
    }
    if (nsig > kMaxDigits) return false;
    // value = int(mantissa digits) * 10^vexp ~ w * 10^dexp, and value < 10^mag
    const int vexp = ev - nfrac;
    const int dexp = vexp + (nsig > 19 ? nsig - 19 : 0);
    const int mag = vexp + nsig;
    if (mag < -343) {  // below half the smallest subnormal: zero
        out = neg ? -0.0 : 0.0;
        return true;
    }
    if (mag > 310) return false;
    // fast path (Clinger): exact operands, one correctly rounded operation
    if (nsig <= 19 && w <= (1ULL << 53) && dexp >= -22 && dexp <= 22) {
        double z = (double)w;
        z = dexp >= 0 ? z * pow10_exact(dexp) : z / pow10_exact(-dexp);
        out = neg ? -z : z;
        return true;
    }
    // all significant digits as an integer V, value = V 10^vexp
    Big V;
    big_set(V, 0);
    for (int j = first_sig; j < mant_end; ++j) {
        if (p[j] == '.') continue;
        if (!big_muladd(V, 10u, (uint32_t)(p[j] - '0'))) return false;
    }
    // estimate, then step to the correctly rounded double by exact midpoint comparisons
    double z = scale10((double)w, dexp);
    if (!(z > 0.0)) z = from_dbits(1);
    if (z > 1.7976931348623157e308) z = 1.7976931348623157e308;
    for (int it = 0; it < 1200; ++it) {
        uint64_t m;
        int e;
        decompose(z, m, e);
        // sign(V 10^vexp - upper midpoint (2m+1) 2^(e-1))
        int r = cmp_bin_dec(2 * m + 1, e - 1, V, vexp);
        if (r == kFail) return false;
        const int cu = -r;
        // lower midpoint: (2m-1) 2^(e-1); a normal power of two has a predecessor half as
        // far: (4m-1) 2^(e-2)
        const bool pow2 = m == (1ULL << 52) && e > -1074;
        r = pow2 ? cmp_bin_dec(4 * m - 1, e - 2, V, vexp) : cmp_bin_dec(2 * m - 1, e - 1, V, vexp);
        if (r == kFail) return false;
        const int cl = -r;
        if (cu > 0 || (cu == 0 && (m & 1u))) {
            const double nz = from_dbits(dbits(z) + 1);
            if (!(nz <= 1.7976931348623157e308)) return false;  // overflow
            z = nz;
            continue;
        }
        if (cl < 0 || (cl == 0 && (m & 1u))) {
            if (dbits(z) == 1) {  // below the smallest subnormal's lower midpoint
                z = 0.0;
                break;
            }
            z = from_dbits(dbits(z) - 1);
            continue;
        }
        break;
    }
    out = neg ? -z : z;
    return true;
}

}  // namespace text
}  // namespace gd
