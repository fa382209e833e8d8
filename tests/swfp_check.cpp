// Host check of gd::swfp (the integer-pipe binary64 multiplication, halving and doubling)
// against the host's IEEE-754 arithmetic.  Usage: swfp_check <cases per class> <seed>.  Prints one line per
// class; exits 1 if any result differs from a * b (two NaNs count as equal: the integer
// path returns the canonical quiet NaN) or if the fast path accepts a case and is wrong.
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cmath>

#include "../golikov_2d_gb300/csrc/gd_swfp.cuh"

using namespace gd::swfp;

static uint64_t s_state;
static uint64_t next64() {  // splitmix64
    uint64_t z = (s_state += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static double make(uint64_t sign, uint64_t exp, uint64_t frac) {
    return from_bits((sign << 63) | ((exp & 0x7ff) << 52) | (frac & 0xfffffffffffffULL));
}

int main(int argc, char** argv) {
    const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
    s_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
    const char* names[] = {"any bits", "typical", "range edges", "short significands",
                           "zeros", "all-ones significands", "subnormal", "inf and nan"};
    int failed = 0;
    for (int cls = 0; cls < 8; ++cls) {
        long long fast = 0, bad = 0;
        for (long long i = 0; i < n; ++i) {
            double a, b;
            const uint64_t r1 = next64(), r2 = next64(), r3 = next64();
            switch (cls) {
                case 0: a = from_bits(r1); b = from_bits(r2); break;
                case 1:
                    a = make(r3 & 1, 1023 - 40 + (r3 >> 8) % 81, r1);
                    b = make((r3 >> 1) & 1, 1023 - 40 + (r3 >> 24) % 81, r2);
                    break;
                case 2: {  // products near the overflow and underflow limits
                    const int ea = 1 + (int)((r3 >> 8) % 2046);
                    const int lo = (r3 & 2) ? 2044 + 1023 - ea : 1023 + 1 - ea;
                    int eb = lo - 60 + (int)((r3 >> 32) % 121);
                    if (eb < 0) eb = 0;
                    if (eb > 2047) eb = 2047;
                    a = make(r3 & 1, ea, r1);
                    b = make((r3 >> 4) & 1, eb, r2);
                    break;
                }
                case 3: {  // few significant bits: exact products and halfway cases
                    const int ka = 1 + (int)(r3 % 40), kb = 1 + (int)((r3 >> 8) % 40);
                    const uint64_t ma = r1 & ~((1ULL << (52 - ka)) - 1) & ((1ULL << 52) - 1);
                    const uint64_t mb = r2 & ~((1ULL << (52 - kb)) - 1) & ((1ULL << 52) - 1);
                    a = make(r3 >> 63, 1000 + (r3 >> 16) % 40, ma | (1ULL << (52 - ka)));
                    b = make((r3 >> 62) & 1, 1000 + (r3 >> 24) % 40, mb | (1ULL << (52 - kb)));
                    if (r3 & 0x100) {  // halfway results near the subnormal boundary too
                        a = make(r3 >> 63, 1 + (r3 >> 16) % 40, ma | (1ULL << (52 - ka)));
                        b = make((r3 >> 62) & 1, 980 + (r3 >> 24) % 40, mb | (1ULL << (52 - kb)));
                    }
                    break;
                }
                case 4:
                    a = make(r3 & 1, 0, 0);
                    b = (r3 & 2) ? from_bits(r2) : make(0, 900 + r2 % 200, r1);
                    if (r3 & 4) { const double t = a; a = b; b = t; }
                    break;
                case 5:
                    a = make(r3 & 1, 1023 + (r3 >> 8) % 30, 0xfffffffffffffULL - (r1 % 4));
                    b = make((r3 >> 1) & 1, 1023 - (r3 >> 16) % 30, 0xfffffffffffffULL - (r2 % 4));
                    break;
                case 6:  // a subnormal operand, the other of any size
                    a = make(r3 & 1, 0, r1 >> (r3 >> 58));
                    b = make((r3 >> 1) & 1, (r3 >> 8) % 2047, r2);
                    if (r3 & 4) { const double t = a; a = b; b = t; }
                    break;
                default: {  // infinities and NaNs against anything
                    const uint64_t fr = (r3 & 8) ? 0 : (r1 | 1);
                    a = make(r3 & 1, 0x7ff, fr);
                    b = (r3 & 2) ? make(0, 0, 0) : from_bits(r2);
                    if (r3 & 4) { const double t = a; a = b; b = t; }
                    break;
                }
            }
            bool ok;
            const double f = dmul_fast(a, b, ok);
            const double s = mul_rn(a, b);
            const double h = a * b;
            const bool same = to_bits(s) == to_bits(h) || (std::isnan(s) && std::isnan(h));
            const bool fast_ok = !ok || to_bits(f) == to_bits(h);
            fast += ok;
            if (!same || !fast_ok) {
                if (bad < 5)
                    printf("MISMATCH %s: %016llx * %016llx = %016llx, integer path %016llx (fast %d)\n",
                           names[cls], (unsigned long long)to_bits(a),
                           (unsigned long long)to_bits(b), (unsigned long long)to_bits(h),
                           (unsigned long long)to_bits(s), (int)ok);
                ++bad;
            }
        }
        printf("%-22s cases %lld fast path %lld mismatches %lld\n", names[cls], n, fast, bad);
        failed += bad != 0;
    }
    // x / 2 and 2 x (half_rn, twice_rn) against the host's x * 0.5 and x + x
    {
        const char* hn[] = {"half/twice any bits", "half/twice subnormal and edges"};
        for (int cls = 0; cls < 2; ++cls) {
            long long bad = 0;
            for (long long i = 0; i < n; ++i) {
                const uint64_t r1 = next64(), r3 = next64();
                double x;
                if (cls == 0) {
                    x = from_bits(r1);
                } else {
                    const uint64_t e = (r3 & 3) == 0 ? 0 : (r3 & 3) == 1 ? 1 : (r3 & 3) == 2 ? 2046 : 2045;
                    x = make((r3 >> 8) & 1, e, r1 >> ((r3 >> 16) % 53));
                }
                const double h = half_rn(x), t = twice_rn(x);
                const double H = x * 0.5, T = x + x;
                const bool okh = to_bits(h) == to_bits(H) || (std::isnan(h) && std::isnan(H));
                const bool okt = to_bits(t) == to_bits(T) || (std::isnan(t) && std::isnan(T));
                if (!okh || !okt) {
                    if (bad < 5)
                        printf("MISMATCH %s: x %016llx half %016llx (%016llx) twice %016llx (%016llx)\n",
                               hn[cls], (unsigned long long)to_bits(x), (unsigned long long)to_bits(h),
                               (unsigned long long)to_bits(H), (unsigned long long)to_bits(t),
                               (unsigned long long)to_bits(T));
                    ++bad;
                }
            }
            printf("%-22s cases %lld mismatches %lld\n", hn[cls], n, bad);
            failed += bad != 0;
        }
    }
    // grow_rel: w (1 + t 2^-52) against the exact value in extended precision, within one unit
    // of the result's last place; a quarter of the cases with w's mantissa near all ones, so
    // that the increment carries into the exponent field
    {
        long long bad = 0, carried = 0;
        for (long long i = 0; i < n; ++i) {
            const uint64_t r1 = next64(), r3 = next64();
            uint64_t frac = r1 & 0xfffffffffffffULL;
            if ((r3 & 3) == 0) frac = 0xfffffffffffffULL - (r1 % 4194304);
            const double w = make((r3 >> 2) & 1, 1000 + (r3 >> 8) % 60, frac);
            const float t = (float)((r3 >> 32) % 2097152) + (float)((r3 >> 16) & 0xffff) / 65536.0f;
            const double g = grow_rel(w, t);
            const long double ex = (long double)w * (1.0L + (long double)t / 4503599627370496.0L);
            const double er = (double)ex;
            const uint64_t gb = to_bits(g), eb = to_bits(er);
            const uint64_t d = gb > eb ? gb - eb : eb - gb;
            carried += ((gb >> 52) & 0x7ff) != ((to_bits(w) >> 52) & 0x7ff);
            if (d > 1) {
                if (bad < 5)
                    printf("MISMATCH grow_rel: w %016llx t %.9g -> %016llx, exact %016llx\n",
                           (unsigned long long)to_bits(w), t, (unsigned long long)gb,
                           (unsigned long long)eb);
                ++bad;
            }
        }
        printf("%-22s cases %lld mismatches %lld (binade carries %lld)\n", "grow_rel", n, bad,
               carried);
        failed += bad != 0;
    }
    return failed ? 1 : 0;
}
