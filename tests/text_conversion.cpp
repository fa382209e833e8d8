// Checks golikov_2d_gb300/csrc/gd_text.cuh -- the exact "%.6g" formatter and the correctly
// rounded parser the state I/O kernels run -- against the C library (snprintf "%.6g",
// strtod) on random and boundary values.  Compiled and run by tests/test_text_conversion.py;
// prints the mismatches and exits non-zero if there are any.
//     text_conversion <values per family>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "../golikov_2d_gb300/csrc/gd_text.cuh"

using namespace gd::text;

static long fails = 0, total = 0;

static void check_fmt(double v) {
    char ref[64], got[64];
    std::snprintf(ref, sizeof ref, "%.6g", v);
    const int n = format_g6(v, got);
    got[n] = 0;
    ++total;
    if (std::strcmp(ref, got)) {
        if (fails < 20) std::printf("format %a: libc '%s' ours '%s'\n", v, ref, got);
        ++fails;
    }
}

static void check_parse(const char* s) {
    const double ref = std::strtod(s, nullptr);
    if (std::isinf(ref)) return;  // overflow: the stream extraction fails, so does ours
    double got = 0.0;
    ++total;
    const bool ok = parse_double(s, (int)std::strlen(s), got);
    if (!ok || std::memcmp(&ref, &got, sizeof ref)) {
        if (fails < 40) std::printf("parse '%s': libc %a ours %a (ok %d)\n", s, ref, got, ok);
        ++fails;
    }
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 200000;
    std::mt19937_64 rng(20261203);
    std::uniform_real_distribution<double> U(-10.0, 10.0);
    for (long i = 0; i < n; ++i) {  // random bit patterns
        const double v = from_dbits(rng());
        if (std::isfinite(v)) check_fmt(v);
    }
    for (long i = 0; i < n; ++i) check_fmt(std::pow(10.0, U(rng)) * ((rng() & 1) ? 1.0 : -1.0));
    for (long k = 1000005; k < 1300000; k += 10) check_fmt((double)k);  // ties at the 7th digit
    for (int j = 1; j < 60; ++j)
        for (int k = 1; k < 400; ++k) check_fmt(std::ldexp((double)k, -j));
    for (int k = -323; k <= 308; ++k) {  // powers of ten and neighbours
        const double p = std::pow(10.0, k);
        for (int d = -3; d <= 3; ++d) check_fmt(from_dbits(dbits(p) + d));
        check_fmt(p * 0.9999995);
        check_fmt(p * 9.999995);
    }
    for (int i = 1; i < 2000; ++i) check_fmt(from_dbits((uint64_t)i));  // subnormals
    const double edges[] = {0.0, -0.0, 1e-5, 1e-4, 123456.0, 999999.5, 99999.95, 0.000099999951,
                            1.7976931348623157e308, 2.2250738585072014e-308, 0.5, 1e21, 1e22,
                            1e23, 100000.5, -123456.5};
    for (double e : edges) check_fmt(e);
    const long fmt_fails = fails, fmt_total = total;
    char buf[160];
    for (long i = 0; i < n; ++i) {
        const double v = from_dbits(rng());
        if (!std::isfinite(v)) continue;
        std::snprintf(buf, sizeof buf, "%.17g", v);
        check_parse(buf);
        std::snprintf(buf, sizeof buf, "%.6g", v);
        check_parse(buf);
        std::snprintf(buf, sizeof buf, "%.*e", (int)(rng() % 25), v);
        check_parse(buf);
    }
    for (long i = 0; i < n; ++i) {
        const double v = std::pow(10.0, U(rng) * 3);
        std::snprintf(buf, sizeof buf, "%.12f", v);
        check_parse(buf);
    }
    const char* hard[] = {"9007199254740993", "9007199254740992.5", "2.2250738585072011e-308",
                          "2.2250738585072012e-308", "4.9406564584124654e-324",
                          "2.4703282292062327e-324", "2.4703282292062328e-324",
                          "1.7976931348623157e308", "0.1", "1e23", "8.98846567431158e307",
                          "1.00000000000000011102230246251565404236316680908203125",
                          "1.00000000000000011102230246251565404236316680908203124",
                          "1.00000000000000011102230246251565404236316680908203126",
                          "123456789012345678901234567890", "7.2057594037927933e16", "-0",
                          "+1.5", ".5", "5.", "1e-400", "00012.500e+002"};
    for (const char* h : hard) check_parse(h);
    for (long i = 0; i < n / 4; ++i) {  // long digit strings
        int len = 0;
        const int nd = 1 + (int)(rng() % 40);
        buf[len++] = (char)('1' + rng() % 9);
        for (int k = 1; k < nd; ++k) {
            buf[len++] = (char)('0' + rng() % 10);
            if (k == 1 && (rng() & 1)) buf[len++] = '.';
        }
        len += std::snprintf(buf + len, 20, "e%d", (int)(rng() % 700) - 350);
        buf[len] = 0;
        check_parse(buf);
    }
    std::printf("format: %ld values, %ld mismatches; parse: %ld strings, %ld mismatches\n",
                fmt_total, fmt_fails, total - fmt_total, fails - fmt_fails);
    return fails != 0;
}
