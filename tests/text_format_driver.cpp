// text_format_driver.cpp -- compares emida_cli::put_f / put_u with printf's
// "%f" / "%llu" over random and edge-case values; prints mismatches and a count.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <string>
#include <vector>

#include "../emida_gb300/cli/text.hpp"

int main()
{
    std::vector<double> v = {0.0, -0.0, 1e-300, -1e-300, 4.9e-324, -4.9e-324, DBL_MAX, -DBL_MAX,
                             0.5e-6, -0.5e-6, 0.0078125, -0.0078125, 1.0 / 128, 2.5e-6, 1e15, 123456.789,
                             std::numeric_limits<double>::quiet_NaN(), -std::numeric_limits<double>::quiet_NaN(),
                             std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity()};
    // exact ties at the 7th decimal: odd multiples of 2^-7 scaled by powers of two
    for (int k = 1; k < 4000; k += 2) v.push_back(k / 128.0), v.push_back(-k / 1024.0);
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> mant(1.0, 2.0);
    std::uniform_int_distribution<int> ex(-60, 60);
    for (int i = 0; i < 2000000; ++i) {
        double x = std::ldexp(mant(rng), ex(rng));
        if (rng() & 1) x = -x;
        v.push_back(x);
    }
    for (int i = 0; i < 200000; ++i) {  // offsets-like values: a few pixels, with 7+ decimals
        double x = (double)(int64_t)(rng() % 20000000) / 1e6 - 10.0;
        v.push_back(x);
        v.push_back(std::nextafter(x, 1e9));
    }
    size_t bad = 0;
    char buf[512];
    std::string s;
    for (double x : v) {
        s.clear();
        emida_cli::put_f(s, x);
        snprintf(buf, sizeof buf, "%f", x);
        if (s != buf) {
            if (bad < 10) printf("mismatch %.17g: put_f '%s' printf '%s'\n", x, s.c_str(), buf);
            ++bad;
        }
    }
    const unsigned long long us[] = {0ull, 1ull, 9ull, 10ull, 4294967295ull, 18446744073709551615ull};
    for (unsigned long long u : us) {
        s.clear();
        emida_cli::put_u(s, u);
        snprintf(buf, sizeof buf, "%llu", u);
        if (s != buf) {
            printf("mismatch %llu\n", u);
            ++bad;
        }
    }
    printf("checked %zu values, %zu mismatches\n", v.size() + 6, bad);
    return bad != 0;
}
