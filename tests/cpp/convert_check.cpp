// Checks sf::f64_to_f32 / sf::f32_to_f64 (csrc/sf_convert.cuh) against the compiler's casts, bit for bit, on
// edge cases and on seeded random inputs.  Prints the number of mismatches and the number of values checked.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "sf_convert.cuh"

static uint32_t fbits(float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    return u;
}
static uint64_t dbits(double v) {
    uint64_t u;
    std::memcpy(&u, &v, 8);
    return u;
}
static double dfrom(uint64_t u) {
    double v;
    std::memcpy(&v, &u, 8);
    return v;
}
static float ffrom(uint32_t u) {
    float v;
    std::memcpy(&v, &u, 4);
    return v;
}

int main() {
    long long bad = 0, n = 0;
    auto check_d = [&](double v) {
        n++;
        const float a = sf::f64_to_f32(v), b = (float)v;
        if (std::isnan(b) ? !std::isnan(a) : fbits(a) != fbits(b)) {
            if (bad < 10) std::printf("f64_to_f32 %a: %a vs %a\n", v, (double)a, (double)b);
            bad++;
        }
    };
    auto check_f = [&](float v) {
        n++;
        const double a = sf::f32_to_f64(v), b = (double)v;
        if (std::isnan(b) ? !std::isnan(a) : dbits(a) != dbits(b)) {
            if (bad < 10) std::printf("f32_to_f64 %a: %a vs %a\n", (double)v, a, b);
            bad++;
        }
    };
    const double edge[] = {0.0, -0.0, 1.0, -1.0, 6.0, 1.0 / 6.0, 2.3, 0.1, 1e-3, 1e-300, -1e-300, 1e300,
                           std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                           std::numeric_limits<double>::quiet_NaN(), (double)std::numeric_limits<float>::max(),
                           (double)std::numeric_limits<float>::min(), (double)std::numeric_limits<float>::denorm_min(),
                           std::numeric_limits<double>::denorm_min(), std::numeric_limits<double>::max()};
    for (double v : edge) {
        check_d(v);
        check_d(std::nextafter(v, 0.0));
        check_d(std::nextafter(v, 1e308));
    }
    // halfway cases and their neighbours around every float binade: float f, f + half ulp, f + half ulp +- 1 ulp(d)
    for (int e = -150; e <= 128; e++)
        for (uint32_t m : {0u, 1u, 2u, 3u, 0x3fffffu, 0x400000u, 0x7ffffeu, 0x7fffffu}) {
            const double base = std::ldexp(1.0 + m / 8388608.0, e);
            const double half = std::ldexp(1.0, e - 24);
            for (double v : {base, base + half, -(base + half), base + 3 * half, base - half / 2}) {
                check_d(v);
                check_d(std::nextafter(v, 0.0));
                check_d(std::nextafter(v, 1e308));
            }
        }
    std::mt19937_64 rng(12345);
    for (int t = 0; t < 4000000; t++) check_d(dfrom(rng()));  // every exponent, NaN payloads included
    std::uniform_real_distribution<double> u(-8.0, 8.0);
    for (int t = 0; t < 4000000; t++) check_d(std::ldexp(u(rng), (int)(rng() % 300) - 150));
    const float fedge[] = {0.f, -0.f, 1.f, -1.f, std::numeric_limits<float>::infinity(),
                           std::numeric_limits<float>::quiet_NaN(), std::numeric_limits<float>::min(),
                           std::numeric_limits<float>::denorm_min(), std::numeric_limits<float>::max()};
    for (float v : fedge) check_f(v);
    for (int t = 0; t < 4000000; t++) check_f(ffrom((uint32_t)rng()));
    std::printf("%lld %lld\n", bad, n);
    return bad != 0;
}
