// Host check of the integer FP64 multiply, FP64 -> FP32 conversion, 0 + x,
// 2 x, x / 2, x / 6, x / 3 and x / 4 (dynearthsol-old_gb300/csrc/des_softf64.cuh)
// against the host's IEEE
// arithmetic, bit for bit, on seeded pseudo-random operands of several kinds.
//   softf64_check <pairs per kind>   -> one line per kind; exit 1 on a mismatch
#include "des_softf64.cuh"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <thread>
#include <vector>

using des::sf::bits;
using des::sf::from_bits;

static inline uint64_t splitmix(uint64_t &s)
{
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static double mk(uint64_t sign, uint64_t e, uint64_t f)
{
    return from_bits(((sign & 1) << 63) | ((e & 0x7ff) << 52) | (f & des::sf::kFrac));
}

// operand pairs: 0 any bits; 1 exponents near 1023; 2 short significands
// (exact products and ties); 3 exponent extremes; 4 products near the
// overflow and underflow thresholds; 5 subnormals; 6 zeros, infinities, NaN
static void pair(int kind, uint64_t &s, double &x, double &y)
{
    const uint64_t r1 = splitmix(s), r2 = splitmix(s), r3 = splitmix(s);
    switch (kind) {
    case 0:
        x = from_bits(r1);
        y = from_bits(r2);
        break;
    case 1:
        x = mk(r1 >> 63, 1023 - 60 + r3 % 121, r1);
        y = mk(r2 >> 63, 1023 - 60 + (r3 >> 12) % 121, r2);
        break;
    case 2:
        x = mk(r1 >> 63, 1000 + r3 % 40, r1 & ~((1ull << (26 + r3 % 26)) - 1));
        y = mk(r2 >> 63, 1000 + (r3 >> 8) % 40, r2 & ~((1ull << (26 + (r3 >> 16) % 26)) - 1));
        break;
    case 3:
        x = mk(r1 >> 63, (r3 & 1) ? r1 % 64 : 2047 - r1 % 64, splitmix(s));
        y = mk(r2 >> 63, (r3 & 2) ? r2 % 64 : 2047 - r2 % 64, splitmix(s));
        break;
    case 4: {
        const int64_t e1 = 1 + (int64_t)(r1 % 2046), target = (r3 & 1) ? 2046 : 1;
        int64_t e2 = target + 1022 - e1 + (int64_t)((r3 >> 8) % 7) - 3;
        e2 = e2 < 0 ? 0 : (e2 > 2047 ? 2047 : e2);
        x = mk(r1 >> 63, (uint64_t)e1, r2);
        y = mk(r2 >> 63, (uint64_t)e2, splitmix(s));
        break;
    }
    case 5:
        x = mk(r1 >> 63, r3 % 3, r1 >> (r3 % 50));
        y = mk(r2 >> 63, (r3 & 64) ? (r3 >> 8) % 3 : 900 + (r3 >> 8) % 250, r2 >> ((r3 >> 16) % 50));
        break;
    default: {
        const uint64_t sp[4] = {0, des::sf::kInf, des::sf::kDefaultNaN, 1};
        x = from_bits((r1 & des::sf::kSign) | ((r3 & 1) ? sp[(r3 >> 1) & 3] : (r1 & 0x3fffffffffffffffull)));
        y = from_bits((r2 & des::sf::kSign) | ((r3 & 8) ? sp[(r3 >> 4) & 3] : (r2 & 0x3fffffffffffffffull)));
        break;
    }
    }
}

// conversion operands: 0 any bits; 1 the FP32 normal range; 2 ties (the low
// 29 bits exactly half); 3 the FP32 subnormal range and below; 4 near
// FP32 overflow
static double single(int kind, uint64_t &s)
{
    const uint64_t r1 = splitmix(s), r3 = splitmix(s);
    switch (kind) {
    case 0: return from_bits(r1);
    case 1: return mk(r1 >> 63, 897 + r3 % 254, r1);
    case 2: return mk(r1 >> 63, 870 + r3 % 310, (r1 & ~0x1fffffffull) | ((r3 & 2) ? 0x10000000ull : 0x0fffffffull + (r3 & 4) / 2));
    case 3: return mk(r1 >> 63, 840 + r3 % 60, (r3 & 8) ? (r1 & ~((1ull << (r3 % 52)) - 1)) : r1);
    default: return mk(r1 >> 63, 1146 + r3 % 6, (r3 & 16) ? ~0ull : r1);
    }
}

// operands of the one-operand helpers: 0 any bits; 1 exponents near 1023; 2
// exponents 0-8 (subnormals, results near the subnormal range); 3 exponents
// 2038-2047 (overflow, infinities, NaN); 4 short significands (ties)
static double unary(int kind, uint64_t &s)
{
    const uint64_t r1 = splitmix(s), r3 = splitmix(s);
    switch (kind) {
    case 0: return from_bits(r1);
    case 1: return mk(r1 >> 63, 1013 + r3 % 21, r1);
    case 2: return mk(r1 >> 63, r3 % 9, (r3 & 32) ? r1 : (r1 >> (r3 % 52)));
    case 3: return mk(r1 >> 63, 2038 + r3 % 10, (r3 & 64) ? r1 : 0);
    default: return mk(r1 >> 63, 1 + r3 % 2046, r1 & ~((1ull << (30 + r3 % 22)) - 1));
    }
}

static bool same(double a, double b) { return bits(a) == bits(b) || (std::isnan(a) && std::isnan(b)); }

static bool same_f(float a, float b)
{
    uint32_t x, y;
    memcpy(&x, &a, 4);
    memcpy(&y, &b, 4);
    return x == y || (std::isnan(a) && std::isnan(b));
}

int main(int argc, char **argv)
{
    const long long per = argc > 1 ? atoll(argv[1]) : 10000000;
    unsigned nt = std::thread::hardware_concurrency();
    nt = nt ? (nt > 32 ? 32 : nt) : 4;
    long long total_bad = 0;
    for (int kind = 0; kind < 7; ++kind) {
        std::atomic<long long> bad{0};
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t)
            th.emplace_back([&, t] {
                uint64_t s = 0x5eed0000ull + 1000003ull * kind + 7919ull * t;
                for (long long i = t; i < per; i += nt) {
                    double x, y;
                    pair(kind, s, x, y);
                    volatile double h = x * y;
                    if (!same(h, des::sf::mul(x, y)) && bad++ < 3)
                        printf("mul %a * %a: host %a, integer %a\n", x, y, (double)h, des::sf::mul(x, y));
                }
            });
        for (auto &x : th) x.join();
        printf("mul kind %d: %lld pairs, %lld mismatches\n", kind, per, bad.load());
        total_bad += bad;
    }
    for (int kind = 0; kind < 5; ++kind) {
        std::atomic<long long> bad{0};
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t)
            th.emplace_back([&, t] {
                uint64_t s = 0xf10a7000ull + 1000003ull * kind + 7919ull * t;
                for (long long i = t; i < per; i += nt) {
                    const double x = single(kind, s);
                    volatile float h = (float)x;
                    if (!same_f(h, des::sf::to_float(x)) && bad++ < 3)
                        printf("to_float %a: host %a, integer %a\n", x, (double)h, (double)des::sf::to_float(x));
                }
            });
        for (auto &x : th) x.join();
        printf("to_float kind %d: %lld values, %lld mismatches\n", kind, per, bad.load());
        total_bad += bad;
    }
    const char *names[6] = {"add0", "twice", "half", "div6", "div3", "quarter"};
    for (int op = 0; op < 6; ++op)
        for (int kind = 0; kind < 5; ++kind) {
            std::atomic<long long> bad{0};
            std::vector<std::thread> th;
            for (unsigned t = 0; t < nt; ++t)
                th.emplace_back([&, t] {
                    uint64_t s = 0xadd06000ull + 1000003ull * (5 * op + kind) + 7919ull * t;
                    for (long long i = t; i < per; i += nt) {
                        const double x = unary(kind, s);
                        volatile double vx = x;
                        double h, g;
                        switch (op) {
                        case 0: h = 0.0 + vx; g = des::sf::add0(x); break;
                        case 1: h = vx * 2.0; g = des::sf::twice(x); break;
                        case 2: h = vx * 0.5; g = des::sf::half(x); break;
                        case 3: h = vx / 6.0; g = des::sf::div6(x); break;
                        case 4: h = vx / 3.0; g = des::sf::div3(x); break;
                        default: h = vx * 0.25; g = des::sf::quarter(x); break;
                        }
                        if (!same(h, g) && bad++ < 3) printf("%s %a: host %a, integer %a\n", names[op], x, h, g);
                    }
                });
            for (auto &x : th) x.join();
            printf("%s kind %d: %lld values, %lld mismatches\n", names[op], kind, per, bad.load());
            total_bad += bad;
        }
    return total_bad ? 1 : 0;
}
