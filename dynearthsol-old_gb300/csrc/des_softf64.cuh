// Exactly rounded FP64 multiply and FP64 -> FP32 conversion on the integer
// pipes.
//
// GB300 retires 2 FP64 instructions per clock per SM, while its integer ALU
// and FMA pipes retire 64 and more lanes per clock.  A kernel bound by the
// FP64 pipe can move part of its multiplies and conversions to these
// routines and run both pipes at once.  Each returns, bit for bit, what the
// FP64 unit returns (IEEE-754 binary64, round to nearest even, subnormals
// kept): the fast path covers normal operands with a normal result, and the
// rest (zeros, subnormals, infinities, NaN, overflow, underflow) takes an
// integer slow path.  Neither path issues an FP64 instruction: the compiler
// predicates short branches, and a predicated FP64 instruction still
// occupies the FP64 pipe.  64-bit leading-zero counts are formed from two
// 32-bit counts for the same reason (the 64-bit count is lowered through a
// conversion on the FP64 unit).
//
// The header compiles as plain C++ too, so that the host can check it
// against its own IEEE arithmetic.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DES_SF_HD __host__ __device__ __forceinline__
#else
#define DES_SF_HD static inline
#endif

namespace des {
namespace sf {

constexpr uint64_t kAbs = 0x7fffffffffffffffull;
constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kFrac = 0x000fffffffffffffull;
constexpr uint64_t kHidden = 0x0010000000000000ull;
constexpr uint64_t kInf = 0x7ff0000000000000ull;
constexpr uint64_t kQuiet = 0x0008000000000000ull;
constexpr uint64_t kDefaultNaN = 0x7ff8000000000000ull;

DES_SF_HD uint64_t bits(double x)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

DES_SF_HD double from_bits(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

DES_SF_HD float float_from_bits(uint32_t b)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    memcpy(&x, &b, 4);
    return x;
#endif
}

DES_SF_HD int clz32(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return __clz((int)x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}

// leading zeros of a 64-bit word from two 32-bit counts
DES_SF_HD int clz64(uint64_t x)
{
    const uint32_t hi = (uint32_t)(x >> 32);
    return hi ? clz32(hi) : 32 + clz32((uint32_t)x);
}

DES_SF_HD uint64_t mulhi64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// round to nearest even on the 11 bits below a 53-bit significand held at
// the top of r (bit 63 down to 11), then pack with the biased exponent e
// (1 <= e; a carry out of the significand moves into the exponent, and
// e = 2046 with a carry gives the infinity the rounding asks for)
DES_SF_HD uint64_t round_pack(uint64_t sign, int e, uint64_t r)
{
    const uint64_t m = r >> 11, rem = r & 0x7ff;
    const uint64_t up = (uint64_t)((rem > 0x400) | ((rem == 0x400) & (uint32_t)m));
    return ((((uint64_t)(e - 1)) << 52) + m + up) | sign;
}

// the cases the fast path of mul leaves: zeros, subnormals, infinities, NaN,
// results outside the normal range
#if defined(__CUDACC__)
static __host__ __device__ __noinline__
#else
static
#endif
uint64_t mul_slow(uint64_t a, uint64_t b)
{
    const uint64_t sign = (a ^ b) & kSign;
    const uint64_t ma = a & kAbs, mb = b & kAbs;
    const int ea = (int)(ma >> 52), eb = (int)(mb >> 52);
    if (ea == 2047 || eb == 2047) {
        if (ma > kInf) return a | kQuiet;
        if (mb > kInf) return b | kQuiet;
        if (ma == 0 || mb == 0) return kDefaultNaN;
        return sign | kInf;
    }
    if (ma == 0 || mb == 0) return sign;
    uint64_t fa = (ma & kFrac) | (ea ? kHidden : 0), fb = (mb & kFrac) | (eb ? kHidden : 0);
    const int la = clz64(fa), lb = clz64(fb);
    fa <<= la;
    fb <<= lb;
    const uint64_t hi = mulhi64(fa, fb), lo = fa * fb;
    const int lz = (int)(1 - (hi >> 63));
    uint64_t r = (hi << lz) | (uint64_t)(lo != 0);
    int e = (ea ? ea : 1) + (eb ? eb : 1) - 1000 - la - lb - lz;
    if (e >= 2047) return sign | kInf;
    if (e < 1) {
        const uint32_t sh = (uint32_t)(1 - e) > 63u ? 63u : (uint32_t)(1 - e);
        uint64_t rs = r >> sh;
        rs |= (uint64_t)((rs << sh) != r);
        r = rs;
        e = 1;
    }
    return round_pack(sign, e, r);
}

// 32x32 -> 64 products with a 64-bit addend; on the device as PTX
// mul.wide.u32 / mad.wide.u32 instructions, which the compiler's IR passes
// keep as they are
DES_SF_HD uint64_t wide_mul(uint32_t x, uint32_t y)
{
#if defined(__CUDA_ARCH__)
    uint64_t r;
    asm("mul.wide.u32 %0, %1, %2;" : "=l"(r) : "r"(x), "r"(y));
    return r;
#else
    return (uint64_t)x * y;
#endif
}

DES_SF_HD uint64_t wide_mad(uint32_t x, uint32_t y, uint64_t c)
{
#if defined(__CUDA_ARCH__)
    uint64_t r;
    asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"(x), "r"(y), "l"(c));
    return r;
#else
    return (uint64_t)x * y + c;
#endif
}

// x * y as the FP64 unit rounds it.  Fast path (normal operands, normal
// result) in 32-bit pieces: with the significands A = a1 2^32 + a0 and
// B = b1 2^32 + b0 (a1, b1 of 21 bits), four 32x32 -> 64 products give the
// 106-bit P = A B as p11 2^64 + mid 2^32 + low.  The significand of the
// result is P >> (52 + t), t = 1 when P >= 2^105; the bits below it decide
// the rounding (round bit, then a sticky OR of the rest).
DES_SF_HD double mul(double x, double y)
{
    const uint64_t a = bits(x), b = bits(y);
    const uint32_t ah = (uint32_t)(a >> 32), bh = (uint32_t)(b >> 32);
    const uint32_t ea = (ah >> 20) & 0x7ff, eb = (bh >> 20) & 0x7ff;
    if (ea - 1 < 2046u && eb - 1 < 2046u) {
        const uint32_t a0 = (uint32_t)a, b0 = (uint32_t)b;
        const uint32_t a1 = (ah & 0xfffffu) | 0x100000u, b1 = (bh & 0xfffffu) | 0x100000u;
        const uint64_t p00 = wide_mul(a0, b0);
        const uint64_t p01 = wide_mad(a0, b1, p00 >> 32);
        const uint64_t p10 = wide_mad(a1, b0, p01);
        const uint64_t p11 = wide_mad(a1, b1, p10 >> 32);
        const uint32_t mid = (uint32_t)p10, low = (uint32_t)p00;
        const uint32_t t = (uint32_t)(p11 >> 41);
        const int e = (int)(ea + eb) - 1023 + (int)t;
        if ((uint32_t)(e - 1) < 2046u) {
            const uint32_t sh = 12 - t;
            const uint64_t m = (p11 << sh) | (mid >> (32 - sh));
            const uint32_t rem = mid << sh;
            const uint32_t up = (rem >> 31) & (uint32_t)((((rem << 1) | low) != 0) | ((uint32_t)m & 1));
            return from_bits(((((uint64_t)(e - 1)) << 52) + m + up) | ((a ^ b) & kSign));
        }
    }
    // a zero times a finite number (frequent: zero velocity components and
    // shape-function derivatives) without the call
    if (((a & kAbs) == 0 && eb != 2047) || ((b & kAbs) == 0 && ea != 2047)) return from_bits((a ^ b) & kSign);
    return from_bits(mul_slow(a, b));
}

// 0.0 + x as the FP64 unit rounds it: x itself, except that -0.0 gives
// +0.0 (a NaN comes back unchanged).  The first addition of a sum that
// starts from zero.
DES_SF_HD double add0(double x)
{
    const uint64_t b = bits(x);
    return from_bits(b == kSign ? 0ull : b);
}

// 2 x and x / 2 (x * 2.0, x * 0.5) as the FP64 unit rounds them: an exponent
// step where the operand and the result are normal, the integer multiply
// otherwise (zeros, subnormals, infinities, NaN, overflow, a subnormal half)
DES_SF_HD double twice(double x)
{
    const uint64_t b = bits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ff;
    if (e - 1 < 2045u) return from_bits(b + (1ull << 52));
    return mul(x, 2.0);
}

DES_SF_HD double half(double x)
{
    const uint64_t b = bits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ff;
    if (e - 2 < 2045u) return from_bits(b - (1ull << 52));
    return mul(x, 0.5);
}

// x / 4 (x * 0.25) as the FP64 unit rounds it
DES_SF_HD double quarter(double x)
{
    const uint64_t b = bits(x);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ff;
    if (e - 3 < 2044u) return from_bits(b - (2ull << 52));
    return mul(x, 0.25);
}

// x / (3 2^k), k = 0 or 1, for the cases the fast path of div3k leaves:
// zeros, subnormals, operands whose quotient is subnormal, infinities, NaN
#if defined(__CUDACC__)
static __host__ __device__ __noinline__
#else
static
#endif
uint64_t div3k_slow(uint64_t a, int k)
{
    const uint64_t sign = a & kSign, ma = a & kAbs;
    int ea = (int)(ma >> 52);
    if (ea == 2047) return ma > kInf ? (a | kQuiet) : a;
    if (ma == 0) return sign;
    uint64_t m = (ma & kFrac) | (ea ? kHidden : 0);
    if (!ea) {                           // normalise a subnormal significand to bit 52
        const int s = clz64(m) - 11;
        m <<= s;
        ea = 1 - s;
    }
    const uint64_t M = m << 11, q = M / 3, r = M - 3 * q;
    const int t = (int)(q >> 62);        // the quotient's top bit is bit 61 + t
    const uint64_t rr = (q << (2 - t)) | (uint64_t)(r != 0);
    int e = ea - 2 - k + t;
    if (e < 1) {
        const uint32_t sh = (uint32_t)(1 - e) > 63u ? 63u : (uint32_t)(1 - e);
        uint64_t rs = rr >> sh;
        rs |= (uint64_t)((rs << sh) != rr);
        return round_pack(sign, 1, rs);
    }
    return round_pack(sign, e, rr);
}

// x / 3 (k = 0) and x / 6 (k = 1) as the FP64 unit's division rounds them.
// With the significand m (2^52 <= m < 2^53), the quotient of M = m 2^11 by 3
// (an integer division by a constant: a high multiply) holds 62 or 63 bits;
// its top 53 are the result's significand, and the bits below them with the
// remainder of the division (sticky) decide the rounding to nearest even.
template <int k>
DES_SF_HD double div3k(double x)
{
    const uint64_t a = bits(x);
    const uint32_t e = (uint32_t)(a >> 52) & 0x7ff;
    if (e - (3 + k) < 2044u - k) {       // the quotient is normal
        const uint64_t M = ((a & kFrac) | kHidden) << 11;
        const uint64_t q = M / 3, r = M - 3 * q;
        const uint32_t t = (uint32_t)(q >> 62);
        const uint32_t sh = 9 + t;
        const uint64_t sig = q >> sh, rem = q & ((1ull << sh) - 1), hf = 1ull << (sh - 1);
        const uint64_t up = (uint64_t)((rem > hf) | ((rem == hf) & ((r != 0) | (uint32_t)(sig & 1))));
        return from_bits(((((uint64_t)(e - 3 - k + t)) << 52) + sig + up) | (a & kSign));
    }
    return from_bits(div3k_slow(a, k));
}

DES_SF_HD double div3(double x) { return div3k<0>(x); }
DES_SF_HD double div6(double x) { return div3k<1>(x); }

// the cases the fast path of to_float leaves: zeros, subnormal FP32
// results, infinities, NaN, overflow
#if defined(__CUDACC__)
static __host__ __device__ __noinline__
#else
static
#endif
uint32_t to_float_slow(uint64_t a)
{
    const uint32_t sign = (uint32_t)(a >> 32) & 0x80000000u;
    const int e = (int)((a >> 52) & 0x7ff);
    if (e == 2047) return (a & kFrac) ? 0x7fffffffu : (sign | 0x7f800000u);
    if (e - 896 >= 255) return sign | 0x7f800000u;
    // FP32 subnormal or zero: k = round(significand / 2^(926 - e)) units of 2^-149
    const int sh = 926 - e;
    if (sh >= 54) return sign;
    const uint64_t f = (a & kFrac) | kHidden;
    const uint64_t k = f >> sh, rem = f & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    const uint64_t up = (uint64_t)((rem > half) | ((rem == half) & (uint32_t)k));
    return sign | (uint32_t)(k + up);
}

// (float)x, round to nearest even, as the FP64 unit converts it
DES_SF_HD float to_float(double x)
{
    const uint64_t a = bits(x);
    const uint32_t hi = (uint32_t)(a >> 32), lo = (uint32_t)a;
    const int ef = (int)((hi >> 20) & 0x7ff) - 896;
    if ((uint32_t)(ef - 1) < 254u) {
        const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);
        const uint32_t rem = lo & 0x1fffffffu;
        const uint32_t up = (uint32_t)((rem > 0x10000000u) | ((rem == 0x10000000u) & m));
        return float_from_bits((hi & 0x80000000u) | ((((uint32_t)ef) << 23) + m + up));
    }
    return float_from_bits(to_float_slow(a));
}

}  // namespace sf
}  // namespace des
