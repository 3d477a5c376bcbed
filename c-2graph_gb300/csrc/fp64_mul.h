// Exact IEEE-754 binary64 product q * (double)w for a positive normal double q and a
// positive normal float w, rounded to nearest-even, computed with 32-bit integer
// multiplies only.
//
// Why: the FP64 residual push multiplies every frontier residual by every edge weight
// (q * w, src/ppr/purn/Main.cu:288).  GB300 issues FP64 instructions at a small
// fraction of its integer rate, so the float->double conversion, the double multiply
// and the double compare of each push kept the FP64 pipe busy (ncu
// sm__pipe_fp64_cycles_active) while memory sat idle.  The result here is bit-identical
// to the hardware multiply (checked against it on the host in tests), so parity with
// the FP64 push is unchanged.
//
// Method (IEEE-754 arithmetic, nothing library-specific): with significands
// Sq = 2^52 + mq (53 bits) and Sw = 2^23 + mw (24 bits), the exact product
// P = Sq * Sw lies in [2^75, 2^77).  Keep its top 53 bits (shift s = 23 or 24), round
// the s dropped bits to nearest-even, and set the exponent to eq + ew + s - 150
// (biased).  A carry out of the rounding lands in the exponent field by adding the
// 53-bit significand (implicit bit included) to (exponent - 1) << 52.
//
// Outside the domain (w zero or subnormal, a product exponent outside the normal
// range) c2g_mul_ok() is false and the caller multiplies in FP64 instead.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define C2G_HD __host__ __device__ __forceinline__
#else
#define C2G_HD inline
#endif

namespace c2g {

struct DSplit {
    uint32_t lo;  // low 32 bits of the significand
    uint32_t hi;  // high 21 bits of the significand, implicit bit included
    int32_t e;    // biased exponent
};

C2G_HD uint64_t c2g_dbits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    union {
        double d;
        uint64_t u;
    } c;
    c.d = x;
    return c.u;
#endif
}

C2G_HD double c2g_bitsd(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    union {
        double d;
        uint64_t u;
    } c;
    c.u = b;
    return c.d;
#endif
}

// Split of a positive normal double (done once per frontier residual).
C2G_HD DSplit c2g_dsplit(double q) {
    const uint64_t b = c2g_dbits(q);
    DSplit s;
    s.lo = (uint32_t)b;
    s.hi = ((uint32_t)(b >> 32) & 0xfffffu) | 0x100000u;
    s.e = (int32_t)((b >> 52) & 0x7ffu);
    return s;
}

// True when q (split) * w (float bits, sign 0) stays in the domain of c2g_mul.
C2G_HD bool c2g_mul_ok(const DSplit& q, uint32_t wb) {
    const int32_t ew = (int32_t)(wb >> 23);
    const int32_t e = q.e + ew - 127;  // product exponent before the +1 of s = 24 and of rounding
    return ew > 0 && ew < 255 && q.e > 0 && q.e < 2047 && e >= 1 && e <= 2044;
}

// q * (double)w, exact and rounded to nearest-even; requires c2g_mul_ok(q, wb).
// With A = lo * Sw (< 2^56) and B = hi * Sw (< 2^45), P = B * 2^32 + A, so
// P >> 24 = (B << 8) + (A >> 24) and P >> 23 = (B << 9) + (A >> 23) exactly (B * 2^32 is a
// multiple of 2^24); the dropped s bits (s <= 24) are the low bits of A.
C2G_HD double c2g_mul(const DSplit& q, uint32_t wb) {
    const uint32_t ew = wb >> 23;
    const uint32_t sw = (wb & 0x7fffffu) | 0x800000u;
    const uint64_t a = (uint64_t)q.lo * sw;  // < 2^56
    const uint64_t b = (uint64_t)q.hi * sw;  // < 2^45
    const uint64_t m24 = (b << 8) + (a >> 24);
    const uint32_t top = (uint32_t)(m24 >> 52);  // 1 when P >= 2^76: keep P >> 24
    const uint32_t s = 23u + top;
    uint64_t m = top ? m24 : (b << 9) + (a >> 23);  // top 53 bits of P
    const uint32_t alo = (uint32_t)a;
    const uint32_t rb = (alo >> (s - 1u)) & 1u;                    // first dropped bit
    const uint32_t sticky = (alo & ((1u << (s - 1u)) - 1u)) != 0u;  // any lower dropped bit
    m += (uint64_t)(rb & (sticky | (uint32_t)(m & 1u)));
    const int64_t e = (int64_t)q.e + (int64_t)ew + (int64_t)s - 150;
    return c2g_bitsd(((uint64_t)(e - 1) << 52) + m);
}

// Range part of c2g_mul_ok that depends on q alone: a residual exponent for which every
// normal float weight keeps the product normal (checked once per frontier residual).
C2G_HD bool c2g_mul_q_ok(const DSplit& q) { return q.e >= 128 && q.e <= 1916; }

// Weight part: w positive, normal and finite (exponent field 1..254).
C2G_HD bool c2g_mul_w_ok(uint32_t wb) { return wb - 0x00800000u < 0x7f000000u; }

// ---------------------------------------------------------------------------------------
// Float pairs (pull rounds of the batched push, which sum messages as hi + lo in FP32).
// Both conversions are integer operations on the bits, since GB300's FP64 pipe is slow.

C2G_HD float c2g_bitsf(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    union {
        float f;
        uint32_t u;
    } c;
    c.u = u;
    return c.f;
#endif
}

struct c2g_pair {
    uint32_t hi, lo;  // float bits
};

// q > 0 with biased exponent in [949, 1150] (q in [2^-74, 2^127)): hi = q cut to 24
// significant bits, lo = the remaining 29 bits cut to 24, so hi + lo <= q with relative
// error below 2^-47.  hi's float exponent is q's rebiased; lo holds q's low 29 bits
// r * 2^(eq - 1075), normalised so that its top bit is the float's implicit one.
C2G_HD bool c2g_split_ok(double q) {
    const uint32_t e = (uint32_t)(c2g_dbits(q) >> 52) & 0x7ffu;
    return e >= 949u && e <= 1150u;
}

C2G_HD c2g_pair c2g_split_pair(double q) {
    const uint64_t b = c2g_dbits(q);
    const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
    c2g_pair p;
    p.hi = ((e - 896u) << 23) | ((uint32_t)(b >> 29) & 0x7fffffu);
    const uint32_t r = (uint32_t)b & 0x1fffffffu;
    p.lo = 0u;
    if (r) {
#if defined(__CUDA_ARCH__)
        const uint32_t lz = (uint32_t)__clz((int)r) - 3u;  // r << lz has its top bit at bit 28
#else
        const uint32_t lz = (uint32_t)__builtin_clz(r) - 3u;
#endif
        p.lo = ((e - 920u - lz) << 23) | (((r << lz) >> 5) & 0x7fffffu);
    }
    return p;
}

// A float (bits) as a double, exactly, for normal floats and zero (subnormals give 0).
C2G_HD double c2g_float_bits_to_double(uint32_t u) {
    const uint32_t e = (u >> 23) & 0xffu;
    if (e == 0u) return 0.0;
    return c2g_bitsd(((uint64_t)(u & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                     ((uint64_t)(u & 0x7fffffu) << 29));
}

}  // namespace c2g
