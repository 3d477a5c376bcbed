// Host check of c2g_mul (integer FP64 product) against the native double multiply.
// Prints "ok <n>" or the first mismatch.  Built and run by tests/test_fp64_mul.py.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>

#include "fp64_mul.h"

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64() {  // splitmix64
    uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static int check(double q, float w) {
    uint32_t wb;
    std::memcpy(&wb, &w, 4);
    const c2g::DSplit s = c2g::c2g_dsplit(q);
    if (c2g::c2g_mul_q_ok(s) && c2g::c2g_mul_w_ok(wb) && !c2g::c2g_mul_ok(s, wb)) {
        std::printf("split range check admits q=%a w=%a\n", q, (double)w);
        return -1;
    }
    if (!c2g::c2g_mul_ok(s, wb)) return 0;
    const volatile double ref = q * (double)w;
    const double got = c2g::c2g_mul(s, wb);
    if (c2g::c2g_dbits(got) != c2g::c2g_dbits(ref)) {
        std::printf("mismatch q=%a w=%a got=%a ref=%a\n", q, (double)w, got, (double)ref);
        return -1;
    }
    return 1;
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 1000000;
    long done = 0;
    // edge cases: significands all ones / exact halves / powers of two
    const double qs[] = {1.0, 1.5, 0.85, 1e-7, 1.0000000000000002, 1.9999999999999998, 0.3333333333333333,
                         8.5e-8, 1.0 - 1e-16, 6.103515625e-05};
    const float ws[] = {1.0f, 0.5f, 1.99999988f, 1.00000012f, 0.1f, 1e-30f, 0.8f, 0.999999940f, 3.0f, 1e-20f};
    for (double q : qs)
        for (float w : ws) {
            const int r = check(q, w);
            if (r < 0) return 1;
            done += r;
        }
    for (long i = 0; i < n; ++i) {
        // random q in the residual range of the push (1e-12 .. 10), random significands;
        // random w over normal floats in (1e-38, 4)
        const uint64_t a = next_u64(), b = next_u64();
        const int qe = 1023 - 40 + (int)(a % 44);
        const double q = c2g::c2g_bitsd(((uint64_t)qe << 52) | (b & 0xfffffffffffffull));
        const uint32_t wb = (uint32_t)(1 + (a >> 40) % 128) << 23 | (uint32_t)(b >> 41);
        float w;
        std::memcpy(&w, &wb, 4);
        const int r = check(q, w);
        if (r < 0) return 1;
        done += r;
        // ties: force the dropped bits to exactly half for one in 8 cases
        if ((a & 7) == 0) {
            const double q2 = c2g::c2g_bitsd(((uint64_t)qe << 52) | ((b & 0xfffffffffffffull) & ~0xffffffull));
            const int r2 = check(q2, w);
            if (r2 < 0) return 1;
            done += r2;
        }
    }
    // float pairs: hi + lo <= q within 2^-47 relative, both parts exact as doubles
    for (long i = 0; i < n; ++i) {
        const uint64_t a = next_u64(), b = next_u64();
        const uint64_t e = 949 + a % 202;
        const double q = c2g::c2g_bitsd((e << 52) | (b & 0xfffffffffffffull));
        if (!c2g::c2g_split_ok(q)) {
            std::printf("split range rejects q=%a\n", q);
            return 1;
        }
        const c2g::c2g_pair p = c2g::c2g_split_pair(q);
        const float hi = c2g::c2g_bitsf(p.hi), lo = c2g::c2g_bitsf(p.lo);
        const double hd = c2g::c2g_float_bits_to_double(p.hi), ld = c2g::c2g_float_bits_to_double(p.lo);
        if (hd != (double)hi || ld != (double)lo) {
            std::printf("float->double mismatch q=%a\n", q);
            return 1;
        }
        const double rel = (q - (hd + ld)) / q;
        if (!(rel >= 0.0 && rel < 0x1p-47)) {
            std::printf("split error q=%a hi=%a lo=%a rel=%g\n", q, (double)hi, (double)lo, rel);
            return 1;
        }
        ++done;
    }
    std::printf("ok %ld\n", done);
    return 0;
}
