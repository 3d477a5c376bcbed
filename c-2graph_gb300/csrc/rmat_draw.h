// The R-MAT generator's random draws, shared by the host writer (rmat.cpp) and the
// device one (rmat_gpu.cu) so both produce the same graph bit for bit.
//
// Every draw is a counter-based splitmix64 output keyed by (seed, stream, index), so the
// graph depends on no thread count or schedule.  Streams: 1 edge endpoints, 2 int32
// weights, 3 flist values.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define C2G_RMAT_HD __host__ __device__ __forceinline__
#else
#define C2G_RMAT_HD inline
#endif

namespace c2g {

C2G_RMAT_HD uint64_t rmat_mix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

C2G_RMAT_HD uint64_t rmat_draw(uint64_t seed, uint64_t stream, uint64_t index, uint64_t k) {
    return rmat_mix64(rmat_mix64(seed ^ (stream * 0xd1342543de82ef95ULL)) + index * 0x9e3779b97f4a7c15ULL + k);
}

// Endpoints of edge draw i: one quadrant per level, the quadrant chosen by a 32-bit draw
// against the cumulative thresholds ta <= tb <= tc (a, a+b, a+b+c scaled by 2^32).
C2G_RMAT_HD void rmat_endpoints(uint64_t seed, uint64_t i, int scale, uint64_t ta, uint64_t tb, uint64_t tc,
                                uint64_t* src, uint64_t* dst) {
    uint64_t s = 0, d = 0, r = 0;
    for (int lvl = 0; lvl < scale; ++lvl) {
        if ((lvl & 1) == 0) r = rmat_draw(seed, 1, i, (uint64_t)(lvl >> 1));
        const uint64_t q = (lvl & 1) ? (r >> 32) : (r & 0xffffffffULL);
        const int bit = scale - 1 - lvl;
        if (q < ta) {
        } else if (q < tb) {
            d |= uint64_t(1) << bit;
        } else if (q < tc) {
            s |= uint64_t(1) << bit;
        } else {
            s |= uint64_t(1) << bit;
            d |= uint64_t(1) << bit;
        }
    }
    *src = s;
    *dst = d;
}

// int32 weight of CSR edge e, uniform in [wmin, wmin + range).
C2G_RMAT_HD int32_t rmat_weight(uint64_t seed, uint64_t e, int32_t wmin, uint64_t range) {
    return (int32_t)((int64_t)wmin + (int64_t)(rmat_draw(seed, 2, e, 0) % range));
}

// Unnormalised flist value of CSR edge e: uniform(0,1) with 24 random bits, exactly
// representable as a float.
C2G_RMAT_HD float rmat_fvalue(uint64_t seed, uint64_t e) {
    return (float)(((double)(rmat_draw(seed, 3, e, 0) >> 40) + 0.5) / 16777216.0);
}

}  // namespace c2g
