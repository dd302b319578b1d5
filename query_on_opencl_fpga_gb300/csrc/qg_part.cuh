// qg_part.cuh -- partition functions: key -> bucket, non-decreasing in the
// unsigned key, so that buckets are key ranges and the concatenation of the
// buckets in order is ordered by key.
//
//   radix:   bucket = (k - kmin) >> shift                      (plain)
//   learned: a piecewise-linear model of the key CDF, 1024 segments between
//            knots at sample quantiles, fp32 slope per segment, plus knots
//            for heavy keys (keys holding at least ~3 buckets' worth of the
//            sample), each of which gets a bucket of its own.
//
// The learned model is fitted on the GPU (k_cdf_fit in qg_pjoin.cu) from a
// sorted key sample and evaluated by every partition kernel through
// qg_cdf_bucket.  Bucket assignment only decides where a row is processed;
// join results are bit-exact whichever function is used.
#pragma once
#include "qg_internal.cuh"

constexpr int QG_CDF_SEGMENTS = 1024;
constexpr int QG_CDF_MAX_HEAVY = 255;
constexpr int QG_CDF_MAX_KNOTS = 1280;  // 1025 quantile knots + heavy knots, deduplicated
constexpr int QG_CDF_INDEX = 4096;       // top-level index over [x0, x_last]

struct qg_cdf_model {
    uint32_t nknots;    // knots in use (>= 1), strictly increasing keys
    uint32_t nbuckets;  // buckets of the partition
    uint32_t ishift;    // index slot of key u: (u - x[0]) >> ishift
    uint32_t nheavy;    // knots flagged heavy
    uint32_t x[QG_CDF_MAX_KNOTS];    // knot keys
    uint32_t bk[QG_CDF_MAX_KNOTS];   // bucket of a key equal to knot i
    uint32_t b0[QG_CDF_MAX_KNOTS];   // first bucket of keys strictly between knots i and i+1
    uint32_t b1[QG_CDF_MAX_KNOTS];   // last bucket of those keys
    float slope[QG_CDF_MAX_KNOTS];   // buckets per key unit between knots i and i+1
    uint32_t idx[QG_CDF_INDEX + 1];  // largest knot <= x[0] + (t << ishift)
};

// Partition function descriptor passed by value to kernels.
struct qg_part_fn {
    int learned;                    // 0 radix, 1 learned model
    uint32_t kmin;                  // radix: smallest key of the domain
    int shift;                      // radix: bucket = (k - kmin) >> shift, 0..32
    const qg_cdf_model *model;      // learned: device model
};

__device__ __forceinline__ uint32_t qg_cdf_bucket(const qg_cdf_model *__restrict__ m, uint32_t u) {
    const uint32_t K = __ldg(&m->nknots);
    const uint32_t x0 = __ldg(&m->x[0]);
    if (u <= x0) return u == x0 ? __ldg(&m->bk[0]) : 0u;
    const uint32_t xl = __ldg(&m->x[K - 1]);
    if (u >= xl) return u == xl ? __ldg(&m->bk[K - 1]) : __ldg(&m->nbuckets) - 1u;
    // Largest i with x[i] <= u lies in [idx[t], idx[t+1]]; x[hi] > u.
    const uint32_t t = (u - x0) >> __ldg(&m->ishift);
    uint32_t lo = __ldg(&m->idx[t]);
    uint32_t hi = min(__ldg(&m->idx[t + 1]) + 1u, K - 1u);
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&m->x[mid]) <= u) lo = mid;
        else hi = mid;
    }
    const uint32_t xi = __ldg(&m->x[lo]);
    if (u == xi) return __ldg(&m->bk[lo]);
    const uint32_t b0 = __ldg(&m->b0[lo]), span = __ldg(&m->b1[lo]) - b0;
    const float f = __ldg(&m->slope[lo]) * (float)(u - xi - 1u);
    return b0 + (f >= (float)span ? span : (uint32_t)f);
}

__device__ __forceinline__ uint32_t qg_part_bucket(const qg_part_fn &pf, uint32_t u) {
    // shift may be 32 (a single bucket over the whole key range)
    return pf.learned ? qg_cdf_bucket(pf.model, u)
                      : (uint32_t)((unsigned long long)(u - pf.kmin) >> pf.shift);
}
