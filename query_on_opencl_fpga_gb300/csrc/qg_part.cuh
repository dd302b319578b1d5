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

// The model may live in global memory (read through the read-only cache) or
// in shared memory (a kernel that evaluates it for every row stages a copy).
template <bool SHARED>
__device__ __forceinline__ uint32_t qg_cdf_ld(const uint32_t *p) { return SHARED ? *p : __ldg(p); }
template <bool SHARED>
__device__ __forceinline__ float qg_cdf_ldf(const float *p) { return SHARED ? *p : __ldg(p); }

template <bool SHARED>
__device__ __forceinline__ uint32_t qg_cdf_bucket_t(const qg_cdf_model *__restrict__ m, uint32_t u) {
    const uint32_t K = qg_cdf_ld<SHARED>(&m->nknots);
    const uint32_t x0 = qg_cdf_ld<SHARED>(&m->x[0]);
    if (u <= x0) return u == x0 ? qg_cdf_ld<SHARED>(&m->bk[0]) : 0u;
    const uint32_t xl = qg_cdf_ld<SHARED>(&m->x[K - 1]);
    if (u >= xl) return u == xl ? qg_cdf_ld<SHARED>(&m->bk[K - 1]) : qg_cdf_ld<SHARED>(&m->nbuckets) - 1u;
    // Largest i with x[i] <= u lies in [idx[t], idx[t+1]]; x[hi] > u.
    const uint32_t t = (u - x0) >> qg_cdf_ld<SHARED>(&m->ishift);
    uint32_t lo = qg_cdf_ld<SHARED>(&m->idx[t]);
    uint32_t hi = min(qg_cdf_ld<SHARED>(&m->idx[t + 1]) + 1u, K - 1u);
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (qg_cdf_ld<SHARED>(&m->x[mid]) <= u) lo = mid;
        else hi = mid;
    }
    const uint32_t xi = qg_cdf_ld<SHARED>(&m->x[lo]);
    if (u == xi) return qg_cdf_ld<SHARED>(&m->bk[lo]);
    const uint32_t b0 = qg_cdf_ld<SHARED>(&m->b0[lo]), span = qg_cdf_ld<SHARED>(&m->b1[lo]) - b0;
    const float f = qg_cdf_ldf<SHARED>(&m->slope[lo]) * (float)(u - xi - 1u);
    return b0 + (f >= (float)span ? span : (uint32_t)f);
}

__device__ __forceinline__ uint32_t qg_cdf_bucket(const qg_cdf_model *__restrict__ m, uint32_t u) {
    return qg_cdf_bucket_t<false>(m, u);
}

// The model's scalar fields, read once by a kernel that evaluates many keys.
struct qg_cdf_head {
    uint32_t K, x0, xl, ishift, nb1, bk0, bkl;
};
template <bool SHARED>
__device__ __forceinline__ qg_cdf_head qg_cdf_load_head(const qg_cdf_model *__restrict__ m) {
    qg_cdf_head h;
    h.K = qg_cdf_ld<SHARED>(&m->nknots);
    h.x0 = qg_cdf_ld<SHARED>(&m->x[0]);
    h.xl = qg_cdf_ld<SHARED>(&m->x[h.K - 1]);
    h.ishift = qg_cdf_ld<SHARED>(&m->ishift);
    h.nb1 = qg_cdf_ld<SHARED>(&m->nbuckets) - 1u;
    h.bk0 = qg_cdf_ld<SHARED>(&m->bk[0]);
    h.bkl = qg_cdf_ld<SHARED>(&m->bk[h.K - 1]);
    return h;
}
// qg_cdf_bucket_t with the scalar fields already in registers.
template <bool SHARED>
__device__ __forceinline__ uint32_t qg_cdf_bucket_h(const qg_cdf_model *__restrict__ m, const qg_cdf_head &h,
                                                    uint32_t u) {
    if (u <= h.x0) return u == h.x0 ? h.bk0 : 0u;
    if (u >= h.xl) return u == h.xl ? h.bkl : h.nb1;
    const uint32_t t = (u - h.x0) >> h.ishift;
    uint32_t lo = qg_cdf_ld<SHARED>(&m->idx[t]);
    uint32_t hi = min(qg_cdf_ld<SHARED>(&m->idx[t + 1]) + 1u, h.K - 1u);
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (qg_cdf_ld<SHARED>(&m->x[mid]) <= u) lo = mid;
        else hi = mid;
    }
    const uint32_t xi = qg_cdf_ld<SHARED>(&m->x[lo]);
    if (u == xi) return qg_cdf_ld<SHARED>(&m->bk[lo]);
    const uint32_t b0 = qg_cdf_ld<SHARED>(&m->b0[lo]), span = qg_cdf_ld<SHARED>(&m->b1[lo]) - b0;
    const float f = qg_cdf_ldf<SHARED>(&m->slope[lo]) * (float)(u - xi - 1u);
    return b0 + (f >= (float)span ? span : (uint32_t)f);
}

__device__ __forceinline__ uint32_t qg_part_bucket(const qg_part_fn &pf, uint32_t u) {
    // shift may be 32 (a single bucket over the whole key range)
    return pf.learned ? qg_cdf_bucket(pf.model, u)
                      : (uint32_t)((unsigned long long)(u - pf.kmin) >> pf.shift);
}
