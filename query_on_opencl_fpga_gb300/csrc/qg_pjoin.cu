// qg_pjoin.cu -- range-partitioned join + filter + sort (the default path of
// qg_join_filter_sort).
//
// Reference operators this replaces: buildHashTable / probeHashTable and the
// filter + bitonic sort of the matches (kernel/hj_filter_sort/1/
// hj_filter_sort_op.cl:25-109, :117-564).  Output contract: every pair
// (R row, S row) with equal uint keys whose S.payload passes the filter,
// emitted as (key, R.payload, S.payload), ordered by the unsigned key; the
// order among equal keys is unspecified (the reference's bitonic sort is not
// stable either).
//
// Pipeline (one GPU, all data in HBM; two host reads before the last):
//   1. R's key and payload ranges.  When R's keys are unique over at most
//      2 nR values (the dense build side), R becomes a table indexed by
//      key - kmin: payloads, with a sentinel payload (or a presence bitmap)
//      marking absent keys, and R is never partitioned.  Otherwise R's
//      records (key << 32 | payload) and their radix digit histograms.
//   2. S: filter on S.payload and on R's key range, compacted in one pass
//      into S' records (key << 32 | S.payload); the order of S' is free, so
//      each tile takes its output range with one atomic.  The filter also
//      counts the S' radix digit histograms.  Host read 1: ranges, counts,
//      histograms, dense flags.
//   3. A partition function maps keys to B buckets (key ranges): radix over
//      (k - kmin), or a learned piecewise-linear CDF model fitted on a sample
//      (qg_part.cuh).  One or two onesweep radix passes over the bucket id
//      (qg_sort.cu; the first need not be stable) put S' -- and R on the
//      general path -- in bucket order.
//   4. Bucket bounds, and consecutive buckets packed into join groups on the
//      device (k_pj_pack / k_pj_place).  Host read 2: the group count.
//   5. One CTA per group (tickets in group order).  Dense build side
//      (k_pj_join_dense): each S' row matches when its key's table entry is
//      filled, the count is published at once, the matching rows are
//      counting-sorted and written in key order (with R's keys filling their
//      span every row matches, and no look-back is needed).  General path
//      (k_pj_join): R's rows in a shared-memory chained table, S' rows probed
//      in registers, the count published, the matching rows sorted and their
//      matches written in key order.  Groups are key ranges, so the output
//      is sorted with no global sort pass.
//   6. Buckets too large for shared memory (general path): a bucket with one
//      key is a cross product (k_pj_cross); all the others are gathered,
//      sorted by key and merge-joined together (k_pj_mj_*: a fixed number of
//      launches however many such buckets there are).  Their match counts are
//      known before step 5, which publishes every such bucket's output
//      offset; the writes of step 6 read it.  On the dense side an oversize
//      bucket sends the call to the general path (R's records made then, the
//      S' partitioning reused).
#include <algorithm>
#include <string.h>
#include <vector>
#include "qg_internal.cuh"
#include "qg_part.cuh"
#include "qg_sort.cuh"

namespace {

// ---------------------------------------------------------------------------
// 1. R columns -> records, key range
// ---------------------------------------------------------------------------
struct PjRange {
    uint32_t kmin, kmax;
    unsigned long long count;  // S' rows (step 2)
};

// Radix partition function of the join over R's key range [kmin, kmax] with
// up to 2^lb2 buckets: bucket = (k - kmin) >> shift.  The host and the
// kernels that read the range from device memory derive it the same way.
struct PjRadix {
    int shift;
    uint32_t nb;  // buckets in use: (kmax - kmin) >> shift, plus one
};
__host__ __device__ inline PjRadix pj_radix(uint32_t kmin, uint32_t kmax, int lb2) {
    const uint32_t range = kmax - kmin;
    int bits = 0;
    while (bits < 32 && (range >> bits) != 0u) bits++;
    const int shift = bits > lb2 ? bits - lb2 : 0;
    return PjRadix{shift, (uint32_t)(((unsigned long long)range >> shift) + 1)};
}

// Dense build side: R's keys unique and spread over at most 2 nR values,
// with buckets of at most PJ_DENSE_BSPAN keys.  Then a presence bitmap and a
// payload table indexed by key - kmin stand for R in key order, and R needs
// no partitioning at all.
constexpr uint32_t PJ_DENSE_BSPAN = 8192;
__host__ __device__ inline bool pj_dense_span(uint32_t kmin, uint32_t kmax, int lb2, long long nR) {
    const unsigned long long w = (unsigned long long)(kmax - kmin) + 1ull;
    return w <= 2ull * (unsigned long long)nR && (1ull << pj_radix(kmin, kmax, lb2).shift) <= PJ_DENSE_BSPAN;
}

// Counts of the join groups packed on the device (k_pj_place): groups, buckets
// listed as oversize, their rows, the largest of them.
struct PjPackOut {
    uint32_t groups, over;
    unsigned long long over_rows;
    uint32_t most, pad;
};

// flags of the dense build side (u32 words): [1] dense span, [2..3] distinct
// keys (u64), [4] / [5] smallest / largest R payload (int32), [6] a sentinel
// payload exists, [7] the sentinel.
enum { PJ_F_DENSE = 1, PJ_F_DISTINCT = 2, PJ_F_PMIN = 4, PJ_F_PMAX = 5, PJ_F_SENT_OK = 6, PJ_F_SENT = 7, PJ_F_WORDS = 8 };

__global__ void k_pj_range_init(PjRange *r, uint32_t *flags) {
    r->kmin = 0xffffffffu;
    r->kmax = 0;
    r->count = 0;
    for (int i = 0; i < PJ_F_WORDS; i++) flags[i] = 0;
    flags[PJ_F_PMIN] = 0x7fffffffu;
    flags[PJ_F_PMAX] = 0x80000000u;
}

__global__ void __launch_bounds__(256)
k_pj_rrec(const int32_t *__restrict__ rkey, const int32_t *__restrict__ rpay, long long nR,
          unsigned long long *__restrict__ rec, PjRange *range) {
    uint32_t lmin = 0xffffffffu, lmax = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nR; i += stride) {
        const uint32_t k = (uint32_t)__ldg(rkey + i);
        const uint32_t p = (uint32_t)__ldg(rpay + i);
        rec[i] = ((unsigned long long)k << 32) | p;
        lmin = min(lmin, k);
        lmax = max(lmax, k);
    }
    lmin = __reduce_min_sync(QG_FULL_MASK, lmin);
    lmax = __reduce_max_sync(QG_FULL_MASK, lmax);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&range->kmin, lmin);
        atomicMax(&range->kmax, lmax);
    }
}

// R's key range and payload range (16-byte loads where aligned).
__global__ void __launch_bounds__(256)
k_pj_rrange(const int32_t *__restrict__ rkey, const int32_t *__restrict__ rpay, long long nR, PjRange *range,
            uint32_t *flags) {
    uint32_t lmin = 0xffffffffu, lmax = 0;
    int32_t pmin = 0x7fffffff, pmax = (int32_t)0x80000000;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool vec = (((uintptr_t)rkey | (uintptr_t)rpay) & 15) == 0;
    const long long nv = vec ? nR / 4 : 0;
    for (long long i = t0; i < nv; i += stride) {
        const int4 v = __ldg(reinterpret_cast<const int4 *>(rkey) + i);
        const int4 p = __ldg(reinterpret_cast<const int4 *>(rpay) + i);
        lmin = min(min(lmin, (uint32_t)v.x), min((uint32_t)v.y, min((uint32_t)v.z, (uint32_t)v.w)));
        lmax = max(max(lmax, (uint32_t)v.x), max((uint32_t)v.y, max((uint32_t)v.z, (uint32_t)v.w)));
        pmin = min(min(pmin, p.x), min(p.y, min(p.z, p.w)));
        pmax = max(max(pmax, p.x), max(p.y, max(p.z, p.w)));
    }
    for (long long i = 4 * nv + t0; i < nR; i += stride) {
        const uint32_t k = (uint32_t)__ldg(rkey + i);
        const int32_t p = __ldg(rpay + i);
        lmin = min(lmin, k);
        lmax = max(lmax, k);
        pmin = min(pmin, p);
        pmax = max(pmax, p);
    }
    lmin = __reduce_min_sync(QG_FULL_MASK, lmin);
    lmax = __reduce_max_sync(QG_FULL_MASK, lmax);
    pmin = __reduce_min_sync(QG_FULL_MASK, pmin);
    pmax = __reduce_max_sync(QG_FULL_MASK, pmax);
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&range->kmin, lmin);
        atomicMax(&range->kmax, lmax);
        atomicMin(reinterpret_cast<int *>(flags + PJ_F_PMIN), pmin);
        atomicMax(reinterpret_cast<int *>(flags + PJ_F_PMAX), pmax);
    }
}

// A payload value that no R row holds and whose four bytes are equal (so a
// byte memset could write it): the first b * 0x01010101 outside [pmin, pmax].
__device__ __forceinline__ bool pj_sentinel(int32_t pmin, int32_t pmax, uint32_t *out) {
    for (uint32_t b = 0; b < 256; b++) {
        const int32_t v = (int32_t)(b * 0x01010101u);
        if (v < pmin || v > pmax) {
            *out = (uint32_t)v;
            return true;
        }
    }
    return false;
}

// Dense span with a sentinel payload: T[0 .. w) = the sentinel (no row yet),
// flags[PJ_F_SENT_OK] = 1, flags[PJ_F_SENT] = the sentinel.
__global__ void __launch_bounds__(256)
k_pj_tfill(uint32_t *__restrict__ T, const PjRange *__restrict__ range, int lb2, long long nR, uint32_t *flags) {
    const uint32_t kmin = range->kmin, kmax = range->kmax;
    if (!pj_dense_span(kmin, kmax, lb2, nR)) return;
    uint32_t sent;
    if (!pj_sentinel((int32_t)flags[PJ_F_PMIN], (int32_t)flags[PJ_F_PMAX], &sent)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        flags[PJ_F_SENT_OK] = 1u;
        flags[PJ_F_SENT] = sent;
    }
    const unsigned long long w = (unsigned long long)(kmax - kmin) + 1ull, w4 = w >> 2;
    uint4 *t4 = reinterpret_cast<uint4 *>(T);  // T is 256-byte aligned
    for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < w4;
         i += (unsigned long long)gridDim.x * blockDim.x)
        t4[i] = make_uint4(sent, sent, sent, sent);
    if (blockIdx.x == 0 && threadIdx.x < (w & 3ull)) T[4 * w4 + threadIdx.x] = sent;
}

// R after its key range is known.  Dense span (pj_dense_span): T[offset] =
// payload, and -- unless k_pj_tfill found a sentinel payload (T then holds it
// where no row is) -- the presence bit of every key offset is set (fire-and-
// forget reductions); flags[PJ_F_DENSE] = 1.  k_pj_distinct then counts the
// keys, and fewer than nR means a duplicate.  (An 8-byte entry holding both, one store
// per row, measured slower: 0.37 against 0.21 ms at 16M rows, its 128 MB of
// scattered partial-sector writes spilling out of L2, where the 64 MB table
// and 2 MB bitmap stay.)  Otherwise: R records (key << 32 | payload) and the
// two 8-bit digit histograms of their radix bucket ids into hist[0 .. 512).
__global__ void __launch_bounds__(256)
k_pj_rtab(const int32_t *__restrict__ rkey, const int32_t *__restrict__ rpay, long long nR,
          const PjRange *__restrict__ range, int lb2, uint32_t *__restrict__ bitmap, uint32_t *__restrict__ T,
          uint32_t *__restrict__ flags, unsigned long long *__restrict__ rec, uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[2][256];
    const uint32_t kmin = range->kmin, kmax = range->kmax;
    const bool dense = pj_dense_span(kmin, kmax, lb2, nR);
    const long long stride = (long long)gridDim.x * blockDim.x;
    if (dense) {
        if (blockIdx.x == 0 && threadIdx.x == 0) flags[PJ_F_DENSE] = 1u;
        const bool sent = flags[PJ_F_SENT_OK] != 0u;  // T holds the sentinel where no row is: no bitmap
        constexpr int U = 4;  // rows in flight per thread
        for (long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; i0 < nR; i0 += U * stride) {
            uint32_t off[U], pay[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const long long i = i0 + u * stride;
                off[u] = i < nR ? (uint32_t)__ldg(rkey + i) - kmin : 0u;
                pay[u] = i < nR ? (uint32_t)__ldg(rpay + i) : 0u;
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (i0 + u * stride >= nR) break;
                if (!sent) atomicOr(&bitmap[off[u] >> 5], 1u << (off[u] & 31u));  // result unused: a reduction
                T[off[u]] = pay[u];
            }
        }
        return;
    }
    for (int i = threadIdx.x; i < 512; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    const PjRadix rp = pj_radix(kmin, kmax, lb2);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nR; i += stride) {
        const uint32_t k = (uint32_t)__ldg(rkey + i);
        rec[i] = ((unsigned long long)k << 32) | (uint32_t)__ldg(rpay + i);
        const uint32_t bk = (uint32_t)((unsigned long long)(k - kmin) >> rp.shift);
        atomicAdd(&h[0][bk & 255u], 1u);
        atomicAdd(&h[1][(bk >> 8) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x)
        if ((&h[0][0])[i]) atomicAdd(&hist[i], (&h[0][0])[i]);
}

// Distinct R keys over the dense span (only when k_pj_rtab built it), added
// to *count: the table entries that are not the sentinel, or the set bits of
// the presence bitmap.
__global__ void __launch_bounds__(256)
k_pj_distinct(const uint32_t *__restrict__ bitmap, const uint32_t *__restrict__ T, const PjRange *__restrict__ range,
              int lb2, long long nR, const uint32_t *__restrict__ flags, unsigned long long *__restrict__ count) {
    const uint32_t kmin = range->kmin, kmax = range->kmax;
    if (!pj_dense_span(kmin, kmax, lb2, nR)) return;
    const unsigned long long w = (unsigned long long)(kmax - kmin) + 1ull;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    const unsigned long long t0 = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t c = 0;
    if (flags[PJ_F_SENT_OK]) {
        const uint32_t sent = flags[PJ_F_SENT];
        const uint4 *t4 = reinterpret_cast<const uint4 *>(T);
        for (unsigned long long i = t0; i < (w >> 2); i += stride) {
            const uint4 x = __ldcs(t4 + i);
            c += (x.x != sent) + (x.y != sent) + (x.z != sent) + (x.w != sent);
        }
        for (unsigned long long i = 4 * (w >> 2) + t0; i < w; i += stride) c += __ldcs(T + i) != sent;
    } else {
        for (unsigned long long i = t0; i < ((w + 31ull) >> 5); i += stride) c += __popc(__ldcg(bitmap + i));
    }
    c = __reduce_add_sync(QG_FULL_MASK, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, (unsigned long long)c);
}

// ---------------------------------------------------------------------------
// 2. S filter + range test, compacted into S' records
// ---------------------------------------------------------------------------
constexpr int SF_THREADS = 256;
constexpr int SF_WARPS = SF_THREADS / 32;
constexpr int SF_ROUNDS = 4;  // int4 of keys + int4 of payloads per round: 4096 rows per tile


// S-filter without input order: S' is repartitioned by key right after, and
// the join leaves the order among equal keys unspecified, so a tile takes
// its output range with one atomic on the S' counter instead of a look-back
// over earlier tiles.  R's key range is read from device memory (no host
// round trip before the launch).  Persistent CTAs walk the tiles.  A tile's
// selected rows are compacted into shared memory and written from there
// with consecutive addresses; on the way out each is counted by the two
// 8-bit digits of its radix bucket id in shared memory (the partition
// passes' digit histograms, so S' is not read again to count them), added to
// hist[0..512) once at the end.
__global__ void __launch_bounds__(SF_THREADS, 4)
k_pj_sfilter(const int32_t *__restrict__ skey, const int32_t *__restrict__ spay, long long n,
               int32_t slo, int32_t shi, const PjRange *__restrict__ range,
               unsigned long long *__restrict__ out, unsigned long long *__restrict__ cursor,
               qg_control *ctl, int lb2, uint32_t *__restrict__ hist) {
    constexpr int TILE = SF_THREADS * SF_ROUNDS * 4;
    __shared__ uint32_t s_woff[SF_ROUNDS * SF_WARPS];
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_cnt;
    __shared__ uint32_t s_h[2][256];
    __shared__ unsigned long long s_out[TILE];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt = qg_lanemask_lt();
    for (int i = tid; i < 512; i += SF_THREADS) (&s_h[0][0])[i] = 0;
    const uint32_t kmin = range->kmin, kmax = range->kmax;
    const PjRadix rp = pj_radix(kmin, kmax, lb2);
    const bool two = rp.nb > 256u;  // the high digit is 0 for every row otherwise
    const long long ntiles = (n + TILE - 1) / TILE;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long base = t * TILE;
        int4 kv[SF_ROUNDS], pv[SF_ROUNDS];
#pragma unroll
        for (int r = 0; r < SF_ROUNDS; r++) {
            const long long idx = base + (long long)(r * SF_THREADS + tid) * 4;
            if (idx + 3 < n) {
                kv[r] = qg_ldg_stream(reinterpret_cast<const int4 *>(skey + idx));
                pv[r] = qg_ldg_stream(reinterpret_cast<const int4 *>(spay + idx));
            } else {
                int tk[4] = {0, 0, 0, 0}, tp[4] = {0, 0, 0, 0};
                for (int j = 0; j < 4; j++)
                    if (idx + j < n) { tk[j] = skey[idx + j]; tp[j] = spay[idx + j]; }
                kv[r] = make_int4(tk[0], tk[1], tk[2], tk[3]);
                pv[r] = make_int4(tp[0], tp[1], tp[2], tp[3]);
            }
        }
        uint32_t fl = 0, lpre[SF_ROUNDS];
#pragma unroll
        for (int r = 0; r < SF_ROUNDS; r++) {
            const long long idx = base + (long long)(r * SF_THREADS + tid) * 4;
            const int32_t kk[4] = {kv[r].x, kv[r].y, kv[r].z, kv[r].w};
            const int32_t pp[4] = {pv[r].x, pv[r].y, pv[r].z, pv[r].w};
            uint32_t f = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const uint32_t u = (uint32_t)kk[j];
                f |= (uint32_t)((idx + j < n) & (pp[j] >= slo) & (pp[j] <= shi) & (u >= kmin) & (u <= kmax)) << j;
            }
            uint32_t c = 0, tot = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const uint32_t bl = __ballot_sync(QG_FULL_MASK, (f >> j) & 1u);
                c += __popc(bl & lt);
                tot += __popc(bl);
            }
            lpre[r] = c;
            if (lane == 0) s_woff[r * SF_WARPS + warp] = tot;
            fl |= f << (4 * r);
        }
        __syncthreads();
        if (warp == 0) {  // exclusive offsets of the tile's (round, warp) pieces; one atomic for the tile
            const uint32_t x = s_woff[lane];  // SF_ROUNDS * SF_WARPS == 32
            uint32_t inc = x;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(QG_FULL_MASK, inc, d);
                if (lane >= d) inc += y;
            }
            s_woff[lane] = inc - x;
            if (lane == 31) {
                s_cnt = inc;
                s_base = inc ? atomicAdd(cursor, (unsigned long long)inc) : 0ull;
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < SF_ROUNDS; r++) {
            uint32_t pos = s_woff[r * SF_WARPS + warp] + lpre[r];
            const int32_t kk[4] = {kv[r].x, kv[r].y, kv[r].z, kv[r].w};
            const int32_t pp[4] = {pv[r].x, pv[r].y, pv[r].z, pv[r].w};
#pragma unroll
            for (int j = 0; j < 4; j++)
                if ((fl >> (4 * r + j)) & 1u) s_out[pos++] = ((unsigned long long)(uint32_t)kk[j] << 32) | (uint32_t)pp[j];
        }
        __syncthreads();
        const unsigned long long tb = s_base;
        const uint32_t cnt = s_cnt;
        for (uint32_t i = tid; i < cnt; i += SF_THREADS) {
            const unsigned long long v = s_out[i];
            if (tb + i < (unsigned long long)n) out[tb + i] = v;
            else qg_record_error(ctl, QG_ERR_INVALID, QG_SITE_PJ_FILTER);
            const uint32_t bk = (uint32_t)((unsigned long long)((uint32_t)(v >> 32) - kmin) >> rp.shift);
            atomicAdd(&s_h[0][bk & 255u], 1u);
            if (two) atomicAdd(&s_h[1][(bk >> 8) & 255u], 1u);
        }
        __syncthreads();  // s_woff, s_base, s_cnt and s_out are rewritten by the next tile
    }
    __syncthreads();
    for (int i = tid; i < 512; i += SF_THREADS)
        if ((&s_h[0][0])[i]) atomicAdd(&hist[i], (&s_h[0][0])[i]);
}
static_assert(SF_ROUNDS * SF_WARPS == 32, "one warp scans the tile's pieces");


// ---------------------------------------------------------------------------
// 3. digit histograms of the bucket id, bucket bounds, CDF sample and fit
// ---------------------------------------------------------------------------
constexpr int PJ_MAX_BUCKETS = 1 << 16;  // two 8-bit partition passes

// Histograms of the two 8-bit digits of each row's bucket (shared-memory
// privatised), for the partition passes' digit bases.  With drange set (radix
// only) the function comes from R's key range in device memory and lb2.
template <bool LEARNED>
__global__ void __launch_bounds__(256)
k_pj_dhist(const unsigned long long *__restrict__ rec, long long n, qg_part_fn pf, uint32_t nb,
           uint32_t *__restrict__ hist, qg_control *ctl, uint16_t *__restrict__ bid,
           const PjRange *__restrict__ drange, int lb2) {
    __shared__ uint32_t h[2][256];
    if (!LEARNED && drange) {
        const PjRadix rp = pj_radix(drange->kmin, drange->kmax, lb2);
        pf = qg_part_fn{0, drange->kmin, rp.shift, nullptr};
        nb = rp.nb;
    }
    // A learned function is evaluated from a shared-memory copy of the model.
    __shared__ __align__(16) unsigned char sm_model[LEARNED ? sizeof(qg_cdf_model) : 16];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) (&h[0][0])[i] = 0;
    if (LEARNED) {
        static_assert(sizeof(qg_cdf_model) % 4 == 0, "model copied in words");
        const uint32_t *gsrc = reinterpret_cast<const uint32_t *>(pf.model);
        uint32_t *sdst = reinterpret_cast<uint32_t *>(sm_model);
        for (int i = threadIdx.x; i < (int)(sizeof(qg_cdf_model) / 4); i += blockDim.x) sdst[i] = __ldg(gsrc + i);
    }
    __syncthreads();
    const qg_cdf_model *sm = reinterpret_cast<const qg_cdf_model *>(sm_model);
    qg_cdf_head hd{};
    if (LEARNED) hd = qg_cdf_load_head<true>(sm);
    const long long stride = (long long)gridDim.x * blockDim.x;
    auto count = [&](long long i, uint32_t b) {
        if (b >= nb) {  // a key outside the partition function's domain
            qg_record_error(ctl, QG_ERR_INVALID, QG_SITE_PJ_HIST);
            return;
        }
        if (bid) bid[i] = (uint16_t)b;  // nb <= 2^16: the id for the partition passes
        atomicAdd(&h[0][b & 255u], 1u);
        atomicAdd(&h[1][b >> 8], 1u);
    };
    // Four rows per thread and round: their loads, then their buckets (four
    // independent model evaluations), then their counts.
    constexpr int U = 4;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < n; i += U * stride) {
        uint32_t u[U], b[U];
#pragma unroll
        for (int j = 0; j < U; j++) u[j] = (uint32_t)(__ldg(rec + i + j * stride) >> 32);
#pragma unroll
        for (int j = 0; j < U; j++) b[j] = LEARNED ? qg_cdf_bucket_h<true>(sm, hd, u[j]) : qg_part_bucket(pf, u[j]);
#pragma unroll
        for (int j = 0; j < U; j++) count(i + j * stride, b[j]);
    }
    for (; i < n; i += stride) {
        const uint32_t u = (uint32_t)(__ldg(rec + i) >> 32);
        count(i, LEARNED ? qg_cdf_bucket_h<true>(sm, hd, u) : qg_part_bucket(pf, u));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 512; i += blockDim.x)
        if ((&h[0][0])[i]) atomicAdd(&hist[i], (&h[0][0])[i]);
}

// After partitioning (rows in bucket order): beg[b] = first row whose bucket
// is >= b, for b in [0, nb]; one thread per bucket, binary search.
__global__ void k_pj_bounds(const unsigned long long *__restrict__ rec, long long n, qg_part_fn pf,
                            uint32_t nb, uint32_t *__restrict__ beg) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > nb) return;
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (qg_part_bucket(pf, (uint32_t)(__ldg(rec + mid) >> 32)) < b) lo = mid + 1;
        else hi = mid;
    }
    beg[b] = (uint32_t)lo;
}

// Bucket counts of the key sample under a partition function (global atomics;
// the sample has at most 2^20 keys).
// The sample is sorted, so neighbouring lanes mostly share a bucket: one add
// per bucket and warp (peers found by a match instruction) instead of one per
// key onto the same L2 word.  A learned function is evaluated from a
// shared-memory copy of the model.
template <bool LEARNED>
__global__ void __launch_bounds__(256)
k_pj_smp_hist(const unsigned long long *__restrict__ smp, long long m, qg_part_fn pf, uint32_t nb,
              uint32_t *__restrict__ counts) {
    __shared__ __align__(16) unsigned char sm_model[LEARNED ? sizeof(qg_cdf_model) : 16];
    if (LEARNED) {
        const uint32_t *gsrc = reinterpret_cast<const uint32_t *>(pf.model);
        uint32_t *sdst = reinterpret_cast<uint32_t *>(sm_model);
        for (int i = threadIdx.x; i < (int)(sizeof(qg_cdf_model) / 4); i += blockDim.x) sdst[i] = __ldg(gsrc + i);
        __syncthreads();
    }
    const qg_cdf_model *sm = reinterpret_cast<const qg_cdf_model *>(sm_model);
    qg_cdf_head hd{};
    if (LEARNED) hd = qg_cdf_load_head<true>(sm);
    const long long stride = (long long)gridDim.x * blockDim.x;
    // whole warps through every round, so the match sees all 32 lanes
    const long long m32 = (m + 31) & ~31ll;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m32; i += stride) {
        uint32_t b = 0xffffffffu;
        if (i < m) {
            const uint32_t u = (uint32_t)(__ldg(smp + i) >> 32);
            b = LEARNED ? qg_cdf_bucket_h<true>(sm, hd, u) : qg_part_bucket(pf, u);
            if (b >= nb) b = 0xffffffffu;
        }
        const uint32_t peers = __match_any_sync(QG_FULL_MASK, b);
        if (b != 0xffffffffu && (threadIdx.x & 31) == (uint32_t)(__ffs(peers) - 1))
            atomicAdd(&counts[b], (uint32_t)__popc(peers));
    }
}

// Sample m keys spread evenly over both inputs (proportionally to their
// sizes), as u64 items with the key in the high word for the radix sort.
__global__ void k_cdf_sample(const unsigned long long *__restrict__ r, long long nR,
                             const unsigned long long *__restrict__ s, long long nS, long long mR,
                             long long m, unsigned long long *__restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x) {
        unsigned long long v;
        if (i < mR) v = __ldg(r + (i * nR) / mR);
        else v = __ldg(s + ((i - mR) * nS) / (m - mR));
        out[i] = v & 0xffffffff00000000ull;
    }
}

__device__ __forceinline__ uint32_t smp_key(const unsigned long long *s, long long i) {
    return (uint32_t)(s[i] >> 32);
}
// First index with key >= u / > u in the sorted sample.
__device__ long long smp_lower(const unsigned long long *s, long long m, uint32_t u) {
    long long lo = 0, hi = m;
    while (lo < hi) {
        long long mid = (lo + hi) >> 1;
        if (smp_key(s, mid) < u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
__device__ long long smp_upper(const unsigned long long *s, long long m, uint32_t u) {
    long long lo = 0, hi = m;
    while (lo < hi) {
        long long mid = (lo + hi) >> 1;
        if (smp_key(s, mid) <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Training of the learned partition function from the sorted sample (one CTA).
//   knots: the keys at the 1025 sample quantiles i/1024, plus every key that
//          holds at least `hthr` sample entries (heavy), deduplicated;
//   bucket of a knot: floor(B * rank / m), rank = first sample index of the
//          knot's key (heavy keys: the middle of their run), so that buckets
//          are filled in proportion to the sample mass;
//   between knots: linear in the key with an fp32 slope, clamped so that the
//          function stays non-decreasing and a heavy key's bucket holds no
//          other key.
constexpr int FIT_THREADS = 1024;
constexpr int FIT_SORT = 2048;  // >= QG_CDF_MAX_KNOTS, power of two

// Heavy keys of the sorted sample: runs of at least hthr equal keys (the
// first QG_CDF_MAX_HEAVY found are kept; which ones, when there are more,
// changes only where rows are processed).  heavy[0] counts them, heavy[1..]
// holds them; heavy[0] is zero on entry.
__global__ void __launch_bounds__(256)
k_cdf_heavy(const unsigned long long *__restrict__ smp, long long m, long long hthr, uint32_t *__restrict__ heavy) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
        const uint32_t u = smp_key(smp, i);
        if (i > 0 && smp_key(smp, i - 1) == u) continue;
        if (i + hthr - 1 >= m || smp_key(smp, i + hthr - 1) != u) continue;
        const uint32_t h = atomicAdd(heavy, 1u);
        if (h < QG_CDF_MAX_HEAVY) heavy[1 + h] = u;
    }
}

__global__ void __launch_bounds__(FIT_THREADS)
k_cdf_fit(const unsigned long long *__restrict__ smp, long long m, uint32_t nb, long long hthr,
          const uint32_t *__restrict__ heavy, qg_cdf_model *__restrict__ model) {
    __shared__ uint32_t cand[FIT_SORT];
    __shared__ uint32_t ncand;
    __shared__ uint32_t s_heavy_n;
    const int tid = threadIdx.x;
    if (tid == 0) { ncand = 0; s_heavy_n = 0; }
    for (int i = tid; i < FIT_SORT; i += FIT_THREADS) cand[i] = 0xffffffffu;
    __syncthreads();
    // quantile knots
    for (int i = tid; i <= QG_CDF_SEGMENTS; i += FIT_THREADS) {
        const long long si = (long long)i * (m - 1) / QG_CDF_SEGMENTS;
        cand[i] = smp_key(smp, si);
    }
    if (tid == 0) ncand = QG_CDF_SEGMENTS + 1;
    __syncthreads();
    // heavy keys (k_cdf_heavy)
    if (tid == 0) s_heavy_n = heavy[0];
    __syncthreads();
    for (uint32_t h = tid; h < min(s_heavy_n, (uint32_t)QG_CDF_MAX_HEAVY); h += FIT_THREADS)
        cand[QG_CDF_SEGMENTS + 1 + h] = heavy[1 + h];
    __syncthreads();
    // bitonic sort of the candidates (unused entries are 0xffffffff and sort last)
    for (int k = 2; k <= FIT_SORT; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < FIT_SORT; i += FIT_THREADS) {
                const int l = i ^ j;
                if (l > i) {
                    const uint32_t a = cand[i], b = cand[l];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) { cand[i] = b; cand[l] = a; }
                }
            }
            __syncthreads();
        }
    }
    const uint32_t nreal = QG_CDF_SEGMENTS + 1 + min(s_heavy_n, (uint32_t)QG_CDF_MAX_HEAVY);
    // deduplicate: keep the first of each run (a real 0xffffffff key among the
    // first nreal entries is kept once)
    __shared__ uint32_t keep_idx[FIT_SORT];
    __shared__ uint32_t wsum[FIT_THREADS / 32];
    {
        // two entries per thread
        uint32_t f[2], c = 0;
        for (int q = 0; q < 2; q++) {
            const int i = tid * 2 + q;
            f[q] = (i < (int)nreal) && (i == 0 || cand[i] != cand[i - 1]);
            c += f[q];
        }
        uint32_t inc = c;
        const int lane = tid & 31, warp = tid >> 5;
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t x = __shfl_up_sync(QG_FULL_MASK, inc, d);
            if (lane >= d) inc += x;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        uint32_t off = 0, tot = 0;
        for (int w = 0; w < FIT_THREADS / 32; w++) {
            if (w < warp) off += wsum[w];
            tot += wsum[w];
        }
        uint32_t pos = off + inc - c;
        const uint32_t k0 = cand[tid * 2], k1 = cand[tid * 2 + 1];
        __syncthreads();
        if (f[0]) keep_idx[pos++] = k0;
        if (f[1]) keep_idx[pos++] = k1;
        if (tid == 0) ncand = tot;
    }
    __syncthreads();
    const uint32_t K = ncand;
    // per-knot bucket and heavy flag
    __shared__ uint32_t bk[QG_CDF_MAX_KNOTS];
    __shared__ uint8_t hv[QG_CDF_MAX_KNOTS];
    for (uint32_t i = tid; i < K; i += FIT_THREADS) {
        const uint32_t u = keep_idx[i];
        const long long lo = smp_lower(smp, m, u), hi = smp_upper(smp, m, u);
        const bool heavy = (hi - lo) >= hthr;
        const long long rank2 = heavy ? (lo + hi) : 2 * lo;  // twice the rank
        long long b = (long long)((unsigned long long)rank2 * nb / (2ull * (unsigned long long)m));
        if (b > (long long)nb - 1) b = nb - 1;
        bk[i] = (uint32_t)b;
        hv[i] = heavy;
        model->x[i] = u;
        model->bk[i] = (uint32_t)b;
    }
    __syncthreads();
    for (uint32_t i = tid; i < K; i += FIT_THREADS) {
        if (i + 1 < K) {
            const uint32_t x0 = keep_idx[i], x1 = keep_idx[i + 1];
            uint32_t lowB = bk[i] + (hv[i] ? 1u : 0u);
            uint32_t highB = hv[i + 1] ? (bk[i + 1] > 0 ? bk[i + 1] - 1u : 0u) : bk[i + 1];
            if (lowB > bk[i + 1]) lowB = bk[i + 1];
            if (highB < lowB) highB = lowB;
            const uint32_t inner = x1 - x0 - 1u;  // keys strictly between the knots
            model->b0[i] = lowB;
            model->b1[i] = highB;
            model->slope[i] = inner ? (float)(highB - lowB + 1u) / (float)inner : 0.0f;
        } else {
            model->b0[i] = bk[i];
            model->b1[i] = bk[i];
            model->slope[i] = 0.0f;
        }
    }
    // top-level index
    const uint32_t x0 = keep_idx[0], xl = keep_idx[K - 1];
    const uint32_t range = xl - x0;
    uint32_t ishift = 0;
    while ((range >> ishift) >= (uint32_t)QG_CDF_INDEX) ishift++;
    for (int t = tid; t <= QG_CDF_INDEX; t += FIT_THREADS) {
        const unsigned long long kt = (unsigned long long)x0 + ((unsigned long long)t << ishift);
        const uint32_t key = kt > xl ? xl : (uint32_t)kt;
        // largest knot index with x <= key
        uint32_t lo = 0, hi = K;  // first index with x > key
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (keep_idx[mid] <= key) lo = mid + 1;
            else hi = mid;
        }
        model->idx[t] = lo ? lo - 1 : 0;
    }
    if (tid == 0) {
        model->nknots = K;
        model->nbuckets = nb;
        model->ishift = ishift;
        model->nheavy = min(s_heavy_n, (uint32_t)QG_CDF_MAX_HEAVY);
    }
}

// Buckets of an array of keys under a partition function (for tests/tools).
__global__ void k_part_eval(const uint32_t *__restrict__ keys, long long n, qg_part_fn pf,
                            uint32_t *__restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = qg_part_bucket(pf, keys[i]);
}

// ---------------------------------------------------------------------------
// 4. per-bucket join (one CTA per bucket, tickets in bucket order)
// ---------------------------------------------------------------------------
constexpr int PB_THREADS = 512;
constexpr int PB_WARPS = PB_THREADS / 32;
constexpr int PB_SMAX = 4096;  // S' rows of a bucket held in shared memory
constexpr int PB_RMAX = 2048;  // R rows of a bucket
constexpr int PB_HEADS_LOG2 = 12;
constexpr int PB_HEADS = 1 << PB_HEADS_LOG2;
constexpr int PB_CSPAN = 8192;  // widest key span that is counting-sorted
static_assert(PB_CSPAN == (int)PJ_DENSE_BSPAN, "a dense group is counting-sorted");
constexpr int PB_IPT = PB_SMAX / PB_THREADS;
constexpr int PB_WSEG = PB_SMAX / PB_WARPS;  // sorted S' rows probed by one warp

struct PbSmem {
    unsigned long long s[PB_SMAX];  // the bucket's S' rows (key << 32 | S.payload), sorted by key
    uint32_t cnt[PB_CSPAN];         // counting-sort counters, then start offsets
    uint32_t rk[PB_RMAX];
    uint32_t rp[PB_RMAX];
    uint32_t head[PB_HEADS];        // 1 + first R row of each chain, 0 = empty
    uint32_t next[PB_RMAX];         // 1 + next R row of the chain, 0 = end
    uint32_t wsum[PB_WARPS];
    uint32_t red[2 * PB_WARPS];
    uint32_t tile, epoch, excl, total;
};

struct PbArgs {
    const unsigned long long *R;  // bucket-ordered R records
    const unsigned long long *S;  // bucket-ordered S' records
    const uint32_t *rbeg;         // [nb + 1]
    const uint32_t *sbeg;         // [nb + 1]
    const uint32_t *big;          // [nb] 1: handled outside, its count in bigcnt
    const unsigned long long *bigcnt;
    unsigned long long *off;      // [nb] output offset of each outside bucket (written)
    unsigned long long *total;    // output rows of all buckets (written by the last bucket)
    uint32_t *out_k, *out_a, *out_b;
    long long cap;
};

__device__ __forceinline__ uint32_t pb_hash(uint32_t k) {
    return (k * 0x9E3779B1u) >> (32 - PB_HEADS_LOG2);
}

// Exclusive prefix of v over the CTA in thread order; *total = sum.
template <int NW = PB_WARPS>
__device__ __forceinline__ uint32_t pb_excl(uint32_t v, uint32_t *wsum, uint32_t *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t x = __shfl_up_sync(QG_FULL_MASK, inc, d);
        if (lane >= d) inc += x;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    uint32_t off = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < NW; w++) {
        const uint32_t x = wsum[w];
        if (w < warp) off += x;
        tot += x;
    }
    __syncthreads();
    *total = tot;
    return off + inc - v;
}

__global__ void __launch_bounds__(PB_THREADS, 2)
k_pj_join(PbArgs a, qg_lookback lb) {
    extern __shared__ __align__(16) unsigned char pb_raw[];
    PbSmem &S = *reinterpret_cast<PbSmem *>(pb_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    qg_lb_begin(lb, &S.tile, &S.epoch);
    const uint32_t b = S.tile;
    const uint32_t rb = a.rbeg[b], rn = a.rbeg[b + 1] - rb;
    const uint32_t sb = a.sbeg[b], sn = a.sbeg[b + 1] - sb;
    const bool outside = a.big[b] != 0;
    bool work = !outside && rn > 0 && sn > 0;
    if (work && (rn > (uint32_t)PB_RMAX || sn > (uint32_t)PB_SMAX)) {  // the packing sends these outside
        if (tid == 0) qg_record_error(lb.ctl, QG_ERR_INVALID, QG_SITE_PJ_BUCKET);
        work = false;
    }
    // S' rows -> registers, each probed against R's chained table right away:
    // the group's output count is then known before any sorting and is
    // published at once (successors' look-backs wait less).  Only rows with
    // matches are sorted.
    unsigned long long it[PB_IPT];
    uint32_t cf[PB_IPT];  // per row: matches << 16 | 1 + first matching R row (0: none)
    uint32_t my_m = 0;
    uint32_t kmn = 0xffffffffu, kmx = 0;
    if (work) {
        for (uint32_t i = tid; i < PB_HEADS; i += PB_THREADS) S.head[i] = 0;
        for (uint32_t i = tid; i < rn; i += PB_THREADS) {
            const unsigned long long v = __ldg(a.R + rb + i);
            S.rk[i] = (uint32_t)(v >> 32);
            S.rp[i] = (uint32_t)v;
        }
#pragma unroll
        for (int j = 0; j < PB_IPT; j++) {
            const uint32_t i = j * PB_THREADS + tid;
            it[j] = i < sn ? __ldg(a.S + sb + i) : 0ull;
        }
        __syncthreads();
        for (uint32_t i = tid; i < rn; i += PB_THREADS)
            S.next[i] = atomicExch(&S.head[pb_hash(S.rk[i])], i + 1);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PB_IPT; j++) {
            cf[j] = 0;
            if (j * PB_THREADS + tid < sn) {
                const uint32_t k = (uint32_t)(it[j] >> 32);
                uint32_t m = 0, first = 0;
                for (uint32_t e = S.head[pb_hash(k)]; e; e = S.next[e - 1])
                    if (S.rk[e - 1] == k) {
                        first = m ? first : e;
                        m++;
                    }
                cf[j] = (m << 16) | first;
                my_m += m;
                if (m) {
                    kmn = min(kmn, k);
                    kmx = max(kmx, k);
                }
            }
        }
    }
    // the group's count (an outside group's comes from its own path) and the
    // matching rows' key range
    {
        const uint32_t wm = __reduce_add_sync(QG_FULL_MASK, my_m);
        const uint32_t wn = __reduce_min_sync(QG_FULL_MASK, kmn), wx = __reduce_max_sync(QG_FULL_MASK, kmx);
        if (lane == 0) {
            S.wsum[warp] = wm;
            S.red[warp] = wn;
            S.red[PB_WARPS + warp] = wx;
        }
    }
    __syncthreads();
    if (tid == 0) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < PB_WARPS; w++) t += S.wsum[w];
        S.total = outside ? (uint32_t)a.bigcnt[b] : t;
        qg_lb_publish_agg(lb, b, S.epoch, S.total);
    }
    kmn = 0xffffffffu;
    kmx = 0;
#pragma unroll
    for (int w = 0; w < PB_WARPS; w++) {
        kmn = min(kmn, S.red[w]);
        kmx = max(kmx, S.red[PB_WARPS + w]);
    }
    __syncthreads();  // S.wsum is read above and rewritten below
    uint32_t ns = 0;  // matching rows, sorted by key into S.s[0 .. ns)
    if (work) {
        uint32_t hit = 0;
#pragma unroll
        for (int j = 0; j < PB_IPT; j++) hit |= (cf[j] >> 16 ? 1u : 0u) << j;
        uint32_t nh = __popc(hit), tot;
        const uint32_t hoff = pb_excl(nh, S.wsum, &tot);  // this thread's first place among the matching rows
        ns = tot;
        const uint32_t span1 = kmx - kmn;  // key span of the matching rows, minus one (read when ns > 0)
        if (ns > 0 && span1 < (uint32_t)PB_CSPAN) {
            // counting sort by (key - kmn); the order among equal keys is free
            for (uint32_t i = tid; i <= span1; i += PB_THREADS) S.cnt[i] = 0;
            __syncthreads();
            uint32_t rk[PB_IPT];
#pragma unroll
            for (int j = 0; j < PB_IPT; j++)
                if ((hit >> j) & 1u) rk[j] = atomicAdd(&S.cnt[(uint32_t)(it[j] >> 32) - kmn], 1u);
            __syncthreads();
            constexpr int PER = PB_CSPAN / PB_THREADS;
            const uint32_t c0 = tid * PER;
            uint32_t sum = 0;
#pragma unroll
            for (int e = 0; e < PER; e++) sum += (c0 + e <= span1) ? S.cnt[c0 + e] : 0u;
            uint32_t t2;
            uint32_t run = pb_excl(sum, S.wsum, &t2);
#pragma unroll
            for (int e = 0; e < PER; e++) {
                if (c0 + e <= span1) {
                    const uint32_t c = S.cnt[c0 + e];
                    S.cnt[c0 + e] = run;
                    run += c;
                }
            }
            __syncthreads();
            uint32_t pos[PB_IPT];
#pragma unroll
            for (int j = 0; j < PB_IPT; j++)
                if ((hit >> j) & 1u) {
                    pos[j] = S.cnt[(uint32_t)(it[j] >> 32) - kmn] + rk[j];
                    S.s[pos[j]] = it[j];
                }
            __syncthreads();
            // the counters are dead: each sorted row keeps its count and first match there
#pragma unroll
            for (int j = 0; j < PB_IPT; j++)
                if ((hit >> j) & 1u) S.cnt[pos[j]] = cf[j];
        } else if (ns > 0) {
            // wide key span: bitonic sort of the matching rows (padded with
            // all-ones), then each sorted row is probed again for its matches
            uint32_t o = hoff;
#pragma unroll
            for (int j = 0; j < PB_IPT; j++)
                if ((hit >> j) & 1u) S.s[o++] = it[j];
            uint32_t P = 1;
            while (P < ns) P <<= 1;
            for (uint32_t i = ns + tid; i < P; i += PB_THREADS) S.s[i] = ~0ull;
            __syncthreads();
            for (uint32_t k = 2; k <= P; k <<= 1) {
                for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                    for (uint32_t i = tid; i < P; i += PB_THREADS) {
                        const uint32_t l = i ^ j;
                        if (l > i) {
                            const unsigned long long x = S.s[i], y = S.s[l];
                            if ((x > y) == ((i & k) == 0)) { S.s[i] = y; S.s[l] = x; }
                        }
                    }
                    __syncthreads();
                }
            }
            for (uint32_t r = tid; r < ns; r += PB_THREADS) {
                const uint32_t k = (uint32_t)(S.s[r] >> 32);
                uint32_t m = 0, first = 0;
                for (uint32_t e = S.head[pb_hash(k)]; e; e = S.next[e - 1])
                    if (S.rk[e - 1] == k) {
                        first = m ? first : e;
                        m++;
                    }
                S.cnt[r] = (m << 16) | first;
            }
        }
    }
    __syncthreads();
    // warp w writes the matches of sorted rows [w * PB_WSEG, ...), 32 at a time
    // (lane L has row step * 32 + L), so that a step's matches are consecutive
    // in the output and their stores coalesce
    const uint32_t r0 = min(ns, (uint32_t)warp * PB_WSEG);
    const uint32_t q = min(ns, r0 + PB_WSEG) - r0;
    uint32_t my_cnt = 0;
    for (uint32_t r = r0 + lane; r < r0 + q; r += 32) my_cnt += S.cnt[r] >> 16;
    const uint32_t wcnt = __reduce_add_sync(QG_FULL_MASK, my_cnt);
    uint32_t tot3;
    const uint32_t my_off = pb_excl(lane == 0 ? wcnt : 0u, S.wsum, &tot3);  // lane 0 holds its warp's offset
    const uint32_t warp_off = __shfl_sync(QG_FULL_MASK, my_off, 0);
    const uint32_t total = S.total;
    if (warp == 0) {
        const uint32_t excl = qg_lb_warp_lookback(lb, b, S.epoch, total);
        if (lane == 0) {
            S.excl = excl;
            if (b == gridDim.x - 1) *a.total = (unsigned long long)excl + total;
            if (outside) a.off[b] = excl;
        }
    }
    __syncthreads();
    if (work && wcnt) {  // warp-uniform
        long long o = (long long)S.excl + warp_off;  // output index of the warp's next step
        const uint32_t lt = qg_lanemask_lt();
        for (uint32_t s0 = r0; s0 < r0 + q; s0 += 32) {
            const uint32_t r = s0 + lane;
            unsigned long long v = 0;
            uint32_t k = 0, m = 0;
            uint32_t first = 0;
            if (r < r0 + q) {
                v = S.s[r];
                k = (uint32_t)(v >> 32);
                const uint32_t x = S.cnt[r];
                m = x >> 16;
                first = x & 0xffffu;
            }
            // exclusive prefix of the lanes' match counts (0 or 1 in the common case)
            uint32_t pre;
            if (__all_sync(QG_FULL_MASK, m <= 1u)) {
                pre = __popc(__ballot_sync(QG_FULL_MASK, m != 0u) & lt);
            } else {
                uint32_t inc = m;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t x = __shfl_up_sync(QG_FULL_MASK, inc, d);
                    if (lane >= d) inc += x;
                }
                pre = inc - m;
            }
            if (m) {
                long long oo = o + pre;
                for (uint32_t e = first; e; e = S.next[e - 1]) {
                    if (S.rk[e - 1] != k) continue;
                    if (oo < a.cap) {
                        a.out_k[oo] = k;
                        a.out_a[oo] = S.rp[e - 1];
                        a.out_b[oo] = (uint32_t)v;
                    }
                    oo++;
                }
            }
            o += __reduce_add_sync(QG_FULL_MASK, m);
        }
    }
    qg_lb_finish(lb, b, gridDim.x - 1, S.epoch);
}

// Dense build side (pj_dense_span, unique keys): one CTA per join group,
// tickets in group order.  (Persistent CTAs taking groups from a counter,
// launched without a host read of the group count, measured slower: 0.58
// against 0.48 ms on config 2; so did a persistent form that bulk-copied the
// next group's rows into a second shared-memory stage: 0.84 ms.)  A group is a key range [kmin + gk[g], kmin +
// gk[g + 1]) of at most PB_CSPAN keys with its S' rows [gs[g], gs[g + 1]).  A
// row matches when its key's presence bit is set, and then produces exactly
// one output row (key, T[key - kmin], S.payload).  So the group's output
// count is known as soon as its rows are loaded: it is published at once
// (successors' look-backs wait less), then the matching rows alone are
// counting-sorted by key in shared memory -- the sorted index of a row is its
// place in the group's output -- and, once the look-back has found the
// group's offset, written with consecutive addresses.
template <int SMAX, int NW>
struct PdSmem {
    unsigned long long s[SMAX];  // the group's matching S' rows, sorted by key
    uint32_t cnt[PB_CSPAN];      // counting-sort counters, then start offsets
    uint32_t red[NW];
    uint32_t wsum[NW];
    uint32_t tile, epoch, excl, total;
};

struct PdArgs {
    const unsigned long long *S;  // bucket-ordered S' records
    const uint32_t *gk, *gs;      // [G + 1] first key offset and first S' row of each group
    const uint32_t *bitmap;       // presence of each key offset (unless sent_ok)
    const uint32_t *T;            // R payload of each present key offset (sent_ok: `sent` where none)
    uint32_t kmin, sent_ok, sent;
    unsigned long long *total;    // output rows (written by the last group)
    uint32_t *out_k, *out_a, *out_b;
    long long cap;
};

// One group of the dense bucket kernels.  THREADS threads, at most SMAX S'
// rows per group (SMAX / THREADS per thread, in registers).  FULL: R's keys
// fill their whole span (a permutation of [kmin, kmax]), so every S' row
// matches (S' holds only keys of that span): the group's output starts at its
// first S' row, with no presence test and no look-back.  Otherwise the
// group's count is published as soon as its rows are loaded and its offset
// comes from the look-back (tickets in group order).
template <int THREADS, int SMAX, bool FULL>
__device__ __forceinline__ void pd_group(const PdArgs &a, const qg_lookback &lb, PdSmem<SMAX, THREADS / 32> &S,
                                         uint32_t g, uint32_t last) {
    constexpr int NW = THREADS / 32, IPT = SMAX / THREADS;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t sb = a.gs[g], sn = a.gs[g + 1] - sb;
    const uint32_t k0 = a.gk[g], span = a.gk[g + 1] - k0;
    bool work = sn > 0 && span > 0;
    if (work && (sn > (uint32_t)SMAX || span > (uint32_t)PB_CSPAN)) {  // the packing keeps groups within both
        if (tid == 0) qg_record_error(lb.ctl, QG_ERR_INVALID, QG_SITE_PJ_BUCKET);
        work = false;
    }
    const uint32_t base = a.kmin + k0;
    unsigned long long v[IPT];
    uint32_t pres = 0, np = 0;
    if (work) {
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            const uint32_t i = j * THREADS + tid;
            v[j] = i < sn ? __ldcs(a.S + sb + i) : 0ull;
        }
        for (uint32_t i = tid; i < span; i += THREADS) S.cnt[i] = 0;
#pragma unroll
        for (int j = 0; j < IPT; j++) {
            const uint32_t i = j * THREADS + tid;
            if (i < sn) {
                uint32_t p = 1u;
                if (!FULL) {
                    const uint32_t off = (uint32_t)(v[j] >> 32) - a.kmin;
                    p = a.sent_ok ? (uint32_t)(__ldg(a.T + off) != a.sent)
                                  : (__ldg(a.bitmap + (off >> 5)) >> (off & 31u)) & 1u;
                }
                pres |= p << j;
                np += p;
            }
        }
    }
    if (FULL) {
        if (tid == 0) S.total = work ? sn : 0u;
        __syncthreads();
    } else {
        np = __reduce_add_sync(QG_FULL_MASK, np);
        if (lane == 0) S.red[warp] = np;
        __syncthreads();
        if (tid == 0) {
            uint32_t t = 0;
#pragma unroll
            for (int w = 0; w < NW; w++) t += S.red[w];
            S.total = t;
            qg_lb_publish_agg(lb, g, S.epoch, t);
        }
    }
    if (work) {
        uint32_t rk[IPT];
#pragma unroll
        for (int j = 0; j < IPT; j++)
            if ((pres >> j) & 1u) rk[j] = atomicAdd(&S.cnt[(uint32_t)(v[j] >> 32) - base], 1u);
        __syncthreads();
        // exclusive scan of the counters: thread t owns PER consecutive ones
        constexpr int PER = PB_CSPAN / THREADS;
        const uint32_t c0 = tid * PER;
        uint32_t sum = 0;
#pragma unroll 8
        for (int e = 0; e < PER; e++) sum += (c0 + e < span) ? S.cnt[c0 + e] : 0u;
        uint32_t tot;
        uint32_t run = pb_excl<NW>(sum, S.wsum, &tot);
#pragma unroll 8
        for (int e = 0; e < PER; e++) {
            if (c0 + e < span) {
                const uint32_t c = S.cnt[c0 + e];
                S.cnt[c0 + e] = run;
                run += c;
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < IPT; j++)
            if ((pres >> j) & 1u) S.s[S.cnt[(uint32_t)(v[j] >> 32) - base] + rk[j]] = v[j];
    }
    __syncthreads();
    const uint32_t total = S.total;
    if (FULL) {
        if (tid == 0 && g == last) *a.total = (unsigned long long)a.gs[g + 1] - a.gs[0];
    } else if (warp == 0) {
        const uint32_t excl = qg_lb_warp_lookback(lb, g, S.epoch, total);
        if (lane == 0) {
            S.excl = excl;
            if (g == last) *a.total = (unsigned long long)excl + total;
        }
    }
    __syncthreads();
    const long long o = FULL ? (long long)(sb - a.gs[0]) : (long long)S.excl;
    for (uint32_t r = tid; r < total; r += THREADS) {
        const unsigned long long x = S.s[r];
        const long long oo = o + r;
        if (oo < a.cap) {
            const uint32_t k = (uint32_t)(x >> 32);
            a.out_k[oo] = k;
            a.out_a[oo] = __ldg(a.T + (k - a.kmin));
            a.out_b[oo] = (uint32_t)x;
        }
    }
}

// One CTA per group: tickets in group order with the look-back, or (FULL) in
// any order.  (Persistent CTAs taking the groups in turn -- by tickets, or
// statically for FULL, launched without a host read of the group count --
// measured slower on config 2: 0.58 against 0.48 ms, and 0.52 against 0.41
// ms; 0.57 ms with the largest shared-memory carveout, which leaves the
// bitmap and payload reads less L1.  A persistent form that bulk-copied the
// next group's rows into a second shared-memory stage took 0.84 ms.)
template <int THREADS, int SMAX, bool FULL>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS)
k_pj_join_dense(PdArgs a, qg_lookback lb) {
    extern __shared__ __align__(16) unsigned char pd_raw[];
    PdSmem<SMAX, THREADS / 32> &S = *reinterpret_cast<PdSmem<SMAX, THREADS / 32> *>(pd_raw);
    if (FULL) {
        pd_group<THREADS, SMAX, true>(a, lb, S, blockIdx.x, gridDim.x - 1);
    } else {
        qg_lb_begin(lb, &S.tile, &S.epoch);
        pd_group<THREADS, SMAX, false>(a, lb, S, S.tile, gridDim.x - 1);
        qg_lb_finish(lb, S.tile, gridDim.x - 1, S.epoch);
    }
}

// Group bounds of the dense build side in key offsets: the buckets' first key
// offsets min(b << shift, w) for b in [0, nb], where the packing reads an R
// "row count" (its key span) per bucket.
__global__ void k_pj_vbounds(uint32_t *__restrict__ rbk, uint32_t nb, int shift, unsigned long long w) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > nb) return;
    const unsigned long long x = (unsigned long long)b << shift;
    rbk[b] = (uint32_t)(x < w ? x : w);
}

// ---------------------------------------------------------------------------
// 5. buckets handled outside the bucket kernel
// ---------------------------------------------------------------------------
struct PjCross {  // a bucket with one key: every R row times every S' row
    uint32_t b, rb, rn, sb, sn;
};
struct PjMj {  // a bucket with several keys, joined by the sort-merge path
    uint32_t b, rb, rn, sb, sn;  // join group; its rows in the partitioned R and S'
    uint32_t roff, soff;         // its rows in the gathered arrays
};

// Join groups from the fine bucket bounds, on the device.  Thread t of CTA c
// packs the buckets of its segment (seg consecutive buckets) greedily:
// consecutive buckets join the open group while it holds at most rmax R rows
// and smax S' rows; a bucket above either limit is a group of its own,
// handled outside the bucket kernel (big = 1) and listed in `over` (b = its
// group) when both sides have rows.  A segment starts a new group, so no
// group spans two segments.  The greedy walk runs twice: once to count each
// segment's groups and listed buckets, then -- after the CTA's exclusive scan
// of the counts -- to write them into the CTA's staging region (span =
// PK_THREADS * seg entries per CTA); k_pj_place then moves every CTA's groups
// to their final places.  Bounds are read 8 buckets at a time with 16-byte
// loads, the next 8 in flight while these are walked (seg is a multiple of 8;
// rbk and sbk hold at least nb + 16 entries).  Several CTAs share the
// scattered reads, which bound this kernel on one SM.
struct PjPackCta {  // one pack CTA's totals
    uint32_t groups, over, most, pad;
    unsigned long long over_rows;
};
constexpr int PK_THREADS = 128;
constexpr int PK_SEG = 64;  // buckets per thread at most

struct PkWalk {
    uint32_t rmax, smax;
    bool open = false;
    uint32_t r0 = 0, s0 = 0, ng = 0, no = 0, most = 0;
    unsigned long long orows = 0;
    // write targets (null in the counting walk)
    uint32_t *gr = nullptr, *gs = nullptr, *big = nullptr;
    PjCross *over = nullptr;
    uint32_t gb = 0, ob = 0;

    __device__ void group(uint32_t re, uint32_t se, uint32_t b) {
        if (gr) {
            gr[gb + ng] = re;
            gs[gb + ng] = se;
            big[gb + ng] = b;
        }
        ng++;
    }
    __device__ void step(uint32_t rb, uint32_t re, uint32_t sb, uint32_t se) {
        if (re - rb > rmax || se - sb > smax) {
            if (open) { group(rb, sb, 0u); open = false; }
            if (re > rb && se > sb) {
                if (over) over[ob + no] = PjCross{ng, rb, re - rb, sb, se - sb};  // b: the CTA-local group
                no++;
                orows += (unsigned long long)(re - rb) + (se - sb);
                most = max(most, max(re - rb, se - sb));
            }
            group(re, se, 1u);
            return;
        }
        if (open && (re - r0 > rmax || se - s0 > smax)) { group(rb, sb, 0u); open = false; }
        if (!open) { r0 = rb; s0 = sb; open = true; }
    }
};

__device__ __forceinline__ void pk_load8(const uint32_t *p, uint32_t *v) {
    const uint4 a = __ldcg(reinterpret_cast<const uint4 *>(p));
    const uint4 b = __ldcg(reinterpret_cast<const uint4 *>(p + 4));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

__device__ void pk_walk(const uint32_t *__restrict__ rbk, const uint32_t *__restrict__ sbk, uint32_t b0,
                        uint32_t b1, PkWalk &w) {
    if (b0 >= b1) return;
    uint32_t rv[8], sv[8];
    pk_load8(rbk + b0, rv);
    pk_load8(sbk + b0, sv);
    for (uint32_t c = b0; c < b1; c += 8) {
        uint32_t rn[8], sn[8];  // the next 8 starts (the first is this chunk's last end)
        pk_load8(rbk + c + 8, rn);
        pk_load8(sbk + c + 8, sn);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (c + j >= b1) break;
            const uint32_t re = j < 7 ? rv[j + 1] : rn[0], se = j < 7 ? sv[j + 1] : sn[0];
            w.step(rv[j], re, sv[j], se);
        }
#pragma unroll
        for (int j = 0; j < 8; j++) { rv[j] = rn[j]; sv[j] = sn[j]; }
    }
    if (w.open) { w.group(rbk[b1], sbk[b1], 0u); w.open = false; }
}

__global__ void __launch_bounds__(PK_THREADS)
k_pj_pack(const uint32_t *__restrict__ rbk, const uint32_t *__restrict__ sbk, uint32_t nb, uint32_t seg,
          uint32_t rmax, uint32_t smax, uint32_t *__restrict__ tgr, uint32_t *__restrict__ tgs,
          uint32_t *__restrict__ tbig, PjCross *__restrict__ tover, PjPackCta *__restrict__ cta) {
    constexpr int W = PK_THREADS / 32;
    __shared__ uint32_t s_g[W], s_o[W], s_m[W];
    __shared__ unsigned long long s_r[W];
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t span = PK_THREADS * seg, cbase = blockIdx.x * span;
    const uint32_t b0 = min(nb, cbase + t * seg), b1 = min(nb, b0 + seg);
    PkWalk w;
    w.rmax = rmax;
    w.smax = smax;
    pk_walk(rbk, sbk, b0, b1, w);
    const uint32_t ng = w.ng, no = w.no;
    uint32_t ig = ng, io = no;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t xg = __shfl_up_sync(QG_FULL_MASK, ig, d), xo = __shfl_up_sync(QG_FULL_MASK, io, d);
        if (lane >= d) { ig += xg; io += xo; }
    }
    unsigned long long wr = w.orows;
    uint32_t wm = w.most;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        wr += __shfl_xor_sync(QG_FULL_MASK, wr, d);
        wm = max(wm, __shfl_xor_sync(QG_FULL_MASK, wm, d));
    }
    if (lane == 31) { s_g[warp] = ig; s_o[warp] = io; }
    if (lane == 0) { s_r[warp] = wr; s_m[warp] = wm; }
    __syncthreads();
    uint32_t gw = 0, ow = 0;  // exclusive offsets of this warp
    if (t == 0) {
        uint32_t G = 0, O = 0, M = 0;
        unsigned long long Rw = 0;
        for (int i = 0; i < W; i++) {
            G += s_g[i];
            O += s_o[i];
            M = max(M, s_m[i]);
            Rw += s_r[i];
        }
        cta[blockIdx.x] = PjPackCta{G, O, M, 0u, Rw};
    }
    for (uint32_t i = 0; i < warp; i++) { gw += s_g[i]; ow += s_o[i]; }
    PkWalk v;
    v.rmax = rmax;
    v.smax = smax;
    v.gr = tgr;
    v.gs = tgs;
    v.big = tbig;
    v.over = tover;
    v.gb = cbase + gw + ig - ng;
    v.ob = cbase + ow + io - no;
    const uint32_t lg = gw + ig - ng;  // CTA-local index of this segment's first group
    pk_walk(rbk, sbk, b0, b1, v);
    // the listed buckets' group indices are segment-local so far: make them CTA-local
    for (uint32_t j = 0; j < no; j++) tover[v.ob + j].b += lg;
}

// Moves each pack CTA's staged groups and listed buckets to their final
// places (CTA c of this grid moves pack CTA c's): gr/gs[0 .. G] bound the
// groups, big/bigcnt[0 .. G) describe them (bigcnt zeroed), `over` lists the
// buckets handled outside, and *out gets the totals.
__global__ void __launch_bounds__(256)
k_pj_place(const uint32_t *__restrict__ rbk, const uint32_t *__restrict__ sbk, uint32_t nb, uint32_t span,
           const uint32_t *__restrict__ tgr, const uint32_t *__restrict__ tgs, const uint32_t *__restrict__ tbig,
           const PjCross *__restrict__ tover, const PjPackCta *__restrict__ cta, uint32_t *__restrict__ gr,
           uint32_t *__restrict__ gs, uint32_t *__restrict__ big, unsigned long long *__restrict__ bigcnt,
           PjCross *__restrict__ over, PjPackOut *__restrict__ out) {
    const uint32_t c = blockIdx.x;
    uint32_t gb = 0, ob = 0;
    for (uint32_t i = 0; i < c; i++) { gb += cta[i].groups; ob += cta[i].over; }
    const uint32_t ng = cta[c].groups, no = cta[c].over;
    const uint32_t src = c * span;
    for (uint32_t i = threadIdx.x; i < ng; i += blockDim.x) {
        gr[gb + i + 1] = tgr[src + i];
        gs[gb + i + 1] = tgs[src + i];
        big[gb + i] = tbig[src + i];
        bigcnt[gb + i] = 0ull;
    }
    for (uint32_t i = threadIdx.x; i < no; i += blockDim.x) {
        PjCross e = tover[src + i];
        e.b += gb;
        over[ob + i] = e;
    }
    if (c == gridDim.x - 1 && threadIdx.x == 0) {
        uint32_t most = 0;
        unsigned long long rows = 0;
        for (uint32_t i = 0; i < gridDim.x; i++) {
            most = max(most, cta[i].most);
            rows += cta[i].over_rows;
        }
        out->groups = gb + ng;
        out->over = ob + no;
        out->over_rows = rows;
        out->most = most;
        gr[0] = nb ? rbk[0] : 0u;
        gs[0] = nb ? sbk[0] : 0u;
    }
}

// Output rows of the cross-product buckets, for the bucket kernel's look-back.
__global__ void k_pj_cross_cnt(const PjCross *__restrict__ list, uint32_t nlist,
                               unsigned long long *__restrict__ bigcnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nlist; i += gridDim.x * blockDim.x)
        bigcnt[list[i].b] = (unsigned long long)list[i].rn * list[i].sn;
}

// blockIdx.y walks the list (nlist entries) with stride gridDim.y.
__global__ void k_pj_cross(const PjCross *__restrict__ list, uint32_t nlist, const unsigned long long *__restrict__ R,
                           const unsigned long long *__restrict__ S, const unsigned long long *__restrict__ off,
                           uint32_t *__restrict__ ok, uint32_t *__restrict__ oa, uint32_t *__restrict__ ob,
                           long long cap) {
    for (uint32_t y = blockIdx.y; y < nlist; y += gridDim.y) {
        const PjCross e = list[y];
        const unsigned long long m = (unsigned long long)e.rn * e.sn;
        const unsigned long long base = off[e.b];
        for (unsigned long long o = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; o < m;
             o += (unsigned long long)gridDim.x * blockDim.x) {
            const unsigned long long g = base + o;
            if (g >= (unsigned long long)cap) break;
            const unsigned long long si = o / e.rn, rj = o - si * e.rn;
            const unsigned long long sv = __ldg(S + e.sb + si), rv = __ldg(R + e.rb + rj);
            ok[g] = (uint32_t)(sv >> 32);
            oa[g] = (uint32_t)rv;
            ob[g] = (uint32_t)sv;
        }
    }
}

// Sort-merge path for the oversize buckets with several keys, all of them in
// a fixed number of launches.  Their rows are gathered into Rb / Sb in bucket
// order and sorted by key there; the buckets are disjoint key ranges in
// ascending order, so every bucket keeps its own segment.  blockIdx.y is the
// bucket.
__global__ void k_pj_mj_gather(const PjMj *__restrict__ list, uint32_t nlist, const unsigned long long *__restrict__ R,
                               const unsigned long long *__restrict__ S, unsigned long long *__restrict__ Rb,
                               unsigned long long *__restrict__ Sb) {
    for (uint32_t y = blockIdx.y; y < nlist; y += gridDim.y) {
        const PjMj e = list[y];
        const uint32_t m = max(e.rn, e.sn);
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
            if (i < e.rn) Rb[e.roff + i] = __ldg(R + e.rb + i);
            if (i < e.sn) Sb[e.soff + i] = __ldg(S + e.sb + i);
        }
    }
}

// Per S row: its matching R rows [lob, lob + cnt) in the bucket's key-sorted
// R segment; the bucket's match count is added to bigcnt[b] (64-bit) for the
// bucket kernel's look-back and to *tot for the host.
__global__ void __launch_bounds__(256)
k_pj_mj_count(const PjMj *__restrict__ list, uint32_t nlist, const unsigned long long *__restrict__ Rb,
              const unsigned long long *__restrict__ Sb, uint32_t *__restrict__ cnt, uint32_t *__restrict__ lob,
              unsigned long long *__restrict__ bigcnt, unsigned long long *__restrict__ tot) {
    __shared__ unsigned long long red[8];
    for (uint32_t y = blockIdx.y; y < nlist; y += gridDim.y) {
    const PjMj e = list[y];
    unsigned long long my = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < e.sn; i += gridDim.x * blockDim.x) {
        const uint32_t k = (uint32_t)(__ldg(Sb + e.soff + i) >> 32);
        uint32_t lo = 0, hi = e.rn;  // first R row with key >= k
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if ((uint32_t)(__ldg(Rb + e.roff + mid) >> 32) < k) lo = mid + 1;
            else hi = mid;
        }
        uint32_t up = lo, h2 = e.rn;  // first R row with key > k
        while (up < h2) {
            const uint32_t mid = (up + h2) >> 1;
            if ((uint32_t)(__ldg(Rb + e.roff + mid) >> 32) <= k) up = mid + 1;
            else h2 = mid;
        }
        cnt[e.soff + i] = up - lo;
        lob[e.soff + i] = e.roff + lo;
        my += up - lo;
    }
    for (int d = 16; d > 0; d >>= 1) my += __shfl_down_sync(QG_FULL_MASK, my, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = my;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        if (t) {
            atomicAdd(bigcnt + e.b, t);
            atomicAdd(tot, t);
        }
    }
    __syncthreads();  // red is reused by the next entry
    }
}

// Matches of each S row at off[b] + (its exclusive prefix within the bucket):
// S rows in key order, so the bucket's output is in key order.
__global__ void k_pj_mj_write(const PjMj *__restrict__ list, uint32_t nlist, const unsigned long long *__restrict__ Rb,
                              const unsigned long long *__restrict__ Sb, const uint32_t *__restrict__ cnt,
                              const uint32_t *__restrict__ lob, const uint32_t *__restrict__ pre,
                              const unsigned long long *__restrict__ off, uint32_t *__restrict__ ok,
                              uint32_t *__restrict__ oa, uint32_t *__restrict__ ob, long long cap) {
    for (uint32_t y = blockIdx.y; y < nlist; y += gridDim.y) {
    const PjMj e = list[y];
    const unsigned long long base = off[e.b];
    const uint32_t p0 = __ldg(pre + e.soff);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < e.sn; i += gridDim.x * blockDim.x) {
        const uint32_t c = cnt[e.soff + i];
        if (!c) continue;
        const unsigned long long sv = __ldg(Sb + e.soff + i);
        const uint32_t l = lob[e.soff + i];
        unsigned long long g = base + (uint32_t)(pre[e.soff + i] - p0);  // 32-bit wrap-safe difference
        for (uint32_t j = 0; j < c && g < (unsigned long long)cap; j++, g++) {
            ok[g] = (uint32_t)(sv >> 32);
            oa[g] = (uint32_t)__ldg(Rb + l + j);
            ob[g] = (uint32_t)sv;
        }
    }
    }
}

// Key range of each listed bucket over its R and S' rows: mn[i], mx[i]
// (preset to 0xffffffff and 0).  Several CTAs share a bucket (blockIdx.x),
// so that a heavy key's bucket of millions of rows is not one CTA's scan;
// blockIdx.y walks the list with stride gridDim.y.
__global__ void __launch_bounds__(256)
k_pj_minmax(const PjCross *__restrict__ list, uint32_t nlist, const unsigned long long *__restrict__ R,
            const unsigned long long *__restrict__ S, uint32_t *__restrict__ mn_out, uint32_t *__restrict__ mx_out) {
    __shared__ uint32_t red[2 * 8];
    for (uint32_t y = blockIdx.y; y < nlist; y += gridDim.y) {
        const PjCross e = list[y];
        uint32_t mn = 0xffffffffu, mx = 0;
        const uint32_t stride = gridDim.x * blockDim.x;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < e.rn; i += stride) {
            const uint32_t k = (uint32_t)(__ldg(R + e.rb + i) >> 32);
            mn = min(mn, k);
            mx = max(mx, k);
        }
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < e.sn; i += stride) {
            const uint32_t k = (uint32_t)(__ldg(S + e.sb + i) >> 32);
            mn = min(mn, k);
            mx = max(mx, k);
        }
        mn = __reduce_min_sync(QG_FULL_MASK, mn);
        mx = __reduce_max_sync(QG_FULL_MASK, mx);
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) { red[w] = mn; red[8 + w] = mx; }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int i = 1; i < (int)(blockDim.x >> 5); i++) {
                mn = min(mn, red[i]);
                mx = max(mx, red[8 + i]);
            }
            if (mn != 0xffffffffu) atomicMin(mn_out + y, mn);
            if (mx != 0) atomicMax(mx_out + y, mx);
        }
        __syncthreads();  // red is reused by the next entry
    }
}

}  // namespace

// ===========================================================================
// host
// ===========================================================================
qg_status qg_join_hash_sort(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay, int64_t nR,
                            const int32_t *skey, const int32_t *spay, int64_t nS, int32_t slo,
                            int32_t shi, int32_t *out_key, int32_t *out_rpay, int32_t *out_spay,
                            int64_t cap, int64_t *out_n);

namespace {

int g_pj_variant = 0;  // 0 auto (radix; learned when a key sample shows that it spreads the rows better), 1 radix, 2 learned, 3 hash join + sort
int g_pj_blog2 = 0;    // 0: fine bucket count from the input size
uint32_t g_pj_smax = PB_SMAX, g_pj_rmax = PB_RMAX;
bool g_pj_dense = true;  // the dense build side where it applies (unique R keys over a dense span)
constexpr long long CDF_SAMPLE = 1 << 20;  // keys sampled to fit (and assess) the learned model

struct PjLevel {
    PjRange *range;
    uint32_t *dh;          // [side R, S'][digit 0, 1][256]
    uint32_t *rbk, *sbk;   // [nb + 1] first row of each fine bucket (room for nb + 16)
    uint32_t *gr, *gs;     // [nb + 1] first row of each join group
    uint32_t *big, *mm;    // [nb] group handled outside the bucket kernel; [2 nb] key ranges
    uint32_t *scnt;        // [2 nb] sample counts under radix, learned
    unsigned long long *bigcnt, *off, *total;
    PjCross *cross;
    PjMj *mj;
    unsigned long long *mjtot;  // matches of the sort-merge buckets
    PjPackOut *pk;              // the packing's counts
    uint32_t *dflags;           // [PJ_F_WORDS] flags of the dense build side (set by k_pj_range_init)
    PjPackCta *pkc;             // [nb / (PK_THREADS * 8) + 1] the pack CTAs' totals
    uint32_t *tg;               // [3][nb + PK_THREADS * PK_SEG] the packing's staging (group ends, flags)
    PjCross *tover;             // [nb + PK_THREADS * PK_SEG] the packing's staging (listed buckets)
    qg_cdf_model *model;             // learned model (top level only)
    uint32_t *heavy;                 // [1 + QG_CDF_MAX_HEAVY] heavy keys of the sample
    unsigned long long *smp, *smp2;  // key sample (top level only)
};

size_t pj_level_bytes(uint32_t nb, bool learned) {
    size_t b = 0;
    auto add = [&](size_t x) { b += qg_align_up(x, 256); };
    add(sizeof(PjRange));
    add(4 * 256 * 4);
    for (int i = 0; i < 4; i++) add((size_t)(nb + 16) * 4);  // the packing reads bounds 8 ahead
    add((size_t)nb * 4);
    add((size_t)2 * nb * 4);
    add((size_t)2 * nb * 4);
    add((size_t)nb * 8);
    add((size_t)nb * 8);
    add(8);
    add((size_t)nb * sizeof(PjCross));
    add((size_t)nb * sizeof(PjMj));
    add(8);
    add(sizeof(PjPackOut));
    add(PJ_F_WORDS * 4);
    add(((size_t)nb / (PK_THREADS * 8) + 1) * sizeof(PjPackCta));
    add((size_t)3 * (nb + PK_THREADS * PK_SEG) * 4);
    add((size_t)(nb + PK_THREADS * PK_SEG) * sizeof(PjCross));
    if (learned) {
        add(sizeof(qg_cdf_model));
        add((size_t)(1 + QG_CDF_MAX_HEAVY) * 4);
        add((size_t)CDF_SAMPLE * 8);
        add((size_t)CDF_SAMPLE * 8);
    }
    return b;
}

void pj_level_carve(char *p, uint32_t nb, bool learned, PjLevel *L) {
    auto take = [&](size_t x) { char *q = p; p += qg_align_up(x, 256); return q; };
    L->range = (PjRange *)take(sizeof(PjRange));
    L->dh = (uint32_t *)take(4 * 256 * 4);
    L->rbk = (uint32_t *)take((size_t)(nb + 16) * 4);
    L->sbk = (uint32_t *)take((size_t)(nb + 16) * 4);
    L->gr = (uint32_t *)take((size_t)(nb + 16) * 4);
    L->gs = (uint32_t *)take((size_t)(nb + 16) * 4);
    L->big = (uint32_t *)take((size_t)nb * 4);
    L->mm = (uint32_t *)take((size_t)2 * nb * 4);
    L->scnt = (uint32_t *)take((size_t)2 * nb * 4);
    L->bigcnt = (unsigned long long *)take((size_t)nb * 8);
    L->off = (unsigned long long *)take((size_t)nb * 8);
    L->total = (unsigned long long *)take(8);
    L->cross = (PjCross *)take((size_t)nb * sizeof(PjCross));
    L->mj = (PjMj *)take((size_t)nb * sizeof(PjMj));
    L->mjtot = (unsigned long long *)take(8);
    L->pk = (PjPackOut *)take(sizeof(PjPackOut));
    L->dflags = (uint32_t *)take(PJ_F_WORDS * 4);
    L->pkc = (PjPackCta *)take(((size_t)nb / (PK_THREADS * 8) + 1) * sizeof(PjPackCta));
    L->tg = (uint32_t *)take((size_t)3 * (nb + PK_THREADS * PK_SEG) * 4);
    L->tover = (PjCross *)take((size_t)(nb + PK_THREADS * PK_SEG) * sizeof(PjCross));
    L->model = nullptr;
    L->heavy = nullptr;
    L->smp = L->smp2 = nullptr;
    if (learned) {
        L->model = (qg_cdf_model *)take(sizeof(qg_cdf_model));
        L->heavy = (uint32_t *)take((size_t)(1 + QG_CDF_MAX_HEAVY) * 4);
        L->smp = (unsigned long long *)take((size_t)CDF_SAMPLE * 8);
        L->smp2 = (unsigned long long *)take((size_t)CDF_SAMPLE * 8);
    }
}

// Grow-only device buffer of the context (the sort-merge arrays).
qg_status pj_pool_get(qg_ctx *ctx, char **slot, size_t *slot_bytes, size_t bytes, char **out) {
    bytes = qg_align_up(bytes ? bytes : 256, 256);
    if (bytes > *slot_bytes) {
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        if (*slot) cudaFree(*slot);
        *slot = nullptr;
        *slot_bytes = 0;
        if (cudaMalloc((void **)slot, bytes + bytes / 4) != cudaSuccess) {
            cudaGetLastError();
            *slot = nullptr;
            return QG_ERR_OOM;
        }
        *slot_bytes = bytes + bytes / 4;
    }
    *out = *slot;
    return QG_OK;
}

int g_pd_ctas_per_sm = 1;  // resident CTAs of k_pj_join_dense per SM

qg_status pj_attrs(qg_ctx *ctx) {
    static bool done = false;
    if (!done) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_pj_join, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PbSmem)), "attr join");
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_pj_join_dense<PB_THREADS, PB_SMAX, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sizeof(PdSmem<PB_SMAX, PB_WARPS>)), "attr join dense");
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_pj_join_dense<PB_THREADS, PB_SMAX, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sizeof(PdSmem<PB_SMAX, PB_WARPS>)), "attr join dense");
        int occ = 0;
        QG_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_pj_join_dense<PB_THREADS, PB_SMAX, false>,
                                                                       PB_THREADS, sizeof(PdSmem<PB_SMAX, PB_WARPS>)), "occupancy");
        g_pd_ctas_per_sm = occ > 0 ? occ : 1;
        done = true;
    }
    return QG_OK;
}

int pj_grid(qg_ctx *ctx, long long work, int per_block, int per_sm) {
    long long b = (work + per_block - 1) / per_block;
    const long long c = (long long)ctx->sm_count * per_sm;
    if (b > c) b = c;
    if (b < 1) b = 1;
    return (int)b;
}

// Digit histograms of both sides' bucket ids into h[0 .. 1024) (synchronises);
// with bid_r / bid_s set, every row's bucket id is also written there.
qg_status pj_dhist(qg_ctx *ctx, const PjLevel &L, const qg_part_fn &pf, uint32_t nb,
                   const unsigned long long *r, long long nR, const unsigned long long *s, long long nS,
                   uint32_t *h, uint16_t *bid_r = nullptr, uint16_t *bid_s = nullptr) {
    QG_TRY_CUDA(ctx, cudaMemsetAsync(L.dh, 0, 4 * 256 * 4, ctx->stream), "memset dhist");
    qg_pre_launch(ctx);
    auto kern = pf.learned ? k_pj_dhist<true> : k_pj_dhist<false>;
    kern<<<pj_grid(ctx, nR, 256, 8), 256, 0, ctx->stream>>>(r, nR, pf, nb, L.dh, ctx->ctl, bid_r, nullptr, 0);
    QG_TRY(qg_check_launch(ctx, "k_pj_dhist"));
    qg_pre_launch(ctx);
    kern<<<pj_grid(ctx, nS, 256, 8), 256, 0, ctx->stream>>>(s, nS, pf, nb, L.dh + 512, ctx->ctl, bid_s, nullptr, 0);
    QG_TRY(qg_check_launch(ctx, "k_pj_dhist"));
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(h, L.dh, 4 * 256 * 4, cudaMemcpyDeviceToHost, ctx->stream), "dhist d2h");
    return qg_collect_error(ctx);  // synchronises: h is filled
}

// Fit the learned model on a sample of both sides' keys (records); the
// sorted sample stays in L.smp (m keys).
qg_status pj_train(qg_ctx *ctx, const PjLevel &L, uint32_t nb, const unsigned long long *r, long long nR,
                   const unsigned long long *s, long long nS, long long *m_out) {
    const long long n = nR + nS;
    const long long m = n < CDF_SAMPLE ? n : CDF_SAMPLE;
    long long mR = nR ? (m * nR) / n : 0;
    if (nR && mR < 1) mR = 1;
    if (nS && mR >= m) mR = m - 1;
    qg_pre_launch(ctx);
    k_cdf_sample<<<pj_grid(ctx, m, 256, 4), 256, 0, ctx->stream>>>(r, nR, s, nS, mR, m, L.smp);
    QG_TRY(qg_check_launch(ctx, "k_cdf_sample"));
    QG_TRY(qg_sort_rec_inplace(ctx, L.smp, L.smp2, m));
    long long hthr = (3 * m + nb - 1) / nb;
    if (hthr < 2) hthr = 2;
    QG_TRY_CUDA(ctx, cudaMemsetAsync(L.heavy, 0, 4, ctx->stream), "memset heavy");
    qg_pre_launch(ctx);
    k_cdf_heavy<<<pj_grid(ctx, m, 256, 4), 256, 0, ctx->stream>>>(L.smp, m, hthr, L.heavy);
    QG_TRY(qg_check_launch(ctx, "k_cdf_heavy"));
    qg_pre_launch(ctx);
    k_cdf_fit<<<1, FIT_THREADS, 0, ctx->stream>>>(L.smp, m, nb, hthr, L.heavy, L.model);
    QG_TRY(qg_check_launch(ctx, "k_cdf_fit"));
    *m_out = m;
    return QG_OK;
}

// Rows (estimated from the sample) that would land in buckets larger than the
// bucket kernel takes, for each function: the comparison between radix and learned.
qg_status pj_compare(qg_ctx *ctx, const PjLevel &L, long long m, long long ntot, const qg_part_fn &radix,
                   uint32_t nb_radix, const qg_part_fn &learned, uint32_t nb, double *over_radix,
                   double *over_learned) {
    QG_TRY_CUDA(ctx, cudaMemsetAsync(L.scnt, 0, (size_t)2 * nb * 4, ctx->stream), "memset scnt");
    qg_pre_launch(ctx);
    k_pj_smp_hist<false><<<pj_grid(ctx, m, 256, 4), 256, 0, ctx->stream>>>(L.smp, m, radix, nb_radix, L.scnt);
    QG_TRY(qg_check_launch(ctx, "k_pj_smp_hist"));
    qg_pre_launch(ctx);
    auto kl = learned.learned ? k_pj_smp_hist<true> : k_pj_smp_hist<false>;
    kl<<<pj_grid(ctx, m, 256, 4), 256, 0, ctx->stream>>>(L.smp, m, learned, nb, L.scnt + nb);
    QG_TRY(qg_check_launch(ctx, "k_pj_smp_hist"));
    std::vector<uint32_t> c((size_t)2 * nb);
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(c.data(), L.scnt, c.size() * 4, cudaMemcpyDeviceToHost, ctx->stream), "scnt d2h");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    const double scale = (double)ntot / (double)m;
    const double lim = 0.8 * (double)(g_pj_smax + g_pj_rmax);
    double o[2] = {0, 0};
    for (int f = 0; f < 2; f++)
        for (uint32_t b = 0; b < (f ? nb : nb_radix); b++) {
            const double est = c[(size_t)f * nb + b] * scale;
            if (est > lim) o[f] += est;
        }
    *over_radix = o[0];
    *over_learned = o[1];
    return QG_OK;
}

// Pinned host staging of one join's reads (grow-once, sized for the largest
// bucket count): the digit histograms, the packing's counts, the list of
// oversize buckets and their key ranges.  Every call ends with a stream sync,
// so the next call may overwrite it.
struct PjPin {
    uint32_t h[1024];                 // [side R, S'][digit 0, 1][256]
    uint32_t dflags[PJ_F_WORDS];
    PjPackOut pk;
    PjCross over[PJ_MAX_BUCKETS];
    uint32_t mm[2 * PJ_MAX_BUCKETS];  // [mins][maxes] of the listed buckets
};

qg_status pj_pin(qg_ctx *ctx, PjPin **out) {
    if (!ctx->pin_join) {
        if (cudaMallocHost(&ctx->pin_join, sizeof(PjPin)) != cudaSuccess) {
            cudaGetLastError();
            ctx->pin_join = nullptr;
            return QG_ERR_OOM;
        }
    }
    *out = (PjPin *)ctx->pin_join;
    return QG_OK;
}

// Fine bucket count (a power of two, at most 2^16) for nR build rows and at
// most nS probe rows: buckets of about a quarter of the bucket kernel's
// capacity, which the packing then joins into groups.  It is taken from the
// S row count before the filter, so that the filter can count the partition
// digits of the rows it keeps.
uint32_t pj_bucket_count(long long nR, long long nS) {
    if (g_pj_blog2 > 0) return 1u << g_pj_blog2;
    const long long ntot = nR + nS;
    uint32_t nb = 1u;
    while (nb < (uint32_t)PJ_MAX_BUCKETS &&
           ((long long)nb * 1024 < ntot || (long long)nb * (g_pj_smax / 4) < nS || (long long)nb * (g_pj_rmax / 4) < nR))
        nb <<= 1;
    return nb;
}

// R's build side when R was not turned into records before the first read
// (dense span): its records and radix digit histograms now (one more read).
struct PjRSide {
    const int32_t *rkey, *rpay;
    bool rec_ready;       // R records (and h[0 .. 512)) exist
    bool dense_ok;        // dense span, no duplicate key: bitmap (or the sentinel) and T describe R
    bool sent_ok;         // T holds `sent` where no R row is (no bitmap)
    uint32_t sent;
    const uint32_t *bitmap, *T;
};

// Partition, join groups, outside buckets.  L: the level's arrays (carved for
// nb = 2^lb2 buckets); pin->h: the radix digit histograms of both sides (R's
// only when R's records exist), read with the S' count.
qg_status pj_core(qg_ctx *ctx, const PjLevel &L, PjPin *pin, uint32_t nb, int lb2, PjRSide &rs,
                  unsigned long long *r, unsigned long long *rsp, long long nR, unsigned long long *s,
                  unsigned long long *ssp, long long nS, uint32_t kmin, uint32_t kmax, int variant, uint32_t *ok,
                  uint32_t *oa, uint32_t *ob, long long cap, long long *M_out) {
    *M_out = 0;
    if (nR == 0 || nS == 0) return QG_OK;
    QG_TRY(pj_attrs(ctx));
    const long long ntot = nR + nS;
    const PjRadix rp = pj_radix(kmin, kmax, lb2);
    const uint32_t nb_radix = rp.nb;
    const bool may_learn = variant != 1;
    const qg_part_fn radix{0, kmin, rp.shift, nullptr};
    const qg_part_fn learned{1, 0u, 0, L.model};
    uint32_t *h = pin->h;
    auto ensure_rrec = [&]() -> qg_status {
        if (rs.rec_ready) return QG_OK;
        QG_TRY_CUDA(ctx, cudaMemsetAsync(L.dh, 0, 512 * 4, ctx->stream), "memset dhist");
        qg_pre_launch(ctx);
        k_pj_rrec<<<pj_grid(ctx, nR, 256, 8), 256, 0, ctx->stream>>>(rs.rkey, rs.rpay, nR, r, L.range);
        QG_TRY(qg_check_launch(ctx, "k_pj_rrec"));
        qg_pre_launch(ctx);
        k_pj_dhist<false><<<pj_grid(ctx, nR, 256, 8), 256, 0, ctx->stream>>>(r, nR, radix, nb_radix, L.dh, ctx->ctl,
                                                                            nullptr, nullptr, 0);
        QG_TRY(qg_check_launch(ctx, "k_pj_dhist"));
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(h, L.dh, 512 * 4, cudaMemcpyDeviceToHost, ctx->stream), "dhist d2h");
        QG_TRY(qg_collect_error(ctx));
        rs.rec_ready = true;
        return QG_OK;
    };

    // A lopsided high digit of the radix histograms means skew, and then a key
    // sample decides whether the learned function spreads the rows better.
    bool use_learned = may_learn && variant == 2;
    bool compared = false;
    if (may_learn && variant == 0 && ntot >= (1 << 16)) {
        const uint32_t *hs = h + 512 + (nb_radix > 256 ? 256 : 0);
        const uint32_t nbin = nb_radix > 256 ? ((nb_radix - 1) >> 8) + 1 : nb_radix;
        uint32_t mx = 0;
        for (uint32_t i = 0; i < nbin; i++) mx = hs[i] > mx ? hs[i] : mx;
        if ((double)mx > 4.0 * (double)nS / (double)nbin) compared = true;
    }
    long long m = 0;
    if (use_learned || compared) {
        QG_TRY(ensure_rrec());
        QG_TRY(pj_train(ctx, L, nb, r, nR, s, nS, &m));
    }
    if (compared) {
        double orad = 0, olrn = 0;
        QG_TRY(pj_compare(ctx, L, m, ntot, radix, nb_radix, learned, nb, &orad, &olrn));
        use_learned = olrn < 0.5 * orad;
    }
    // Dense build side: only S' is partitioned, by the radix function.
    bool dense = rs.dense_ok && !use_learned;
    if (!dense) QG_TRY(ensure_rrec());
    // The learned function is evaluated once per row: its bucket ids go to a
    // sidecar that the partition passes carry along (ping-pong per side).
    uint16_t *bidr[2] = {nullptr, nullptr}, *bids[2] = {nullptr, nullptr};
    if (use_learned) {
        const size_t rb2 = qg_align_up((size_t)nR * 2, 256), sb2 = qg_align_up((size_t)nS * 2, 256);
        char *side;
        QG_TRY(pj_pool_get(ctx, &ctx->pj_tmp, &ctx->pj_tmp_bytes, 2 * rb2 + 2 * sb2, &side));
        bidr[0] = (uint16_t *)side;
        bidr[1] = (uint16_t *)(side + rb2);
        bids[0] = (uint16_t *)(side + 2 * rb2);
        bids[1] = (uint16_t *)(side + 2 * rb2 + sb2);
        QG_TRY(pj_dhist(ctx, L, learned, nb, r, nR, s, nS, h, bidr[0], bids[0]));
    }
    const qg_part_fn &pf = use_learned ? learned : radix;
    const uint32_t nbu = use_learned ? nb : nb_radix;

    // partition a side by bucket (one or two stable 8-bit passes)
    const int npos = nbu > 256 ? 2 : (nbu > 1 ? 1 : 0);
    auto partition = [&](bool side_r) -> qg_status {
        if (npos == 0) return QG_OK;
        uint32_t hist[4 * QG_RADIX] = {0}, bases[4 * QG_RADIX];
        int passes[4];
        bool in_b = false;
        memcpy(hist, h + (side_r ? 0 : 512), 512 * 4);
        const long long n = side_r ? nR : nS;
        const int np = qg_sort_plan(hist, npos, n, passes, bases);
        unsigned long long *&a = side_r ? r : s, *&bb = side_r ? rsp : ssp;
        uint16_t **bid = side_r ? bidr : bids;
        QG_TRY(qg_radix_passes_pf(ctx, false, qg_sort_bufs{a, nullptr, nullptr, nullptr, bid[0]},
                                  qg_sort_bufs{bb, nullptr, nullptr, nullptr, bid[1]}, n, pf, passes, np, bases,
                                  &in_b, true));  // buckets in order; rows within a bucket in any order
        if (in_b) std::swap(a, bb);
        return QG_OK;
    };
    auto pack_launch = [&](uint32_t rmax) -> qg_status {
        const uint32_t nctas = (nbu + PK_THREADS * PK_SEG - 1) / (PK_THREADS * PK_SEG);
        const uint32_t seg = ((nbu + PK_THREADS * nctas - 1) / (PK_THREADS * nctas) + 7) & ~7u;
        const size_t tgn = (size_t)nb + PK_THREADS * PK_SEG;
        qg_pre_launch(ctx);
        k_pj_pack<<<nctas, PK_THREADS, 0, ctx->stream>>>(L.rbk, L.sbk, nbu, seg, rmax, g_pj_smax, L.tg, L.tg + tgn,
                                                         L.tg + 2 * tgn, L.tover, L.pkc);
        QG_TRY(qg_check_launch(ctx, "k_pj_pack"));
        qg_pre_launch(ctx);
        k_pj_place<<<nctas, 256, 0, ctx->stream>>>(L.rbk, L.sbk, nbu, PK_THREADS * seg, L.tg, L.tg + tgn,
                                                   L.tg + 2 * tgn, L.tover, L.pkc, L.gr, L.gs, L.big, L.bigcnt,
                                                   L.cross, L.pk);
        return qg_check_launch(ctx, "k_pj_place");
    };
    auto pack_check = [&](const PjPackOut &pk) -> qg_status {
        return (pk.groups == 0 || pk.groups > nbu || pk.over > pk.groups) ? QG_ERR_INVALID : QG_OK;  // G <= buckets
    };
    // fine bucket bounds, then the join groups packed on the device (one read of the counts)
    auto pack = [&](uint32_t rmax, PjPackOut *pk) -> qg_status {
        QG_TRY(pack_launch(rmax));
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(&pin->pk, L.pk, sizeof(PjPackOut), cudaMemcpyDeviceToHost, ctx->stream), "pack d2h");
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        *pk = pin->pk;
        return pack_check(*pk);
    };
    auto r_bounds = [&]() -> qg_status {
        qg_pre_launch(ctx);
        k_pj_bounds<<<(nbu + 256) / 256, 256, 0, ctx->stream>>>(r, nR, pf, nbu, L.rbk);
        return qg_check_launch(ctx, "k_pj_bounds");
    };
    QG_TRY(partition(false));
    if (!dense) QG_TRY(partition(true));
    qg_pre_launch(ctx);
    k_pj_bounds<<<(nbu + 256) / 256, 256, 0, ctx->stream>>>(s, nS, pf, nbu, L.sbk);
    QG_TRY(qg_check_launch(ctx, "k_pj_bounds"));
    PjPackOut pk;
    if (dense) {
        // A group's "R rows" are its key span, at most a counting sort's.
        qg_pre_launch(ctx);
        k_pj_vbounds<<<(nbu + 256) / 256, 256, 0, ctx->stream>>>(L.rbk, nbu, rp.shift,
                                                                (unsigned long long)(kmax - kmin) + 1ull);
        QG_TRY(qg_check_launch(ctx, "k_pj_vbounds"));
        QG_TRY(pack(PJ_DENSE_BSPAN, &pk));
        if (pk.over == 0) {
            // every S' row matches when R's keys fill their span (S' keys lie in it)
            const bool full = (unsigned long long)(kmax - kmin) + 1ull == (unsigned long long)nR;
            qg_lookback lb;
            QG_TRY(qg_lb_make(ctx, pk.groups, QG_SITE_JOIN_PROBE, &lb));
            PdArgs da{s, L.gr, L.gs, rs.bitmap, rs.T, kmin, rs.sent_ok ? 1u : 0u, rs.sent, L.total, ok, oa, ob, cap};
            qg_pre_launch(ctx);
            auto kern = full ? k_pj_join_dense<PB_THREADS, PB_SMAX, true> : k_pj_join_dense<PB_THREADS, PB_SMAX, false>;
            kern<<<pk.groups, PB_THREADS, sizeof(PdSmem<PB_SMAX, PB_WARPS>), ctx->stream>>>(da, lb);
            QG_TRY(qg_check_launch(ctx, "k_pj_join_dense"));
            QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pinned, L.total, 8, cudaMemcpyDeviceToHost, ctx->stream), "total d2h");
            QG_TRY(qg_collect_error(ctx));
            *M_out = ctx->pinned[0];
            ctx->pj_stats[0] = 4;
            ctx->pj_stats[1] = nbu;
            for (int i = 2; i < 8; i++) ctx->pj_stats[i] = 0;
            ctx->pj_stats[5] = (uint32_t)g_pd_ctas_per_sm;  // no model on this path: the bucket kernel's CTAs per SM
            return QG_OK;
        }
        // an S' bucket above the bucket kernel's capacity: R's records after all
        dense = false;
        QG_TRY(ensure_rrec());
        QG_TRY(partition(true));
        QG_TRY(r_bounds());
        QG_TRY(pack(g_pj_rmax, &pk));
    } else {
        QG_TRY(r_bounds());
        QG_TRY(pack(g_pj_rmax, &pk));
    }
    const uint32_t G = pk.groups;
    const uint32_t no = pk.over;

    // Outside groups: a bucket with one key is a cross product (k_pj_cross);
    // the others all go through the sort-merge path together (k_pj_mj_*).
    std::vector<PjCross> cross;
    std::vector<PjMj> mj;
    long long nrb = 0, nsb = 0;
    unsigned long long cross_rows = 0;  // output rows of the cross products
    if (no > 0) {
        QG_TRY_CUDA(ctx, cudaMemsetAsync(L.mm, 0xff, (size_t)no * 4, ctx->stream), "memset mins");
        QG_TRY_CUDA(ctx, cudaMemsetAsync(L.mm + no, 0, (size_t)no * 4, ctx->stream), "memset maxes");
        qg_pre_launch(ctx);
        k_pj_minmax<<<dim3((unsigned)pj_grid(ctx, ((long long)pk.most + 3) / 4, 256, 4), (unsigned)std::min<uint32_t>(no, 65535)),
                      256, 0, ctx->stream>>>(L.cross, no, r, s, L.mm, L.mm + no);
        QG_TRY(qg_check_launch(ctx, "k_pj_minmax"));
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(pin->over, L.cross, (size_t)no * sizeof(PjCross), cudaMemcpyDeviceToHost, ctx->stream), "list d2h");
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(pin->mm, L.mm, (size_t)2 * no * 4, cudaMemcpyDeviceToHost, ctx->stream), "mm d2h");
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        for (uint32_t i = 0; i < no; i++) {
            const PjCross &e = pin->over[i];
            if (pin->mm[i] == pin->mm[no + i]) {
                cross.push_back(e);
                cross_rows += (unsigned long long)e.rn * e.sn;
            } else {
                mj.push_back(PjMj{e.b, e.rb, e.rn, e.sb, e.sn, (uint32_t)nrb, (uint32_t)nsb});
                nrb += e.rn;
                nsb += e.sn;
            }
        }
        if (!cross.empty()) {  // their output counts, for the bucket kernel's look-back
            QG_TRY_CUDA(ctx, cudaMemcpyAsync(L.cross, cross.data(), cross.size() * sizeof(PjCross), cudaMemcpyHostToDevice, ctx->stream), "cross h2d");
            qg_pre_launch(ctx);
            k_pj_cross_cnt<<<(unsigned)((cross.size() + 255) / 256), 256, 0, ctx->stream>>>(L.cross, (uint32_t)cross.size(), L.bigcnt);
            QG_TRY(qg_check_launch(ctx, "k_pj_cross_cnt"));
        }
    }
    QG_TRY_CUDA(ctx, cudaMemsetAsync(L.mjtot, 0, 8, ctx->stream), "memset mjtot");

    // sort-merge buckets: gather, sort by key, count each S row's matches
    // (into bigcnt, before the bucket kernel reads it), scan the counts
    unsigned long long *Rb = nullptr, *Sb = nullptr;
    uint32_t *mcnt = nullptr, *mlob = nullptr, *mpre = nullptr;
    uint32_t mj_rows = 0;  // the largest bucket's rows: the grid's x extent
    for (auto &e : mj) mj_rows = max(mj_rows, max(e.rn, e.sn));
    const unsigned mgx = (unsigned)pj_grid(ctx, (mj_rows + 3) / 4, 256, 4);
    const unsigned mgy = (unsigned)std::min<size_t>(mj.size(), 65535);
    if (!mj.empty()) {
        const size_t rbb = qg_align_up((size_t)nrb * 8, 256), sbb = qg_align_up((size_t)nsb * 8, 256),
                     cb = qg_align_up((size_t)nsb * 4, 256);
        char *tmp;
        QG_TRY(pj_pool_get(ctx, &ctx->pj_tmp, &ctx->pj_tmp_bytes, 2 * rbb + 2 * sbb + 3 * cb, &tmp));
        Rb = (unsigned long long *)tmp;
        unsigned long long *Rt = (unsigned long long *)(tmp + rbb);
        Sb = (unsigned long long *)(tmp + 2 * rbb);
        unsigned long long *St = (unsigned long long *)(tmp + 2 * rbb + sbb);
        mcnt = (uint32_t *)(tmp + 2 * rbb + 2 * sbb);
        mlob = (uint32_t *)(tmp + 2 * rbb + 2 * sbb + cb);
        mpre = (uint32_t *)(tmp + 2 * rbb + 2 * sbb + 2 * cb);
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(L.mj, mj.data(), mj.size() * sizeof(PjMj), cudaMemcpyHostToDevice, ctx->stream), "mj h2d");
        qg_pre_launch(ctx);
        k_pj_mj_gather<<<dim3(mgx, mgy), 256, 0, ctx->stream>>>(L.mj, (uint32_t)mj.size(), r, s, Rb, Sb);
        QG_TRY(qg_check_launch(ctx, "k_pj_mj_gather"));
        QG_TRY(qg_sort_rec_inplace(ctx, Rb, Rt, nrb));
        QG_TRY(qg_sort_rec_inplace(ctx, Sb, St, nsb));
        qg_pre_launch(ctx);
        k_pj_mj_count<<<dim3(mgx, mgy), 256, 0, ctx->stream>>>(L.mj, (uint32_t)mj.size(), Rb, Sb, mcnt, mlob,
                                                               L.bigcnt, L.mjtot);
        QG_TRY(qg_check_launch(ctx, "k_pj_mj_count"));
        QG_TRY(qg_scan_excl_i32(ctx, (const int32_t *)mcnt, (int32_t *)mpre, nsb));
    }

    // the bucket kernel over the join groups
    qg_lookback lb;
    QG_TRY(qg_lb_make(ctx, G, QG_SITE_JOIN_PROBE, &lb));
    PbArgs args{r, s, L.gr, L.gs, L.big, L.bigcnt, L.off, L.total, ok, oa, ob, cap};
    qg_pre_launch(ctx);
    k_pj_join<<<G, PB_THREADS, sizeof(PbSmem), ctx->stream>>>(args, lb);
    QG_TRY(qg_check_launch(ctx, "k_pj_join"));
    if (!cross.empty()) {
        qg_pre_launch(ctx);
        k_pj_cross<<<dim3((unsigned)pj_grid(ctx, 1LL << 24, 256, 4), (unsigned)std::min<size_t>(cross.size(), 65535)),
                     256, 0, ctx->stream>>>(L.cross, (uint32_t)cross.size(), r, s, L.off, ok, oa, ob, cap);
        QG_TRY(qg_check_launch(ctx, "k_pj_cross"));
    }
    if (!mj.empty()) {
        qg_pre_launch(ctx);
        k_pj_mj_write<<<dim3(mgx, mgy), 256, 0, ctx->stream>>>(L.mj, (uint32_t)mj.size(), Rb, Sb, mcnt, mlob, mpre,
                                                               L.off, ok, oa, ob, cap);
        QG_TRY(qg_check_launch(ctx, "k_pj_mj_write"));
    }
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pinned + 1, L.mjtot, 8, cudaMemcpyDeviceToHost, ctx->stream), "mjtot d2h");
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pinned, L.total, 8, cudaMemcpyDeviceToHost, ctx->stream), "total d2h");
    if (use_learned)  // the model's knot and heavy-key counts, for qg_join_stats
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pinned + 2, L.model, 16, cudaMemcpyDeviceToHost, ctx->stream),
                    "model header d2h");
    QG_TRY(qg_collect_error(ctx));  // synchronises: the counts (and header) are in
    const unsigned long long total = (unsigned long long)ctx->pinned[0];
    // The look-back sums are 32-bit: report the outside groups' 64-bit sum
    // when they alone could wrap it (a capacity error follows).
    *M_out = (long long)total;
    {
        const unsigned long long outside = (unsigned long long)ctx->pinned[1] + cross_rows;
        if (outside >= (1ull << 32)) *M_out = (long long)outside;
    }
    ctx->pj_stats[0] = use_learned ? 2 : 1;
    ctx->pj_stats[1] = nbu;
    ctx->pj_stats[2] = no;
    ctx->pj_stats[3] = pk.over_rows > 0xffffffffull ? 0xffffffffu : (uint32_t)pk.over_rows;
    ctx->pj_stats[4] = (uint32_t)mj.size();
    ctx->pj_stats[5] = 0;
    ctx->pj_stats[6] = 0;
    if (use_learned) {
        const uint32_t *hk = reinterpret_cast<const uint32_t *>(ctx->pinned + 2);
        ctx->pj_stats[5] = hk[0];
        ctx->pj_stats[6] = hk[3];
    }
    ctx->pj_stats[7] = (compared && use_learned) ? 1 : 0;
    return QG_OK;
}

}  // namespace

extern "C" QG_API qg_status qg_join_set_knobs(int variant, int buckets_log2, uint32_t bucket_s_max,
                                              uint32_t bucket_r_max) {
    if (variant < 0 || variant > 3 || buckets_log2 < 0 || buckets_log2 > 16) return QG_ERR_INVALID;
    if (bucket_s_max > (uint32_t)PB_SMAX || bucket_r_max > (uint32_t)PB_RMAX) return QG_ERR_INVALID;
    g_pj_variant = variant;
    g_pj_blog2 = buckets_log2;
    g_pj_smax = bucket_s_max ? bucket_s_max : PB_SMAX;
    g_pj_rmax = bucket_r_max ? bucket_r_max : PB_RMAX;
    return QG_OK;
}

extern "C" QG_API qg_status qg_join_set_dense(int enable) {
    if (enable != 0 && enable != 1) return QG_ERR_INVALID;
    g_pj_dense = enable != 0;
    return QG_OK;
}

extern "C" QG_API qg_status qg_join_stats(qg_ctx *ctx, uint32_t *out8) {
    if (!ctx || !out8) return QG_ERR_INVALID;
    memcpy(out8, ctx->pj_stats, sizeof(ctx->pj_stats));
    return QG_OK;
}

int qg_join_default_variant() { return g_pj_variant; }

static qg_status join_filter_sort_impl(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay, int64_t nR,
                                       const int32_t *skey, const int32_t *spay, int64_t nS, int32_t slo,
                                       int32_t shi, int32_t *out_key, int32_t *out_rpay, int32_t *out_spay,
                                       int64_t cap, int64_t *out_n);

extern "C" QG_API qg_status qg_join_filter_sort(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay,
                                                int64_t nR, const int32_t *skey, const int32_t *spay,
                                                int64_t nS, int32_t slo, int32_t shi, int32_t *out_key,
                                                int32_t *out_rpay, int32_t *out_spay, int64_t cap,
                                                int64_t *out_n) {
    if (!ctx) return QG_ERR_INVALID;
    // With a cost model attached the variant is its choice for these sizes;
    // the S filter's selectivity is estimated by its share of the int32 range.
    qg_steer_call sc;
    qg_steer_begin(ctx, QG_STEER_JOIN, nS, nR, ((double)shi - (double)slo + 1.0) / 4294967296.0, &sc);
    const qg_status st = join_filter_sort_impl(ctx, rkey, rpay, nR, skey, spay, nS, slo, shi, out_key, out_rpay,
                                               out_spay, cap, out_n);
    qg_steer_end(ctx, &sc, st);
    return st;
}

static qg_status join_filter_sort_impl(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay, int64_t nR,
                                       const int32_t *skey, const int32_t *spay, int64_t nS, int32_t slo,
                                       int32_t shi, int32_t *out_key, int32_t *out_rpay, int32_t *out_spay,
                                       int64_t cap, int64_t *out_n) {
    if (!ctx || nR < 0 || nS < 0 || cap < 0 || !out_n) return QG_ERR_INVALID;
    const int variant = qg_effective_variant(ctx, QG_STEER_JOIN, g_pj_variant);
    if ((nR > 0 && (!rkey || !rpay)) || (nS > 0 && (!skey || !spay)) ||
        (cap > 0 && (!out_key || !out_rpay || !out_spay)))
        return QG_ERR_INVALID;
    if ((((uintptr_t)skey) | ((uintptr_t)spay)) & 15) return QG_ERR_INVALID;
    if (cap >= (1LL << 30) || nS >= (1LL << 40)) return QG_ERR_UNSUPPORTED;
    if (variant == 3 || nS >= (1LL << 30) || nR >= (1LL << 30))
        return qg_join_hash_sort(ctx, rkey, rpay, nR, skey, spay, nS, slo, shi, out_key, out_rpay,
                                 out_spay, cap, out_n);
    *out_n = 0;
    memset(ctx->pj_stats, 0, sizeof(ctx->pj_stats));
    if (nR == 0 || nS == 0) return QG_OK;
    // aux: R records + spare (the spare doubles as the dense build side's
    // payload table), S' records + spare, the presence bitmap, level-0 arrays
    const size_t rb = qg_align_up((size_t)nR * 8, 256), sb = qg_align_up((size_t)nS * 8, 256);
    const size_t bmb = qg_align_up(((size_t)2 * nR + 63) / 32 * 4, 256);
    char *aux;
    QG_TRY(qg_aux(ctx, 2 * rb + 2 * sb + bmb + pj_level_bytes(PJ_MAX_BUCKETS, true), &aux));
    PjPin *pin;
    QG_TRY(pj_pin(ctx, &pin));
    unsigned long long *R = (unsigned long long *)aux, *Rsp = (unsigned long long *)(aux + rb);
    unsigned long long *S = (unsigned long long *)(aux + 2 * rb), *Ssp = (unsigned long long *)(aux + 2 * rb + sb);
    uint32_t *bitmap = (uint32_t *)(aux + 2 * rb + 2 * sb);
    uint32_t *T = (uint32_t *)Rsp;  // the dense build side's payloads (2 nR entries at most)
    const uint32_t nb = pj_bucket_count(nR, nS);
    int lb2 = 0;
    while ((1u << lb2) < nb) lb2++;
    PjLevel L;
    pj_level_carve(aux + 2 * rb + 2 * sb + bmb, nb, variant != 1, &L);
    QG_TRY_CUDA(ctx, cudaMemsetAsync(L.dh, 0, 4 * 256 * 4, ctx->stream), "memset dhist");
    QG_TRY_CUDA(ctx, cudaMemsetAsync(bitmap, 0, bmb, ctx->stream), "memset bitmap");
    qg_pre_launch(ctx);
    k_pj_range_init<<<1, 1, 0, ctx->stream>>>(L.range, L.dflags);
    QG_TRY(qg_check_launch(ctx, "k_pj_range_init"));
    qg_pre_launch(ctx);
    k_pj_rrange<<<pj_grid(ctx, nR, 256, 8), 256, 0, ctx->stream>>>(rkey, rpay, nR, L.range, L.dflags);
    QG_TRY(qg_check_launch(ctx, "k_pj_rrange"));
    // R: payload table (+ presence bitmap without a sentinel) on a dense span, else records + digit histograms
    qg_pre_launch(ctx);
    k_pj_tfill<<<pj_grid(ctx, nR / 2, 256, 8), 256, 0, ctx->stream>>>(T, L.range, lb2, nR, L.dflags);
    QG_TRY(qg_check_launch(ctx, "k_pj_tfill"));
    qg_pre_launch(ctx);
    k_pj_rtab<<<pj_grid(ctx, nR, 256, 8), 256, 0, ctx->stream>>>(rkey, rpay, nR, L.range, lb2, bitmap, T,
                                                                 L.dflags, R, L.dh);
    QG_TRY(qg_check_launch(ctx, "k_pj_rtab"));
    qg_pre_launch(ctx);
    k_pj_distinct<<<pj_grid(ctx, nR, 256, 8), 256, 0, ctx->stream>>>(
        bitmap, T, L.range, lb2, nR, L.dflags, reinterpret_cast<unsigned long long *>(L.dflags + PJ_F_DISTINCT));
    QG_TRY(qg_check_launch(ctx, "k_pj_distinct"));
    // S filter with the S' digit histograms of the radix function
    constexpr int SF_TILE = SF_THREADS * SF_ROUNDS * 4;
    const long long tiles = (nS + SF_TILE - 1) / SF_TILE;
    qg_pre_launch(ctx);
    k_pj_sfilter<<<(unsigned)std::min<long long>(tiles, (long long)ctx->sm_count * 4), SF_THREADS, 0, ctx->stream>>>(
        skey, spay, nS, slo, shi, L.range, S, &L.range->count, ctx->ctl, lb2, L.dh + 512);
    QG_TRY(qg_check_launch(ctx, "k_pj_sfilter"));
    // one read brings R's key range, the S' count, the histograms, the dense flags and the error word
    static_assert(sizeof(PjRange) <= 2 * sizeof(long long), "two pinned slots");
    PjRange *hp = reinterpret_cast<PjRange *>(ctx->pinned + 4);
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(hp, L.range, sizeof(PjRange), cudaMemcpyDeviceToHost, ctx->stream), "range d2h");
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(pin->h, L.dh, 4 * 256 * 4, cudaMemcpyDeviceToHost, ctx->stream), "dhist d2h");
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(pin->dflags, L.dflags, PJ_F_WORDS * 4, cudaMemcpyDeviceToHost, ctx->stream), "flags d2h");
    QG_TRY(qg_collect_error(ctx));
    const PjRange hr = *hp;
    const long long ns1 = (long long)hr.count;
    unsigned long long distinct;
    memcpy(&distinct, pin->dflags + PJ_F_DISTINCT, 8);
    PjRSide rs{rkey, rpay, pin->dflags[PJ_F_DENSE] == 0u,
               pin->dflags[PJ_F_DENSE] != 0u && distinct == (unsigned long long)nR && g_pj_dense,
               pin->dflags[PJ_F_SENT_OK] != 0u, pin->dflags[PJ_F_SENT],
               bitmap, T};
    long long M = 0;
    // pj_core ends with a read of the output count and the error word
    QG_TRY(pj_core(ctx, L, pin, nb, lb2, rs, R, Rsp, nR, S, Ssp, ns1, hr.kmin, hr.kmax, variant,
                   (uint32_t *)out_key, (uint32_t *)out_rpay, (uint32_t *)out_spay, cap, &M));
    *out_n = M;
    return M > cap ? QG_ERR_CAPACITY : QG_OK;
}

// ---- learned partition function as a stand-alone tool ---------------------
extern "C" QG_API int64_t qg_part_model_bytes(void) { return (int64_t)sizeof(qg_cdf_model); }

namespace {
__global__ void k_keys_to_items(const uint32_t *__restrict__ keys, long long n, long long m,
                                unsigned long long *__restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = (unsigned long long)__ldg(keys + (i * n) / m) << 32;
}
}  // namespace

extern "C" QG_API qg_status qg_part_learn(qg_ctx *ctx, const uint32_t *keys, int64_t n, uint32_t nbuckets,
                                          void *d_model) {
    if (!ctx || !keys || n <= 0 || !d_model || nbuckets < 1 || nbuckets > (uint32_t)PJ_MAX_BUCKETS)
        return QG_ERR_INVALID;
    const long long m = n < CDF_SAMPLE ? n : CDF_SAMPLE;
    char *aux;
    QG_TRY(qg_aux(ctx, (size_t)m * 16 + (size_t)(1 + QG_CDF_MAX_HEAVY) * 4 + 256, &aux));
    unsigned long long *smp = (unsigned long long *)aux, *smp2 = smp + m;
    uint32_t *heavy = (uint32_t *)(smp2 + m);
    qg_pre_launch(ctx);
    k_keys_to_items<<<pj_grid(ctx, m, 256, 4), 256, 0, ctx->stream>>>(keys, n, m, smp);
    QG_TRY(qg_check_launch(ctx, "k_keys_to_items"));
    QG_TRY(qg_sort_rec_inplace(ctx, smp, smp2, m));
    long long hthr = (3 * m + nbuckets - 1) / nbuckets;
    if (hthr < 2) hthr = 2;
    QG_TRY_CUDA(ctx, cudaMemsetAsync(heavy, 0, 4, ctx->stream), "memset heavy");
    qg_pre_launch(ctx);
    k_cdf_heavy<<<pj_grid(ctx, m, 256, 4), 256, 0, ctx->stream>>>(smp, m, hthr, heavy);
    QG_TRY(qg_check_launch(ctx, "k_cdf_heavy"));
    qg_pre_launch(ctx);
    k_cdf_fit<<<1, FIT_THREADS, 0, ctx->stream>>>(smp, m, nbuckets, hthr, heavy, (qg_cdf_model *)d_model);
    QG_TRY(qg_check_launch(ctx, "k_cdf_fit"));
    return qg_ctx_check(ctx);
}

extern "C" QG_API qg_status qg_part_eval(qg_ctx *ctx, const void *d_model, uint32_t kmin, int shift,
                                         const uint32_t *keys, int64_t n, uint32_t *buckets) {
    if (!ctx || n < 0 || shift < 0 || shift > 31 || (n > 0 && (!keys || !buckets))) return QG_ERR_INVALID;
    if (n == 0) return QG_OK;
    qg_part_fn pf{d_model ? 1 : 0, kmin, shift, (const qg_cdf_model *)d_model};
    qg_pre_launch(ctx);
    k_part_eval<<<pj_grid(ctx, n, 256, 8), 256, 0, ctx->stream>>>(keys, n, pf, buckets);
    QG_TRY(qg_check_launch(ctx, "k_part_eval"));
    return qg_ctx_check(ctx);
}
