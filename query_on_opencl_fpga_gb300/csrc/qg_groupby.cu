// qg_groupby.cu -- group-by and aggregation.
//
// Two operators:
//
// 1. The reference's sorted contract (host/host/testGroupBy.cpp:81-154,
//    host/host/testAggAfterGB.cpp:69-123): sort Records by key, label group
//    boundaries (scanGroupLabel_kernel, kernel/aggregation/1/
//    group_by_cu_op_dp.cl:293-327), scan the labels and write startPos
//    (:505-528), then aggregate .x per group (parallelAggregate_kernel,
//    :547-716).  Here the label + scan + outSize + write chain is one
//    single-pass compaction kernel, and the per-group aggregation runs over
//    fixed row chunks (a group spanning chunks combines with atomics) instead
//    of one work-group per group in chunks of 512 launches.
//
// 2. Column group-by with int64 SUM + COUNT, optionally fused with a range
//    predicate on a second column (configs 1 / 1-fused; the fused
//    filter_aggregation image, kernel/filter_aggregation/
//    filter_aggregation_cu_op_dp.cl).  Instead of sort -> label -> scan ->
//    aggregate, rows are aggregated in tables: the default path is the
//    dense-window kernels of qg_gbdense.cu (keys within a 2^22-key window,
//    emitted in key order).  Keys that do not fit a window take two passes
//    (k_gb_part, k_gb_merge, section 2' below) -- per-SM shared-memory tables
//    absorb the heavy hitters, the remaining rows are spilled into hash
//    partitions and each partition is summed by one CTA in shared memory.
//    The single-pass global-table kernel (k_groupby_hash: shared-memory table
//    + global open-addressing table of 32-byte {tag, sum, count} slots
//    updated with atomicCAS / 64-bit atomicAdd) is the fallback for inputs
//    that overflow the spill buckets.  QG_ORDER_KEY then ranks or sorts the
//    groups by key (unsigned, the order groupByImpl's sorted array gives).
#include "qg_internal.cuh"
#include "qg_sort.cuh"

namespace {

// ---------------------------------------------------------------------------
// 1a. group boundaries of sorted records -> startPos (stable compaction)
// ---------------------------------------------------------------------------
constexpr int GBD_THREADS = 256;
constexpr int GBD_WARPS = GBD_THREADS / 32;
constexpr int GBD_ROUNDS = 8;  // 2 records per round: 4096 records per tile

__global__ void __launch_bounds__(GBD_THREADS)
k_group_bounds(const uint4 *__restrict__ in, long long n, int32_t *__restrict__ startPos,
               long long cap, long long *__restrict__ d_count, qg_lookback lb) {
    constexpr int TILE = GBD_THREADS * GBD_ROUNDS * 2;
    __shared__ uint32_t s_tile, s_epoch, s_excl;
    __shared__ uint32_t s_woff[GBD_ROUNDS * GBD_WARPS];
    qg_lb_begin(lb, &s_tile, &s_epoch);
    const uint32_t tile = s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long base = (long long)tile * TILE;
    const uint32_t lt = qg_lanemask_lt();
    const uint2 *in2 = reinterpret_cast<const uint2 *>(in);
    uint32_t fl = 0, lpre[GBD_ROUNDS];
    // Loads of all rounds first (keys of the thread's pair and of the record
    // before it), then the ballots, so the DRAM latencies overlap.
    uint32_t k0[GBD_ROUNDS], k1[GBD_ROUNDS], kp[GBD_ROUNDS];
#pragma unroll
    for (int r = 0; r < GBD_ROUNDS; r++) {
        long long idx = base + (long long)(r * GBD_THREADS + tid) * 2;
        k0[r] = k1[r] = kp[r] = 0;
        if (idx < n) {
            if (idx + 1 < n) {
                int4 t = qg_ldg_stream(reinterpret_cast<const int4 *>(in) + (idx >> 1));
                k0[r] = (uint32_t)t.y;
                k1[r] = (uint32_t)t.w;
            } else {
                k0[r] = in2[idx].y;
            }
            if (idx > 0) kp[r] = __ldg(&in2[idx - 1].y);
        }
    }
#pragma unroll
    for (int r = 0; r < GBD_ROUNDS; r++) {
        long long idx = base + (long long)(r * GBD_THREADS + tid) * 2;
        bool f0 = (idx < n) && ((idx == 0) || (kp[r] != k0[r]));
        bool f1 = (idx + 1 < n) && (k1[r] != k0[r]);
        uint32_t b0 = __ballot_sync(QG_FULL_MASK, f0), b1 = __ballot_sync(QG_FULL_MASK, f1);
        lpre[r] = __popc(b0 & lt) + __popc(b1 & lt);
        if (lane == 0) s_woff[r * GBD_WARPS + warp] = __popc(b0) + __popc(b1);
        fl |= ((uint32_t)f0 << (2 * r)) | ((uint32_t)f1 << (2 * r + 1));
    }
    __syncthreads();
    if (warp == 0)
        qg_tile_compact_offsets<GBD_ROUNDS * GBD_WARPS>(s_woff, lb, tile, s_epoch, &s_excl, d_count);
    __syncthreads();
    const long long excl = s_excl;
#pragma unroll
    for (int r = 0; r < GBD_ROUNDS; r++) {
        long long idx = base + (long long)(r * GBD_THREADS + tid) * 2;
        long long pos = excl + s_woff[r * GBD_WARPS + warp] + lpre[r];
        if ((fl >> (2 * r)) & 1u) {
            if (pos < cap) startPos[pos] = (int32_t)idx;
            pos++;
        }
        if ((fl >> (2 * r + 1)) & 1u)
            if (pos < cap) startPos[pos] = (int32_t)(idx + 1);
    }
    qg_lb_finish(lb, tile, gridDim.x - 1, s_epoch);
}

// ---------------------------------------------------------------------------
// 1b. per-group aggregation of .x over sorted records
// ---------------------------------------------------------------------------
constexpr int AGG_CHUNK = 2048;  // rows per warp work item

__device__ __forceinline__ int32_t agg_identity(int op) {
    return op == QG_REDUCE_MIN ? (1 << 30) : 0;
}

__global__ void k_agg_init(int32_t *agg, long long g0, long long g1, int op) {
    long long stride = (long long)gridDim.x * blockDim.x;
    int32_t id = agg_identity(op);
    for (long long i = g0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g1; i += stride)
        agg[i] = id;
}

// Groups [g0, g1) of G: rows [startPos[g0], startPos[g1] or n) in chunks of
// AGG_CHUNK rows counted from the range start.
__global__ void __launch_bounds__(256)
k_agg_chunks(const uint2 *__restrict__ rec, long long n, const int32_t *__restrict__ startPos,
             long long G, long long g0, long long g1, int op, int32_t *__restrict__ agg) {
    const int lane = threadIdx.x & 31;
    const long long warp_id = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long rs = __ldg(&startPos[g0]);
    const long long re = (g1 == G) ? n : (long long)__ldg(&startPos[g1]);
    const long long nchunks = (re - rs + AGG_CHUNK - 1) / AGG_CHUNK;
    for (long long c = warp_id; c < nchunks; c += nwarps) {
        const long long cs = rs + c * AGG_CHUNK;
        const long long ce = (cs + AGG_CHUNK < re) ? cs + AGG_CHUNK : re;
        // last group of the range starting at or before cs
        long long lo = g0, hi = g1 - 1;
        while (lo < hi) {
            long long mid = (lo + hi + 1) >> 1;
            if ((long long)__ldg(&startPos[mid]) <= cs) lo = mid; else hi = mid - 1;
        }
        long long g = lo;
        long long pos = cs;
        while (pos < ce && g < g1) {
            const long long gs = __ldg(&startPos[g]);
            const long long ge = (g == G - 1) ? n : (long long)__ldg(&startPos[g + 1]);
            const long long se = ge < ce ? ge : ce;
            int32_t acc = agg_identity(op);
            uint32_t sum = 0;
            for (long long i = pos + lane; i < se; i += 32) {
                int32_t v = (int32_t)rec[i].x;
                if (op == QG_REDUCE_MAX) acc = v > acc ? v : acc;
                else if (op == QG_REDUCE_MIN) acc = v < acc ? v : acc;
                else sum += (uint32_t)v;
            }
            if (op == QG_REDUCE_MAX) acc = __reduce_max_sync(QG_FULL_MASK, acc);
            else if (op == QG_REDUCE_MIN) acc = __reduce_min_sync(QG_FULL_MASK, acc);
            else sum = __reduce_add_sync(QG_FULL_MASK, sum);
            if (lane == 0) {
                const bool whole = (pos == gs) && (se == ge);
                if (op == QG_REDUCE_MAX) { if (whole) agg[g] = acc; else atomicMax(&agg[g], acc); }
                else if (op == QG_REDUCE_MIN) { if (whole) agg[g] = acc; else atomicMin(&agg[g], acc); }
                else if (whole) {
                    agg[g] = (op == QG_REDUCE_AVERAGE) ? ((int32_t)sum) / (int32_t)(ge - gs) : (int32_t)sum;
                } else {
                    atomicAdd((unsigned int *)&agg[g], sum);
                }
            }
            pos = se;
            g++;
        }
    }
}

// AVG of groups that spanned chunks: the atomics left the wrapped sum.
__global__ void k_agg_avg_finish(const int32_t *__restrict__ startPos, long long n, long long G,
                                 long long g0, long long g1, int32_t *__restrict__ agg) {
    long long stride = (long long)gridDim.x * blockDim.x;
    const long long rs = startPos[g0];
    for (long long g = g0 + (long long)blockIdx.x * blockDim.x + threadIdx.x; g < g1; g += stride) {
        long long gs = startPos[g], ge = (g == G - 1) ? n : startPos[g + 1];
        bool spans = ((gs - rs) / AGG_CHUNK) != ((ge - 1 - rs) / AGG_CHUNK);
        if (spans) agg[g] = agg[g] / (int32_t)(ge - gs);
    }
}

// ---------------------------------------------------------------------------
// 2. column hash group-by
// ---------------------------------------------------------------------------
struct __align__(32) GSlot {
    unsigned long long tag;  // 0 = empty, else (1 << 32) | key
    unsigned long long sum;
    unsigned long long cnt;
    unsigned long long pad;
};

constexpr int GB_THREADS = 512;
constexpr uint32_t SM_EMPTY = 0xffffffffu;
constexpr int SM_MAX_PROBE = 8;

__device__ __forceinline__ void gtable_add(GSlot *__restrict__ tab, uint32_t mask, uint32_t key,
                                           unsigned long long sum, unsigned long long cnt,
                                           qg_control *ctl) {
    const unsigned long long tag = (1ull << 32) | key;
    uint32_t h = qg_hash32(key) & mask;
    for (uint32_t p = 0; p <= mask; p++) {
        unsigned long long cur = tab[h].tag;
        if (cur == 0) cur = atomicCAS(&tab[h].tag, 0ull, tag);
        if (cur == 0 || cur == tag) {
            atomicAdd(&tab[h].sum, sum);
            atomicAdd(&tab[h].cnt, cnt);
            return;
        }
        h = (h + 1) & mask;
    }
    qg_record_error(ctl, QG_ERR_TABLE_FULL, QG_SITE_GROUPBY);
}

template <bool PRED>
__global__ void __launch_bounds__(GB_THREADS)
k_groupby_hash(const int32_t *__restrict__ key, const int32_t *__restrict__ val,
               const int32_t *__restrict__ val2, int32_t lo2, int32_t hi2, long long n,
               GSlot *__restrict__ tab, uint32_t tmask, int slog2, qg_control *ctl) {
    extern __shared__ __align__(16) unsigned char gb_raw[];
    const int S = 1 << slog2;
    const uint32_t smask = (uint32_t)S - 1;
    unsigned long long *s_sum = reinterpret_cast<unsigned long long *>(gb_raw);
    uint32_t *s_key = reinterpret_cast<uint32_t *>(s_sum + S);
    uint32_t *s_cnt = s_key + S;
    for (int i = threadIdx.x; i < S; i += GB_THREADS) {
        s_key[i] = SM_EMPTY;
        s_sum[i] = 0;
        s_cnt[i] = 0;
    }
    __syncthreads();

    auto process = [&](int32_t k, int32_t v) {
        const uint32_t uk = (uint32_t)k;
        if (uk != SM_EMPTY) {
            uint32_t h = qg_hash32(uk) & smask;
#pragma unroll 1
            for (int p = 0; p < SM_MAX_PROBE; p++) {
                uint32_t cur = s_key[h];
                if (cur == SM_EMPTY) cur = atomicCAS(&s_key[h], SM_EMPTY, uk);
                if (cur == SM_EMPTY || cur == uk) {
                    atomicAdd(&s_sum[h], (unsigned long long)(long long)v);
                    atomicAdd(&s_cnt[h], 1u);
                    return;
                }
                h = (h + 1) & smask;
            }
        }
        gtable_add(tab, tmask, uk, (unsigned long long)(long long)v, 1ull, ctl);
    };

    const long long nv = n >> 2;  // full int4 groups
    const long long stride = (long long)gridDim.x * GB_THREADS;
    for (long long q = (long long)blockIdx.x * GB_THREADS + threadIdx.x; q < nv; q += stride) {
        int4 k4 = qg_ldg_stream(reinterpret_cast<const int4 *>(key) + q);
        int4 v4 = qg_ldg_stream(reinterpret_cast<const int4 *>(val) + q);
        bool m0 = true, m1 = true, m2 = true, m3 = true;
        if (PRED) {
            int4 w4 = qg_ldg_stream(reinterpret_cast<const int4 *>(val2) + q);
            m0 = (w4.x >= lo2) & (w4.x <= hi2);
            m1 = (w4.y >= lo2) & (w4.y <= hi2);
            m2 = (w4.z >= lo2) & (w4.z <= hi2);
            m3 = (w4.w >= lo2) & (w4.w <= hi2);
        }
        if (m0) process(k4.x, v4.x);
        if (m1) process(k4.y, v4.y);
        if (m2) process(k4.z, v4.z);
        if (m3) process(k4.w, v4.w);
    }
    // tail rows
    if (blockIdx.x == 0) {
        for (long long i = (nv << 2) + threadIdx.x; i < n; i += GB_THREADS) {
            if (PRED && !((val2[i] >= lo2) & (val2[i] <= hi2))) continue;
            process(key[i], val[i]);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < S; i += GB_THREADS) {
        uint32_t k = s_key[i];
        if (k != SM_EMPTY) gtable_add(tab, tmask, k, s_sum[i], (unsigned long long)s_cnt[i], ctl);
    }
}

// Compact occupied slots into (key, sum, count) columns, clearing the table.
// With `rec` set, also writes Record {x = output index, y = key} for a sort.
__global__ void __launch_bounds__(256)
k_groupby_emit(GSlot *__restrict__ tab, long long nslots, int32_t *__restrict__ gkey,
               long long *__restrict__ gsum, long long *__restrict__ gcnt, long long cap,
               unsigned long long *__restrict__ cursor, unsigned long long *__restrict__ rec) {
    // One output reservation per CTA and round (not per warp): the cursor is
    // a single global word.
    __shared__ uint32_t s_wc[8];
    __shared__ unsigned long long s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lt = qg_lanemask_lt();
    long long stride = (long long)gridDim.x * blockDim.x;
    long long start = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long iters = (nslots + stride - 1) / stride;
    for (long long it = 0; it < iters; it++) {
        long long s = start + it * stride;
        GSlot e;
        bool occ = false;
        if (s < nslots) {
            e = tab[s];
            occ = e.tag != 0;
        }
        uint32_t b = __ballot_sync(QG_FULL_MASK, occ);
        if (lane == 0) s_wc[warp] = __popc(b);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int w = 0; w < 8; w++) {
                const uint32_t x = s_wc[w];
                s_wc[w] = t;
                t += x;
            }
            s_base = t ? atomicAdd(cursor, (unsigned long long)t) : 0ull;
        }
        __syncthreads();
        const unsigned long long basepos = s_base + s_wc[warp];
        __syncthreads();  // s_wc and s_base are rewritten next round
        if (occ) {
            long long pos = (long long)basepos + __popc(b & lt);
            if (pos < cap) {
                gkey[pos] = (int32_t)(uint32_t)e.tag;
                gsum[pos] = (long long)e.sum;
                gcnt[pos] = (long long)e.cnt;
                if (rec) rec[pos] = ((unsigned long long)(uint32_t)e.tag << 32) | (unsigned long long)pos;
            }
            GSlot z;
            z.tag = 0; z.sum = 0; z.cnt = 0; z.pad = 0;
            tab[s] = z;
        }
    }
}

// Gather the key-sorted order: rec[i] = {x = old index, y = key}.
// With d_n set, the count is min(g, *d_n), read on the device.
__global__ void k_groupby_gather(const unsigned long long *__restrict__ rec, long long g,
                                 const long long *__restrict__ tsum, const long long *__restrict__ tcnt,
                                 int32_t *__restrict__ gkey, long long *__restrict__ gsum,
                                 long long *__restrict__ gcnt, const long long *__restrict__ d_n) {
    if (d_n && *d_n < g) g = *d_n;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g; i += stride) {
        unsigned long long r = rec[i];
        uint32_t idx = (uint32_t)r;
        gkey[i] = (int32_t)(r >> 32);
        gsum[i] = tsum[idx];
        gcnt[i] = tcnt[idx];
    }
}

// ---------------------------------------------------------------------------
// 2'. two-pass column group-by (keys that do not fit the dense window)
//
// Pass 1 (k_gb_part): one CTA per SM reads a contiguous slice of the rows.
// Keys that find a place in the CTA's shared-memory table (the heavy
// hitters, which arrive first under skew) are summed there.  Every other row
// is written as (key, value) into the CTA's own spill bucket for partition
// hash(key) >> (32 - plog2) -- a shared-memory cursor per partition, no
// global atomics; the scattered 8-byte stores merge in L2 because each
// bucket is written sequentially.  At the end the CTA writes its per-
// partition spill counts and its shared-memory table, counting-sorted by
// partition, as (key, count, sum) partials.
// Pass 2 (k_gb_merge): one CTA per partition gathers that partition's spill
// rows and partials from every pass-1 CTA, sums them in a shared-memory table
// and emits the final groups.  No global hash table, no global atomics on the
// data path; the L2-atomic bound of a global table is gone.
// A bucket that overflows its capacity (an adversarial key order) raises a
// flag and the host reruns the call with the global-table kernel above.
// ---------------------------------------------------------------------------
struct GPartial {
    uint32_t key;
    uint32_t cnt;
    long long sum;
};

struct GbSpill {
    uint2 *miss;      // [C][P][capm] (key, value)
    uint32_t *mcnt;   // [P][GB_MAX_C] rows in each bucket (clamped to capm)
    GPartial *part;   // [C][S] shared-memory tables, partition-sorted
    uint32_t *poff;   // [P+1][GB_MAX_C] partition offsets into part[c]
    uint32_t capm;
    int plog2;
    int slog2;
};

constexpr int GB_MAX_C = 256;  // pass-1 CTAs (one per SM)
constexpr int P1_THREADS = 1024;
constexpr int P2_THREADS = 256;
constexpr int P2_TLOG2 = 11;  // pass-2 table slots (2048) + 1 for key 0xffffffff
constexpr int GB_SKETCH_WORDS = 8192;  // 16K 16-bit admission counters (32 KB)
// Key-order bitmap window (the dense order, section 2''): 2^27 keys, 16 MB.
constexpr long long GB_DENSE_RANGE = 1LL << 27;
constexpr size_t GB_DENSE_WORDS = GB_DENSE_RANGE / 32;

// In-place exclusive scan of a[0..L) in shared memory by the whole CTA;
// returns the total.  `wsum` holds one word per warp.
__device__ uint32_t block_excl_scan(uint32_t *a, int L, uint32_t *wsum) {
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (L + T - 1) / T;
    const int b = tid * per, e = min(b + per, L);
    uint32_t s = 0;
    for (int i = b; i < e; i++) s += a[i];
    uint32_t inc = s;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t x = __shfl_up_sync(QG_FULL_MASK, inc, d);
        if (lane >= d) inc += x;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    uint32_t woff = 0, total = 0;
    for (int w = 0; w < (T >> 5); w++) {
        uint32_t x = wsum[w];
        if (w < warp) woff += x;
        total += x;
    }
    uint32_t run = woff + inc - s;
    for (int i = b; i < e; i++) {
        uint32_t x = a[i];
        a[i] = run;
        run += x;
    }
    __syncthreads();
    return total;
}

// 64-bit two's-complement accumulation with 32-bit shared-memory atomics:
// the low word takes the addend, the high word takes the addend's sign
// extension plus this add's carry out of the low word.  Each add is exact, so
// the pair holds the int64 sum whatever the interleaving.
__device__ __forceinline__ void smem_add_i64(uint32_t *lo, uint32_t *hi, long long v) {
    const uint32_t vl = (uint32_t)v;
    const uint32_t old = atomicAdd(lo, vl);
    const uint32_t carry = (old + vl) < old ? 1u : 0u;
    const uint32_t inc = (uint32_t)((unsigned long long)v >> 32) + carry;
    if (inc) atomicAdd(hi, inc);
}

// L2 eviction policy for data read once: evicted first, so that the spill
// buckets being filled stay resident and are written back as whole sectors.
__device__ __forceinline__ unsigned long long l2_evict_first_policy() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ int4 ldg_stream_ef(const int4 *p, unsigned long long pol) {
    int4 v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.s32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}

// Hashes of the two-pass group-by.  Fibonacci (multiplicative) hashing: one
// multiply; the high bits index the pass-1 bucket, the bits below them pick
// the spill partition.  Pass 2 uses an independent multiplier.
__device__ __forceinline__ uint32_t gb_h1(uint32_t k) { return k * 0x9E3779B1u; }
__device__ __forceinline__ uint32_t gb_h2(uint32_t k) { return (k ^ (k >> 16)) * 0x85EBCA77u; }

// Word index of slot s's low and high sum halves in a table of `slots` slots.
// SUM64 interleaves them (one 8-byte atomic per add); the carry scheme keeps
// two separate arrays so that the low words of neighbouring slots fall in
// different banks.
template <bool SUM64>
__device__ __forceinline__ uint32_t gb_lo(uint32_t s) { return SUM64 ? 2 * s : s; }
template <bool SUM64>
__device__ __forceinline__ uint32_t gb_hi(uint32_t s, uint32_t slots) { return SUM64 ? 2 * s + 1 : slots + s; }

// Shared-memory accumulator update.  SUM64: one 64-bit shared atomic add;
// otherwise the two-word carry scheme of smem_add_i64.
template <bool SUM64>
__device__ __forceinline__ void gb_acc(uint32_t *cnt, uint32_t *lo, uint32_t *hi, uint32_t add_cnt,
                                       long long v) {
    atomicAdd(cnt, add_cnt);
    if (SUM64) {
        // lo/hi are the two halves of one 8-byte aligned word
        atomicAdd(reinterpret_cast<unsigned long long *>(lo), (unsigned long long)v);
    } else {
        smem_add_i64(lo, hi, v);
    }
}

// Pass 1.  Hot table = S slots in S/4 buckets of 4 ways; one 16-byte shared
// load compares a key against a whole bucket.  sums are interleaved (lo, hi)
// words per slot so that SUM64 can use one 8-byte atomic.
template <bool PRED, bool SUM64>
__global__ void __launch_bounds__(P1_THREADS, 1)
k_gb_part(const int32_t *__restrict__ key, const int32_t *__restrict__ val,
          const int32_t *__restrict__ val2, int32_t lo2, int32_t hi2, long long n, GbSpill sp,
          unsigned int *__restrict__ flags) {
    extern __shared__ __align__(16) unsigned char p1_raw[];
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t s_max;
    const int S = 1 << sp.slog2, P = 1 << sp.plog2;
    const int blog2 = sp.slog2 - 2;
    const uint32_t bshift = 32 - blog2, pshift = 32 - blog2 - sp.plog2, pmask = (uint32_t)P - 1;
    const uint32_t capm = sp.capm;
    uint32_t *hk = reinterpret_cast<uint32_t *>(p1_raw);  // [S], read 4 at a time
    uint32_t *hsum = hk + S;                                // [2S] (lo, hi) per slot
    uint32_t *hc = hsum + 2 * S;                            // [S]
    uint32_t *cur = hc + S;                                 // [P]
    uint32_t *sk = cur + P;                                 // [GB_SKETCH_WORDS]
    const int tid = threadIdx.x;
    for (int i = tid; i < S; i += P1_THREADS) {
        hk[i] = SM_EMPTY;
        hc[i] = 0;
        hsum[gb_lo<SUM64>(i)] = 0;
        hsum[gb_hi<SUM64>(i, S)] = 0;
    }
    for (int i = tid; i < P; i += P1_THREADS) cur[i] = 0;
    for (int i = tid; i < GB_SKETCH_WORDS; i += P1_THREADS) sk[i] = 0;
    if (tid == 0) s_max = 0;
    __syncthreads();
    const int c = blockIdx.x, C = gridDim.x;
    uint2 *mine = sp.miss + (size_t)c * P * capm;
    const unsigned long long pol = l2_evict_first_policy();

    // A row whose key is in the table only adds; any other row goes through
    // admission and, failing that, the spill bucket of its partition.
    auto try_hit = [&](uint32_t uk, int32_t v) -> bool {
        if (uk == SM_EMPTY) return false;
        const uint32_t b = gb_h1(uk) >> bshift;
        const uint4 w = reinterpret_cast<const uint4 *>(hk)[b];
        const int way = (w.x == uk) ? 0 : (w.y == uk) ? 1 : (w.z == uk) ? 2 : (w.w == uk) ? 3 : -1;
        if (way < 0) return false;
        const uint32_t s = b * 4 + way;
        gb_acc<SUM64>(&hc[s], &hsum[gb_lo<SUM64>(s)], &hsum[gb_hi<SUM64>(s, S)], 1u, (long long)v);
        return true;
    };
    auto miss = [&](uint32_t uk, int32_t v) {
        const uint32_t h = gb_h1(uk);
        const uint32_t b = h >> bshift;
        if (uk != SM_EMPTY) {
            const uint4 w = reinterpret_cast<const uint4 *>(hk)[b];
            int way = (w.x == uk) ? 0 : (w.y == uk) ? 1 : (w.z == uk) ? 2 : (w.w == uk) ? 3 : -1;
            if (way < 0) {
                const int e = (w.x == SM_EMPTY) ? 0 : (w.y == SM_EMPTY) ? 1 : (w.z == SM_EMPTY) ? 2
                              : (w.w == SM_EMPTY) ? 3 : -1;
                if (e >= 0) {
                    // Admission on the second sighting (16-bit counters, two per word).
                    const uint32_t sw = (h >> 3) & (GB_SKETCH_WORDS - 1), sh = (h >> 2) & 16u;
                    const uint32_t old = atomicAdd(&sk[sw], 1u << sh);
                    if (((old >> sh) & 0xffffu) != 0) {
                        for (int t = e; t < 4; t++) {
                            const uint32_t cu = atomicCAS(&hk[b * 4 + t], SM_EMPTY, uk);
                            if (cu == SM_EMPTY || cu == uk) { way = t; break; }
                        }
                    }
                }
            }
            if (way >= 0) {
                const uint32_t s = b * 4 + way;
                gb_acc<SUM64>(&hc[s], &hsum[gb_lo<SUM64>(s)], &hsum[gb_hi<SUM64>(s, S)], 1u, (long long)v);
                return;
            }
        }
        const uint32_t p = (h >> pshift) & pmask;
        const uint32_t pos = atomicAdd(&cur[p], 1u);
        if (pos < capm) mine[(size_t)p * capm + pos] = make_uint2(uk, (uint32_t)v);
        else atomicOr(flags, 1u);
    };
    auto process = [&](int32_t k, int32_t v) {
        if (!try_hit((uint32_t)k, v)) miss((uint32_t)k, v);
    };

    const long long nv = n >> 2;
    const long long qb = nv * c / C, qe = nv * (c + 1) / C;
    long long q = qb + tid;
    int4 k4n = make_int4(0, 0, 0, 0), v4n = k4n, w4n = k4n;
    if (q < qe) {
        k4n = ldg_stream_ef(reinterpret_cast<const int4 *>(key) + q, pol);
        v4n = ldg_stream_ef(reinterpret_cast<const int4 *>(val) + q, pol);
        if (PRED) w4n = ldg_stream_ef(reinterpret_cast<const int4 *>(val2) + q, pol);
    }
    for (; q < qe; q += P1_THREADS) {
        const int4 k4 = k4n, v4 = v4n, w4 = w4n;
        const long long qn = q + P1_THREADS;
        if (qn < qe) {  // next vector in flight while this one is processed
            k4n = ldg_stream_ef(reinterpret_cast<const int4 *>(key) + qn, pol);
            v4n = ldg_stream_ef(reinterpret_cast<const int4 *>(val) + qn, pol);
            if (PRED) w4n = ldg_stream_ef(reinterpret_cast<const int4 *>(val2) + qn, pol);
        }
        const int32_t ks[4] = {k4.x, k4.y, k4.z, k4.w};
        const int32_t vs[4] = {v4.x, v4.y, v4.z, v4.w};
        uint32_t live = 0xfu;
        if (PRED) {
            live = (uint32_t)((w4.x >= lo2) & (w4.x <= hi2)) | ((uint32_t)((w4.y >= lo2) & (w4.y <= hi2)) << 1) |
                   ((uint32_t)((w4.z >= lo2) & (w4.z <= hi2)) << 2) | ((uint32_t)((w4.w >= lo2) & (w4.w <= hi2)) << 3);
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
            if ((live >> j) & 1u) process(ks[j], vs[j]);
    }
    if (c == C - 1) {
        for (long long i = (nv << 2) + tid; i < n; i += P1_THREADS) {
            if (PRED && !((val2[i] >= lo2) & (val2[i] <= hi2))) continue;
            process(key[i], val[i]);
        }
    }
    __syncthreads();
    // Fullest bucket (for qg_groupby_stats): reduced in the CTA, then one
    // global atomic per CTA -- a global atomic per bucket would put ~10^5
    // atomics on one address at the kernel's end.
    uint32_t mx = 0;
    for (int p = tid; p < P; p += P1_THREADS) {
        mx = max(mx, cur[p]);
        sp.mcnt[(size_t)p * GB_MAX_C + c] = min(cur[p], capm);
        cur[p] = 0;
    }
    mx = __reduce_max_sync(QG_FULL_MASK, mx);
    if ((tid & 31) == 0 && mx) atomicMax(&s_max, mx);
    __syncthreads();
    if (tid == 0 && s_max) atomicMax(flags + 1, s_max);
    // Counting sort of the shared-memory table by partition.
    for (int s = tid; s < S; s += P1_THREADS)
        if (hc[s]) atomicAdd(&cur[(gb_h1(hk[s]) >> pshift) & pmask], 1u);
    __syncthreads();
    const uint32_t total = block_excl_scan(cur, P, wsum);
    for (int p = tid; p < P; p += P1_THREADS) sp.poff[(size_t)p * GB_MAX_C + c] = cur[p];
    if (tid == 0) sp.poff[(size_t)P * GB_MAX_C + c] = total;
    __syncthreads();
    GPartial *pt = sp.part + (size_t)c * S;
    for (int s = tid; s < S; s += P1_THREADS) {
        if (!hc[s]) continue;
        const uint32_t r = atomicAdd(&cur[(gb_h1(hk[s]) >> pshift) & pmask], 1u);
        GPartial g;
        g.key = hk[s];
        g.cnt = hc[s];
        g.sum = (long long)(((unsigned long long)hsum[gb_hi<SUM64>(s, S)] << 32) | hsum[gb_lo<SUM64>(s)]);
        pt[r] = g;
    }
}

// Pass 2, persistent: each CTA takes partitions from an atomic work counter.
// Table = 2048 slots in 512 buckets of 4 ways (+1 slot for key 0xffffffff);
// a full bucket continues in the next one.
template <bool SUM64>
__global__ void __launch_bounds__(P2_THREADS, 5)
k_gb_merge(GbSpill sp, int C, int32_t *__restrict__ gkey, long long *__restrict__ gsum,
           long long *__restrict__ gcnt, long long cap, unsigned long long *__restrict__ cursor,
           unsigned long long *__restrict__ rec, unsigned int *__restrict__ flags,
           unsigned int *__restrict__ work, uint32_t *__restrict__ ghist, uint32_t *__restrict__ mm,
           uint32_t *__restrict__ bits, uint32_t kbase) {
    constexpr int T = 1 << P2_TLOG2;
    constexpr int NB = T / 4;
    constexpr int W = P2_THREADS / 32;
    __shared__ __align__(16) uint32_t tk[T + 4];
    __shared__ __align__(16) uint32_t tsum[2 * (T + 1)];
    __shared__ uint32_t tc[T + 1];
    __shared__ uint32_t s_part;
    __shared__ uint32_t s_wc[P2_THREADS / 32];
    __shared__ unsigned long long s_base;
    // per source: spill rows, first partial, exclusive prefix of the partial counts
    __shared__ uint32_t s_m[GB_MAX_C], s_q0[GB_MAX_C], s_pp[GB_MAX_C];
    __shared__ uint32_t s_ptot;
    static_assert(GB_MAX_C <= P2_THREADS, "one source per thread");
    __shared__ uint32_t dh[4][256];  // ghist set: digit counts of the emitted keys
    __shared__ uint32_t s_mn, s_mx;   // mm set: smallest and largest emitted key
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int P = 1 << sp.plog2, S = 1 << sp.slog2;
    const uint32_t lt = qg_lanemask_lt();

    auto insert = [&](uint32_t k, uint32_t cnt, long long sum) {
        uint32_t s = T;  // the extra slot holds key 0xffffffff
        if (k != SM_EMPTY) {
            uint32_t b = gb_h2(k) >> (32 - (P2_TLOG2 - 2));
            int found = -1;
            for (int probes = 0; probes < NB && found < 0; probes++) {
                const uint4 w = reinterpret_cast<const uint4 *>(tk)[b];
                found = (w.x == k) ? 0 : (w.y == k) ? 1 : (w.z == k) ? 2 : (w.w == k) ? 3 : -1;
                if (found < 0) {
                    int e = (w.x == SM_EMPTY) ? 0 : (w.y == SM_EMPTY) ? 1 : (w.z == SM_EMPTY) ? 2
                            : (w.w == SM_EMPTY) ? 3 : -1;
                    for (int t = (e < 0 ? 4 : e); t < 4; t++) {
                        const uint32_t cu = atomicCAS(&tk[b * 4 + t], SM_EMPTY, k);
                        if (cu == SM_EMPTY || cu == k) { found = t; break; }
                    }
                }
                if (found < 0) b = (b + 1) & (NB - 1);
            }
            if (found < 0) {
                atomicOr(flags, 2u);
                return;
            }
            s = b * 4 + found;
        } else {
            tk[T] = k;
        }
        gb_acc<SUM64>(&tc[s], &tsum[gb_lo<SUM64>(s)], &tsum[gb_hi<SUM64>(s, T + 1)], cnt, sum);
    };

    if (ghist)
        for (int i = tid; i < 4 * 256; i += P2_THREADS) (&dh[0][0])[i] = 0;
    if (tid == 0) {
        s_mn = 0xffffffffu;
        s_mx = 0;
    }
    uint32_t kmn = 0xffffffffu, kmx = 0;
    while (true) {
        __syncthreads();
        if (tid == 0) s_part = atomicAdd(work, 1u);
        for (int i = tid; i <= T; i += P2_THREADS) {
            tk[i] = SM_EMPTY;
            tc[i] = 0;
            tsum[gb_lo<SUM64>(i)] = 0;
            tsum[gb_hi<SUM64>(i, T + 1)] = 0;
        }
        __syncthreads();
        const uint32_t p = s_part;
        if (p >= (uint32_t)P) break;
        const uint32_t *mcnt = sp.mcnt + (size_t)p * GB_MAX_C;
        const uint32_t *po = sp.poff + (size_t)p * GB_MAX_C;
        const uint32_t *po1 = sp.poff + (size_t)(p + 1) * GB_MAX_C;
        // Every source's spill count and partial range in one round trip (one
        // source per thread), with the exclusive prefix of the partial counts.
        uint32_t pc = 0;
        if (tid < C) {
            s_m[tid] = mcnt[tid];
            const uint32_t q0 = po[tid];
            s_q0[tid] = q0;
            pc = po1[tid] - q0;
        }
        uint32_t pin = pc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(QG_FULL_MASK, pin, d);
            if (lane >= d) pin += v;
        }
        if (lane == 31) s_wc[warp] = pin;
        __syncthreads();
        {
            uint32_t woff = 0, tot = 0;
#pragma unroll
            for (int w = 0; w < W; w++) {
                const uint32_t v = s_wc[w];
                woff += (w < warp) ? v : 0u;
                tot += v;
            }
            if (tid < C) s_pp[tid] = woff + pin - pc;
            if (tid == 0) s_ptot = tot;
        }
        // The first source's spill loads are issued before the partials.
        uint2 rn[4];
        auto first_loads = [&](int cc) {
            if (cc >= C) return;
            const uint32_t m = s_m[cc];
            const uint2 *bk = sp.miss + ((size_t)cc * P + p) * sp.capm;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const uint32_t e = u * 32 + lane;
                rn[u] = e < m ? bk[e] : make_uint2(0, 0);
            }
        };
        first_loads(warp);
        __syncthreads();
        // Partials: a few per source, so they are taken as one flat list over
        // all sources (a source found by binary search over the prefix), with
        // every lane busy.
        const uint32_t ptot = s_ptot;
        for (uint32_t t0 = 0; t0 < ptot; t0 += 2 * P2_THREADS) {
            GPartial y[2];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const uint32_t t = t0 + u * P2_THREADS + tid;
                if (t < ptot) {
                    int lo = 0, hi = C;
                    while (hi - lo > 1) {
                        const int mid = (lo + hi) >> 1;
                        if (s_pp[mid] <= t) lo = mid;
                        else hi = mid;
                    }
                    y[u] = sp.part[(size_t)lo * S + s_q0[lo] + (t - s_pp[lo])];
                }
            }
#pragma unroll
            for (int u = 0; u < 2; u++)
                if (t0 + u * P2_THREADS + tid < ptot) insert(y[u].key, y[u].cnt, y[u].sum);
        }
        // Spill rows: one warp per source CTA, its first 128 rows in one round
        // trip, the rest after.  The warp's next source is loaded before this
        // one is inserted, so that its round trip overlaps.
        for (int cc = warp; cc < C; cc += W) {
            const uint32_t m = s_m[cc];
            const uint2 *bk = sp.miss + ((size_t)cc * P + p) * sp.capm;
            uint2 r[4];
#pragma unroll
            for (int u = 0; u < 4; u++) r[u] = rn[u];
            first_loads(cc + W);
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (u * 32 + lane < m) insert(r[u].x, 1u, (long long)(int32_t)r[u].y);
            for (uint32_t e0 = 128; e0 < m; e0 += 128) {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const uint32_t e = e0 + u * 32 + lane;
                    r[u] = e < m ? bk[e] : make_uint2(0, 0);
                }
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (e0 + u * 32 + lane < m) insert(r[u].x, 1u, (long long)(int32_t)r[u].y);
            }
        }
        __syncthreads();
        // The partition's groups take one range of the output: count them per
        // warp, reserve the range with one global atomic, emit.
        uint32_t wc = 0;
        for (int base = 0; base <= T; base += P2_THREADS) {
            const int s = base + tid;
            wc += __popc(__ballot_sync(QG_FULL_MASK, (s <= T) && tc[s] != 0));
        }
        if (lane == 0) s_wc[warp] = wc;
        __syncthreads();
        if (tid == 0) {
            uint32_t t = 0;
            for (int w = 0; w < P2_THREADS / 32; w++) {
                const uint32_t x = s_wc[w];
                s_wc[w] = t;
                t += x;
            }
            s_base = t ? atomicAdd(cursor, (unsigned long long)t) : 0ull;
        }
        __syncthreads();
        unsigned long long o = s_base + s_wc[warp];
        for (int base = 0; base <= T; base += P2_THREADS) {
            const int s = base + tid;
            const bool occ = (s <= T) && tc[s] != 0;
            const uint32_t b = __ballot_sync(QG_FULL_MASK, occ);
            const unsigned long long o_here = o;
            o += __popc(b);
            if (occ) {
                const long long pos = (long long)o_here + __popc(b & lt);
                if (pos < cap) {
                    gkey[pos] = (int32_t)tk[s];
                    gsum[pos] = (long long)(((unsigned long long)tsum[gb_hi<SUM64>(s, T + 1)] << 32) | tsum[gb_lo<SUM64>(s)]);
                    gcnt[pos] = (long long)tc[s];
                    if (rec) {
                        const uint32_t k = tk[s];
                        rec[pos] = ((unsigned long long)k << 32) | (unsigned long long)pos;
                        if (ghist) {
#pragma unroll
                            for (int d = 0; d < 4; d++) atomicAdd(&dh[d][(k >> (8 * d)) & 255u], 1u);
                        }
                        kmn = min(kmn, k);
                        kmx = max(kmx, k);
                        if (bits) {  // the key's bit in the dense-order window
                            const uint32_t u = k - kbase;
                            if (u < (uint32_t)GB_DENSE_RANGE) atomicOr(&bits[u >> 5], 1u << (u & 31));
                        }
                    }
                }
            }
        }
    }
    // the loop ends for every thread at once (s_part is shared)
    if (ghist) {
        __syncthreads();
        for (int i = tid; i < 4 * 256; i += P2_THREADS)
            if ((&dh[0][0])[i]) atomicAdd(&ghist[i], (&dh[0][0])[i]);
    }
    if (mm) {
        kmn = __reduce_min_sync(QG_FULL_MASK, kmn);
        kmx = __reduce_max_sync(QG_FULL_MASK, kmx);
        if (lane == 0) {
            atomicMin(&s_mn, kmn);
            atomicMax(&s_mx, kmx);
        }
        __syncthreads();
        // mm[0] keeps the largest complement (both words start at zero)
        if (tid == 0 && s_mn <= s_mx) {
            atomicMax(&mm[0], ~s_mn);
            atomicMax(&mm[1], s_mx);
        }
    }
}

// ---------------------------------------------------------------------------
// 2''. key order over a dense key range
//
// A group's place in unsigned key order is the number of present keys below
// it.  The host picks a window [kbase, kbase + GB_DENSE_RANGE) (from the
// context's previous key-ordered call); the merge sets one bit per emitted
// key in a bitmap over that window, and records the smallest and largest key
// it wrote (mm).  When every key fell inside the window, k_gb_dense_scan turns
// the bitmap words of [kmin, kmax] into (bits below this word, word) pairs and
// clears them, and k_gb_dense_place writes each group at its word's prefix
// plus the popcount of the lower bits of its word.  Otherwise the scan clears
// the whole window instead, the place kernel stays idle and the host sorts;
// either way the bitmap arena is all-zero again afterwards.
// ---------------------------------------------------------------------------
constexpr int DN_THREADS = 256;
constexpr int DN_WPT = 8;  // bitmap words per thread and round (two 16-byte loads)

// Did every emitted key fall inside the window?  Then [*w0, *w1] are the
// bitmap words that hold them.  hi < lo means no group at all.
__host__ __device__ __forceinline__ bool gb_dense_fits(uint32_t lo, uint32_t hi, uint32_t kbase, uint32_t *w0,
                                                       uint32_t *w1) {
    if (hi < lo) return false;
    const uint32_t a = lo - kbase, b = hi - kbase;
    if (a > b || b >= (uint32_t)GB_DENSE_RANGE) return false;
    *w0 = a >> 5;
    *w1 = b >> 5;
    return true;
}

// One CTA per chunk of whole 8-word groups of [w0, w1]; chunk c's prefix
// comes from a look-back over chunks 0..c-1 (CTA index = chunk index).
__global__ void __launch_bounds__(DN_THREADS)
k_gb_dense_scan(uint32_t *__restrict__ bits, uint2 *__restrict__ pre, const uint32_t *__restrict__ mm,
                uint32_t kbase, qg_lookback lb) {
    constexpr int NW = DN_THREADS / 32;
    constexpr uint32_t ROUND = DN_THREADS * DN_WPT;
    __shared__ uint32_t s_tile, s_epoch, s_excl;
    __shared__ uint32_t s_woff[NW], s_tmp[2 * NW + 1];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lo_key = ~mm[0], hi_key = mm[1];
    uint32_t w0, w1;
    if (!gb_dense_fits(lo_key, hi_key, kbase, &w0, &w1)) {
        if (hi_key < lo_key) return;  // no group: no bit was set
        // Some keys fell outside the window: clear every bit the merge may
        // have set (the whole window), with no look-back.
        uint4 *b4 = reinterpret_cast<uint4 *>(bits);
        for (size_t i = (size_t)blockIdx.x * DN_THREADS + tid; i < GB_DENSE_WORDS / 4;
             i += (size_t)gridDim.x * DN_THREADS)
            b4[i] = make_uint4(0, 0, 0, 0);
        return;
    }
    const uint32_t g0 = w0 / 8, ng = w1 / 8 + 1 - g0;       // 8-word groups of [w0, w1]
    const uint32_t per = (ng + gridDim.x - 1) / gridDim.x;  // groups per chunk
    qg_lb_begin(lb, &s_tile, &s_epoch);
    const uint32_t tile = s_tile;
    const uint32_t lo = (g0 + min(ng, tile * per)) * 8, hi = (g0 + min(ng, (tile + 1) * per)) * 8;
    auto load8 = [&](uint32_t w, uint32_t *x) {
        const uint4 a = reinterpret_cast<const uint4 *>(bits + w)[0];
        const uint4 b = reinterpret_cast<const uint4 *>(bits + w)[1];
        x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
        x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
    };
    uint32_t c = 0;
    for (uint32_t w = lo + tid * DN_WPT; w < hi; w += ROUND) {
        uint32_t x[DN_WPT];
        load8(w, x);
#pragma unroll
        for (int k = 0; k < DN_WPT; k++) c += __popc(x[k]);
    }
    c = __reduce_add_sync(QG_FULL_MASK, c);
    if (lane == 0) s_woff[warp] = c;
    qg_tile_offsets_wide<NW, NW>(s_woff, lb, tile, s_epoch, &s_excl, s_tmp, nullptr, gridDim.x - 1);
    uint32_t run = s_excl;
    for (uint32_t r0 = lo; r0 < hi; r0 += ROUND) {
        const uint32_t w = r0 + tid * DN_WPT;
        uint32_t x[DN_WPT];
        uint32_t t = 0;
        if (w < hi) {
            load8(w, x);
#pragma unroll
            for (int k = 0; k < DN_WPT; k++) t += __popc(x[k]);
        }
        uint32_t incl = t;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(QG_FULL_MASK, incl, d);
            if (lane >= d) incl += v;
        }
        __syncthreads();  // s_woff of the previous round is read
        if (lane == 31) s_woff[warp] = incl;
        __syncthreads();
        uint32_t before = 0, total = 0;
#pragma unroll
        for (int k = 0; k < NW; k++) {
            const uint32_t v = s_woff[k];
            before += (k < warp) ? v : 0u;
            total += v;
        }
        if (w < hi) {
            uint32_t q = run + before + incl - t;
            uint4 *dst = reinterpret_cast<uint4 *>(pre + w);
#pragma unroll
            for (int k = 0; k < DN_WPT; k += 2) {
                const uint32_t q1 = q + __popc(x[k]);
                dst[k / 2] = make_uint4(q, x[k], q1, x[k + 1]);
                q = q1 + __popc(x[k + 1]);
            }
            reinterpret_cast<uint4 *>(bits + w)[0] = make_uint4(0, 0, 0, 0);
            reinterpret_cast<uint4 *>(bits + w)[1] = make_uint4(0, 0, 0, 0);
        }
        run += total;
    }
    qg_lb_finish(lb, tile, gridDim.x - 1, s_epoch);
}

__global__ void __launch_bounds__(256)
k_gb_dense_place(const unsigned long long *__restrict__ rec, long long cap, const long long *__restrict__ d_n,
                 const uint32_t *__restrict__ mm, uint32_t kbase, const uint2 *__restrict__ pre,
                 const long long *__restrict__ tsum, const long long *__restrict__ tcnt,
                 int32_t *__restrict__ gkey, long long *__restrict__ gsum, long long *__restrict__ gcnt) {
    uint32_t w0, w1;
    if (!gb_dense_fits(~mm[0], mm[1], kbase, &w0, &w1)) return;
    const long long g = *d_n < cap ? *d_n : cap;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g; i += stride) {
        const uint32_t k = (uint32_t)(__ldg(rec + i) >> 32);
        const uint32_t u = k - kbase;
        const uint2 p = __ldg(pre + (u >> 5));
        const uint32_t pos = p.x + __popc(p.y & ((1u << (u & 31)) - 1u));
        gkey[pos] = (int32_t)k;
        gsum[pos] = __ldg(tsum + i);
        gcnt[pos] = __ldg(tcnt + i);
    }
}

}  // namespace

static int grid_for(qg_ctx *ctx, long long work, int per_block, int max_per_sm) {
    long long b = (work + per_block - 1) / per_block;
    long long cap = (long long)ctx->sm_count * max_per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// ---------------------------------------------------------------------------
// host: sorted-contract group-by
// ---------------------------------------------------------------------------
extern "C" QG_API qg_status qg_groupby_rec(qg_ctx *ctx, const void *in, int64_t n, void *sorted_out,
                                           int32_t *startPos, int64_t cap_groups,
                                           int64_t *num_groups) {
    if (!ctx || n < 0 || !num_groups || (n > 0 && (!in || !sorted_out || !startPos)))
        return QG_ERR_INVALID;
    if ((((uintptr_t)in) & 15) || (((uintptr_t)sorted_out) & 15)) return QG_ERR_INVALID;
    if (n > 0x7fffffffLL) return QG_ERR_UNSUPPORTED;
    *num_groups = 0;
    if (n == 0) return QG_OK;
    char *tmp = nullptr;
    QG_TRY(qg_aux(ctx, (size_t)n * 8, &tmp));
    qg_status s = QG_OK;
    if (in != sorted_out)
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(sorted_out, in, (size_t)n * 8, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
    s = qg_sort_rec_inplace(ctx, (unsigned long long *)sorted_out, (unsigned long long *)tmp, n);
    if (s == QG_OK) {
        constexpr int TILE = GBD_THREADS * GBD_ROUNDS * 2;
        int64_t tiles = qg_ceil_div(n, TILE);
        qg_lookback lb;
        s = qg_lb_make(ctx, tiles, QG_SITE_GROUPBY, &lb);
        if (s == QG_OK) {
            long long *d_count = (long long *)&ctx->ctl->counter[0];
            qg_pre_launch(ctx);
            k_group_bounds<<<(unsigned)tiles, GBD_THREADS, 0, ctx->stream>>>(
                (const uint4 *)sorted_out, n, startPos, cap_groups, d_count, lb);
            s = qg_check_launch(ctx, "k_group_bounds");
            long long h = 0;
            if (s == QG_OK) s = qg_read_count(ctx, d_count, &h);
            if (s == QG_OK) {
                *num_groups = h;
                if (h > cap_groups) s = QG_ERR_CAPACITY;
            }
        }
    }
    return s;
}

extern "C" QG_API qg_status qg_aggregate_group_range(qg_ctx *ctx, const void *sorted, int64_t n,
                                                     const int32_t *startPos, int64_t G,
                                                     int64_t first, int64_t count, int op,
                                                     int32_t *agg) {
    if (!ctx || n < 0 || G < 0 || op < 0 || op > 3 || first < 0 || count < 0 || first + count > G)
        return QG_ERR_INVALID;
    if (count == 0) return QG_OK;
    if (!sorted || !startPos || !agg || n == 0) return QG_ERR_INVALID;
    const long long g0 = first, g1 = first + count;
    int ib = grid_for(ctx, count, 256, 8);
    qg_pre_launch(ctx);
    k_agg_init<<<ib, 256, 0, ctx->stream>>>(agg, g0, g1, op);
    QG_TRY(qg_check_launch(ctx, "k_agg_init"));
    // The row range is only known on the device; size the grid for all rows.
    long long chunks = (n + AGG_CHUNK - 1) / AGG_CHUNK;
    int blocks = grid_for(ctx, chunks * 32, 256, 8);
    qg_pre_launch(ctx);
    k_agg_chunks<<<blocks, 256, 0, ctx->stream>>>((const uint2 *)sorted, n, startPos, G, g0, g1, op, agg);
    QG_TRY(qg_check_launch(ctx, "k_agg_chunks"));
    if (op == QG_REDUCE_AVERAGE) {
        qg_pre_launch(ctx);
        k_agg_avg_finish<<<ib, 256, 0, ctx->stream>>>(startPos, n, G, g0, g1, agg);
        QG_TRY(qg_check_launch(ctx, "k_agg_avg_finish"));
    }
    return qg_ctx_check(ctx);
}

extern "C" QG_API qg_status qg_aggregate_groups(qg_ctx *ctx, const void *sorted, int64_t n,
                                                const int32_t *startPos, int64_t G, int op,
                                                int32_t *agg) {
    return qg_aggregate_group_range(ctx, sorted, n, startPos, G, 0, G, op, agg);
}


// ---------------------------------------------------------------------------
// host: column hash group-by
// ---------------------------------------------------------------------------
// Variant (qg_groupby_set_knobs mode): 0 the dense-window path (qg_gbdense.cu)
// first, two-pass when it does not apply; 1 the global table only; 2 two-pass
// with 64-bit shared adds; 3 two-pass.  A steered call may run another.
static int g_gb_knob = 0;
static int g_gb_hot_slog2 = 13;      // pass-1 shared-memory table slots (log2)
static int g_gb_plog2 = 0;           // spill partitions (log2); 0 = chosen from cap
static uint32_t g_gb_capm = 0;       // spill bucket capacity override (0 = automatic)
// 0 (default): int64 sums as two 32-bit words with explicit carry; 1: one
// 64-bit shared atomic per add.  Measured on GB300 (64M rows, Zipf 1M groups):
// pass 1 takes 0.44 ms with the carry scheme and 1.22 ms with 64-bit atomics.
static uint32_t g_gb_last_capm = 0;  // bucket capacity of the last two-pass launch
static const int g_gb_slog2 = 12;    // fallback kernel: shared-memory table slots (log2)

// Path and overflow diagnostics of the context's last qg_groupby_cols call:
// out[0] = 0 two-pass / 1 global table / 2 dense window, out[1] = overflow
// flags (bit 0 spill bucket, bit 1 pass-2 table), out[2] = fullest spill
// bucket, out[3] = bucket capacity (the last three 0 on the dense path).
extern "C" QG_API qg_status qg_groupby_stats(qg_ctx *ctx, uint32_t *out) {
    if (!ctx || !out) return QG_ERR_INVALID;
    for (int i = 0; i < 4; i++) out[i] = ctx->gb_stats[i];
    return QG_OK;
}
static const int g_gb_blocks_per_sm = 2;

int qg_groupby_default_mode() { return g_gb_knob; }

// The variant a call on ctx runs (steered calls of either group-by form set it).
static int gb_mode(const qg_ctx *ctx) {
    const int f = ctx->steer_force[QG_STEER_GROUPBY] >= 0 ? ctx->steer_force[QG_STEER_GROUPBY]
                                                           : ctx->steer_force[QG_STEER_FUSED];
    return f >= 0 ? f : g_gb_knob;
}

extern "C" QG_API qg_status qg_groupby_set_knobs(int mode, int hot_slots_log2, int partitions_log2,
                                                 uint32_t bucket_cap) {
    if (mode < 0 || mode > 3 || hot_slots_log2 < 8 || hot_slots_log2 > 13 || partitions_log2 < 0 ||
        partitions_log2 > 13)
        return QG_ERR_INVALID;
    g_gb_knob = mode;
    g_gb_hot_slog2 = hot_slots_log2;
    g_gb_plog2 = partitions_log2;
    g_gb_capm = bucket_cap;
    return QG_OK;
}

struct GbOut {
    int32_t *k;
    long long *s, *c;
    unsigned long long *rec;  // non-null when the output is sorted afterwards
};

// Where the groups go: the caller's columns, or key-order temporaries in aux.
static qg_status gb_outputs(qg_ctx *ctx, int32_t *gkey, int64_t *gsum, int64_t *gcnt, int64_t cap,
                            int order, GbOut *o) {
    o->k = gkey;
    if (order == QG_ORDER_KEY) {
        // rec | tsum | tcnt | sort ping-pong, in the aux arena so the sort's
        // own scratch use cannot move them.
        char *scr;
        size_t cb = (size_t)(cap > 0 ? cap : 1);
        QG_TRY(qg_aux(ctx, cb * 32, &scr));
        o->rec = (unsigned long long *)scr;
        o->s = (long long *)(o->rec + cb);
        o->c = o->s + cb;
    } else {
        o->rec = nullptr;
        o->s = (long long *)gsum;
        o->c = (long long *)gcnt;
    }
    return QG_OK;
}

// Single-pass global-table path (fallback).
static qg_status gb_launch_global(qg_ctx *ctx, const int32_t *key, const int32_t *val,
                                  const int32_t *val2, int32_t lo2, int32_t hi2, int64_t n,
                                  const GbOut &o, int64_t cap, long long *d_num) {
    uint64_t slots = 1024;
    while (slots < (uint64_t)cap * 2) slots <<= 1;
    if (slots > (1ull << 31)) return QG_ERR_UNSUPPORTED;
    char *tabp;
    QG_TRY(qg_table(ctx, slots * sizeof(GSlot), &tabp));
    GSlot *tab = (GSlot *)tabp;
    const int slog2 = g_gb_slog2;
    const size_t smem = ((size_t)1 << slog2) * 16;
    static bool attr[2] = {false, false};
    const bool pred = val2 != nullptr;
    if (!attr[pred]) {
        if (pred)
            QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_groupby_hash<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
        else
            QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_groupby_hash<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
        attr[pred] = true;
    }
    if (n > 0) {
        int blocks = grid_for(ctx, (n + 3) / 4, GB_THREADS, g_gb_blocks_per_sm);
        qg_pre_launch(ctx);
        if (pred)
            k_groupby_hash<true><<<blocks, GB_THREADS, smem, ctx->stream>>>(
                key, val, val2, lo2, hi2, n, tab, (uint32_t)(slots - 1), slog2, ctx->ctl);
        else
            k_groupby_hash<false><<<blocks, GB_THREADS, smem, ctx->stream>>>(
                key, val, nullptr, 0, 0, n, tab, (uint32_t)(slots - 1), slog2, ctx->ctl);
        QG_TRY(qg_check_launch(ctx, pred ? "k_groupby_hash_fused" : "k_groupby_hash"));
    }
    unsigned long long *cursor = (unsigned long long *)d_num;
    QG_TRY_CUDA(ctx, cudaMemsetAsync(cursor, 0, 8, ctx->stream), "memset cursor");
    int eb = grid_for(ctx, (long long)slots, 256, 8);
    qg_pre_launch(ctx);
    k_groupby_emit<<<eb, 256, 0, ctx->stream>>>(tab, (long long)slots, o.k, o.s, o.c, cap, cursor, o.rec);
    return qg_check_launch(ctx, "k_groupby_emit");
}

// Two-pass path.  *d_flags != 0 afterwards means a spill bucket or a pass-2
// table overflowed and the call must be redone with gb_launch_global.
// Key order: ghist receives the digit counts of the emitted keys (the
// device-planned sort), mm their smallest and largest key, and bits (when
// set) one bit per key of the window [kbase, kbase + GB_DENSE_RANGE) (the
// dense order).
static qg_status gb_launch_twopass(qg_ctx *ctx, const int32_t *key, const int32_t *val,
                                   const int32_t *val2, int32_t lo2, int32_t hi2, int64_t n,
                                   const GbOut &o, int64_t cap, long long *d_num,
                                   unsigned int *d_flags, uint32_t *ghist, uint32_t *mm,
                                   uint32_t *bits = nullptr, uint32_t kbase = 0) {
    int C = ctx->sm_count;
    if (C > GB_MAX_C) C = GB_MAX_C;
    const int slog2 = g_gb_hot_slog2;
    const int S = 1 << slog2;
    int plog2 = g_gb_plog2;
    if (plog2 == 0) {
        // at most ~1024 groups per partition when cap is the true group count
        // (the pass-2 table has 2048 slots)
        plog2 = 6;
        while (plog2 < 13 && ((long long)1 << plog2) * 1024 < cap) plog2++;
    }
    const int P = 1 << plog2;
    const long long rows_per_cta = (n + C - 1) / C;
    // Spill buckets hold 4x the rows a bucket gets when every row spills and
    // hashes evenly; mid-frequency keys that miss the hot table make buckets
    // lumpy, and this headroom keeps the fallback for adversarial orders.
    uint32_t capm = g_gb_capm ? g_gb_capm : (uint32_t)(rows_per_cta * 4 / P + 64);
    g_gb_last_capm = capm;
    // scratch: miss [C][P][capm] uint2 | mcnt [P][GB_MAX_C] | poff [P+1][GB_MAX_C] | part [C][S]
    const size_t miss_b = qg_align_up((size_t)C * P * capm * 8, 256);
    const size_t mcnt_b = qg_align_up((size_t)P * GB_MAX_C * 4, 256);
    const size_t poff_b = qg_align_up((size_t)(P + 1) * GB_MAX_C * 4, 256);
    const size_t part_b = qg_align_up((size_t)C * S * sizeof(GPartial), 256);
    char *scr;
    QG_TRY(qg_scratch(ctx, miss_b + mcnt_b + poff_b + part_b, &scr));
    GbSpill sp;
    sp.miss = (uint2 *)scr;
    sp.mcnt = (uint32_t *)(scr + miss_b);
    sp.poff = (uint32_t *)(scr + miss_b + mcnt_b);
    sp.part = (GPartial *)(scr + miss_b + mcnt_b + poff_b);
    sp.capm = capm;
    sp.plog2 = plog2;
    sp.slog2 = slog2;
    const size_t smem1 = (size_t)S * 16 + (size_t)P * 4 + (size_t)GB_SKETCH_WORDS * 4;
    const bool pred = val2 != nullptr;
    const bool s64 = gb_mode(ctx) == 2;
    auto part = pred ? (s64 ? k_gb_part<true, true> : k_gb_part<true, false>)
                     : (s64 ? k_gb_part<false, true> : k_gb_part<false, false>);
    static size_t attr[4] = {0, 0, 0, 0};
    const int ai = (pred ? 2 : 0) + (s64 ? 1 : 0);
    if (attr[ai] < smem1) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(part, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1), "attr");
        attr[ai] = smem1;
    }
    // d_flags is the low word of one control counter; the pass-2 work counter
    // is the next counter (both cleared together).
    unsigned int *work = d_flags + 2;
    qg_control *ctl = ctx->ctl;
    if ((void *)d_num == (void *)&ctl->counter[1] && (void *)d_flags == (void *)&ctl->counter[2] &&
        (!ghist || ghist == ctl->ghist) && (!mm || mm == (uint32_t *)&ctl->counter[4])) {
        // cursor, flags, work counter and (key order) the key range or the
        // digit counts: one memset from counter[1] on (counters 4 and 5 hold
        // nothing across calls)
        const size_t from = offsetof(qg_control, counter) + 8;
        const size_t to = ghist == ctl->ghist ? offsetof(qg_control, ghist) + sizeof(ctl->ghist)
                          : mm == (uint32_t *)&ctl->counter[4] ? from + 32
                                                                : from + 24;
        QG_TRY_CUDA(ctx, cudaMemsetAsync((char *)ctl + from, 0, to - from, ctx->stream), "memset control");
    } else {
        QG_TRY_CUDA(ctx, cudaMemsetAsync(d_flags, 0, 16, ctx->stream), "memset flags");
        QG_TRY_CUDA(ctx, cudaMemsetAsync(d_num, 0, 8, ctx->stream), "memset cursor");
        if (ghist) QG_TRY_CUDA(ctx, cudaMemsetAsync(ghist, 0, 4 * 256 * 4, ctx->stream), "memset ghist");
        if (mm) QG_TRY_CUDA(ctx, cudaMemsetAsync(mm, 0, 8, ctx->stream), "memset key range");
    }
    qg_pre_launch(ctx);
    part<<<C, P1_THREADS, smem1, ctx->stream>>>(key, val, val2, lo2, hi2, n, sp, d_flags);
    QG_TRY(qg_check_launch(ctx, pred ? "k_gb_part_fused" : "k_gb_part"));
    const int g2 = P < ctx->sm_count * 6 ? P : ctx->sm_count * 6;
    qg_pre_launch(ctx);
    if (s64)
        k_gb_merge<true><<<g2, P2_THREADS, 0, ctx->stream>>>(sp, C, o.k, o.s, o.c, cap,
                                                             (unsigned long long *)d_num, o.rec, d_flags, work,
                                                             ghist, mm, bits, kbase);
    else
        k_gb_merge<false><<<g2, P2_THREADS, 0, ctx->stream>>>(sp, C, o.k, o.s, o.c, cap,
                                                              (unsigned long long *)d_num, o.rec, d_flags, work,
                                                              ghist, mm, bits, kbase);
    return qg_check_launch(ctx, "k_gb_merge");
}

__global__ void k_gb_flags_to_error(const unsigned int *flags, qg_control *ctl) {
    if (*flags) qg_record_error(ctl, QG_ERR_TABLE_FULL, QG_SITE_GROUPBY);
}

// Key order for the two-pass path, planned on the device: the merge counted
// the digits of the keys it wrote (ctl->ghist) and the group count is in
// d_num, so four stable passes over (key, index) records and the gather run
// without a host round trip.  Records past cap were never written, and both
// the passes and the gather stop at min(count, cap).
static qg_status gb_key_order_dev(qg_ctx *ctx, const GbOut &o, int64_t cap, long long *d_num,
                                  int32_t *gkey, int64_t *gsum, int64_t *gcnt) {
    if (cap <= 0) return QG_OK;
    unsigned long long *tmp = o.rec + 3 * cap;  // the aux arena's sort ping-pong (gb_outputs)
    char *work;
    QG_TRY(qg_scratch(ctx, qg_radix_dev_work_bytes(cap), &work));
    qg_sort_bufs A{o.rec, nullptr, nullptr, nullptr}, B{tmp, nullptr, nullptr, nullptr};
    bool in_b = false;
    QG_TRY(qg_radix_passes_dev(ctx, false, A, B, cap, (const unsigned long long *)d_num, ctx->ctl->ghist, 4, 0u,
                               work, &in_b));
    if (in_b) return QG_ERR_INVALID;  // four passes end where they began
    const int gb = grid_for(ctx, cap, 256, 8);
    qg_pre_launch(ctx);
    k_groupby_gather<<<gb, 256, 0, ctx->stream>>>(o.rec, cap, o.s, o.c, gkey, (long long *)gsum,
                                                  (long long *)gcnt, d_num);
    return qg_check_launch(ctx, "k_groupby_gather");
}

// Dense key order after a merge that set the window's bits (see
// k_gb_dense_scan): two launches, the place kernel idle when a key fell
// outside the window.
static qg_status gb_key_order_dense(qg_ctx *ctx, const GbOut &o, int64_t cap, const long long *d_num,
                                    const uint32_t *mm, uint32_t *bits, uint32_t kbase, int32_t *gkey,
                                    int64_t *gsum, int64_t *gcnt) {
    char *prep;
    qg_status st = qg_scratch(ctx, GB_DENSE_WORDS * 8, &prep);
    qg_lookback lb;
    if (st == QG_OK) st = qg_lb_make(ctx, ctx->sm_count, QG_SITE_GROUPBY, &lb);
    if (st == QG_OK) {
        qg_pre_launch(ctx);
        k_gb_dense_scan<<<ctx->sm_count, DN_THREADS, 0, ctx->stream>>>(bits, (uint2 *)prep, mm, kbase, lb);
        st = qg_check_launch(ctx, "k_gb_dense_scan");
    }
    if (st != QG_OK) {
        ctx->table_dirty = true;  // the merge's bits may be left set
        return st;
    }
    if (cap <= 0) return QG_OK;
    const int gb = grid_for(ctx, cap, 256, 8);
    qg_pre_launch(ctx);
    k_gb_dense_place<<<gb, 256, 0, ctx->stream>>>(o.rec, cap, d_num, mm, kbase, (const uint2 *)prep, o.s, o.c,
                                                  gkey, (long long *)gsum, (long long *)gcnt);
    return qg_check_launch(ctx, "k_gb_dense_place");
}

// The next call's window: centred on this call's keys (so that a range that
// moves a little still fits), not below key 0.
static uint32_t gb_dense_next_base(uint32_t lo, uint32_t hi) {
    const uint32_t slack = (uint32_t)((GB_DENSE_RANGE - ((unsigned long long)(hi - lo) + 1)) / 2);
    return lo > slack ? lo - slack : 0u;
}

extern "C" QG_API qg_status qg_groupby_cols_async(qg_ctx *ctx, const int32_t *key,
                                                  const int32_t *val, const int32_t *val2,
                                                  int32_t lo2, int32_t hi2, int64_t n,
                                                  int32_t *gkey, int64_t *gsum, int64_t *gcnt,
                                                  int64_t cap, int order, int64_t *d_num) {
    if (!ctx || n < 0 || cap < 0 || !d_num || (n > 0 && (!key || !val))) return QG_ERR_INVALID;
    if (order != QG_ORDER_NONE && order != QG_ORDER_KEY) return QG_ERR_INVALID;
    // key order is planned on the device by the two-pass path only
    if (order == QG_ORDER_KEY && (gb_mode(ctx) == 1 || cap >= (1LL << 30))) return QG_ERR_UNSUPPORTED;
    if ((((uintptr_t)key) | ((uintptr_t)val) | ((uintptr_t)val2)) & 15) return QG_ERR_INVALID;
    if (n >= (1LL << 32)) return QG_ERR_UNSUPPORTED;
    GbOut o;
    QG_TRY(gb_outputs(ctx, gkey, gsum, gcnt, cap, order, &o));
    if (gb_mode(ctx) == 1)
        return gb_launch_global(ctx, key, val, val2, lo2, hi2, n, o, cap, (long long *)d_num);
    unsigned int *flags = (unsigned int *)&ctx->ctl->counter[2];
    QG_TRY(gb_launch_twopass(ctx, key, val, val2, lo2, hi2, n, o, cap, (long long *)d_num, flags,
                             o.rec ? ctx->ctl->ghist : nullptr, nullptr));
    if (o.rec) QG_TRY(gb_key_order_dev(ctx, o, cap, (long long *)d_num, gkey, gsum, gcnt));
    // An overflow cannot be redone without a host round trip here: report it
    // through the error word (qg_ctx_check returns QG_ERR_TABLE_FULL).
    k_gb_flags_to_error<<<1, 1, 0, ctx->stream>>>(flags, ctx->ctl);
    return qg_check_launch(ctx, "k_gb_flags_to_error");
}

namespace {
// Sync-free dense-window group-by: a row outside the window (which the
// synchronous form would hand to the two-pass path) is reported instead.
__global__ void k_gbd_outside_error(qg_control *ctl) {
    if (ctl->gbd[QG_GBD_OUTSIDE]) qg_record_error(ctl, QG_ERR_UNSUPPORTED, QG_SITE_GROUPBY);
}
}  // namespace

// The dense-window path without a host round trip (batches): output in key
// order, the group count in *d_num; keys outside the sampled window are
// reported as QG_ERR_UNSUPPORTED by qg_ctx_check (nothing valid is written).
qg_status qg_groupby_dense_async(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2,
                                 int32_t lo2, int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum, int64_t *gcnt,
                                 int64_t cap, int64_t *d_num) {
    if (!ctx || n < 0 || cap < 0 || !d_num || (n > 0 && (!key || !val))) return QG_ERR_INVALID;
    if ((((uintptr_t)key) | ((uintptr_t)val) | ((uintptr_t)val2)) & 15) return QG_ERR_INVALID;
    if (n == 0 || n >= (1LL << 32))
        return qg_groupby_cols_async(ctx, key, val, val2, lo2, hi2, n, gkey, gsum, gcnt, cap, QG_ORDER_NONE, d_num);
    QG_TRY(qg_gbd_launch(ctx, key, val, val2, lo2, hi2, n, gkey, gsum, gcnt, cap, (long long *)d_num));
    qg_pre_launch(ctx);
    k_gbd_outside_error<<<1, 1, 0, ctx->stream>>>(ctx->ctl);
    return qg_check_launch(ctx, "k_gbd_outside_error");
}

// One synchronous run of the dense-window path: *ok when every row fell in
// the window (the outputs then hold the result).
qg_status qg_groupby_dense_probe(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2,
                                 int32_t lo2, int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum, int64_t *gcnt,
                                 int64_t cap, int64_t *d_num, bool *ok) {
    *ok = false;
    if (!ctx || n <= 0 || n >= (1LL << 32) || !key || !val || !d_num) return QG_OK;
    if ((((uintptr_t)key) | ((uintptr_t)val) | ((uintptr_t)val2)) & 15) return QG_OK;
    QG_TRY(qg_gbd_launch(ctx, key, val, val2, lo2, hi2, n, gkey, gsum, gcnt, cap, (long long *)d_num));
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pin_ctl, ctx->ctl, offsetof(qg_control, ghist), cudaMemcpyDeviceToHost,
                                     ctx->stream),
                "ctl d2h");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    if (ctx->pin_ctl->err != 0) return qg_collect_error(ctx);
    *ok = ctx->pin_ctl->gbd[QG_GBD_OUTSIDE] == 0;
    return QG_OK;
}

static qg_status groupby_cols_impl(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2,
                                   int32_t lo2, int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum,
                                   int64_t *gcnt, int64_t cap, int order, int64_t *num_groups);

extern "C" QG_API qg_status qg_groupby_cols(qg_ctx *ctx, const int32_t *key, const int32_t *val,
                                            const int32_t *val2, int32_t lo2, int32_t hi2,
                                            int64_t n, int32_t *gkey, int64_t *gsum,
                                            int64_t *gcnt, int64_t cap, int order,
                                            int64_t *num_groups) {
    if (!ctx) return QG_ERR_INVALID;
    // With a cost model attached the variant is its choice for this size; the
    // group count is estimated by the output capacity, the fused predicate's
    // selectivity by the share of the int32 range it keeps.
    qg_steer_call sc;
    const bool fused = val2 != nullptr;
    qg_steer_begin(ctx, fused ? QG_STEER_FUSED : QG_STEER_GROUPBY, n, cap,
                   fused ? ((double)hi2 - (double)lo2 + 1.0) / 4294967296.0 : 1.0, &sc);
    const qg_status st = groupby_cols_impl(ctx, key, val, val2, lo2, hi2, n, gkey, gsum, gcnt, cap, order,
                                           num_groups);
    qg_steer_end(ctx, &sc, st);
    return st;
}

static qg_status groupby_cols_impl(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2,
                                   int32_t lo2, int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum,
                                   int64_t *gcnt, int64_t cap, int order, int64_t *num_groups) {
    if (!ctx || n < 0 || cap < 0 || !num_groups || (n > 0 && (!key || !val)))
        return QG_ERR_INVALID;
    if (order != QG_ORDER_NONE && order != QG_ORDER_KEY) return QG_ERR_INVALID;
    if ((((uintptr_t)key) | ((uintptr_t)val) | ((uintptr_t)val2)) & 15) return QG_ERR_INVALID;
    if (n >= (1LL << 32)) return QG_ERR_UNSUPPORTED;
    long long *d_num = (long long *)&ctx->ctl->counter[1];
    unsigned int *flags = (unsigned int *)&ctx->ctl->counter[2];
    GbOut o;
    QG_TRY(gb_outputs(ctx, gkey, gsum, gcnt, cap, order, &o));
    long long g = 0;
    const int gm = gb_mode(ctx);
    bool global = gm == 1;
    bool done = false;  // the two-pass path wrote the final output (any order)
    // Key order: the dense order unless the context's last key-ordered call
    // found its keys too widely spread, then the device-planned sort (up to
    // 2^30 records).  Whatever neither placed is sorted after the host has
    // read the count.
    if (gm == 0 && !global && n > 0) {
        // Dense-window path: output in key order whatever `order` asks for;
        // one read of the control block brings the error word, the group
        // count and whether every row fell inside the window.
        QG_TRY(qg_gbd_launch(ctx, key, val, val2, lo2, hi2, n, gkey, gsum, gcnt, cap, d_num));
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pin_ctl, ctx->ctl, offsetof(qg_control, ghist),
                                         cudaMemcpyDeviceToHost, ctx->stream),
                    "ctl d2h");
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        if (ctx->pin_ctl->err != 0) return qg_collect_error(ctx);
        const uint32_t outside = ctx->pin_ctl->gbd[QG_GBD_OUTSIDE];
        if (outside == 0) {
            g = (long long)ctx->pin_ctl->counter[1];
            ctx->gb_stats[0] = 2u;
            ctx->gb_stats[1] = ctx->gb_stats[2] = ctx->gb_stats[3] = 0;
            *num_groups = g;
            return g > cap ? QG_ERR_CAPACITY : QG_OK;
        }
        // some key fell outside the sampled window (or the sample spread too
        // wide for one): the two-pass path below writes the output instead
    }
    const bool dense = o.rec && !ctx->gb_wide_keys;
    const bool dev_order = o.rec && !dense && cap < (1LL << 30);
    uint32_t *mm = (uint32_t *)&ctx->ctl->counter[4];
    uint32_t *bits = nullptr;
    const uint32_t kbase = ctx->gb_kbase;
    if (!global) {
        if (dense) {
            char *bitp;
            QG_TRY(qg_table(ctx, GB_DENSE_WORDS * 4, &bitp));
            bits = (uint32_t *)bitp;
        }
        QG_TRY(gb_launch_twopass(ctx, key, val, val2, lo2, hi2, n, o, cap, d_num, flags,
                                 dev_order ? ctx->ctl->ghist : nullptr, o.rec ? mm : nullptr, bits, kbase));
        if (dense) QG_TRY(gb_key_order_dense(ctx, o, cap, d_num, mm, bits, kbase, gkey, gsum, gcnt));
        if (dev_order) QG_TRY(gb_key_order_dev(ctx, o, cap, d_num, gkey, gsum, gcnt));
        // One read of the control block, at the end, brings the error word,
        // the group count (counter[1]) and the overflow flags (counter[2]).
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pin_ctl, ctx->ctl, offsetof(qg_control, ghist),
                                         cudaMemcpyDeviceToHost, ctx->stream),
                    "ctl d2h");
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        if (ctx->pin_ctl->err != 0) return qg_collect_error(ctx);
        g = (long long)ctx->pin_ctl->counter[1];
        const unsigned long long fl = ctx->pin_ctl->counter[2];
        global = (fl & 0xffffffffull) != 0;
        bool placed = dev_order;
        if (o.rec && g > 0) {  // the merge recorded the key range either way
            const uint32_t *pm = (const uint32_t *)&ctx->pin_ctl->counter[4];
            const uint32_t lo = ~pm[0], hi = pm[1];
            const bool fits = hi >= lo && (unsigned long long)(hi - lo) + 1ull <= (unsigned long long)GB_DENSE_RANGE;
            uint32_t w0, w1;
            if (dense) placed = gb_dense_fits(lo, hi, kbase, &w0, &w1);
            ctx->gb_wide_keys = !fits;
            if (fits) ctx->gb_kbase = gb_dense_next_base(lo, hi);
        }
        done = !global && (!o.rec || placed || g == 0);
        ctx->gb_stats[0] = global ? 1u : 0u;
        ctx->gb_stats[1] = (uint32_t)fl;
        ctx->gb_stats[2] = (uint32_t)(fl >> 32);
        ctx->gb_stats[3] = g_gb_last_capm;
    } else {
        ctx->gb_stats[0] = 1u;
        ctx->gb_stats[1] = ctx->gb_stats[2] = ctx->gb_stats[3] = 0;
    }
    if (global) {
        QG_TRY(gb_launch_global(ctx, key, val, val2, lo2, hi2, n, o, cap, d_num));
        QG_TRY(qg_read_count(ctx, d_num, &g));
    }
    *num_groups = g;
    if (g > cap) return QG_ERR_CAPACITY;
    if (done) return QG_OK;
    if (order == QG_ORDER_KEY && g > 1) {
        // Global-table path (or a very large cap): sort (key, index) records,
        // then gather the sums and counts.
        unsigned long long *tmp = (unsigned long long *)(o.c + (cap > 0 ? cap : 1));
        QG_TRY(qg_sort_rec_inplace(ctx, o.rec, tmp, g));
        int gb = grid_for(ctx, g, 256, 8);
        qg_pre_launch(ctx);
        k_groupby_gather<<<gb, 256, 0, ctx->stream>>>(o.rec, g, o.s, o.c, gkey, (long long *)gsum,
                                                      (long long *)gcnt, nullptr);
        QG_TRY(qg_check_launch(ctx, "k_groupby_gather"));
        return qg_ctx_check(ctx);
    } else if (order == QG_ORDER_KEY && g == 1) {
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(gsum, o.s, 8, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(gcnt, o.c, 8, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        return qg_ctx_check(ctx);
    }
    return QG_OK;
}
