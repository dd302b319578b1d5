// qg_gbdense.cu -- column group-by (int64 SUM + COUNT per key, optionally only
// rows with lo2 <= val2 <= hi2) over a direct-indexed key window: the default
// path of qg_groupby_cols.
//
// The reference computes the same groups by sort -> label -> scan -> write ->
// parallelAggregate (kernel/aggregation/1/group_by_cu_op_dp.cl:89-716, host
// testAggAfterGB.cpp:127-255; fused form kernel/filter_aggregation/
// filter_aggregation_cu_op_dp.cl): output in ascending key order, SUM over the
// value column.  Here the key order comes from the table's index order, so no
// sort pass exists.
//
// Four launches, no host round trip until the caller's one read at the end:
//  1. k_gbd_sample -- 2^18 keys (1024 runs of 256 consecutive rows spread over
//                     the column, or every row of a smaller input) are counted
//                     per CTA in shared memory; each CTA adds its distinct
//                     keys' counts to a two-row count-min sketch in L2 (fire-
//                     and-forget reductions) and lists the keys.  The
//                     smallest and largest sampled key are recorded.
//  2. k_gbd_cands  -- every listed key whose sketch count is at least 2 (at
//                     least 1 when the whole input was sampled) bids for the
//                     heavy-key slot its hash selects with one 64-bit atomicMax
//                     of (count << 32 | key): each of the 16384 slots ends up
//                     holding its most frequent candidate.  The key window
//                     [kbase, kbase + 2^22) is centred on the sample's key range
//                     (no window when that range spans more than 2^21 keys).
//  3. k_gbd_main   -- one 1024-thread CTA per SM over a contiguous slice.  The
//                     slot image becomes a read-only direct-mapped table of
//                     window offsets in shared memory, so a row's lookup is one
//                     32-bit shared load, issued for all four rows of a
//                     thread's vector before any update.  A heavy key adds to
//                     its shared count and sum (red.shared, no return); any
//                     other key adds one packed word to dense[key - kbase] in
//                     L2 (red.global.add.u64: count << shift | value).  At the
//                     end the shared table is added to the dense table.
//  4. k_gbd_emit   -- one CTA per SM takes a contiguous chunk of the touched
//                     index range of the dense table, counts its non-empty
//                     entries, finds its output place by a decoupled look-back
//                     over the chunks, and writes every non-empty entry as a
//                     group in key order, clearing the entries (and its share
//                     of the slot image and sketch).
//
// The shared-memory pipeline (L1TEX) bounds the main pass: a row costs about
// one wavefront (its lookup, its shared or global update), which is why the
// lookup is a single 32-bit load rather than a 4-way bucket.
//
// Exactness.  count < 2^C with C = bit length of n, so count << shift with
// shift = 64 - C never overflows.  A value v with 0 <= v <= fast_max adds to
// the packed word's low part, which n * fast_max < 2^shift keeps from
// carrying into the count; a CTA's shared sum stays below 2^32 the same way.
// Any other value (negative or large) adds its sign-extended int64 to
// extra[key - kbase] instead.  So SUM = low part + extra, COUNT = high part,
// bit-exact for every input (int64 two's-complement, as the oracle).
//
// A row whose key falls outside the window is counted in QG_GBD_OUTSIDE; the
// caller then runs the two-pass path instead (the emit still clears the
// table).  The table arena stays all-zero between calls.
#include <stddef.h>

#include "qg_internal.cuh"

namespace {

constexpr int GBD_WLOG2 = 22;
constexpr uint32_t GBD_W = 1u << GBD_WLOG2;       // window keys (dense table entries)
constexpr int GBD_SLOG2 = 14;
constexpr int GBD_S = 1 << GBD_SLOG2;             // heavy-key slots (direct-mapped)
constexpr int GBD_TLOG2 = 19;                     // counters per row of the sample's count sketch
constexpr uint32_t GBD_TMASK = (1u << GBD_TLOG2) - 1;
constexpr int GBD_SAMPLE_RUNS = 1024;
constexpr int GBD_RUN = 256;                      // consecutive rows per sample run
constexpr int GBD_SAMPLE_CTAS = 128;              // runs b, b + 128, ... : at most 8 per CTA
constexpr int GBD_SAMPLE_THREADS = 1024;          // four lanes of 256 threads, two runs each
constexpr int GBD_RUNS_PER_CTA = GBD_SAMPLE_RUNS / GBD_SAMPLE_CTAS;
constexpr int GBD_SSLOTS = 4096;                  // per-CTA sample table (<= 2048 keys)
constexpr int GBD_LIST = GBD_RUNS_PER_CTA * GBD_RUN;  // distinct keys a sample CTA lists (at most)
constexpr int GBD_CANDS_THREADS = 512;
constexpr int GBD_THREADS = 1024;
constexpr uint32_t GBD_EMPTY = 0xffffffffu;

// ctl->gbd word indices
enum {
    G_NSMIN = 0,   // ~(smallest sampled key), by atomicMax
    G_SMAX = 1,    // largest sampled key
    G_OK = 2,      // 1: the window below is valid
    G_KBASE = 3,   // first key of the window
    G_NUMIN = 4,   // ~(smallest window offset of a counted row), by atomicMax
    G_UMAX = 5,    // largest window offset of a counted row
    G_OUTSIDE = QG_GBD_OUTSIDE,  // rows outside the window (or 1 when no window)
    G_EXTRA = 7,   // 1: some value went to the extra (int64) table
    G_BAR = 8,     // k_gbd_single: grid barrier arrivals
    G_WORDS = 9
};
static_assert(G_WORDS <= 48, "gbd state words");
static_assert(GBD_RUNS_PER_CTA * GBD_RUN * 2 <= GBD_SSLOTS, "sample table load <= 1/2");
static_assert(GBD_SSLOTS % GBD_SAMPLE_THREADS == 0 && GBD_RUN % 32 == 0, "the sample's flush walks the table in whole warps");
static_assert(GBD_RUNS_PER_CTA * GBD_RUN == 2 * GBD_SAMPLE_THREADS, "two runs per sample thread");
static_assert(GBD_LIST % GBD_CANDS_THREADS == 0, "cands: whole list per CTA");

// Heavy-key slot of a (raw) key: Fibonacci hashing, top GBD_SLOG2 bits.
__device__ __forceinline__ uint32_t gbd_slot(uint32_t k) { return (k * 0x9E3779B1u) >> (32 - GBD_SLOG2); }

__device__ __forceinline__ void red_global_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("red.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_shared_u32(uint32_t *p, uint32_t v) {
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(qg_smem_u32(p)), "r"(v) : "memory");
}

// The two rows of the sample's count-min sketch: a key's count is the smaller
// of its two counters, never below its true count.
__device__ __forceinline__ uint32_t gbd_h1(uint32_t k) { return qg_hash32(k) & GBD_TMASK; }
__device__ __forceinline__ uint32_t gbd_h2(uint32_t k) { return qg_hash32(k * 0x85EBCA77u + 0x27D4EB2Fu) & GBD_TMASK; }

// 1. Sample.  Run r covers rows [start_r, start_r + 256); CTA b takes runs
// b, b + 128, ..., b + 896, one per 256-thread lane and round.  Each thread
// loads its (up to) two keys first, and the CTA counts them in a shared-memory
// table of 32-bit keys and
// counts (64-bit shared atomics are several times slower).  Each distinct
// key then adds its count to both rows of an L2 count sketch with
// fire-and-forget reductions (no compare-and-swap round trips) and is listed
// in the CTA's segment of `lst`.  The sketch only ranks candidates for the
// heavy-key table, which decides where a row is added, never what it adds,
// so a counter shared by two keys costs speed at most.  Key 0xffffffff is the
// shared table's empty mark and is never a candidate (its rows take the dense
// table like any other key's).
__global__ void __launch_bounds__(GBD_SAMPLE_THREADS)
k_gbd_sample(const int32_t *__restrict__ key, long long n, int runs, bool every_row,
             uint32_t *__restrict__ sketch, uint32_t *__restrict__ lst, uint32_t *__restrict__ lcnt,
             uint32_t *__restrict__ st) {
    __shared__ uint32_t tkey[GBD_SSLOTS], tcnt[GBD_SSLOTS], s_n, s_mm[2];
    for (int i = threadIdx.x; i < GBD_SSLOTS; i += GBD_SAMPLE_THREADS) {
        tkey[i] = GBD_EMPTY;
        tcnt[i] = 0;
    }
    if (threadIdx.x == 0) s_n = 0;
    if (threadIdx.x < 2) s_mm[threadIdx.x] = threadIdx.x == 0 ? 0xffffffffu : 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        // The call's state words that later kernels set start at zero; the
        // sampled key range was cleared by the previous call's candidates
        // kernel (or the context's creation), so no memset precedes this.
        st[G_OK] = 0;
        st[G_KBASE] = 0;
        st[G_NUMIN] = 0;
        st[G_UMAX] = 0;
        st[G_OUTSIDE] = 0;
        st[G_EXTRA] = 0;
    }
    uint32_t k[2];
    bool have[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const int r = blockIdx.x + ((threadIdx.x >> 8) + 4 * j) * GBD_SAMPLE_CTAS;
        const long long start = every_row ? (long long)r * GBD_RUN : (n - GBD_RUN) * (long long)r / (runs - 1);
        const long long i = start + (threadIdx.x & (GBD_RUN - 1));
        have[j] = r < runs && i < n;
        k[j] = have[j] ? (uint32_t)key[i] : 0u;
    }
    __syncthreads();
    uint32_t lmin = 0xffffffffu, lmax = 0;
#pragma unroll
    for (int j = 0; j < 2; j++) {
        if (!have[j]) continue;
        lmin = min(lmin, k[j]);
        lmax = max(lmax, k[j]);
        if (k[j] == GBD_EMPTY) continue;
        // load <= 1/2 (at most 1024 keys), so a free or matching slot exists
        uint32_t h = qg_hash32(k[j]) & (GBD_SSLOTS - 1);
        for (int p = 0; p < GBD_SSLOTS; p++, h = (h + 1) & (GBD_SSLOTS - 1)) {
            const uint32_t old = atomicCAS(&tkey[h], GBD_EMPTY, k[j]);
            if (old == GBD_EMPTY || old == k[j]) {
                atomicAdd(&tcnt[h], 1u);
                break;
            }
        }
    }
    __syncthreads();
    uint32_t *mine = lst + (size_t)blockIdx.x * GBD_LIST;
    const uint32_t lane = threadIdx.x & 31;
    for (int sl = threadIdx.x; sl < GBD_SSLOTS; sl += GBD_SAMPLE_THREADS) {  // whole warps every round
        const uint32_t c = tcnt[sl];
        const uint32_t kk = tkey[sl];
        if (c) {
            atomicAdd(sketch + gbd_h1(kk), c);  // result unused: compiled as a reduction
            atomicAdd(sketch + (1u << GBD_TLOG2) + gbd_h2(kk), c);
        }
        // one list reservation per warp (a single shared counter would serialise the keys)
        const uint32_t m = __ballot_sync(QG_FULL_MASK, c != 0u);
        uint32_t at = 0;
        if (lane == 0 && m) at = atomicAdd(&s_n, (uint32_t)__popc(m));
        at = __shfl_sync(QG_FULL_MASK, at, 0);
        if (c) mine[at + __popc(m & qg_lanemask_lt())] = kk;
    }
    lmin = __reduce_min_sync(QG_FULL_MASK, lmin);
    lmax = __reduce_max_sync(QG_FULL_MASK, lmax);
    if ((threadIdx.x & 31) == 0 && lmin <= lmax) {  // one global pair per CTA, not per warp
        atomicMin(&s_mm[0], lmin);
        atomicMax(&s_mm[1], lmax);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        lcnt[blockIdx.x] = s_n;
        if (s_mm[0] <= s_mm[1]) {
            atomicMax(&st[G_NSMIN], ~s_mm[0]);
            atomicMax(&st[G_SMAX], s_mm[1]);
        }
    }
}

// 2. Candidates bid for their slots; the window.  CTA b reads sample CTA b's
// list.  A key listed by several sample CTAs bids several times with the
// same word, which atomicMax makes harmless.
__global__ void __launch_bounds__(GBD_CANDS_THREADS)
k_gbd_cands(const uint32_t *__restrict__ sketch, const uint32_t *__restrict__ lst,
            const uint32_t *__restrict__ lcnt, unsigned long long *__restrict__ img, uint32_t min_count,
            uint32_t *__restrict__ st) {
    const uint32_t m = lcnt[blockIdx.x];
    const uint32_t *mine = lst + (size_t)blockIdx.x * GBD_LIST;
    constexpr int PER = GBD_LIST / GBD_CANDS_THREADS;
    uint32_t kk[PER], c[PER];
#pragma unroll
    for (int j = 0; j < PER; j++) {  // all lookups in flight before any bid
        const uint32_t i = j * GBD_CANDS_THREADS + threadIdx.x;
        kk[j] = i < m ? mine[i] : 0u;
        c[j] = i < m ? min(sketch[gbd_h1(kk[j])], sketch[(1u << GBD_TLOG2) + gbd_h2(kk[j])]) : 0u;
    }
#pragma unroll
    for (int j = 0; j < PER; j++)  // the image word orders candidates by count, ties by key
        if (c[j] >= min_count && c[j] > 0) atomicMax(img + gbd_slot(kk[j]), ((unsigned long long)c[j] << 32) | kk[j]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t smin = ~st[G_NSMIN], smax = st[G_SMAX];
        st[G_NSMIN] = 0;  // cleared for the next call's sample (nothing else reads them)
        st[G_SMAX] = 0;
        if (smin <= smax) {
            const unsigned long long span = (unsigned long long)(smax - smin) + 1ull;
            if (span <= GBD_W / 2) {
                const unsigned long long slack = (GBD_W - span) / 2;
                unsigned long long kb = smin > slack ? smin - slack : 0ull;
                if (kb + GBD_W > (1ull << 32)) kb = (1ull << 32) - GBD_W;
                st[G_KBASE] = (uint32_t)kb;
                st[G_OK] = 1u;
            }
        }
    }
}

// 3. Main pass: the body, shared by k_gbd_main and k_gbd_single.  `raw` is
// the 192 KB of dynamic shared memory; img is read through L2 (the single
// launch wrote it moments before).
template <bool PRED>
__device__ __forceinline__ void gbd_main_body(const int32_t *__restrict__ key, const int32_t *__restrict__ val,
                                              const int32_t *__restrict__ val2, int32_t lo2, int32_t hi2, long long n,
                                              const unsigned long long *img, uint32_t kbase, uint32_t *st,
                                              unsigned long long *dense, long long *extra, uint32_t shift,
                                              uint32_t fast_max, unsigned char *raw, uint32_t *s_red) {
    uint32_t *hk = reinterpret_cast<uint32_t *>(raw);  // [GBD_S] window offsets, EMPTY if none
    uint32_t *hc = hk + GBD_S;                           // [GBD_S] counts
    uint32_t *hl = hc + GBD_S;                           // [GBD_S] sums of fast values
    const int tid = threadIdx.x;
    for (int i = tid; i < GBD_S; i += GBD_THREADS) {
        const unsigned long long w = __ldcg(img + i);
        // a candidate is a sampled key, and the window covers the sample
        hk[i] = w ? (uint32_t)w - kbase : GBD_EMPTY;
        hc[i] = 0;
        hl[i] = 0;
    }
    if (tid < 4) s_red[tid] = tid == 0 ? 0xffffffffu : 0u;
    __syncthreads();
    uint32_t umin = 0xffffffffu, umax = 0, outside = 0, extra_used = 0;
    const unsigned long long one = 1ull << shift;
    auto row = [&](uint32_t u, uint32_t s, uint32_t w, int32_t v) {
        if (u >= GBD_W) {
            outside++;
            return;
        }
        umin = min(umin, u);
        umax = max(umax, u);
        const bool fast = (uint32_t)v <= fast_max;
        if (w == u) {
            red_shared_u32(&hc[s], 1u);
            if (fast) red_shared_u32(&hl[s], (uint32_t)v);
        } else {
            red_global_u64(dense + u, one + (fast ? (unsigned long long)(uint32_t)v : 0ull));
        }
        if (!fast) {
            red_global_u64(reinterpret_cast<unsigned long long *>(extra) + u, (unsigned long long)(long long)v);
            extra_used = 1;
        }
    };
    const long long nv = n >> 2;
    const long long qb = nv * blockIdx.x / gridDim.x, qe = nv * (blockIdx.x + 1) / gridDim.x;
    const int4 *k4p = reinterpret_cast<const int4 *>(key);
    const int4 *v4p = reinterpret_cast<const int4 *>(val);
    const int4 *w4p = reinterpret_cast<const int4 *>(val2);
    long long q = qb + tid;
    int4 k4n = make_int4(0, 0, 0, 0), v4n = k4n, w4n = k4n;
    if (q < qe) {
        k4n = qg_ldg_stream(k4p + q);
        v4n = qg_ldg_stream(v4p + q);
        if (PRED) w4n = qg_ldg_stream(w4p + q);
    }
    for (; q < qe; q += GBD_THREADS) {
        const int4 k4 = k4n, v4 = v4n, w4 = w4n;
        if (q + GBD_THREADS < qe) {  // the next vector in flight while this one is processed
            k4n = qg_ldg_stream(k4p + q + GBD_THREADS);
            v4n = qg_ldg_stream(v4p + q + GBD_THREADS);
            if (PRED) w4n = qg_ldg_stream(w4p + q + GBD_THREADS);
        }
        const uint32_t ks[4] = {(uint32_t)k4.x, (uint32_t)k4.y, (uint32_t)k4.z, (uint32_t)k4.w};
        const int32_t vs[4] = {v4.x, v4.y, v4.z, v4.w};
        uint32_t live = 0xfu;
        if (PRED) {
            live = (uint32_t)((w4.x >= lo2) & (w4.x <= hi2)) | ((uint32_t)((w4.y >= lo2) & (w4.y <= hi2)) << 1) |
                   ((uint32_t)((w4.z >= lo2) & (w4.z <= hi2)) << 2) | ((uint32_t)((w4.w >= lo2) & (w4.w <= hi2)) << 3);
        }
        uint32_t s[4], w[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {  // the table is read-only: all four lookups first
            s[j] = gbd_slot(ks[j]);
            w[j] = hk[s[j]];
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
            if ((live >> j) & 1u) row(ks[j] - kbase, s[j], w[j], vs[j]);
    }
    if (blockIdx.x == gridDim.x - 1) {
        for (long long i = (nv << 2) + tid; i < n; i += GBD_THREADS) {
            if (PRED && !((val2[i] >= lo2) & (val2[i] <= hi2))) continue;
            const uint32_t k = (uint32_t)key[i], s = gbd_slot(k);
            row(k - kbase, s, hk[s], val[i]);
        }
    }
    umin = __reduce_min_sync(QG_FULL_MASK, umin);
    umax = __reduce_max_sync(QG_FULL_MASK, umax);
    outside = __reduce_add_sync(QG_FULL_MASK, outside);
    extra_used = __reduce_or_sync(QG_FULL_MASK, extra_used);
    if ((tid & 31) == 0) {
        atomicMin(&s_red[0], umin);
        atomicMax(&s_red[1], umax);
        if (outside) atomicAdd(&s_red[2], outside);
        if (extra_used) s_red[3] = 1u;
    }
    __syncthreads();
    // The CTA's heavy keys join the dense table (count and fast-value sum packed).
    for (int i = tid; i < GBD_S; i += GBD_THREADS)
        if (hc[i]) red_global_u64(dense + hk[i], ((unsigned long long)hc[i] << shift) + hl[i]);
    if (tid == 0) {
        if (s_red[0] <= s_red[1]) {
            atomicMax(&st[G_NUMIN], ~s_red[0]);
            atomicMax(&st[G_UMAX], s_red[1]);
        }
        if (s_red[2]) atomicAdd(&st[G_OUTSIDE], s_red[2]);
        if (s_red[3]) atomicOr(&st[G_EXTRA], 1u);
    }
}

template <bool PRED>
__global__ void __launch_bounds__(GBD_THREADS, 1)
k_gbd_main(const int32_t *__restrict__ key, const int32_t *__restrict__ val, const int32_t *__restrict__ val2,
           int32_t lo2, int32_t hi2, long long n, const unsigned long long *__restrict__ img,
           uint32_t *__restrict__ st, unsigned long long *__restrict__ dense, long long *__restrict__ extra,
           uint32_t shift, uint32_t fast_max) {
    extern __shared__ __align__(16) unsigned char gbd_main_raw[];
    __shared__ uint32_t s_red[4];
    if (!st[G_OK]) {  // no window: the caller takes the two-pass path
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st[G_OUTSIDE], 1u);
        return;
    }
    gbd_main_body<PRED>(key, val, val2, lo2, hi2, n, img, st[G_KBASE], st, dense, extra, shift, fast_max,
                        gbd_main_raw, s_red);
}

// 4. Emit in key order.  One 1024-thread CTA per SM; the touched index
// range [umin, umax] is split into one contiguous chunk per CTA (chunk ids in
// CTA start order).  A CTA counts its chunk's non-empty entries, publishes the
// count to a decoupled look-back over the chunks (one wide round reads 256
// predecessors, so no chain of waits forms), and then writes its groups from
// that place on, in tiles of 8192 entries (8 per thread; the (round, warp)
// cells ranked in row order), clearing the entries as it goes.  Every CTA also
// clears its share of the slot image and the sample's sketch.
constexpr int GBD_EPER = 8;  // emit entries per thread and tile
constexpr int GBD_ETILE = GBD_THREADS * GBD_EPER;
constexpr int GBD_ENW = GBD_THREADS / 32;
static_assert(GBD_EPER * GBD_ENW == 8 * 32, "emit cells: 8 per lane of warp 0");

struct GbdChunk {
    unsigned long long cb, ce;  // entries [cb, ce) of the dense table
};

// Chunk c of C over the touched range (empty when nothing was counted).
__device__ __forceinline__ GbdChunk gbd_chunk(uint32_t c, uint32_t C, bool any, uint32_t umin, uint32_t hi) {
    const unsigned long long len = any ? (unsigned long long)(hi - umin) + 1ull : 0ull;
    const unsigned long long ch = ((len + C - 1) / C + 31) & ~31ull;
    const unsigned long long cb = (unsigned long long)umin + c * ch;
    return {cb, min(cb + ch, (unsigned long long)umin + len)};
}

// Clear this CTA's share (CTA c of C) of the slot image and the sketch.
__device__ __forceinline__ void gbd_clear_sample(unsigned long long *img, uint32_t *sketch, uint32_t c, uint32_t C) {
    for (uint32_t i = c * GBD_THREADS + threadIdx.x; i < (uint32_t)GBD_S; i += C * GBD_THREADS) img[i] = 0ull;
    uint4 *sk4 = reinterpret_cast<uint4 *>(sketch);
    constexpr uint32_t W4 = (2u << GBD_TLOG2) / 4;
    for (uint32_t i = c * GBD_THREADS + threadIdx.x; i < W4; i += C * GBD_THREADS) sk4[i] = make_uint4(0, 0, 0, 0);
}

// Non-empty entries of a chunk, summed over the CTA (every thread gets it).
__device__ __forceinline__ uint32_t gbd_chunk_count(const unsigned long long *dense, GbdChunk k, uint32_t *s_wsum) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t cnt = 0;
    for (unsigned long long t0 = k.cb; t0 < k.ce; t0 += GBD_ETILE) {
        unsigned long long e[GBD_EPER];
#pragma unroll
        for (int r = 0; r < GBD_EPER; r++) {
            const unsigned long long i = t0 + r * GBD_THREADS + tid;
            e[r] = i < k.ce ? __ldcg(dense + i) : 0ull;
        }
#pragma unroll
        for (int r = 0; r < GBD_EPER; r++) cnt += e[r] != 0ull;
    }
    cnt = __reduce_add_sync(QG_FULL_MASK, cnt);
    if (lane == 0) s_wsum[warp] = cnt;
    __syncthreads();
    const uint32_t t = __reduce_add_sync(QG_FULL_MASK, s_wsum[lane]);
    __syncthreads();
    return t;
}

// Writes a chunk's groups from output place `base` on and clears its entries.
__device__ __forceinline__ void gbd_chunk_write(unsigned long long *dense, long long *extra, GbdChunk k,
                                                unsigned long long base, uint32_t kbase, bool xtra, uint32_t shift,
                                                int32_t *__restrict__ gkey, long long *__restrict__ gsum,
                                                long long *__restrict__ gcnt, long long cap, uint32_t *s_off,
                                                uint32_t *s_tot) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned long long mask = (1ull << shift) - 1ull;
    for (unsigned long long t0 = k.cb; t0 < k.ce; t0 += GBD_ETILE) {
        unsigned long long e[GBD_EPER];
#pragma unroll
        for (int r = 0; r < GBD_EPER; r++) {
            const unsigned long long i = t0 + r * GBD_THREADS + tid;
            e[r] = i < k.ce ? __ldcg(dense + i) : 0ull;
            const uint32_t m = __ballot_sync(QG_FULL_MASK, e[r] != 0ull);
            if (lane == 0) s_off[r * GBD_ENW + warp] = __popc(m);
        }
        __syncthreads();
        if (warp == 0) {  // exclusive offsets of the (round, warp) cells in row order
            uint32_t c[8], sum = 0;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                c[q] = s_off[lane * 8 + q];
                sum += c[q];
            }
            uint32_t incl = sum;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t x = __shfl_up_sync(QG_FULL_MASK, incl, d);
                if (lane >= d) incl += x;
            }
            uint32_t run = incl - sum;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                s_off[lane * 8 + q] = run;
                run += c[q];
            }
            if (lane == 31) *s_tot = incl;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < GBD_EPER; r++) {
            const uint32_t m = __ballot_sync(QG_FULL_MASK, e[r] != 0ull);
            if (e[r] == 0ull) continue;
            const unsigned long long i = t0 + r * GBD_THREADS + tid;
            const long long pos = (long long)(base + s_off[r * GBD_ENW + warp] + __popc(m & qg_lanemask_lt()));
            long long sm = (long long)(e[r] & mask);
            if (xtra) {
                sm += __ldcg(extra + i);
                extra[i] = 0;
            }
            if (pos < cap) {
                gkey[pos] = (int32_t)(kbase + (uint32_t)i);
                gsum[pos] = sm;
                gcnt[pos] = (long long)(e[r] >> shift);
            }
            dense[i] = 0ull;
        }
        base += *s_tot;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(GBD_THREADS)
k_gbd_emit(unsigned long long *__restrict__ dense, long long *__restrict__ extra,
           unsigned long long *__restrict__ img, uint32_t *__restrict__ sketch, const uint32_t *__restrict__ st,
           uint32_t shift, int32_t *__restrict__ gkey, long long *__restrict__ gsum, long long *__restrict__ gcnt,
           long long cap, long long *__restrict__ d_num, qg_lookback lb) {
    __shared__ uint32_t s_tile, s_epoch, s_tot, s_wsum[GBD_ENW], s_off[GBD_EPER * GBD_ENW], s_tmp[2 * 8];
    gbd_clear_sample(img, sketch, blockIdx.x, gridDim.x);
    qg_lb_begin_dyn(lb, &s_tile, &s_epoch);  // chunk ids in CTA start order: predecessors are running
    const uint32_t chunk = s_tile, epoch = s_epoch, C = gridDim.x;
    const uint32_t umin = ~st[G_NUMIN], hi = st[G_UMAX];
    const bool any = st[G_OK] && umin <= hi;
    const GbdChunk k = gbd_chunk(chunk, C, any, umin, hi);
    const uint32_t total = gbd_chunk_count(dense, k, s_wsum);
    if (threadIdx.x < 8 * 32) {  // the wide look-back: 256 predecessors per round
        const uint32_t excl = qg_lb_wide_exclusive<8>(lb, chunk, epoch, total, s_tmp);
        if (threadIdx.x == 0) {
            s_wsum[0] = excl;
            if (chunk == C - 1) *d_num = (long long)excl + total;
        }
    }
    __syncthreads();
    gbd_chunk_write(dense, extra, k, s_wsum[0], st[G_KBASE], st[G_EXTRA] != 0u, shift, gkey, gsum, gcnt, cap, s_off,
                    &s_tot);
    // The last chunk ends after every earlier chunk published (its look-back
    // waited for them), and every CTA took its chunk before that.
    qg_lb_finish_dyn(lb, chunk, C - 1, epoch);
}


// ---------------------------------------------------------------------------
// The four steps in one cooperative launch (k_gbd_single): one 1024-thread
// CTA per SM runs the sample, the candidates, the main pass and the emit,
// with a grid barrier between them, so the short steps use every SM at full
// occupancy instead of a few latency-bound CTAs each, and no launch gap
// separates them.
//   A  sample: CTA b takes runs b, b + C, ... (at most 8, C >= 128); its
//      distinct keys stay in its shared table (4096 slots, load <= 1/2).
//   B  candidates: each CTA bids for its own distinct keys (the sketch is
//      complete after the barrier); every CTA derives the window itself.
//   C  main pass (gbd_main_body).
//   D  emit: the touched range splits into C contiguous chunks; each CTA
//      counts its chunk's groups, and after a barrier places them at the sum
//      of the earlier chunks' counts, in tiles of 8192 entries held in
//      registers.  The sketch, slot image and entries are cleared as before.
// Every barrier wait is bounded (QG_ERR_TIMEOUT); the barrier counter lives
// in the per-call state words the host clears before the launch.
// ---------------------------------------------------------------------------
constexpr int GBD1_SSLOTS = 4096;   // per-CTA sample table: up to 8 runs = 2048 keys
constexpr int GBD1_MAX_RUNS = 8;    // runs per CTA (2 per thread)
static_assert(GBD1_SSLOTS * 8 <= GBD_S * 12, "sample table inside the main pass's shared memory");
static_assert(GBD1_MAX_RUNS * GBD_RUN * 2 <= GBD1_SSLOTS, "sample table load <= 1/2");
static_assert(GBD_THREADS == 4 * GBD_RUN, "four run lanes per CTA");

__device__ __forceinline__ bool gbd_grid_sync(uint32_t *bar, uint32_t target, uint32_t spin_limit, qg_control *ctl,
                                              volatile uint32_t *s_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        uint32_t ok = 1u, polls = 0;
        while (qg_ld_relaxed_u32(bar) < target) {
            if (polls++ >= spin_limit) {
                qg_record_error(ctl, QG_ERR_TIMEOUT, QG_SITE_GROUPBY);
                ok = 0u;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0u;
}

template <bool PRED>
__global__ void __launch_bounds__(GBD_THREADS, 1)
k_gbd_single(const int32_t *__restrict__ key, const int32_t *__restrict__ val, const int32_t *__restrict__ val2,
             int32_t lo2, int32_t hi2, long long n, int runs, bool every_row, uint32_t *sketch,
             unsigned long long *img, uint32_t *st, unsigned long long *dense, long long *extra, uint32_t shift,
             uint32_t fast_max, int32_t *__restrict__ gkey, long long *__restrict__ gsum,
             long long *__restrict__ gcnt, long long cap, long long *d_num, uint32_t *counts, qg_control *ctl,
             uint32_t spin_limit) {
    extern __shared__ __align__(16) unsigned char gbd_main_raw[];
    __shared__ uint32_t s_red[4], s_wsum[GBD_ENW], s_off[GBD_EPER * GBD_ENW];
    __shared__ volatile uint32_t s_ok;
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_tot;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t C = gridDim.x, b = blockIdx.x;

    // A. sample
    uint32_t *tkey = reinterpret_cast<uint32_t *>(gbd_main_raw), *tcnt = tkey + GBD1_SSLOTS;
    for (int i = tid; i < GBD1_SSLOTS; i += GBD_THREADS) {
        tkey[i] = GBD_EMPTY;
        tcnt[i] = 0;
    }
    if (tid < 2) s_red[tid] = tid == 0 ? 0xffffffffu : 0u;
    uint32_t k[2];
    bool have[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const long long r = (long long)b + (long long)((tid >> 8) + 4 * j) * C;
        const long long start = every_row ? r * GBD_RUN : (n - GBD_RUN) * r / (runs - 1);
        const long long i = start + (tid & (GBD_RUN - 1));
        have[j] = r < runs && i < n;
        k[j] = have[j] ? (uint32_t)key[i] : 0u;
    }
    __syncthreads();
    uint32_t lmin = 0xffffffffu, lmax = 0;
#pragma unroll
    for (int j = 0; j < 2; j++) {
        if (!have[j]) continue;
        lmin = min(lmin, k[j]);
        lmax = max(lmax, k[j]);
        if (k[j] == GBD_EMPTY) continue;
        uint32_t h = qg_hash32(k[j]) & (GBD1_SSLOTS - 1);
        for (int p = 0; p < GBD1_SSLOTS; p++, h = (h + 1) & (GBD1_SSLOTS - 1)) {
            const uint32_t old = atomicCAS(&tkey[h], GBD_EMPTY, k[j]);
            if (old == GBD_EMPTY || old == k[j]) {
                atomicAdd(&tcnt[h], 1u);
                break;
            }
        }
    }
    __syncthreads();
    for (int sl = tid; sl < GBD1_SSLOTS; sl += GBD_THREADS) {
        const uint32_t c = tcnt[sl];
        if (c) {
            const uint32_t kk = tkey[sl];
            atomicAdd(sketch + gbd_h1(kk), c);
            atomicAdd(sketch + (1u << GBD_TLOG2) + gbd_h2(kk), c);
        }
    }
    // the sampled key range: one pair of global atomics per CTA (atomics on
    // one address from every warp of the grid would queue at its L2 slice)
    lmin = __reduce_min_sync(QG_FULL_MASK, lmin);
    lmax = __reduce_max_sync(QG_FULL_MASK, lmax);
    if (lane == 0 && lmin <= lmax) {
        atomicMin(&s_red[0], lmin);
        atomicMax(&s_red[1], lmax);
    }
    __syncthreads();
    if (tid == 0 && s_red[0] <= s_red[1]) {
        atomicMax(&st[G_NSMIN], ~s_red[0]);
        atomicMax(&st[G_SMAX], s_red[1]);
    }
    if (!gbd_grid_sync(&st[G_BAR], C, spin_limit, ctl, &s_ok)) return;

    // B. candidates and the window
    const uint32_t smin = ~__ldcg(&st[G_NSMIN]), smax = __ldcg(&st[G_SMAX]);
    bool ok = false;
    uint32_t kbase = 0;
    if (smin <= smax) {
        const unsigned long long span = (unsigned long long)(smax - smin) + 1ull;
        if (span <= GBD_W / 2) {
            const unsigned long long slack = (GBD_W - span) / 2;
            unsigned long long kb = smin > slack ? smin - slack : 0ull;
            if (kb + GBD_W > (1ull << 32)) kb = (1ull << 32) - GBD_W;
            kbase = (uint32_t)kb;
            ok = true;
        }
    }
    if (b == 0 && tid == 0) {
        st[G_KBASE] = kbase;
        st[G_OK] = ok ? 1u : 0u;
        if (!ok) atomicAdd(&st[G_OUTSIDE], 1u);  // no window: the caller takes the two-pass path
    }
    const uint32_t min_count = every_row ? 1u : 2u;
    for (int sl = tid; sl < GBD1_SSLOTS; sl += GBD_THREADS) {
        const uint32_t kk = tkey[sl];
        if (!tcnt[sl]) continue;
        const uint32_t c = min(__ldcg(sketch + gbd_h1(kk)), __ldcg(sketch + (1u << GBD_TLOG2) + gbd_h2(kk)));
        if (c >= min_count) atomicMax(img + gbd_slot(kk), ((unsigned long long)c << 32) | kk);
    }
    if (!gbd_grid_sync(&st[G_BAR], 2 * C, spin_limit, ctl, &s_ok)) return;
    if (b == 0 && tid == 0) {  // every CTA has read the sampled key range: cleared for a four-launch call
        st[G_NSMIN] = 0;
        st[G_SMAX] = 0;
    }

    // C. main pass
    if (ok) gbd_main_body<PRED>(key, val, val2, lo2, hi2, n, img, kbase, st, dense, extra, shift, fast_max,
                                gbd_main_raw, s_red);
    if (!gbd_grid_sync(&st[G_BAR], 3 * C, spin_limit, ctl, &s_ok)) return;

    // D. emit: count this CTA's chunk, then (after a barrier) place its groups
    // after the earlier chunks' counts.
    gbd_clear_sample(img, sketch, b, C);
    const uint32_t umin = ~__ldcg(&st[G_NUMIN]), hi = __ldcg(&st[G_UMAX]);
    const bool xtra = __ldcg(&st[G_EXTRA]) != 0u;
    const GbdChunk ck = gbd_chunk(b, C, ok && umin <= hi, umin, hi);
    const uint32_t cnt = gbd_chunk_count(dense, ck, s_wsum);
    if (tid == 0) __stcg(counts + b, cnt);
    if (!gbd_grid_sync(&st[G_BAR], 4 * C, spin_limit, ctl, &s_ok)) return;
    if (warp == 0) {
        unsigned long long before = 0, all = 0;
        for (uint32_t j = lane; j < C; j += 32) {
            const uint32_t c = __ldcg(counts + j);
            all += c;
            if (j < b) before += c;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            before += __shfl_down_sync(QG_FULL_MASK, before, d);
            all += __shfl_down_sync(QG_FULL_MASK, all, d);
        }
        if (lane == 0) {
            s_base = before;
            if (b == 0) *d_num = (long long)all;
        }
    }
    __syncthreads();
    gbd_chunk_write(dense, extra, ck, s_base, kbase, xtra, shift, gkey, gsum, gcnt, cap, s_off, &s_tot);
}

}  // namespace

static int g_gbd_single = 0;  // 1: the four steps in one cooperative launch where it fits

extern "C" QG_API qg_status qg_groupby_set_single_launch(int enable) {
    if (enable != 0 && enable != 1) return QG_ERR_INVALID;
    g_gbd_single = enable;
    return QG_OK;
}

qg_status qg_gbd_launch(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2, int32_t lo2,
                        int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum, int64_t *gcnt, int64_t cap,
                        long long *d_num) {
    // table arena (kept all-zero between calls):
    //   dense [W] u64 | extra [W] i64 | sample sketch [2][2^19] u32 | slot image [GBD_S] u64
    const size_t dense_b = (size_t)GBD_W * 8, sk_b = ((size_t)2 << GBD_TLOG2) * 4, img_b = (size_t)GBD_S * 8;
    char *tab;
    QG_TRY(qg_table(ctx, 2 * dense_b + sk_b + img_b, &tab));
    unsigned long long *dense = (unsigned long long *)tab;
    long long *extra = (long long *)(tab + dense_b);
    uint32_t *sketch = (uint32_t *)(tab + 2 * dense_b);
    unsigned long long *img = (unsigned long long *)(tab + 2 * dense_b + sk_b);
    // scratch: the sample CTAs' key lists [GBD_SAMPLE_CTAS][GBD_LIST] | their lengths
    const size_t lst_b = (size_t)GBD_SAMPLE_CTAS * GBD_LIST * 4;
    char *scr;
    QG_TRY(qg_scratch(ctx, lst_b + GBD_SAMPLE_CTAS * 4, &scr));
    uint32_t *lst = (uint32_t *)scr, *lcnt = (uint32_t *)(scr + lst_b);
    qg_lookback lb;
    QG_TRY(qg_lb_make(ctx, ctx->sm_count, QG_SITE_GROUPBY, &lb));
    uint32_t *st = ctx->ctl->gbd;

    const int C = ctx->sm_count;
    const long long nv = n >> 2;
    const long long rows_per_cta = 4 * (nv / C + 1) + 4;
    const int cbits = 64 - __builtin_clzll((unsigned long long)(n > 0 ? n : 1));
    const uint32_t shift = (uint32_t)(64 - cbits);  // 32..63 for 1 <= n < 2^32
    unsigned long long fm = ((1ull << shift) - 1ull) / (unsigned long long)(n > 0 ? n : 1);
    const unsigned long long fm2 = 0xffffffffull / (unsigned long long)rows_per_cta;
    if (fm > fm2) fm = fm2;
    const uint32_t fast_max = (uint32_t)fm;

    static size_t attr_main[2] = {0, 0};  // (the single launch's attribute is set with its occupancy check)
    const size_t smem_main = (size_t)GBD_S * 12;
    const bool pred = val2 != nullptr;
    auto mainf = pred ? k_gbd_main<true> : k_gbd_main<false>;
    if (attr_main[pred] < smem_main) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(mainf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_main),
                    "attr");
        attr_main[pred] = smem_main;
    }

    const bool every_row = n <= (long long)GBD_SAMPLE_RUNS * GBD_RUN;
    const int runs = every_row ? (int)qg_ceil_div(n, GBD_RUN) : GBD_SAMPLE_RUNS;
    qg_status s = QG_OK;

    // One cooperative launch when every SM can hold one CTA and the stream is
    // not being captured (graphs take the four launches below).
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (g_gbd_single) QG_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cs), "capture status");
    static int single_fits[2] = {-1, -1};
    if (g_gbd_single && n > 0 && cs == cudaStreamCaptureStatusNone && C >= 128 &&
        (long long)C * GBD1_MAX_RUNS >= runs) {
        auto singlef = pred ? k_gbd_single<true> : k_gbd_single<false>;
        if (single_fits[pred] < 0) {
            int nb = 0;
            QG_TRY_CUDA(ctx, cudaFuncSetAttribute(singlef, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_main),
                        "attr");
            QG_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, singlef, GBD_THREADS, smem_main),
                        "occupancy");
            single_fits[pred] = nb >= 1;
        }
        if (single_fits[pred]) {
            QG_TRY_CUDA(ctx, cudaMemsetAsync(st, 0, G_WORDS * 4, ctx->stream), "memset gbd state");
            uint32_t *counts = (uint32_t *)scr;  // [C] groups per emit chunk (the sample lists are unused)
            bool er = every_row;
            int32_t l2 = lo2, h2 = hi2;
            long long nn = n, cp = cap;
            uint32_t sh = shift, fm32 = fast_max, spin = ctx->spin_limit;
            const int32_t *k0 = key, *v0 = val, *w0 = val2;
            int rn = runs;
            qg_control *ctl = ctx->ctl;
            long long *gs = (long long *)gsum, *gc = (long long *)gcnt;
            void *args[] = {&k0, &v0, &w0, &l2, &h2, &nn, &rn, &er, &sketch, &img, &st, &dense, &extra, &sh,
                            &fm32, &gkey, &gs, &gc, &cp, &d_num, &counts, &ctl, &spin};
            qg_pre_launch(ctx);
            const cudaError_t e = cudaLaunchCooperativeKernel((const void *)singlef, dim3(C), dim3(GBD_THREADS), args,
                                                              smem_main, ctx->stream);
            if (e != cudaSuccess) {
                ctx->table_dirty = true;
                return qg_cuda_fail(ctx, e, "k_gbd_single");
            }
            s = qg_check_launch(ctx, pred ? "k_gbd_single_fused" : "k_gbd_single");
            if (s != QG_OK) ctx->table_dirty = true;
            return s;
        }
    }
    qg_pre_launch(ctx);  // with runs == 0 (n == 0) every CTA lists nothing
    k_gbd_sample<<<GBD_SAMPLE_CTAS, GBD_SAMPLE_THREADS, 0, ctx->stream>>>(key, n, runs, every_row, sketch, lst, lcnt,
                                                                          st);
    s = qg_check_launch(ctx, "k_gbd_sample");
    if (s == QG_OK) {
        qg_pre_launch(ctx);
        k_gbd_cands<<<GBD_SAMPLE_CTAS, GBD_CANDS_THREADS, 0, ctx->stream>>>(sketch, lst, lcnt, img,
                                                                            every_row ? 1u : 2u, st);
        s = qg_check_launch(ctx, "k_gbd_cands");
    }
    if (s == QG_OK && n > 0) {
        qg_pre_launch(ctx);
        mainf<<<C, GBD_THREADS, smem_main, ctx->stream>>>(key, val, val2, lo2, hi2, n, img, st, dense, extra,
                                                          shift, fast_max);
        s = qg_check_launch(ctx, pred ? "k_gbd_main_fused" : "k_gbd_main");
    }
    if (s == QG_OK) {
        qg_pre_launch(ctx);
        k_gbd_emit<<<C, GBD_THREADS, 0, ctx->stream>>>(dense, extra, img, sketch, st, shift, gkey, (long long *)gsum,
                                                       (long long *)gcnt, cap, d_num, lb);
        s = qg_check_launch(ctx, "k_gbd_emit");
    }
    if (s != QG_OK) ctx->table_dirty = true;  // the dense table may hold partial sums
    return s;
}
