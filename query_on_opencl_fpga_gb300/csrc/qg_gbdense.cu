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
// Five launches, no host round trip until the caller's one read at the end:
//  1. k_gbd_sample  -- 2^18 keys (1024 runs of 256 consecutive rows spread
//                      over the column, or every row of a smaller input) are
//                      counted in an L2 open-addressing table; their smallest
//                      and largest key are recorded.
//  2. k_gbd_cands   -- sampled keys seen at least twice (every key when the
//                      whole input was sampled) become heavy-key candidates,
//                      bucketed by floor(log2(count)); the table is cleared.
//                      The key window [kbase, kbase + 2^22) is centred on the
//                      sample's key range (no window when it spans > 2^21).
//  3. k_gbd_build   -- one CTA inserts the candidates, most frequent level
//                      first, into a 4-way table image of 8192 window offsets.
//  4. k_gbd_main    -- one 1024-thread CTA per SM over a contiguous slice:
//                      the image is a read-only table in shared memory, so the
//                      four bucket loads of a thread's 4-row vector are issued
//                      before any update.  A heavy key adds to its shared
//                      count and sum (red.shared, no return); any other key
//                      adds one packed word to dense[key - kbase] in L2
//                      (red.global.add.u64: count << shift | value).  At the
//                      end the shared table is added to the dense table.
//  5. k_gbd_emit    -- the touched index range of the dense table is read in
//                      order, every non-empty entry becomes a group, and the
//                      entries are cleared.  Output positions come from a
//                      decoupled look-back over 4096-entry tiles.
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
constexpr int GBD_SLOG2 = 13;
constexpr int GBD_S = 1 << GBD_SLOG2;             // heavy-key table slots
constexpr int GBD_BLOG2 = GBD_SLOG2 - 2;          // 4-way buckets
constexpr int GBD_TLOG2 = 19;                     // sample counting table slots
constexpr uint32_t GBD_TMASK = (1u << GBD_TLOG2) - 1;
constexpr int GBD_SAMPLE_RUNS = 1024;
constexpr int GBD_RUN = 256;                      // consecutive rows per sample run
constexpr int GBD_MAX_CAND = GBD_SAMPLE_RUNS * GBD_RUN;
constexpr int GBD_BUILD_CAP = 16384;              // candidates the build CTA places
constexpr int GBD_THREADS = 1024;
constexpr int GBD_EMIT_THREADS = 256;
constexpr int GBD_EMIT_PER = 16;                  // entries per emit thread
constexpr int GBD_EMIT_TILE = GBD_EMIT_THREADS * GBD_EMIT_PER;
constexpr uint32_t GBD_EMIT_TILES = GBD_W / GBD_EMIT_TILE;
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
    G_NCAND = 8,   // heavy-key candidates
    G_HIST = 16,   // [32] candidates per level floor(log2(sample count))
    G_WORDS = 48
};
static_assert(G_HIST + 32 <= G_WORDS, "gbd state words");

__device__ __forceinline__ uint32_t gbd_bucket(uint32_t u) { return (u * 0x9E3779B1u) >> (32 - GBD_BLOG2); }

__device__ __forceinline__ void red_global_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("red.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_shared_u32(uint32_t *p, uint32_t v) {
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(qg_smem_u32(p)), "r"(v) : "memory");
}

// 1. Sample.  Run r covers rows [start_r, start_r + 256); grid-stride over runs.
__global__ void __launch_bounds__(GBD_RUN)
k_gbd_sample(const int32_t *__restrict__ key, long long n, int runs, bool every_row,
             unsigned long long *__restrict__ ct, uint32_t *__restrict__ st) {
    uint32_t lmin = 0xffffffffu, lmax = 0;
    for (int r = blockIdx.x; r < runs; r += gridDim.x) {
        const long long start = every_row ? (long long)r * GBD_RUN : (n - GBD_RUN) * (long long)r / (runs - 1);
        const long long i = start + threadIdx.x;
        if (i >= n) continue;
        const uint32_t k = (uint32_t)key[i];
        lmin = min(lmin, k);
        lmax = max(lmax, k);
        // entry = key << 32 | count, 0 = empty; load <= 1/2, so a free or
        // matching slot is always found within the table
        uint32_t h = qg_hash32(k) & GBD_TMASK;
        for (uint32_t p = 0; p <= GBD_TMASK; p++, h = (h + 1) & GBD_TMASK) {
            const unsigned long long old = atomicCAS(ct + h, 0ull, ((unsigned long long)k << 32) | 1ull);
            if (old == 0ull) break;
            if ((uint32_t)(old >> 32) == k) {
                atomicAdd(ct + h, 1ull);
                break;
            }
        }
    }
    lmin = __reduce_min_sync(QG_FULL_MASK, lmin);
    lmax = __reduce_max_sync(QG_FULL_MASK, lmax);
    if ((threadIdx.x & 31) == 0 && lmin <= lmax) {
        atomicMax(&st[G_NSMIN], ~lmin);
        atomicMax(&st[G_SMAX], lmax);
    }
}

// 2. Candidates and the window.
__global__ void __launch_bounds__(256)
k_gbd_cands(unsigned long long *__restrict__ ct, unsigned long long *__restrict__ cand, uint32_t min_count,
            uint32_t *__restrict__ st) {
    __shared__ uint32_t hist[32];
    if (threadIdx.x < 32) hist[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 <= GBD_TMASK; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        unsigned long long e = 0;
        if (i <= GBD_TMASK) {
            e = ct[i];
            if (e) ct[i] = 0ull;
        }
        const uint32_t c = (uint32_t)e;
        const bool take = e != 0ull && c >= min_count;
        const uint32_t m = __ballot_sync(QG_FULL_MASK, take);
        if (!m) continue;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&st[G_NCAND], (uint32_t)__popc(m));
        base = __shfl_sync(QG_FULL_MASK, base, 0);
        if (take) {
            const uint32_t pos = base + __popc(m & qg_lanemask_lt());
            if (pos < (uint32_t)GBD_MAX_CAND) cand[pos] = e;
            atomicAdd(&hist[31 - __clz(c)], 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x < 32 && hist[threadIdx.x]) atomicAdd(&st[G_HIST + threadIdx.x], hist[threadIdx.x]);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const uint32_t smin = ~st[G_NSMIN], smax = st[G_SMAX];
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

// 3. Heavy-key table image: window offsets in 4-way buckets, the candidates of
// the most frequent levels first (only as many levels as GBD_BUILD_CAP holds).
__global__ void __launch_bounds__(1024)
k_gbd_build(const unsigned long long *__restrict__ cand, const uint32_t *__restrict__ st,
            uint32_t *__restrict__ image) {
    extern __shared__ __align__(16) unsigned char gbd_build_raw[];
    uint32_t *tk = reinterpret_cast<uint32_t *>(gbd_build_raw);        // [GBD_S]
    uint32_t *ck = tk + GBD_S;                                          // [GBD_BUILD_CAP] offsets
    __shared__ uint32_t off[32], lcap[32], cur[32], s_lmin;
    const int tid = threadIdx.x;
    for (int i = tid; i < GBD_S; i += blockDim.x) tk[i] = GBD_EMPTY;
    if (tid == 0) {
        // levels from the most frequent down until GBD_BUILD_CAP candidates
        // are placed; the last level taken may be taken in part
        uint32_t acc = 0, lmin = 32;
        for (int l = 31; l >= 0 && acc < (uint32_t)GBD_BUILD_CAP; l--) {
            const uint32_t h = min(st[G_HIST + l], (uint32_t)GBD_BUILD_CAP - acc);
            off[l] = acc;
            lcap[l] = h;
            acc += h;
            lmin = (uint32_t)l;
        }
        s_lmin = lmin;
    }
    if (tid < 32) cur[tid] = 0;
    __syncthreads();
    const uint32_t lmin = s_lmin;
    if (st[G_OK]) {
        const uint32_t kbase = st[G_KBASE];
        const uint32_t nc = min(st[G_NCAND], (uint32_t)GBD_MAX_CAND);
        for (uint32_t i = tid; i < nc; i += blockDim.x) {
            const unsigned long long e = cand[i];
            const uint32_t l = 31 - __clz((uint32_t)e);
            if (l >= lmin) {
                const uint32_t pos = atomicAdd(&cur[l], 1u);
                if (pos < lcap[l]) ck[off[l] + pos] = (uint32_t)(e >> 32) - kbase;
            }
        }
        __syncthreads();
        for (int l = 31; l >= (int)lmin; l--) {
            const uint32_t c = min(cur[l], lcap[l]);
            for (uint32_t i = tid; i < c; i += blockDim.x) {
                const uint32_t u = ck[off[l] + i];  // in the window: the window covers the sample
                const uint32_t b = gbd_bucket(u);
                for (int w = 0; w < 4; w++) {
                    const uint32_t old = atomicCAS(&tk[b * 4 + w], GBD_EMPTY, u);
                    if (old == GBD_EMPTY || old == u) break;
                }
            }
            __syncthreads();
        }
    }
    __syncthreads();
    for (int i = tid; i < GBD_S; i += blockDim.x) image[i] = tk[i];
}

// 4. Main pass.
template <bool PRED>
__global__ void __launch_bounds__(GBD_THREADS, 1)
k_gbd_main(const int32_t *__restrict__ key, const int32_t *__restrict__ val, const int32_t *__restrict__ val2,
           int32_t lo2, int32_t hi2, long long n, const uint32_t *__restrict__ image, uint32_t *__restrict__ st,
           unsigned long long *__restrict__ dense, long long *__restrict__ extra, uint32_t shift,
           uint32_t fast_max) {
    extern __shared__ __align__(16) unsigned char gbd_main_raw[];
    uint32_t *hk = reinterpret_cast<uint32_t *>(gbd_main_raw);  // [GBD_S] window offsets
    uint32_t *hc = hk + GBD_S;                                    // [GBD_S] counts
    uint32_t *hl = hc + GBD_S;                                    // [GBD_S] sums of fast values
    __shared__ uint32_t s_red[4];
    const int tid = threadIdx.x;
    if (!st[G_OK]) {  // no window: the caller takes the two-pass path
        if (blockIdx.x == 0 && tid == 0) atomicAdd(&st[G_OUTSIDE], 1u);
        return;
    }
    const uint32_t kbase = st[G_KBASE];
    for (int i = tid; i < GBD_S; i += GBD_THREADS) {
        hk[i] = image[i];
        hc[i] = 0;
        hl[i] = 0;
    }
    if (tid < 4) s_red[tid] = tid == 0 ? 0xffffffffu : 0u;
    __syncthreads();
    uint32_t umin = 0xffffffffu, umax = 0, outside = 0, extra_used = 0;
    const unsigned long long one = 1ull << shift;
    auto row = [&](uint32_t u, uint32_t b, uint4 w, int32_t v) {
        if (u >= GBD_W) {
            outside++;
            return;
        }
        umin = min(umin, u);
        umax = max(umax, u);
        const int way = (w.x == u) ? 0 : (w.y == u) ? 1 : (w.z == u) ? 2 : (w.w == u) ? 3 : -1;
        const bool fast = (uint32_t)v <= fast_max;
        if (way >= 0) {
            const uint32_t s = b * 4 + (uint32_t)way;
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
        const uint32_t u[4] = {(uint32_t)k4.x - kbase, (uint32_t)k4.y - kbase, (uint32_t)k4.z - kbase,
                               (uint32_t)k4.w - kbase};
        const int32_t vs[4] = {v4.x, v4.y, v4.z, v4.w};
        uint32_t live = 0xfu;
        if (PRED) {
            live = (uint32_t)((w4.x >= lo2) & (w4.x <= hi2)) | ((uint32_t)((w4.y >= lo2) & (w4.y <= hi2)) << 1) |
                   ((uint32_t)((w4.z >= lo2) & (w4.z <= hi2)) << 2) | ((uint32_t)((w4.w >= lo2) & (w4.w <= hi2)) << 3);
        }
        uint32_t b[4];
        uint4 w[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {  // the table is read-only: all four bucket loads first
            b[j] = gbd_bucket(u[j]);
            w[j] = reinterpret_cast<const uint4 *>(hk)[b[j]];
        }
#pragma unroll
        for (int j = 0; j < 4; j++)
            if ((live >> j) & 1u) row(u[j], b[j], w[j], vs[j]);
    }
    if (blockIdx.x == gridDim.x - 1) {
        for (long long i = (nv << 2) + tid; i < n; i += GBD_THREADS) {
            if (PRED && !((val2[i] >= lo2) & (val2[i] <= hi2))) continue;
            const uint32_t u = (uint32_t)key[i] - kbase;
            const uint32_t b = gbd_bucket(u);
            row(u, b, reinterpret_cast<const uint4 *>(hk)[b], val[i]);
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
    for (int s = tid; s < GBD_S; s += GBD_THREADS)
        if (hc[s]) red_global_u64(dense + hk[s], ((unsigned long long)hc[s] << shift) + hl[s]);
    if (tid == 0) {
        if (s_red[0] <= s_red[1]) {
            atomicMax(&st[G_NUMIN], ~s_red[0]);
            atomicMax(&st[G_UMAX], s_red[1]);
        }
        if (s_red[2]) atomicAdd(&st[G_OUTSIDE], s_red[2]);
        if (s_red[3]) atomicOr(&st[G_EXTRA], 1u);
    }
}

// 5. Emit in key order.  Tile t (taken from the control block's tile counter,
// so tiles start in order) covers entries [lo + t*4096, lo + (t+1)*4096) of the
// touched range [lo, hi]; thread i of a tile owns 16 consecutive entries.
__global__ void __launch_bounds__(GBD_EMIT_THREADS)
k_gbd_emit(unsigned long long *__restrict__ dense, long long *__restrict__ extra, const uint32_t *__restrict__ st,
           uint32_t shift, int32_t *__restrict__ gkey, long long *__restrict__ gsum, long long *__restrict__ gcnt,
           long long cap, long long *__restrict__ d_num, qg_lookback lb) {
    __shared__ uint32_t s_tile, s_epoch, s_excl, s_wsum[GBD_EMIT_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_tile = atomicAdd(&lb.ctl->tile_ctr, 1u);
        s_epoch = *(volatile uint32_t *)&lb.ctl->epoch;
    }
    __syncthreads();
    const uint32_t tile = s_tile, epoch = s_epoch;
    const uint32_t lo = (~st[G_NUMIN]) & ~15u, hi = st[G_UMAX];
    const bool any = st[G_OK] && (~st[G_NUMIN]) <= hi;
    const uint32_t kbase = st[G_KBASE];
    const bool xtra = st[G_EXTRA] != 0;
    const unsigned long long mask = (1ull << shift) - 1ull;
    const unsigned long long first = (unsigned long long)lo + (unsigned long long)tile * GBD_EMIT_TILE +
                                     (unsigned long long)tid * GBD_EMIT_PER;
    unsigned long long e[GBD_EMIT_PER];
    uint32_t cnt = 0;
#pragma unroll
    for (int k = 0; k < GBD_EMIT_PER; k += 2) {
        const unsigned long long i = first + k;  // even: lo and the strides are multiples of 16
        if (any && i <= hi) {
            const ulonglong2 p = *reinterpret_cast<const ulonglong2 *>(dense + i);
            e[k] = p.x;
            e[k + 1] = (i + 1 <= hi) ? p.y : 0ull;
        } else {
            e[k] = e[k + 1] = 0ull;
        }
        cnt += (e[k] != 0ull) + (e[k + 1] != 0ull);
    }
    // exclusive scan of the per-thread counts (thread order = key order)
    uint32_t incl = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(QG_FULL_MASK, incl, d);
        if (lane >= d) incl += t;
    }
    if (lane == 31) s_wsum[warp] = incl;
    __syncthreads();
    uint32_t woff = 0, total = 0;
#pragma unroll
    for (int w = 0; w < GBD_EMIT_THREADS / 32; w++) {
        const uint32_t x = s_wsum[w];
        woff += (w < warp) ? x : 0u;
        total += x;
    }
    if (warp == 0) {
        const uint32_t excl = qg_lb_warp_exclusive(lb, tile, epoch, total);
        if (lane == 0) {
            s_excl = excl;
            if (tile == GBD_EMIT_TILES - 1) *d_num = (long long)excl + total;
        }
    }
    __syncthreads();
    long long pos = (long long)s_excl + woff + incl - cnt;
#pragma unroll
    for (int k = 0; k < GBD_EMIT_PER; k++) {
        if (e[k] == 0ull) continue;
        const unsigned long long i = first + k;
        long long s = (long long)(e[k] & mask);
        if (xtra) {
            s += extra[i];
            extra[i] = 0;
        }
        if (pos < cap) {
            gkey[pos] = (int32_t)(kbase + (uint32_t)i);
            gsum[pos] = s;
            gcnt[pos] = (long long)(e[k] >> shift);
        }
        dense[i] = 0ull;
        pos++;
    }
    qg_lb_end(lb);
}

}  // namespace

qg_status qg_gbd_launch(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2, int32_t lo2,
                        int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum, int64_t *gcnt, int64_t cap,
                        long long *d_num) {
    // table arena (kept all-zero): dense [W] u64 | extra [W] i64 | sample counts [2^19] u64
    const size_t dense_b = (size_t)GBD_W * 8, ct_b = ((size_t)1 << GBD_TLOG2) * 8;
    char *tab;
    QG_TRY(qg_table(ctx, 2 * dense_b + ct_b, &tab));
    unsigned long long *dense = (unsigned long long *)tab;
    long long *extra = (long long *)(tab + dense_b);
    unsigned long long *ct = (unsigned long long *)(tab + 2 * dense_b);
    // scratch: candidates [2^18] u64 | table image [8192] u32
    const size_t cand_b = (size_t)GBD_MAX_CAND * 8;
    char *scr;
    QG_TRY(qg_scratch(ctx, cand_b + (size_t)GBD_S * 4, &scr));
    unsigned long long *cand = (unsigned long long *)scr;
    uint32_t *image = (uint32_t *)(scr + cand_b);
    qg_lookback lb;
    QG_TRY(qg_lb_make(ctx, GBD_EMIT_TILES, QG_SITE_GROUPBY, &lb));
    uint32_t *st = ctx->ctl->gbd;

    const int C = ctx->sm_count;
    const long long nv = n >> 2;
    const long long rows_per_cta = 4 * (nv / C + 1) + 4;
    const int cbits = 64 - __builtin_clzll((unsigned long long)(n > 0 ? n : 1));
    const uint32_t shift = (uint32_t)(64 - cbits);
    unsigned long long fm = ((shift >= 64 ? ~0ull : (1ull << shift) - 1ull)) / (unsigned long long)(n > 0 ? n : 1);
    const unsigned long long fm2 = 0xffffffffull / (unsigned long long)rows_per_cta;
    if (fm > fm2) fm = fm2;
    const uint32_t fast_max = (uint32_t)fm;

    static size_t attr_build = 0, attr_main[2] = {0, 0};
    const size_t smem_build = (size_t)GBD_S * 4 + (size_t)GBD_BUILD_CAP * 4;
    const size_t smem_main = (size_t)GBD_S * 12;
    const bool pred = val2 != nullptr;
    auto mainf = pred ? k_gbd_main<true> : k_gbd_main<false>;
    if (attr_build < smem_build) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_gbd_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_build),
                    "attr");
        attr_build = smem_build;
    }
    if (attr_main[pred] < smem_main) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(mainf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_main),
                    "attr");
        attr_main[pred] = smem_main;
    }
    QG_TRY_CUDA(ctx, cudaMemsetAsync(st, 0, G_WORDS * 4, ctx->stream), "memset gbd state");

    const bool every_row = n <= (long long)GBD_SAMPLE_RUNS * GBD_RUN;
    const int runs = every_row ? (int)qg_ceil_div(n, GBD_RUN) : GBD_SAMPLE_RUNS;
    qg_status s = QG_OK;
    if (runs > 0) {
        qg_pre_launch(ctx);
        k_gbd_sample<<<runs < 4 * C ? runs : 4 * C, GBD_RUN, 0, ctx->stream>>>(key, n, runs, every_row, ct, st);
        s = qg_check_launch(ctx, "k_gbd_sample");
    }
    if (s == QG_OK) {
        qg_pre_launch(ctx);
        k_gbd_cands<<<C * 2, 256, 0, ctx->stream>>>(ct, cand, every_row ? 1u : 2u, st);
        s = qg_check_launch(ctx, "k_gbd_cands");
    }
    if (s == QG_OK) {
        qg_pre_launch(ctx);
        k_gbd_build<<<1, 1024, smem_build, ctx->stream>>>(cand, st, image);
        s = qg_check_launch(ctx, "k_gbd_build");
    }
    if (s == QG_OK && n > 0) {
        qg_pre_launch(ctx);
        mainf<<<C, GBD_THREADS, smem_main, ctx->stream>>>(key, val, val2, lo2, hi2, n, image, st, dense, extra,
                                                          shift, fast_max);
        s = qg_check_launch(ctx, pred ? "k_gbd_main_fused" : "k_gbd_main");
    }
    if (s == QG_OK) {
        qg_pre_launch(ctx);
        k_gbd_emit<<<GBD_EMIT_TILES, GBD_EMIT_THREADS, 0, ctx->stream>>>(
            dense, extra, st, shift, gkey, (long long *)gsum, (long long *)gcnt, cap, d_num, lb);
        s = qg_check_launch(ctx, "k_gbd_emit");
    }
    if (s != QG_OK) ctx->table_dirty = true;  // the dense table may hold partial sums
    return s;
}
