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
//    aggregate, rows are hashed once: each CTA keeps a private open-addressing
//    table in shared memory for the keys it sees first (Zipf heavy hitters land
//    there), other rows go to a global open-addressing table whose 32-byte
//    slots {tag, sum, count} sit in one L2 sector and are updated with
//    atomicCAS / 64-bit atomicAdd.  A final pass compacts the table into the
//    output columns and clears it for the next call; QG_ORDER_KEY then sorts
//    the groups by key (unsigned, the order groupByImpl's sorted array gives).
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
#pragma unroll
    for (int r = 0; r < GBD_ROUNDS; r++) {
        long long idx = base + (long long)(r * GBD_THREADS + tid) * 2;
        bool f0 = false, f1 = false;
        if (idx < n) {
            uint32_t k0, k1 = 0;
            if (idx + 1 < n) {
                int4 t = qg_ldg_stream(reinterpret_cast<const int4 *>(in) + (idx >> 1));
                k0 = (uint32_t)t.y;
                k1 = (uint32_t)t.w;
                f1 = k1 != k0;
            } else {
                k0 = in2[idx].y;
            }
            f0 = (idx == 0) || (__ldg(&in2[idx - 1].y) != k0);
        }
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
    qg_lb_end(lb);
}

// ---------------------------------------------------------------------------
// 1b. per-group aggregation of .x over sorted records
// ---------------------------------------------------------------------------
constexpr int AGG_CHUNK = 2048;  // rows per warp work item

__device__ __forceinline__ int32_t agg_identity(int op) {
    return op == QG_REDUCE_MIN ? (1 << 30) : 0;
}

__global__ void k_agg_init(int32_t *agg, long long g, int op) {
    long long stride = (long long)gridDim.x * blockDim.x;
    int32_t id = agg_identity(op);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g; i += stride) agg[i] = id;
}

__global__ void __launch_bounds__(256)
k_agg_chunks(const uint2 *__restrict__ rec, long long n, const int32_t *__restrict__ startPos,
             long long G, int op, int32_t *__restrict__ agg) {
    const int lane = threadIdx.x & 31;
    const long long warp_id = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long nchunks = (n + AGG_CHUNK - 1) / AGG_CHUNK;
    for (long long c = warp_id; c < nchunks; c += nwarps) {
        const long long cs = c * AGG_CHUNK;
        const long long ce = (cs + AGG_CHUNK < n) ? cs + AGG_CHUNK : n;
        // last group starting at or before cs
        long long lo = 0, hi = G - 1;
        while (lo < hi) {
            long long mid = (lo + hi + 1) >> 1;
            if ((long long)__ldg(&startPos[mid]) <= cs) lo = mid; else hi = mid - 1;
        }
        long long g = lo;
        long long pos = cs;
        while (pos < ce && g < G) {
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
                                 int32_t *__restrict__ agg) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x; g < G; g += stride) {
        long long gs = startPos[g], ge = (g == G - 1) ? n : startPos[g + 1];
        bool spans = (gs / AGG_CHUNK) != ((ge - 1) / AGG_CHUNK);
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
    const int lane = threadIdx.x & 31;
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
        unsigned long long basepos = 0;
        if (lane == 0 && b) basepos = atomicAdd(cursor, (unsigned long long)__popc(b));
        basepos = __shfl_sync(QG_FULL_MASK, basepos, 0);
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
__global__ void k_groupby_gather(const unsigned long long *__restrict__ rec, long long g,
                                 const long long *__restrict__ tsum, const long long *__restrict__ tcnt,
                                 int32_t *__restrict__ gkey, long long *__restrict__ gsum,
                                 long long *__restrict__ gcnt) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < g; i += stride) {
        unsigned long long r = rec[i];
        uint32_t idx = (uint32_t)r;
        gkey[i] = (int32_t)(r >> 32);
        gsum[i] = tsum[idx];
        gcnt[i] = tcnt[idx];
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
        char *scr;
        s = qg_scratch(ctx, qg_lb_bytes(tiles), &scr);
        if (s == QG_OK) {
            qg_lookback lb{(unsigned long long *)scr, ctx->ctl, ctx->spin_limit, QG_SITE_GROUPBY};
            long long *d_count = (long long *)&ctx->ctl->counter[0];
            qg_pre_launch(ctx);
            k_group_bounds<<<(unsigned)tiles, GBD_THREADS, 0, ctx->stream>>>(
                (const uint4 *)sorted_out, n, startPos, cap_groups, d_count, lb);
            s = qg_check_launch(ctx, "k_group_bounds");
            long long h = 0;
            if (s == QG_OK) s = qg_read_i64(ctx, d_count, &h);
            if (s == QG_OK) s = qg_collect_error(ctx);
            if (s == QG_OK) {
                *num_groups = h;
                if (h > cap_groups) s = QG_ERR_CAPACITY;
            }
        }
    }
    return s;
}

extern "C" QG_API qg_status qg_aggregate_groups(qg_ctx *ctx, const void *sorted, int64_t n,
                                                const int32_t *startPos, int64_t G, int op,
                                                int32_t *agg) {
    if (!ctx || n < 0 || G < 0 || op < 0 || op > 3) return QG_ERR_INVALID;
    if (G == 0) return QG_OK;
    if (!sorted || !startPos || !agg || n == 0) return QG_ERR_INVALID;
    int ib = grid_for(ctx, G, 256, 8);
    qg_pre_launch(ctx);
    k_agg_init<<<ib, 256, 0, ctx->stream>>>(agg, G, op);
    QG_TRY(qg_check_launch(ctx, "k_agg_init"));
    long long chunks = (n + AGG_CHUNK - 1) / AGG_CHUNK;
    int blocks = grid_for(ctx, chunks * 32, 256, 8);
    qg_pre_launch(ctx);
    k_agg_chunks<<<blocks, 256, 0, ctx->stream>>>((const uint2 *)sorted, n, startPos, G, op, agg);
    QG_TRY(qg_check_launch(ctx, "k_agg_chunks"));
    if (op == QG_REDUCE_AVERAGE) {
        qg_pre_launch(ctx);
        k_agg_avg_finish<<<ib, 256, 0, ctx->stream>>>(startPos, n, G, agg);
        QG_TRY(qg_check_launch(ctx, "k_agg_avg_finish"));
    }
    return qg_ctx_check(ctx);
}

// ---------------------------------------------------------------------------
// host: column hash group-by
// ---------------------------------------------------------------------------
static int g_gb_slog2 = 12;          // shared-memory table slots (log2)
static int g_gb_blocks_per_sm = 2;

extern "C" QG_API qg_status qg_groupby_set_knobs(int smem_slots_log2, int blocks_per_sm) {
    if (smem_slots_log2 < 6 || smem_slots_log2 > 13 || blocks_per_sm < 1 || blocks_per_sm > 8)
        return QG_ERR_INVALID;
    g_gb_slog2 = smem_slots_log2;
    g_gb_blocks_per_sm = blocks_per_sm;
    return QG_OK;
}

qg_status qg_groupby_cols_launch(qg_ctx *ctx, const int32_t *key, const int32_t *val,
                                 const int32_t *val2, int32_t lo2, int32_t hi2, int64_t n,
                                 int32_t *gkey, int64_t *gsum, int64_t *gcnt, int64_t cap,
                                 int order, long long *d_num, unsigned long long **rec_out,
                                 long long **tsum_out, long long **tcnt_out) {
    // Table: power of two >= 2 * cap slots, at least 1024.
    uint64_t slots = 1024;
    while (slots < (uint64_t)cap * 2) slots <<= 1;
    if (slots > (1ull << 31)) return QG_ERR_UNSUPPORTED;
    char *tabp;
    QG_TRY(qg_table(ctx, slots * sizeof(GSlot), &tabp));
    GSlot *tab = (GSlot *)tabp;
    const int slog2 = g_gb_slog2;
    const size_t smem = ((size_t)1 << slog2) * 16;
    static size_t attr_smem[2] = {0, 0};
    const bool pred = val2 != nullptr;
    if (attr_smem[pred] < smem) {
        if (pred)
            QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_groupby_hash<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
        else
            QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_groupby_hash<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
        attr_smem[pred] = smem;
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
    // Output: straight into the caller's columns, or into scratch for the sort.
    unsigned long long *cursor = (unsigned long long *)d_num;
    QG_TRY_CUDA(ctx, cudaMemsetAsync(cursor, 0, 8, ctx->stream), "memset cursor");
    int eb = grid_for(ctx, (long long)slots, 256, 8);
    if (order == QG_ORDER_KEY) {
        // rec | tsum | tcnt | sort ping-pong, all in the aux arena so the
        // sort's own scratch use cannot move them.
        char *scr;
        size_t cb = (size_t)(cap > 0 ? cap : 1);
        QG_TRY(qg_aux(ctx, cb * 32, &scr));
        unsigned long long *rec = (unsigned long long *)scr;
        long long *tsum = (long long *)(rec + cb);
        long long *tcnt = tsum + cb;
        qg_pre_launch(ctx);
        k_groupby_emit<<<eb, 256, 0, ctx->stream>>>(tab, (long long)slots, gkey, tsum, tcnt, cap,
                                                    cursor, rec);
        *rec_out = rec;
        *tsum_out = tsum;
        *tcnt_out = tcnt;
    } else {
        qg_pre_launch(ctx);
        k_groupby_emit<<<eb, 256, 0, ctx->stream>>>(tab, (long long)slots, gkey, (long long *)gsum, (long long *)gcnt, cap,
                                                    cursor, nullptr);
    }
    return qg_check_launch(ctx, "k_groupby_emit");
}

extern "C" QG_API qg_status qg_groupby_cols_async(qg_ctx *ctx, const int32_t *key,
                                                  const int32_t *val, const int32_t *val2,
                                                  int32_t lo2, int32_t hi2, int64_t n,
                                                  int32_t *gkey, int64_t *gsum, int64_t *gcnt,
                                                  int64_t cap, int order, int64_t *d_num) {
    if (!ctx || n < 0 || cap < 0 || !d_num || (n > 0 && (!key || !val))) return QG_ERR_INVALID;
    if (order != QG_ORDER_NONE) return QG_ERR_UNSUPPORTED;  // sorted order needs the sync form
    if ((((uintptr_t)key) | ((uintptr_t)val) | ((uintptr_t)val2)) & 15) return QG_ERR_INVALID;
    unsigned long long *rec;
    long long *ts, *tc;
    return qg_groupby_cols_launch(ctx, key, val, val2, lo2, hi2, n, gkey, gsum, gcnt, cap, order,
                                  (long long *)d_num, &rec, &ts, &tc);
}

extern "C" QG_API qg_status qg_groupby_cols(qg_ctx *ctx, const int32_t *key, const int32_t *val,
                                            const int32_t *val2, int32_t lo2, int32_t hi2,
                                            int64_t n, int32_t *gkey, int64_t *gsum,
                                            int64_t *gcnt, int64_t cap, int order,
                                            int64_t *num_groups) {
    if (!ctx || n < 0 || cap < 0 || !num_groups || (n > 0 && (!key || !val)))
        return QG_ERR_INVALID;
    if (order != QG_ORDER_NONE && order != QG_ORDER_KEY) return QG_ERR_INVALID;
    if ((((uintptr_t)key) | ((uintptr_t)val) | ((uintptr_t)val2)) & 15) return QG_ERR_INVALID;
    long long *d_num = (long long *)&ctx->ctl->counter[1];
    unsigned long long *rec = nullptr;
    long long *tsum = nullptr, *tcnt = nullptr;
    QG_TRY(qg_groupby_cols_launch(ctx, key, val, val2, lo2, hi2, n, gkey, gsum, gcnt, cap, order,
                                  d_num, &rec, &tsum, &tcnt));
    long long g = 0;
    QG_TRY(qg_read_i64(ctx, d_num, &g));
    QG_TRY(qg_collect_error(ctx));
    *num_groups = g;
    if (g > cap) return QG_ERR_CAPACITY;
    if (order == QG_ORDER_KEY && g > 1) {
        // Sort (key, index) records, then gather the sums and counts.
        unsigned long long *tmp = (unsigned long long *)(tcnt + cap);
        QG_TRY(qg_sort_rec_inplace(ctx, rec, tmp, g));
        int gb = grid_for(ctx, g, 256, 8);
        qg_pre_launch(ctx);
        k_groupby_gather<<<gb, 256, 0, ctx->stream>>>(rec, g, tsum, tcnt, gkey, (long long *)gsum, (long long *)gcnt);
        QG_TRY(qg_check_launch(ctx, "k_groupby_gather"));
        return qg_ctx_check(ctx);
    } else if (order == QG_ORDER_KEY && g == 1) {
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(gsum, tsum, 8, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(gcnt, tcnt, 8, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        return qg_ctx_check(ctx);
    }
    return QG_OK;
}
