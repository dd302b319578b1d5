// qg_filter.cu -- single-pass stable range filter.
//
// Reference chain replaced (kernel/filter/filter_op.cl, host/host/testFilter.cpp:92-154):
//   filterImpl_map_kernel (:6-31)       mark[i] = lo <= (int)Rin[i].y <= hi
//   ScanLargeArrays/prefixSum/blockAddition (:51-207)  exclusive scan of mark
//   filterImpl_outSize_kernel (:211-215) count = mark[n-1] + scan[n-1]
//   filterImpl_write_kernel (:220-238)   Rout[scan[i]] = Rin[i] if mark[i]
// The reference moves each row through HBM about six times and launches
// 2*pass+3 kernels.  Here one kernel reads each row once with 128-bit loads,
// ranks the selected rows with warp ballots + popc, gets the tile's output
// offset from a decoupled look-back over earlier tiles, and writes the
// selected rows in input order (stable, as the reference's scatter is).
#include "qg_internal.cuh"

namespace {

constexpr int FT_THREADS = 256;
constexpr int FT_WARPS = FT_THREADS / 32;
constexpr int FT_LB_WARPS = 4;  // warps doing the look-back: 128 predecessors per round

// Records (uint2 {x, y}), two per 128-bit load.  ROUNDS loads per thread.
template <int ROUNDS>
__global__ void __launch_bounds__(FT_THREADS, 5)
k_filter_rec(const uint4 *__restrict__ in, long long n, int32_t lo, int32_t hi,
             uint2 *__restrict__ out, long long cap, long long *__restrict__ d_count,
             qg_lookback lb) {
    constexpr int TILE = FT_THREADS * ROUNDS * 2;
    __shared__ uint32_t s_tile, s_epoch, s_excl;
    __shared__ uint32_t s_woff[ROUNDS * FT_WARPS];
    const uint32_t tile = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long base = (long long)tile * TILE;
    const uint32_t lt = qg_lanemask_lt();

    uint4 v[ROUNDS];
    uint32_t fl = 0;            // bit 2r: first record of round r, bit 2r+1: second
    uint32_t lpre[ROUNDS];      // selected records of lower lanes in this round
    // Every load of the tile is issued before the first ballot, so the
    // rounds' DRAM latencies overlap instead of adding up.
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long idx = base + (long long)(r * FT_THREADS + tid) * 2;
        if (idx + 1 < n) {
            int4 t = qg_ldg_stream(reinterpret_cast<const int4 *>(in) + (idx >> 1));
            v[r] = make_uint4(t.x, t.y, t.z, t.w);
        } else if (idx < n) {
            uint2 a = reinterpret_cast<const uint2 *>(in)[idx];
            v[r] = make_uint4(a.x, a.y, 0, 0);
        } else {
            v[r] = make_uint4(0, 0, 0, 0);
        }
    }
    qg_lb_begin(lb, &s_tile, &s_epoch);  // epoch read while the loads are in flight
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long idx = base + (long long)(r * FT_THREADS + tid) * 2;
        bool f0 = (idx < n) & ((int32_t)v[r].y >= lo) & ((int32_t)v[r].y <= hi);
        bool f1 = (idx + 1 < n) & ((int32_t)v[r].w >= lo) & ((int32_t)v[r].w <= hi);
        uint32_t b0 = __ballot_sync(QG_FULL_MASK, f0), b1 = __ballot_sync(QG_FULL_MASK, f1);
        lpre[r] = __popc(b0 & lt) + __popc(b1 & lt);
        if (lane == 0) s_woff[r * FT_WARPS + warp] = __popc(b0) + __popc(b1);
        fl |= (uint32_t)f0 << (2 * r);
        fl |= (uint32_t)f1 << (2 * r + 1);
    }
    // Exclusive offsets of the ROUNDS*WARPS per-warp counts, round-major (the
    // order of the rows they cover), and the tile's offset from the look-back.
    __shared__ uint32_t s_tmp[2 * FT_LB_WARPS + 1];
    qg_tile_offsets_wide<ROUNDS * FT_WARPS, FT_LB_WARPS>(s_woff, lb, tile, s_epoch, &s_excl, s_tmp,
                                                         d_count, gridDim.x - 1);
    const long long excl = s_excl;
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long pos = excl + s_woff[r * FT_WARPS + warp] + lpre[r];
        if ((fl >> (2 * r)) & 1u) {
            if (pos < cap) out[pos] = make_uint2(v[r].x, v[r].y);
            pos++;
        }
        if ((fl >> (2 * r + 1)) & 1u) {
            if (pos < cap) out[pos] = make_uint2(v[r].z, v[r].w);
        }
    }
    qg_lb_finish(lb, tile, gridDim.x - 1, s_epoch);
}

// Columns: int32 key and payload, four rows per 128-bit load.  Output is the
// int32 pair (row id, payload).  The tile id is taken from the control
// block's tile counter (the CTAs' start order), so a tile only ever waits for
// tiles that are already running.
template <int ROUNDS>
__global__ void __launch_bounds__(FT_THREADS, 5)
k_filter_cols(const int32_t *__restrict__ key, const int32_t *__restrict__ pay, long long n,
              int32_t lo, int32_t hi, int2 *__restrict__ out, long long cap,
              long long *__restrict__ d_count, qg_lookback lb) {
    constexpr int TILE = FT_THREADS * ROUNDS * 4;
    __shared__ uint32_t s_tile, s_epoch, s_excl;
    __shared__ uint32_t s_woff[ROUNDS * FT_WARPS];
    qg_lb_begin_dyn(lb, &s_tile, &s_epoch);
    const uint32_t tile = s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long base = (long long)tile * TILE;
    const uint32_t lt = qg_lanemask_lt();

    int4 kv[ROUNDS], pv[ROUNDS];
    uint32_t fl = 0;  // bit 4r+j
    uint32_t lpre[ROUNDS];
    // All loads first (see k_filter_rec), then the predicates and ballots.
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long idx = base + (long long)(r * FT_THREADS + tid) * 4;
        if (idx + 3 < n) {
            kv[r] = qg_ldg_stream(reinterpret_cast<const int4 *>(key + idx));
            pv[r] = qg_ldg_stream(reinterpret_cast<const int4 *>(pay + idx));
        } else {
            int t[4] = {0, 0, 0, 0}, p[4] = {0, 0, 0, 0};
            for (int j = 0; j < 4; j++)
                if (idx + j < n) { t[j] = key[idx + j]; p[j] = pay[idx + j]; }
            kv[r] = make_int4(t[0], t[1], t[2], t[3]);
            pv[r] = make_int4(p[0], p[1], p[2], p[3]);
        }
    }
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long idx = base + (long long)(r * FT_THREADS + tid) * 4;
        uint32_t f = 0;
        f |= (uint32_t)((kv[r].x >= lo) & (kv[r].x <= hi) & (idx + 0 < n)) << 0;
        f |= (uint32_t)((kv[r].y >= lo) & (kv[r].y <= hi) & (idx + 1 < n)) << 1;
        f |= (uint32_t)((kv[r].z >= lo) & (kv[r].z <= hi) & (idx + 2 < n)) << 2;
        f |= (uint32_t)((kv[r].w >= lo) & (kv[r].w <= hi) & (idx + 3 < n)) << 3;
        uint32_t c = 0, tot = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            uint32_t b = __ballot_sync(QG_FULL_MASK, (f >> j) & 1u);
            c += __popc(b & lt);
            tot += __popc(b);
        }
        lpre[r] = c;
        if (lane == 0) s_woff[r * FT_WARPS + warp] = tot;
        fl |= f << (4 * r);
    }
    __shared__ uint32_t s_tmp[2 * FT_LB_WARPS + 1];
    qg_tile_offsets_wide<ROUNDS * FT_WARPS, FT_LB_WARPS>(s_woff, lb, tile, s_epoch, &s_excl, s_tmp,
                                                         d_count, gridDim.x - 1);
    const long long excl = s_excl;
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long pos = excl + s_woff[r * FT_WARPS + warp] + lpre[r];
        const long long idx = base + (long long)(r * FT_THREADS + tid) * 4;
        const int kk[4] = {pv[r].x, pv[r].y, pv[r].z, pv[r].w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if ((fl >> (4 * r + j)) & 1u) {
                if (pos < cap) out[pos] = make_int2((int32_t)(idx + j), kk[j]);
                pos++;
            }
        }
    }
    qg_lb_finish_dyn(lb, tile, gridDim.x - 1, s_epoch);
}

constexpr int REC_ROUNDS = 8;   // 4096 records per tile
constexpr int COL_ROUNDS = 4;   // 4096 rows per tile

// Persistent column filter: each CTA streams tiles of 4096 rows (keys and
// payloads, 32 KB) through a 3-stage shared-memory ring filled by the bulk-copy
// (TMA) engine, so the next tiles are in flight while a tile's look-back
// resolves.  Tile ids come from the context's atomic counter in the order the
// CTAs ask for them; a CTA processes its tiles in increasing order, so every
// tile's predecessors belong to running CTAs and the look-back always ends.
constexpr int FP_THREADS = 256;
constexpr int FP_WARPS = FP_THREADS / 32;
constexpr int FP_TILE = 4096;
constexpr int FP_ROUNDS = FP_TILE / FP_THREADS;  // 16: one row per thread per round
constexpr int FP_STAGES = 3;

struct FpSmem {
    int32_t k[FP_STAGES][FP_TILE];
    int32_t p[FP_STAGES][FP_TILE];
    unsigned long long bar[FP_STAGES];
    uint32_t tile_of[FP_STAGES];
    uint32_t pending[FP_STAGES];  // a copy (or arrival) was issued into the stage and not yet seen to land
    uint32_t phase[FP_STAGES];    // phases of the stage's barrier seen to complete
    uint32_t broken;              // a wait gave up: no more copies, every later tile read from global
    uint32_t woff[FP_ROUNDS * FP_WARPS];
    uint32_t bal[FP_ROUNDS * FP_WARPS];
    uint32_t lbtmp[2 * FT_LB_WARPS + 1];
    uint32_t excl, epoch;
};

__device__ __forceinline__ void fp_issue(FpSmem &S, int s, const int32_t *key, const int32_t *pay,
                                         long long n, uint32_t t) {
    const long long base = (long long)t * FP_TILE;
    long long rows = n - base;
    if (rows > FP_TILE) rows = FP_TILE;
    const uint32_t bytes = (uint32_t)(rows & ~3LL) * 4u;
    if (bytes) {
        qg_mbar_arrive_expect_tx(&S.bar[s], 2 * bytes);
        qg_bulk_g2s(S.k[s], key + base, bytes, &S.bar[s]);
        qg_bulk_g2s(S.p[s], pay + base, bytes, &S.bar[s]);
    } else {
        qg_mbar_arrive(&S.bar[s]);
    }
}

__global__ void __launch_bounds__(FP_THREADS)
k_filter_cols_tma(const int32_t *__restrict__ key, const int32_t *__restrict__ pay, long long n,
                  int32_t lo, int32_t hi, int2 *__restrict__ out, long long cap,
                  long long *__restrict__ d_count, qg_lookback lb, uint32_t num_tiles) {
    extern __shared__ __align__(128) unsigned char fp_raw[];
    FpSmem &S = *reinterpret_cast<FpSmem *>(fp_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt = qg_lanemask_lt();
    if (tid == 0) {
        for (int s = 0; s < FP_STAGES; s++) qg_mbar_init(&S.bar[s], 1);
        qg_mbar_fence_init();
        S.epoch = *(volatile uint32_t *)&lb.ctl->epoch;
        S.broken = 0;
        for (int s = 0; s < FP_STAGES; s++) {
            const uint32_t t = atomicAdd(&lb.ctl->tile_ctr, 1u);
            S.tile_of[s] = t;
            S.phase[s] = 0;
            S.pending[s] = t < num_tiles ? 1u : 0u;
            if (t < num_tiles) fp_issue(S, s, key, pay, n, t);
        }
    }
    __syncthreads();
    for (uint32_t it = 0;; it++) {
        const int s = (int)(it % FP_STAGES);
        const uint32_t t = S.tile_of[s];
        if (t >= num_tiles) break;
        // Bounded wait for the stage's copy.  The CTA uses the staged tile only
        // when every thread saw it land; otherwise it reports QG_ERR_TIMEOUT,
        // reads this and every later tile from global memory, issues no more
        // copies, and never reads a stage whose copy it did not see land.
        const bool waited = !S.broken && S.pending[s];
        bool landed = false;
        if (waited) {
            const uint32_t parity = S.phase[s] & 1u;
            uint32_t w = 0;
            landed = true;
            while (!qg_mbar_try_wait(&S.bar[s], parity)) {
                if (++w >= lb.spin_limit) {
                    landed = false;
                    break;
                }
            }
        }
        const bool all = __syncthreads_and(landed) != 0;
        const bool some = __syncthreads_or(landed) != 0;
        if (waited && tid == 0) {
            if (!all) {
                qg_record_error(lb.ctl, QG_ERR_TIMEOUT, lb.site);
                S.broken = 1;
            }
            if (some) {  // the copy completed (a thread saw its phase end)
                S.pending[s] = 0;
                S.phase[s]++;
            }
        }
        const long long base = (long long)t * FP_TILE;
        long long rows_l = n - base;
        const int rows = rows_l > FP_TILE ? FP_TILE : (int)rows_l;
        const int bulk_rows = (waited && all) ? (rows & ~3) : 0;
#pragma unroll
        for (int r = 0; r < FP_ROUNDS; r++) {
            const int row = r * FP_THREADS + tid;
            bool f = false;
            if (row < rows) {
                const int32_t k = row < bulk_rows ? S.k[s][row] : key[base + row];
                f = (k >= lo) & (k <= hi);
            }
            const uint32_t b = __ballot_sync(QG_FULL_MASK, f);
            if (lane == 0) {
                S.woff[r * FP_WARPS + warp] = __popc(b);
                S.bal[r * FP_WARPS + warp] = b;
            }
        }
        qg_tile_offsets_wide<FP_ROUNDS * FP_WARPS, FT_LB_WARPS>(S.woff, lb, t, S.epoch, &S.excl,
                                                                S.lbtmp, d_count, num_tiles - 1);
        const long long excl = S.excl;
#pragma unroll
        for (int r = 0; r < FP_ROUNDS; r++) {
            const uint32_t b = S.bal[r * FP_WARPS + warp];
            if ((b >> lane) & 1u) {
                const int row = r * FP_THREADS + tid;
                const long long pos = excl + S.woff[r * FP_WARPS + warp] + __popc(b & lt);
                const int32_t pv = row < bulk_rows ? S.p[s][row] : pay[base + row];
                if (pos < cap) out[pos] = make_int2((int32_t)(base + row), pv);
            }
        }
        __syncthreads();
        if (tid == 0) {
            const uint32_t t2 = atomicAdd(&lb.ctl->tile_ctr, 1u);
            S.tile_of[s] = t2;
            if (t2 < num_tiles && !S.broken && !S.pending[s]) {
                fp_issue(S, s, key, pay, n, t2);
                S.pending[s] = 1;
            }
        }
        __syncthreads();
    }
    // A copy still in flight into this CTA's shared memory must land before the
    // CTA exits (only after a wait gave up): wait for it, again with a limit --
    // its own, not the caller's poll limit, which may be 0 (a copy from valid
    // memory lands within microseconds; the limit only bounds the loop).
    if (tid == 0 && S.broken) {
        constexpr uint32_t DRAIN_POLLS = 1u << 22;
        for (int s = 0; s < FP_STAGES; s++) {
            if (!S.pending[s]) continue;
            for (uint32_t w = 0; w < DRAIN_POLLS && !qg_mbar_try_wait(&S.bar[s], S.phase[s] & 1u); w++) {
            }
        }
    }
    __syncthreads();
    qg_lb_end(lb);
}

}  // namespace

static qg_status finish_count(qg_ctx *ctx, long long *d_count, int64_t cap, int64_t *out_n) {
    long long h = 0;
    QG_TRY(qg_read_count(ctx, d_count, &h));
    *out_n = h;
    if (h > cap) return QG_ERR_CAPACITY;
    return QG_OK;
}

// ---------------------------------------------------------------------------
// Column filter, two passes with no waiting between tiles (variant 2).
//   pass A (k_filter_count): keys only; the selected-row count of every tile,
//          per group of 256 tiles the sum of their counts, and every row's
//          predicate bit (16 bits per thread);
//   pass B (k_filter_write): the predicate bits and the payloads of the
//          selected rows only (the output is row id + payload); each tile's
//          output offset is the sum of the group sums before it plus its
//          group's earlier tile counts (at most 255), read while its own
//          loads are in flight.
// No tile waits for another: both passes stream at the memory's pace, where
// the single-pass chain of look-backs does not.
// ---------------------------------------------------------------------------
constexpr int TP_THREADS = 256;
constexpr int TP_WARPS = TP_THREADS / 32;
constexpr int TP_ROUNDS = 4;
constexpr int TP_TILE = TP_THREADS * TP_ROUNDS * 4;  // 4096 rows
constexpr int TP_GROUP = 256;                         // tiles per group sum

__device__ __forceinline__ void tp_load_keys(const int32_t *__restrict__ key, long long idx, long long n, int4 &k) {
    if (idx + 3 < n) {
        k = qg_ldg_stream(reinterpret_cast<const int4 *>(key + idx));
    } else {
        int t[4] = {0, 0, 0, 0};
        for (int j = 0; j < 4; j++)
            if (idx + j < n) t[j] = key[idx + j];
        k = make_int4(t[0], t[1], t[2], t[3]);
    }
}

__device__ __forceinline__ uint32_t tp_flags(const int4 &k, long long idx, long long n, int32_t lo, int32_t hi) {
    return (uint32_t)((k.x >= lo) & (k.x <= hi) & (idx + 0 < n)) | ((uint32_t)((k.y >= lo) & (k.y <= hi) & (idx + 1 < n)) << 1) |
           ((uint32_t)((k.z >= lo) & (k.z <= hi) & (idx + 2 < n)) << 2) |
           ((uint32_t)((k.w >= lo) & (k.w <= hi) & (idx + 3 < n)) << 3);
}

// With mask set, each thread also stores its 16 rows' predicate bits (bit
// 4 * round + j), so that pass B need not read the keys again.
__global__ void __launch_bounds__(TP_THREADS)
k_filter_count(const int32_t *__restrict__ key, long long n, int32_t lo, int32_t hi, uint32_t *__restrict__ counts,
               uint32_t *__restrict__ gsum, uint16_t *__restrict__ mask, uint32_t *__restrict__ arrivals) {
    __shared__ uint32_t ws[TP_WARPS];
    __shared__ uint32_t s_last;
    const int tid = threadIdx.x;
    const long long base = (long long)blockIdx.x * TP_TILE;
    int4 kv[TP_ROUNDS];
#pragma unroll
    for (int r = 0; r < TP_ROUNDS; r++) tp_load_keys(key, base + (long long)(r * TP_THREADS + tid) * 4, n, kv[r]);
    uint32_t fl = 0;
#pragma unroll
    for (int r = 0; r < TP_ROUNDS; r++)
        fl |= tp_flags(kv[r], base + (long long)(r * TP_THREADS + tid) * 4, n, lo, hi) << (4 * r);
    if (mask) mask[(size_t)blockIdx.x * TP_THREADS + tid] = (uint16_t)fl;
    uint32_t c = __popc(fl);
    c = __reduce_add_sync(QG_FULL_MASK, c);
    if ((tid & 31) == 0) ws[tid >> 5] = c;
    __syncthreads();
    const uint32_t g = blockIdx.x / TP_GROUP;
    const uint32_t gsize = min((uint32_t)TP_GROUP, gridDim.x - g * TP_GROUP);
    if (tid == 0) {
        uint32_t t = 0;
        for (int w = 0; w < TP_WARPS; w++) t += ws[w];
        counts[blockIdx.x] = t;
        __threadfence();
        // atomicInc wraps to zero on the group's last arrival, which then
        // sums the group's counts (all stored and fenced before their arrivals)
        s_last = atomicInc(&arrivals[g], gsize - 1) == gsize - 1;
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    uint32_t gc = tid < (int)gsize ? __ldcg(counts + (size_t)g * TP_GROUP + tid) : 0u;
    static_assert(TP_GROUP == TP_THREADS, "one count per thread");
    gc = __reduce_add_sync(QG_FULL_MASK, gc);
    if ((tid & 31) == 0) ws[tid >> 5] = gc;
    __syncthreads();
    if (tid == 0) {
        uint32_t t = 0;
        for (int w = 0; w < TP_WARPS; w++) t += ws[w];
        gsum[g] = t;
    }
}

// Pass B from pass A's predicate bits: the keys are not read again, and a
// thread loads its four payloads only when one of them is selected (the
// output holds row ids and payloads, never keys).
__global__ void __launch_bounds__(TP_THREADS)
k_filter_write(const uint16_t *__restrict__ mask, const int32_t *__restrict__ pay, long long n,
                 const uint32_t *__restrict__ counts, const uint32_t *__restrict__ gsum, int2 *__restrict__ out,
                 long long cap, long long *__restrict__ d_count) {
    __shared__ uint32_t s_woff[TP_ROUNDS * TP_WARPS];
    __shared__ unsigned long long s_pre[TP_WARPS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t tile = blockIdx.x;
    const long long base = (long long)tile * TP_TILE;
    const uint32_t lt = qg_lanemask_lt();
    const uint32_t fl = __ldg(mask + (size_t)tile * TP_THREADS + tid);
    int4 pv[TP_ROUNDS];
#pragma unroll
    for (int r = 0; r < TP_ROUNDS; r++) {
        pv[r] = make_int4(0, 0, 0, 0);
        if ((fl >> (4 * r)) & 0xfu) tp_load_keys(pay, base + (long long)(r * TP_THREADS + tid) * 4, n, pv[r]);
    }
    // offset of this tile: earlier groups' sums, then this group's earlier tiles
    unsigned long long pre = 0;
    const uint32_t g = tile / TP_GROUP;
    for (uint32_t i = tid; i < g; i += TP_THREADS) pre += __ldg(gsum + i);
    for (uint32_t i = g * TP_GROUP + tid; i < tile; i += TP_THREADS) pre += __ldg(counts + i);
    uint32_t lpre[TP_ROUNDS];
#pragma unroll
    for (int r = 0; r < TP_ROUNDS; r++) {
        const uint32_t f = (fl >> (4 * r)) & 0xfu;
        uint32_t c = 0, tot = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t b = __ballot_sync(QG_FULL_MASK, (f >> j) & 1u);
            c += __popc(b & lt);
            tot += __popc(b);
        }
        lpre[r] = c;
        if (lane == 0) s_woff[r * TP_WARPS + warp] = tot;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) pre += __shfl_down_sync(QG_FULL_MASK, pre, d);
    if (lane == 0) s_pre[warp] = pre;
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the 32 (round, warp) counts in row order
        const uint32_t x = s_woff[lane];
        uint32_t inc = x;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(QG_FULL_MASK, inc, d);
            if (lane >= d) inc += y;
        }
        s_woff[lane] = inc - x;
        if (lane == 31) {
            unsigned long long e = 0;
            for (int w = 0; w < TP_WARPS; w++) e += s_pre[w];
            s_pre[0] = e;
            if (tile == gridDim.x - 1) *d_count = (long long)(e + inc);
        }
    }
    __syncthreads();
    const long long excl = (long long)s_pre[0];
#pragma unroll
    for (int r = 0; r < TP_ROUNDS; r++) {
        long long pos = excl + s_woff[r * TP_WARPS + warp] + lpre[r];
        const long long idx = base + (long long)(r * TP_THREADS + tid) * 4;
        const int pp[4] = {pv[r].x, pv[r].y, pv[r].z, pv[r].w};
#pragma unroll
        for (int j = 0; j < 4; j++) {
            if ((fl >> (4 * r + j)) & 1u) {
                if (pos < cap) out[pos] = make_int2((int)(idx + j), pp[j]);
                pos++;
            }
        }
    }
}

qg_status qg_filter_rec_launch(qg_ctx *ctx, const void *in, int64_t n, int32_t lo, int32_t hi,
                               void *out, int64_t cap, long long *d_count) {
    constexpr int TILE = FT_THREADS * REC_ROUNDS * 2;
    if (n == 0) {
        QG_TRY_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(long long), ctx->stream), "memset");
        return QG_OK;
    }
    if (((uintptr_t)in & 15) != 0 || ((uintptr_t)out & 7) != 0) return QG_ERR_INVALID;
    int64_t tiles = qg_ceil_div(n, TILE);
    if (tiles > 0x7fffffff) return QG_ERR_UNSUPPORTED;
    qg_lookback lb;
    QG_TRY(qg_lb_make(ctx, tiles, QG_SITE_FILTER, &lb));
    qg_pre_launch(ctx);
    k_filter_rec<REC_ROUNDS><<<(unsigned)tiles, FT_THREADS, 0, ctx->stream>>>(
        (const uint4 *)in, n, lo, hi, (uint2 *)out, cap, d_count, lb);
    return qg_check_launch(ctx, "k_filter_rec");
}

static int g_filter_variant = 2;  // two passes: fastest measured (42 us vs 68 us at 16M rows)

qg_status qg_filter_cols_launch(qg_ctx *ctx, const int32_t *key, const int32_t *pay, int64_t n,
                                int32_t lo, int32_t hi, int32_t *out, int64_t cap,
                                long long *d_count) {
    constexpr int TILE = FT_THREADS * COL_ROUNDS * 4;
    if (n == 0) {
        QG_TRY_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(long long), ctx->stream), "memset");
        return QG_OK;
    }
    if (((uintptr_t)key & 15) || ((uintptr_t)pay & 15) || ((uintptr_t)out & 7))
        return QG_ERR_INVALID;
    int64_t tiles = qg_ceil_div(n, TILE);
    if (tiles > 0x7fffffff || n > 0x7fffffffLL) return QG_ERR_UNSUPPORTED;
    qg_lookback lb;
    QG_TRY(qg_lb_make(ctx, tiles, QG_SITE_FILTER, &lb));
    const int variant = qg_effective_variant(ctx, QG_STEER_FILTER, g_filter_variant);
    if (variant == 2) {
        const long long tp_tiles = qg_ceil_div(n, TP_TILE);
        const long long groups = qg_ceil_div(tp_tiles, TP_GROUP);
        char *scr;
        const size_t cg_bytes = qg_align_up((size_t)(tp_tiles + groups) * 4, 256);
        QG_TRY(qg_scratch(ctx, cg_bytes + (size_t)tp_tiles * TP_THREADS * 2, &scr));
        uint32_t *counts = (uint32_t *)scr, *gsum = counts + tp_tiles;
        uint16_t *mask = (uint16_t *)(scr + cg_bytes);
        static_assert(sizeof(((qg_control *)0)->fgroup) / 4 * (long long)TP_GROUP * TP_TILE >= 0x7fffffffLL,
                      "one arrival counter per group of the largest accepted input");
        qg_pre_launch(ctx);
        k_filter_count<<<(unsigned)tp_tiles, TP_THREADS, 0, ctx->stream>>>(key, n, lo, hi, counts, gsum, mask,
                                                                         ctx->ctl->fgroup);
        QG_TRY(qg_check_launch(ctx, "k_filter_count"));
        qg_pre_launch(ctx);
        k_filter_write<<<(unsigned)tp_tiles, TP_THREADS, 0, ctx->stream>>>(mask, pay, n, counts, gsum, (int2 *)out,
                                                                         cap, d_count);
        return qg_check_launch(ctx, "k_filter_write");
    }
    if (variant == 1) {
        static bool attr = false;
        if (!attr) {
            QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_filter_cols_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)sizeof(FpSmem)), "attr");
            attr = true;
        }
        const long long ftiles = qg_ceil_div(n, FP_TILE);
        const int grid = (int)(ftiles < ctx->sm_count * 2LL ? ftiles : ctx->sm_count * 2LL);
        qg_pre_launch(ctx);
        k_filter_cols_tma<<<grid, FP_THREADS, sizeof(FpSmem), ctx->stream>>>(
            key, pay, n, lo, hi, (int2 *)out, cap, d_count, lb, (uint32_t)ftiles);
        return qg_check_launch(ctx, "k_filter_cols_tma");
    }
    qg_pre_launch(ctx);
    k_filter_cols<COL_ROUNDS><<<(unsigned)tiles, FT_THREADS, 0, ctx->stream>>>(
        key, pay, n, lo, hi, (int2 *)out, cap, d_count, lb);
    return qg_check_launch(ctx, "k_filter_cols");
}

// 0: one tile per CTA, rows staged in registers, decoupled look-back;
// 1: persistent CTAs with a bulk-copy ring; 2: two passes (count, write)
// with no look-back (all bit-identical; chosen by measurement).
int qg_filter_default_variant() { return g_filter_variant; }

extern "C" QG_API qg_status qg_filter_set_variant(int variant) {
    if (variant < 0 || variant > 2) return QG_ERR_INVALID;
    g_filter_variant = variant;
    return QG_OK;
}

extern "C" {

QG_API qg_status qg_filter_range_rec_async(qg_ctx *ctx, const void *in, int64_t n, int32_t lo,
                                           int32_t hi, void *out, int64_t cap, int64_t *d_out_n) {
    if (!ctx || n < 0 || cap < 0 || !d_out_n || (n > 0 && (!in || !out))) return QG_ERR_INVALID;
    if (n >= (1LL << 32)) return QG_ERR_UNSUPPORTED;
    return qg_filter_rec_launch(ctx, in, n, lo, hi, out, cap, (long long *)d_out_n);
}

QG_API qg_status qg_filter_range_rec(qg_ctx *ctx, const void *in, int64_t n, int32_t lo,
                                     int32_t hi, void *out, int64_t cap, int64_t *out_n) {
    if (!ctx || !out_n) return QG_ERR_INVALID;
    long long *d_count = (long long *)&ctx->ctl->counter[0];
    QG_TRY(qg_filter_range_rec_async(ctx, in, n, lo, hi, out, cap, (int64_t *)d_count));
    return finish_count(ctx, d_count, cap, out_n);
}

QG_API qg_status qg_filter_cols_async(qg_ctx *ctx, const int32_t *key, const int32_t *pay,
                                      int64_t n, int32_t lo, int32_t hi, int32_t *out, int64_t cap,
                                      int64_t *d_out_n) {
    if (!ctx || n < 0 || cap < 0 || !d_out_n || (n > 0 && (!key || !pay || !out)))
        return QG_ERR_INVALID;
    return qg_filter_cols_launch(ctx, key, pay, n, lo, hi, out, cap, (long long *)d_out_n);
}

QG_API qg_status qg_filter_cols(qg_ctx *ctx, const int32_t *key, const int32_t *pay, int64_t n,
                                int32_t lo, int32_t hi, int32_t *out, int64_t cap,
                                int64_t *out_n) {
    if (!ctx || !out_n) return QG_ERR_INVALID;
    // With a cost model attached the variant is its choice for this size; the
    // selectivity estimate is the predicate's share of the int32 range.
    qg_steer_call sc;
    qg_steer_begin(ctx, QG_STEER_FILTER, n, 0, ((double)hi - (double)lo + 1.0) / 4294967296.0, &sc);
    long long *d_count = (long long *)&ctx->ctl->counter[0];
    qg_status st = qg_filter_cols_async(ctx, key, pay, n, lo, hi, out, cap, (int64_t *)d_count);
    if (st == QG_OK) st = finish_count(ctx, d_count, cap, out_n);
    qg_steer_end(ctx, &sc, st);
    return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Column filter that allocates nothing.
//
// For callers that cannot allocate device memory themselves -- code running
// inside an allocator or memory-pool callback, in a process whose device
// memory is carved up by a framework that forbids extra cudaMalloc calls, or
// on a path that must never block on the allocator -- and so cannot create a
// qg_ctx (qg_ctx_create allocates its control block and scratch).  The
// look-back status words and the control block this kernel needs live in the
// file-scope device array below instead, sized for at most
// QG_NOALLOC_MAX_ROWS rows; every GPU that loads the library holds it
// (about 128 KB) until the process exits.
//
// Host code only sees a stand-in for the array, not its device address, so
// the first call on a device (with that device current) looks the address up
// with cudaGetSymbolAddress and keeps it; make that first call before any
// stream capture.  Every call shares the one array: the counters and the
// status words the call uses are cleared at the start of each call (stream
// ordered), and calls that overlap on the GPU (on different streams, or from
// different threads without ordering) race on it.
// ---------------------------------------------------------------------------
#define QG_NOALLOC_MAX_ROWS (1LL << 26)
#define QG_NOALLOC_TILE (FT_THREADS * COL_ROUNDS * 4)
#define QG_NOALLOC_MAX_TILES ((QG_NOALLOC_MAX_ROWS + QG_NOALLOC_TILE - 1) / QG_NOALLOC_TILE)
#define QG_NOALLOC_MAX_DEVICES 64

struct qg_noalloc_scratch {
    qg_control ctl;
    unsigned long long status[QG_NOALLOC_MAX_TILES];
};
static_assert((long long)QG_NOALLOC_MAX_TILES * QG_NOALLOC_TILE >= QG_NOALLOC_MAX_ROWS,
              "no-alloc status words cover the largest accepted input");

static __device__ __align__(256) qg_noalloc_scratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device, looked up by the first call
// on that device.  A cudaDeviceReset (or any teardown of the device's primary
// context) makes the remembered address stale; qg_noalloc_forget() drops it.
static qg_noalloc_scratch *g_noalloc_addr[QG_NOALLOC_MAX_DEVICES];
// Polls a look-back wait of the no-alloc filter makes before it gives up.
static uint32_t g_noalloc_spin = 1u << 22;

extern "C" QG_API qg_status qg_noalloc_set_spin_limit(uint32_t polls) {
    g_noalloc_spin = polls;
    return QG_OK;
}

extern "C" QG_API qg_status qg_noalloc_forget(void) {
    for (int i = 0; i < QG_NOALLOC_MAX_DEVICES; i++) g_noalloc_addr[i] = nullptr;
    return QG_OK;
}

// Reports a device-side error of the call through the count (as -code) and
// clears the error word for the next call.
__global__ void k_noalloc_report(qg_noalloc_scratch *s, long long *d_count) {
    const int e = s->ctl.err;
    if (e) {
        *d_count = -(long long)e;
        s->ctl.err = 0;
        s->ctl.err_site = 0;
    }
}

extern "C" QG_API qg_status qg_filter_cols_noalloc(const int32_t *key, const int32_t *pay, int64_t n,
                                                   int32_t lo, int32_t hi, int32_t *out,
                                                   int64_t cap, int64_t *d_out_n, void *stream) {
    constexpr int TILE = QG_NOALLOC_TILE;
    if (n < 0 || cap < 0 || !d_out_n || (n > 0 && (!key || !pay || !out))) return QG_ERR_INVALID;
    if (n > QG_NOALLOC_MAX_ROWS || (n + TILE - 1) / TILE > QG_NOALLOC_MAX_TILES) return QG_ERR_UNSUPPORTED;
    if (((uintptr_t)key & 15) || ((uintptr_t)pay & 15) || ((uintptr_t)out & 7) ||
        ((uintptr_t)d_out_n & 7))
        return QG_ERR_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= QG_NOALLOC_MAX_DEVICES) {
        cudaGetLastError();
        return QG_ERR_CUDA;
    }
    if (!g_noalloc_addr[dev]) {  // set-up, once per device
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return QG_ERR_CUDA;
        }
        g_noalloc_addr[dev] = (qg_noalloc_scratch *)p;
    }
    qg_noalloc_scratch *s = g_noalloc_addr[dev];
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0)
        return cudaMemsetAsync(d_out_n, 0, sizeof(long long), st) == cudaSuccess ? QG_OK : QG_ERR_CUDA;
    const long long tiles = (n + TILE - 1) / TILE;
    // Counters and error word start at zero; status words of this call's
    // tiles are cleared so nothing from an earlier call can be read as ready.
    if (cudaMemsetAsync(&s->ctl, 0, sizeof(qg_control), st) != cudaSuccess ||
        cudaMemsetAsync(s->status, 0, (size_t)tiles * sizeof(unsigned long long), st) != cudaSuccess) {
        cudaGetLastError();
        return QG_ERR_CUDA;
    }
    qg_lookback lb{s->status, &s->ctl, g_noalloc_spin, QG_SITE_FILTER};
    k_filter_cols<COL_ROUNDS><<<(unsigned)tiles, FT_THREADS, 0, st>>>(
        key, pay, n, lo, hi, (int2 *)out, cap, (long long *)d_out_n, lb);
    k_noalloc_report<<<1, 1, 0, st>>>(s, (long long *)d_out_n);
    if (cudaGetLastError() != cudaSuccess) return QG_ERR_CUDA;
    return QG_OK;
}
