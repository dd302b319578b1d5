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

// Records (uint2 {x, y}), two per 128-bit load.  ROUNDS loads per thread.
template <int ROUNDS>
__global__ void __launch_bounds__(FT_THREADS)
k_filter_rec(const uint4 *__restrict__ in, long long n, int32_t lo, int32_t hi,
             uint2 *__restrict__ out, long long cap, long long *__restrict__ d_count,
             qg_lookback lb) {
    constexpr int TILE = FT_THREADS * ROUNDS * 2;
    __shared__ uint32_t s_tile, s_epoch, s_excl;
    __shared__ uint32_t s_woff[ROUNDS * FT_WARPS];
    qg_lb_begin(lb, &s_tile, &s_epoch);
    const uint32_t tile = s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long base = (long long)tile * TILE;
    const uint32_t lt = qg_lanemask_lt();

    uint4 v[ROUNDS];
    uint32_t fl = 0;            // bit 2r: first record of round r, bit 2r+1: second
    uint32_t lpre[ROUNDS];      // selected records of lower lanes in this round
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long idx = base + (long long)(r * FT_THREADS + tid) * 2;
        bool f0 = false, f1 = false;
        if (idx + 1 < n) {
            int4 t = qg_ldg_stream(reinterpret_cast<const int4 *>(in) + (idx >> 1));
            v[r] = make_uint4(t.x, t.y, t.z, t.w);
            f0 = ((int32_t)v[r].y >= lo) & ((int32_t)v[r].y <= hi);
            f1 = ((int32_t)v[r].w >= lo) & ((int32_t)v[r].w <= hi);
        } else if (idx < n) {
            const uint2 *in2 = reinterpret_cast<const uint2 *>(in);
            uint2 a = in2[idx];
            v[r] = make_uint4(a.x, a.y, 0, 0);
            f0 = ((int32_t)a.y >= lo) & ((int32_t)a.y <= hi);
        } else {
            v[r] = make_uint4(0, 0, 0, 0);
        }
        uint32_t b0 = __ballot_sync(QG_FULL_MASK, f0), b1 = __ballot_sync(QG_FULL_MASK, f1);
        lpre[r] = __popc(b0 & lt) + __popc(b1 & lt);
        if (lane == 0) s_woff[r * FT_WARPS + warp] = __popc(b0) + __popc(b1);
        fl |= (uint32_t)f0 << (2 * r);
        fl |= (uint32_t)f1 << (2 * r + 1);
    }
    __syncthreads();
    if (warp == 0) {
        // Exclusive scan of the ROUNDS*WARPS per-warp counts, round-major
        // (the order of the rows they cover).
        constexpr int E = ROUNDS * FT_WARPS;
        constexpr int PER = (E + 31) / 32;
        uint32_t loc[PER];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            int e = lane * PER + k;
            loc[k] = (e < E) ? s_woff[e] : 0u;
            sum += loc[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(QG_FULL_MASK, incl, d);
            if (lane >= d) incl += t;
        }
        uint32_t total = __shfl_sync(QG_FULL_MASK, incl, 31);
        uint32_t run = incl - sum;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            int e = lane * PER + k;
            if (e < E) s_woff[e] = run;
            run += loc[k];
        }
        uint32_t excl = qg_lb_warp_exclusive(lb, tile, s_epoch, total);
        if (lane == 0) {
            s_excl = excl;
            if (tile == gridDim.x - 1) *d_count = (long long)excl + total;
        }
    }
    __syncthreads();
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
    qg_lb_end(lb);
}

// Columns: int32 key and payload, four rows per 128-bit load.  Output is the
// int32 pair (row id, payload).
template <int ROUNDS>
__global__ void __launch_bounds__(FT_THREADS)
k_filter_cols(const int32_t *__restrict__ key, const int32_t *__restrict__ pay, long long n,
              int32_t lo, int32_t hi, int2 *__restrict__ out, long long cap,
              long long *__restrict__ d_count, qg_lookback lb) {
    constexpr int TILE = FT_THREADS * ROUNDS * 4;
    __shared__ uint32_t s_tile, s_epoch, s_excl;
    __shared__ uint32_t s_woff[ROUNDS * FT_WARPS];
    qg_lb_begin(lb, &s_tile, &s_epoch);
    const uint32_t tile = s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long base = (long long)tile * TILE;
    const uint32_t lt = qg_lanemask_lt();

    int4 kv[ROUNDS], pv[ROUNDS];
    uint32_t fl = 0;  // bit 4r+j
    uint32_t lpre[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        long long idx = base + (long long)(r * FT_THREADS + tid) * 4;
        uint32_t f = 0;
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
    __syncthreads();
    if (warp == 0) {
        constexpr int E = ROUNDS * FT_WARPS;
        constexpr int PER = (E + 31) / 32;
        uint32_t loc[PER];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            int e = lane * PER + k;
            loc[k] = (e < E) ? s_woff[e] : 0u;
            sum += loc[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(QG_FULL_MASK, incl, d);
            if (lane >= d) incl += t;
        }
        uint32_t total = __shfl_sync(QG_FULL_MASK, incl, 31);
        uint32_t run = incl - sum;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            int e = lane * PER + k;
            if (e < E) s_woff[e] = run;
            run += loc[k];
        }
        uint32_t excl = qg_lb_warp_exclusive(lb, tile, s_epoch, total);
        if (lane == 0) {
            s_excl = excl;
            if (tile == gridDim.x - 1) *d_count = (long long)excl + total;
        }
    }
    __syncthreads();
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
    qg_lb_end(lb);
}

constexpr int REC_ROUNDS = 8;   // 4096 records per tile
constexpr int COL_ROUNDS = 4;   // 4096 rows per tile

}  // namespace

static qg_status finish_count(qg_ctx *ctx, long long *d_count, int64_t cap, int64_t *out_n) {
    long long h = 0;
    QG_TRY(qg_read_i64(ctx, d_count, &h));
    QG_TRY(qg_collect_error(ctx));
    *out_n = h;
    if (h > cap) return QG_ERR_CAPACITY;
    return QG_OK;
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
    char *scr;
    QG_TRY(qg_scratch(ctx, qg_lb_bytes(tiles), &scr));
    qg_lookback lb{(unsigned long long *)scr, ctx->ctl, ctx->spin_limit, QG_SITE_FILTER};
    qg_pre_launch(ctx);
    k_filter_rec<REC_ROUNDS><<<(unsigned)tiles, FT_THREADS, 0, ctx->stream>>>(
        (const uint4 *)in, n, lo, hi, (uint2 *)out, cap, d_count, lb);
    return qg_check_launch(ctx, "k_filter_rec");
}

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
    char *scr;
    QG_TRY(qg_scratch(ctx, qg_lb_bytes(tiles), &scr));
    qg_lookback lb{(unsigned long long *)scr, ctx->ctl, ctx->spin_limit, QG_SITE_FILTER};
    qg_pre_launch(ctx);
    k_filter_cols<COL_ROUNDS><<<(unsigned)tiles, FT_THREADS, 0, ctx->stream>>>(
        key, pay, n, lo, hi, (int2 *)out, cap, d_count, lb);
    return qg_check_launch(ctx, "k_filter_cols");
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
    long long *d_count = (long long *)&ctx->ctl->counter[0];
    QG_TRY(qg_filter_cols_async(ctx, key, pay, n, lo, hi, out, cap, (int64_t *)d_count));
    return finish_count(ctx, d_count, cap, out_n);
}

}  // extern "C"
