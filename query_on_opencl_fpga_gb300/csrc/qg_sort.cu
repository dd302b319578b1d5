// qg_sort.cu -- LSD radix sort by an unsigned 32-bit key.
//
// Replaces the reference's bitonic sort (bitonicSortShared +
// bitonicMergeGlobal, kernel/aggregation/1/group_by_cu_op_dp.cl:89-291,
// driven by radixSortImpl_sm, host/host/testSort.cpp:24-136), which needs a
// power-of-two n >= 2048 and O(n log^2 n) global passes.  Here:
//   1. one histogram pass counts the 8-bit digits of every key position (or
//      the producer of the data counted them already, as the join probe does);
//   2. the host skips digit positions where all keys share one digit;
//   3. each remaining position is one "onesweep" pass: a tile is ranked by
//      digit in shared memory (warp ballots give peer masks), its per-digit
//      global offsets come from a decoupled look-back over earlier tiles, and
//      the tile is reordered in shared memory so that each digit's run is
//      written with consecutive addresses.
// Every pass is stable, so the LSD composition is a correct sort; the order
// among equal keys is input order (the reference's is unspecified).
//
// Two item layouts:
//   REC: 64-bit items, key = high 32 bits (a Record uint2 {x, y} read as one
//        little-endian u64 has y in the high word).
//   KV3: three u32 columns (key, a, b) -- the join output (key, R.payload,
//        S.payload).
#include <string.h>
#include <utility>
#include <vector>
#include "qg_internal.cuh"
#include "qg_sort.cuh"
#include "qg_part.cuh"

namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;  // 4096
constexpr int RS_LB = 8;  // predecessors read per look-back round

constexpr uint32_t ST_AGG = 1u << 30;
constexpr uint32_t ST_PRE = 2u << 30;
constexpr uint32_t ST_VAL = (1u << 30) - 1;

__global__ void __launch_bounds__(256)
k_radix_hist(const uint32_t *__restrict__ kin, const unsigned long long *__restrict__ rin,
             long long n, uint32_t key_off, int npos, uint32_t *__restrict__ ghist,
             unsigned long long *__restrict__ copy) {
    __shared__ uint32_t sh[4][QG_RADIX];
    for (int i = threadIdx.x; i < 4 * QG_RADIX; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    // Four items per thread and round, all loaded before any is counted: with
    // one load in flight per thread the kernel waited on DRAM latency
    // (long-scoreboard stalls, 41 % of DRAM bandwidth).
    constexpr int U = 4;
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < n; i += U * stride) {
        uint32_t k[U];
        if (kin) {
#pragma unroll
            for (int u = 0; u < U; u++) k[u] = __ldg(kin + i + u * stride);
        } else {
            unsigned long long v[U];
#pragma unroll
            for (int u = 0; u < U; u++) v[u] = __ldg(rin + i + u * stride);
#pragma unroll
            for (int u = 0; u < U; u++) {
                if (copy) copy[i + u * stride] = v[u];  // records: optionally a copy for the passes to start from
                k[u] = (uint32_t)(v[u] >> 32);
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const uint32_t ku = k[u] - key_off;
            for (int p = 0; p < npos; p++) atomicAdd(&sh[p][(ku >> (8 * p)) & 255u], 1u);
        }
    }
    for (; i < n; i += stride) {
        uint32_t k;
        if (kin) {
            k = __ldg(kin + i) - key_off;
        } else {
            const unsigned long long v = __ldg(rin + i);
            if (copy) copy[i] = v;
            k = (uint32_t)(v >> 32) - key_off;
        }
        for (int p = 0; p < npos; p++) atomicAdd(&sh[p][(k >> (8 * p)) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < npos * QG_RADIX; i += blockDim.x) {
        uint32_t c = (&sh[0][0])[i];
        if (c) atomicAdd(&ghist[i], c);
    }
}

template <bool KV3, bool SIDE = false>
struct RsSmem {
    uint32_t whist[RS_WARPS][QG_RADIX];
    uint32_t dstart[QG_RADIX];
    uint32_t goff[QG_RADIX];
    uint32_t wsum[RS_WARPS];
    uint32_t tile;
    // REC: v holds the u64 items; KV3: v holds (a, b) pairs and k the keys
    unsigned long long v[RS_TILE];
    uint32_t k[KV3 ? RS_TILE : 1];
    uint16_t bid[SIDE ? RS_TILE : 1];  // REC with a bucket-id sidecar: the reordered ids
    uint8_t dg[RS_TILE];  // digit of each reordered item
};

// Digit of a key: radix form ((k - key_off) >> shift) & 255, or the bits
// [shift, shift + 8) of the learned partition bucket of k.
template <bool LEARNED>
__device__ __forceinline__ uint32_t rs_digit(uint32_t k, uint32_t key_off, int shift,
                                             const qg_cdf_model *model) {
    if (LEARNED) return (qg_cdf_bucket(model, k) >> shift) & 255u;
    return (uint32_t)((unsigned long long)(k - key_off) >> shift) & 255u;  // shift may exceed 31
}

// Four CTAs per SM (64 registers; a few bytes spill): one CTA's load phase
// overlaps another's ranking and writes.  Three passes over 64M REC items
// took 1.29 ms this way against 1.57 ms with two CTAs at 126 registers.
// DIG: 0 radix digit of the key, 1 learned partition function of the key,
// 2 bits of the bucket id in the source's sidecar (REC only).
// RANK: how an item's rank within its digit is found -- 0 eight warp ballots,
// 1 one match instruction, 3 one match instruction on the digit's high four
// bits (at most 16 groups, where match is fast) and four ballots on the low
// four (stable all three), 2 one shared-memory atomic on the tile's digit
// counter (not stable: for a first LSD pass whose order among equal digits
// nothing after it needs).
template <bool KV3, int DIG, int RANK = 0>
__global__ void __launch_bounds__(RS_THREADS, 4)
k_radix_pass(qg_sort_bufs src, qg_sort_bufs dst, long long n, int shift, uint32_t key_off,
             const qg_cdf_model *model, const uint32_t *__restrict__ dbase,
             uint32_t *__restrict__ status, qg_control *ctl, uint32_t spin_limit,
             const unsigned long long *__restrict__ d_n, const uint32_t *__restrict__ trivial) {
    extern __shared__ __align__(16) unsigned char rs_raw[];
    constexpr bool side = !KV3 && DIG == 2;  // digits from the bucket-id sidecar
    RsSmem<KV3, side> &S = *reinterpret_cast<RsSmem<KV3, side> *>(rs_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Item count known only on the device (graph-captured sorts): the grid
    // covers the bound n, and CTAs past the real count leave at once (no
    // tile before them waits on them).
    if (d_n && *d_n < (unsigned long long)n) n = (long long)*d_n;
    if ((long long)blockIdx.x * RS_TILE >= n) return;
    if (trivial && __ldg(trivial)) {  // one digit value holds every item: a stable pass is the identity
        // every load of the tile before any store (the buffers are distinct,
        // which the compiler cannot see)
        const long long b0 = (long long)blockIdx.x * RS_TILE;
        const int cnt = (int)min((long long)RS_TILE, n - b0);
        unsigned long long v[RS_ITEMS];
        uint32_t kk[KV3 ? RS_ITEMS : 1];
#pragma unroll
        for (int i = 0; i < RS_ITEMS; i++) {
            const int j = i * RS_THREADS + tid;
            if (j < cnt) {
                if (KV3) {
                    kk[i] = __ldcs(src.k + b0 + j);
                    v[i] = ((unsigned long long)__ldcs(src.b + b0 + j) << 32) | __ldcs(src.a + b0 + j);
                } else {
                    v[i] = __ldcs(src.rec + b0 + j);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < RS_ITEMS; i++) {
            const int j = i * RS_THREADS + tid;
            if (j < cnt) {
                if (KV3) {
                    dst.k[b0 + j] = kk[i];
                    dst.a[b0 + j] = (uint32_t)v[i];
                    dst.b[b0 + j] = (uint32_t)(v[i] >> 32);
                } else {
                    dst.rec[b0 + j] = v[i];
                    if (side && dst.bid) dst.bid[b0 + j] = src.bid[b0 + j];
                }
            }
        }
        return;
    }
    for (int i = tid; i < RS_WARPS * QG_RADIX; i += RS_THREADS) (&S.whist[0][0])[i] = 0;
    __syncthreads();
    // Tile i is CTA i (started in index order); the status words are cleared
    // before every pass, so nothing has to be reset at the end.
    const uint32_t tile = blockIdx.x;
    const long long base = (long long)tile * RS_TILE;
    const long long wbase = base + (long long)warp * 32 * RS_ITEMS;
    const uint32_t lt = qg_lanemask_lt();

    // REC items carry their key in the high word, so only KV3 keeps a key
    // array; each item's digit and rank share one word (rank < 2^24).
    uint32_t key[KV3 ? RS_ITEMS : 1];
    unsigned long long val[RS_ITEMS];
    uint32_t rd[RS_ITEMS];  // digit << 24 | rank within the warp's digit
    // All loads are issued before any ranking: __syncwarp orders memory, so
    // a load placed after one in program order cannot be hoisted above it,
    // and interleaving would pay one DRAM latency per item.
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        long long idx = wbase + i * 32 + lane;
        if (idx < n) {
            if (KV3) {
                key[i] = __ldcs(src.k + idx);
                val[i] = ((unsigned long long)__ldcs(src.b + idx) << 32) | __ldcs(src.a + idx);
            } else {
                val[i] = __ldcs(src.rec + idx);
                if (side) rd[i] = __ldcs(src.bid + idx);  // the bucket id, until its digit replaces it
            }
        } else {
            val[i] = 0;
            if (KV3) key[i] = 0;
            if (side) rd[i] = 0;
        }
    }
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        long long idx = wbase + i * 32 + lane;
        bool valid = idx < n;
        const uint32_t ki = KV3 ? key[i] : (uint32_t)(val[i] >> 32);
        const uint32_t d = side ? (rd[i] >> shift) & 255u : rs_digit<DIG == 1>(ki, key_off, shift, model);
        rd[i] = d << 24;
        // lanes holding the same digit: one match instruction (passes with
        // few digit values in use) or eight ballots
        if constexpr (RANK == 2) {
            if (valid) rd[i] |= atomicAdd(&S.whist[0][d], 1u);
            continue;
        }
        uint32_t peers;
        if (RANK == 1) {
            peers = __match_any_sync(QG_FULL_MASK, valid ? d : 256u);  // the tail's invalid lanes share 256
        } else if (RANK == 3) {
            peers = __match_any_sync(QG_FULL_MASK, valid ? d >> 4 : 16u);  // the tail's invalid lanes share 16
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const uint32_t bal = __ballot_sync(QG_FULL_MASK, (d >> b) & 1u);
                peers &= ((d >> b) & 1u) ? bal : ~bal;
            }
        } else if (RANK == 4) {
            peers = __match_any_sync(QG_FULL_MASK, valid ? d >> 4 : 16u) &
                    __match_any_sync(QG_FULL_MASK, valid ? d & 15u : 16u);
        } else {
            peers = __ballot_sync(QG_FULL_MASK, valid);
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const uint32_t bal = __ballot_sync(QG_FULL_MASK, (d >> b) & 1u);
                peers &= ((d >> b) & 1u) ? bal : ~bal;
            }
        }
        uint32_t before = valid ? S.whist[warp][d] : 0u;
        __syncwarp();
        if (valid) {
            rd[i] |= before + __popc(peers & lt);
            if (lane == 31 - __clz(peers)) S.whist[warp][d] = before + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    {
        // Thread t owns digit t: offsets of each warp within the digit, the
        // tile's count of the digit, then its place among the digits.
        const int t = tid;
        uint32_t run = 0;
        if constexpr (RANK == 2) {
            run = S.whist[0][t];  // ranks are tile-wide already
        } else {
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++) {
                uint32_t c = S.whist[w][t];
                S.whist[w][t] = run;
                run += c;
            }
        }
        const uint32_t total = run;
        uint32_t inc = total;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t x = __shfl_up_sync(QG_FULL_MASK, inc, d);
            if (lane >= d) inc += x;
        }
        if (lane == 31) S.wsum[warp] = inc;
        __syncthreads();
        uint32_t woff = 0;
        for (int w = 0; w < warp; w++) woff += S.wsum[w];
        const uint32_t dstart = woff + inc - total;
        S.dstart[t] = dstart;

        // Look-back for digit t over earlier tiles.
        uint32_t *st = status + (size_t)tile * QG_RADIX + t;
        uint32_t excl = 0;
        if (tile == 0) {
            qg_st_relaxed_u32(st, ST_PRE | total);
        } else {
            qg_st_relaxed_u32(st, ST_AGG | total);
            // Windowed look-back: RS_LB predecessors' words are loaded
            // together, so a chain of tiles that only published aggregates
            // costs one L2 round trip per RS_LB tiles instead of per tile.
            long long j = (long long)tile - 1;
            bool done = false;
            while (!done) {
                uint32_t w[RS_LB];
#pragma unroll
                for (int u = 0; u < RS_LB; u++)
                    w[u] = (j - u >= 0) ? qg_ld_relaxed_u32(status + (size_t)(j - u) * QG_RADIX + t) : ST_PRE;
#pragma unroll
                for (int u = 0; u < RS_LB; u++) {
                    if (done) break;
                    uint32_t spins = 0;
                    while (!(w[u] & (ST_AGG | ST_PRE))) {
                        if (spins >= spin_limit) {
                            qg_record_error(ctl, QG_ERR_TIMEOUT, QG_SITE_SORT_LOOKBACK);
                            w[u] = ST_PRE;
                            break;
                        }
                        spins++;
                        __nanosleep(32);
                        w[u] = qg_ld_relaxed_u32(status + (size_t)(j - u) * QG_RADIX + t);
                    }
                    excl += w[u] & ST_VAL;
                    if (w[u] & ST_PRE) done = true;
                }
                j -= RS_LB;
            }
            qg_st_relaxed_u32(st, ST_PRE | ((excl + total) & ST_VAL));
        }
        S.goff[t] = dbase[t] + excl - dstart;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        long long idx = wbase + i * 32 + lane;
        if (idx < n) {
            const uint32_t d = rd[i] >> 24;
            uint32_t pos = S.dstart[d] + (RANK == 2 ? 0u : S.whist[warp][d]) + (rd[i] & 0xffffffu);
            S.v[pos] = val[i];
            S.dg[pos] = (uint8_t)d;
            if (KV3) S.k[pos] = key[i];
            if (!KV3 && side && dst.bid) S.bid[pos] = __ldg(src.bid + idx);  // read again: no register held
        }
    }
    __syncthreads();
    long long cnt = n - base;
    if (cnt > RS_TILE) cnt = RS_TILE;
    for (int p = tid; p < cnt; p += RS_THREADS) {
        unsigned long long v = S.v[p];
        uint32_t k = KV3 ? S.k[p] : (uint32_t)(v >> 32);
        uint32_t d = S.dg[p];
        uint32_t g = S.goff[d] + (uint32_t)p;
        if (KV3) {
            dst.k[g] = k;
            dst.a[g] = (uint32_t)v;
            dst.b[g] = (uint32_t)(v >> 32);
        } else {
            dst.rec[g] = v;
            if (side && dst.bid) dst.bid[g] = S.bid[p];
        }
    }
}

}  // namespace

int qg_sort_positions(int bits) {
    int npos = (bits + 7) / 8;
    if (npos < 1) npos = 1;
    if (npos > 4) npos = 4;
    return npos;
}

qg_status qg_radix_histogram(qg_ctx *ctx, const qg_sort_bufs &src, bool kv3, long long n,
                             uint32_t key_off, int npos, uint32_t *d_hist, unsigned long long *copy) {
    QG_TRY_CUDA(ctx, cudaMemsetAsync(d_hist, 0, 4 * QG_RADIX * 4, ctx->stream), "memset hist");
    if (n == 0) return QG_OK;
    int hblocks = ctx->sm_count * 8;  // 2048 threads per SM at 32 registers
    long long maxb = (n + 255) / 256;
    if (hblocks > maxb) hblocks = (int)maxb;
    qg_pre_launch(ctx);
    k_radix_hist<<<hblocks, 256, 0, ctx->stream>>>(kv3 ? src.k : nullptr, kv3 ? nullptr : src.rec,
                                                   n, key_off, npos, d_hist, kv3 ? nullptr : copy);
    return qg_check_launch(ctx, "k_radix_hist");
}

int qg_sort_plan(const uint32_t *h_hist, int npos, long long n, int *passes, uint32_t *bases) {
    int np = 0;
    for (int p = 0; p < npos; p++) {
        bool trivial = false;
        uint32_t run = 0;
        for (int d = 0; d < QG_RADIX; d++) {
            uint32_t c = h_hist[p * QG_RADIX + d];
            if ((long long)c == n) trivial = true;
            bases[p * QG_RADIX + d] = run;
            run += c;
        }
        if (!trivial) passes[np++] = p;
    }
    return np;
}

template <bool KV3, int DIG>
static qg_status rs_set_attr(qg_ctx *ctx) {
    static bool done = false;
    if (!done) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_radix_pass<KV3, DIG, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sizeof(RsSmem<KV3, DIG == 2>)), "attr");
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_radix_pass<KV3, DIG, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sizeof(RsSmem<KV3, DIG == 2>)), "attr");
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_radix_pass<KV3, DIG, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sizeof(RsSmem<KV3, DIG == 2>)), "attr");
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_radix_pass<KV3, DIG, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sizeof(RsSmem<KV3, DIG == 2>)), "attr");
        if constexpr (!KV3)
            QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_radix_pass<KV3, DIG, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)sizeof(RsSmem<KV3, DIG == 2>)), "attr");
        done = true;
    }
    return QG_OK;
}

// Ranking by match instruction for a pass with at most 16 digit values in
// use (the top pass of narrow keys): measured faster there (the 64M-record
// sort of 20-bit keys, 1.30 -> 1.22 ms over its passes), while passes with
// many digit values were slower with it (the join's partition passes 1.10 ->
// 1.38 ms) and keep the eight ballots.
// Stable ranking of the passes with many digit values: -1 the default (3),
// else forced -- 0 eight ballots, 3 a match on the high four bits and four
// ballots, 4 a match on each half (ANDed).  Measured on GB300 with 0 / 3 / 4:
// the 64M-record sort of a fresh unsorted copy, passes 1.290 / 1.265 /
// 1.437 ms; the join's stable partition pass 0.778 / 0.766 / 0.855 ms.  (Form
// 4 had looked fastest when the sort was timed re-sorting its own sorted
// output, where a warp's items share their high digits.)
static int g_rs_stable_rank = -1;

extern "C" QG_API qg_status qg_sort_set_rank(int mode) {
    if (mode != -1 && mode != 0 && mode != 3 && mode != 4) return QG_ERR_INVALID;
    g_rs_stable_rank = mode;
    return QG_OK;
}

static bool rs_few_digits(const uint32_t *hb, long long n) {
    int used = 0;
    for (int d = 0; d < QG_RADIX; d++) {
        const unsigned long long hi = d + 1 < QG_RADIX ? hb[d + 1] : (unsigned long long)n;
        used += hi > hb[d];
    }
    return used <= 16;
}

qg_status qg_radix_passes_pf(qg_ctx *ctx, bool kv3, qg_sort_bufs a, qg_sort_bufs b, long long n,
                             const qg_part_fn &pf, const int *passes, int np, const uint32_t *h_bases,
                             bool *result_in_b, bool first_unstable) {
    *result_in_b = false;
    if (np == 0 || n <= 1) return QG_OK;
    if (n >= (1LL << 30)) return QG_ERR_UNSUPPORTED;
    if (kv3 && pf.learned) return QG_ERR_UNSUPPORTED;
    const long long tiles = (n + RS_TILE - 1) / RS_TILE;
    size_t need = 4 * QG_RADIX * 4 + (size_t)tiles * QG_RADIX * 4;
    char *scr;
    QG_TRY(qg_scratch(ctx, need, &scr));
    uint32_t *dbase = (uint32_t *)scr;
    uint32_t *status = dbase + 4 * QG_RADIX;
    // 4 KB of digit bases, in stream order before the passes that read them.
    QG_TRY(qg_stage_bases(ctx, h_bases, dbase));
    // REC items with a bucket-id sidecar: digits come from the sidecar, whatever
    // the partition function (it was evaluated once, when the ids were written).
    const bool side = !kv3 && a.bid != nullptr && b.bid != nullptr;
    const size_t smem = kv3 ? sizeof(RsSmem<true>) : side ? sizeof(RsSmem<false, true>) : sizeof(RsSmem<false>);
    if (kv3) QG_TRY((rs_set_attr<true, 0>(ctx)));
    else if (side) QG_TRY((rs_set_attr<false, 2>(ctx)));
    else if (pf.learned) QG_TRY((rs_set_attr<false, 1>(ctx)));
    else QG_TRY((rs_set_attr<false, 0>(ctx)));
    bool in_a = true;
    for (int i = 0; i < np; i++) {
        const int p = passes[i];
        QG_TRY_CUDA(ctx, cudaMemsetAsync(status, 0, (size_t)tiles * QG_RADIX * 4, ctx->stream), "memset status");
        const qg_sort_bufs &s = in_a ? a : b;
        qg_sort_bufs d = in_a ? b : a;
        if (side && i == np - 1) d.bid = nullptr;  // the last pass's ids are not read again
        const int shift = (pf.learned || side) ? 8 * p : pf.shift + 8 * p;
        const bool m = rs_few_digits(h_bases + p * QG_RADIX, n);
        // the first pass of a caller that needs only the grouping need not be stable
        const int sr = g_rs_stable_rank >= 0 ? g_rs_stable_rank : 3;
        const int rk = (first_unstable && i == 0 && !kv3) ? 2 : (m ? 1 : sr);
        auto kern = kv3 ? (m ? k_radix_pass<true, 0, 1> : sr == 3 ? k_radix_pass<true, 0, 3> : sr == 4 ? k_radix_pass<true, 0, 4> : k_radix_pass<true, 0, 0>)
                    : side ? (rk == 2 ? k_radix_pass<false, 2, 2> : rk == 1 ? k_radix_pass<false, 2, 1> : rk == 3 ? k_radix_pass<false, 2, 3> : rk == 4 ? k_radix_pass<false, 2, 4> : k_radix_pass<false, 2, 0>)
                    : pf.learned ? (rk == 2 ? k_radix_pass<false, 1, 2> : rk == 1 ? k_radix_pass<false, 1, 1> : rk == 3 ? k_radix_pass<false, 1, 3> : rk == 4 ? k_radix_pass<false, 1, 4> : k_radix_pass<false, 1, 0>)
                                 : (rk == 2 ? k_radix_pass<false, 0, 2> : rk == 1 ? k_radix_pass<false, 0, 1> : rk == 3 ? k_radix_pass<false, 0, 3> : rk == 4 ? k_radix_pass<false, 0, 4> : k_radix_pass<false, 0, 0>);
        qg_pre_launch(ctx);
        kern<<<(unsigned)tiles, RS_THREADS, smem, ctx->stream>>>(s, d, n, shift, (kv3 || !(side || pf.learned)) ? pf.kmin : 0u,
                                                                 pf.learned && !side ? pf.model : nullptr,
                                                                 dbase + p * QG_RADIX, status, ctx->ctl, ctx->spin_limit,
                                                                 nullptr, nullptr);
        QG_TRY(qg_check_launch(ctx, "k_radix_pass"));
        in_a = !in_a;
    }
    *result_in_b = !in_a;
    return QG_OK;
}

// Exclusive digit bases of every position from a device histogram [npos][256];
// trivial[p] = 1 when one digit value holds every item of position p (that
// pass is then a copy).
__global__ void k_radix_bases(const uint32_t *__restrict__ hist, int npos, uint32_t *__restrict__ bases,
                              uint32_t *__restrict__ trivial) {
    __shared__ uint32_t ws[QG_RADIX / 32], wm[QG_RADIX / 32];
    const int d = threadIdx.x, lane = d & 31, w = d >> 5;
    for (int p = 0; p < npos; p++) {
        const uint32_t c = hist[p * QG_RADIX + d];
        uint32_t inc = c;
#pragma unroll
        for (int k = 1; k < 32; k <<= 1) {
            const uint32_t x = __shfl_up_sync(QG_FULL_MASK, inc, k);
            if (lane >= k) inc += x;
        }
        const uint32_t mx = __reduce_max_sync(QG_FULL_MASK, c);
        if (lane == 31) ws[w] = inc;
        if (lane == 0) wm[w] = mx;
        __syncthreads();
        uint32_t off = 0;
        for (int i = 0; i < w; i++) off += ws[i];
        bases[p * QG_RADIX + d] = off + inc - c;
        if (d == 0) {
            uint32_t tot = 0, big = 0;
            for (int i = 0; i < QG_RADIX / 32; i++) {
                tot += ws[i];
                big = max(big, wm[i]);
            }
            trivial[p] = big == tot ? 1u : 0u;
        }
        __syncthreads();
    }
}

qg_status qg_radix_passes_dev(qg_ctx *ctx, bool kv3, qg_sort_bufs a, qg_sort_bufs b, long long n_bound,
                              const unsigned long long *d_n, const uint32_t *d_hist, int npos, uint32_t key_off,
                              char *work, bool *result_in_b) {
    *result_in_b = false;
    if (n_bound <= 1 || npos <= 0) return QG_OK;
    if (npos > 4) return QG_ERR_INVALID;  // the work area holds four status regions
    if (n_bound >= (1LL << 30)) return QG_ERR_UNSUPPORTED;
    const long long tiles = (n_bound + RS_TILE - 1) / RS_TILE;
    uint32_t *dbase = (uint32_t *)work;
    uint32_t *trivial = dbase + 4 * QG_RADIX;  // [4], in a 256-byte slot
    uint32_t *status = trivial + 64;           // [npos][tiles][256]: one region per pass, cleared at once
    const size_t st_words = (size_t)tiles * QG_RADIX;
    const size_t smem = kv3 ? sizeof(RsSmem<true>) : sizeof(RsSmem<false>);
    if (kv3) QG_TRY((rs_set_attr<true, 0>(ctx)));
    else QG_TRY((rs_set_attr<false, 0>(ctx)));
    qg_pre_launch(ctx);
    k_radix_bases<<<1, QG_RADIX, 0, ctx->stream>>>(d_hist, npos, dbase, trivial);
    QG_TRY(qg_check_launch(ctx, "k_radix_bases"));
    QG_TRY_CUDA(ctx, cudaMemsetAsync(status, 0, (size_t)npos * st_words * 4, ctx->stream), "memset status");
    bool in_a = true;
    for (int p = 0; p < npos; p++) {
        const qg_sort_bufs &s = in_a ? a : b;
        const qg_sort_bufs &d = in_a ? b : a;
        uint32_t *stp = status + (size_t)p * st_words;
        qg_pre_launch(ctx);
        if (kv3)
            k_radix_pass<true, 0><<<(unsigned)tiles, RS_THREADS, smem, ctx->stream>>>(
                s, d, n_bound, 8 * p, key_off, nullptr, dbase + p * QG_RADIX, stp, ctx->ctl, ctx->spin_limit, d_n,
                trivial + p);
        else
            k_radix_pass<false, 0><<<(unsigned)tiles, RS_THREADS, smem, ctx->stream>>>(
                s, d, n_bound, 8 * p, key_off, nullptr, dbase + p * QG_RADIX, stp, ctx->ctl, ctx->spin_limit, d_n,
                trivial + p);
        QG_TRY(qg_check_launch(ctx, "k_radix_pass"));
        in_a = !in_a;
    }
    *result_in_b = !in_a;
    return QG_OK;
}

size_t qg_radix_dev_work_bytes(long long n_bound) {
    return 4 * QG_RADIX * 4 + 256 + 4 * (size_t)((n_bound + RS_TILE - 1) / RS_TILE) * QG_RADIX * 4;
}

qg_status qg_radix_passes(qg_ctx *ctx, bool kv3, qg_sort_bufs a, qg_sort_bufs b, long long n,
                          uint32_t key_off, const int *passes, int np, const uint32_t *h_bases,
                          bool *result_in_b) {
    qg_part_fn pf{0, key_off, 0, nullptr};
    return qg_radix_passes_pf(ctx, kv3, a, b, n, pf, passes, np, h_bases, result_in_b, false);
}

// Sort REC items in `data` (n u64) using `tmp` (n u64) as the ping-pong
// buffer; the result ends in `data`.  Synchronises once to plan the passes.
qg_status qg_sort_rec_inplace(qg_ctx *ctx, unsigned long long *data, unsigned long long *tmp,
                              long long n) {
    if (n <= 1) return QG_OK;
    char *scr;
    QG_TRY(qg_scratch(ctx, 4 * QG_RADIX * 4, &scr));
    uint32_t *d_hist = (uint32_t *)scr;
    qg_sort_bufs a{};
    a.rec = data;
    // An odd number of passes ends in tmp.  When the context's last sort
    // needed an odd number, the histogram kernel (bound by its shared-memory
    // atomics, not by DRAM) also copies the records to tmp, and the passes
    // start there and end in data; otherwise a copy back follows.
    const bool pre_copy = ctx->sort_odd_passes;
    QG_TRY(qg_radix_histogram(ctx, a, false, n, 0u, 4, d_hist, pre_copy ? tmp : nullptr));
    std::vector<uint32_t> h(4 * QG_RADIX), bases(4 * QG_RADIX);
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(h.data(), d_hist, 4 * QG_RADIX * 4, cudaMemcpyDeviceToHost, ctx->stream), "hist d2h");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    int passes[4];
    int np = qg_sort_plan(h.data(), 4, n, passes, bases.data());
    ctx->sort_odd_passes = (np & 1) != 0;
    qg_sort_bufs b{};
    b.rec = tmp;
    if ((np & 1) && pre_copy) std::swap(a, b);  // from the copy in tmp into data
    bool in_b = false;
    QG_TRY(qg_radix_passes(ctx, false, a, b, n, 0u, passes, np, bases.data(), &in_b));
    if ((in_b ? b.rec : a.rec) != data)
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(data, tmp, (size_t)n * 8, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
    return QG_OK;
}

extern "C" QG_API qg_status qg_sort_rec_by_y(qg_ctx *ctx, void *records, int64_t n) {
    if (!ctx || n < 0 || (n > 0 && !records)) return QG_ERR_INVALID;
    if (((uintptr_t)records) & 7) return QG_ERR_INVALID;
    if (n <= 1) return QG_OK;
    if (n >= (1LL << 30)) return QG_ERR_UNSUPPORTED;
    char *tmp = nullptr;
    QG_TRY(qg_aux(ctx, (size_t)n * 8, &tmp));
    QG_TRY(qg_sort_rec_inplace(ctx, (unsigned long long *)records, (unsigned long long *)tmp, n));
    return qg_ctx_check(ctx);
}
