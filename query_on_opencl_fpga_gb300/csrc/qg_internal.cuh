// qg_internal.cuh -- context, scratch arena and device helpers shared by all
// operator translation units of libqg.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include "qg.h"

// ---------------------------------------------------------------------------
// Device-resident control block (one per context).
// ---------------------------------------------------------------------------
struct qg_control {
    int32_t err;        // first error code recorded by any kernel (0 = none)
    int32_t err_site;   // which kernel recorded it
    uint32_t epoch;     // look-back epoch; status words of older launches are stale
    uint32_t tile_ctr;  // dynamic tile counter of the running single-pass kernel
    uint32_t done_ctr;  // finished CTAs of the running single-pass kernel
    uint32_t pad0;
    unsigned long long counter[6];  // scratch counters (output cursors)
    uint32_t gbd[48];               // per-call state of the dense-window group-by (qg_gbdense.cu)
    uint32_t ghist[4 * 256];        // digit counts of emitted group keys (group-by in key order)
    // Arrivals of the two-pass column filter's tiles per group of 256 tiles
    // (inputs below 2^31 rows make at most 2048 groups).  The last tile of a
    // group wraps its counter back to zero, so no launch has to clear them.
    uint32_t fgroup[2048];
};

#define QG_MAX_TIMED 4096
struct qg_ctx {
    cudaStream_t stream;
    int device;
    int sm_count;
    char *scratch;          // grow-only arena for per-call temporaries
    size_t scratch_bytes;
    char *table;            // grow-only hash-table arena; kept all-zero between calls
    size_t table_bytes;
    char *aux;              // grow-only arena for operator temporaries that must
    size_t aux_bytes;       //   survive nested calls (e.g. a sort inside group-by)
    unsigned long long *lbstat;  // look-back status words, used by nothing else
    size_t lbstat_words;
    qg_control *ctl;        // device
    long long *pinned;      // host pinned readback slots (8)
    qg_control *pin_ctl;    // host pinned copy of the control block (one read brings error, counters, ghist)
    uint32_t *pin_bases;    // ring of 8 host pinned 4 KB slots for radix digit bases
    cudaEvent_t pin_ev[8];  // a slot may be refilled once its copy (event) has completed
    int pin_next;
    uint32_t spin_limit;
    uint64_t launches;
    bool table_dirty;       // group-by table must be cleared before next use
    uint32_t gb_stats[4];   // last qg_groupby_cols: path, flags, fullest bucket, bucket cap
    bool gb_wide_keys;      // last key-ordered group-by's keys spanned too wide a range for the dense order
    uint32_t gb_kbase;      // first key of the next dense-order window (from the last call's keys)
    bool sort_odd_passes;   // the last in-place record sort took an odd number of passes
    uint32_t pj_stats[8];   // last qg_join_filter_sort (see qg_join_stats)
    char *pj_tmp;           // the join's sort-merge arrays (grow-only)
    size_t pj_tmp_bytes;
    void *pin_join;         // host pinned bucket bounds and group plan of the join (allocated on first use)
    char msg[256];
    // Learned variant choice (qg_steer.cu): the model's decision table and
    // judge state when one is attached, and the variant a steered call runs
    // (per operator QG_STEER_*, -1 = the process-wide knob).
    struct qg_steer_state *steer;
    int steer_force[4];
    // Per-kernel CUDA-event timing (qg_ctx_enable_timing): a pair of events
    // brackets every launch on the context's stream.
    bool timing;
    int ev_used;
    cudaEvent_t ev[2 * QG_MAX_TIMED];
    const char *ev_name[QG_MAX_TIMED];
};

// Record the start event of the next launch (no-op unless timing is on).
void qg_pre_launch(qg_ctx *ctx);

// Site tags for the error word.
enum {
    QG_SITE_FILTER = 1, QG_SITE_SCAN = 2, QG_SITE_SORT = 3, QG_SITE_GROUPBY = 4,
    QG_SITE_AGG = 5, QG_SITE_JOIN_BUILD = 6, QG_SITE_JOIN_PROBE = 7, QG_SITE_SORT_LOOKBACK = 8,
    QG_SITE_PJ_HIST = 9, QG_SITE_PJ_FILTER = 10, QG_SITE_PJ_BUCKET = 11
};

qg_status qg_cuda_fail(qg_ctx *ctx, cudaError_t e, const char *what);
// Dense-window column group-by (qg_gbdense.cu): launches the whole path on the
// context's stream, output in ascending unsigned key order; the caller reads
// ctl->gbd[QG_GBD_OUTSIDE] (non-zero: the path did not apply, nothing valid
// was written) and the group count (*d_num) after its one synchronisation.
qg_status qg_gbd_launch(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2,
                        int32_t lo2, int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum, int64_t *gcnt,
                        int64_t cap, long long *d_num);
enum { QG_GBD_OUTSIDE = 6 };
qg_status qg_groupby_dense_async(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2,
                                 int32_t lo2, int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum, int64_t *gcnt,
                                 int64_t cap, int64_t *d_num);
qg_status qg_groupby_dense_probe(qg_ctx *ctx, const int32_t *key, const int32_t *val, const int32_t *val2,
                                 int32_t lo2, int32_t hi2, int64_t n, int32_t *gkey, int64_t *gsum, int64_t *gcnt,
                                 int64_t cap, int64_t *d_num, bool *ok);

// Operators the learned variant choice covers (the batch's OP_* order).
enum { QG_STEER_FILTER = 0, QG_STEER_GROUPBY = 1, QG_STEER_FUSED = 2, QG_STEER_JOIN = 3, QG_STEER_OPS = 4 };
// The process-wide (plain) variant of each operator: the default the learned
// choice is judged against.
int qg_filter_default_variant();
int qg_groupby_default_mode();
int qg_join_default_variant();
// The variant a call of `op` on ctx runs: the steered one, else the knob.
static inline int qg_effective_variant(const qg_ctx *ctx, int op, int knob) {
    const int f = ctx->steer_force[op];
    return f >= 0 ? f : knob;
}
// A steered synchronous call (qg_steer.cu): _begin picks the variant and
// starts the call's device timer, _end reads it (the call has synchronised)
// and updates the judge.  No-ops without an attached model.
struct qg_steer_call {
    int op, cell, variant;
    bool active;
};
void qg_steer_begin(qg_ctx *ctx, int op, int64_t n, int64_t n2, double sel, qg_steer_call *c);
void qg_steer_end(qg_ctx *ctx, qg_steer_call *c, qg_status st);
void qg_steer_free(qg_ctx *ctx);
// Ensure the scratch arena holds at least `bytes`; newly grown memory is zeroed.
qg_status qg_scratch(qg_ctx *ctx, size_t bytes, char **out);
// Ensure the operator-temporary arena holds at least `bytes` (not zeroed).
qg_status qg_aux(qg_ctx *ctx, size_t bytes, char **out);
// Ensure the hash-table arena holds at least `bytes` of zeroed memory.
qg_status qg_table(qg_ctx *ctx, size_t bytes, char **out);
// Look-back descriptor for a single-pass kernel of `tiles` tiles.  Its status
// words live in an arena of their own: a word there is either zero or was
// written by an earlier look-back launch (an older epoch), never by other
// data that could mimic a current-epoch word.
struct qg_lookback;
qg_status qg_lb_make(qg_ctx *ctx, int64_t tiles, int site, qg_lookback *out);
// Upload 4 KB of digit bases to d_dst in stream order without synchronising
// (through the pinned ring).
qg_status qg_stage_bases(qg_ctx *ctx, const uint32_t *h_bases, uint32_t *d_dst);
// Copy a device int64 to host (synchronises the stream).
qg_status qg_read_i64(qg_ctx *ctx, const long long *d, long long *h);
qg_status qg_check_launch(qg_ctx *ctx, const char *what);
// Read the device error word (after the stream's work), clear it and map it.
qg_status qg_collect_error(qg_ctx *ctx);
// qg_read_i64 and qg_collect_error with one synchronisation: the count in *h,
// the device error (if any) as the status.
qg_status qg_read_count(qg_ctx *ctx, const long long *d, long long *h);

#define QG_TRY_CUDA(ctx, expr, what)                            \
    do {                                                        \
        cudaError_t _e = (expr);                                \
        if (_e != cudaSuccess) return qg_cuda_fail(ctx, _e, what); \
    } while (0)
#define QG_TRY(expr)                        \
    do {                                    \
        qg_status _s = (expr);              \
        if (_s != QG_OK) return _s;         \
    } while (0)

static inline size_t qg_align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
static inline int64_t qg_ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------
#define QG_FULL_MASK 0xffffffffu

__device__ __forceinline__ void qg_record_error(qg_control *ctl, int code, int site) {
    if (atomicCAS(&ctl->err, 0, code) == 0) ctl->err_site = site;
}

__device__ __forceinline__ unsigned long long qg_ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void qg_st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t qg_ld_relaxed_u32(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void qg_st_relaxed_u32(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t qg_lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Streaming 128-bit load (read once, do not keep in L1).
__device__ __forceinline__ int4 qg_ldg_stream(const int4 *p) {
    int4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.s32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

// 32-bit integer mix (murmur3 finaliser constants from the public MurmurHash3).
__device__ __forceinline__ uint32_t qg_hash32(uint32_t k) {
    k ^= k >> 16;
    k *= 0x85ebca6bu;
    k ^= k >> 13;
    k *= 0xc2b2ae35u;
    k ^= k >> 16;
    return k;
}

// ---------------------------------------------------------------------------
// Decoupled look-back (single-pass prefix over tiles).
//
// Status word per tile (64 bit): [63:34] epoch, [33:32] flag, [31:0] value.
// flag 1 = tile aggregate published, flag 2 = inclusive prefix published.
// A word whose epoch differs from the running launch's epoch is "not yet
// written".  Tile i is CTA i: the hardware starts CTAs in index order, so
// every predecessor of a running tile has started and will publish (and a
// wait that exceeds the poll limit reports QG_ERR_TIMEOUT instead of hanging).
// The last CTA to finish advances the epoch, so no memset is needed between
// launches, also when a launch is replayed from a CUDA graph.
// ---------------------------------------------------------------------------
struct qg_lookback {
    unsigned long long *status;
    qg_control *ctl;
    uint32_t spin_limit;
    int site;
};

#define QG_LB_AGG 1ull
#define QG_LB_PREFIX 2ull

__device__ __forceinline__ unsigned long long qg_lb_word(uint32_t epoch, unsigned long long flag,
                                                          uint32_t value) {
    return ((unsigned long long)epoch << 34) | (flag << 32) | (unsigned long long)value;
}

// Called by all threads of the CTA at kernel start; returns the tile id and
// the running epoch through shared memory.
__device__ __forceinline__ void qg_lb_begin(const qg_lookback &lb, uint32_t *s_tile,
                                            uint32_t *s_epoch) {
    if (threadIdx.x == 0) {
        *s_tile = blockIdx.x;
        *s_epoch = *(volatile uint32_t *)&lb.ctl->epoch;
    }
    __syncthreads();
}

// Tile id from the control block's tile counter instead of blockIdx.x:
// tiles are numbered in the order the CTAs start, so every predecessor of a
// waiting tile is running (or done) whatever order the hardware schedules
// CTAs in.  Called by all threads at kernel start, before the tile's loads.
// Pair with qg_lb_finish_dyn.
__device__ __forceinline__ void qg_lb_begin_dyn(const qg_lookback &lb, uint32_t *s_tile,
                                                uint32_t *s_epoch) {
    if (threadIdx.x == 0) {
        *s_tile = atomicAdd(&lb.ctl->tile_ctr, 1u);
        *s_epoch = *(volatile uint32_t *)&lb.ctl->epoch;
    }
    __syncthreads();
}

// Called by all threads of warp 0 only.  Publishes the tile aggregate, looks
// back over predecessors and returns the exclusive prefix of this tile (mod 2^32).
__device__ __forceinline__ uint32_t qg_lb_warp_exclusive(const qg_lookback &lb, uint32_t tile,
                                                          uint32_t epoch, uint32_t aggregate) {
    const int lane = threadIdx.x & 31;
    if (tile == 0) {
        if (lane == 0) qg_st_relaxed_u64(&lb.status[0], qg_lb_word(epoch, QG_LB_PREFIX, aggregate));
        return 0;
    }
    if (lane == 0) qg_st_relaxed_u64(&lb.status[tile], qg_lb_word(epoch, QG_LB_AGG, aggregate));
    uint32_t excl = 0;
    long long pred = (long long)tile - 1;
    while (true) {
        long long j = pred - lane;
        unsigned long long flag = QG_LB_PREFIX;
        uint32_t value = 0;
        if (j >= 0) {
            uint32_t spins = 0;
            unsigned long long w;
            // spin_limit is the number of polls allowed: 0 gives up at once.
            while (true) {
                if (spins >= lb.spin_limit) {
                    qg_record_error(lb.ctl, QG_ERR_TIMEOUT, lb.site);
                    w = qg_lb_word(epoch, QG_LB_PREFIX, 0);
                    break;
                }
                w = qg_ld_relaxed_u64(&lb.status[j]);
                if ((uint32_t)(w >> 34) == (epoch & 0x3fffffffu) && ((w >> 32) & 3ull) != 0) break;
                spins++;
                __nanosleep(32);
            }
            flag = (w >> 32) & 3ull;
            value = (uint32_t)w;
        }
        uint32_t pmask = __ballot_sync(QG_FULL_MASK, flag == QG_LB_PREFIX);
        int stop = pmask ? (__ffs(pmask) - 1) : 31;
        uint32_t contrib = (lane <= stop) ? value : 0u;
        excl += __reduce_add_sync(QG_FULL_MASK, contrib);
        if (pmask) break;
        pred -= 32;
    }
    if (lane == 0)
        qg_st_relaxed_u64(&lb.status[tile], qg_lb_word(epoch, QG_LB_PREFIX, excl + aggregate));
    return excl;
}

// qg_lb_warp_exclusive split in two, so that a tile can publish its aggregate
// as soon as it is known and look back later (successors then wait less):
// qg_lb_publish_agg by one thread, then qg_lb_warp_lookback by warp 0.
__device__ __forceinline__ void qg_lb_publish_agg(const qg_lookback &lb, uint32_t tile, uint32_t epoch,
                                                  uint32_t aggregate) {
    qg_st_relaxed_u64(&lb.status[tile], qg_lb_word(epoch, tile == 0 ? QG_LB_PREFIX : QG_LB_AGG, aggregate));
}
__device__ __forceinline__ uint32_t qg_lb_warp_lookback(const qg_lookback &lb, uint32_t tile, uint32_t epoch,
                                                        uint32_t aggregate) {
    const int lane = threadIdx.x & 31;
    if (tile == 0) return 0;
    uint32_t excl = 0;
    long long pred = (long long)tile - 1;
    while (true) {
        long long j = pred - lane;
        unsigned long long flag = QG_LB_PREFIX;
        uint32_t value = 0;
        if (j >= 0) {
            uint32_t spins = 0;
            unsigned long long w;
            while (true) {
                if (spins >= lb.spin_limit) {
                    qg_record_error(lb.ctl, QG_ERR_TIMEOUT, lb.site);
                    w = qg_lb_word(epoch, QG_LB_PREFIX, 0);
                    break;
                }
                w = qg_ld_relaxed_u64(&lb.status[j]);
                if ((uint32_t)(w >> 34) == (epoch & 0x3fffffffu) && ((w >> 32) & 3ull) != 0) break;
                spins++;
                __nanosleep(32);
            }
            flag = (w >> 32) & 3ull;
            value = (uint32_t)w;
        }
        uint32_t pmask = __ballot_sync(QG_FULL_MASK, flag == QG_LB_PREFIX);
        int stop = pmask ? (__ffs(pmask) - 1) : 31;
        uint32_t contrib = (lane <= stop) ? value : 0u;
        excl += __reduce_add_sync(QG_FULL_MASK, contrib);
        if (pmask) break;
        pred -= 32;
    }
    if (lane == 0)
        qg_st_relaxed_u64(&lb.status[tile], qg_lb_word(epoch, QG_LB_PREFIX, excl + aggregate));
    return excl;
}

// Wide look-back: called by the NW*32 threads of warps 0..NW-1, which read
// NW*32 predecessors per round (one each), synchronising on named barrier 1.
// The inclusive-prefix frontier then advances NW*32 tiles per L2 round trip
// instead of 32, which is what bounds a single-pass scan's throughput.
// s_tmp needs 2*NW words.  Returns the tile's exclusive prefix to every caller.
template <int NW>
__device__ __forceinline__ uint32_t qg_lb_wide_exclusive(const qg_lookback &lb, uint32_t tile,
                                                         uint32_t epoch, uint32_t aggregate,
                                                         uint32_t *s_tmp) {
    constexpr int NT = NW * 32;
    const int t0 = threadIdx.x, lane = t0 & 31, warp = t0 >> 5;
    if (tile == 0) {
        if (t0 == 0) qg_st_relaxed_u64(&lb.status[0], qg_lb_word(epoch, QG_LB_PREFIX, aggregate));
        return 0;
    }
    if (t0 == 0) qg_st_relaxed_u64(&lb.status[tile], qg_lb_word(epoch, QG_LB_AGG, aggregate));
    uint32_t excl = 0;
    long long pred = (long long)tile - 1;
    while (true) {
        const long long j = pred - t0;
        unsigned long long flag = QG_LB_PREFIX;
        uint32_t value = 0;
        if (j >= 0) {
            uint32_t spins = 0;
            unsigned long long w;
            // spin_limit is the number of polls allowed: 0 gives up at once.
            while (true) {
                if (spins >= lb.spin_limit) {
                    qg_record_error(lb.ctl, QG_ERR_TIMEOUT, lb.site);
                    w = qg_lb_word(epoch, QG_LB_PREFIX, 0);
                    break;
                }
                w = qg_ld_relaxed_u64(&lb.status[j]);
                if ((uint32_t)(w >> 34) == (epoch & 0x3fffffffu) && ((w >> 32) & 3ull) != 0) break;
                spins++;
                __nanosleep(20);
            }
            flag = (w >> 32) & 3ull;
            value = (uint32_t)w;
        }
        const uint32_t pmask = __ballot_sync(QG_FULL_MASK, flag == QG_LB_PREFIX);
        if (lane == 0) s_tmp[warp] = pmask ? (uint32_t)(warp * 32 + __ffs(pmask) - 1) : 0xffffffffu;
        asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
        uint32_t stop = 0xffffffffu;
#pragma unroll
        for (int w = 0; w < NW; w++) stop = min(stop, s_tmp[w]);
        const uint32_t contrib = ((uint32_t)t0 <= stop) ? value : 0u;
        const uint32_t ws = __reduce_add_sync(QG_FULL_MASK, contrib);
        if (lane == 0) s_tmp[NW + warp] = ws;
        asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
#pragma unroll
        for (int w = 0; w < NW; w++) excl += s_tmp[NW + w];
        asm volatile("bar.sync 1, %0;" ::"r"(NT) : "memory");
        if (stop != 0xffffffffu) break;
        pred -= NT;
    }
    if (t0 == 0)
        qg_st_relaxed_u64(&lb.status[tile], qg_lb_word(epoch, QG_LB_PREFIX, excl + aggregate));
    return excl;
}

// Called by ALL threads of a single-pass compaction tile after the E per-warp
// counts (in row order) are in s_woff: turns them into exclusive offsets,
// runs the wide look-back on warps 0..NW-1 and leaves the tile's output
// offset in *s_excl; the last tile stores the grand total in *d_count.
// s_tmp needs 2*NW+1 words.
template <int E, int NW>
__device__ __forceinline__ void qg_tile_offsets_wide(uint32_t *s_woff, const qg_lookback &lb,
                                                     uint32_t tile, uint32_t epoch,
                                                     uint32_t *s_excl, uint32_t *s_tmp,
                                                     long long *d_count, uint32_t last_tile) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (warp == 0) {
        constexpr int PER = (E + 31) / 32;
        uint32_t loc[PER];
        uint32_t sum = 0;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            const int e = lane * PER + k;
            loc[k] = (e < E) ? s_woff[e] : 0u;
            sum += loc[k];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(QG_FULL_MASK, incl, d);
            if (lane >= d) incl += t;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int k = 0; k < PER; k++) {
            const int e = lane * PER + k;
            if (e < E) s_woff[e] = run;
            run += loc[k];
        }
        if (lane == 31) s_tmp[2 * NW] = incl;
    }
    __syncthreads();
    if (warp < NW) {
        const uint32_t total = s_tmp[2 * NW];
        const uint32_t excl = qg_lb_wide_exclusive<NW>(lb, tile, epoch, total, s_tmp);
        if (threadIdx.x == 0) {
            *s_excl = excl;
            if (tile == last_tile && d_count) *d_count = (long long)excl + total;
        }
    }
    __syncthreads();
}

// End of a one-tile-per-CTA look-back kernel: the CTA of the last tile
// advances the epoch.  When that CTA gets here every other tile has published
// (its look-back waited for its predecessors, and theirs for theirs), so
// every CTA of the launch has read the epoch already; no fence or counter.
__device__ __forceinline__ void qg_lb_finish(const qg_lookback &lb, uint32_t tile,
                                             uint32_t last_tile, uint32_t epoch) {
    if (threadIdx.x == 0 && tile == last_tile) *(volatile uint32_t *)&lb.ctl->epoch = epoch + 1u;
}

// qg_lb_finish for tiles numbered by qg_lb_begin_dyn: the last tile also
// resets the tile counter (every CTA has taken its tile by then).
__device__ __forceinline__ void qg_lb_finish_dyn(const qg_lookback &lb, uint32_t tile,
                                                 uint32_t last_tile, uint32_t epoch) {
    if (threadIdx.x == 0 && tile == last_tile) {
        lb.ctl->tile_ctr = 0;
        *(volatile uint32_t *)&lb.ctl->epoch = epoch + 1u;
    }
}

// End of a persistent look-back kernel whose CTAs take tiles from
// ctl->tile_ctr: the last CTA to finish resets the counters and advances
// the epoch.
__device__ __forceinline__ void qg_lb_end(const qg_lookback &lb) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        uint32_t done = atomicAdd(&lb.ctl->done_ctr, 1u);
        if (done == gridDim.x - 1) {
            lb.ctl->tile_ctr = 0;
            lb.ctl->done_ctr = 0;
            lb.ctl->epoch = (lb.ctl->epoch + 1) & 0x3fffffffu;
            __threadfence();
        }
    }
}

// Warp 0 of a single-pass compaction tile: exclusive scan of the E per-warp
// counts in s_woff (in row order), look-back for the tile's output offset,
// publish the total count from the last tile.  Leaves exclusive offsets in
// s_woff and the tile offset in *s_excl.
template <int E>
__device__ __forceinline__ void qg_tile_compact_offsets(uint32_t *s_woff, const qg_lookback &lb,
                                                        uint32_t tile, uint32_t epoch,
                                                        uint32_t *s_excl, long long *d_count,
                                                        uint32_t last_tile = 0xffffffffu) {
    if (last_tile == 0xffffffffu) last_tile = gridDim.x - 1;
    const int lane = threadIdx.x & 31;
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
    uint32_t excl = qg_lb_warp_exclusive(lb, tile, epoch, total);
    if (lane == 0) {
        *s_excl = excl;
        if (tile == last_tile && d_count) *d_count = (long long)excl + total;
    }
}

// ---- mbarrier / bulk-copy (TMA engine) helpers (PTX ISA: mbarrier, cp.async.bulk)
__device__ __forceinline__ uint32_t qg_smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void qg_mbar_init(unsigned long long *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(qg_smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void qg_mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void qg_mbar_arrive_expect_tx(unsigned long long *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(qg_smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void qg_mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(qg_smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool qg_mbar_try_wait(unsigned long long *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(qg_smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// 1-D bulk copy global -> shared; completes `bytes` of transaction count on
// `bar`.  Source and destination 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void qg_bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                            unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            qg_smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(qg_smem_u32(bar))
        : "memory");
}

// Host side: status words needed for `tiles` tiles.
static inline size_t qg_lb_bytes(int64_t tiles) { return (size_t)tiles * 8; }
