// qg_bpersist.cu -- the persistent executor of a batch: every filter, group-by
// and fused filter + group-by query of a batch runs inside ONE kernel launch.
//
// The reference runs one operator per call, each kernel followed by clFinish
// (host/host/common.cpp:28-31).  Here the batch's work is cut, on the host,
// into items -- (query, kind, tile) -- in one queue, and a grid of persistent
// CTAs pops them in order from a device counter:
//   filter tile (4096 rows)  predicate, ballot ranking, and the tile's place
//                            in the query's output from a decoupled look-back
//                            over the query's earlier tiles: stable output, as
//                            filterImpl (kernel/filter/filter_op.cl:6-238);
//   group tile (2^g rows)    rows (the fused form: those with lo <= value2 <=
//                            hi) pre-aggregated in a shared-memory hash table
//                            (rows it has no room for set aside), then added
//                            to the query's open-addressing table in global
//                            memory (count and int64 sum), several updates in
//                            flight per thread; a key new to that table
//                            appends its slot to the query's list of groups;
//   emit tile (4096 groups)  after every group tile of its query is done (a
//                            bounded wait), writes list entries [4096e,
//                            4096(e+1)) as output groups (key, SUM int64,
//                            COUNT int64, unordered as QG_ORDER_NONE) and
//                            clears their slots; the query's last emit tile
//                            publishes the group count.
// A waiting item only ever waits for items popped before it, which running
// CTAs hold, so every wait ends; each is also bounded by the batch context's
// poll limit and reports QG_ERR_TIMEOUT when it gives up.  The last CTA to
// finish resets the queue and advances the look-back epoch, so the launch can
// be replayed from a CUDA graph.  Tables and lists are left cleared.
#include <algorithm>
#include <vector>

#include "qg_internal.cuh"

namespace {

constexpr int BP_THREADS = 256;
constexpr int BP_WARPS = BP_THREADS / 32;
constexpr int BP_FTILE = 4096;                             // filter rows per item
constexpr int BP_FROUNDS = BP_FTILE / (BP_THREADS * 4);    // int4 rounds per thread
constexpr int BP_ETILE = 4096;                             // list entries per emit item
constexpr int BP_SSLOTS = 2048;                            // shared pre-aggregation slots
constexpr int BP_SPROBE = 16;                              // shared probes before a row is set aside
constexpr int BP_OVF = 2048;                               // rows set aside per group tile (then L2)
constexpr int BP_FLUSH = 4;                                // L2 updates a thread has in flight
constexpr uint32_t BP_EMPTY = 0xffffffffu;
enum { BK_FILTER = 0u, BK_GROUP = 1u, BK_EMIT = 2u };

struct BQ {
    const int32_t *k, *v, *w;      // filter: key, payload; group-by: key, value, value2 (fused) or null
    void *o0, *o1, *o2;            // filter: pairs; group-by: key, sum, count
    long long n, cap;
    int32_t lo, hi;
    long long *d_count;
    unsigned long long *status;    // filter: look-back words, one per tile
    uint32_t ntiles;               // filter or group tiles
    uint32_t etiles;               // emit items (group-by)
    unsigned long long *tab;       // group-by: per slot (count << 32 | key, sum); 0 = empty
    uint32_t mask;                 // slots - 1
    uint32_t *list;                // group-by: the slot of every group, in insertion order
    uint32_t *cnt;                 // group-by: [0] groups listed, [1] group tiles done, [2] emits done
};

struct BItem {
    uint32_t q;
    uint32_t kt;  // kind << 30 | tile
};

struct BCtl {
    qg_control ctl;  // error word and look-back epoch
    uint32_t head;   // next item
    uint32_t done;   // finished CTAs
};

__device__ __forceinline__ uint32_t bp_hash(uint32_t k) { return qg_hash32(k ^ 0x5bd1e995u); }

__device__ __forceinline__ void bp_red_shared(uint32_t *p, uint32_t v) {
    asm volatile("red.shared.add.u32 [%0], %1;" ::"r"(qg_smem_u32(p)), "r"(v) : "memory");
}
// A tile's int64 sum per key without carries: the low 16 bits of each value
// (unsigned) and its high 16 bits (signed) are summed apart; over at most
// 2^16 rows both stay within 32 bits, and sum = hi * 65536 + lo exactly.
__device__ __forceinline__ void bp_add_split(uint32_t *lo, uint32_t *hi, int32_t v) {
    bp_red_shared(lo, (uint32_t)v & 0xffffu);
    bp_red_shared(hi, (uint32_t)(v >> 16));
}
__device__ __forceinline__ long long bp_split_sum(uint32_t lo, uint32_t hi) {
    return (long long)(int32_t)hi * 65536 + (long long)lo;
}

// Adds (c rows, sum s) of key k to the query's L2 table; returns the slot and
// whether the key was new there (or -1 when the table is full).
__device__ __forceinline__ long long bp_l2_add(const BQ &Q, uint32_t k, uint32_t c, long long s, bool *fresh,
                                               qg_control *ctl) {
    uint32_t h = bp_hash(k) & Q.mask;
    const unsigned long long init = ((unsigned long long)c << 32) | k;
    for (uint32_t p = 0; p <= Q.mask; p++, h = (h + 1) & Q.mask) {
        const unsigned long long old = atomicCAS(Q.tab + 2 * h, 0ull, init);
        if (old == 0ull || (uint32_t)old == k) {
            if (old != 0ull) atomicAdd(Q.tab + 2 * h, (unsigned long long)c << 32);
            atomicAdd(Q.tab + 2 * h + 1, (unsigned long long)s);
            *fresh = old == 0ull;
            return h;
        }
    }
    qg_record_error(ctl, QG_ERR_TABLE_FULL, QG_SITE_GROUPBY);
    *fresh = false;
    return -1;
}

struct BShared {
    uint32_t tk[BP_SSLOTS], tc[BP_SSLOTS], tl[BP_SSLOTS], th[BP_SSLOTS];
    uint32_t ok[BP_OVF];  // rows set aside: key and value
    int32_t ov[BP_OVF];
    uint32_t woff[BP_FROUNDS * BP_WARPS];
    uint32_t item, epoch, excl, nov;
};

// L2 updates of (key, rows, sum) entries with BP_FLUSH first attempts in
// flight per thread before any result is used; an entry whose first slot holds
// another key probes on alone.  Keys new to the table are listed (one list
// reservation per warp and round).  Called by all threads; entry e of the
// thread's round r is get(r * BP_FLUSH + e), or absent when it returns false.
template <typename Get>
__device__ __forceinline__ void bp_l2_flush(const BQ &Q, int rounds, Get get, qg_control *ctl) {
    const int lane = threadIdx.x & 31;
    for (int r = 0; r < rounds; r++) {
        uint32_t k[BP_FLUSH], c[BP_FLUSH], h[BP_FLUSH];
        long long sm[BP_FLUSH];
        unsigned long long old[BP_FLUSH];
        bool have[BP_FLUSH];
#pragma unroll
        for (int e = 0; e < BP_FLUSH; e++) {
            have[e] = get(r * BP_FLUSH + e, &k[e], &c[e], &sm[e]);
            h[e] = bp_hash(k[e]) & Q.mask;
            old[e] = have[e] ? atomicCAS(Q.tab + 2 * h[e], 0ull, ((unsigned long long)c[e] << 32) | k[e]) : 1ull;
        }
#pragma unroll
        for (int e = 0; e < BP_FLUSH; e++) {
            bool fresh = false;
            long long sl = -1;
            if (have[e]) {
                if (old[e] == 0ull || (uint32_t)old[e] == k[e]) {
                    if (old[e] != 0ull) atomicAdd(Q.tab + 2 * h[e], (unsigned long long)c[e] << 32);
                    atomicAdd(Q.tab + 2 * h[e] + 1, (unsigned long long)sm[e]);
                    fresh = old[e] == 0ull;
                    sl = h[e];
                } else {
                    sl = bp_l2_add(Q, k[e], c[e], sm[e], &fresh, ctl);
                }
            }
            const bool put = fresh && sl >= 0;
            const uint32_t m = __ballot_sync(QG_FULL_MASK, put);
            uint32_t b = 0;
            if (lane == 0 && m) b = atomicAdd(&Q.cnt[0], (uint32_t)__popc(m));
            b = __shfl_sync(QG_FULL_MASK, b, 0);
            if (put) Q.list[b + __popc(m & qg_lanemask_lt())] = (uint32_t)sl;
        }
    }
}

__device__ void bp_filter_tile(BShared &S, const BQ &Q, uint32_t tile, uint32_t epoch, qg_lookback lb) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt = qg_lanemask_lt();
    const long long base = (long long)tile * BP_FTILE;
    int4 kv[BP_FROUNDS], pv[BP_FROUNDS];
#pragma unroll
    for (int r = 0; r < BP_FROUNDS; r++) {  // all loads first
        const long long idx = base + (long long)(r * BP_THREADS + tid) * 4;
        if (idx + 3 < Q.n) {
            kv[r] = qg_ldg_stream(reinterpret_cast<const int4 *>(Q.k + idx));
            pv[r] = qg_ldg_stream(reinterpret_cast<const int4 *>(Q.v + idx));
        } else {
            int t[4] = {0, 0, 0, 0}, p[4] = {0, 0, 0, 0};
            for (int j = 0; j < 4; j++)
                if (idx + j < Q.n) {
                    t[j] = Q.k[idx + j];
                    p[j] = Q.v[idx + j];
                }
            kv[r] = make_int4(t[0], t[1], t[2], t[3]);
            pv[r] = make_int4(p[0], p[1], p[2], p[3]);
        }
    }
    uint32_t fl = 0, lpre[BP_FROUNDS];
#pragma unroll
    for (int r = 0; r < BP_FROUNDS; r++) {
        const long long idx = base + (long long)(r * BP_THREADS + tid) * 4;
        const int32_t ks[4] = {kv[r].x, kv[r].y, kv[r].z, kv[r].w};
        uint32_t f = 0, c = 0, tot = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) f |= (uint32_t)((ks[j] >= Q.lo) & (ks[j] <= Q.hi) & (idx + j < Q.n)) << j;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t b = __ballot_sync(QG_FULL_MASK, (f >> j) & 1u);
            c += __popc(b & lt);
            tot += __popc(b);
        }
        lpre[r] = c;
        if (lane == 0) S.woff[r * BP_WARPS + warp] = tot;
        fl |= f << (4 * r);
    }
    __syncthreads();
    if (warp == 0)  // cell offsets, the look-back, and (last tile) the query's count
        qg_tile_compact_offsets<BP_FROUNDS * BP_WARPS>(S.woff, lb, tile, epoch, &S.excl, Q.d_count, Q.ntiles - 1);
    __syncthreads();
    const long long excl = S.excl;
    int2 *out = reinterpret_cast<int2 *>(Q.o0);
#pragma unroll
    for (int r = 0; r < BP_FROUNDS; r++) {
        long long pos = excl + S.woff[r * BP_WARPS + warp] + lpre[r];
        const long long idx = base + (long long)(r * BP_THREADS + tid) * 4;
        const int32_t ps[4] = {pv[r].x, pv[r].y, pv[r].z, pv[r].w};
#pragma unroll
        for (int j = 0; j < 4; j++)
            if ((fl >> (4 * r + j)) & 1u) {
                if (pos < Q.cap) out[pos] = make_int2((int32_t)(idx + j), ps[j]);
                pos++;
            }
    }
    __syncthreads();  // woff and excl are reused by the next item
}

__device__ void bp_group_tile(BShared &S, const BQ &Q, uint32_t tile, int gtile_log2, qg_control *ctl) {
    const int tid = threadIdx.x, lane = tid & 31;
    for (int i = tid; i < BP_SSLOTS; i += BP_THREADS) {
        S.tk[i] = BP_EMPTY;
        S.tc[i] = 0;
        S.tl[i] = 0;
        S.th[i] = 0;
    }
    if (tid == 0) S.nov = 0;
    __syncthreads();
    const long long base = (long long)tile << gtile_log2;
    const int rounds = (1 << gtile_log2) / (BP_THREADS * 4);
    const bool pred = Q.w != nullptr;
    auto row = [&](uint32_t k, int32_t v) {
        if (k != BP_EMPTY) {
            uint32_t h = bp_hash(k) & (BP_SSLOTS - 1);
            for (int p = 0; p < BP_SPROBE; p++, h = (h + 1) & (BP_SSLOTS - 1)) {
                // a key already in its slot needs no compare-and-swap
                uint32_t cur = *(volatile uint32_t *)&S.tk[h];
                if (cur == BP_EMPTY) cur = atomicCAS(&S.tk[h], BP_EMPTY, k);
                if (cur == BP_EMPTY || cur == k) {
                    bp_red_shared(&S.tc[h], 1u);
                    bp_add_split(&S.tl[h], &S.th[h], v);
                    return;
                }
            }
        }
        // the empty mark's key, or a shared table without room: set aside for
        // the flush (straight to L2 when the buffer is full too)
        const uint32_t o = atomicAdd(&S.nov, 1u);
        if (o < (uint32_t)BP_OVF) {
            S.ok[o] = k;
            S.ov[o] = v;
            return;
        }
        bool fresh;
        const long long sl = bp_l2_add(Q, k, 1u, (long long)v, &fresh, ctl);
        if (fresh && sl >= 0) Q.list[atomicAdd(&Q.cnt[0], 1u)] = (uint32_t)sl;
    };
    for (int r = 0; r < rounds; r++) {
        const long long idx = base + (long long)(r * BP_THREADS + tid) * 4;
        if (idx >= Q.n) break;
        if (idx + 3 < Q.n) {
            const int4 k4 = qg_ldg_stream(reinterpret_cast<const int4 *>(Q.k + idx));
            const int4 v4 = qg_ldg_stream(reinterpret_cast<const int4 *>(Q.v + idx));
            int4 w4 = make_int4(0, 0, 0, 0);
            if (pred) w4 = qg_ldg_stream(reinterpret_cast<const int4 *>(Q.w + idx));
            const int32_t ks[4] = {k4.x, k4.y, k4.z, k4.w}, vs[4] = {v4.x, v4.y, v4.z, v4.w},
                          ws[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (!pred || ((ws[j] >= Q.lo) & (ws[j] <= Q.hi))) row((uint32_t)ks[j], vs[j]);
        } else {
            for (int j = 0; j < 4 && idx + j < Q.n; j++)
                if (!pred || ((Q.w[idx + j] >= Q.lo) & (Q.w[idx + j] <= Q.hi))) row((uint32_t)Q.k[idx + j], Q.v[idx + j]);
        }
    }
    __syncthreads();
    // flush: one L2 update per distinct key of the shared table and per row
    // set aside, several in flight per thread
    const uint32_t nov = min(S.nov, (uint32_t)BP_OVF);
    bp_l2_flush(Q, BP_SSLOTS / (BP_THREADS * BP_FLUSH),
                [&](int j, uint32_t *k, uint32_t *c, long long *sm) {
                    const int i = j * BP_THREADS + tid;
                    if (!S.tc[i]) return false;
                    *k = S.tk[i];
                    *c = S.tc[i];
                    *sm = bp_split_sum(S.tl[i], S.th[i]);
                    return true;
                },
                ctl);
    bp_l2_flush(Q, (int)((nov + BP_THREADS * BP_FLUSH - 1) / (BP_THREADS * BP_FLUSH)),
                [&](int j, uint32_t *k, uint32_t *c, long long *sm) {
                    const uint32_t i = (uint32_t)j * BP_THREADS + tid;
                    if (i >= nov) return false;
                    *k = S.ok[i];
                    *c = 1u;
                    *sm = (long long)S.ov[i];
                    return true;
                },
                ctl);
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        atomicAdd(&Q.cnt[1], 1u);
    }
}

__device__ void bp_emit_tile(const BQ &Q, uint32_t tile, uint32_t spin, qg_control *ctl) {
    __shared__ uint32_t s_len;
    const int tid = threadIdx.x;
    if (tid == 0) {
        uint32_t polls = 0;
        while (qg_ld_relaxed_u32(&Q.cnt[1]) < Q.ntiles) {
            if (polls++ >= spin) {
                qg_record_error(ctl, QG_ERR_TIMEOUT, QG_SITE_GROUPBY);
                break;
            }
            __nanosleep(64);
        }
        __threadfence();  // the group tiles' table updates are visible from here on
        s_len = qg_ld_relaxed_u32(&Q.cnt[0]);
    }
    __syncthreads();
    const uint32_t len = s_len;
    const uint32_t b = tile * BP_ETILE, e = min(len, b + BP_ETILE);
    int32_t *gk = reinterpret_cast<int32_t *>(Q.o0);
    long long *gs = reinterpret_cast<long long *>(Q.o1), *gc = reinterpret_cast<long long *>(Q.o2);
    for (uint32_t i = b + tid; i < e; i += BP_THREADS) {
        const uint32_t sl = Q.list[i];
        const unsigned long long kc = Q.tab[2 * sl];
        const long long s = (long long)Q.tab[2 * sl + 1];
        if ((long long)i < Q.cap) {
            gk[i] = (int32_t)(uint32_t)kc;
            gs[i] = s;
            gc[i] = (long long)(kc >> 32);
        }
        Q.tab[2 * sl] = 0ull;
        Q.tab[2 * sl + 1] = 0ull;
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&Q.cnt[2], 1u) == Q.etiles - 1) {  // the query's last emit item
            *Q.d_count = len;
            Q.cnt[0] = 0;
            Q.cnt[1] = 0;
            Q.cnt[2] = 0;
            __threadfence();
        }
    }
}

__global__ void __launch_bounds__(BP_THREADS, 3)
k_bpersist(const BQ *__restrict__ qs, const BItem *__restrict__ items, uint32_t nitems, BCtl *bc, uint32_t spin,
           int gtile_log2) {
    extern __shared__ __align__(16) unsigned char bp_raw[];
    BShared &S = *reinterpret_cast<BShared *>(bp_raw);
    const int tid = threadIdx.x;
    if (tid == 0) S.epoch = *(volatile uint32_t *)&bc->ctl.epoch;
    for (;;) {
        if (tid == 0) S.item = atomicAdd(&bc->head, 1u);
        __syncthreads();
        const uint32_t it = S.item;
        const uint32_t epoch = S.epoch;
        __syncthreads();
        if (it >= nitems) break;
        const BItem I = items[it];
        const BQ &Q = qs[I.q];
        const uint32_t kind = I.kt >> 30, tile = I.kt & 0x3fffffffu;
        if (kind == BK_FILTER)
            bp_filter_tile(S, Q, tile, epoch, qg_lookback{Q.status, &bc->ctl, spin, QG_SITE_FILTER});
        else if (kind == BK_GROUP)
            bp_group_tile(S, Q, tile, gtile_log2, &bc->ctl);
        else
            bp_emit_tile(Q, tile, spin, &bc->ctl);
    }
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(&bc->done, 1u) == gridDim.x - 1) {  // every CTA has finished: reset for the next replay
            bc->head = 0;
            bc->done = 0;
            bc->ctl.epoch = (S.epoch + 1u) & 0x3fffffffu;
            __threadfence();
        }
    }
}

}  // namespace

// Host side: the queue, the per-query state and the launch.
struct qg_bpersist {
    char *mem = nullptr;  // one allocation: queries | items | control | status words | tables | lists | counters
    BQ *qs = nullptr;
    BItem *items = nullptr;
    BCtl *ctl = nullptr;
    uint32_t nitems = 0;
    int grid = 0;
    int gtile_log2 = 13;
};

qg_status qg_bpersist_create(qg_ctx *ctx, const qg_query *q, int nq, const std::vector<int> &use, int gtile_log2,
                             qg_bpersist **out) {
    *out = nullptr;
    if (gtile_log2 < 10 || gtile_log2 > 16) return QG_ERR_INVALID;  // <= 2^16 rows keep the split sums exact
    std::vector<BQ> hq(nq);
    std::vector<BItem> tiles, emits;
    // sizes first: status words (filter), tables, lists and counters (group-by)
    size_t status_w = 0, tab_w = 0, list_w = 0, cnt_w = 0;
    std::vector<size_t> st_off(nq), tab_off(nq), list_off(nq), cnt_off(nq);
    std::vector<uint32_t> slots(nq, 0);
    for (int i : use) {
        const qg_query &x = q[i];
        if (x.n < 0 || x.n >= (1LL << 31) || x.cap < 0) return QG_ERR_UNSUPPORTED;
        if (((uintptr_t)x.in[0] | (uintptr_t)x.in[1] | (uintptr_t)(x.op == QG_OP_FUSED ? x.in[2] : nullptr)) & 15)
            return QG_ERR_INVALID;
        if (x.op == QG_OP_FILTER) {
            const uint32_t nt = (uint32_t)qg_ceil_div(x.n > 0 ? x.n : 1, BP_FTILE);
            st_off[i] = status_w;
            status_w += nt;
        } else {
            uint64_t s = 1024;  // load <= 1/2 for up to min(cap, n) groups
            const int64_t g = std::min<int64_t>(x.cap, x.n);
            while (s < (uint64_t)g * 2) s <<= 1;
            if (s > (1ull << 30)) return QG_ERR_UNSUPPORTED;
            slots[i] = (uint32_t)s;
            tab_off[i] = tab_w;
            tab_w += 2 * s;
            list_off[i] = list_w;
            list_w += s;
            cnt_off[i] = cnt_w;
            cnt_w += 4;
        }
    }
    const size_t qb = qg_align_up((size_t)nq * sizeof(BQ), 256);
    // items: filter tiles and group tiles first (largest queries first), emits after
    std::vector<int> order(use);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return q[a].n > q[b].n; });
    for (int i : order) {
        const qg_query &x = q[i];
        const uint32_t per = x.op == QG_OP_FILTER ? BP_FTILE : (1u << gtile_log2);
        const uint32_t nt = (uint32_t)qg_ceil_div(x.n > 0 ? x.n : 1, per);
        const uint32_t kind = x.op == QG_OP_FILTER ? (uint32_t)BK_FILTER : (uint32_t)BK_GROUP;
        for (uint32_t t = 0; t < nt; t++) tiles.push_back(BItem{(uint32_t)i, (kind << 30) | t});
        if (x.op != QG_OP_FILTER)
            for (uint32_t e = 0; e < slots[i] / BP_ETILE + (slots[i] % BP_ETILE ? 1 : 0); e++)
                emits.push_back(BItem{(uint32_t)i, ((uint32_t)BK_EMIT << 30) | e});
    }
    tiles.insert(tiles.end(), emits.begin(), emits.end());
    const size_t ib = qg_align_up(tiles.size() * sizeof(BItem), 256);
    const size_t cb = qg_align_up(sizeof(BCtl), 256);
    const size_t sb = qg_align_up(status_w * 8, 256), tb = qg_align_up(tab_w * 8, 256);
    const size_t lb = qg_align_up(list_w * 4, 256), nb = qg_align_up(cnt_w * 4, 256);
    qg_bpersist *p = new qg_bpersist();
    const size_t total = qb + ib + cb + sb + tb + lb + nb;
    if (cudaMalloc((void **)&p->mem, total) != cudaSuccess) {
        cudaGetLastError();
        delete p;
        return QG_ERR_OOM;
    }
    char *m = p->mem;
    p->qs = (BQ *)m;
    p->items = (BItem *)(m + qb);
    p->ctl = (BCtl *)(m + qb + ib);
    unsigned long long *status = (unsigned long long *)(m + qb + ib + cb);
    unsigned long long *tab = (unsigned long long *)(m + qb + ib + cb + sb);
    uint32_t *list = (uint32_t *)(m + qb + ib + cb + sb + tb);
    uint32_t *cnt = (uint32_t *)(m + qb + ib + cb + sb + tb + lb);
    for (int i = 0; i < nq; i++) {
        BQ &b = hq[i];
        memset(&b, 0, sizeof(b));
        const qg_query &x = q[i];
        b.k = x.in[0];
        b.v = x.in[1];
        b.w = x.op == QG_OP_FUSED ? x.in[2] : nullptr;
        b.o0 = x.out[0];
        b.o1 = x.out[1];
        b.o2 = x.out[2];
        b.n = x.n;
        b.cap = x.cap;
        b.lo = x.lo;
        b.hi = x.hi;
        b.d_count = (long long *)x.d_count;
        if (x.op == QG_OP_FILTER) {
            b.status = status + st_off[i];
            b.ntiles = (uint32_t)qg_ceil_div(x.n > 0 ? x.n : 1, BP_FTILE);
        } else if (x.op == QG_OP_GROUPBY || x.op == QG_OP_FUSED) {
            b.ntiles = (uint32_t)qg_ceil_div(x.n > 0 ? x.n : 1, 1LL << gtile_log2);
            b.etiles = slots[i] / BP_ETILE + (slots[i] % BP_ETILE ? 1 : 0);
            b.tab = tab + tab_off[i];
            b.mask = slots[i] - 1;
            b.list = list + list_off[i];
            b.cnt = cnt + cnt_off[i];
        }
    }
    cudaError_t e = cudaMemsetAsync(p->mem + qb + ib, 0, cb + sb + tb + lb + nb, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p->qs, hq.data(), (size_t)nq * sizeof(BQ), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(p->items, tiles.data(), tiles.size() * sizeof(BItem), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    int per_sm = 0;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_bpersist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BShared));
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bpersist, BP_THREADS, sizeof(BShared));
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(p->mem);
        delete p;
        return QG_ERR_CUDA;
    }
    p->nitems = (uint32_t)tiles.size();
    const long long g = (long long)ctx->sm_count * (per_sm > 0 ? per_sm : 1);
    p->grid = (int)std::max<long long>(1, std::min<long long>(g, p->nitems));
    p->gtile_log2 = gtile_log2;
    *out = p;
    return QG_OK;
}

qg_status qg_bpersist_launch(qg_ctx *ctx, qg_bpersist *p) {
    if (!p->nitems) return QG_OK;
    qg_pre_launch(ctx);
    k_bpersist<<<p->grid, BP_THREADS, sizeof(BShared), ctx->stream>>>(p->qs, p->items, p->nitems, p->ctl,
                                                                      ctx->spin_limit,
                                                        p->gtile_log2);
    return qg_check_launch(ctx, "k_bpersist");
}

// The first device error of the persistent launches (cleared once read).
qg_status qg_bpersist_check(qg_ctx *ctx, qg_bpersist *p) {
    int err = 0;
    QG_TRY_CUDA(ctx, cudaMemcpy(&err, &p->ctl->ctl.err, 4, cudaMemcpyDeviceToHost), "d2h");
    if (err) {
        int zero[2] = {0, 0};
        QG_TRY_CUDA(ctx, cudaMemcpy(&p->ctl->ctl.err, zero, 8, cudaMemcpyHostToDevice), "h2d");
        return (qg_status)err;
    }
    return QG_OK;
}

void qg_bpersist_destroy(qg_bpersist *p) {
    if (!p) return;
    if (p->mem) cudaFree(p->mem);
    delete p;
}
