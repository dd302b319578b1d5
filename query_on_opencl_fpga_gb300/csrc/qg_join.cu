// qg_join.cu -- hash join + filter + sort.
//
// Reference (kernel/hj_filter_sort/1/hj_filter_sort_op.cl):
//   buildHashTable (:25-60)  one 128-item work-group appends (key, val) into
//                            bucket key & (B-1) under a local spin lock,
//   probeHashTable (:62-109) scans every slot of the bucket and writes each
//                            match (S.val, R.val) into a per-work-item region,
//   then the filter (:117-349) and bitonic sort (:362-564) of the matches.
// The reference ships no host for this chain; the contract here is the one
// the operator list implies, with config 2's filter on S.payload applied
// before the join.
//
// GB300 design:
//   build  -- grid-wide open-addressing table of 64-bit slots
//             (key << 32 | payload) filled with atomicCAS; duplicate build
//             keys each take their own slot, so every match is found.  The
//             build also records min/max key for the sort.
//   probe  -- persistent CTAs stream S through shared memory in 2048-row
//             tiles fetched by the bulk-copy (TMA) engine with mbarrier
//             completion, double-buffered so the next tile lands while the
//             current one is probed.  The S-filter is applied on the staged
//             tile; surviving rows look up the table (first slots of all rows
//             loaded together for memory-level parallelism); matches are
//             staged in shared memory and written with one output reservation
//             per tile.  The probe also counts the sort digits of its output.
//   sort   -- LSD radix passes over (key - min_key) on the three output
//             columns (qg_sort.cu), ping-ponging between a temporary and the
//             caller's output so that the last pass lands in the output.
#include <string.h>
#include <vector>
#include "qg_internal.cuh"
#include "qg_sort.cuh"

namespace {

constexpr unsigned long long EMPTY_SLOT = ~0ull;

struct JoinCtl {
    uint32_t kmin, kmax;
    unsigned long long n_special;  // build rows equal to EMPTY_SLOT (key -1, payload -1)
    unsigned long long cursor;     // output rows produced
    unsigned long long sortn;      // rows the device-planned sort orders (0 when over capacity)
    uint32_t hist[4][QG_RADIX];
};

// Reference-layout hash table (qg_hash_build_ref / qg_hash_probe_ref): this
// header, padded to 256 bytes, then `slots` 8-byte slots (key << 32 | value,
// EMPTY_SLOT = free).
struct RefHashHdr {
    JoinCtl jc;      // key range and the count of build rows equal to EMPTY_SLOT
    uint32_t slots;  // a power of two
    uint32_t magic;
};
constexpr uint32_t REF_HASH_MAGIC = 0x71684a31u;
constexpr size_t REF_HASH_HDR = (sizeof(RefHashHdr) + 255) / 256 * 256;

__global__ void k_join_ctl_init(JoinCtl *jc) {
    int t = threadIdx.x;
    if (t == 0) {
        jc->kmin = 0xffffffffu;
        jc->kmax = 0;
        jc->n_special = 0;
        jc->cursor = 0;
        jc->sortn = 0;
    }
    for (int i = t; i < 4 * QG_RADIX; i += blockDim.x) (&jc->hist[0][0])[i] = 0;
}

// Build: rows i of R at rkey[i * stride], rpay[i * stride].
__global__ void __launch_bounds__(256)
k_join_build(const int32_t *__restrict__ rkey, const int32_t *__restrict__ rpay, long long stride_el,
             long long nR, unsigned long long *__restrict__ tab, uint32_t mask, JoinCtl *jc,
             qg_control *ctl) {
    uint32_t lmin = 0xffffffffu, lmax = 0;
    unsigned long long nspec = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nR; i += stride) {
        const uint32_t k = (uint32_t)__ldg(rkey + i * stride_el);
        const uint32_t p = (uint32_t)__ldg(rpay + i * stride_el);
        lmin = min(lmin, k);
        lmax = max(lmax, k);
        const unsigned long long packed = ((unsigned long long)k << 32) | p;
        if (packed == EMPTY_SLOT) { nspec++; continue; }
        uint32_t h = qg_hash32(k) & mask;
        uint32_t probes = 0;
        while (atomicCAS(&tab[h], EMPTY_SLOT, packed) != EMPTY_SLOT) {
            h = (h + 1) & mask;
            if (++probes > mask) { qg_record_error(ctl, QG_ERR_TABLE_FULL, QG_SITE_JOIN_BUILD); break; }
        }
    }
    lmin = __reduce_min_sync(QG_FULL_MASK, lmin);
    lmax = __reduce_max_sync(QG_FULL_MASK, lmax);
    if ((threadIdx.x & 31) == 0) {
        if (lmin != 0xffffffffu) atomicMin(&jc->kmin, lmin);
        if (lmax != 0) atomicMax(&jc->kmax, lmax);
    }
    if (nspec) atomicAdd(&jc->n_special, nspec);
}

// ---- mbarrier / bulk-copy helpers (PTX ISA: mbarrier, cp.async.bulk) ------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

constexpr int PJ_THREADS = 256;
constexpr int PJ_ROWS = 8;
constexpr int PJ_TILE = PJ_THREADS * PJ_ROWS;  // 2048 S rows per tile
constexpr int PJ_STAGES = 2;
constexpr int PJ_OUT = PJ_TILE;  // staged matches per tile before overflow

struct PjSmem {
    int32_t sk[PJ_STAGES][PJ_TILE];
    int32_t sp[PJ_STAGES][PJ_TILE];
    uint32_t ok[PJ_OUT], oa[PJ_OUT], ob[PJ_OUT];
    uint32_t hist[4][QG_RADIX];
    unsigned long long bar[PJ_STAGES];
    uint32_t ocount, oc, obase;
    int abort;
};

struct ProbeOut {
    uint32_t *k, *a, *b;
};

__device__ __forceinline__ void pj_issue(PjSmem &S, int stage, const int32_t *skey,
                                         const int32_t *spay, long long nS, long long t) {
    long long rows = nS - t * PJ_TILE;
    if (rows > PJ_TILE) rows = PJ_TILE;
    const uint32_t bulk = (uint32_t)(rows & ~3LL) * 4u;
    if (bulk) {
        mbar_arrive_expect_tx(&S.bar[stage], 2 * bulk);
        bulk_g2s(S.sk[stage], skey + t * PJ_TILE, bulk, &S.bar[stage]);
        bulk_g2s(S.sp[stage], spay + t * PJ_TILE, bulk, &S.bar[stage]);
    } else {
        mbar_arrive(&S.bar[stage]);
    }
}

__global__ void __launch_bounds__(PJ_THREADS)
k_join_probe(const int32_t *__restrict__ skey, const int32_t *__restrict__ spay, long long nS,
             int32_t slo, int32_t shi, const unsigned long long *__restrict__ tab, uint32_t mask,
             JoinCtl *jc, ProbeOut out, long long cap, uint32_t key_off, int npos,
             qg_control *ctl, uint32_t spin_limit) {
    extern __shared__ __align__(128) unsigned char pj_raw[];
    PjSmem &S = *reinterpret_cast<PjSmem *>(pj_raw);
    const int tid = threadIdx.x;
    const long long ntiles = (nS + PJ_TILE - 1) / PJ_TILE;
    const unsigned long long nspec = jc->n_special;
    for (int i = tid; i < 4 * QG_RADIX; i += PJ_THREADS) (&S.hist[0][0])[i] = 0;
    if (tid == 0) {
        for (int s = 0; s < PJ_STAGES; s++) mbar_init(&S.bar[s], 1);
        mbar_fence_init();
        S.ocount = 0;
        S.abort = 0;
    }
    __syncthreads();
    if (tid == 0) {
        for (int s = 0; s < PJ_STAGES; s++) {
            long long t = blockIdx.x + (long long)s * gridDim.x;
            if (t < ntiles) pj_issue(S, s, skey, spay, nS, t);
        }
    }

    const int lane = tid & 31;
    const uint32_t lt = qg_lanemask_lt();
    // Warp-aggregated emission: one shared-memory reservation per warp step.
    auto warp_emit = [&](bool hit, uint32_t k, uint32_t a, uint32_t b) {
        const uint32_t bal = __ballot_sync(QG_FULL_MASK, hit);
        if (!bal) return;
        const int leader = __ffs(bal) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&S.ocount, (uint32_t)__popc(bal));
        base = __shfl_sync(QG_FULL_MASK, base, leader);
        if (hit) {
            const uint32_t pos = base + __popc(bal & lt);
            if (pos < PJ_OUT) {
                S.ok[pos] = k;
                S.oa[pos] = a;
                S.ob[pos] = b;
            } else {
                unsigned long long g = atomicAdd(&jc->cursor, 1ull);
                if ((long long)g < cap) {
                    out.k[g] = k;
                    out.a[g] = a;
                    out.b[g] = b;
                }
            }
            const uint32_t kk = k - key_off;
            for (int q = 0; q < npos; q++) atomicAdd(&S.hist[q][(kk >> (8 * q)) & 255u], 1u);
        }
    };

    for (long long it = 0;; it++) {
        const long long t = blockIdx.x + it * gridDim.x;
        if (t >= ntiles) break;
        const int stage = (int)(it % PJ_STAGES);
        const uint32_t parity = (uint32_t)((it / PJ_STAGES) & 1);
        // Bounded wait for this tile's bulk copies.
        bool ready = false;
        for (uint32_t w = 0; w < spin_limit; w++)
            if (mbar_try_wait(&S.bar[stage], parity)) { ready = true; break; }
        if (!ready) {
            qg_record_error(ctl, QG_ERR_TIMEOUT, QG_SITE_JOIN_PROBE);
            S.abort = 1;
        }
        __syncthreads();
        if (S.abort) break;
        long long rows = nS - t * PJ_TILE;
        if (rows > PJ_TILE) rows = PJ_TILE;
        const int bulk_rows = (int)(rows & ~3LL);
        const long long gbase = t * PJ_TILE;

        int32_t k[PJ_ROWS], p[PJ_ROWS];
        bool act[PJ_ROWS];
        uint32_t h[PJ_ROWS];
        unsigned long long slot[PJ_ROWS];
#pragma unroll
        for (int j = 0; j < PJ_ROWS; j++) {
            const int r = tid + j * PJ_THREADS;
            act[j] = false;
            k[j] = 0;
            p[j] = 0;
            if (r < rows) {
                if (r < bulk_rows) {
                    k[j] = S.sk[stage][r];
                    p[j] = S.sp[stage][r];
                } else {
                    k[j] = skey[gbase + r];
                    p[j] = spay[gbase + r];
                }
                act[j] = (p[j] >= slo) & (p[j] <= shi);
            }
            h[j] = qg_hash32((uint32_t)k[j]) & mask;
        }
        // First slot of every surviving row, all loads in flight together.
#pragma unroll
        for (int j = 0; j < PJ_ROWS; j++) slot[j] = act[j] ? __ldg(&tab[h[j]]) : EMPTY_SLOT;
#pragma unroll
        for (int j = 0; j < PJ_ROWS; j++) {
            const uint32_t uk = (uint32_t)k[j];
            // Build rows equal to the empty-slot pattern (key -1, payload -1)
            // are counted, not stored; a probe key of -1 matches each of them.
            unsigned long long spec = (act[j] && uk == 0xffffffffu) ? nspec : 0ull;
            while (__any_sync(QG_FULL_MASK, spec != 0)) {
                warp_emit(spec != 0, uk, 0xffffffffu, (uint32_t)p[j]);
                if (spec) spec--;
            }
            bool a = act[j];
            uint32_t hh = h[j];
            unsigned long long sl = slot[j];
            uint32_t probes = 0;
            while (__any_sync(QG_FULL_MASK, a)) {
                bool hit = false;
                uint32_t rv = 0;
                if (a) {
                    if (sl == EMPTY_SLOT || probes > mask) {
                        a = false;
                    } else {
                        if ((uint32_t)(sl >> 32) == uk) { hit = true; rv = (uint32_t)sl; }
                        hh = (hh + 1) & mask;
                        sl = __ldg(&tab[hh]);
                        probes++;
                    }
                }
                warp_emit(hit, uk, rv, (uint32_t)p[j]);
            }
        }
        __syncthreads();
        if (tid == 0) {
            const long long nt = t + (long long)PJ_STAGES * gridDim.x;
            if (nt < ntiles) pj_issue(S, stage, skey, spay, nS, nt);
            uint32_t c = S.ocount < PJ_OUT ? S.ocount : PJ_OUT;
            S.oc = c;
            S.obase = c ? (uint32_t)atomicAdd(&jc->cursor, (unsigned long long)c) : 0u;
            S.ocount = 0;
        }
        __syncthreads();
        const uint32_t c = S.oc;
        const long long ob = S.obase;
        for (uint32_t q = tid; q < c; q += PJ_THREADS) {
            const long long g = ob + q;
            if (g < cap) {
                out.k[g] = S.ok[q];
                out.a[g] = S.oa[q];
                out.b[g] = S.ob[q];
            }
        }
    }
    __syncthreads();
    if (S.abort && tid == 0) {
        // Give in-flight copies a bounded chance to land before the CTA exits.
        for (int s = 0; s < PJ_STAGES; s++)
            for (uint32_t w = 0; w < spin_limit; w++)
                if (mbar_try_wait(&S.bar[s], 0) || mbar_try_wait(&S.bar[s], 1)) break;
    }
    for (int i = tid; i < npos * QG_RADIX; i += PJ_THREADS) {
        uint32_t c = (&S.hist[0][0])[i];
        if (c) atomicAdd(&(&jc->hist[0][0])[i], c);
    }
}

// Reference-layout probe: interleaved (key, val) S pairs, output (S.val, R.val).
__global__ void __launch_bounds__(256)
k_join_probe_ref(const uint32_t *__restrict__ s, long long nS, const unsigned long long *__restrict__ tab,
                 const RefHashHdr *__restrict__ hdr, unsigned long long *__restrict__ cursor,
                 uint32_t *__restrict__ out, long long cap) {
    const int lane = threadIdx.x & 31;
    const uint32_t lt = qg_lanemask_lt();
    const unsigned long long nspec = hdr->jc.n_special;
    const uint32_t mask = hdr->slots - 1;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long iters = (nS + stride - 1) / stride;
    for (long long it = 0; it < iters; it++) {
        const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x + it * stride;
        bool act = i < nS;
        uint32_t k = 0, v = 0;
        if (act) {
            uint2 kv = *reinterpret_cast<const uint2 *>(s + 2 * i);
            k = kv.x;
            v = kv.y;
        }
        uint32_t h = qg_hash32(k) & mask;
        unsigned long long spec_left = (act && k == 0xffffffffu) ? nspec : 0;
        uint32_t probes = 0;
        while (__any_sync(QG_FULL_MASK, act || spec_left)) {
            bool hit = false;
            uint32_t rv = 0;
            if (spec_left) {
                hit = true;
                rv = 0xffffffffu;
                spec_left--;
            } else if (act) {
                unsigned long long sl = __ldg(&tab[h]);
                if (sl == EMPTY_SLOT || ++probes > mask) {
                    act = false;
                } else {
                    if ((uint32_t)(sl >> 32) == k) { hit = true; rv = (uint32_t)sl; }
                    h = (h + 1) & mask;
                }
            }
            uint32_t b = __ballot_sync(QG_FULL_MASK, hit);
            unsigned long long base = 0;
            if (lane == 0 && b) base = atomicAdd(cursor, (unsigned long long)__popc(b));
            base = __shfl_sync(QG_FULL_MASK, base, 0);
            if (hit) {
                long long g = (long long)base + __popc(b & lt);
                if (g < cap) {
                    out[2 * g] = v;
                    out[2 * g + 1] = rv;
                }
            }
        }
    }
}

}  // namespace

static int grid_cap(qg_ctx *ctx, long long work, int per_block, int per_sm) {
    long long b = (work + per_block - 1) / per_block;
    long long c = (long long)ctx->sm_count * per_sm;
    if (b > c) b = c;
    if (b < 1) b = 1;
    return (int)b;
}

static int g_join_table_factor = 2;  // table slots >= factor * build rows (a power of two)

static uint32_t table_slots(long long nR) {
    uint64_t c = 1024;
    while (c < (uint64_t)nR * g_join_table_factor) c <<= 1;
    return (uint32_t)c;
}

void qg_join_set_table_factor(int factor) { g_join_table_factor = factor < 2 ? 2 : (factor > 8 ? 8 : factor); }

namespace {
// After the probe of the device-planned join: publish the count, and let the
// sort run only when the output fits.
__global__ void k_join_finish_async(JoinCtl *jc, long long cap, unsigned long long *d_count, qg_control *ctl) {
    const unsigned long long m = jc->cursor;
    *d_count = m;
    if (m > (unsigned long long)cap) {
        jc->sortn = 0;
        qg_record_error(ctl, QG_ERR_CAPACITY, QG_SITE_JOIN_PROBE);
    } else {
        jc->sortn = m;
    }
}
}  // namespace

// Build the table in aux; returns the control block (in scratch) and mask.
static qg_status join_build(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay, long long stride,
                            long long nR, size_t extra_aux, unsigned long long **tab_out,
                            uint32_t *mask_out, JoinCtl **jc_out, char **aux_tail) {
    if (nR >= (1LL << 30)) return QG_ERR_UNSUPPORTED;
    const uint32_t slots = table_slots(nR);
    const size_t tbytes = (size_t)slots * 8;
    char *aux;
    QG_TRY(qg_aux(ctx, tbytes + extra_aux + 256, &aux));
    char *scr;
    QG_TRY(qg_scratch(ctx, sizeof(JoinCtl), &scr));
    JoinCtl *jc = (JoinCtl *)scr;
    unsigned long long *tab = (unsigned long long *)aux;
    QG_TRY_CUDA(ctx, cudaMemsetAsync(tab, 0xff, tbytes, ctx->stream), "memset table");
    qg_pre_launch(ctx);
    k_join_ctl_init<<<1, 256, 0, ctx->stream>>>(jc);
    QG_TRY(qg_check_launch(ctx, "k_join_ctl_init"));
    if (nR > 0) {
        int blocks = grid_cap(ctx, nR, 256, 8);
        qg_pre_launch(ctx);
        k_join_build<<<blocks, 256, 0, ctx->stream>>>(rkey, rpay, stride, nR, tab, slots - 1, jc,
                                                      ctx->ctl);
        QG_TRY(qg_check_launch(ctx, "k_join_build"));
    }
    *tab_out = tab;
    *mask_out = slots - 1;
    *jc_out = jc;
    *aux_tail = aux + qg_align_up(tbytes, 256);
    return QG_OK;
}

// Hash join + filter + radix sort of the output (the variant of
// qg_join_filter_sort selected by qg_join_set_knobs(3, ...)).
qg_status qg_join_hash_sort(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay, int64_t nR,
                            const int32_t *skey, const int32_t *spay, int64_t nS, int32_t slo,
                            int32_t shi, int32_t *out_key, int32_t *out_rpay, int32_t *out_spay,
                            int64_t cap, int64_t *out_n) {
    if (!ctx || nR < 0 || nS < 0 || cap < 0 || !out_n) return QG_ERR_INVALID;
    if ((nR > 0 && (!rkey || !rpay)) || (nS > 0 && (!skey || !spay)) ||
        (cap > 0 && (!out_key || !out_rpay || !out_spay)))
        return QG_ERR_INVALID;
    if ((((uintptr_t)skey) | ((uintptr_t)spay)) & 15) return QG_ERR_INVALID;
    if (cap >= (1LL << 30) || nS >= (1LL << 40)) return QG_ERR_UNSUPPORTED;
    *out_n = 0;
    if (nR == 0 || nS == 0) return QG_OK;
    unsigned long long *tab;
    uint32_t mask;
    JoinCtl *jc;
    char *tail;
    const size_t colbytes = qg_align_up((size_t)(cap > 0 ? cap : 1) * 4, 256);
    QG_TRY(join_build(ctx, rkey, rpay, 1, nR, 3 * colbytes, &tab, &mask, &jc, &tail));
    JoinCtl hjc;
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(&hjc, jc, 16, cudaMemcpyDeviceToHost, ctx->stream), "ctl d2h");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    QG_TRY(qg_collect_error(ctx));
    const uint32_t key_off = hjc.kmin;
    const uint32_t range = hjc.kmax - hjc.kmin;
    const int bits = range ? 32 - __builtin_clz(range) : 0;
    const int npos = bits ? qg_sort_positions(bits) : 0;
    qg_sort_bufs A{nullptr, (uint32_t *)tail, (uint32_t *)(tail + colbytes),
                   (uint32_t *)(tail + 2 * colbytes)};
    qg_sort_bufs B{nullptr, (uint32_t *)out_key, (uint32_t *)out_rpay, (uint32_t *)out_spay};
    // Land the probe where an odd/even number of passes ends in B.
    const bool probe_to_a = (npos % 2) == 1;
    const qg_sort_bufs &P = probe_to_a ? A : B;
    ProbeOut po{P.k, P.a, P.b};
    const size_t smem = sizeof(PjSmem);
    static bool attr = false;
    if (!attr) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_join_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
        attr = true;
    }
    const long long ntiles = (nS + PJ_TILE - 1) / PJ_TILE;
    int blocks = (int)(ntiles < (long long)ctx->sm_count * 3 ? ntiles : (long long)ctx->sm_count * 3);
    qg_pre_launch(ctx);
    k_join_probe<<<blocks, PJ_THREADS, smem, ctx->stream>>>(skey, spay, nS, slo, shi, tab, mask, jc,
                                                             po, cap, key_off, npos, ctx->ctl,
                                                             ctx->spin_limit);
    QG_TRY(qg_check_launch(ctx, "k_join_probe"));
    std::vector<uint32_t> hh(4 * QG_RADIX);
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(&hjc, jc, sizeof(JoinCtl), cudaMemcpyDeviceToHost, ctx->stream), "ctl d2h");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    QG_TRY(qg_collect_error(ctx));
    const long long m = (long long)hjc.cursor;
    *out_n = m;
    if (m > cap) return QG_ERR_CAPACITY;
    if (m == 0) return QG_OK;
    int passes[4];
    uint32_t bases[4 * QG_RADIX];
    int np = npos ? qg_sort_plan(&hjc.hist[0][0], npos, m, passes, bases) : 0;
    bool in_other = false;
    QG_TRY(qg_radix_passes(ctx, true, P, probe_to_a ? B : A, m, key_off, passes, np, bases,
                           &in_other));
    const bool in_a = probe_to_a ? !in_other : in_other;
    if (in_a) {
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(out_key, A.k, (size_t)m * 4, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(out_rpay, A.a, (size_t)m * 4, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(out_spay, A.b, (size_t)m * 4, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
    }
    return qg_ctx_check(ctx);
}

// The hash join + filter + sort with no host round trip (for CUDA graph
// capture, e.g. by qg_batch): the sort always takes all four key digits and
// is planned on the device from the probe's digit counts.  d_count (device
// int64) receives the match count; more matches than cap records
// QG_ERR_CAPACITY in the context's error word and leaves the output unsorted.
qg_status qg_join_hash_sort_async(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay, int64_t nR,
                                  const int32_t *skey, const int32_t *spay, int64_t nS, int32_t slo,
                                  int32_t shi, int32_t *out_key, int32_t *out_rpay, int32_t *out_spay,
                                  int64_t cap, int64_t *d_count) {
    if (!ctx || nR < 0 || nS < 0 || cap < 0 || !d_count) return QG_ERR_INVALID;
    if ((nR > 0 && (!rkey || !rpay)) || (nS > 0 && (!skey || !spay)) ||
        (cap > 0 && (!out_key || !out_rpay || !out_spay)))
        return QG_ERR_INVALID;
    if ((((uintptr_t)skey) | ((uintptr_t)spay)) & 15) return QG_ERR_INVALID;
    if (cap >= (1LL << 30) || nS >= (1LL << 40)) return QG_ERR_UNSUPPORTED;
    if (nR == 0 || nS == 0 || cap == 0) {
        QG_TRY_CUDA(ctx, cudaMemsetAsync(d_count, 0, 8, ctx->stream), "memset count");
        return QG_OK;
    }
    const size_t colbytes = qg_align_up((size_t)cap * 4, 256);
    const size_t work = qg_align_up(qg_radix_dev_work_bytes(cap), 256);
    unsigned long long *tab;
    uint32_t mask;
    JoinCtl *jc;
    char *tail;
    QG_TRY(join_build(ctx, rkey, rpay, 1, nR, 3 * colbytes + work, &tab, &mask, &jc, &tail));
    qg_sort_bufs A{nullptr, (uint32_t *)out_key, (uint32_t *)out_rpay, (uint32_t *)out_spay};
    qg_sort_bufs B{nullptr, (uint32_t *)tail, (uint32_t *)(tail + colbytes), (uint32_t *)(tail + 2 * colbytes)};
    ProbeOut po{A.k, A.a, A.b};
    const size_t smem = sizeof(PjSmem);
    static bool attr = false;
    if (!attr) {
        QG_TRY_CUDA(ctx, cudaFuncSetAttribute(k_join_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "attr");
        attr = true;
    }
    const long long ntiles = (nS + PJ_TILE - 1) / PJ_TILE;
    int blocks = (int)(ntiles < (long long)ctx->sm_count * 3 ? ntiles : (long long)ctx->sm_count * 3);
    qg_pre_launch(ctx);
    k_join_probe<<<blocks, PJ_THREADS, smem, ctx->stream>>>(skey, spay, nS, slo, shi, tab, mask, jc, po, cap,
                                                             0u, 4, ctx->ctl, ctx->spin_limit);
    QG_TRY(qg_check_launch(ctx, "k_join_probe"));
    qg_pre_launch(ctx);
    k_join_finish_async<<<1, 1, 0, ctx->stream>>>(jc, cap, (unsigned long long *)d_count, ctx->ctl);
    QG_TRY(qg_check_launch(ctx, "k_join_finish_async"));
    bool in_b = false;
    QG_TRY(qg_radix_passes_dev(ctx, true, A, B, cap, &jc->sortn, &jc->hist[0][0], 4, 0u,
                               tail + 3 * colbytes, &in_b));
    return in_b ? QG_ERR_INVALID : QG_OK;  // four passes end where they began
}

// ---------------------------------------------------------------------------
// Reference layout: buildHashTable / probeHashTable
// (kernel/hj_filter_sort/1/hj_filter_sort_op.cl:25-60 and 62-109).  The
// reference's caller allocates the table (rHashTable, rHashCount) and may
// probe it with several S tables; here the caller allocates
// qg_hash_table_bytes(nR) bytes, qg_hash_build_ref fills them, and any number
// of qg_hash_probe_ref calls read them.
// ---------------------------------------------------------------------------
static uint32_t ref_table_slots(long long nR) {
    uint64_t c = 1024;
    while (c < (uint64_t)nR * 2) c <<= 1;
    return (uint32_t)c;
}

namespace {
__global__ void k_ref_hash_hdr_init(RefHashHdr *hdr, uint32_t slots) {
    if (threadIdx.x == 0) {
        hdr->slots = slots;
        hdr->magic = REF_HASH_MAGIC;
    }
}
}  // namespace

extern "C" QG_API int64_t qg_hash_table_bytes(int64_t nR) {
    if (nR < 0 || nR >= (1LL << 30)) return -1;
    return (int64_t)(REF_HASH_HDR + (size_t)ref_table_slots(nR) * 8);
}

extern "C" QG_API qg_status qg_hash_build_ref(qg_ctx *ctx, const uint32_t *r, int64_t nR, void *table,
                                              int64_t table_bytes) {
    if (!ctx || nR < 0 || !table || (nR > 0 && !r)) return QG_ERR_INVALID;
    if ((((uintptr_t)r) & 7) || (((uintptr_t)table) & 255)) return QG_ERR_INVALID;
    if (nR >= (1LL << 30)) return QG_ERR_UNSUPPORTED;
    if (table_bytes < qg_hash_table_bytes(nR)) return QG_ERR_CAPACITY;
    const uint32_t slots = ref_table_slots(nR);
    RefHashHdr *hdr = (RefHashHdr *)table;
    unsigned long long *tab = (unsigned long long *)((char *)table + REF_HASH_HDR);
    QG_TRY_CUDA(ctx, cudaMemsetAsync(tab, 0xff, (size_t)slots * 8, ctx->stream), "memset table");
    qg_pre_launch(ctx);
    k_join_ctl_init<<<1, 256, 0, ctx->stream>>>(&hdr->jc);
    QG_TRY(qg_check_launch(ctx, "k_join_ctl_init"));
    qg_pre_launch(ctx);
    k_ref_hash_hdr_init<<<1, 32, 0, ctx->stream>>>(hdr, slots);
    QG_TRY(qg_check_launch(ctx, "k_ref_hash_hdr_init"));
    if (nR > 0) {
        int blocks = grid_cap(ctx, nR, 256, 8);
        qg_pre_launch(ctx);
        k_join_build<<<blocks, 256, 0, ctx->stream>>>((const int32_t *)r, (const int32_t *)r + 1, 2, nR, tab,
                                                      slots - 1, &hdr->jc, ctx->ctl);
        QG_TRY(qg_check_launch(ctx, "k_join_build"));
    }
    // a table that fills up (cannot happen at 2 slots per row) reports TABLE_FULL
    return qg_ctx_check(ctx);
}

extern "C" QG_API qg_status qg_hash_probe_ref(qg_ctx *ctx, const void *table, const uint32_t *s, int64_t nS,
                                              uint32_t *out, int64_t cap, int64_t *out_n) {
    if (!ctx || !table || nS < 0 || cap < 0 || !out_n) return QG_ERR_INVALID;
    if ((nS > 0 && !s) || (cap > 0 && !out)) return QG_ERR_INVALID;
    if ((((uintptr_t)s) | ((uintptr_t)out)) & 7 || (((uintptr_t)table) & 255)) return QG_ERR_INVALID;
    *out_n = 0;
    if (nS == 0) return QG_OK;
    const RefHashHdr *hdr = (const RefHashHdr *)table;
    const unsigned long long *tab = (const unsigned long long *)((const char *)table + REF_HASH_HDR);
    unsigned long long *cursor = &ctx->ctl->counter[0];
    QG_TRY_CUDA(ctx, cudaMemsetAsync(cursor, 0, 8, ctx->stream), "memset cursor");
    int blocks = grid_cap(ctx, nS, 256, 8);
    qg_pre_launch(ctx);
    k_join_probe_ref<<<blocks, 256, 0, ctx->stream>>>(s, nS, tab, hdr, cursor, out, cap);
    QG_TRY(qg_check_launch(ctx, "k_join_probe_ref"));
    long long m = 0;
    QG_TRY(qg_read_count(ctx, (const long long *)cursor, &m));
    *out_n = m;
    return m > cap ? QG_ERR_CAPACITY : QG_OK;
}

extern "C" QG_API qg_status qg_hash_join_ref(qg_ctx *ctx, const uint32_t *r, int64_t nR,
                                             const uint32_t *s, int64_t nS, uint32_t *out,
                                             int64_t cap, int64_t *out_n) {
    if (!ctx || nR < 0 || nS < 0 || cap < 0 || !out_n) return QG_ERR_INVALID;
    if ((nR > 0 && !r) || (nS > 0 && !s) || (cap > 0 && !out)) return QG_ERR_INVALID;
    if ((((uintptr_t)r) | ((uintptr_t)s) | ((uintptr_t)out)) & 7) return QG_ERR_INVALID;
    *out_n = 0;
    if (nR == 0 || nS == 0) return QG_OK;
    const int64_t tb = qg_hash_table_bytes(nR);
    if (tb < 0) return QG_ERR_UNSUPPORTED;
    char *aux;
    QG_TRY(qg_aux(ctx, (size_t)tb, &aux));  // the aux arena is 256-byte aligned
    QG_TRY(qg_hash_build_ref(ctx, r, nR, aux, tb));
    return qg_hash_probe_ref(ctx, aux, s, nS, out, cap, out_n);
}
