// qg_reduce.cu -- whole-column reduce and the radix split operator.
//
// Reduce: the reference checks a whole-column SUM / MAX / MIN / AVERAGE of
// Record.y against its own loop (validateReduce, host/host/Validate.cpp:
// 372-468) but ships no kernel for it.  Semantics follow that loop: .y is an
// unsigned int (Record = uint2, common.h:28), the sum wraps modulo 2^32, MAX
// and MIN compare unsigned (the loop's int accumulator is promoted to
// unsigned), AVERAGE = wrapped sum / n in unsigned arithmetic.
//
// Split: splitImpl (host/host/testSplit.cpp:156-209) maps each Record to a
// partition id, counts, scans and scatters so that d_S holds the records
// grouped by partition and d_bound the start of every partition.  Its
// kernels (mapPart_kernel, countHist_int, writeHist_int, getBound_int) are
// not shipped; here the partition id is y mod numPart and the split is
// stable (input order within a partition), built from the library's radix
// passes over the partition id.
#include <vector>
#include "qg_internal.cuh"
#include "qg_sort.cuh"

namespace {

__global__ void __launch_bounds__(256)
k_reduce_rec(const uint2 *__restrict__ in, long long n, int op, unsigned int *__restrict__ out) {
    unsigned int acc = op == QG_REDUCE_MIN ? 0xffffffffu : 0u;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned int y = __ldg(&in[i]).y;
        if (op == QG_REDUCE_MAX) acc = max(acc, y);
        else if (op == QG_REDUCE_MIN) acc = min(acc, y);
        else acc += y;
    }
    if (op == QG_REDUCE_MAX) acc = __reduce_max_sync(QG_FULL_MASK, acc);
    else if (op == QG_REDUCE_MIN) acc = __reduce_min_sync(QG_FULL_MASK, acc);
    else acc = __reduce_add_sync(QG_FULL_MASK, acc);
    if ((threadIdx.x & 31) == 0) {
        if (op == QG_REDUCE_MAX) atomicMax(out, acc);
        else if (op == QG_REDUCE_MIN) atomicMin(out, acc);
        else atomicAdd(out, acc);
    }
}

// Records -> KV3 items (partition id, x, y) and back.
__global__ void k_split_pack(const uint2 *__restrict__ in, long long n, uint32_t parts, uint32_t *__restrict__ k,
                             uint32_t *__restrict__ a, uint32_t *__restrict__ b) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const uint2 r = __ldg(&in[i]);
        k[i] = r.y % parts;
        a[i] = r.x;
        b[i] = r.y;
    }
}
__global__ void k_split_unpack(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b, long long n,
                               uint2 *__restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = make_uint2(__ldg(a + i), __ldg(b + i));
}

// bound[p] = first row of partition p in the split output (ids sorted).
__global__ void k_split_bounds(const uint32_t *__restrict__ pid, long long n, int32_t parts,
                               int32_t *__restrict__ bound) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= parts) return;
    long long lo = 0, hi = n;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (__ldg(pid + mid) < (uint32_t)p) lo = mid + 1;
        else hi = mid;
    }
    bound[p] = (int32_t)lo;
}

int grid_of(qg_ctx *ctx, long long n) {
    long long b = (n + 255) / 256, c = (long long)ctx->sm_count * 8;
    return (int)(b < 1 ? 1 : (b > c ? c : b));
}

}  // namespace

extern "C" QG_API qg_status qg_reduce_rec(qg_ctx *ctx, const void *in, int64_t n, int op, uint32_t *result) {
    if (!ctx || !result || n < 0 || op < QG_REDUCE_SUM || op > QG_REDUCE_AVERAGE || (n > 0 && !in))
        return QG_ERR_INVALID;
    if ((uintptr_t)in & 7) return QG_ERR_INVALID;
    if (n == 0) {  // the reference divides by rLen for AVERAGE; an empty column has no value
        if (op == QG_REDUCE_AVERAGE) return QG_ERR_INVALID;
        *result = op == QG_REDUCE_MIN ? 0xffffffffu : 0u;
        return QG_OK;
    }
    unsigned int *d = (unsigned int *)&ctx->ctl->counter[3];
    const unsigned int init = op == QG_REDUCE_MIN ? 0xffffffffu : 0u;
    QG_TRY_CUDA(ctx, cudaMemsetAsync(d, init ? 0xff : 0, 4, ctx->stream), "memset result");
    qg_pre_launch(ctx);
    k_reduce_rec<<<grid_of(ctx, n), 256, 0, ctx->stream>>>((const uint2 *)in, n, op, d);
    QG_TRY(qg_check_launch(ctx, "k_reduce_rec"));
    long long h = 0;
    QG_TRY(qg_read_count(ctx, (const long long *)d, &h));
    uint32_t v = (uint32_t)(unsigned long long)h;
    if (op == QG_REDUCE_AVERAGE) v = v / (uint32_t)n;
    *result = v;
    return QG_OK;
}

extern "C" QG_API qg_status qg_split_rec(qg_ctx *ctx, const void *in, int64_t n, int32_t num_part, void *out,
                                         int32_t *bound) {
    if (!ctx || n < 0 || num_part < 1 || (n > 0 && (!in || !out)) || !bound) return QG_ERR_INVALID;
    if (((uintptr_t)in & 7) || ((uintptr_t)out & 7)) return QG_ERR_INVALID;
    if (n >= (1LL << 30)) return QG_ERR_UNSUPPORTED;
    if (n == 0) {
        QG_TRY_CUDA(ctx, cudaMemsetAsync(bound, 0, (size_t)num_part * 4, ctx->stream), "memset bound");
        return qg_ctx_check(ctx);
    }
    // aux: two KV3 buffers (partition id, x, y)
    const size_t col = qg_align_up((size_t)n * 4, 256);
    char *aux;
    QG_TRY(qg_aux(ctx, 6 * col, &aux));
    qg_sort_bufs A{nullptr, (uint32_t *)aux, (uint32_t *)(aux + col), (uint32_t *)(aux + 2 * col)};
    qg_sort_bufs B{nullptr, (uint32_t *)(aux + 3 * col), (uint32_t *)(aux + 4 * col), (uint32_t *)(aux + 5 * col)};
    qg_pre_launch(ctx);
    k_split_pack<<<grid_of(ctx, n), 256, 0, ctx->stream>>>((const uint2 *)in, n, (uint32_t)num_part, A.k, A.a, A.b);
    QG_TRY(qg_check_launch(ctx, "k_split_pack"));
    const uint32_t maxpid = (uint32_t)num_part - 1;
    const int bits = maxpid ? 32 - __builtin_clz(maxpid) : 0;
    bool in_b = false;
    std::vector<uint32_t> h(4 * QG_RADIX), bases(4 * QG_RADIX);
    char *scr;
    QG_TRY(qg_scratch(ctx, 4 * QG_RADIX * 4, &scr));
    const int npos = bits ? qg_sort_positions(bits) : 0;
    if (npos) {
        QG_TRY(qg_radix_histogram(ctx, A, true, n, 0u, npos, (uint32_t *)scr));
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(h.data(), scr, 4 * QG_RADIX * 4, cudaMemcpyDeviceToHost, ctx->stream), "hist d2h");
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "sync");
        int passes[4];
        const int np = qg_sort_plan(h.data(), npos, n, passes, bases.data());
        QG_TRY(qg_radix_passes(ctx, true, A, B, n, 0u, passes, np, bases.data(), &in_b));
    }
    const qg_sort_bufs &R = in_b ? B : A;
    qg_pre_launch(ctx);
    k_split_unpack<<<grid_of(ctx, n), 256, 0, ctx->stream>>>(R.a, R.b, n, (uint2 *)out);
    QG_TRY(qg_check_launch(ctx, "k_split_unpack"));
    qg_pre_launch(ctx);
    k_split_bounds<<<(num_part + 255) / 256, 256, 0, ctx->stream>>>(R.k, n, num_part, bound);
    QG_TRY(qg_check_launch(ctx, "k_split_bounds"));
    return qg_ctx_check(ctx);
}
