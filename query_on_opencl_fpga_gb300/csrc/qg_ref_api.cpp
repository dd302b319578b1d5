// qg_ref_api.cpp -- the reference's operator surface (include/qg_ref.h) over
// the C ABI of libqg.so.  Each function names the reference function it
// stands in for; the arithmetic all happens in the CUDA kernels behind qg.h.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>

#include "qg.h"
#include "qg_ref.h"

namespace {

thread_local qg_status t_last = QG_OK;
std::mutex g_default_mu;
qg_ctx *g_default_ctx = nullptr;
int g_default_dev = -1;

qg_ctx *pick(qg_ctx *ctx) { return ctx ? ctx : qg_ref_default_ctx(); }

// Record a status; a failure prints one line (the reference printed and exited).
bool ok(qg_status s, const char *where, qg_ctx *ctx) {
    t_last = s;
    if (s != QG_OK) {
        fprintf(stderr, "%s: %s%s%s\n", where, qg_status_string(s), ctx ? " -- " : "",
                ctx ? qg_last_error_message(ctx) : "");
        return false;
    }
    return true;
}

bool cuda_ok(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return true;
    cudaGetLastError();
    t_last = QG_ERR_CUDA;
    fprintf(stderr, "%s: %s\n", where, cudaGetErrorString(e));
    return false;
}

// Device copy of a host array (freed by the caller with cudaFree).
template <typename T>
T *to_device(const T *h, size_t count, const char *where) {
    void *d = nullptr;
    if (!cuda_ok(cudaMalloc(&d, count ? count * sizeof(T) : 16), where)) return nullptr;
    if (count && !cuda_ok(cudaMemcpy(d, h, count * sizeof(T), cudaMemcpyHostToDevice), where)) {
        cudaFree(d);
        return nullptr;
    }
    return (T *)d;
}

}  // namespace

extern "C" {

QG_API qg_status qg_ref_last_status(void) { return t_last; }

QG_API qg_ctx *qg_ref_default_ctx(void) {
    std::lock_guard<std::mutex> lock(g_default_mu);
    int dev = 0;
    cudaGetDevice(&dev);
    if (!g_default_ctx || dev != g_default_dev) {
        qg_ctx *c = nullptr;
        if (qg_ctx_create(&c, nullptr) != QG_OK) return nullptr;
        g_default_ctx = c;  // a context per process, as the reference's global OpenCL state
        g_default_dev = dev;
    }
    return g_default_ctx;
}

QG_API qg_status qg_buf_alloc(qg_buf *b, size_t bytes) {
    if (!b) return QG_ERR_INVALID;
    b->ptr = nullptr;
    b->bytes = 0;
    if (cudaMalloc(&b->ptr, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        b->ptr = nullptr;
        return QG_ERR_OOM;
    }
    b->bytes = bytes;
    return QG_OK;
}

QG_API void qg_buf_free(qg_buf *b) {
    if (b && b->ptr) {
        cudaDeviceSynchronize();
        cudaFree(b->ptr);
        b->ptr = nullptr;
        b->bytes = 0;
    }
}

// ---- filter -----------------------------------------------------------------
// filterImpl (host/host/testFilter.cpp:92-154): map -> scan -> outSize ->
// write becomes one single-pass kernel.  *d_Rout is allocated with rLen
// records, as the reference does (testFilter.cpp:137).  Rows are
// d_Rin[beginPos .. beginPos + rLen), the range validateFilter checks
// (host/host/Validate.cpp:326).
QG_API void filterImpl(qg_buf d_Rin, int beginPos, int rLen, qg_buf *d_Rout, int *outSize,
                       int numThread, int numBlock, int smallKey, int largeKey, qg_ctx *ctx) {
    (void)numThread;
    (void)numBlock;
    ctx = pick(ctx);
    if (!d_Rout || !outSize || rLen < 0 || beginPos < 0) {
        ok(QG_ERR_INVALID, "filterImpl", ctx);
        return;
    }
    *outSize = 0;
    if (!ok(qg_buf_alloc(d_Rout, (size_t)rLen * sizeof(qg_record)), "filterImpl", ctx)) return;
    const qg_record *in = (const qg_record *)d_Rin.ptr + beginPos;
    int64_t n = 0;
    if (ok(qg_filter_range_rec(ctx, in, rLen, smallKey, largeKey, d_Rout->ptr, rLen, &n),
           "filterImpl", ctx))
        *outSize = (int)n;
}

// range_selection (host/host/Selection.cpp:6-16)
QG_API int range_selection(qg_buf d_Rin, int rLen, int rangeSmallKey, int rangeLargeKey,
                           qg_buf *d_Rout, int numThreadPB, int numBlock, qg_ctx *ctx) {
    int outSize = 0;
    filterImpl(d_Rin, 0, rLen, d_Rout, &outSize, numThreadPB, numBlock, rangeSmallKey, rangeLargeKey,
               ctx);
    return t_last == QG_OK ? outSize : -1;
}

// CL_RangeSelection (host/host/Selection.cpp:19-50)
QG_API int CL_RangeSelection(qg_record *h_Rin, int rLen, int rangeSmallKey, int rangeLargeKey,
                             qg_record **h_Rout, int numThreadPB, int numBlock, int _CPU_GPU) {
    (void)_CPU_GPU;
    if (!h_Rout || rLen < 0 || (rLen > 0 && !h_Rin)) {
        ok(QG_ERR_INVALID, "CL_RangeSelection", nullptr);
        return -1;
    }
    qg_record *d_in = to_device(h_Rin, (size_t)rLen, "CL_RangeSelection");
    if (!d_in) return -1;
    qg_buf in{d_in, (size_t)rLen * sizeof(qg_record)}, out{nullptr, 0};
    int outSize = range_selection(in, rLen, rangeSmallKey, rangeLargeKey, &out, numThreadPB, numBlock,
                                  nullptr);
    if (outSize >= 0) {
        *h_Rout = (qg_record *)malloc(sizeof(qg_record) * (outSize ? outSize : 1));
        if (!cuda_ok(cudaMemcpy(*h_Rout, out.ptr, sizeof(qg_record) * outSize, cudaMemcpyDeviceToHost),
                     "CL_RangeSelection"))
            outSize = -1;
    }
    cudaFree(d_in);
    qg_buf_free(&out);
    return outSize;
}

// ---- scan -------------------------------------------------------------------
// initScan (host/host/testScan.cpp:26-83): the pass count the multi-level scan
// would use, kept for callers that print it; nothing is allocated.
QG_API void initScan(int rLen, ScanPara *SP) {
    if (!SP) return;
    SP->gLength = (uint32_t)rLen;
    SP->blockSize = 256;
    float t = rLen > 0 ? logf((float)rLen) / logf(256.0f) : 0.0f;
    SP->pass = (uint32_t)t;
    if (fabsf(t - (float)SP->pass) < 1e-7f && SP->pass > 0) SP->pass--;
    t_last = QG_OK;
}

// scanImpl (host/host/testScan.cpp:278-340): exclusive int32 scan, one kernel.
QG_API void scanImpl(qg_buf d_Src, int rLen, qg_buf d_Dst, ScanPara *SP, qg_ctx *ctx) {
    (void)SP;
    ctx = pick(ctx);
    if (ok(qg_scan_excl_i32(ctx, (const int32_t *)d_Src.ptr, (int32_t *)d_Dst.ptr, rLen), "scanImpl",
           ctx))
        ok(qg_ctx_check(ctx), "scanImpl", ctx);
}

// closeScan (host/host/testScan.cpp:229-275): nothing to release.
QG_API void closeScan(ScanPara *SP) {
    (void)SP;
    t_last = QG_OK;
}

// ---- sort -------------------------------------------------------------------
// radixSortImpl_sm (host/host/testSort.cpp:24-136): ascending by unsigned .y, in place.
QG_API void radixSortImpl_sm(qg_buf d_R, int rLen, int meaningless, int numThreadPB, int numBlock,
                             qg_ctx *ctx) {
    (void)meaningless;
    (void)numThreadPB;
    (void)numBlock;
    ctx = pick(ctx);
    ok(qg_sort_rec_by_y(ctx, d_R.ptr, rLen), "radixSortImpl_sm", ctx);
}

// CL_RadixSort (host/host/Sort.cpp:34-67)
QG_API void CL_RadixSort(qg_record *h_Rin, int rLen, qg_record *h_Rout, int numThread,
                         int numBlock, int _CPU_GPU) {
    (void)_CPU_GPU;
    if (rLen < 0 || (rLen > 0 && (!h_Rin || !h_Rout))) {
        ok(QG_ERR_INVALID, "CL_RadixSort", nullptr);
        return;
    }
    qg_record *d = to_device(h_Rin, (size_t)rLen, "CL_RadixSort");
    if (!d) return;
    radixSortImpl_sm(qg_buf{d, (size_t)rLen * sizeof(qg_record)}, rLen, 32, numThread, numBlock,
                     nullptr);
    if (t_last == QG_OK)
        cuda_ok(cudaMemcpy(h_Rout, d, sizeof(qg_record) * rLen, cudaMemcpyDeviceToHost), "CL_RadixSort");
    cudaFree(d);
}

// ---- group-by ---------------------------------------------------------------
// groupByImpl (host/host/testGroupBy.cpp:81-154)
QG_API int groupByImpl(qg_buf d_Rin, int rLen, qg_buf d_Rout, qg_buf *d_startPos, int numThread,
                       int numBlock, qg_ctx *ctx) {
    (void)numThread;
    (void)numBlock;
    ctx = pick(ctx);
    if (!d_startPos || rLen < 0) {
        ok(QG_ERR_INVALID, "groupByImpl", ctx);
        return -1;
    }
    qg_buf tmp{nullptr, 0};
    if (!ok(qg_buf_alloc(&tmp, (size_t)(rLen ? rLen : 1) * sizeof(int32_t)), "groupByImpl", ctx))
        return -1;
    int64_t g = 0;
    if (!ok(qg_groupby_rec(ctx, d_Rin.ptr, rLen, d_Rout.ptr, (int32_t *)tmp.ptr, rLen, &g),
            "groupByImpl", ctx)) {
        qg_buf_free(&tmp);
        return -1;
    }
    // *d_startPos holds numGroups ints, as the reference allocates it (:142).
    if (!ok(qg_buf_alloc(d_startPos, (size_t)(g ? g : 1) * sizeof(int32_t)), "groupByImpl", ctx) ||
        !cuda_ok(cudaMemcpy(d_startPos->ptr, tmp.ptr, (size_t)g * sizeof(int32_t),
                            cudaMemcpyDeviceToDevice), "groupByImpl")) {
        qg_buf_free(&tmp);
        return -1;
    }
    qg_buf_free(&tmp);
    return (int)g;
}

// CL_GroupBy (host/host/GroupBy.cpp:7-45)
QG_API int CL_GroupBy(qg_record *h_Rin, int rLen, qg_record *h_Rout, int **h_startPos,
                      int numThread, int numBlock, int _CPU_GPU) {
    (void)_CPU_GPU;
    if (!h_startPos || rLen < 0 || (rLen > 0 && (!h_Rin || !h_Rout))) {
        ok(QG_ERR_INVALID, "CL_GroupBy", nullptr);
        return -1;
    }
    qg_record *d_in = to_device(h_Rin, (size_t)rLen, "CL_GroupBy");
    if (!d_in) return -1;
    qg_buf in{d_in, (size_t)rLen * sizeof(qg_record)}, sp{nullptr, 0};
    int g = groupByImpl(in, rLen, in, &sp, numThread, numBlock, nullptr);
    if (g >= 0) {
        *h_startPos = (int *)malloc(sizeof(int) * (g ? g : 1));
        if (!cuda_ok(cudaMemcpy(*h_startPos, sp.ptr, sizeof(int) * g, cudaMemcpyDeviceToHost), "CL_GroupBy") ||
            !cuda_ok(cudaMemcpy(h_Rout, d_in, sizeof(qg_record) * rLen, cudaMemcpyDeviceToHost), "CL_GroupBy"))
            g = -1;
    }
    cudaFree(d_in);
    qg_buf_free(&sp);
    return g;
}

// ---- aggregation ------------------------------------------------------------
// parallelAggregate_init (host/host/testAggAfterGB.cpp:69-91)
QG_API void parallelAggregate_init(qg_buf d_S, qg_buf d_startPos, qg_buf d_aggResults,
                                   int OPERATOR, int blockOffset, int numGroups, int numBlock,
                                   int numThread, int sharedMemSize, int rLen, qg_ctx *ctx) {
    (void)numThread;
    (void)sharedMemSize;
    ctx = pick(ctx);
    ok(qg_aggregate_group_range(ctx, d_S.ptr, rLen, (const int32_t *)d_startPos.ptr, numGroups,
                                blockOffset, numBlock, OPERATOR, (int32_t *)d_aggResults.ptr),
       "parallelAggregate_init", ctx);
}

// aggAfterGroupByImpl (host/host/testAggAfterGB.cpp:92-123): gather
// S[i] = Ragg[Rin[i].x] (mapBeforeGather + gatherImpl), then aggregate .x of S
// (parallelAggregate_kernel reads d_S[i].x, group_by_cu_op_dp.cl:570; the
// reference's validator reads .y instead, Validate.cpp:195-231).  One launch
// for all groups instead of chunks of 512.
QG_API void aggAfterGroupByImpl(qg_buf d_Rin, int rLen, qg_buf d_startPos, int numGroups,
                                qg_buf d_Ragg, qg_buf d_aggResults, int OPERATOR, int numThread,
                                qg_ctx *ctx) {
    (void)numThread;
    ctx = pick(ctx);
    qg_buf S{nullptr, 0};
    if (!ok(qg_buf_alloc(&S, (size_t)(rLen ? rLen : 1) * sizeof(qg_record)), "aggAfterGroupByImpl", ctx))
        return;
    const int64_t aggLen = (int64_t)(d_Ragg.bytes / sizeof(qg_record));
    if (ok(qg_gather_rec(ctx, d_Ragg.ptr, aggLen, (const int32_t *)d_Rin.ptr, 2, rLen, S.ptr),
           "aggAfterGroupByImpl", ctx))
        ok(qg_aggregate_groups(ctx, S.ptr, rLen, (const int32_t *)d_startPos.ptr, numGroups, OPERATOR,
                               (int32_t *)d_aggResults.ptr),
           "aggAfterGroupByImpl", ctx);
    qg_buf_free(&S);
}

static void cl_agg(const char *name, int op, qg_record *h_Rin, int rLen, int *h_startPos,
                   int numGroups, qg_record *h_Ragg, int *h_aggResults, int numThread) {
    if (rLen < 0 || numGroups < 0 || (rLen > 0 && (!h_Rin || !h_Ragg)) ||
        (numGroups > 0 && (!h_startPos || !h_aggResults))) {
        ok(QG_ERR_INVALID, name, nullptr);
        return;
    }
    qg_record *d_in = to_device(h_Rin, (size_t)rLen, name);
    int *d_sp = to_device(h_startPos, (size_t)numGroups, name);
    qg_record *d_agg_in = to_device(h_Ragg, (size_t)rLen, name);
    int *d_out = to_device(h_aggResults, (size_t)numGroups, name);
    if (d_in && d_sp && d_agg_in && d_out) {
        aggAfterGroupByImpl(qg_buf{d_in, (size_t)rLen * 8}, rLen, qg_buf{d_sp, (size_t)numGroups * 4},
                            numGroups, qg_buf{d_agg_in, (size_t)rLen * 8},
                            qg_buf{d_out, (size_t)numGroups * 4}, op, numThread, nullptr);
        if (t_last == QG_OK)
            cuda_ok(cudaMemcpy(h_aggResults, d_out, sizeof(int) * numGroups, cudaMemcpyDeviceToHost), name);
    }
    cudaFree(d_in);
    cudaFree(d_sp);
    cudaFree(d_agg_in);
    cudaFree(d_out);
}

// CL_agg_{max,min,sum,avg}_afterGroupBy (host/host/AggAfterGroupBy.cpp:30-170)
QG_API void CL_agg_max_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread, int) {
    cl_agg("CL_agg_max_afterGroupBy", QG_REDUCE_MAX, h_Rin, rLen, h_startPos, numGroups, h_Ragg,
           h_aggResults, numThread);
}
QG_API void CL_agg_min_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread, int) {
    cl_agg("CL_agg_min_afterGroupBy", QG_REDUCE_MIN, h_Rin, rLen, h_startPos, numGroups, h_Ragg,
           h_aggResults, numThread);
}
QG_API void CL_agg_sum_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread, int) {
    cl_agg("CL_agg_sum_afterGroupBy", QG_REDUCE_SUM, h_Rin, rLen, h_startPos, numGroups, h_Ragg,
           h_aggResults, numThread);
}
QG_API void CL_agg_avg_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread, int) {
    cl_agg("CL_agg_avg_afterGroupBy", QG_REDUCE_AVERAGE, h_Rin, rLen, h_startPos, numGroups, h_Ragg,
           h_aggResults, numThread);
}

// ---- gather / scatter (host/host/testScatter.cpp:63-137) ---------------------
QG_API void gatherImpl(qg_buf d_R, int rLen, qg_buf d_loc, qg_buf d_S, int sLen, int numThreadPB,
                       int numBlock, qg_ctx *ctx) {
    (void)numThreadPB;
    (void)numBlock;
    ctx = pick(ctx);
    if (ok(qg_gather_rec(ctx, d_R.ptr, rLen, (const int32_t *)d_loc.ptr, 1, sLen, d_S.ptr), "gatherImpl",
           ctx))
        ok(qg_ctx_check(ctx), "gatherImpl", ctx);
}

QG_API void scatterImpl(qg_buf d_R, int rLen, qg_buf d_loc, qg_buf d_S, int numThreadPB,
                        int numBlock, qg_ctx *ctx) {
    (void)numThreadPB;
    (void)numBlock;
    ctx = pick(ctx);
    const int64_t sLen = (int64_t)(d_S.bytes / sizeof(qg_record));
    if (ok(qg_scatter_rec(ctx, d_R.ptr, rLen, (const int32_t *)d_loc.ptr, 1, d_S.ptr, sLen), "scatterImpl",
           ctx))
        ok(qg_ctx_check(ctx), "scatterImpl", ctx);
}

// host/host/testSplit.cpp:156-209: d_S gets the records grouped by partition
// (stable; partition id = y mod numPart), d_bound the first row of each
// partition.  SPLIT_TYPE chose the reference's (unshipped) map kernel and is
// accepted and ignored.
QG_API void splitImpl(qg_buf d_R, int rLen, int numPart, qg_buf d_S, qg_buf d_bound, int numThreadPB,
                      int numBlock, int SPLIT_TYPE, qg_ctx *ctx) {
    (void)numThreadPB;
    (void)numBlock;
    (void)SPLIT_TYPE;
    ctx = pick(ctx);
    ok(qg_split_rec(ctx, d_R.ptr, rLen, numPart, d_S.ptr, (int32_t *)d_bound.ptr), "splitImpl", ctx);
}

}  // extern "C"
