/*
 * qg_ref.h -- the reference's operator surface (the host/host headers of
 * Xtra-Computing/Query_on_OpenCL_FPGA) over libqg.so.
 *
 * Same function names, argument order and meaning as the reference, so a
 * caller of the reference's host API switches by relinking.  Differences,
 * all forced by leaving OpenCL and the FPGA behind:
 *   - cl_mem becomes qg_buf (device pointer + bytes); callee-allocated
 *     buffers (filterImpl's *d_Rout, groupByImpl's *d_startPos) are freed
 *     with qg_buf_free.
 *   - The OpenCL scheduling tail (int *index, cl_event *eventList,
 *     cl_kernel *Kernel, int *Flag_CPU_GPU, double *burden, int _CPU_GPU)
 *     becomes one qg_ctx * (NULL = a process-wide default context on the
 *     current device).  The CL_* wrappers keep their trailing int _CPU_GPU,
 *     which selected the second FPGA image and is ignored here.
 *   - numThread / numBlock / sharedMemSize were work-group shapes for the FPGA
 *     images; they are accepted and ignored (launch shapes are the library's).
 *   - Errors: the reference prints and calls exit() (src/AOCL_Utils.cpp:
 *     228-252).  Here nothing exits: the failing call prints one line to
 *     stderr, count-returning calls return -1, and qg_ref_last_status()
 *     gives the status of the last call.
 *   - Sizes the reference cannot handle (scan with n <= 65536, sort with n
 *     not a power of two >= 2048) work here.
 */
#ifndef QG_REF_H
#define QG_REF_H
#include <stddef.h>
#include <stdint.h>
#include "qg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    void *ptr;     /* device pointer */
    size_t bytes;  /* size of the allocation */
} qg_buf;

typedef struct {
    uint32_t x, y; /* Record = uint2 (host/host/common.h:27-28): y key, x payload */
} qg_record;

/* Scan bookkeeping kept for source compatibility (host/host/testScan.h:4-12);
 * the single-pass scan needs no per-level buffers. */
typedef struct {
    uint32_t pass;
    uint32_t gLength;
    uint32_t blockSize;
} ScanPara;

QG_API qg_status qg_ref_last_status(void);
QG_API qg_ctx *qg_ref_default_ctx(void);
QG_API qg_status qg_buf_alloc(qg_buf *b, size_t bytes);
QG_API void qg_buf_free(qg_buf *b);

/* host/host/testFilter.h:4-5 (testFilter.cpp:92-154) */
QG_API void filterImpl(qg_buf d_Rin, int beginPos, int rLen, qg_buf *d_Rout, int *outSize,
                       int numThread, int numBlock, int smallKey, int largeKey, qg_ctx *ctx);
/* host/host/Selection.cpp:6-16 */
QG_API int range_selection(qg_buf d_Rin, int rLen, int rangeSmallKey, int rangeLargeKey,
                           qg_buf *d_Rout, int numThreadPB, int numBlock, qg_ctx *ctx);
/* host/host/Selection.cpp:19-50: host in, host out (*h_Rout malloc'ed, caller frees) */
QG_API int CL_RangeSelection(qg_record *h_Rin, int rLen, int rangeSmallKey, int rangeLargeKey,
                             qg_record **h_Rout, int numThreadPB, int numBlock, int _CPU_GPU);

/* host/host/testScan.h:14-18 (testScan.cpp:26-340) */
QG_API void initScan(int rLen, ScanPara *SP);
QG_API void scanImpl(qg_buf d_Src, int rLen, qg_buf d_Dst, ScanPara *SP, qg_ctx *ctx);
QG_API void closeScan(ScanPara *SP);

/* host/host/testSort.cpp:24 and Sort.cpp:34 */
QG_API void radixSortImpl_sm(qg_buf d_R, int rLen, int meaningless, int numThreadPB, int numBlock,
                             qg_ctx *ctx);
QG_API void CL_RadixSort(qg_record *h_Rin, int rLen, qg_record *h_Rout, int numThread,
                         int numBlock, int _CPU_GPU);

/* host/host/testGroupBy.h:5 (testGroupBy.cpp:81-154): sorts d_Rin into
 * d_Rout (d_Rout may be d_Rin, as the reference's drivers pass), allocates
 * *d_startPos, returns numGroups.  The reference sorts d_Rout in place and
 * never reads d_Rin (its copy is commented out, testGroupBy.cpp:89), so its
 * CL_GroupBy sorts an uninitialised buffer; here d_Rin is the input. */
QG_API int groupByImpl(qg_buf d_Rin, int rLen, qg_buf d_Rout, qg_buf *d_startPos, int numThread,
                       int numBlock, qg_ctx *ctx);
/* host/host/GroupBy.cpp:7-45: *h_startPos malloc'ed, caller frees */
QG_API int CL_GroupBy(qg_record *h_Rin, int rLen, qg_record *h_Rout, int **h_startPos,
                      int numThread, int numBlock, int _CPU_GPU);

/* host/host/testAggAfterGB.cpp:69-91: groups [blockOffset, blockOffset+numBlock)
 * of numGroups, aggregating .x of d_S; d_aggResults indexed by group number. */
QG_API void parallelAggregate_init(qg_buf d_S, qg_buf d_startPos, qg_buf d_aggResults,
                                   int OPERATOR, int blockOffset, int numGroups, int numBlock,
                                   int numThread, int sharedMemSize, int rLen, qg_ctx *ctx);
/* host/host/testAggAfterGB.cpp:92-123: S[i] = d_Ragg[d_Rin[i].x] (gather), then
 * OPERATOR over S[.].x per group (one launch for all groups). */
QG_API void aggAfterGroupByImpl(qg_buf d_Rin, int rLen, qg_buf d_startPos, int numGroups,
                                qg_buf d_Ragg, qg_buf d_aggResults, int OPERATOR, int numThread,
                                qg_ctx *ctx);
/* host/host/AggAfterGroupBy.cpp:30-170 */
QG_API void CL_agg_max_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread,
                                    int _CPU_GPU);
QG_API void CL_agg_min_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread,
                                    int _CPU_GPU);
QG_API void CL_agg_sum_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread,
                                    int _CPU_GPU);
QG_API void CL_agg_avg_afterGroupBy(qg_record *h_Rin, int rLen, int *h_startPos, int numGroups,
                                    qg_record *h_Ragg, int *h_aggResults, int numThread,
                                    int _CPU_GPU);

/* host/host/testScatter.h:2-5 (testScatter.cpp:63-137) */
QG_API void gatherImpl(qg_buf d_R, int rLen, qg_buf d_loc, qg_buf d_S, int sLen, int numThreadPB,
                       int numBlock, qg_ctx *ctx);
QG_API void scatterImpl(qg_buf d_R, int rLen, qg_buf d_loc, qg_buf d_S, int numThreadPB,
                        int numBlock, qg_ctx *ctx);

/* host/host/testSplit.cpp:156-209 (its kernels are not shipped): records
 * grouped by partition id y mod numPart, stable; d_bound[p] = first row of p. */
QG_API void splitImpl(qg_buf d_R, int rLen, int numPart, qg_buf d_S, qg_buf d_bound, int numThreadPB,
                      int numBlock, int SPLIT_TYPE, qg_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* QG_REF_H */
