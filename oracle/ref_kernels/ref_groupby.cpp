// The reference's sort, group-by and aggregation on host cores: its own
// kernels from kernel/aggregation/1/group_by_cu_op_dp.cl (compiled through
// clshim.h), driven the way host/host/testSort.cpp:24-136 (radixSortImpl_sm),
// testGroupBy.cpp:81-154 (groupByImpl) and testAggAfterGB.cpp:127-193
// (testAggAfterGroupByImpl) drive them.  Test infrastructure only.
#include <vector>

#include "ref_scan.h"

namespace rg {
#include REF_GROUPBY_CL
}

namespace {

int scan(int *src, int n, int *dst) {
    return refscan::scan(
        src, n, dst,
        [&](unsigned len, int *i, int *o, int *bs) {
            clshim::launch(len / 2, 128, [&] { rg::ScanLargeArrays_kernel(o, i, 256u, len, bs); });
        },
        [&](unsigned len, int *i, int *o) {
            clshim::launch(len / 2, len / 2, [&] { rg::prefixSum_kernel(o, i, len); });
        },
        [&](unsigned len, int *i, int *o) {
            clshim::launch(len, 256, [&] { rg::blockAddition_kernel(i, o); });
        });
}

}  // namespace

extern "C" {

// radixSortImpl_sm (testSort.cpp:24-136): a shared-memory bitonic sort of
// tiles of SHARED_SIZE_LIMIT records, then for each larger size global merge
// steps (three strides per launch) down to the tile size and a shared-memory
// merge of the rest.  Ascending by .y (unsigned); n a power of two >= 2048.
int ref_sort_rec(uint2 *d, int n) {
    if (n < 2 * SHARED_SIZE_LIMIT || (n & (n - 1))) return -1;
    const unsigned rLen = (unsigned)n;
    const unsigned threadCount = SHARED_SIZE_LIMIT / 2;
    clshim::launch(rLen / 2, threadCount,
                   [&] { rg::bitonicSortShared(d, rLen, 2u, (unsigned)SHARED_SIZE_LIMIT, 0u, 0u, (unsigned)SHARED_SIZE_LIMIT); });
    int log_rLen = -1;
    for (int m = n; m; m >>= 1) log_rLen++;
    const unsigned dir = 1;
    for (unsigned size = 2 * SHARED_SIZE_LIMIT, log_size = 11; (int)log_size <= log_rLen; size <<= 1, log_size++) {
        for (unsigned stride = size / 2, log_stride = log_size - 1; stride > 0; stride >>= 3, log_stride -= 3) {
            if (stride >= SHARED_SIZE_LIMIT) {
                clshim::launch(rLen / 8, 256, [&] { rg::bitonicMergeGlobal(d, rLen, log_size, log_stride, dir); });
            } else {
                clshim::launch(rLen / 2, threadCount, [&] {
                    rg::bitonicSortShared(d, rLen, (unsigned)SHARED_SIZE_LIMIT, (unsigned)SHARED_SIZE_LIMIT, dir, 1u, size);
                });
                break;
            }
        }
    }
    return 0;
}

// groupByImpl: sort in place, group labels (numThread x numBlock
// work-items), exclusive scan, numGroups (one work-item), startPos.
// sorted receives the sorted records (in may equal sorted); startPos holds n.
int ref_groupby_rec(const uint2 *in, int n, int numThread, int numBlock, uint2 *sorted, int *startPos,
                    int *numGroups) {
    if (sorted != in)
        for (int i = 0; i < n; i++) sorted[i] = in[i];
    int st = ref_sort_rec(sorted, n);
    if (st != 0) return st;
    std::vector<int> label((size_t)n), writePos((size_t)n);
    clshim::launch((size_t)numThread * numBlock, (size_t)numThread,
                   [&] { rg::scanGroupLabel_kernel(sorted, n, label.data()); });
    st = scan(label.data(), n, writePos.data());
    if (st != 0) return st;
    int g = 0;
    clshim::launch(1, 1, [&] { rg::groupByImpl_outSize_kernel(&g, label.data(), writePos.data(), n); });
    clshim::launch((size_t)numThread * numBlock, (size_t)numThread,
                   [&] { rg::groupByImpl_write_kernel(startPos, label.data(), writePos.data(), n); });
    *numGroups = g;
    return 0;
}

// parallelAggregate over sorted records, in chunks of MAX_NUM_BLOCK = 512
// groups (testAggAfterGB.cpp:37,170-190), numThread work-items per group and
// sizeof(int) * numThread ints of local memory (the host passes
// sharedMemSize * sizeof(cl_int) bytes, testAggAfterGB.cpp:83).
int ref_aggregate(const uint2 *sorted, int n, const int *startPos, int numGroups, int op, int numThread, int *agg) {
    const int maxBlock = 512;
    const int numChunk = (numGroups + maxBlock - 1) / maxBlock;
    const int sharedInts = (int)sizeof(int) * numThread;
    uint2 *s = const_cast<uint2 *>(sorted);
    int *sp = const_cast<int *>(startPos);
    for (int c = 0; c < numChunk; c++) {
        const int blockOffset = c * maxBlock;
        const int numBlock = c == numChunk - 1 ? numGroups - c * maxBlock : maxBlock;
        clshim::launch((size_t)numThread * numBlock, (size_t)numThread, [&] {
            static thread_local std::vector<int> local;
            if ((int)local.size() < sharedInts) local.assign((size_t)sharedInts, 0);
            rg::parallelAggregate_kernel(s, sp, agg, op, blockOffset, numGroups, n, local.data());
        });
    }
    return 0;
}

}  // extern "C"
