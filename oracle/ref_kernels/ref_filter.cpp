// The reference's filter chain on host cores: its own kernels from
// kernel/filter/filter_op.cl (compiled through clshim.h), driven the way
// host/host/testFilter.cpp:92-154 (filterImpl) drives them.  Test
// infrastructure only.
#include <vector>

#include "ref_scan.h"

namespace rf {
#include REF_FILTER_CL
}

extern "C" {

// filterImpl: map (numThread x numBlock work-items, testFilter.cpp:27-50),
// exclusive scan of the marks (testScan.cpp:242-334), outSize (one work-item,
// :51-72), write (:73-89).  n must be 2^k, 17 <= k <= 24 (the reference
// scan's own limits).  Returns 0, or -1 when n is outside those limits.
int ref_filter_rec(const uint2 *in, int n, int lo, int hi, int numThread, int numBlock, uint2 *out, int *out_n) {
    std::vector<int> mark((size_t)n), markOut((size_t)n), temp((size_t)n);
    uint2 *rin = const_cast<uint2 *>(in);
    clshim::launch((size_t)numThread * numBlock, (size_t)numThread,
                   [&] { rf::filterImpl_map_kernel(rin, 0, n, mark.data(), lo, hi, temp.data()); });
    const int st = refscan::scan(
        mark.data(), n, markOut.data(),
        [&](unsigned len, int *i, int *o, int *bs) {
            clshim::launch(len / 2, 128, [&] { rf::ScanLargeArrays_kernel(o, i, 256u, len, bs); });
        },
        [&](unsigned len, int *i, int *o) {
            clshim::launch(len / 2, len / 2, [&] { rf::prefixSum_kernel(o, i, len); });
        },
        [&](unsigned len, int *i, int *o) {
            clshim::launch(len, 256, [&] { rf::blockAddition_kernel(i, o); });
        });
    if (st != 0) return st;
    int outSize = 0;
    clshim::launch(1, 1, [&] { rf::filterImpl_outSize_kernel(&outSize, mark.data(), markOut.data(), n); });
    clshim::launch((size_t)numThread * numBlock, (size_t)numThread,
                   [&] { rf::filterImpl_write_kernel(out, rin, mark.data(), markOut.data(), 0, n); });
    *out_n = outSize;
    return 0;
}

// The reference's exclusive scan alone (scanImpl over its filter program).
int ref_scan(const int *in, int n, int *out) {
    std::vector<int> src(in, in + n);
    return refscan::scan(
        src.data(), n, out,
        [&](unsigned len, int *i, int *o, int *bs) {
            clshim::launch(len / 2, 128, [&] { rf::ScanLargeArrays_kernel(o, i, 256u, len, bs); });
        },
        [&](unsigned len, int *i, int *o) {
            clshim::launch(len / 2, len / 2, [&] { rf::prefixSum_kernel(o, i, len); });
        },
        [&](unsigned len, int *i, int *o) {
            clshim::launch(len, 256, [&] { rf::blockAddition_kernel(i, o); });
        });
}

}  // extern "C"
