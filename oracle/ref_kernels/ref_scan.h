// The reference's host orchestration of its exclusive scan, restated over the
// reference's own scan kernels (test infrastructure; see clshim.h).
//
// host/host/testScan.cpp:26-83 initScan, :86-227 bScan_int / pScan_int /
// bAddition_int and :242-334 scanImpl (with REDUCE_MEM_COPY defined):
//   pass = floor(log(n) / log(256)) in fp32, one less when that is exact;
//   block scans of 256 elements (work-groups of 128) down the levels, one
//   prefixSum over the last level's block sums (a single work-group of
//   tempLength / 2 items), then block additions back up to the output.
// The reference needs pass >= 2 (for pass == 1 it reads outputBuffer[1],
// which initScan never creates, testScan.cpp:317-318) and a length that the
// block sizes divide; the driver accepts n = 2^k with 17 <= k <= 24 only.
#pragma once
#include <cmath>
#include <vector>

#include "clshim.h"

namespace refscan {

// bscan(len, in, out, blocksum), pscan(len, in, out), badd(len, in, out)
// launch the three kernels with the reference's global / local sizes.
template <class BScan, class PScan, class BAdd>
inline int scan(int *src, int n, int *dst, BScan bscan, PScan pscan, BAdd badd) {
    const int blockSize = 256;
    const float t = std::log((float)n) / std::log((float)blockSize);
    int pass = (int)t;
    if (std::fabs(t - (float)pass) < 1e-7f) pass--;
    if (pass < 2) return -1;
    std::vector<std::vector<int>> output(pass), blockSum(pass);
    for (int i = 0; i < pass; i++) {
        output[i].assign((size_t)(n / std::pow((float)blockSize, (float)i)), 0);
        blockSum[i].assign((size_t)(n / std::pow((float)blockSize, (float)(i + 1))), 0);
    }
    const int tempLength = (int)(n / std::pow((float)blockSize, (float)pass));
    std::vector<int> temp((size_t)tempLength, 0);

    bscan((unsigned)n, src, dst, blockSum[0].data());
    for (int i = 1; i < pass; i++)
        bscan((unsigned)(n / std::pow((float)blockSize, (float)i)), blockSum[i - 1].data(), output[i].data(),
              blockSum[i].data());
    pscan((unsigned)tempLength, blockSum[pass - 1].data(), temp.data());
    badd((unsigned)(n / std::pow((float)blockSize, (float)(pass - 1))), temp.data(), output[pass - 1].data());
    for (int i = pass - 1; i > 1; i--)
        badd((unsigned)(n / std::pow((float)blockSize, (float)(i - 1))), output[i].data(), output[i - 1].data());
    badd((unsigned)n, output[1].data(), dst);
    return 0;
}

}  // namespace refscan
