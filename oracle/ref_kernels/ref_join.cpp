// The reference's hash join on host cores: buildHashTable and
// probeHashTable from kernel/hj_filter_sort/1/hj_filter_sort_op.cl (compiled
// through clshim.h).  The reference ships no host code for them; the launch
// follows the kernels' own attributes: reqd_work_group_size(128) for both and
// num_compute_units(1) for the build, i.e. one work-group of 128 items.
// Test infrastructure only.
#include <vector>

#include "clshim.h"

namespace rj {
#include REF_JOIN_CL
}

extern "C" {

// R and S hold interleaved (key, value) uints.  The build's table has
// bucketNum buckets (a power of two; bucket = key & (bucketNum - 1)) of
// bucketSize slots; the kernel has no overflow check, so the caller passes a
// bucketSize no smaller than the fullest bucket.  The probe runs probeGroups
// work-groups of 128 and writes each match (S.value, R.value) at
// gid * unit_size + its own counter, unit_size = 2 * nS / global size
// (hj_filter_sort_op.cl:73,101-104), leaving holes; slots are pre-set to
// 0xffffffff and the matches are returned compacted in slot order.  nS must
// be a multiple of 128 * probeGroups, and every S row may match at most
// unit_size / 2 R rows (so that no item writes past its own slots).
int ref_hash_join(const uint *R, int nR, const uint *S, int nS, int bucketNum, int bucketSize, int probeGroups,
                  uint *pairs, int *npairs) {
    if (bucketNum <= 0 || (bucketNum & (bucketNum - 1)) || probeGroups <= 0 || nS % (128 * probeGroups)) return -1;
    std::vector<uint> table((size_t)bucketNum * bucketSize * 2, 0), count((size_t)bucketNum, 0);
    std::vector<uint> matched((size_t)2 * nS, 0xffffffffu);
    uint *r = const_cast<uint *>(R), *s = const_cast<uint *>(S);
    clshim::launch(128, 128, [&] {
        rj::buildHashTable(r, table.data(), (uint)nR, (uint)bucketNum, (uint)bucketSize, count.data());
    });
    clshim::launch((size_t)128 * probeGroups, 128, [&] {
        rj::probeHashTable(table.data(), s, matched.data(), (uint)nS, (uint)bucketNum, (uint)bucketSize, count.data());
    });
    int m = 0;
    for (size_t i = 0; i + 1 < matched.size(); i += 2) {
        if (matched[i] == 0xffffffffu && matched[i + 1] == 0xffffffffu) continue;
        pairs[2 * m] = matched[i];
        pairs[2 * m + 1] = matched[i + 1];
        m++;
    }
    *npairs = m;
    return 0;
}

}  // extern "C"
