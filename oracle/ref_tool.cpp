// ref_tool.cpp -- command-line harness around the reference's own CPU code.
//
// TEST INFRASTRUCTURE ONLY (oracle pin).  oracle/build_ref.sh compiles this
// file together with the reference's host/host/generator.cpp,
// host/host/Validate.cpp and host/dynamic_programming.cpp, read where they
// lie in the reference checkout, into oracle/_ref/ref_tool.  The tests and
// tests/golden/make_golden.py run it as a subprocess: the reference
// validators print a verdict and call exit() on a mismatch, so each check is
// one process.  Records are uint2 {x, y} (host/host/common.h:27-28), stored
// little-endian as raw binary files.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <vector>
#include "common.h"

// The reference links these from src/AOCL_Utils.cpp, which needs a real
// OpenCL runtime; the pinned sources only use the two allocation helpers.
namespace aocl_utils {
void *alignedMalloc(size_t size) {
    void *p = nullptr;
    if (posix_memalign(&p, 64, size ? size : 64) != 0) return nullptr;
    return p;
}
void alignedFree(void *ptr) { free(ptr); }
}  // namespace aocl_utils

// host/host/generator.cpp
extern void generateRand(Record *R, int maxmax, int rLen, int seed);
extern void generateRandInt(int *R, int max, int rLen, int seed);
// host/host/Validate.cpp
extern void validateScan(int *input, int rLen, int *output);
extern void validateFilter(Record *h_Rin, int beginPos, int rLen, Record *h_Rout, int outSize,
                           int smallKey, int largeKey);
extern void validateSort(Record *h_Rin, int rLen);
extern void validateGroupBy(Record *h_Rin, int rLen, Record *h_Rout, int *h_startPos, int numGroup);
extern void validateAggAfterGroupBy(Record *h_Rin, int rLen, int *startPos, int numGroups,
                                    Record *Ragg, int *aggResults, int OPERATOR);
extern void validateAggAfterGroupBy_easy(Record *h_Rin, int rLen, int *startPos, int numGroups,
                                         int *aggResults, int OPERATOR);
// host/dynamic_programming.cpp
extern void dp_test(int sub_index, float size);

template <typename T>
static std::vector<T> load(const char *path, size_t count) {
    std::vector<T> v(count ? count : 1);
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    size_t got = fread(v.data(), sizeof(T), count, f);
    fclose(f);
    if (got != count) { fprintf(stderr, "short read %s\n", path); exit(2); }
    return v;
}

template <typename T>
static void save(const char *path, const T *p, size_t count) {
    FILE *f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    fwrite(p, sizeof(T), count, f);
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_tool <cmd> ...\n"); return 2; }
    std::string cmd = argv[1];
    if (cmd == "gen_rand" && argc == 6) {  // maxmax n seed out
        int maxmax = atoi(argv[2]), n = atoi(argv[3]), seed = atoi(argv[4]);
        std::vector<Record> r(n ? n : 1);
        generateRand(r.data(), maxmax, n, seed);
        save(argv[5], r.data(), (size_t)n);
        // testFilterImpl draws smallKey = rand() % 100 from the same stream
        // right after generateRand (host/host/testFilter.cpp:212-215).
        printf("next_rand=%d\n", rand());
        return 0;
    }
    if (cmd == "gen_rand_int" && argc == 6) {  // max n seed out
        int mx = atoi(argv[2]), n = atoi(argv[3]), seed = atoi(argv[4]);
        std::vector<int> r(n ? n : 1);
        generateRandInt(r.data(), mx, n, seed);
        save(argv[5], r.data(), (size_t)n);
        return 0;
    }
    if (cmd == "validate_filter" && argc == 8) {  // in n out outSize small large
        int n = atoi(argv[3]), outSize = atoi(argv[5]);
        auto in = load<Record>(argv[2], n);
        auto out = load<Record>(argv[4], outSize);
        validateFilter(in.data(), 0, n, out.data(), outSize, atoi(argv[6]), atoi(argv[7]));
        return 0;
    }
    if (cmd == "validate_scan" && argc == 5) {  // in n out
        int n = atoi(argv[3]);
        auto in = load<int>(argv[2], n);
        auto out = load<int>(argv[4], n);
        validateScan(in.data(), n, out.data());
        return 0;
    }
    if (cmd == "validate_sort" && argc == 4) {  // rec n
        int n = atoi(argv[3]);
        auto r = load<Record>(argv[2], n);
        validateSort(r.data(), n);
        return 0;
    }
    if (cmd == "validate_groupby" && argc == 7) {  // in n sorted startPos numGroups
        int n = atoi(argv[3]), g = atoi(argv[6]);
        auto in = load<Record>(argv[2], n);
        auto srt = load<Record>(argv[4], n);
        auto sp = load<int>(argv[5], g);
        validateGroupBy(in.data(), n, srt.data(), sp.data(), g);
        return 0;
    }
    if (cmd == "validate_agg_easy" && argc == 8) {  // sorted n startPos numGroups agg op
        int n = atoi(argv[3]), g = atoi(argv[5]);
        auto srt = load<Record>(argv[2], n);
        auto sp = load<int>(argv[4], g);
        auto agg = load<int>(argv[6], g);
        validateAggAfterGroupBy_easy(srt.data(), n, sp.data(), g, agg.data(), atoi(argv[7]));
        return 0;
    }
    if (cmd == "validate_agg" && argc == 9) {  // rin n startPos numGroups ragg agg op
        int n = atoi(argv[3]), g = atoi(argv[5]);
        auto rin = load<Record>(argv[2], n);
        auto sp = load<int>(argv[4], g);
        auto ragg = load<Record>(argv[6], n);
        auto agg = load<int>(argv[7], g);
        validateAggAfterGroupBy(rin.data(), n, sp.data(), g, ragg.data(), agg.data(), atoi(argv[8]));
        return 0;
    }
    if (cmd == "dp" && argc == 4) {  // sub_index size(M)
        dp_test(atoi(argv[2]), (float)atof(argv[3]));
        return 0;
    }
    fprintf(stderr, "bad command\n");
    return 2;
}
