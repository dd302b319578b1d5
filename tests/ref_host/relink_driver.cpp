// A host program written against the reference's operator API, the way the
// reference's own drivers call it (host/host/testFilter.cpp:197-232 for the
// filter, host/host/testAggAfterGB.cpp:127-193 for group-by + aggregation),
// compiled against include/qg_ref.h and linked with -lqg in place of the
// OpenCL host library.  Device buffers move with cudaMemcpy where the
// reference used clEnqueueWriteBuffer / clEnqueueReadBuffer.
//
//   relink_driver FILTER_IN GROUP_IN OUT_DIR SMALL LARGE
//
// FILTER_IN and GROUP_IN hold an int32 count n followed by n Records {x, y}.
// OUT_DIR receives sel.bin (CL_RangeSelection), filt.bin (filterImpl),
// sorted.bin and startpos.bin (groupByImpl) and agg0.bin .. agg3.bin
// (parallelAggregate_init with REDUCE_SUM / MAX / MIN / AVERAGE, in chunks of
// 512 groups as the reference's driver launches them); each file is an int32
// count followed by the data.  The exit status is 0 when every call reported
// QG_OK, else the number of the first failing step.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "qg_ref.h"

static std::vector<qg_record> read_records(const char *path) {
    std::vector<qg_record> r;
    FILE *f = std::fopen(path, "rb");
    if (!f) return r;
    int32_t n = 0;
    if (std::fread(&n, 4, 1, f) == 1 && n > 0) {
        r.resize((size_t)n);
        if (std::fread(r.data(), sizeof(qg_record), (size_t)n, f) != (size_t)n) r.clear();
    }
    std::fclose(f);
    return r;
}

static bool write_ints(const std::string &path, const void *data, int32_t count, size_t elem_bytes) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    bool ok = std::fwrite(&count, 4, 1, f) == 1;
    if (ok && count > 0) ok = std::fwrite(data, elem_bytes, (size_t)count, f) == (size_t)count;
    return std::fclose(f) == 0 && ok;
}

int main(int argc, char **argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s FILTER_IN GROUP_IN OUT_DIR SMALL LARGE\n", argv[0]);
        return 100;
    }
    const std::string out = argv[3];
    const int smallKey = std::atoi(argv[4]), largeKey = std::atoi(argv[5]);
    std::vector<qg_record> rin = read_records(argv[1]), gin = read_records(argv[2]);
    if (rin.empty() || gin.empty()) return 101;
    const int rLen = (int)rin.size(), gLen = (int)gin.size();
    const int numThread = 256, numBlock = 512;

    // 1. CL_RangeSelection: host in, host out (testFilter.cpp:197-232)
    qg_record *h_Rout = nullptr;
    const int sel = CL_RangeSelection(rin.data(), rLen, smallKey, largeKey, &h_Rout, numThread, numBlock, 0);
    if (qg_ref_last_status() != QG_OK || sel < 0) return 1;
    if (!write_ints(out + "/sel.bin", h_Rout, sel, sizeof(qg_record))) return 90;
    std::free(h_Rout);

    // 2. filterImpl on a device buffer; the callee allocates *d_Rout
    qg_buf d_Rin{nullptr, 0}, d_Rout{nullptr, 0};
    if (qg_buf_alloc(&d_Rin, (size_t)rLen * sizeof(qg_record)) != QG_OK) return 2;
    if (cudaMemcpy(d_Rin.ptr, rin.data(), d_Rin.bytes, cudaMemcpyHostToDevice) != cudaSuccess) return 2;
    int outSize = 0;
    filterImpl(d_Rin, 0, rLen, &d_Rout, &outSize, numThread, numBlock, smallKey, largeKey, nullptr);
    if (qg_ref_last_status() != QG_OK) return 2;
    std::vector<qg_record> filt((size_t)outSize);
    if (outSize > 0 &&
        cudaMemcpy(filt.data(), d_Rout.ptr, (size_t)outSize * sizeof(qg_record), cudaMemcpyDeviceToHost) != cudaSuccess)
        return 2;
    if (!write_ints(out + "/filt.bin", filt.data(), outSize, sizeof(qg_record))) return 90;
    qg_buf_free(&d_Rout);
    qg_buf_free(&d_Rin);

    // 3. groupByImpl with the same buffer as input and output (testAggAfterGB.cpp:161)
    qg_buf d_R{nullptr, 0}, d_startPos{nullptr, 0};
    if (qg_buf_alloc(&d_R, (size_t)gLen * sizeof(qg_record)) != QG_OK) return 3;
    if (cudaMemcpy(d_R.ptr, gin.data(), d_R.bytes, cudaMemcpyHostToDevice) != cudaSuccess) return 3;
    const int numGroups = groupByImpl(d_R, gLen, d_R, &d_startPos, numThread, numBlock, nullptr);
    if (qg_ref_last_status() != QG_OK || numGroups < 0) return 3;
    std::vector<qg_record> sorted((size_t)gLen);
    std::vector<int32_t> startPos((size_t)numGroups);
    if (cudaMemcpy(sorted.data(), d_R.ptr, d_R.bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    if (numGroups > 0 &&
        cudaMemcpy(startPos.data(), d_startPos.ptr, (size_t)numGroups * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return 3;
    if (!write_ints(out + "/sorted.bin", sorted.data(), gLen, sizeof(qg_record))) return 90;
    if (!write_ints(out + "/startpos.bin", startPos.data(), numGroups, 4)) return 90;

    // 4. parallelAggregate_init per operator, 512 groups per launch
    //    (testAggAfterGB.cpp:101-120: MAX_NUM_BLOCK = 512)
    qg_buf d_agg{nullptr, 0};
    if (qg_buf_alloc(&d_agg, (size_t)(numGroups > 0 ? numGroups : 1) * 4) != QG_OK) return 4;
    const int MAX_NUM_BLOCK = 512;
    for (int op = 0; op < 4; op++) {
        for (int off = 0; off < numGroups; off += MAX_NUM_BLOCK) {
            const int nb = numGroups - off < MAX_NUM_BLOCK ? numGroups - off : MAX_NUM_BLOCK;
            parallelAggregate_init(d_R, d_startPos, d_agg, op, off, numGroups, nb, numThread, 0, gLen, nullptr);
            if (qg_ref_last_status() != QG_OK) return 5 + op;
        }
        std::vector<int32_t> agg((size_t)numGroups);
        if (numGroups > 0 &&
            cudaMemcpy(agg.data(), d_agg.ptr, (size_t)numGroups * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return 5 + op;
        if (!write_ints(out + "/agg" + std::to_string(op) + ".bin", agg.data(), numGroups, 4)) return 90;
    }
    qg_buf_free(&d_agg);
    qg_buf_free(&d_startPos);
    qg_buf_free(&d_R);
    return 0;
}
