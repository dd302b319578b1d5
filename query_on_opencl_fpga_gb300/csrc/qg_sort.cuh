// qg_sort.cuh -- radix sort building blocks shared by group-by and join.
#pragma once
#include "qg_internal.cuh"

constexpr int QG_RADIX = 256;

// Buffers of one side of the ping-pong: REC uses `rec` (u64 items, key in the
// high word); KV3 uses the three u32 columns k (key), a, b.
// REC items may carry a sidecar of 16-bit bucket ids (bid, aligned with rec):
// a pass whose source has one takes its digits from it instead of computing
// them, and writes the reordered ids to the destination's sidecar if that has
// one (a learned partition function is then evaluated once per row, not once
// per pass).
struct qg_sort_bufs {
    unsigned long long *rec;
    uint32_t *k;
    uint32_t *a;
    uint32_t *b;
    uint16_t *bid;
};

// Number of 8-bit digit positions covering `bits` key bits (1..4).
int qg_sort_positions(int bits);
// Device histogram of (key - key_off) digits for `npos` positions into
// d_hist[4][256]; for records, `copy` (if set) also receives a copy of them.
qg_status qg_radix_histogram(qg_ctx *ctx, const qg_sort_bufs &src, bool kv3, long long n,
                             uint32_t key_off, int npos, uint32_t *d_hist,
                             unsigned long long *copy = nullptr);
// From a host copy of the histogram: the non-trivial positions (returned
// count) and every position's exclusive digit bases.
int qg_sort_plan(const uint32_t *h_hist, int npos, long long n, int *passes, uint32_t *bases);
// Run the planned passes, starting in `a` and alternating; *result_in_b tells
// where the sorted data ended.
qg_status qg_radix_passes(qg_ctx *ctx, bool kv3, qg_sort_bufs a, qg_sort_bufs b, long long n,
                          uint32_t key_off, const int *passes, int np, const uint32_t *h_bases,
                          bool *result_in_b);
// Same, with the digits taken from a partition function: pass position p
// sorts by bits [8p, 8p + 8) of the bucket (radix form: of (k - kmin) >> shift).
// first_unstable: the caller needs the items grouped by bucket only, not in
// input order within a bucket, so the first pass ranks with shared-memory
// atomics instead of stable warp ballots (REC items only).
struct qg_part_fn;
qg_status qg_radix_passes_pf(qg_ctx *ctx, bool kv3, qg_sort_bufs a, qg_sort_bufs b, long long n,
                             const qg_part_fn &pf, const int *passes, int np, const uint32_t *h_bases,
                             bool *result_in_b, bool first_unstable = false);
// Passes planned on the device, for sequences without host round trips
// (CUDA graph capture): all `npos` positions from the device histogram d_hist
// [npos][256] of (key - key_off) digits, over at most n_bound items whose real
// count is *d_n.  work: qg_radix_dev_work_bytes(n_bound) bytes of device memory.
qg_status qg_radix_passes_dev(qg_ctx *ctx, bool kv3, qg_sort_bufs a, qg_sort_bufs b, long long n_bound,
                              const unsigned long long *d_n, const uint32_t *d_hist, int npos, uint32_t key_off,
                              char *work, bool *result_in_b);
size_t qg_radix_dev_work_bytes(long long n_bound);
// Sort REC items in place with `tmp` as the second buffer (synchronises once).
qg_status qg_sort_rec_inplace(qg_ctx *ctx, unsigned long long *data, unsigned long long *tmp,
                              long long n);
