/*
 * qg.h -- C ABI of the GB300-native relational-operator library (libqg.so).
 *
 * Plain pointers and sizes only.  All data pointers are DEVICE pointers unless
 * a parameter says "host".  Every entry point returns a qg_status; none calls
 * exit().  Work is enqueued on the context's CUDA stream; entry points whose
 * result count is returned through a host pointer synchronise that stream,
 * the "_async" forms write the count to a device int64 instead.
 *
 * Record layout follows the reference: Record = uint2 {x, y}, y = key,
 * x = payload / row id (host/host/common.h:27-28).  Range predicates are
 * inclusive and signed, as in filterImpl_map_kernel
 * (kernel/filter/filter_op.cl:19-21).
 */
#ifndef QG_H
#define QG_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QG_API __attribute__((visibility("default")))

typedef enum {
    QG_OK = 0,
    QG_ERR_INVALID = 1,     /* bad argument (null pointer, negative size, misalignment) */
    QG_ERR_CUDA = 2,        /* a CUDA runtime call failed; see qg_last_error_message */
    QG_ERR_CAPACITY = 3,    /* output larger than the capacity given; *out_n holds the size needed */
    QG_ERR_TABLE_FULL = 4,  /* hash table probe gave up (more distinct keys than the table holds) */
    QG_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up (look-back or pipeline barrier) */
    QG_ERR_OOM = 6,         /* device scratch allocation failed */
    QG_ERR_UNSUPPORTED = 7  /* size or option outside what the operator supports */
} qg_status;

/* Aggregation operators, same numbering as the reference (host/host/common.h:89-92). */
enum { QG_REDUCE_SUM = 0, QG_REDUCE_MAX = 1, QG_REDUCE_MIN = 2, QG_REDUCE_AVERAGE = 3 };

/* Output order of the column group-by. */
enum { QG_ORDER_NONE = 0, QG_ORDER_KEY = 1 };

typedef struct qg_ctx qg_ctx;

/* ---- context --------------------------------------------------------- */
/* One context per host thread of use; separate contexts are independent.
 * `stream` is a cudaStream_t (NULL = the legacy default stream).  The device
 * is the one current on the calling thread. */
QG_API qg_status qg_ctx_create(qg_ctx **out, void *stream);
QG_API qg_status qg_ctx_destroy(qg_ctx *ctx);
QG_API qg_status qg_ctx_set_stream(qg_ctx *ctx, void *stream);
QG_API qg_status qg_ctx_sync(qg_ctx *ctx);
/* Device-side waits give up after this many polls and report QG_ERR_TIMEOUT. */
QG_API qg_status qg_ctx_set_spin_limit(qg_ctx *ctx, uint32_t polls);
/* Reads and clears the device error word; returns QG_OK or the first error
 * any kernel of this context recorded since the last check.  Synchronises. */
QG_API qg_status qg_ctx_check(qg_ctx *ctx);
QG_API const char *qg_status_string(qg_status s);
QG_API const char *qg_last_error_message(qg_ctx *ctx);
/* Bytes of scratch the context currently holds. */
QG_API size_t qg_ctx_scratch_bytes(qg_ctx *ctx);
/* Reserve scratch up front (so later calls allocate nothing). */
QG_API qg_status qg_ctx_reserve(qg_ctx *ctx, size_t bytes);
/* Number of kernels this context has launched (for launch accounting). */
QG_API uint64_t qg_ctx_launch_count(qg_ctx *ctx);
/* Per-kernel timing: with timing on, CUDA events on the context's stream
 * bracket every kernel launch (up to 4096 between reports).  The report
 * synchronises, writes one "kernel_name launches total_ms" line per kernel
 * into buf and clears the log; it returns the number of lines or -1.  The
 * reference timed stages with host wall-clock around clFinish
 * (host/host/testFilter.cpp:110-141); this measures device time. */
QG_API qg_status qg_ctx_enable_timing(qg_ctx *ctx, int on);
QG_API int qg_ctx_timing_report(qg_ctx *ctx, char *buf, size_t len);
/* Milliseconds from the start of the first to the end of the last launch
 * logged since timing was enabled or last reported (an operator's device
 * span, gaps between its kernels included); -1 when nothing was logged. */
QG_API double qg_ctx_timing_span(qg_ctx *ctx);

/* Device buffers handed out by callee-allocates entry points. */
QG_API qg_status qg_malloc(qg_ctx *ctx, void **ptr, size_t bytes);
QG_API qg_status qg_free(qg_ctx *ctx, void *ptr);

/* ---- filter (kernel/filter/filter_op.cl) ----------------------------- */
/* Stable range selection over Records: keeps in[i] when lo <= (int)in[i].y <= hi,
 * in input order.  Replaces filterImpl_map_kernel + ScanLargeArrays/prefixSum/
 * blockAddition + filterImpl_outSize + filterImpl_write
 * (kernel/filter/filter_op.cl:6-238, host/host/testFilter.cpp:92-154) with one
 * single-pass kernel.  `out` holds `cap` records. */
QG_API qg_status qg_filter_range_rec(qg_ctx *ctx, const void *in_records, int64_t n, int32_t lo,
                                     int32_t hi, void *out_records, int64_t cap, int64_t *out_n);
QG_API qg_status qg_filter_range_rec_async(qg_ctx *ctx, const void *in_records, int64_t n,
                                           int32_t lo, int32_t hi, void *out_records, int64_t cap,
                                           int64_t *d_out_n);
/* Column form (config 0): keeps row i when lo <= key[i] <= hi and writes the
 * int32 pair (i, payload[i]) in input order.  `out_pairs` holds `cap` pairs. */
QG_API qg_status qg_filter_cols(qg_ctx *ctx, const int32_t *key, const int32_t *payload, int64_t n,
                                int32_t lo, int32_t hi, int32_t *out_pairs, int64_t cap,
                                int64_t *out_n);
QG_API qg_status qg_filter_cols_async(qg_ctx *ctx, const int32_t *key, const int32_t *payload,
                                      int64_t n, int32_t lo, int32_t hi, int32_t *out_pairs,
                                      int64_t cap, int64_t *d_out_n);

/* Column filter that allocates nothing.  No counterpart in the reference.
 * For callers that cannot allocate device memory (inside an allocator or
 * memory-pool callback, under a framework that owns all device memory, on a
 * path that must not block on the allocator) and therefore cannot create a
 * qg_ctx: same result as qg_filter_cols_async, but the kernel's scratch (its
 * look-back status words and counters) is a fixed device array inside the
 * library, sized for n <= 2^26 rows (larger n returns QG_ERR_UNSUPPORTED);
 * each GPU that loads the library keeps about 128 KB for it until exit.  The
 * first call on a device looks the array's address up (make that call before
 * any stream capture).  All calls share the array: calls that overlap on the
 * GPU race.  The selected-row count goes to the device int64 *d_out_n; a
 * device-side wait that gave up is reported there as -QG_ERR_TIMEOUT.
 * `stream` is a cudaStream_t (NULL = legacy default stream). */
QG_API qg_status qg_filter_cols_noalloc(const int32_t *key, const int32_t *payload, int64_t n,
                                        int32_t lo, int32_t hi, int32_t *out_pairs, int64_t cap,
                                        int64_t *d_out_n, void *stream);
/* Companions of qg_filter_cols_noalloc (no counterpart in the reference).
 * qg_noalloc_set_spin_limit: polls a look-back wait of that filter makes
 * before it gives up and reports -QG_ERR_TIMEOUT (process-wide; default
 * 2^22).  qg_noalloc_forget: drops the remembered device addresses of its
 * array; call it after cudaDeviceReset (or any teardown of a device's primary
 * context), since the next call must look the address up again.  Note also
 * that qg_filter_cols_noalloc returns QG_OK when the count exceeds `cap`:
 * only `cap` pairs are written and *d_out_n holds the full count, so the
 * caller compares the two. */
QG_API qg_status qg_noalloc_set_spin_limit(uint32_t polls);
QG_API qg_status qg_noalloc_forget(void);

/* Column filter kernel choice (process-wide): 0 = one 4096-row tile per CTA
 * held in registers with a decoupled look-back, 1 = persistent CTAs
 * streaming tiles through a 3-stage bulk-copy (TMA) ring, 2 = two passes
 * (per-tile counts from the keys, then the writes) with no look-back, the
 * default.  Results are identical. */
QG_API qg_status qg_filter_set_variant(int variant);

/* ---- scan (ScanLargeArrays/prefixSum/blockAddition, host/host/testScan.cpp:278-340) */
/* Exclusive int32 prefix sum with two's-complement wrap; in == out allowed. */
QG_API qg_status qg_scan_excl_i32(qg_ctx *ctx, const int32_t *in, int32_t *out, int64_t n);

/* ---- sort (bitonicSortShared/bitonicMergeGlobal, host/host/testSort.cpp:24-136) */
/* Ascending sort of Records by .y as unsigned, in place.  Order among equal
 * keys is unspecified, as in the reference. */
QG_API qg_status qg_sort_rec_by_y(qg_ctx *ctx, void *records, int64_t n);
/* Stable ranking of the radix passes whose digits take many values
 * (process-wide): -1 (default) mode 3, measured fastest for sorts of unsorted
 * input and the join's partition passes; 0 eight warp ballots; 3 one match
 * instruction on a digit's high four bits and four ballots on its low four;
 * 4 one match instruction on each half.  Results are identical. */
QG_API qg_status qg_sort_set_rank(int mode);

/* ---- group-by on Records (host/host/testGroupBy.cpp:81-154) ---------- */
/* Sorts `in` by key into `sorted_out` (may equal `in`), then writes the first
 * row index of each group to startPos (capacity `cap_groups`) and the group
 * count to *num_groups. */
QG_API qg_status qg_groupby_rec(qg_ctx *ctx, const void *in_records, int64_t n, void *sorted_out,
                                int32_t *startPos, int64_t cap_groups, int64_t *num_groups);
/* parallelAggregate_kernel (kernel/aggregation/1/group_by_cu_op_dp.cl:547-716):
 * agg[g] = op over .x of rows [startPos[g], startPos[g+1] or n) of sorted records. */
QG_API qg_status qg_aggregate_groups(qg_ctx *ctx, const void *sorted_records, int64_t n,
                                     const int32_t *startPos, int64_t num_groups, int op,
                                     int32_t *agg);
/* The same for groups [first, first+count) only (parallelAggregate_init's
 * blockOffset / numBlock chunks, host/host/testAggAfterGB.cpp:69-91);
 * agg is indexed by absolute group number. */
QG_API qg_status qg_aggregate_group_range(qg_ctx *ctx, const void *sorted_records, int64_t n,
                                          const int32_t *startPos, int64_t num_groups,
                                          int64_t first, int64_t count, int op, int32_t *agg);

/* ---- gather / scatter (gatherImpl / scatterImpl, host/host/testScatter.cpp:63-137;
 * optGather_kernel body: kernel/aggregation/1/group_by_cu_op_dp.cl:860-872)
 * gather : S[i] = R[loc[i*loc_stride]] for i < sLen when 0 <= loc < rLen (else S[i] kept)
 * scatter: S[loc[i*loc_stride]] = R[i] for i < rLen when 0 <= loc < sLen
 * R and S are Records; loc_stride 2 with loc = (int32_t*)records + 0 uses the
 * records' .x as the location. */
QG_API qg_status qg_gather_rec(qg_ctx *ctx, const void *R, int64_t rLen, const int32_t *loc,
                               int64_t loc_stride, int64_t sLen, void *S);
QG_API qg_status qg_scatter_rec(qg_ctx *ctx, const void *R, int64_t rLen, const int32_t *loc,
                                int64_t loc_stride, void *S, int64_t sLen);

/* ---- column group-by + aggregate, optionally fused with a filter (configs 1, 1-fused)
 * Groups rows by key, SUM(val) as int64 and COUNT as int64.  When val2 is not
 * NULL only rows with lo2 <= val2[i] <= hi2 take part (the fused
 * filter_aggregation pipeline, kernel/filter_aggregation/
 * filter_aggregation_cu_op_dp.cl).  Outputs hold `cap` groups; order is
 * QG_ORDER_KEY (ascending unsigned key, the reference's sorted order) or
 * QG_ORDER_NONE.  By default the keys are first aggregated in a direct-indexed
 * window of 2^22 keys placed on a sample's key range (output in key order
 * either way); when the sample spans more than 2^21 keys or any row's key
 * falls outside the window, the call runs the two-pass hash path instead.
 * There `cap` also sizes the spill partitions (about 1024 groups each), so a
 * cap near the true group count is fastest, and for key order the context
 * remembers the key range of its previous call and ranks keys in a bitmap
 * window placed there; results never depend on either, only the path does
 * (keys outside the bitmap window are sorted after the count).
 * qg_groupby_cols_async is the same without a host round trip: the group
 * count goes to device memory (*d_num_groups); key order is sorted on the
 * device (two-pass path, cap < 2^30); a spill overflow is reported by
 * qg_ctx_check as QG_ERR_TABLE_FULL instead of being redone. */
QG_API qg_status qg_groupby_cols(qg_ctx *ctx, const int32_t *key, const int32_t *val,
                                 const int32_t *val2, int32_t lo2, int32_t hi2, int64_t n,
                                 int32_t *gkey, int64_t *gsum, int64_t *gcount, int64_t cap,
                                 int order, int64_t *num_groups);
QG_API qg_status qg_groupby_cols_async(qg_ctx *ctx, const int32_t *key, const int32_t *val,
                                       const int32_t *val2, int32_t lo2, int32_t hi2, int64_t n,
                                       int32_t *gkey, int64_t *gsum, int64_t *gcount, int64_t cap,
                                       int order, int64_t *d_num_groups);

/* Tuning of qg_groupby_cols (process-wide).  mode 0 (default): the
 * dense-window path, else two-pass shared-memory aggregation, with the
 * global-table kernel as automatic fallback of the two-pass path; mode 1:
 * global-table kernel only; mode 2: two-pass with the int64 sums as 64-bit
 * shared atomics instead of two 32-bit words with explicit carry (slower on
 * GB300, kept for comparison); mode 3: two-pass (no dense-window attempt).
 * A context with a cost model attached (qg_steer_attach) may run another
 * mode per call.  hot_slots_log2: the two-pass path's per-SM shared-memory
 * table (8..13); partitions_log2: spill partitions (0 = chosen from cap,
 * else 1..13); bucket_cap: spill bucket capacity (0 = automatic; a small
 * value forces the fallback, for testing). */
QG_API qg_status qg_groupby_set_knobs(int mode, int hot_slots_log2, int partitions_log2,
                                      uint32_t bucket_cap);
/* The dense-window path's four steps (sample, candidates, main pass, emit)
 * as one cooperative launch with grid barriers between them (enable = 1), or
 * as four launches (0, the default; also what runs while the stream is being
 * captured into a graph).  Process-wide; results are identical. */
QG_API qg_status qg_groupby_set_single_launch(int enable);
/* Diagnostics of the context's last qg_groupby_cols call: out[0] = path
 * (0 two-pass, 1 global table, 2 dense window), out[1] = overflow flags
 * (bit 0 spill bucket, bit 1 pass-2 table), out[2] = fullest spill bucket,
 * out[3] = bucket capacity (the last three 0 on the dense-window path). */
QG_API qg_status qg_groupby_stats(qg_ctx *ctx, uint32_t *out4);

/* ---- hash join + filter + sort (config 2; kernel/hj_filter_sort/1/hj_filter_sort_op.cl)
 * Inner equi-join of R(rkey, rpay) and S(skey, spay) on uint key equality,
 * keeping only S rows with slo <= spay <= shi, every match emitted (duplicate
 * build keys allowed).  Output columns (key, R.payload, S.payload) sorted
 * ascending by key (unsigned); order among equal keys unspecified. */
QG_API qg_status qg_join_filter_sort(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay,
                                     int64_t nR, const int32_t *skey, const int32_t *spay,
                                     int64_t nS, int32_t slo, int32_t shi, int32_t *out_key,
                                     int32_t *out_rpay, int32_t *out_spay, int64_t cap,
                                     int64_t *out_n);
/* Join algorithm knobs (process-wide).  variant: 0 auto -- range
 * partitioning by radix over the key, switching to the learned CDF partition
 * function when radix leaves more than 2% of the rows in buckets too large
 * for shared memory and the model does better on the same counts; 1 radix
 * only; 2 learned only; 3 the global hash table + radix sort of the output.
 * buckets_log2: 0 = from the input size (about 2560 rows per bucket), else
 * 1..15.  bucket_s_max / bucket_r_max: rows of a bucket that the shared-memory
 * bucket kernel takes (0 = its capacity, 4096 / 2048); smaller values send
 * more buckets to the outside paths (testing).  No reference counterpart:
 * the reference has a single join kernel pair. */
QG_API qg_status qg_join_set_knobs(int variant, int buckets_log2, uint32_t bucket_s_max,
                                   uint32_t bucket_r_max);
/* Dense build side (process-wide, on by default): when R's keys are unique
 * and spread over at most 2 nR values, a presence bitmap and a payload table
 * indexed by key - min(key) stand for R, so only S is partitioned (radix
 * partitioning; an S bucket above the bucket kernel's capacity, or the learned
 * function, takes the general path instead).  enable = 0 always takes the
 * general path.  Results are identical. */
QG_API qg_status qg_join_set_dense(int enable);
/* Diagnostics of the context's last qg_join_filter_sort: out[0] path
 * (1 radix, 2 learned, 3 hash join + sort, 4 radix with the dense build side,
 * 0 nothing to join), out[1]
 * buckets, out[2] buckets handled outside the bucket kernel, out[3] their
 * rows, out[4] those of them with several keys (joined together by the
 * sort-merge path; the others are single-key cross products), out[5] knots
 * of the learned model (path 4: the dense bucket kernel's CTAs per SM),
 * out[6] heavy keys among them, out[7] 1 when the automatic choice moved
 * from radix to the learned function. */
QG_API qg_status qg_join_stats(qg_ctx *ctx, uint32_t *out8);

/* ---- whole-column reduce (the check of host/host/Validate.cpp:372-468; the
 * reference ships no kernel) ----  SUM (wrapping modulo 2^32), MAX and MIN
 * (unsigned compare) or AVERAGE (wrapped sum / n, unsigned) of Record.y. */
QG_API qg_status qg_reduce_rec(qg_ctx *ctx, const void *in_records, int64_t n, int op,
                               uint32_t *result);
/* ---- radix split (splitImpl, host/host/testSplit.cpp:156-209; kernels not
 * shipped) ----  out = the records grouped by partition id (y mod num_part),
 * stable within a partition; bound[p] (device, num_part int32) = first row of
 * partition p. */
QG_API qg_status qg_split_rec(qg_ctx *ctx, const void *in_records, int64_t n, int32_t num_part,
                              void *out_records, int32_t *bound);

/* ---- batched queries (no reference counterpart: the reference runs one
 * operator per call, each followed by clFinish and host reads) ----
 * A batch of filter / group-by / fused filter+group-by / join+sort queries is
 * run once eagerly, captured into a CUDA graph of the operators' sync-free
 * forms (one graph per autotuner candidate: group-by shared table of 2^12 or
 * 2^13 slots x join hash table at 2x or 4x the build rows), timed, and the
 * fastest graph kept; qg_batch_run replays it with one graph launch.  The
 * batch owns a private context whose work arenas the graph addresses.
 * Inputs and outputs stay the caller's and must stay valid while the batch
 * exists.  Joins in a batch use the global hash table + device-planned sort;
 * group-by outputs are unordered (QG_ORDER_NONE).  A group-by query on the
 * default variant is run once at creation on the dense-window path; when its
 * keys fit a window, the graph takes that path for it (sync-free, output in
 * key order), else the two-pass path.  Errors of a replay (a join over cap:
 * QG_ERR_CAPACITY; a group-by spill overflow: QG_ERR_TABLE_FULL; new data in
 * a dense-window query's buffers whose keys no longer fit a window:
 * QG_ERR_UNSUPPORTED, create the batch again) are reported by
 * qg_batch_check. */
typedef enum { QG_OP_FILTER = 0, QG_OP_GROUPBY = 1, QG_OP_FUSED = 2, QG_OP_JOIN = 3 } qg_op;
typedef struct {
    int op;                /* qg_op */
    int variant;           /* -1 default; filter 0, 1 or 2 (default 2); group-by 0 dense window when the keys fit one, else
                              two-pass (default), 1 global table, 2 two-pass 64-bit adds, 3 two-pass */
    int64_t n;             /* rows (join: S rows) */
    int64_t n2;            /* join: R rows */
    const int32_t *in[4];  /* filter: key, payload; group-by: key, value, value2 (fused); join: rkey, rpay, skey, spay */
    int32_t lo, hi;        /* filter: key range; fused: value2 range; join: S.payload range */
    void *out[3];          /* filter: (row id, payload) int32 pairs; group-by: key int32, sum int64, count int64;
                              join: key, R.payload, S.payload int32 */
    int64_t cap;           /* output rows room (group-by: groups) */
    int64_t *d_count;      /* device int64: rows produced */
} qg_query;
typedef struct qg_batch qg_batch;
QG_API qg_status qg_batch_create(const qg_query *queries, int nq, int autotune, qg_batch **out);
/* Enqueue the batch on `stream` (a cudaStream_t; NULL = the default stream). */
QG_API qg_status qg_batch_run(qg_batch *b, void *stream);
/* Synchronise `stream` and report the first device error of the batch's kernels. */
QG_API qg_status qg_batch_check(qg_batch *b, void *stream);
/* out4: group-by table slots log2, join table factor, best replay in us, graph nodes. */
QG_API qg_status qg_batch_info(const qg_batch *b, int32_t *out4);
QG_API qg_status qg_batch_destroy(qg_batch *b);
/* Lanes of the batches created after this call (process-wide, 1..16; default
 * 8): the queries are spread over that many streams, each with a private
 * context, and the graph runs the lanes side by side. */
QG_API qg_status qg_batch_set_lanes(int lanes);
/* Form of the batches created after this call (process-wide): 1
 * persistent -- every filter, group-by and fused query runs inside one
 * persistent kernel launch whose CTAs take (query, tile) work items from a
 * device queue (filter tiles with a per-query look-back, group-by tiles into
 * a per-query table, emit tiles after the query's tiles; the kernel's table
 * and tile sizes are the autotuner's group tile of 2^13 or 2^14 rows), the
 * joins as their own launches on the other lanes beside it; 0 (default)
 * lanes -- every query as its operator's launches (faster on mixed queries
 * with high-cardinality group-bys, whose per-query tables the persistent
 * kernel touches at about one random sector per group).  In the persistent
 * form a filter or group-by query's `variant` is not used. */
QG_API qg_status qg_batch_set_persistent(int on);

/* ---- learned cost model (no reference counterpart; it stands beside the
 * static unit-cost table of host/dynamic_programming.cpp:152-167) ----
 * A 16 -> 64 (ReLU) -> 1 fp32 MLP over plan features, trained on timings the
 * engine records, predicting an operator variant's log run time.  params is
 * a device array of qg_mlp_param_count() floats: W1[64][16], b1[64], W2[64],
 * b2.  X is n x 16 row-major, y and out n floats, all on the device. */
QG_API int64_t qg_mlp_param_count(void);
/* Deterministic initialisation from a seed (uniform +-1/sqrt(fan_in), zero biases). */
QG_API qg_status qg_mlp_init(qg_ctx *ctx, float *params, uint32_t seed);
QG_API qg_status qg_mlp_predict(qg_ctx *ctx, const float *params, const float *X, int64_t n,
                                float *out);
/* Gradient of mean((f(X) - y)^2) into grad (param_count floats); loss (device
 * float, may be NULL) receives the loss.  Deterministic (no atomics). */
QG_API qg_status qg_mlp_grad(qg_ctx *ctx, const float *params, const float *X, const float *y,
                             int64_t n, float *grad, float *loss);
/* `steps` full-batch Adam steps.  opt: 3 * param_count device floats, zeroed
 * before the first call of a training run; *t counts the steps taken. */
QG_API qg_status qg_mlp_train(qg_ctx *ctx, float *params, const float *X, const float *y, int64_t n,
                              int steps, float lr, float *opt, int *t, float *loss);

/* ---- the cost model steering the engine (replaces the static variant
 * choice of host/dynamic_programming.cpp:874-996 with the model's, the plain
 * choice kept as fallback and judge) ----
 * Operators: 0 filter (qg_filter_cols), 1 group-by, 2 fused filter +
 * group-by (qg_groupby_cols without / with val2), 3 join (qg_join_filter_sort).
 * qg_steer_attach evaluates the model (device params, as trained) once on a
 * grid of plan features with the inference kernel and keeps the predicted
 * time of every variant per grid cell on the context.  From then on each
 * synchronous call of those operators on the context runs its cell's
 * predicted-fastest variant and times itself; a call slower than
 * (1 + tolerance) x its prediction makes the cell's next call run the plain
 * variant (the process-wide knob), and the cell keeps whichever of the two
 * ran faster.  Results are identical whichever variant runs.
 * qg_steer_choose: the variant the context would run (without running it)
 * and its predicted ms.  qg_steer_stats: per operator, out[0] calls,
 * [1] calls that ran the model's non-plain choice, [2] calls that ran the
 * plain variant, [3] judge runs of the plain variant, [4] cells that fell
 * back to it, [5] cells whose choice a judge run confirmed, [6] the last
 * call's variant, [7] its measured and [8] its predicted time in us,
 * [9] grid cells where the model's choice differs from the plain one.
 * qg_steer_plan: the reference's DP (dp_test sub_index 0-3, size in M rows)
 * over a cost table of the model's per-variant predictions (one row per
 * primitive and variant, scan primitives at zero cost: they are fused into
 * the operators); *variant receives the operator variant the plan chose. */
QG_API qg_status qg_steer_attach(qg_ctx *ctx, const float *d_params, float tolerance);
QG_API qg_status qg_steer_detach(qg_ctx *ctx);
QG_API qg_status qg_steer_choose(qg_ctx *ctx, int op, int64_t n, int64_t n2, float sel, int *variant,
                                 float *pred_ms);
QG_API qg_status qg_steer_stats(qg_ctx *ctx, int op, int64_t *out10);

/* ---- learned partition function (no reference counterpart) ----
 * A piecewise-linear model of a key CDF (1024 fp32 segments plus heavy-key
 * knots) mapping keys to nbuckets buckets, non-decreasing in the unsigned
 * key; fitted on the GPU from a sample of up to 2^20 of the keys.  d_model is
 * a device buffer of qg_part_model_bytes() bytes. */
QG_API int64_t qg_part_model_bytes(void);
QG_API qg_status qg_part_learn(qg_ctx *ctx, const uint32_t *keys, int64_t n, uint32_t nbuckets,
                               void *d_model);
/* Buckets of n keys: under the learned model d_model, or (d_model NULL) the
 * radix function (key - kmin) >> shift. */
QG_API qg_status qg_part_eval(qg_ctx *ctx, const void *d_model, uint32_t kmin, int shift,
                              const uint32_t *keys, int64_t n, uint32_t *buckets);

/* Reference layout (buildHashTable/probeHashTable, hj_filter_sort_op.cl:25-109):
 * r and s are interleaved uint (key, val) pairs; every match writes the pair
 * (S.val, R.val).  Compacted output (the reference leaves holes); order
 * unspecified. */
QG_API qg_status qg_hash_join_ref(qg_ctx *ctx, const uint32_t *r_pairs, int64_t nR,
                                  const uint32_t *s_pairs, int64_t nS, uint32_t *out_pairs,
                                  int64_t cap, int64_t *out_n);

/* The same join in its two reference steps, so one build serves many probe
 * batches.  Replaces buildHashTable (hj_filter_sort_op.cl:25-60), whose caller
 * allocates the table (rHashTable, rHashCount): the caller allocates
 * qg_hash_table_bytes(nR) bytes of device memory, 256-byte aligned, and
 * qg_hash_build_ref fills them from the interleaved (key, val) pairs of R
 * (synchronous; QG_ERR_CAPACITY if table_bytes is too small).  Replaces
 * probeHashTable (hj_filter_sort_op.cl:62-109): qg_hash_probe_ref reads the
 * table (which it does not change, so several probes, also on different
 * contexts, may read one table) and writes every match as (S.val, R.val),
 * compacted, order unspecified; *out_n is the match count (QG_ERR_CAPACITY
 * when above cap).  qg_hash_table_bytes returns -1 for nR outside [0, 2^30). */
QG_API int64_t qg_hash_table_bytes(int64_t nR);
QG_API qg_status qg_hash_build_ref(qg_ctx *ctx, const uint32_t *r_pairs, int64_t nR, void *table,
                                   int64_t table_bytes);
QG_API qg_status qg_hash_probe_ref(qg_ctx *ctx, const void *table, const uint32_t *s_pairs, int64_t nS,
                                   uint32_t *out_pairs, int64_t cap, int64_t *out_n);

#ifdef __cplusplus
}
#endif
#endif /* QG_H */
