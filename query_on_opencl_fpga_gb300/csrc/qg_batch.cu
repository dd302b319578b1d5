// qg_batch.cu -- many queries of uneven sizes as one CUDA graph.
//
// Two forms.  Persistent (qg_batch_set_persistent(1)): every
// filter, group-by and fused query runs inside one persistent kernel launch
// (qg_bpersist.cu) on lane 0, and the joins run as their operators' launches
// on the other lanes beside it.  Lanes: every query runs as its operator's
// own sync-free launches, spread over the lanes (the default: faster on the
// mixed workload measured).  In both forms:
//
// The reference runs one operator per call, each call followed by clFinish
// and host reads (host/host/common.cpp:31, testFilter.cpp:128-133).  A batch
// here is a list of filter / group-by / fused filter+group-by / join+sort
// queries that is
//   1. run once eagerly per candidate configuration, so that every work arena
//      reaches its final size (a graph may not allocate, and later growth
//      would move memory the graph's kernels address),
//   2. captured, for every candidate configuration of the autotuner (the
//      group-by's shared-memory table size and the join's hash-table load),
//      into a CUDA graph of the sync-free forms of the operators
//      (qg_filter_cols_async, qg_groupby_cols_async, qg_join_hash_sort_async),
//   3. timed by replays, keeping the fastest graph.
// qg_batch_run then replays that graph on the caller's stream: the whole
// batch costs one graph launch and no host round trip.  Each query's kernel
// variant comes from the query (chosen by the caller, e.g. by the learned
// cost model) or is the default.  The batch owns a private context, so its
// arenas are never moved by other calls.
#include <algorithm>
#include <vector>
#include "qg_internal.cuh"

qg_status qg_join_hash_sort_async(qg_ctx *ctx, const int32_t *rkey, const int32_t *rpay, int64_t nR,
                                  const int32_t *skey, const int32_t *spay, int64_t nS, int32_t slo,
                                  int32_t shi, int32_t *out_key, int32_t *out_rpay, int32_t *out_spay,
                                  int64_t cap, int64_t *d_count);
void qg_join_set_table_factor(int factor);
struct qg_bpersist;
qg_status qg_bpersist_create(qg_ctx *ctx, const qg_query *q, int nq, const std::vector<int> &use, int gtile_log2,
                             qg_bpersist **out);
qg_status qg_bpersist_launch(qg_ctx *ctx, qg_bpersist *p);
qg_status qg_bpersist_check(qg_ctx *ctx, qg_bpersist *p);
void qg_bpersist_destroy(qg_bpersist *p);

// The queries are independent, so they are spread over lanes: each lane has
// its own stream and private context (arenas, control block), and the graph
// forks into the lanes and joins them, so that small queries run beside
// large ones instead of one after another.
constexpr int QG_BATCH_MAX_LANES = 16;
static int g_batch_lanes = 8;
// Measured on config 3 (512 mixed queries): lanes 18 ms, persistent 28 ms.
// The persistent kernel's group-by tables are touched at about one random
// sector per group, and Zipf keys over 1M groups give nearly as many groups
// as rows, so its DRAM traffic runs at about 5x the input (ncu); the lanes'
// two-pass group-by spills sequentially instead.  Lanes is the default.
static int g_batch_persistent = 0;

struct qg_batch {
    int lanes = 1;
    qg_ctx *own[QG_BATCH_MAX_LANES] = {};
    cudaStream_t ls[QG_BATCH_MAX_LANES] = {};  // lane streams; lane 0's is the capture origin
    cudaEvent_t fork = nullptr, join[QG_BATCH_MAX_LANES] = {};
    cudaStream_t stream = nullptr;  // == ls[0]
    std::vector<qg_query> q;
    std::vector<int> lane;  // lane of each query
    cudaGraphExec_t exec = nullptr;
    int32_t info[4] = {0, 0, 0, 0};  // hot slots / group tile log2, table factor, best replay us, graph nodes
    bool persistent = false;
    std::vector<char> gdense;        // lanes: the group-by query takes the dense-window path
    std::vector<int> pq;             // queries of the persistent kernel
    qg_bpersist *bp = nullptr;       // its state (of the kept graph)
};

namespace {

struct BatchCfg {
    int hot_log2;  // lanes: group-by shared table slots; persistent: group tile rows (log2)
    int table_factor;
};

qg_status enqueue(qg_batch *b, const BatchCfg &c, qg_bpersist *bp) {
    qg_status st = QG_OK;
    if (b->persistent && bp) st = qg_bpersist_launch(b->own[0], bp);
    for (size_t i = 0; i < b->q.size() && st == QG_OK; i++) {
        const qg_query &q = b->q[i];
        if (b->persistent && q.op != QG_OP_JOIN) continue;  // in the persistent kernel
        qg_ctx *ctx = b->own[b->lane[i]];
        const int v = q.variant >= 0 ? q.variant : (q.op == QG_OP_FILTER ? 2 : 0);  // the operators' defaults
        switch (q.op) {
        case QG_OP_FILTER:
            st = qg_filter_set_variant(v);
            if (st == QG_OK)
                st = qg_filter_cols_async(ctx, q.in[0], q.in[1], q.n, q.lo, q.hi, (int32_t *)q.out[0], q.cap,
                                          q.d_count);
            break;
        case QG_OP_GROUPBY:
        case QG_OP_FUSED:
            if (i < b->gdense.size() && b->gdense[i]) {
                st = qg_groupby_dense_async(ctx, q.in[0], q.in[1], q.op == QG_OP_FUSED ? q.in[2] : nullptr, q.lo,
                                            q.hi, q.n, (int32_t *)q.out[0], (int64_t *)q.out[1],
                                            (int64_t *)q.out[2], q.cap, q.d_count);
                break;
            }
            st = qg_groupby_set_knobs(v, c.hot_log2, 0, 0);
            if (st == QG_OK)
                st = qg_groupby_cols_async(ctx, q.in[0], q.in[1], q.op == QG_OP_FUSED ? q.in[2] : nullptr, q.lo,
                                           q.hi, q.n, (int32_t *)q.out[0], (int64_t *)q.out[1],
                                           (int64_t *)q.out[2], q.cap, QG_ORDER_NONE, q.d_count);
            break;
        case QG_OP_JOIN:
            qg_join_set_table_factor(c.table_factor);
            st = qg_join_hash_sort_async(ctx, q.in[0], q.in[1], q.n2, q.in[2], q.in[3], q.n, q.lo, q.hi,
                                         (int32_t *)q.out[0], (int32_t *)q.out[1], (int32_t *)q.out[2], q.cap,
                                         q.d_count);
            break;
        default:
            st = QG_ERR_INVALID;
        }
        if (st != QG_OK) break;
    }
    qg_filter_set_variant(2);
    qg_groupby_set_knobs(0, 13, 0, 0);
    qg_join_set_table_factor(2);
    return st;
}

// Lanes 1.. wait on lane 0 before their queries; lane 0 waits on all of them
// after.  Inside a capture this makes the fork and join of the graph; in an
// eager run it orders the lanes the same way.
cudaError_t fork_lanes(qg_batch *b) {
    cudaError_t e = cudaEventRecord(b->fork, b->ls[0]);
    for (int l = 1; l < b->lanes && e == cudaSuccess; l++) e = cudaStreamWaitEvent(b->ls[l], b->fork, 0);
    return e;
}
cudaError_t join_lanes(qg_batch *b) {
    cudaError_t e = cudaSuccess;
    for (int l = 1; l < b->lanes && e == cudaSuccess; l++) {
        e = cudaEventRecord(b->join[l], b->ls[l]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->ls[0], b->join[l], 0);
    }
    return e;
}

qg_status capture(qg_batch *b, const BatchCfg &c, qg_bpersist *bp, cudaGraphExec_t *exec, size_t *nodes) {
    cudaGraph_t g = nullptr;
    QG_TRY_CUDA(b->own[0], cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    cudaError_t ef = fork_lanes(b);
    const qg_status st = ef == cudaSuccess ? enqueue(b, c, bp) : QG_ERR_CUDA;
    const cudaError_t ej = join_lanes(b);
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (st != QG_OK || ef != cudaSuccess || ej != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return st != QG_OK ? st : QG_ERR_CUDA;
    }
    QG_TRY_CUDA(b->own[0], e, "end capture");
    cudaError_t ei = cudaGraphGetNodes(g, nullptr, nodes);
    if (ei == cudaSuccess) ei = cudaGraphInstantiate(exec, g, 0);
    cudaGraphDestroy(g);
    QG_TRY_CUDA(b->own[0], ei, "instantiate graph");
    return QG_OK;
}

float replay_ms(qg_batch *b, cudaGraphExec_t exec, int reps) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaGraphLaunch(exec, b->stream);
    cudaEventRecord(e0, b->stream);
    for (int i = 0; i < reps; i++) cudaGraphLaunch(exec, b->stream);
    cudaEventRecord(e1, b->stream);
    float ms = -1.f;
    if (cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / reps;
}

}  // namespace

extern "C" {

QG_API qg_status qg_batch_create(const qg_query *queries, int nq, int autotune, qg_batch **out) {
    if (!queries || nq <= 0 || !out) return QG_ERR_INVALID;
    *out = nullptr;
    qg_batch *b = new qg_batch();
    b->q.assign(queries, queries + nq);
    b->lanes = std::min(g_batch_lanes, nq);
    qg_status st = QG_OK;
    if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) st = QG_ERR_CUDA;
    for (int l = 0; l < b->lanes && st == QG_OK; l++) {
        if (cudaStreamCreateWithFlags(&b->ls[l], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join[l], cudaEventDisableTiming) != cudaSuccess)
            st = QG_ERR_CUDA;
        if (st == QG_OK) st = qg_ctx_create(&b->own[l], b->ls[l]);
    }
    if (st != QG_OK) {
        cudaGetLastError();
        qg_batch_destroy(b);
        return st;
    }
    b->stream = b->ls[0];
    b->persistent = g_batch_persistent != 0;
    for (int i = 0; i < nq && b->persistent; i++)
        if (b->q[i].op != QG_OP_JOIN) b->pq.push_back(i);
    // Largest queries first, each to the lane with the fewest rows so far
    // (persistent form: lane 0 runs the persistent kernel, the joins share
    // the other lanes).
    {
        std::vector<int> order;
        for (int i = 0; i < nq; i++)
            if (!b->persistent || b->q[i].op == QG_OP_JOIN) order.push_back(i);
        auto rows = [&](int i) { return b->q[i].n + (b->q[i].op == QG_OP_JOIN ? b->q[i].n2 : 0); };
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return rows(x) > rows(y); });
        const int first = b->persistent && b->lanes > 1 ? 1 : 0;
        std::vector<long long> load(b->lanes, 0);
        b->lane.assign(nq, 0);
        for (int i : order) {
            int best = first;
            for (int l = first + 1; l < b->lanes; l++)
                if (load[l] < load[best]) best = l;
            b->lane[i] = best;
            load[best] += rows(i);
        }
    }
    // Lanes: a group-by query on the default variant (dense window first) is
    // run once on the dense-window path; when every row fell in the window the
    // captured form takes that path too, sync-free (rows outside the window on
    // a later replay are reported, QG_ERR_UNSUPPORTED, not handed over to the
    // two-pass path, which needs a host read).  The others keep the sync-free
    // two-pass path.
    b->gdense.assign(nq, 0);
    for (int i = 0; i < nq && st == QG_OK && !b->persistent; i++) {
        const qg_query &q = b->q[i];
        if ((q.op != QG_OP_GROUPBY && q.op != QG_OP_FUSED) || (q.variant >= 0 && q.variant != 0)) continue;
        bool ok = false;
        st = qg_groupby_dense_probe(b->own[b->lane[i]], q.in[0], q.in[1], q.op == QG_OP_FUSED ? q.in[2] : nullptr,
                                    q.lo, q.hi, q.n, (int32_t *)q.out[0], (int64_t *)q.out[1], (int64_t *)q.out[2],
                                    q.cap, q.d_count, &ok);
        b->gdense[i] = ok ? 1 : 0;
    }
    std::vector<BatchCfg> cands;
    if (autotune) {
        for (int h : (b->persistent ? std::vector<int>{13, 14} : std::vector<int>{12, 13}))
            for (int t : {2, 4}) cands.push_back(BatchCfg{h, t});
    } else {
        cands.push_back(BatchCfg{13, 2});
    }
    // 1. The persistent kernel's state of every group tile the candidates use
    //    (its items depend on it), and one eager run of every candidate, so
    //    that every work arena reaches its final size before any capture: a
    //    graph may not allocate, and an arena that grew after a capture would
    //    have moved memory the captured graph addresses.
    std::vector<qg_bpersist *> bps(cands.size(), nullptr);
    for (size_t i = 0; i < cands.size() && st == QG_OK; i++) {
        if (!b->persistent || b->pq.empty()) continue;
        for (size_t j = 0; j < i; j++)
            if (cands[j].hot_log2 == cands[i].hot_log2) bps[i] = bps[j];
        if (!bps[i]) st = qg_bpersist_create(b->own[0], b->q.data(), nq, b->pq, cands[i].hot_log2, &bps[i]);
    }
    for (size_t i = 0; i < cands.size() && st == QG_OK; i++) {
        if (fork_lanes(b) != cudaSuccess) st = QG_ERR_CUDA;
        if (st == QG_OK) st = enqueue(b, cands[i], bps[i]);
        if (st == QG_OK && join_lanes(b) != cudaSuccess) st = QG_ERR_CUDA;
        for (int l = 0; l < b->lanes && st == QG_OK; l++) st = qg_ctx_check(b->own[l]);
        if (st == QG_OK && bps[i]) st = qg_bpersist_check(b->own[0], bps[i]);
    }
    // 2. capture and time every candidate, keep the fastest graph (and the
    //    persistent state it launches)
    float best = 0.f;
    int kept = -1;
    for (size_t i = 0; i < cands.size() && st == QG_OK; i++) {
        cudaGraphExec_t ex = nullptr;
        size_t nodes = 0;
        st = capture(b, cands[i], bps[i], &ex, &nodes);
        if (st != QG_OK) break;
        const float ms = replay_ms(b, ex, 3);
        for (int l = 0; l < b->lanes && st == QG_OK; l++) st = qg_ctx_check(b->own[l]);
        if (st == QG_OK && bps[i]) st = qg_bpersist_check(b->own[0], bps[i]);
        if (st != QG_OK || ms < 0.f) {
            cudaGraphExecDestroy(ex);
            if (st == QG_OK) st = QG_ERR_CUDA;
            break;
        }
        if (!b->exec || ms < best) {
            if (b->exec) cudaGraphExecDestroy(b->exec);
            b->exec = ex;
            kept = (int)i;
            best = ms;
            b->info[0] = cands[i].hot_log2;
            b->info[1] = cands[i].table_factor;
            b->info[2] = (int32_t)(ms * 1000.f);
            b->info[3] = (int32_t)nodes;
        } else {
            cudaGraphExecDestroy(ex);
        }
    }
    // the kept graph's persistent state stays with the batch; the others go
    if (st == QG_OK && kept >= 0) b->bp = bps[kept];
    for (size_t i = 0; i < bps.size(); i++) {
        if (!bps[i] || bps[i] == b->bp) continue;
        bool freed = false;
        for (size_t j = 0; j < i; j++) freed |= bps[j] == bps[i];
        if (!freed) qg_bpersist_destroy(bps[i]);
    }
    if (st != QG_OK) {
        qg_batch_destroy(b);
        return st;
    }
    *out = b;
    return QG_OK;
}

QG_API qg_status qg_batch_run(qg_batch *b, void *stream) {
    if (!b || !b->exec) return QG_ERR_INVALID;
    if (cudaGraphLaunch(b->exec, (cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();
        return QG_ERR_CUDA;
    }
    return QG_OK;
}

QG_API qg_status qg_batch_check(qg_batch *b, void *stream) {
    if (!b) return QG_ERR_INVALID;
    if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess) {
        cudaGetLastError();
        return QG_ERR_CUDA;
    }
    qg_status st = QG_OK;
    for (int l = 0; l < b->lanes && st == QG_OK; l++) st = qg_ctx_check(b->own[l]);
    if (st == QG_OK && b->bp) st = qg_bpersist_check(b->own[0], b->bp);
    return st;
}

QG_API qg_status qg_batch_info(const qg_batch *b, int32_t *out4) {
    if (!b || !out4) return QG_ERR_INVALID;
    for (int i = 0; i < 4; i++) out4[i] = b->info[i];
    return QG_OK;
}

QG_API qg_status qg_batch_destroy(qg_batch *b) {
    if (!b) return QG_ERR_INVALID;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    qg_bpersist_destroy(b->bp);
    for (int l = 0; l < QG_BATCH_MAX_LANES; l++) {
        if (b->own[l]) qg_ctx_destroy(b->own[l]);
        if (b->ls[l]) cudaStreamDestroy(b->ls[l]);
        if (b->join[l]) cudaEventDestroy(b->join[l]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    delete b;
    return QG_OK;
}

// Form of the batches created after this call: 1 persistent, 0 lanes (default).
QG_API qg_status qg_batch_set_persistent(int on) {
    g_batch_persistent = on ? 1 : 0;
    return QG_OK;
}

// Lanes of the batches created after this call (1..16; default 8).
QG_API qg_status qg_batch_set_lanes(int lanes) {
    if (lanes < 1 || lanes > QG_BATCH_MAX_LANES) return QG_ERR_INVALID;
    g_batch_lanes = lanes;
    return QG_OK;
}

}  // extern "C"
