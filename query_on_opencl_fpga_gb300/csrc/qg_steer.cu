// qg_steer.cu -- the learned cost model inside the engine: the operators'
// kernel-variant choice and the planner's cost table come from the MLP
// (qg_mlp.cu) trained on timings the engine recorded, with the plain choice
// (the process-wide variant knobs, the DP planner's input) as the fallback and
// the judge of mispredictions.
//
// The reference plans with a static table of unit costs per FPGA kernel
// variant (host/dynamic_programming.cpp:133-185) searched by
// dp_for_selection (:874-996).  Here:
//   - qg_steer_attach runs the library's inference kernel once over a grid of
//     plan features (operator, log2 rows in half steps, log2 second size,
//     the filter's selectivity in eighths) and keeps, per grid cell, the
//     predicted time of every variant: a decision table on the host, so a
//     call looks its variant up without a device round trip;
//   - a synchronous operator call (qg_filter_cols, qg_groupby_cols,
//     qg_join_filter_sort) on a context with a model runs the cell's
//     predicted-fastest variant and times itself with an event pair on the
//     context's stream (read after the call's own synchronisation);
//   - the judge: when a call takes longer than (1 + tolerance) times its
//     prediction, the cell's next call runs the plain variant instead; if that
//     is faster, the cell falls back to it for good, otherwise the model's
//     choice is confirmed and no longer tried against it;
//   - qg_steer_plan fills the DP planner's cost table with the predictions of
//     every variant (one row per primitive and variant, the operator's
//     predicted time split over its primitives) and runs the reference's DP
//     over the chosen pipeline.
// Results are identical whatever the choice: every variant is bit-exact.
#include <math.h>
#include <string.h>

#include <vector>

#include "qg_internal.cuh"
#include "qg_plan.h"

qg_status qg_plan_pipeline_rows(const qg_plan_variant *rows, int n_rows, int fpga_model, int sub_index,
                                float size_m, qg_plan *out);

namespace {

constexpr int NF = 16;         // plan features
constexpr int NV = 4;          // variants per operator at most
const int NVAR[QG_STEER_OPS] = {3, 4, 4, 4};  // filter 0-2; group-by and fused 0-3; join 0-3
constexpr int GA = 65;         // log2(rows) in half steps, 0 .. 32
constexpr int GB = 33;         // log2(second size + 1), 0 .. 32
constexpr int GS = 9;          // filter selectivity in eighths, 0 .. 8
// Selectivity the other operators' cells are predicted at: the value their
// timings were recorded with (group-by keeps every row; the fused form and
// the join's S filter were recorded at 0.5 and 0.3).
const double OP_SEL[QG_STEER_OPS] = {0.0, 1.0, 0.5, 0.3};

enum { S_MODEL = 0, S_TRIAL = 1, S_FALLBACK = 2, S_CONFIRMED = 3 };
enum { T_CALLS, T_MODEL_CALLS, T_DEFAULT_CALLS, T_TRIALS, T_FALLBACKS, T_CONFIRMED, T_LAST_VARIANT,
       T_LAST_US, T_LAST_PRED_US, T_CELLS_NONDEFAULT, T_N };

struct Cell {
    float pred[NV];  // predicted ms per variant
    int8_t model;    // argmin of pred
    uint8_t state;
    float t_model;   // the model choice's time that sent the cell to trial
};

int ncells(int op) { return op == QG_STEER_FILTER ? GA * GS : GA * GB; }

int grid_a(int64_t n) {
    const double a = 2.0 * log2((double)(n > 1 ? n : 1));
    const int i = (int)lround(a);
    return i < 0 ? 0 : (i >= GA ? GA - 1 : i);
}
int grid_b(int64_t n2) {
    const int i = (int)lround(log2((double)(n2 > 0 ? n2 : 0) + 1.0));
    return i < 0 ? 0 : (i >= GB ? GB - 1 : i);
}
int grid_s(double sel) {
    const int i = (int)lround(sel * 8.0);
    return i < 0 ? 0 : (i >= GS ? GS - 1 : i);
}
int cell_of(int op, int64_t n, int64_t n2, double sel) {
    return op == QG_STEER_FILTER ? grid_a(n) * GS + grid_s(sel) : grid_a(n) * GB + grid_b(n2);
}

// The 16 plan features of one variant of `op` on one input; the same
// definition as the cost model's training (costmodel.features): operator and
// variant one-hot, log2 sizes over 32, selectivity, skew and products.
void features(int op, int variant, double n, double n2, double sel, double skew, float *f) {
    for (int i = 0; i < NF; i++) f[i] = 0.0f;
    f[op] = 1.0f;
    f[4 + variant] = 1.0f;
    const double ln = log2(n > 1.0 ? n : 1.0) / 32.0;
    const double l2 = log2((n2 > 0.0 ? n2 : 0.0) + 1.0) / 32.0;
    f[8] = (float)ln;
    f[9] = (float)l2;
    f[10] = (float)sel;
    f[11] = (float)skew;
    f[12] = (float)(ln * ln);
    f[13] = (float)(ln * skew);
    f[14] = (float)(l2 * skew);
    f[15] = 1.0f;
}

// Grid point of a cell: rows 2^(a/2), second size 2^b - 1, selectivity s/8.
void cell_point(int op, int c, double *n, double *n2, double *sel) {
    if (op == QG_STEER_FILTER) {
        *n = exp2(0.5 * (c / GS));
        *n2 = 0.0;
        *sel = (c % GS) / 8.0;
    } else {
        *n = exp2(0.5 * (c / GB));
        *n2 = exp2((double)(c % GB)) - 1.0;
        *sel = OP_SEL[op];
    }
}

int default_variant(int op) {
    const int v = op == QG_STEER_FILTER ? qg_filter_default_variant()
                  : op == QG_STEER_JOIN ? qg_join_default_variant()
                                        : qg_groupby_default_mode();
    return v >= 0 && v < NVAR[op] ? v : 0;
}

}  // namespace

struct qg_steer_state {
    float tol;
    std::vector<Cell> cells[QG_STEER_OPS];
    int64_t stats[QG_STEER_OPS][T_N];
    cudaEvent_t ev0, ev1;
};

void qg_steer_free(qg_ctx *ctx) {
    if (!ctx || !ctx->steer) return;
    cudaEventDestroy(ctx->steer->ev0);
    cudaEventDestroy(ctx->steer->ev1);
    delete ctx->steer;
    ctx->steer = nullptr;
    for (int i = 0; i < QG_STEER_OPS; i++) ctx->steer_force[i] = -1;
}

void qg_steer_begin(qg_ctx *ctx, int op, int64_t n, int64_t n2, double sel, qg_steer_call *c) {
    c->active = false;
    if (!ctx || !ctx->steer || n <= 0 || op < 0 || op >= QG_STEER_OPS) return;
    qg_steer_state *st = ctx->steer;
    c->op = op;
    c->cell = cell_of(op, n, n2, sel);
    const Cell &C = st->cells[op][c->cell];
    const int dflt = default_variant(op);
    c->variant = (C.state == S_TRIAL || C.state == S_FALLBACK) ? dflt : C.model;
    ctx->steer_force[op] = c->variant;
    if (cudaEventRecord(st->ev0, ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        ctx->steer_force[op] = -1;
        return;
    }
    c->active = true;
}

void qg_steer_end(qg_ctx *ctx, qg_steer_call *c, qg_status status) {
    if (!c->active) return;
    const int op = c->op;
    ctx->steer_force[op] = -1;
    qg_steer_state *st = ctx->steer;
    if (status != QG_OK) return;  // only completed calls are judged
    float ms = 0.0f;
    if (cudaEventRecord(st->ev1, ctx->stream) != cudaSuccess || cudaEventSynchronize(st->ev1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, st->ev0, st->ev1) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    Cell &C = st->cells[op][c->cell];
    int64_t *S = st->stats[op];
    const int dflt = default_variant(op);
    S[T_CALLS]++;
    if (c->variant == C.model && C.model != dflt) S[T_MODEL_CALLS]++;
    else S[T_DEFAULT_CALLS]++;
    S[T_LAST_VARIANT] = c->variant;
    S[T_LAST_US] = (int64_t)llround(ms * 1000.0);
    S[T_LAST_PRED_US] = (int64_t)llround(C.pred[c->variant] * 1000.0);
    switch (C.state) {
        case S_MODEL:
            if (C.model == dflt) {
                C.state = S_CONFIRMED;  // nothing to judge: the model agrees with the plain choice
            } else if (ms > C.pred[C.model] * (1.0f + st->tol)) {
                C.t_model = ms;  // slower than predicted: the plain variant runs next time
                C.state = S_TRIAL;
            }
            break;
        case S_TRIAL:
            S[T_TRIALS]++;
            if (c->variant == dflt) {
                if (ms < C.t_model) {
                    C.state = S_FALLBACK;
                    S[T_FALLBACKS]++;
                } else {
                    C.state = S_CONFIRMED;
                    S[T_CONFIRMED]++;
                }
            }
            break;
        default:
            break;
    }
}

extern "C" {

QG_API qg_status qg_steer_attach(qg_ctx *ctx, const float *d_params, float tolerance) {
    if (!ctx || !d_params || !(tolerance >= 0.0f)) return QG_ERR_INVALID;
    int total = 0;
    for (int op = 0; op < QG_STEER_OPS; op++) total += ncells(op) * NVAR[op];
    std::vector<float> X((size_t)total * NF);
    size_t r = 0;
    for (int op = 0; op < QG_STEER_OPS; op++)
        for (int c = 0; c < ncells(op); c++) {
            double n, n2, sel;
            cell_point(op, c, &n, &n2, &sel);
            for (int v = 0; v < NVAR[op]; v++) features(op, v, n, n2, sel, 0.0, &X[(r++) * NF]);
        }
    char *scr;
    const size_t xb = qg_align_up(X.size() * 4, 256);
    QG_TRY(qg_scratch(ctx, xb + (size_t)total * 4, &scr));
    float *dX = (float *)scr, *dY = (float *)(scr + xb);
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(dX, X.data(), X.size() * 4, cudaMemcpyHostToDevice, ctx->stream), "h2d");
    QG_TRY(qg_mlp_predict(ctx, d_params, dX, total, dY));  // the inference kernel; synchronises
    std::vector<float> Y((size_t)total);
    QG_TRY_CUDA(ctx, cudaMemcpy(Y.data(), dY, Y.size() * 4, cudaMemcpyDeviceToHost), "d2h");
    qg_steer_state *st = new qg_steer_state();
    st->tol = tolerance;
    memset(st->stats, 0, sizeof(st->stats));
    r = 0;
    for (int op = 0; op < QG_STEER_OPS; op++) {
        st->cells[op].resize((size_t)ncells(op));
        const int dflt = default_variant(op);
        for (Cell &C : st->cells[op]) {
            int best = 0;
            for (int v = 0; v < NV; v++) C.pred[v] = v < NVAR[op] ? expf(Y[r + v]) : INFINITY;
            for (int v = 1; v < NVAR[op]; v++)
                if (C.pred[v] < C.pred[best]) best = v;
            C.model = (int8_t)best;
            C.state = S_MODEL;
            C.t_model = 0.0f;
            r += NVAR[op];
            if (best != dflt) st->stats[op][T_CELLS_NONDEFAULT]++;
        }
    }
    if (cudaEventCreate(&st->ev0) != cudaSuccess || cudaEventCreate(&st->ev1) != cudaSuccess) {
        cudaGetLastError();
        delete st;
        return QG_ERR_CUDA;
    }
    qg_steer_free(ctx);
    ctx->steer = st;
    return QG_OK;
}

QG_API qg_status qg_steer_detach(qg_ctx *ctx) {
    if (!ctx) return QG_ERR_INVALID;
    qg_steer_free(ctx);
    return QG_OK;
}

QG_API qg_status qg_steer_choose(qg_ctx *ctx, int op, int64_t n, int64_t n2, float sel, int *variant,
                                 float *pred_ms) {
    if (!ctx || !variant || op < 0 || op >= QG_STEER_OPS || n < 0) return QG_ERR_INVALID;
    if (!ctx->steer) {
        *variant = default_variant(op);
        if (pred_ms) *pred_ms = 0.0f;
        return QG_OK;
    }
    const Cell &C = ctx->steer->cells[op][cell_of(op, n, n2, sel)];
    const int v = (C.state == S_TRIAL || C.state == S_FALLBACK) ? default_variant(op) : C.model;
    *variant = v;
    if (pred_ms) *pred_ms = C.pred[v];
    return QG_OK;
}

QG_API qg_status qg_steer_stats(qg_ctx *ctx, int op, int64_t *out10) {
    if (!ctx || !out10 || op < 0 || op >= QG_STEER_OPS) return QG_ERR_INVALID;
    for (int i = 0; i < T_N; i++) out10[i] = ctx->steer ? ctx->steer->stats[op][i] : 0;
    return QG_OK;
}

QG_API qg_status qg_steer_plan(qg_ctx *ctx, int sub_index, float size_m, qg_plan *out, int *variant) {
    if (!ctx || !ctx->steer || !out || sub_index < 0 || sub_index > 3 || !(size_m > 0.0f)) return QG_ERR_INVALID;
    // The operator each pipeline runs as on the GPU, and its primitives (the
    // scan primitives are fused into the operators' kernels: zero cost).
    static const int PRIM_FILTER[] = {QG_K_FILTER_MAP, QG_K_FILTER_WRITE};
    static const int PRIM_GROUP[] = {QG_K_SORT, QG_K_GROUP_LABEL, QG_K_GROUP_WRITE, QG_K_AGG};
    static const int PRIM_FUSED[] = {QG_K_FILTER_MAP, QG_K_FILTER_WRITE, QG_K_SORT, QG_K_GROUP_LABEL,
                                     QG_K_GROUP_WRITE, QG_K_AGG};
    int op = -1, nprim = 0;
    const int *prim = nullptr;
    double sel = 1.0;
    int64_t n2 = 0;
    switch (sub_index) {
        case 0: op = QG_STEER_FILTER; prim = PRIM_FILTER; nprim = 2; sel = 0.1; break;
        case 1: op = QG_STEER_GROUPBY; prim = PRIM_GROUP; nprim = 4; n2 = 1 << 20; break;
        case 2: op = QG_STEER_FUSED; prim = PRIM_FUSED; nprim = 6; n2 = 1 << 20; sel = 0.5; break;
        default: break;
    }
    const int64_t n = (int64_t)((double)size_m * 1048576.0);
    const Cell *C = op >= 0 ? &ctx->steer->cells[op][cell_of(op, n, n2, sel)] : nullptr;
    static const char *VNAME[QG_STEER_OPS][NV] = {
        {"gpu_filter_v0", "gpu_filter_v1", "gpu_filter_v2", ""},
        {"gpu_groupby_v0", "gpu_groupby_v1", "gpu_groupby_v2", "gpu_groupby_v3"},
        {"gpu_fused_v0", "gpu_fused_v1", "gpu_fused_v2", "gpu_fused_v3"},
        {"", "", "", ""}};
    std::vector<qg_plan_variant> rows;
    for (int k = 0; k < QG_K_NUM; k++) {
        bool mine = false;
        for (int i = 0; i < nprim; i++) mine |= prim[i] == k;
        if (!mine) {
            rows.push_back(qg_plan_variant{"fused_into_operator", k, 0, 0, 0, 0, 0.0f, 0.0f, 0.0f});
            continue;
        }
        for (int v = 0; v < NVAR[op]; v++)  // the variant's predicted ms per M rows, split over its primitives
            rows.push_back(qg_plan_variant{VNAME[op][v], k, 0, 0, 0, 0,
                                           (float)(C->pred[v] / nprim / size_m), 0.0f, 0.0f});
    }
    QG_TRY(qg_plan_pipeline_rows(rows.data(), (int)rows.size(), 0, sub_index, size_m, out));
    if (variant) {
        *variant = -1;
        for (int i = 0; i < out->image_num && *variant < 0; i++)
            for (int j = 0; j < out->images[i].num_kernels; j++)
                if (out->images[i].kernels[j].kernel_id == (nprim ? prim[0] : -1)) {
                    *variant = out->images[i].kernels[j].variant;
                    break;
                }
    }
    return QG_OK;
}

}  // extern "C"
