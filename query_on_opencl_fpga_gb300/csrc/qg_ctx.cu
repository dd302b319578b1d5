// qg_ctx.cu -- context, scratch arena, error word and buffer helpers.
//
// Replaces the reference's launch/buffer glue (host/host/common.cpp:13-125)
// and its error convention (src/AOCL_Utils.cpp:228-252 prints and exits):
// here every call returns a status and the device records the first error in
// a control word that the host reads after synchronising.
#include <stdlib.h>
#include <string.h>
#include "qg_internal.cuh"

extern "C" {

QG_API const char *qg_status_string(qg_status s) {
    switch (s) {
        case QG_OK: return "ok";
        case QG_ERR_INVALID: return "invalid argument";
        case QG_ERR_CUDA: return "CUDA runtime error";
        case QG_ERR_CAPACITY: return "output capacity exceeded";
        case QG_ERR_TABLE_FULL: return "hash table full";
        case QG_ERR_TIMEOUT: return "device wait timed out";
        case QG_ERR_OOM: return "device scratch allocation failed";
        case QG_ERR_UNSUPPORTED: return "unsupported size or option";
    }
    return "unknown status";
}

QG_API qg_status qg_ctx_create(qg_ctx **out, void *stream) {
    if (!out) return QG_ERR_INVALID;
    *out = nullptr;
    qg_ctx *ctx = (qg_ctx *)calloc(1, sizeof(qg_ctx));
    if (!ctx) return QG_ERR_OOM;
    ctx->stream = (cudaStream_t)stream;
    ctx->spin_limit = 1u << 22;
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) e = cudaMalloc((void **)&ctx->ctl, sizeof(qg_control));
    if (e == cudaSuccess) e = cudaMemset(ctx->ctl, 0, sizeof(qg_control));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ctx->pinned, 8 * sizeof(long long));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ctx->pin_ctl, sizeof(qg_control));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ctx->pin_bases, 8 * 1024 * sizeof(uint32_t));
    for (int i = 0; i < 8 && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&ctx->pin_ev[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        if (ctx->ctl) cudaFree(ctx->ctl);
        if (ctx->pinned) cudaFreeHost(ctx->pinned);
        if (ctx->pin_ctl) cudaFreeHost(ctx->pin_ctl);
        if (ctx->pin_bases) cudaFreeHost(ctx->pin_bases);
        for (int i = 0; i < 8; i++)
            if (ctx->pin_ev[i]) cudaEventDestroy(ctx->pin_ev[i]);
        free(ctx);
        return QG_ERR_CUDA;
    }
    ctx->table_dirty = true;
    for (int i = 0; i < QG_STEER_OPS; i++) ctx->steer_force[i] = -1;
    *out = ctx;
    return QG_OK;
}

QG_API qg_status qg_ctx_destroy(qg_ctx *ctx) {
    if (!ctx) return QG_ERR_INVALID;
    cudaStreamSynchronize(ctx->stream);
    qg_steer_free(ctx);
    if (ctx->ev[0])
        for (int i = 0; i < 2 * QG_MAX_TIMED; i++) cudaEventDestroy(ctx->ev[i]);
    if (ctx->scratch) cudaFree(ctx->scratch);
    if (ctx->lbstat) cudaFree(ctx->lbstat);
    if (ctx->pj_tmp) cudaFree(ctx->pj_tmp);
    if (ctx->table) cudaFree(ctx->table);
    if (ctx->aux) cudaFree(ctx->aux);
    if (ctx->ctl) cudaFree(ctx->ctl);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->pin_ctl) cudaFreeHost(ctx->pin_ctl);
    if (ctx->pin_bases) cudaFreeHost(ctx->pin_bases);
    if (ctx->pin_join) cudaFreeHost(ctx->pin_join);
    for (int i = 0; i < 8; i++)
        if (ctx->pin_ev[i]) cudaEventDestroy(ctx->pin_ev[i]);
    free(ctx);
    return QG_OK;
}

QG_API qg_status qg_ctx_set_stream(qg_ctx *ctx, void *stream) {
    if (!ctx) return QG_ERR_INVALID;
    ctx->stream = (cudaStream_t)stream;
    return QG_OK;
}

QG_API qg_status qg_ctx_sync(qg_ctx *ctx) {
    if (!ctx) return QG_ERR_INVALID;
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return QG_OK;
}

QG_API qg_status qg_ctx_set_spin_limit(qg_ctx *ctx, uint32_t polls) {
    if (!ctx) return QG_ERR_INVALID;
    ctx->spin_limit = polls;
    return QG_OK;
}

QG_API qg_status qg_ctx_check(qg_ctx *ctx) {
    if (!ctx) return QG_ERR_INVALID;
    return qg_collect_error(ctx);  // waits for the stream's work
}

QG_API const char *qg_last_error_message(qg_ctx *ctx) { return ctx ? ctx->msg : "no context"; }

QG_API size_t qg_ctx_scratch_bytes(qg_ctx *ctx) { return ctx ? ctx->scratch_bytes : 0; }

QG_API uint64_t qg_ctx_launch_count(qg_ctx *ctx) { return ctx ? ctx->launches : 0; }

QG_API qg_status qg_ctx_reserve(qg_ctx *ctx, size_t bytes) {
    if (!ctx) return QG_ERR_INVALID;
    char *p;
    return qg_scratch(ctx, bytes, &p);
}

QG_API qg_status qg_malloc(qg_ctx *ctx, void **ptr, size_t bytes) {
    if (!ctx || !ptr) return QG_ERR_INVALID;
    *ptr = nullptr;
    cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        snprintf(ctx->msg, sizeof(ctx->msg), "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
        return QG_ERR_OOM;
    }
    return QG_OK;
}

QG_API qg_status qg_free(qg_ctx *ctx, void *ptr) {
    if (!ctx) return QG_ERR_INVALID;
    if (!ptr) return QG_OK;
    cudaStreamSynchronize(ctx->stream);
    QG_TRY_CUDA(ctx, cudaFree(ptr), "cudaFree");
    return QG_OK;
}

}  // extern "C"

qg_status qg_cuda_fail(qg_ctx *ctx, cudaError_t e, const char *what) {
    snprintf(ctx->msg, sizeof(ctx->msg), "%s: %s", what, cudaGetErrorString(e));
    cudaGetLastError();
    return QG_ERR_CUDA;
}



void qg_pre_launch(qg_ctx *ctx) {
    if (!ctx->timing || ctx->ev_used >= QG_MAX_TIMED) return;
    cudaEventRecord(ctx->ev[2 * ctx->ev_used], ctx->stream);
}

qg_status qg_check_launch(qg_ctx *ctx, const char *what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return qg_cuda_fail(ctx, e, what);
    if (ctx->timing && ctx->ev_used < QG_MAX_TIMED) {
        cudaEventRecord(ctx->ev[2 * ctx->ev_used + 1], ctx->stream);
        ctx->ev_name[ctx->ev_used] = what;
        ctx->ev_used++;
    }
    return QG_OK;
}

extern "C" {

QG_API qg_status qg_ctx_enable_timing(qg_ctx *ctx, int on) {
    if (!ctx) return QG_ERR_INVALID;
    if (on && !ctx->ev[0]) {
        for (int i = 0; i < 2 * QG_MAX_TIMED; i++)
            QG_TRY_CUDA(ctx, cudaEventCreate(&ctx->ev[i]), "cudaEventCreate");
    }
    ctx->timing = on != 0;
    ctx->ev_used = 0;
    return QG_OK;
}

// After synchronising: milliseconds from the start of the first launch to
// the end of the last launch logged since timing was enabled (or the last
// report) -- an operator's device span including the gaps between its
// kernels.  -1 when nothing was logged.
QG_API double qg_ctx_timing_span(qg_ctx *ctx) {
    if (!ctx || !ctx->timing || ctx->ev_used == 0) return -1.0;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return -1.0;
    float ms = -1.f;
    if (cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[2 * (ctx->ev_used - 1) + 1]) != cudaSuccess) return -1.0;
    return ms;
}

// After synchronising: one "name launches total_ms" line per kernel name for
// the launches since the last report (or enable), then resets the log.
QG_API int qg_ctx_timing_report(qg_ctx *ctx, char *buf, size_t len) {
    if (!ctx || !buf || len == 0) return -1;
    buf[0] = 0;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return -1;
    const char *names[QG_MAX_TIMED];
    double tot[QG_MAX_TIMED];
    int cnt[QG_MAX_TIMED];
    int k = 0;
    for (int i = 0; i < ctx->ev_used; i++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[2 * i], ctx->ev[2 * i + 1]);
        int j = 0;
        while (j < k && strcmp(names[j], ctx->ev_name[i]) != 0) j++;
        if (j == k) { names[k] = ctx->ev_name[i]; tot[k] = 0; cnt[k] = 0; k++; }
        tot[j] += ms;
        cnt[j]++;
    }
    size_t off = 0;
    for (int j = 0; j < k && off < len; j++)
        off += snprintf(buf + off, len - off, "%s %d %.6f\n", names[j], cnt[j], tot[j]);
    ctx->ev_used = 0;
    return k;
}

}  // extern "C"

qg_status qg_scratch(qg_ctx *ctx, size_t bytes, char **out) {
    bytes = qg_align_up(bytes ? bytes : 256, 256);
    if (bytes > ctx->scratch_bytes) {
        // Grow by at least 25% to avoid repeated reallocation.
        size_t want = bytes + bytes / 4;
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        if (ctx->scratch) cudaFree(ctx->scratch);
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
        cudaError_t e = cudaMalloc((void **)&ctx->scratch, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            snprintf(ctx->msg, sizeof(ctx->msg), "scratch cudaMalloc(%zu): %s", want,
                     cudaGetErrorString(e));
            return QG_ERR_OOM;
        }
        QG_TRY_CUDA(ctx, cudaMemset(ctx->scratch, 0, want), "cudaMemset scratch");
        QG_TRY_CUDA(ctx, cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        ctx->scratch_bytes = want;
    }
    *out = ctx->scratch;
    return QG_OK;
}

qg_status qg_lb_make(qg_ctx *ctx, int64_t tiles, int site, qg_lookback *out) {
    const size_t words = (size_t)(tiles > 0 ? tiles : 1);
    if (words > ctx->lbstat_words) {
        const size_t want = words + words / 4 + 1024;
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        if (ctx->lbstat) cudaFree(ctx->lbstat);
        ctx->lbstat = nullptr;
        ctx->lbstat_words = 0;
        cudaError_t e = cudaMalloc((void **)&ctx->lbstat, want * 8);
        if (e != cudaSuccess) {
            cudaGetLastError();
            snprintf(ctx->msg, sizeof(ctx->msg), "look-back status cudaMalloc(%zu): %s", want * 8,
                     cudaGetErrorString(e));
            return QG_ERR_OOM;
        }
        QG_TRY_CUDA(ctx, cudaMemset(ctx->lbstat, 0, want * 8), "cudaMemset look-back status");
        QG_TRY_CUDA(ctx, cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        ctx->lbstat_words = want;
    }
    *out = qg_lookback{ctx->lbstat, ctx->ctl, ctx->spin_limit, site};
    return QG_OK;
}

qg_status qg_aux(qg_ctx *ctx, size_t bytes, char **out) {
    bytes = qg_align_up(bytes ? bytes : 256, 256);
    if (bytes > ctx->aux_bytes) {
        size_t want = bytes + bytes / 4;
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        if (ctx->aux) cudaFree(ctx->aux);
        ctx->aux = nullptr;
        ctx->aux_bytes = 0;
        cudaError_t e = cudaMalloc((void **)&ctx->aux, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            snprintf(ctx->msg, sizeof(ctx->msg), "aux cudaMalloc(%zu): %s", want,
                     cudaGetErrorString(e));
            return QG_ERR_OOM;
        }
        ctx->aux_bytes = want;
    }
    *out = ctx->aux;
    return QG_OK;
}

qg_status qg_table(qg_ctx *ctx, size_t bytes, char **out) {
    bytes = qg_align_up(bytes ? bytes : 256, 256);
    if (bytes > ctx->table_bytes) {
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        if (ctx->table) cudaFree(ctx->table);
        ctx->table = nullptr;
        ctx->table_bytes = 0;
        cudaError_t e = cudaMalloc((void **)&ctx->table, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            snprintf(ctx->msg, sizeof(ctx->msg), "table cudaMalloc(%zu): %s", bytes,
                     cudaGetErrorString(e));
            return QG_ERR_OOM;
        }
        ctx->table_bytes = bytes;
        ctx->table_dirty = true;
    }
    if (ctx->table_dirty) {
        QG_TRY_CUDA(ctx, cudaMemsetAsync(ctx->table, 0, ctx->table_bytes, ctx->stream),
                    "cudaMemsetAsync table");
        ctx->table_dirty = false;
    }
    *out = ctx->table;
    return QG_OK;
}

qg_status qg_stage_bases(qg_ctx *ctx, const uint32_t *h_bases, uint32_t *d_dst) {
    const int slot = ctx->pin_next;
    ctx->pin_next = (slot + 1) & 7;
    QG_TRY_CUDA(ctx, cudaEventSynchronize(ctx->pin_ev[slot]), "wait bases slot");
    uint32_t *p = ctx->pin_bases + (size_t)slot * 1024;
    memcpy(p, h_bases, 1024 * sizeof(uint32_t));
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(d_dst, p, 1024 * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream),
                "bases h2d");
    QG_TRY_CUDA(ctx, cudaEventRecord(ctx->pin_ev[slot], ctx->stream), "record bases slot");
    return QG_OK;
}

qg_status qg_read_i64(qg_ctx *ctx, const long long *d, long long *h) {
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pinned, d, sizeof(long long), cudaMemcpyDeviceToHost,
                                     ctx->stream),
                "cudaMemcpyAsync count");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    *h = ctx->pinned[0];
    return QG_OK;
}

// Pinned slot 7 receives the error word and its site.
static qg_status map_error(qg_ctx *ctx, const int32_t *h) {
    if (h[0] == 0) return QG_OK;
    // A kernel that gave up may have left the single-pass counters or the
    // group-by table mid-way: reset them (in stream order).
    cudaMemsetAsync(&ctx->ctl->err, 0, 2 * sizeof(int32_t), ctx->stream);
    cudaMemsetAsync(&ctx->ctl->tile_ctr, 0, 2 * sizeof(uint32_t), ctx->stream);
    cudaMemsetAsync(ctx->ctl->gbd, 0, sizeof(ctx->ctl->gbd), ctx->stream);  // dense group-by state words
    cudaStreamSynchronize(ctx->stream);  // done before any later stream of this context runs
    ctx->table_dirty = true;
    snprintf(ctx->msg, sizeof(ctx->msg), "device error %d (%s) at site %d", h[0],
             qg_status_string((qg_status)h[0]), h[1]);
    return (qg_status)h[0];
}

qg_status qg_collect_error(qg_ctx *ctx) {
    int32_t *h = reinterpret_cast<int32_t *>(ctx->pinned + 7);
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(h, &ctx->ctl->err, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream),
                "read error word");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return map_error(ctx, h);
}

qg_status qg_read_count(qg_ctx *ctx, const long long *d, long long *h) {
    const uintptr_t base = (uintptr_t)ctx->ctl, at = (uintptr_t)d;
    const size_t off = (size_t)(at - base);
    if (at >= base && off + sizeof(long long) <= offsetof(qg_control, gbd)) {
        // A count kept in the control block comes back with the error word
        // in one copy.
        QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pin_ctl, ctx->ctl, off + sizeof(long long), cudaMemcpyDeviceToHost,
                                         ctx->stream),
                    "cudaMemcpyAsync count");
        QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        memcpy(h, (const char *)ctx->pin_ctl + off, sizeof(long long));
        const int32_t e[2] = {ctx->pin_ctl->err, ctx->pin_ctl->err_site};
        return map_error(ctx, e);
    }
    int32_t *e = reinterpret_cast<int32_t *>(ctx->pinned + 7);
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(ctx->pinned, d, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream),
                "cudaMemcpyAsync count");
    QG_TRY_CUDA(ctx, cudaMemcpyAsync(e, &ctx->ctl->err, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream),
                "read error word");
    QG_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    *h = ctx->pinned[0];
    return map_error(ctx, e);
}
