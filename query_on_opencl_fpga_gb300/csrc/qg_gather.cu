// qg_gather.cu -- record gather and scatter.
//
// Reference: gatherImpl / scatterImpl (host/host/testScatter.cpp:63-137) run
// optGather_kernel / optScatter_kernel in 8 runs of loc ranges; only the gather
// kernel's body survives, commented out, in
// kernel/aggregation/1/group_by_cu_op_dp.cl:860-872:
//     if (from <= loc[pos] < to) S[pos] = R[loc[pos]]
// Over the 8 runs that covers every loc in [0, rLen): S[i] = R[loc[i]], and a
// loc outside [0, rLen) leaves S[i] untouched.  The scatter is the inverse,
// S[loc[i]] = R[i] for loc in [0, sLen).  One launch each here; loc may be
// strided so that a Record array's .x (the row id after a sort) serves as loc
// directly, which is how aggAfterGroupByImpl uses it
// (host/host/testAggAfterGB.cpp:39-67).
#include "qg_internal.cuh"

namespace {

__global__ void k_gather_rec(const uint2 *__restrict__ R, long long rLen,
                             const int32_t *__restrict__ loc, long long stride, long long sLen,
                             uint2 *__restrict__ S) {
    const long long step = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < sLen; i += step) {
        const long long t = __ldg(loc + i * stride);
        if (t >= 0 && t < rLen) S[i] = __ldg(R + t);
    }
}

__global__ void k_scatter_rec(const uint2 *__restrict__ R, long long rLen,
                              const int32_t *__restrict__ loc, long long stride, long long sLen,
                              uint2 *__restrict__ S) {
    const long long step = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < rLen; i += step) {
        const long long t = __ldg(loc + i * stride);
        if (t >= 0 && t < sLen) S[t] = __ldg(R + i);
    }
}

int grid_of(qg_ctx *ctx, long long n) {
    long long b = (n + 255) / 256, cap = (long long)ctx->sm_count * 8;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

extern "C" QG_API qg_status qg_gather_rec(qg_ctx *ctx, const void *R, int64_t rLen,
                                          const int32_t *loc, int64_t loc_stride, int64_t sLen,
                                          void *S) {
    if (!ctx || rLen < 0 || sLen < 0 || loc_stride < 1) return QG_ERR_INVALID;
    if (sLen == 0) return QG_OK;
    if (!R || !loc || !S || (((uintptr_t)R | (uintptr_t)S) & 7) || ((uintptr_t)loc & 3))
        return QG_ERR_INVALID;
    qg_pre_launch(ctx);
    k_gather_rec<<<grid_of(ctx, sLen), 256, 0, ctx->stream>>>((const uint2 *)R, rLen, loc, loc_stride,
                                                              sLen, (uint2 *)S);
    return qg_check_launch(ctx, "k_gather_rec");
}

extern "C" QG_API qg_status qg_scatter_rec(qg_ctx *ctx, const void *R, int64_t rLen,
                                           const int32_t *loc, int64_t loc_stride, void *S,
                                           int64_t sLen) {
    if (!ctx || rLen < 0 || sLen < 0 || loc_stride < 1) return QG_ERR_INVALID;
    if (rLen == 0) return QG_OK;
    if (!R || !loc || !S || (((uintptr_t)R | (uintptr_t)S) & 7) || ((uintptr_t)loc & 3))
        return QG_ERR_INVALID;
    qg_pre_launch(ctx);
    k_scatter_rec<<<grid_of(ctx, rLen), 256, 0, ctx->stream>>>((const uint2 *)R, rLen, loc, loc_stride,
                                                               sLen, (uint2 *)S);
    return qg_check_launch(ctx, "k_scatter_rec");
}
