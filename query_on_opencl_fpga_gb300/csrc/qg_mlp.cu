// qg_mlp.cu -- the learned cost model: a 16 -> 64 (ReLU) -> 1 fp32 MLP that
// predicts the log run time of an operator variant from plan features.
//
// It stands beside the reference's static cost model (the per-variant unit
// costs of host/dynamic_programming.cpp:152-167, which describe FPGA images):
// trained on timings the engine records on this GPU, it predicts what each
// operator variant costs here; the host uses the predictions to choose
// kernel variants and to fill the planner's cost table (qg_plan_set_table).
// The plain table stays the fallback, and results are bit-exact whichever
// variant is chosen.
//
// Parameters, one fp32 array of QG_MLP_PARAMS:
//   W1[64][16], b1[64], W2[64], b2[1]
// Training: mean squared error over a batch, Adam.  Every gradient is a
// per-parameter sum over the batch in sample order (no atomics), so training
// is deterministic.
#include <math.h>
#include "qg_internal.cuh"

namespace {

constexpr int MI = 16, MH = 64;
// parameter layout: W1 at 0, then b1, W2, b2
constexpr int P_B1 = MI * MH, P_W2 = P_B1 + MH, P_B2 = P_W2 + MH;
constexpr int NPARAM = P_B2 + 1;  // 1153

// Forward for n samples; keeps the hidden pre-activations (for backward) when z != null.
__global__ void __launch_bounds__(MH)
k_mlp_fwd(const float *__restrict__ p, const float *__restrict__ X, int n, float *__restrict__ out,
          float *__restrict__ z) {
    __shared__ float w1[MH * MI + MH];
    __shared__ float red[MH / 32];
    const int j = threadIdx.x;
    for (int i = j; i < MH * MI + MH; i += MH) w1[i] = p[i];
    __syncthreads();
    const float w2 = p[P_W2 + j], b2 = p[P_B2];
    for (int s = blockIdx.x; s < n; s += gridDim.x) {
        const float *x = X + (size_t)s * MI;
        float a = w1[P_B1 + j];
#pragma unroll
        for (int k = 0; k < MI; k++) a = fmaf(w1[j * MI + k], __ldg(x + k), a);
        if (z) z[(size_t)s * MH + j] = a;
        float v = fmaxf(a, 0.0f) * w2;
        // fixed-order reduction over the 64 hidden units
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(QG_FULL_MASK, v, d);
        if ((j & 31) == 0) red[j >> 5] = v;
        __syncthreads();
        if (j == 0) out[s] = red[0] + red[1] + b2;
        __syncthreads();
    }
}

// Gradient of L = mean((out - y)^2) with respect to every parameter, from
// the forward's outputs and pre-activations.  One thread per parameter,
// summing over samples in order.
__global__ void k_mlp_bwd(const float *__restrict__ p, const float *__restrict__ X, const float *__restrict__ y,
                          int n, const float *__restrict__ out, const float *__restrict__ z,
                          float *__restrict__ grad) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= NPARAM) return;
    const float inv = 2.0f / (float)n;
    float g = 0.0f;
    if (q < P_B1) {  // W1[j][k]
        const int j = q / MI, k = q % MI;
        const float w2 = p[P_W2 + j];
        for (int s = 0; s < n; s++)
            if (z[(size_t)s * MH + j] > 0.0f) g = fmaf((out[s] - y[s]) * w2, X[(size_t)s * MI + k], g);
    } else if (q < P_W2) {  // b1[j]
        const int j = q - P_B1;
        const float w2 = p[P_W2 + j];
        for (int s = 0; s < n; s++)
            if (z[(size_t)s * MH + j] > 0.0f) g += (out[s] - y[s]) * w2;
    } else if (q < P_B2) {  // W2[j]
        const int j = q - P_W2;
        for (int s = 0; s < n; s++) g = fmaf(out[s] - y[s], fmaxf(z[(size_t)s * MH + j], 0.0f), g);
    } else {  // b2
        for (int s = 0; s < n; s++) g += out[s] - y[s];
    }
    grad[q] = g * inv;
}

__global__ void k_mlp_loss(const float *__restrict__ out, const float *__restrict__ y, int n,
                           float *__restrict__ loss) {
    __shared__ float red[32];
    float v = 0.0f;
    for (int s = threadIdx.x; s < n; s += blockDim.x) {
        const float d = out[s] - y[s];
        v = fmaf(d, d, v);
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(QG_FULL_MASK, v, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        *loss = t / (float)n;
    }
}

// Adam step (t = step number, 1-based).
__global__ void k_mlp_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                           float *__restrict__ v, int t, float lr) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= NPARAM) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float mq = b1 * m[q] + (1.0f - b1) * g[q];
    const float vq = b2 * v[q] + (1.0f - b2) * g[q] * g[q];
    m[q] = mq;
    v[q] = vq;
    const float mh = mq / (1.0f - powf(b1, (float)t));
    const float vh = vq / (1.0f - powf(b2, (float)t));
    p[q] -= lr * mh / (sqrtf(vh) + eps);
}

// Deterministic initialisation: uniform(-a, a) from a 32-bit integer hash of
// (seed, index), a = 1/sqrt(fan_in); biases zero.
__global__ void k_mlp_init(float *__restrict__ p, uint32_t seed) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= NPARAM) return;
    uint32_t h = seed * 0x9E3779B9u ^ (uint32_t)q * 0x85EBCA6Bu;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    const float u = (float)(h >> 8) * (1.0f / 16777216.0f) * 2.0f - 1.0f;  // [-1, 1)
    float v = 0.0f;
    if (q < P_B1) v = u * 0.25f;             // 1/sqrt(16)
    else if (q >= P_W2 && q < P_B2) v = u * 0.125f;  // 1/sqrt(64)
    p[q] = v;
}

}  // namespace

extern "C" QG_API int64_t qg_mlp_param_count(void) { return NPARAM; }

extern "C" QG_API qg_status qg_mlp_init(qg_ctx *ctx, float *params, uint32_t seed) {
    if (!ctx || !params) return QG_ERR_INVALID;
    qg_pre_launch(ctx);
    k_mlp_init<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(params, seed);
    QG_TRY(qg_check_launch(ctx, "k_mlp_init"));
    return qg_ctx_check(ctx);
}

extern "C" QG_API qg_status qg_mlp_predict(qg_ctx *ctx, const float *params, const float *X, int64_t n,
                                           float *out) {
    if (!ctx || !params || n < 0 || n > (1 << 24) || (n > 0 && (!X || !out))) return QG_ERR_INVALID;
    if (n == 0) return QG_OK;
    const int grid = (int)(n < ctx->sm_count * 16LL ? n : ctx->sm_count * 16LL);
    qg_pre_launch(ctx);
    k_mlp_fwd<<<grid, MH, 0, ctx->stream>>>(params, X, (int)n, out, nullptr);
    QG_TRY(qg_check_launch(ctx, "k_mlp_fwd"));
    return qg_ctx_check(ctx);
}

// Needs n * (64 + 1) floats of work space; takes it from the context's scratch.
static qg_status mlp_fwd_bwd(qg_ctx *ctx, const float *params, const float *X, const float *y, int n,
                             float *grad, float *loss) {
    char *scr;
    QG_TRY(qg_scratch(ctx, (size_t)n * (MH + 1) * 4 + 256, &scr));
    float *out = (float *)scr, *z = out + qg_align_up((size_t)n, 64);
    const int grid = n < ctx->sm_count * 16 ? n : ctx->sm_count * 16;
    qg_pre_launch(ctx);
    k_mlp_fwd<<<grid, MH, 0, ctx->stream>>>(params, X, n, out, z);
    QG_TRY(qg_check_launch(ctx, "k_mlp_fwd"));
    if (loss) {
        qg_pre_launch(ctx);
        k_mlp_loss<<<1, 1024, 0, ctx->stream>>>(out, y, n, loss);
        QG_TRY(qg_check_launch(ctx, "k_mlp_loss"));
    }
    qg_pre_launch(ctx);
    k_mlp_bwd<<<(NPARAM + 127) / 128, 128, 0, ctx->stream>>>(params, X, y, n, out, z, grad);
    return qg_check_launch(ctx, "k_mlp_bwd");
}

extern "C" QG_API qg_status qg_mlp_grad(qg_ctx *ctx, const float *params, const float *X, const float *y,
                                        int64_t n, float *grad, float *loss) {
    if (!ctx || !params || !X || !y || !grad || n <= 0 || n > (1 << 20)) return QG_ERR_INVALID;
    QG_TRY(mlp_fwd_bwd(ctx, params, X, y, (int)n, grad, loss));
    return qg_ctx_check(ctx);
}

// `steps` full-batch Adam steps.  opt holds 3 * param_count floats (gradient,
// first and second moments; zero them before the first call of a run) and
// *t counts steps across calls.  loss (device, may be null) receives the
// loss of the last step's forward pass.
extern "C" QG_API qg_status qg_mlp_train(qg_ctx *ctx, float *params, const float *X, const float *y,
                                         int64_t n, int steps, float lr, float *opt, int *t, float *loss) {
    if (!ctx || !params || !X || !y || !opt || !t || n <= 0 || n > (1 << 20) || steps < 0 || !(lr > 0.0f))
        return QG_ERR_INVALID;
    float *g = opt, *m = opt + NPARAM, *v = opt + 2 * NPARAM;
    for (int i = 0; i < steps; i++) {
        QG_TRY(mlp_fwd_bwd(ctx, params, X, y, (int)n, g, i == steps - 1 ? loss : nullptr));
        ++*t;
        qg_pre_launch(ctx);
        k_mlp_adam<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(params, g, m, v, *t, lr);
        QG_TRY(qg_check_launch(ctx, "k_mlp_adam"));
    }
    return qg_ctx_check(ctx);
}
