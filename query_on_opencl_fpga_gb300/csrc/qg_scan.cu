// qg_scan.cu -- single-pass exclusive int32 prefix sum.
//
// Replaces the reference's multi-level Blelloch scan
// (ScanLargeArrays_kernel / prefixSum_kernel / blockAddition_kernel,
// kernel/filter/filter_op.cl:51-207, driven by host/host/testScan.cpp:26-340
// with 2*pass+1 launches and per-level buffers).  One kernel: each tile is
// scanned in registers and shared memory, the tile's carry-in comes from a
// decoupled look-back.  Arithmetic wraps mod 2^32 like the reference's int
// adds, and any n >= 0 is accepted (the reference needs n > 65536,
// testScan.cpp:317-318, and block-aligned sizes).
#include "qg_internal.cuh"

namespace {

constexpr int SC_THREADS = 256;
constexpr int SC_WARPS = SC_THREADS / 32;
constexpr int SC_ROUNDS = 4;  // int4 loads per thread: 4096 ints per tile

template <bool VEC>
__global__ void __launch_bounds__(SC_THREADS)
k_scan_excl(const int32_t *in, int32_t *out, long long n, qg_lookback lb) {
    constexpr int TILE = SC_THREADS * SC_ROUNDS * 4;
    __shared__ uint32_t s_tile, s_epoch, s_excl;
    __shared__ uint32_t s_woff[SC_ROUNDS * SC_WARPS];
    qg_lb_begin(lb, &s_tile, &s_epoch);
    const uint32_t tile = s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long base = (long long)tile * TILE;

    uint32_t v[SC_ROUNDS][4];
    uint32_t texcl[SC_ROUNDS];  // exclusive prefix of this thread within its warp, per round
#pragma unroll
    for (int r = 0; r < SC_ROUNDS; r++) {
        long long idx = base + (long long)(r * SC_THREADS + tid) * 4;
        if (VEC && idx + 3 < n) {
            int4 t = *reinterpret_cast<const int4 *>(in + idx);
            v[r][0] = t.x; v[r][1] = t.y; v[r][2] = t.z; v[r][3] = t.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++) v[r][j] = (idx + j < n) ? (uint32_t)in[idx + j] : 0u;
        }
    }
    // Loads of all rounds are in flight before the first shared store.
#pragma unroll
    for (int r = 0; r < SC_ROUNDS; r++) {
        uint32_t s = v[r][0] + v[r][1] + v[r][2] + v[r][3];
        uint32_t inc = s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(QG_FULL_MASK, inc, d);
            if (lane >= d) inc += t;
        }
        texcl[r] = inc - s;
        if (lane == 31) s_woff[r * SC_WARPS + warp] = inc;
    }
    __syncthreads();
    if (warp == 0) {
        constexpr int E = SC_ROUNDS * SC_WARPS;  // 32: one entry per lane
        uint32_t x = (lane < E) ? s_woff[lane] : 0u;
        uint32_t inc = x;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(QG_FULL_MASK, inc, d);
            if (lane >= d) inc += t;
        }
        uint32_t total = __shfl_sync(QG_FULL_MASK, inc, 31);
        if (lane < E) s_woff[lane] = inc - x;
        uint32_t excl = qg_lb_warp_exclusive(lb, tile, s_epoch, total);
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    const uint32_t excl = s_excl;
#pragma unroll
    for (int r = 0; r < SC_ROUNDS; r++) {
        long long idx = base + (long long)(r * SC_THREADS + tid) * 4;
        uint32_t run = excl + s_woff[r * SC_WARPS + warp] + texcl[r];
        uint32_t o[4];
#pragma unroll
        for (int j = 0; j < 4; j++) { o[j] = run; run += v[r][j]; }
        if (VEC && idx + 3 < n) {
            *reinterpret_cast<int4 *>(out + idx) = make_int4(o[0], o[1], o[2], o[3]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++)
                if (idx + j < n) out[idx + j] = (int32_t)o[j];
        }
    }
    qg_lb_finish(lb, tile, gridDim.x - 1, s_epoch);
}

}  // namespace

qg_status qg_scan_launch(qg_ctx *ctx, const int32_t *in, int32_t *out, int64_t n) {
    constexpr int TILE = SC_THREADS * SC_ROUNDS * 4;
    if (n == 0) return QG_OK;
    int64_t tiles = qg_ceil_div(n, TILE);
    if (tiles > 0x7fffffff) return QG_ERR_UNSUPPORTED;
    qg_lookback lb;
    QG_TRY(qg_lb_make(ctx, tiles, QG_SITE_SCAN, &lb));
    bool vec = (((uintptr_t)in | (uintptr_t)out) & 15) == 0;
    qg_pre_launch(ctx);
    if (vec)
        k_scan_excl<true><<<(unsigned)tiles, SC_THREADS, 0, ctx->stream>>>(in, out, n, lb);
    else
        k_scan_excl<false><<<(unsigned)tiles, SC_THREADS, 0, ctx->stream>>>(in, out, n, lb);
    return qg_check_launch(ctx, "k_scan_excl");
}

extern "C" QG_API qg_status qg_scan_excl_i32(qg_ctx *ctx, const int32_t *in, int32_t *out,
                                             int64_t n) {
    if (!ctx || n < 0 || (n > 0 && (!in || !out))) return QG_ERR_INVALID;
    if ((((uintptr_t)in) | ((uintptr_t)out)) & 3) return QG_ERR_INVALID;
    return qg_scan_launch(ctx, in, out, n);
}
