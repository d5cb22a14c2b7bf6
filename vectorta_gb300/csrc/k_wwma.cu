// Weighted-window moving averages on CUDA cores (FP32 FMA):
//   out[c][t] = sum_k W[c][k] * x[t - K + 1 + k]
// with the rows of W right-aligned (zero-padded on the left) to a common K.
// This is the "plain FP32 kernel" path: the comparison baseline for the
// tcgen05 contraction and the path for shapes the contraction does not take.
//
// Batch tile: 16 combos x 256 times per 128-thread block; each thread keeps a
// 4-combo x 8-time register tile and slides a 16-register window of x over the
// shared-memory copy of the series span (8 new loads per 256 FMAs).
#include "vta_internal.h"

namespace vta {
namespace {

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }
__device__ __forceinline__ int pad32(int i) { return i + (i >> 5); }  // bank-spread index

constexpr int kBT = 256;     // times per block
constexpr int kBC = 16;      // combos per block
constexpr int kThreads = 128;

__global__ void __launch_bounds__(kThreads)
k_wwma_batch_plain(WwmaBatchArgs a) {
    extern __shared__ float sm[];
    const int t0 = blockIdx.x * kBT;
    const int cb = blockIdx.y * kBC;
    const int K = a.tile_kmax[blockIdx.y];
    const int K8 = (K + 7) & ~7;
    const int span = kBT + K8 - 1 + 8;  // +8: the window read-ahead past the last k
    float* ws = sm;                      // [kBC][K8]
    float* xs = sm + kBC * K8;           // padded span
    // weights, right-aligned to K8 within the tile
    for (int i = threadIdx.x; i < kBC * K8; i += kThreads) {
        const int c = i / K8, k = i - c * K8;
        const int cg = cb + c;
        float w = 0.f;
        const int kk = a.kmax - K8 + k;  // column in the global right-aligned matrix
        if (cg < a.n_combos && kk >= 0) w = a.w[(size_t)cg * a.kmax + kk];
        ws[i] = w;
    }
    const int xb = t0 - K8 + 1;
    for (int i = threadIdx.x; i < span; i += kThreads) {
        const int g = xb + i;
        float v = 0.f;
        if (g >= a.first && g < a.n) {
            v = a.x[g];
            if (isnan(v)) v = 0.f;  // masked in the epilogue
        }
        xs[pad32(i)] = v;
    }
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cw = warp * 4;  // this warp's 4 combos within the tile
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    const int xl = lane * 8;
    float xw[16];
#pragma unroll
    for (int j = 0; j < 8; ++j) xw[j] = xs[pad32(xl + j)];
    for (int k0 = 0; k0 < K8; k0 += 8) {
#pragma unroll
        for (int j = 0; j < 8; ++j) xw[8 + j] = xs[pad32(xl + k0 + 8 + j)];
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            float w[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) w[i] = ws[(cw + i) * K8 + k0 + kk];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(w[i], xw[j + kk], acc[i][j]);
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) xw[j] = xw[8 + j];
    }
    // epilogue: warm-up and NaN masks, then store
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int c = cb + cw + i;
        if (c >= a.n_combos) break;
        const int p = a.periods[c];
        const int warm = a.first + p - 1 + (a.warm_extra ? a.warm_extra[c] : 0);
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int t = t0 + xl + j;
            float r = acc[i][j];
            if (t < warm || t >= a.n) r = qnan();
            else if (a.nanp) {
                const double hi = a.nanp[t];
                const double lo = (a.nan_mode == 0 && t - p >= 0) ? a.nanp[t - p] : 0.0;
                if (hi - lo > 0.5) r = qnan();
            }
            v[j] = r;
        }
        float* o = a.out + (size_t)c * a.n + t0 + xl;
        const int tl = t0 + xl;
        if (tl + 8 <= a.n && ((reinterpret_cast<uintptr_t>(o) & 15) == 0)) {
            reinterpret_cast<float4*>(o)[0] = make_float4(v[0], v[1], v[2], v[3]);
            reinterpret_cast<float4*>(o)[1] = make_float4(v[4], v[5], v[6], v[7]);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (tl + j < a.n) o[j] = v[j];
        }
    }
}

// Time-major, one parameter set: lane = series (coalesced), 8 consecutive
// times per thread with a sliding register window over global loads.
constexpr int kTmT = 8;
constexpr int kTmTiles = 8;  // tiles of 8 times per thread

__global__ void k_wwma_tm(WwmaTmArgs a, const int* first_nan) {
    extern __shared__ float wsm[];
    for (int i = threadIdx.x; i < a.period; i += blockDim.x) wsm[i] = a.w[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.cols) return;
    const size_t S = a.cols;
    const int p = a.period, f = a.first[s];
    const int fn = first_nan ? first_nan[s] : a.rows;
    for (int tile = 0; tile < kTmTiles; ++tile) {
        const int t0 = (blockIdx.y * kTmTiles + tile) * kTmT;
        if (t0 >= a.rows) return;
        float acc[kTmT];
#pragma unroll
        for (int j = 0; j < kTmT; ++j) acc[j] = 0.f;
        const int base = t0 - p + 1;
        float win[kTmT];
#pragma unroll
        for (int j = 0; j < kTmT; ++j) {
            const int g = base + j;
            win[j] = (g >= 0 && g < a.rows) ? __ldg(a.x_tm + (size_t)g * S + s) : 0.f;
        }
        for (int k = 0; k < p; ++k) {
            const float w = wsm[k];
#pragma unroll
            for (int j = 0; j < kTmT; ++j) acc[j] = fmaf(w, win[j], acc[j]);
#pragma unroll
            for (int j = 0; j < kTmT - 1; ++j) win[j] = win[j + 1];
            const int g = base + k + kTmT;
            win[kTmT - 1] = (g >= 0 && g < a.rows) ? __ldg(a.x_tm + (size_t)g * S + s) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < kTmT; ++j) {
            const int t = t0 + j;
            if (t >= a.rows) break;
            float r = acc[j];
            if (t < f + p - 1 + a.warm_extra || (a.nan_mode == 1 && t >= fn)) r = qnan();
            a.out_tm[(size_t)t * S + s] = r;
        }
    }
}

__global__ void k_first_nan_tm(const float* __restrict__ x, int cols, int rows, const int* first,
                               int* out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cols) return;
    int t = first[s] + 1;
    while (t < rows && !isnan(x[(size_t)t * cols + s])) ++t;
    out[s] = t < rows ? t : rows;
}

}  // namespace

vta_status launch_wwma_batch_plain(const WwmaBatchArgs& a, cudaStream_t st) {
    const int kmax8 = (a.kmax + 7) & ~7;
    const size_t smem = (size_t)(kBC * kmax8 + (kBT + kmax8 + 8 + 32) * 33 / 32 + 64) * sizeof(float);
    if (smem > 227 * 1024) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "wwma: period too large");
    VTA_CUDA_TRY(cudaFuncSetAttribute(k_wwma_batch_plain, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    dim3 grid(ceil_div(a.n, kBT), ceil_div(a.n_combos, kBC));
    if (grid.y > 65535) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "wwma: too many combos");
    ktimer_begin(st);
    k_wwma_batch_plain<<<grid, kThreads, smem, st>>>(a);
    ktimer_end(st);
    return check_launch("k_wwma_batch_plain");
}

// first_nan scratch (cols ints) is carved by the caller right after `first`
vta_status launch_wwma_tm(const WwmaTmArgs& a, cudaStream_t st) {
    const int* fn = nullptr;
    if (a.nan_mode == 1) {
        int* first_nan = const_cast<int*>(a.first) + a.cols;
        k_first_nan_tm<<<ceil_div(a.cols, 128), 128, 0, st>>>(a.x_tm, a.cols, a.rows, a.first, first_nan);
        VTA_TRY(check_launch("k_first_nan_tm"));
        fn = first_nan;
    }
    dim3 grid(ceil_div(a.cols, 128), ceil_div(a.rows, kTmT * kTmTiles));
    const size_t smem = (size_t)a.period * sizeof(float);
    if (smem > 227 * 1024) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "wwma tm: period too large");
    if (smem > 48 * 1024)
        VTA_CUDA_TRY(cudaFuncSetAttribute(k_wwma_tm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ktimer_begin(st);
    k_wwma_tm<<<grid, 128, smem, st>>>(a, fn);
    ktimer_end(st);
    return check_launch("k_wwma_tm");
}

}  // namespace vta
