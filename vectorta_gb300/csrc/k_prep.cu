// Series preparation kernels: per-series first-valid scan for time-major
// inputs and the blocked FP64 prefix scan behind the SMA/variance windows.
//
// The prefix is the only FP64 bulk arithmetic of the library (GB300's FP64
// rate is a small fraction of FP32): one f64 add per element in a 3-phase
// scan (block reduce -> scan of block sums -> block scan + offset), then the
// result is packed as double-single float2 (hi = f32(P), lo = f32(P - hi)) so
// the per-output window kernels work in FP32 only.
#include "vta_internal.h"

namespace vta {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanBlock = kScanThreads * kScanItems;  // elements per block

// First valid row per series: one thread per series (coalesced across the
// series of a row), rows examined kFvRows at a time.  The block's loads are
// all issued before any is tested (row indices clamped into the matrix, no
// short-circuit), so a NaN lead of a few hundred rows costs a few dozen
// memory round trips instead of one per row.
constexpr int kFvRows = 16;

__global__ void k_first_valid_tm(const float* __restrict__ x, int cols, int rows, int* first) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cols) return;
    int found = rows;
    for (int t0 = 0; t0 < rows && found == rows; t0 += kFvRows) {
        float v[kFvRows];
#pragma unroll
        for (int j = 0; j < kFvRows; ++j) v[j] = __ldg(x + (size_t)min(t0 + j, rows - 1) * cols + s);
#pragma unroll
        for (int j = kFvRows - 1; j >= 0; --j)
            if ((t0 + j < rows) & !isnan(v[j])) found = t0 + j;
    }
    first[s] = found;
}

__global__ void k_first_valid_tm_hlc(const float* __restrict__ h, const float* __restrict__ l,
                                     const float* __restrict__ c, int cols, int rows, int* first) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cols) return;
    int found = rows;
    for (int t0 = 0; t0 < rows && found == rows; t0 += kFvRows) {
        float hv[kFvRows], lv[kFvRows], cv[kFvRows];
#pragma unroll
        for (int j = 0; j < kFvRows; ++j) {
            const size_t i = (size_t)min(t0 + j, rows - 1) * cols + s;
            hv[j] = __ldg(h + i);
            lv[j] = __ldg(l + i);
            cv[j] = __ldg(c + i);
        }
#pragma unroll
        for (int j = kFvRows - 1; j >= 0; --j)
            if ((t0 + j < rows) & !isnan(hv[j]) & !isnan(lv[j]) & !isnan(cv[j])) found = t0 + j;
    }
    first[s] = found;
}

__device__ __forceinline__ double prefix_value(const float* x, int i, int first, int kind) {
    if (i < first) return 0.0;
    const double v = (double)x[i];
    switch (kind) {
        case PK_X: return v;
        case PK_X2: return v * v;
        case PK_NAN: return isnan(x[i]) ? 1.0 : 0.0;
        case PK_GAIN:
        case PK_LOSS: {
            if (i == first) return 0.0;
            const double d = v - (double)x[i - 1];
            if (!isfinite(d)) return __longlong_as_double(0x7ff8000000000000ll);
            if (kind == PK_GAIN) return d > 0.0 ? d : 0.0;
            return d < 0.0 ? -d : 0.0;
        }
    }
    return 0.0;
}

__device__ __forceinline__ double warp_incl_scan(double v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Block-wide exclusive scan of one double per thread (true exclusive: a NaN
// in thread i reaches threads > i only); leaves the block total in *total.
__device__ double block_excl_scan(double v, double* total) {
    constexpr int kW = kScanThreads / 32;
    __shared__ double wsum[kW];
    __shared__ double wtot;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double inc = warp_incl_scan(v);
    double exc = __shfl_up_sync(0xffffffffu, inc, 1);
    if (lane == 0) exc = 0.0;
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const double w = lane < kW ? wsum[lane] : 0.0;
        const double wi = warp_incl_scan(w);
        double we = __shfl_up_sync(0xffffffffu, wi, 1);
        if (lane == 0) we = 0.0;
        if (lane < kW) wsum[lane] = we;  // exclusive warp offsets
        if (lane == kW - 1) wtot = wi;
    }
    __syncthreads();
    const double res = wsum[warp] + exc;
    *total = wtot;
    __syncthreads();
    return res;
}

__global__ void k_prefix_reduce(const float* __restrict__ x, int n, int first, int kind,
                                double* block_sums) {
    const int base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int i = base + k;
        if (i < n) s += prefix_value(x, i, first, kind);
    }
    double total;
    block_excl_scan(s, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Exclusive scan of the block sums in place (single block, any count).
__global__ void k_prefix_scan_blocks(double* block_sums, int nb) {
    double carry = 0.0;
    for (int base = 0; base < nb; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const double v = i < nb ? block_sums[i] : 0.0;
        double total;
        const double exc = block_excl_scan(v, &total);
        if (i < nb) block_sums[i] = carry + exc;
        carry += total;
    }
}

__global__ void k_prefix_apply(const float* __restrict__ x, int n, int first, int kind,
                               const double* __restrict__ block_offsets, double* out_f64,
                               float2* out_ds) {
    const int base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
    double v[kScanItems];
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int i = base + k;
        v[k] = i < n ? prefix_value(x, i, first, kind) : 0.0;
        s += v[k];
    }
    double total;
    double run = block_offsets[blockIdx.x] + block_excl_scan(s, &total);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int i = base + k;
        run += v[k];
        if (i < n) {
            if (out_f64) out_f64[i] = run;
            if (out_ds) {
                const float hi = (float)run;
                const float lo = (float)(run - (double)hi);
                out_ds[i] = make_float2(hi, lo);
            }
        }
    }
}

}  // namespace

vta_status launch_first_valid_tm(const float* x_tm, int cols, int rows, int* first, cudaStream_t st) {
    k_first_valid_tm<<<ceil_div(cols, 128), 128, 0, st>>>(x_tm, cols, rows, first);
    return check_launch("k_first_valid_tm");
}

vta_status launch_first_valid_tm_hlc(const float* h, const float* l, const float* c, int cols,
                                     int rows, int* first, cudaStream_t st) {
    k_first_valid_tm_hlc<<<ceil_div(cols, 128), 128, 0, st>>>(h, l, c, cols, rows, first);
    return check_launch("k_first_valid_tm_hlc");
}

size_t prefix_tmp_doubles(int n) { return ceil_div(n, kScanBlock) + 1; }

vta_status launch_prefix_f64(const float* x, int n, int first, int kind, double* out_f64,
                             float2* out_ds, double* block_tmp, cudaStream_t st) {
    const int nb = (int)ceil_div(n, kScanBlock);
    k_prefix_reduce<<<nb, kScanThreads, 0, st>>>(x, n, first, kind, block_tmp);
    VTA_TRY(check_launch("k_prefix_reduce"));
    k_prefix_scan_blocks<<<1, kScanThreads, 0, st>>>(block_tmp, nb);
    VTA_TRY(check_launch("k_prefix_scan_blocks"));
    k_prefix_apply<<<nb, kScanThreads, 0, st>>>(x, n, first, kind, block_tmp, out_f64, out_ds);
    return check_launch("k_prefix_apply");
}

// Row-major [rows][cols] -> [cols][rows] through 32 x 33 shared tiles (one
// coalesced read and one coalesced write per element).
namespace {
__global__ void k_transpose(const float* __restrict__ in, int rows, int cols, float* __restrict__ out) {
    __shared__ float tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int r = r0 + j, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[j][threadIdx.x] = in[(size_t)r * cols + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {
        const int c = c0 + j, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[(size_t)c * rows + r] = tile[threadIdx.x][j];
    }
}
}  // namespace

vta_status launch_transpose(const float* in, int rows, int cols, float* out, cudaStream_t st) {
    if (rows <= 0 || cols <= 0) return VTA_OK;
    const dim3 grid(ceil_div(cols, 32), ceil_div(rows, 32));
    if (grid.y > 65535) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "transpose: too many rows");
    k_transpose<<<grid, dim3(32, 8), 0, st>>>(in, rows, cols, out);
    return check_launch("k_transpose");
}

}  // namespace vta
