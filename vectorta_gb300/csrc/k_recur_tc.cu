// Chunk aggregates of the chunked recurrences (EMA, DEMA, TEMA, RSI batch
// sweeps) as a split-precision tcgen05 contraction.
//
// The AGG pass of the chunked scan needs, for every (lane, chunk), the state a
// chunk reaches from a zero state.  For the EMA cascades and RSI's Wilder
// averages that state is a fixed linear functional of the chunk's L inputs:
//   EMA / DEMA / TEMA  e_q(end) = sum_k h_q(L-1-k) x[c0+k]       (a = 2/(p+1), b = 1-a)
//       h_1(m) = a b^m,  h_2(m) = a^2 (m+1) b^m,  h_3(m) = a^3 (m+1)(m+2)/2 b^m
//   RSI  ag(end) = sum_k (1/p) b^(L-1-k) gain[c0+k],  al likewise on the losses  (b = 1-1/p)
// so the aggregates of all full chunks are one GEMM
//   D[rows = (component, lane)][cols = chunk (RSI: gains | losses)] = W[rows][K = L] * X[K][cols].
// W depends on the periods and L only (double-single powers of b); the
// caller keeps it across calls.  X comes from the series, each column
// centred on its chunk's first value and scaled by a power of two.  Both are
// split into FP16 hi + lo parts, and each K step issues Wh Xh + Wh Xl + Wl Xh
// with FP32 accumulation in TMEM (a few 1e-7 relative, like the FP32
// recurrence it replaces).
//
// Kernels: k_agg_weights packs W (core-matrix K-major order, per-row
// power-of-two scale, row sums for the centring term); k_agg_pack_x packs X
// and marks the chunks whose inputs are all finite; k_agg_gemm computes one
// 128 x 128 tile over one of S slices of K (split K: the tiles alone would
// not fill the GPU, and a split's accumulation chain stays short) and writes
// its partial sums.  Per CTA (128 threads, two
// CTAs per SM): thread 0 streams 32-wide K slices of both operands through a
// three-stage cp.async.bulk + mbarrier ring, thread 32 issues the MMAs, and
// the four warps read the accumulator back (tcgen05.ld) and store the
// partials lane-contiguous.  The AGG pass of k_recur.cu sums the S partials
// of every finite full chunk, applies the scales and the centring term and
// writes the chunk's record; it computes the seed chunk, the last (short)
// chunk and any chunk with a non-finite input itself.  Every mbarrier wait is
// bounded; on expiry the kernel raises the error word and returns, and the
// AGG pass then computes every chunk on the CUDA cores.
#include <cstdio>

#include "tc_ops.cuh"
#include "vta_internal.h"

namespace vta {
namespace {

using namespace tc;

constexpr int kTM = 128;           // rows per tile (MMA M)
constexpr int kTN = 128;           // columns per tile (MMA N)
constexpr int kKS = 32;            // K per pipeline slice
constexpr int kStages = 3;
constexpr int kGemmThreads = 128;  // thread 0: copies; thread 32: MMA issue; all: epilogue
// TMEM: columns [0, 128) accumulate Wh Xh, [128, 256) the cross terms Wh Xl +
// Wl Xh, so the small terms never round against the large accumulator
constexpr uint32_t kTmemColsAgg = 256;
// K of one split at most: the tensor cores' FP32 accumulation loses up to an
// ulp of the accumulator per MMA (not round-to-nearest), so a split's chain
// of Wh Xh MMAs stays short (kMaxSplitK / 16 of them) and the splits are
// summed on the CUDA cores with round-to-nearest adds
constexpr int kMaxSplitK = 512;
constexpr uint32_t kABytes = kTM * kKS * 2, kBBytes = kTN * kKS * 2;  // one hi or lo part
constexpr uint32_t kStageBytes = 2 * kABytes + 2 * kBBytes;

struct DS {
    float hi, lo;
};
__device__ __forceinline__ DS ds_mul(DS a, DS b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    const float s = p + e;
    return {s, e - (s - p)};
}
__device__ __forceinline__ DS ds_of(double v) {
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}

__host__ __device__ inline size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// Packed offsets (elements) of A [rows/128][L/8][16][8][8] and X
// [npad/128][L/8][16][8][8]: core matrices of 8 rows x 8 K-consecutive
// elements (128 bytes), 16 row groups per K group of a 128-row tile.
__device__ __forceinline__ size_t core_off(int r, int k, int L) {
    return (((size_t)(r >> 7) * (L >> 3) + (k >> 3)) * 16 + ((r & 127) >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

struct Wts {  // carved from RecurTcArgs::wts
    uint16_t *a_hi, *a_lo;
    float *row_scale, *row_sum;
};
inline Wts carve_w(void* base, const RecurTcGeo& g, int L) {
    char* p = static_cast<char*>(base);
    Wts w;
    w.a_hi = reinterpret_cast<uint16_t*>(p);
    w.a_lo = reinterpret_cast<uint16_t*>(p + al256((size_t)g.rows * L * 2));
    w.row_scale = reinterpret_cast<float*>(p + g.row_scale_off);
    w.row_sum = reinterpret_cast<float*>(p + g.row_sum_off);
    return w;
}
struct Ws {  // carved from RecurTcArgs::ws
    uint16_t *b_hi, *b_lo;
    float *col_scale, *col_ref, *part;
};
inline Ws carve_ws(void* base, const RecurTcGeo& g, int L) {
    char* p = static_cast<char*>(base);
    Ws w;
    w.b_hi = reinterpret_cast<uint16_t*>(p);
    w.b_lo = reinterpret_cast<uint16_t*>(p + al256((size_t)g.npad * L * 2));
    w.col_scale = reinterpret_cast<float*>(p + g.col_scale_off);
    w.col_ref = reinterpret_cast<float*>(p + g.col_ref_off);
    w.part = reinterpret_cast<float*>(p + g.part_off);
    return w;
}

// ------------------------------------------------------------ weights -----
// One warp per weight row r = q * mpad + lane.  w(m) = a^q coef_q(m) b^m with
// b^m in double-single: b^lane by squaring, then steps of b^32.  Pass 1 takes
// the row maximum and sum, pass 2 writes the scaled hi / lo parts.
__global__ void __launch_bounds__(256) k_agg_weights(RecurTcArgs a, Wts w) {
    const RecurTcGeo& g = a.geo;
    const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (r >= g.rows) return;
    const int q = r / g.mpad, li = r % g.mpad;
    const int L = a.L;
    const bool live = li < a.n_lanes;
    double al = 0.0, bd = 0.0;
    if (live) {
        const double p = (double)a.periods[li];
        if (a.kind == RK_RSI) {
            al = 1.0 / p;
            bd = 1.0 - 1.0 / p;
        } else {
            al = 2.0 / (p + 1.0);
            bd = 1.0 - al;
        }
    }
    const DS b = ds_of(bd);
    const DS aq = ds_of(q == 0 ? al : q == 1 ? al * al : al * al * al);
    DS b32 = b;
#pragma unroll
    for (int i = 0; i < 5; ++i) b32 = ds_mul(b32, b32);
    DS bl = {1.f, 0.f}, sq = b;  // b^lane
    for (int e = lane; e; e >>= 1, sq = ds_mul(sq, sq))
        if (e & 1) bl = ds_mul(bl, sq);
    auto weight = [&](int m, DS pw) {
        // the cascade coefficient 1, m + 1 or (m + 1)(m + 2) / 2, as an exact pair
        DS c = {1.f, 0.f};
        if (q == 1) c = {(float)(m + 1), 0.f};
        if (q == 2) {
            const float u = (float)(m + 1), v = (float)(m + 2);
            const float hi = u * v;
            c = {hi * 0.5f, fmaf(u, v, -hi) * 0.5f};
        }
        const DS v = ds_mul(aq, ds_mul(pw, c));
        return v.hi + v.lo;
    };
    float mx = 0.f;
    DS pw = bl;
    float s_hi = 0.f, s_lo = 0.f;
    for (int m = lane; m < L; m += 32, pw = ds_mul(pw, b32)) {
        const float v = live ? weight(m, pw) : 0.f;
        mx = fmaxf(mx, fabsf(v));
        const float t = s_hi + v;  // Neumaier
        s_lo += fabsf(s_hi) >= fabsf(v) ? (s_hi - t) + v : (v - t) + s_hi;
        s_hi = t;
    }
    double sum = (double)s_hi + (double)s_lo;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
    }
    int ex = 0;
    if (mx > 0.f) frexpf(mx, &ex);
    const int e = 14 - ex;  // row maximum in [2^13, 2^14)
    const float sc = mx > 0.f ? ldexpf(1.f, e) : 0.f;
    if (lane == 0) {
        w.row_scale[r] = mx > 0.f ? ldexpf(1.f, -e) : 0.f;
        w.row_sum[r] = (float)sum;
    }
    pw = bl;
    for (int m = lane; m < L; m += 32, pw = ds_mul(pw, b32)) {
        const float v = live ? weight(m, pw) * sc : 0.f;
        uint16_t h, l;
        Split<0>::run(v, h, l);
        const size_t o = core_off(r, L - 1 - m, L);
        w.a_hi[o] = h;
        w.a_lo[o] = l;
    }
}

// ------------------------------------------------------------ inputs ------
// One block per column j (chunk g0 + j % nc; RSI: gains for j < nc, losses
// after): the chunk's L inputs, centred on the chunk's first value (EMAs) and
// scaled by a power of two, split hi / lo.  done[chunk] = every input finite.
// The column's inputs are staged in shared memory (L <= kPackSmemL, 16-byte
// loads; longer chunks read them from global memory in both passes) and the
// split values written one core-matrix row (8 K-consecutive elements, 16
// bytes per part) per thread and store.
constexpr int kPackSmemL = 8192;

__global__ void __launch_bounds__(256) k_agg_pack_x(RecurTcArgs a, Ws w) {
    const RecurTcGeo& g = a.geo;
    const int j = blockIdx.x;
    const int L = a.L;
    extern __shared__ float colv[];  // L + 1 inputs when staged
    __shared__ float red[8];
    const int ngrp = L >> 3;
    auto store_row = [&](int kg, const float (&v)[8], float ref, float sc, bool fin) {
        uint16_t h[8], l[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            h[e] = 0;
            l[e] = 0;
            if (fin) Split<0>::run((v[e] - ref) * sc, h[e], l[e]);
        }
        const size_t o = core_off(j, kg * 8, L);
        *reinterpret_cast<uint4*>(w.b_hi + o) = make_uint4(h[0] | (uint32_t)h[1] << 16, h[2] | (uint32_t)h[3] << 16,
                                                           h[4] | (uint32_t)h[5] << 16, h[6] | (uint32_t)h[7] << 16);
        *reinterpret_cast<uint4*>(w.b_lo + o) = make_uint4(l[0] | (uint32_t)l[1] << 16, l[2] | (uint32_t)l[3] << 16,
                                                           l[4] | (uint32_t)l[5] << 16, l[6] | (uint32_t)l[7] << 16);
    };
    if (j >= g.ncol) {  // padding column: zeros
        const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int kg = threadIdx.x; kg < ngrp; kg += blockDim.x) store_row(kg, z, 0.f, 0.f, false);
        if (threadIdx.x == 0) { w.col_scale[j] = 0.f; w.col_ref[j] = 0.f; }
        return;
    }
    const bool rsi = a.kind == RK_RSI;
    const int c = a.g0 + j % a.nc, half = j / a.nc;
    const int c0 = a.chunk0 + (c - 1) * L;  // c >= 1
    const bool staged = L <= kPackSmemL;
    // staged: colv[0] = x[c0 - 1] (RSI), colv[1 + k] = x[c0 + k], loaded 16
    // bytes at a time when the chunk start is 16-byte aligned
    const float* src = a.x + c0;
    if (staged) {
        if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
            for (int i = threadIdx.x; i < (L >> 2); i += blockDim.x) {
                const float4 v = __ldg(reinterpret_cast<const float4*>(src) + i);
                colv[1 + 4 * i] = v.x;
                colv[2 + 4 * i] = v.y;
                colv[3 + 4 * i] = v.z;
                colv[4 + 4 * i] = v.w;
            }
        } else {
            for (int k = threadIdx.x; k < L; k += blockDim.x) colv[1 + k] = __ldg(src + k);
        }
        if (threadIdx.x == 0) colv[0] = rsi ? __ldg(src - 1) : 0.f;
        __syncthreads();
    }
    auto xat = [&](int k) { return staged ? colv[1 + k] : __ldg(src + k); };  // k >= -1
    // EMAs: the input; RSI: the gain (half 0) or loss (half 1) of the
    // difference to the previous bar.  `bad`: a non-finite input / difference.
    auto value = [&](int k, int& bad) {
        const float v = xat(k);
        if (!rsi) {
            bad |= !isfinite(v);
            return v;
        }
        const float d = v - xat(k - 1);
        bad |= !isfinite(d);
        return half == 0 ? (d > 0.f ? d : 0.f) : (d < 0.f ? -d : 0.f);
    };
    const float ref = rsi ? 0.f : xat(0);
    float mx = 0.f;
    int bad = 0;
#pragma unroll 4
    for (int k = threadIdx.x; k < L; k += blockDim.x) mx = fmaxf(mx, fabsf(value(k, bad) - ref));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    const bool fin = __syncthreads_or(bad) == 0;
    mx = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) mx = fmaxf(mx, red[i]);
    int ex = 0;
    if (mx > 0.f) frexpf(mx, &ex);
    const int e = 13 - ex;  // chunk maximum in [2^12, 2^13)
    const float sc = (fin && mx > 0.f) ? ldexpf(1.f, e) : 0.f;
    for (int kg = threadIdx.x; kg < ngrp; kg += blockDim.x) {
        float v[8];
        int unused = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) v[q] = fin ? value(kg * 8 + q, unused) : 0.f;
        store_row(kg, v, ref, sc, fin);
    }
    if (threadIdx.x == 0) {
        w.col_scale[j] = (fin && mx > 0.f) ? ldexpf(1.f, -e) : 0.f;
        w.col_ref[j] = ref;
        if (half == 0) a.done[c] = fin ? 1 : 0;
    }
}

// ------------------------------------------------------------ GEMM --------
struct __align__(16) AggCtl {
    uint64_t full[kStages];
    uint64_t free_[kStages];
    uint64_t acc_done;
    uint32_t tmem_base;
    int abort_flag;
    int committed;  // acc_done was committed (MMAs to drain)
    int issued;     // operand slices whose copies were issued
};

__global__ void __launch_bounds__(kGemmThreads, 2) k_agg_gemm(RecurTcArgs a, Wts wt, Ws w) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    const RecurTcGeo& g = a.geo;
    // stage st: A hi, A lo, X hi, X lo
    auto a_hi = [&](int st) { return smem_raw + st * kStageBytes; };
    auto a_lo = [&](int st) { return smem_raw + st * kStageBytes + kABytes; };
    auto b_hi = [&](int st) { return smem_raw + st * kStageBytes + 2 * kABytes; };
    auto b_lo = [&](int st) { return smem_raw + st * kStageBytes + 2 * kABytes + kBBytes; };
    AggCtl* ctl = reinterpret_cast<AggCtl*>(smem_raw + kStages * kStageBytes);
    const int mt = blockIdx.x, nt = blockIdx.y, ks = blockIdx.z;
    const int L = a.L;
    const int ns_all = L / kKS;
    const int s_begin = (int)((long long)ks * ns_all / g.S), s_end = (int)((long long)(ks + 1) * ns_all / g.S);
    const int ns = s_end - s_begin;  // >= 1 (S <= ns_all)
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    volatile int* abort_flag = &ctl->abort_flag;
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&ctl->full[s], 1);
            mbar_init(&ctl->free_[s], 1);
        }
        mbar_init(&ctl->acc_done, 1);
        ctl->abort_flag = 0;
        ctl->committed = 0;
        ctl->issued = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&ctl->tmem_base)),
                     "r"(kTmemColsAgg)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = ctl->tmem_base;

    if (tid == 0) {
        // ============ producer: operand slices into the stage ring ==========
        const size_t tile_a = (size_t)mt * (L >> 3) * 1024, tile_b = (size_t)nt * (L >> 3) * 1024;
        constexpr size_t kSliceEl = (kKS / 8) * 1024;  // elements of one slice of a 128-row tile
        bool ok = true;
        for (int i = 0; i < ns && ok; ++i) {
            const int st = i % kStages;
            if (i >= kStages) ok = mbar_wait(&ctl->free_[st], ((i / kStages) - 1) & 1, abort_flag);
            if (!ok) break;
            const size_t off = (size_t)(s_begin + i) * kSliceEl;
            mbar_arrive_tx(&ctl->full[st], kStageBytes);
            bulk_g2s(a_hi(st), wt.a_hi + tile_a + off, kABytes, &ctl->full[st]);
            bulk_g2s(a_lo(st), wt.a_lo + tile_a + off, kABytes, &ctl->full[st]);
            bulk_g2s(b_hi(st), w.b_hi + tile_b + off, kBBytes, &ctl->full[st]);
            bulk_g2s(b_lo(st), w.b_lo + tile_b + off, kBBytes, &ctl->full[st]);
            ctl->issued = i + 1;
        }
        if (!ok) ctl->abort_flag = 1;
    } else if (tid == 32) {
        // ============ MMA issue ============================================
        const uint32_t idesc = instr_desc_f16(0u, kTM, kTN, 0u);  // f16, A and B K-major
        bool ok = true;
        int done_i = 0;
        for (int i = 0; i < ns && ok; ++i) {
            const int st = i % kStages;
            ok = mbar_wait(&ctl->full[st], (i / kStages) & 1, abort_flag);
            if (!ok) break;
            tc_fence_after();
            const uint32_t ahs = smem_u32(a_hi(st)), als = smem_u32(a_lo(st));
            const uint32_t bhs = smem_u32(b_hi(st)), bls = smem_u32(b_lo(st));
#pragma unroll
            for (int kk = 0; kk < kKS / 16; ++kk) {
                // K step of 16 = two core-matrix columns of 16 groups x 128 B
                const uint64_t dah = smem_desc(ahs + kk * 4096, 2048, 128);
                const uint64_t dal = smem_desc(als + kk * 4096, 2048, 128);
                const uint64_t dbh = smem_desc(bhs + kk * 4096, 2048, 128);
                const uint64_t dbl = smem_desc(bls + kk * 4096, 2048, 128);
                const uint32_t acc = (i > 0 || kk > 0) ? 1u : 0u;
                tc_mma(tmem, dah, dbh, idesc, acc);
                tc_mma(tmem + kTN, dah, dbl, idesc, acc);
                tc_mma(tmem + kTN, dal, dbh, idesc, 1u);
            }
            tc_commit(&ctl->free_[st]);
            done_i = i + 1;
        }
        if (!ok) ctl->abort_flag = 1;
        if (done_i > 0) {
            // also on abort: the drain below waits for the MMAs issued
            tc_commit(&ctl->acc_done);
            ctl->committed = 1;
        }
    }
    // ============ epilogue: warp w reads TMEM lanes 32 w .. 32 w + 31 ========
    {
        int ok = 1;
        if (lane == 0) {
            ok = mbar_wait(&ctl->acc_done, 0, abort_flag);
            if (!ok) ctl->abort_flag = 1;
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        __syncwarp();
        if (ok && !ctl->abort_flag) {
            tc_fence_after();
            const int r = mt * kTM + warp * 32 + lane;
            float* dst = w.part + ((size_t)ks * g.npad + (size_t)nt * kTN) * g.rows + r;
#pragma unroll 1
            for (int cg = 0; cg < kTN / 32; ++cg) {
                uint32_t v[32], u[32];
                const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cg * 32);
                TC_LD32(ta, v);
                TC_WAIT_LD32(v);
                TC_LD32(ta + kTN, u);
                TC_WAIT_LD32(u);
#pragma unroll
                for (int cc = 0; cc < 32; ++cc)
                    dst[(size_t)(cg * 32 + cc) * g.rows] = __uint_as_float(v[cc]) + __uint_as_float(u[cc]);
            }
        }
    }
    // drain: the MMAs must have completed before TMEM is freed and, after an
    // abort, the last copy issued into each stage must have landed
    __syncthreads();
    if (tid == 0) {
        volatile int no_abort = 0;
        if (ctl->committed) mbar_wait(&ctl->acc_done, 0, &no_abort);
        if (ctl->abort_flag) {
            const int issued = ctl->issued;
            for (int i = max(0, issued - kStages); i < issued; ++i)
                mbar_wait(&ctl->full[i % kStages], (i / kStages) & 1, &no_abort);
            atomicExch(a.err, 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    __syncwarp();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemColsAgg)
                     : "memory");
}

constexpr size_t kGemmSmem = (size_t)kStages * kStageBytes + sizeof(AggCtl) + 128;

}  // namespace

RecurTcGeo recur_agg_tc_geo(int kind, int n_lanes, int L, int nc, int num_sms) {
    RecurTcGeo g{};
    g.nsr = kind == RK_TEMA ? 3 : kind == RK_DEMA ? 2 : 1;
    g.mpad = (n_lanes + kTM - 1) / kTM * kTM;
    g.rows = g.nsr * g.mpad;
    g.ncol = kind == RK_RSI ? 2 * nc : nc;
    g.npad = (g.ncol + kTN - 1) / kTN * kTN;
    // split K until one wave of CTAs (two per SM) is in flight, each CTA
    // with at least four K slices
    const long long tiles = (long long)(g.rows / kTM) * (g.npad / kTN);
    const int ns_all = L / kKS;
    long long S = (2LL * num_sms + tiles - 1) / tiles;
    if (S > ns_all / 4) S = ns_all / 4;
    const long long s_acc = (L + kMaxSplitK - 1) / kMaxSplitK;  // accuracy bound
    if (S < s_acc) S = s_acc;
    if (S > ns_all) S = ns_all;
    if (S < 1) S = 1;
    g.S = (int)S;
    const size_t a_part = al256((size_t)g.rows * L * 2), b_part = al256((size_t)g.npad * L * 2);
    g.row_scale_off = 2 * a_part;
    g.row_sum_off = g.row_scale_off + al256((size_t)g.rows * 4);
    g.w_bytes = g.row_sum_off + al256((size_t)g.rows * 4);
    g.col_scale_off = 2 * b_part;
    g.col_ref_off = g.col_scale_off + al256((size_t)g.npad * 4);
    g.part_off = g.col_ref_off + al256((size_t)g.npad * 4);
    g.ws_bytes = g.part_off + al256((size_t)g.S * g.npad * g.rows * 4);
    return g;
}

size_t recur_agg_tc_smem() { return kGemmSmem; }

vta_status launch_recur_agg_tc(const RecurTcArgs& a, size_t smem_optin, cudaStream_t st) {
    if (a.nc <= 0) return VTA_OK;
    if ((a.L % kKS) || a.L <= 0) return fail(VTA_ERR_INVALID_INPUT, "tc aggregates: chunk length");
    if (kGemmSmem > smem_optin) return fail(VTA_ERR_NOT_IMPLEMENTED, "tc aggregates: shared memory");
    const RecurTcGeo& g = a.geo;
    const Wts wt = carve_w(a.wts, g, a.L);
    const Ws w = carve_ws(a.ws, g, a.L);
    VTA_CUDA_TRY(cudaMemsetAsync(a.err, 0, sizeof(int), st));
    if (a.build_weights) {
        k_agg_weights<<<(g.rows + 7) / 8, 256, 0, st>>>(a, wt);
        VTA_TRY(check_launch("k_agg_weights"));
    }
    k_agg_pack_x<<<g.npad, 256, a.L <= kPackSmemL ? (size_t)(a.L + 1) * sizeof(float) : 0, st>>>(a, w);
    VTA_TRY(check_launch("k_agg_pack_x"));
    static int smem_set_dev = -1;  // the attribute is per device; set it once
    int dev = 0;
    VTA_CUDA_TRY(cudaGetDevice(&dev));
    if (smem_set_dev != dev) {
        VTA_CUDA_TRY(cudaFuncSetAttribute(k_agg_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem));
        smem_set_dev = dev;
    }
    dim3 grid(g.rows / kTM, g.npad / kTN, g.S);
    k_agg_gemm<<<grid, kGemmThreads, kGemmSmem, st>>>(a, wt, w);
    return check_launch("k_agg_gemm");
}

}  // namespace vta
