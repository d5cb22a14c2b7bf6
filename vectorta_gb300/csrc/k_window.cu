// Window indicators: prefix-sum windows (SMA, StdDev, Z-score, Bollinger),
// sliding min/max (Donchian, Williams %R) and nearest-rank percentile.
//
// Precision plan (GB300's FP64 rate is a small fraction of FP32):
//   * batch: each block builds a double-single (float pair) prefix of x and
//     of x^2 over its own input span only, so every window sum is a
//     difference of two local prefix entries whose magnitude is that of the
//     span's data, not of the whole series (a global prefix loses the
//     variance where a series falls far below its earlier levels); the
//     variance is formed as (p*S2 - S1^2) / p^2 from error-free products;
//   * time-major: each thread slides compensated (double-single) running sums
//     over its time chunk, re-initialised exactly at the chunk start.
// NaN semantics follow the crate's running-sum code: a NaN after the first
// valid index poisons every later output of that series, an infinite input
// every output from p steps after it (where it leaves the window: inf - inf).
#include <algorithm>

#include "pnr_ops.cuh"
#include "vta_internal.h"

namespace vta {
namespace {

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

// ------------------------------------------------- double-single helpers --
struct DS {
    float hi, lo;
};
__device__ __forceinline__ DS two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ DS fast_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ DS ds_sub2(float2 a, float2 b) {
    const DS s = two_sum(a.x, -b.x);
    return fast_two_sum(s.hi, s.lo + (a.y - b.y));
}
// a - b for a.x >= b.x >= 0 (a prefix of squares: non-decreasing), where the
// error of the leading difference is exact by Fast2Sum
__device__ __forceinline__ DS ds_sub2_ge(float2 a, float2 b) {
    const float d = a.x - b.x;
    const float e = (a.x - d) - b.x;
    return fast_two_sum(d, e + (a.y - b.y));
}
__device__ __forceinline__ DS ds_add_f(DS a, float b) {
    const DS s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ float ds_f(DS a) { return a.hi + a.lo; }

// Evaluates one prefix-window output family from the window sums S1, S2.
struct WinOut {
    float o0, o1, o2;
};
// inv_p = 1/p and inv_p2 = 1/p^2 are per-combo constants (no division per
// output).
__device__ __forceinline__ WinOut window_eval(int kind, DS s1, DS s2, float pf, float inv_p, float inv_p2,
                                              float xt, float k1, float k2) {
    WinOut r = {0.f, 0.f, 0.f};
    const float mean = ds_f(s1) * inv_p;
    if (kind == WK_SMA) {
        r.o0 = mean;
        return r;
    }
    // p*S2 - S1^2 = p^2 * var, from the error-free products p*S2.hi and
    // S1.hi^2 (their difference is exact where it cancels) plus the
    // first-order low-part terms; the dropped S1.lo^2 is 2^-48 of S1^2
    const float h = s1.hi * s1.hi, eh = fmaf(s1.hi, s1.hi, -h);
    const float g = pf * s2.hi, eg = fmaf(pf, s2.hi, -g);
    float corr = fmaf(pf, s2.lo, eg - eh);
    corr = fmaf(-2.f * s1.hi, s1.lo, corr);
    const float var = ((g - h) + corr) * inv_p2;
    if (kind == WK_STDDEV) {
        r.o0 = var <= 0.f ? 0.f : sqrtf(var) * k1;
        return r;
    }
    if (kind == WK_ZSCORE) {
        const float sd = var <= 0.f ? 0.f : sqrtf(var) * k1;
        const float dev = xt - mean;
        r.o0 = (sd == 0.f || isnan(sd)) ? qnan() : __fdividef(dev, sd);
        return r;
    }
    // Bollinger (population std, devtype 0)
    const float sd = sqrtf(fmaxf(var, 0.f));
    r.o1 = mean;
    r.o0 = mean + k1 * sd;
    r.o2 = mean - k2 * sd;
    return r;
}

// ---------------------------------------------- prefix windows, batch ------
// One block per time tile of kPwTile steps serves every combo: the block
// builds the local double-single prefix of x and x^2 over the tile's input
// span [t0 - pmax, t0 + kPwTile) in shared memory, each thread keeps the
// prefix at its kPwPer times in registers and loops over combos.
constexpr int kPwThreads = 256;
constexpr int kPwPer = 4;
constexpr int kPwTile = kPwThreads * kPwPer;

__device__ __forceinline__ DS ds_add(DS a, DS b) {
    const DS s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

// first NaN / first infinite input at or after `first`, stored as n - index
// (bad[] starts at 0 = none, so a memset clears it)
__global__ void k_first_bad(const float* __restrict__ x, int n, int first, int* bad) {
    int fn = n, fi = n;
    for (int i = first + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float v = x[i];
        if (isnan(v)) fn = min(fn, i);
        else if (isinf(v)) fi = min(fi, i);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        fn = min(fn, __shfl_xor_sync(0xffffffffu, fn, o));
        fi = min(fi, __shfl_xor_sync(0xffffffffu, fi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (fn < n) atomicMax(bad, n - fn);
        if (fi < n) atomicMax(bad + 1, n - fi);
    }
}

// ---- clean-tile fast path ---------------------------------------------
// In a tile whose input span holds no NaN or infinite value (the usual case)
// each local prefix entry P = (hi, lo) is re-split as P = A + a with A a
// multiple of one quantum Q per span: Q = 2^(e-21) for a bound 2^(e+1) on
// |P| over the span, so every |A| <= 2^22 Q and every difference A(t) -
// A(t-p) is a multiple of Q of at most 2^23 Q: exact in f32.  A window sum is
// then the exact f32 difference of the A parts plus the (small) difference of
// the a parts, two subtractions instead of a double-single subtraction.
// A = (hi + C) - C with C = 1.5 * 2^(e+2) rounds hi to the nearest multiple
// of Q (|hi| <= 2^(e+1) keeps hi + C inside [2^(e+2), 2^(e+3))); hi - A is
// exact and a = (hi - A) + lo rounds at Q * 2^-25, i.e. 2^-47 of the bound.
struct Quant {
    float c;
};
__device__ __forceinline__ Quant quant_of(float bound) {
    int e = (int)((__float_as_uint(bound) >> 23) & 0xffu) - 127;  // bound < 2^(e+1)
    e = max(e, -100);
    return {__uint_as_float(((unsigned)(e + 2 + 127) << 23) | 0x400000u)};
}
__device__ __forceinline__ float2 quant_split(float2 v, Quant q) {
    const float A = __fsub_rn(__fadd_rn(v.x, q.c), q.c);
    return make_float2(A, __fadd_rn(__fsub_rn(v.x, A), v.y));
}

// p^2 * var = p * S2 - S1^2 from the split window sums S1 = d1h + d1l and
// S2 = d2h + d2l (d1h, d2h exact): the error-free products p * d2h and d1h^2
// (their difference is exact where it cancels) plus p * d2l - 2 d1h d1l -
// d1l^2.  The last term matters: d1l is up to one quantum of the span's
// bound, which for a short window is not negligible against S1.
__device__ __forceinline__ float window_d(float d1h, float d1l, float d2h, float d2l, float pf) {
    const float g = __fmul_rn(pf, d2h), eg = fmaf(pf, d2h, -g);
    const float h = __fmul_rn(d1h, d1h), eh = fmaf(d1h, d1h, -h);
    float t = fmaf(pf, d2l, __fsub_rn(eg, eh));
    t = fmaf(-__fadd_rn(d1h, d1h), d1l, t);
    t = fmaf(-d1l, d1l, t);
    return __fadd_rn(__fsub_rn(g, h), t);
}

// Per-combo constants of the fast path, computed once per block into shared
// memory: x = period (int bits), y = 1/p (correctly rounded), z = the output
// scale (StdDev: nbdev / p; Z-score: p / nbdev, NaN for nbdev 0; BB: devup),
// w = BB devdn.
__device__ __forceinline__ float4 combo_consts(int K, int p, float k1, float k2) {
    const float pf = (float)p;
    const float inv_p = __frcp_rn(pf);
    float z = k1;
    if (K == WK_STDDEV) z = __fmul_rn(k1, inv_p);
    if (K == WK_ZSCORE) z = (k1 == 0.f || isnan(k1)) ? qnan() : __fdiv_rn(pf, k1);
    return make_float4(__int_as_float(p), inv_p, z, k2);
}

// 1/sqrt(v) for a normal positive v: the hardware approximation (max
// relative error about 2^-22.9), one instruction.
__device__ __forceinline__ float rsqrt_approx(float v) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
    return r;
}

// One combo's outputs at this thread's kPwPer times of a clean tile.
// q1[k], q2[k]: split prefix at t; b1, b2: split prefix array shifted to t - p.
template <int K, bool FULL>
__device__ __forceinline__ void fast_outputs(const float2 (&q1)[4], const float2 (&q2)[4], const float (&xt)[4],
                                             const float2* b1, const float2* b2, float4 cc, float ref, float* r0,
                                             float* r1, float* r2, int t, int n, int warm) {
    const float pf = (float)__float_as_int(cc.x);
    const float inv_p = cc.y;
    // stddev: sqrt(var) * k1 = sqrt(D) * (k1 / p); z-score: dev / (sqrt(var) k1)
    // = dev * rsqrt(D) * (p / k1); BB: sqrt(max(var, 0)) = sqrt(max(D, 0)) / p
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int tk = t + k * kPwThreads;
        if (!FULL && (tk >= n || tk < warm)) {
            if (tk < n) {
                r0[k * kPwThreads] = qnan();
                if (K == WK_BB) { r1[k * kPwThreads] = qnan(); r2[k * kPwThreads] = qnan(); }
            }
            continue;
        }
        const float2 v1 = b1[k * kPwThreads];
        const float d1h = __fsub_rn(q1[k].x, v1.x), d1l = __fsub_rn(q1[k].y, v1.y);
        if (K == WK_SMA) {
            r0[k * kPwThreads] = __fadd_rn(ref, __fmul_rn(__fadd_rn(d1h, d1l), inv_p));
            continue;
        }
        const float2 v2 = b2[k * kPwThreads];
        const float D = window_d(d1h, d1l, __fsub_rn(q2[k].x, v2.x), __fsub_rn(q2[k].y, v2.y), pf);
        const float r = rsqrt_approx(fmaxf(D, 1.17549435e-38f));
        if (K == WK_STDDEV) {
            r0[k * kPwThreads] = D > 0.f ? __fmul_rn(__fmul_rn(D, r), cc.z) : 0.f;
        } else if (K == WK_ZSCORE) {
            const float dev = __fsub_rn(xt[k], __fmul_rn(__fadd_rn(d1h, d1l), inv_p));
            r0[k * kPwThreads] = D > 0.f ? __fmul_rn(__fmul_rn(dev, r), cc.z) : qnan();
        } else {
            const float mean = __fadd_rn(ref, __fmul_rn(__fadd_rn(d1h, d1l), inv_p));
            const float sd = __fmul_rn(__fmul_rn(fmaxf(D, 0.f), r), inv_p);
            r1[k * kPwThreads] = mean;
            r0[k * kPwThreads] = fmaf(cc.z, sd, mean);
            r2[k * kPwThreads] = fmaf(-cc.w, sd, mean);
        }
    }
}

constexpr int kPwComboGroup = 256;  // combos whose constants share memory holds at a time
static_assert(kPwComboGroup <= kPwThreads, "one thread per combo of a group");

template <int K>
__device__ void fast_tile(const PrefixWinArgs& a, const float2* s1, const float2* s2, int pmax, int t0,
                          float r0, int cb, int ce, float4* cc) {
    static_assert(kPwPer == 4, "fast_outputs is written for 4 outputs per thread");
    float2 q1[4], q2[4];
    float xt[4];
    const int tid = threadIdx.x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int l = pmax + tid + k * kPwThreads;
        const int t = t0 + tid + k * kPwThreads;
        q1[k] = s1[l];
        q2[k] = K == WK_SMA ? make_float2(0.f, 0.f) : s2[l];
        xt[k] = (K == WK_ZSCORE && t < a.n) ? __fsub_rn(__ldg(a.x + t), r0) : 0.f;  // y(t)
    }
    const bool tail = t0 + kPwTile > a.n;
    for (int g0 = cb; g0 < ce; g0 += kPwComboGroup) {
        const int gn = min(kPwComboGroup, ce - g0);
        __syncthreads();  // the previous group's constants are no longer read
        if (tid < gn) {
            const int c = g0 + tid;
            cc[tid] = combo_consts(K, __ldg(a.periods + c), a.k1 ? __ldg(a.k1 + c) : 1.f,
                                   a.k2 ? __ldg(a.k2 + c) : 1.f);
        }
        __syncthreads();
        for (int j = 0; j < gn; ++j) {
            const float4 k4 = cc[j];
            const int p = __float_as_int(k4.x);
            const int warm = a.first + p - 1;
            const size_t o = (size_t)(g0 + j) * a.n + t0 + tid;
            const int sh = pmax - p + tid;
            float* o1 = a.out1 ? a.out1 + o : nullptr;
            float* o2 = a.out2 ? a.out2 + o : nullptr;
            if (!tail && t0 >= warm)  // the whole tile is past this combo's warm-up
                fast_outputs<K, true>(q1, q2, xt, s1 + sh, s2 + sh, k4, r0, a.out0 + o, o1, o2, t0 + tid, a.n, warm);
            else
                fast_outputs<K, false>(q1, q2, xt, s1 + sh, s2 + sh, k4, r0, a.out0 + o, o1, o2, t0 + tid, a.n, warm);
        }
    }
}

// Block (tile, g): the tile's kPwTile times for the combos [g cpb, (g + 1)
// cpb); a tile's prefix is rebuilt by each of its combo groups (a few percent
// of a group's work), so the grid fills the GPU in whole waves.
__global__ void __launch_bounds__(kPwThreads)
k_prefix_window_batch(PrefixWinArgs a, int pmax, int cpb) {
    extern __shared__ float2 psm[];
    __shared__ float4 cc[kPwComboGroup];  // combo constants of the fast path
    const int cb = blockIdx.y * cpb, ce = min(a.n_combos, cb + cpb);
    __shared__ DS wsum1[kPwThreads / 32], wsum2[kPwThreads / 32];
    const int t0 = blockIdx.x * kPwTile;
    const int span = kPwTile + pmax;
    const int base = t0 - pmax;  // global index of slot 0
    const bool two = a.kind != WK_SMA;
    float2* s1 = psm;
    float2* s2 = psm + span;
    const float2 z = make_float2(0.f, 0.f);
    // 1. local inclusive prefix: each thread sums a run of `per` slots, the
    // run totals are scanned across the block, then added back
    const int per = (span + kPwThreads - 1) / kPwThreads;
    const int i0 = threadIdx.x * per, i1 = min(i0 + per, span);
    // no NaN / infinite input at or after `first` before the tile's end: no
    // output of the tile is poisoned and the span's prefixes are finite
    const bool clean = a.n - a.bad[0] >= t0 + kPwTile && a.n - a.bad[1] >= t0 + kPwTile;
    // A clean tile's prefixes are of y = x - r0, centred on the tile's first
    // valid value: window variances are shift-invariant, and the centred sums
    // are smaller, so both the cancellation in p S2 - S1^2 and the quantum of
    // the split below shrink with the span's spread instead of its level.
    const float r0 = clean && a.first < a.n ? __ldg(a.x + max(t0, a.first)) : 0.f;
    DS a1 = {0.f, 0.f}, a2 = {0.f, 0.f};
    float abs1 = 0.f;  // sum of |y| over this thread's run: bounds |prefix of y|
    for (int i = i0; i < i1; ++i) {
        const int g = base + i;
        const float v = (g >= a.first && g < a.n) ? __fsub_rn(__ldg(a.x + g), r0) : 0.f;
        abs1 += fabsf(v);
        a1 = ds_add_f(a1, v);
        s1[i] = make_float2(a1.hi, a1.lo);
        if (two) {
            const float h = v * v;
            a2 = ds_add_f(ds_add_f(a2, h), fmaf(v, v, -h));
            s2[i] = make_float2(a2.hi, a2.lo);
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    DS e1 = a1, e2 = a2;  // inclusive scan of the run totals within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const DS u1 = {__shfl_up_sync(0xffffffffu, e1.hi, o), __shfl_up_sync(0xffffffffu, e1.lo, o)};
        const DS u2 = {__shfl_up_sync(0xffffffffu, e2.hi, o), __shfl_up_sync(0xffffffffu, e2.lo, o)};
        if (lane >= o) {
            e1 = ds_add(u1, e1);
            e2 = ds_add(u2, e2);
        }
    }
    if (lane == 31) {
        wsum1[warp] = e1;
        wsum2[warp] = e2;
    }
    // exclusive offset of this thread's run: the totals of the earlier warps,
    // then the previous lanes' inclusive total
    DS ex1 = {__shfl_up_sync(0xffffffffu, e1.hi, 1), __shfl_up_sync(0xffffffffu, e1.lo, 1)};
    DS ex2 = {__shfl_up_sync(0xffffffffu, e2.hi, 1), __shfl_up_sync(0xffffffffu, e2.lo, 1)};
    if (lane == 0) ex1 = ex2 = DS{0.f, 0.f};
    __syncthreads();
    DS off1 = {0.f, 0.f}, off2 = {0.f, 0.f};
    for (int w = 0; w < warp; ++w) {
        off1 = ds_add(off1, wsum1[w]);
        off2 = ds_add(off2, wsum2[w]);
    }
    off1 = ds_add(off1, ex1);
    off2 = ds_add(off2, ex2);
    for (int i = i0; i < i1; ++i) {
        const float2 v1 = s1[i];
        const DS r1 = ds_add(off1, DS{v1.x, v1.y});
        s1[i] = make_float2(r1.hi, r1.lo);
        if (two) {
            const float2 v2 = s2[i];
            const DS r2 = ds_add(off2, DS{v2.x, v2.y});
            s2[i] = make_float2(r2.hi, r2.lo);
        }
    }
    if (clean) {
        // bounds of |prefix| over the span: sum |x| (the x^2 prefix is
        // non-decreasing, so its last entry), rounded up by a factor 2^-20
        __shared__ float red[kPwThreads / 32 + 1];
        float b = abs1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
        if (lane == 0) red[warp] = b;
        // the last prefix entry, read by its owner before anyone splits it
        if (two && i0 <= span - 1 && span - 1 < i1) red[kPwThreads / 32] = s2[span - 1].x + s2[span - 1].y;
        __syncthreads();
        float bound1 = 0.f;
        for (int w = 0; w < kPwThreads / 32; ++w) bound1 += red[w];
        bound1 *= 1.f + 0x1p-20f;
        const float bound2 = two ? red[kPwThreads / 32] * (1.f + 0x1p-20f) : 0.f;
        if (bound1 < 0x1p120f && bound2 < 0x1p120f) {
            const Quant q1 = quant_of(bound1), q2 = quant_of(bound2);
            for (int i = i0; i < i1; ++i) {
                s1[i] = quant_split(s1[i], q1);
                if (two) s2[i] = quant_split(s2[i], q2);
            }
            __syncthreads();
            switch (a.kind) {
                case WK_SMA: fast_tile<WK_SMA>(a, s1, s2, pmax, t0, r0, cb, ce, cc); break;
                case WK_STDDEV: fast_tile<WK_STDDEV>(a, s1, s2, pmax, t0, r0, cb, ce, cc); break;
                case WK_ZSCORE: fast_tile<WK_ZSCORE>(a, s1, s2, pmax, t0, r0, cb, ce, cc); break;
                default: fast_tile<WK_BB>(a, s1, s2, pmax, t0, r0, cb, ce, cc); break;
            }
            return;
        }
    }
    __syncthreads();
    const int first_nan = a.n - a.bad[0], first_inf = a.n - a.bad[1];
    float2 p1t[kPwPer], p2t[kPwPer];
    float xt[kPwPer];
#pragma unroll
    for (int k = 0; k < kPwPer; ++k) {
        const int l = pmax + threadIdx.x + k * kPwThreads;  // local index of t
        const int t = t0 + threadIdx.x + k * kPwThreads;
        p1t[k] = s1[l];
        p2t[k] = two ? s2[l] : z;
        xt[k] = (a.kind == WK_ZSCORE && t < a.n) ? __fsub_rn(a.x[t], r0) : 0.f;
    }
    for (int c = cb; c < ce; ++c) {
        const int p = a.periods[c];
        const int warm = a.first + p - 1;
        const int poison = min(first_nan, first_inf < a.n ? first_inf + p : a.n);
        const float k1 = a.k1 ? a.k1[c] : 1.f;
        const float k2 = a.k2 ? a.k2[c] : 1.f;
        const float pf = (float)p;
        const float inv_p = __frcp_rn(pf), inv_p2 = inv_p * inv_p;  // 1/p correctly rounded
        float* row0 = a.out0 + (size_t)c * a.n;
#pragma unroll
        for (int k = 0; k < kPwPer; ++k) {
            const int t = t0 + threadIdx.x + k * kPwThreads;
            if (t >= a.n) break;
            const size_t o = (size_t)c * a.n + t;
            if (t < warm || t >= poison) {
                row0[t] = qnan();
                if (a.kind == WK_BB) { a.out1[o] = qnan(); a.out2[o] = qnan(); }
                continue;
            }
            const int lb = pmax + threadIdx.x + k * kPwThreads - p;  // local index of t - p
            const DS w1 = ds_sub2(p1t[k], s1[lb]);
            const DS w2 = two ? ds_sub2_ge(p2t[k], s2[lb]) : DS{0.f, 0.f};
            WinOut r = window_eval(a.kind, w1, w2, pf, inv_p, inv_p2, xt[k], k1, k2);
            // r0 is 0 unless a clean tile's bound check failed after its
            // prefixes were built centred on r0 (values near the f32 range)
            if (a.kind == WK_SMA || a.kind == WK_BB) {
                r.o0 = __fadd_rn(r.o0, r0);
                r.o1 = __fadd_rn(r.o1, r0);
                r.o2 = __fadd_rn(r.o2, r0);
            }
            row0[t] = r.o0;
            if (a.kind == WK_BB) { a.out1[o] = r.o1; a.out2[o] = r.o2; }
        }
    }
}

// ---------------------------------------------- prefix windows, time-major -
constexpr int kTmChunk = 512;

__global__ void k_prefix_window_tm(PrefixWinTmArgs a, const int* first_nan) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.cols) return;
    const int c0 = blockIdx.y * kTmChunk;
    const int c1 = min(c0 + kTmChunk, a.rows);
    const int f = a.first[s];
    const int fn = first_nan[s];
    const int p = a.period;
    const int warm = f + p - 1;
    const size_t S = a.cols;
    const float pf = (float)p;
    const float inv_p = 1.f / pf, inv_p2 = inv_p * inv_p;
    auto X = [&](int t) { return __ldg(a.x_tm + (size_t)t * S + s); };
    int t = c0;
    for (; t < c1 && t < warm; ++t) {
        a.out0[(size_t)t * S + s] = qnan();
        if (a.kind == WK_BB) { a.out1[(size_t)t * S + s] = qnan(); a.out2[(size_t)t * S + s] = qnan(); }
    }
    if (t >= c1) return;
    DS s1 = {0.f, 0.f}, s2 = {0.f, 0.f};
    for (int k = t - p + 1; k <= t; ++k) {
        const float v = X(k);
        s1 = ds_add_f(s1, v);
        const float vv = v * v;
        s2 = ds_add_f(ds_add_f(s2, vv), fmaf(v, v, -vv));
    }
    for (; t < c1; ++t) {
        if (t > c0 && t > warm) {
            const float vn = X(t), vo = X(t - p);
            s1 = ds_add_f(ds_add_f(s1, vn), -vo);
            const float nn = vn * vn, oo = vo * vo;
            s2 = ds_add_f(ds_add_f(s2, nn), fmaf(vn, vn, -nn));
            s2 = ds_add_f(ds_add_f(s2, -oo), -fmaf(vo, vo, -oo));
        }
        const size_t o = (size_t)t * S + s;
        if (t >= fn) {
            a.out0[o] = qnan();
            if (a.kind == WK_BB) { a.out1[o] = qnan(); a.out2[o] = qnan(); }
            continue;
        }
        const WinOut r = window_eval(a.kind, s1, s2, pf, inv_p, inv_p2, a.kind == WK_ZSCORE ? X(t) : 0.f, a.k1, a.k2);
        a.out0[o] = r.o0;
        if (a.kind == WK_BB) { a.out1[o] = r.o1; a.out2[o] = r.o2; }
    }
}

// First NaN strictly after the first valid index, per time-major series.
__global__ void k_first_nan_after_tm(const float* __restrict__ x, int cols, int rows,
                                     const int* first, int* out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= cols) return;
    int t = first[s] + 1;
    while (t < rows && !isnan(x[(size_t)t * cols + s])) ++t;
    out[s] = t < rows ? t : rows;
}

// ------------------------------------------------- min/max, batch ----------
// One block per output time tile; a sparse table of window maxima of `high`
// and minima of `low` over the tile's input span lives in shared memory and
// serves every combo: max over [t-p+1, t] = max(M_k[t-p+1], M_k[t-2^k+1])
// with k = floor(log2 p).  Invalid inputs are counted in prefix arrays so a
// window containing one yields NaN (NaN rule for WillR and Donchian p <= 32,
// non-finite rule for Donchian p > 32, donchian.rs:327-346 / 413-480).
constexpr int kMmThreads = 512;

// WillR of a slot whose range hmax - lmin lies in [2^-100, 2^120]
// (willr_wide_ok): the hardware reciprocal of a range whose reciprocal is
// normal (relative error within about 2^-23, like the fast divide) with no
// zero guard or subnormal handling.  Tiles use it when every slot of the warp
// qualifies; the others take the guarded form.
__device__ __forceinline__ bool willr_wide_ok(float range) {
    return range >= 0x1p-100f && range <= 0x1p120f;
}
__device__ __forceinline__ float willr_wide(float hmax, float lmin, float c) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(hmax - lmin));
    return fmaf(-100.f, (hmax - c) * r, 0.f);
}

// Outputs of a clean tile (every window past its warm-up is valid): combo-
// outer, so a combo's table offsets are read once for the thread's PER times
// t = t0 + tid + k * THREADS; the closes are read once for all combos.
template <int KIND, int PER, int THREADS>
__device__ __forceinline__ void minmax_clean(const MinMaxArgs& a, const float* mx, const float* mn,
                                             const int4* ctab, int t0, int tile, int cb, int ce) {
    const int tid = threadIdx.x;
    const bool full = t0 + tile <= a.n;
    float cl[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int t = t0 + tid + k * THREADS;
        cl[k] = (KIND == MM_WILLR && t < a.n) ? __ldg(a.c + t) : 0.f;
    }
    const int ie0 = tid + a.pmax - 1;  // local index of t0 + tid
    for (int c = cb; c < ce; ++c) {
        const int4 ct = ctab[c];
        const size_t o = (size_t)c * a.n + t0 + tid;
        float* r0 = a.out0 + o;
        const float* mz = mx + ie0 + ct.z;
        const float* mw = mx + ie0 + ct.w;
        const float* nz = mn + ie0 + ct.z;
        const float* nw = mn + ie0 + ct.w;
        float* r1 = KIND == MM_DONCHIAN ? a.out1 + o : nullptr;
        float* r2 = KIND == MM_DONCHIAN ? a.out2 + o : nullptr;
        // value of slot k (hmax, lmin and the close are finite prices: the
        // fast divide is within 2 ulp)
        auto emit = [&](int k, bool valid) {
            const float hmax = fmaxf(mz[k * THREADS], mw[k * THREADS]);
            const float lmin = fminf(nz[k * THREADS], nw[k * THREADS]);
            if (KIND == MM_DONCHIAN) {
                r0[k * THREADS] = valid ? hmax : qnan();
                r1[k * THREADS] = valid ? fmaf(hmax - lmin, 0.5f, lmin) : qnan();
                r2[k * THREADS] = valid ? lmin : qnan();
            } else {
                const float den = hmax - lmin;
                const float v = den == 0.f ? 0.f : fmaf(-100.f, __fdividef(hmax - cl[k], den), 0.f);
                r0[k * THREADS] = valid ? v : qnan();
            }
        };
        if (full && t0 >= ct.y) {  // the whole tile is valid for this combo (uniform branch)
            bool fast = KIND == MM_WILLR;
            if (KIND == MM_WILLR) {
                bool wide = true;
#pragma unroll
                for (int k = 0; k < PER; ++k)
                    wide = wide && willr_wide_ok(fmaxf(mz[k * THREADS], mw[k * THREADS]) -
                                                 fminf(nz[k * THREADS], nw[k * THREADS]));
                fast = __all_sync(0xffffffffu, wide);
            }
            if (fast) {
#pragma unroll
                for (int k = 0; k < PER; ++k) {
                    const float hmax = fmaxf(mz[k * THREADS], mw[k * THREADS]);
                    const float lmin = fminf(nz[k * THREADS], nw[k * THREADS]);
                    r0[k * THREADS] = willr_wide(hmax, lmin, cl[k]);
                }
            } else {
#pragma unroll
                for (int k = 0; k < PER; ++k) emit(k, true);
            }
        } else {
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const int t = t0 + tid + k * THREADS;
                if (t < a.n) emit(k, t >= ct.y);
            }
        }
    }
}

// THREADS threads per block (the autotuner's choice with the tile): fewer
// threads give each more times per combo, which spreads the combo's table and
// pointer set-up over more outputs.
// Block (tile, g): the tile's times for the combos [g cpb, (g + 1) cpb); each
// combo group rebuilds the tile's table (a few combos' worth of work), so the
// grid fills the GPU in whole waves.
template <int THREADS>
__global__ void __launch_bounds__(THREADS)
k_minmax_batch(MinMaxArgs a, int tile, int levels, int cpb) {
    if (a.skip_clean && !a.dirty[blockIdx.x]) return;  // k_minmax_ap wrote this tile
    extern __shared__ float sm[];
    const int cb = blockIdx.y * cpb, ce = min(a.n_combos, cb + cpb);
    const int t0 = blockIdx.x * tile;
    const int lo_i = t0 - (a.pmax - 1);  // global index of smem slot 0
    const int nloc = tile + a.pmax - 1;
    float* mx = sm;                          // [levels][nloc]
    float* mn = sm + (size_t)levels * nloc;  // [levels][nloc]
    int* bad_nan = reinterpret_cast<int*>(mn + (size_t)levels * nloc);  // [nloc+1]
    int* bad_fin = bad_nan + nloc + 1;                                   // [nloc+1]
    // per combo: window start and first output index, and the two table
    // offsets of the window's sparse-table lookups (level k, positions
    // t - p + 1 and t - 2^k + 1 relative to the local index of t)
    const size_t ctab_at = ((size_t)2 * levels * nloc + 2 * ((size_t)nloc + 1) + 3) & ~size_t(3);  // 16-byte aligned
    int4* ctab = reinterpret_cast<int4*>(reinterpret_cast<int*>(sm) + ctab_at);
    for (int c = cb + threadIdx.x; c < ce; c += blockDim.x) {
        const int p = a.periods[c];
        const int k = 31 - __clz(p);
        ctab[c] = make_int4(p, a.first + p - 1, k * nloc - p + 1, k * nloc - (1 << k) + 1);
    }
    // level 0 + invalid flags; a span whose valid part holds only finite
    // highs and lows (and closes at the tile's times) is clean: every window
    // of the tile is then valid past its warm-up, and no counts are needed
    int any_bad = 0;
    for (int i = threadIdx.x; i < nloc; i += blockDim.x) {
        const int g = lo_i + i;
        float hv = -INFINITY, lv = INFINITY;
        int fnan = 0, ffin = 0;
        if (g >= 0 && g < a.n) {
            const float h = a.h[g], l = a.l[g];
            fnan = (isnan(h) || isnan(l)) ? 1 : 0;
            ffin = (isfinite(h) && isfinite(l)) ? 0 : 1;
            if (!fnan) { hv = h; lv = l; }
            if (g >= a.first) any_bad |= ffin;
            if (a.kind == MM_WILLR && g >= a.first && i >= a.pmax - 1 && isnan(a.c[g])) any_bad = 1;
        }
        mx[i] = hv;
        mn[i] = lv;
        bad_nan[i + 1] = fnan;
        bad_fin[i + 1] = ffin;
    }
    if (threadIdx.x == 0) { bad_nan[0] = 0; bad_fin[0] = 0; }
    const bool clean = !__syncthreads_or(any_bad);

    // prefix counts (single warp, sequential per lane-strided segments)
    if (!clean && threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const int seg = (nloc + 31) / 32;
        const int b = 1 + lane * seg, e = min(nloc + 1, b + seg);
        int cn = 0, cf = 0;
        for (int i = b; i < e; ++i) { cn += bad_nan[i]; cf += bad_fin[i]; bad_nan[i] = cn; bad_fin[i] = cf; }
        int on = cn, of = cf;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int un = __shfl_up_sync(0xffffffffu, on, o);
            const int uf = __shfl_up_sync(0xffffffffu, of, o);
            if (lane >= o) { on += un; of += uf; }
        }
        on -= cn; of -= cf;  // exclusive offsets
        for (int i = b; i < e; ++i) { bad_nan[i] += on; bad_fin[i] += of; }
    }
    // higher levels
    for (int k = 1; k < levels; ++k) {
        __syncthreads();
        const int half = 1 << (k - 1);
        const float* pmx = mx + (size_t)(k - 1) * nloc;
        const float* pmn = mn + (size_t)(k - 1) * nloc;
        float* cmx = mx + (size_t)k * nloc;
        float* cmn = mn + (size_t)k * nloc;
        for (int i = threadIdx.x; i + half < nloc; i += blockDim.x) {
            cmx[i] = fmaxf(pmx[i], pmx[i + half]);
            cmn[i] = fminf(pmn[i], pmn[i + half]);
        }
    }
    __syncthreads();
    if (clean && tile >= THREADS && tile <= 8 * THREADS) {
        const int per = tile / THREADS;  // 1, 2, 4 or 8
        if (a.kind == MM_DONCHIAN) {
            if (per == 1) minmax_clean<MM_DONCHIAN, 1, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
            else if (per == 2) minmax_clean<MM_DONCHIAN, 2, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
            else if (per == 4) minmax_clean<MM_DONCHIAN, 4, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
            else minmax_clean<MM_DONCHIAN, 8, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
        } else {
            if (per == 1) minmax_clean<MM_WILLR, 1, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
            else if (per == 2) minmax_clean<MM_WILLR, 2, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
            else if (per == 4) minmax_clean<MM_WILLR, 4, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
            else minmax_clean<MM_WILLR, 8, THREADS>(a, mx, mn, ctab, t0, tile, cb, ce);
        }
        return;
    }
    for (int tt = threadIdx.x; tt < tile; tt += blockDim.x) {
        const int t = t0 + tt;
        if (t >= a.n) break;
        const float cl = a.kind == MM_WILLR ? a.c[t] : 0.f;
        const int ie = t - lo_i;  // local index of t
        float* o0 = a.out0 + (size_t)cb * a.n + t;
        float* o1 = a.out1 + (size_t)cb * a.n + t;
        float* o2 = a.out2 + (size_t)cb * a.n + t;
        for (int c = cb; c < ce; ++c, o0 += a.n, o1 += a.n, o2 += a.n) {
            const int4 ct = ctab[c];
            const int p = ct.x;
            float r0 = qnan(), r1 = qnan(), r2 = qnan();
            if (t >= ct.y) {
                const int ib = ie - p + 1;
                const float hmax = fmaxf(mx[ie + ct.z], mx[ie + ct.w]);
                const float lmin = fminf(mn[ie + ct.z], mn[ie + ct.w]);
                const int nn = clean ? 0 : bad_nan[ie + 1] - bad_nan[ib];
                if (a.kind == MM_DONCHIAN) {
                    const int nb = clean ? 0 : (p > 32 ? bad_fin[ie + 1] - bad_fin[ib] : nn);
                    if (nb == 0) {
                        r0 = hmax;
                        r2 = lmin;
                        r1 = fmaf(hmax - lmin, 0.5f, lmin);
                    }
                } else {
                    if (!isnan(cl) && nn == 0 && isfinite(hmax) && isfinite(lmin)) {
                        const float den = hmax - lmin;
                        // hmax, lmin and cl are finite prices: the fast divide
                        // is within 2 ulp
                        r0 = den == 0.f ? 0.f : fmaf(-100.f, __fdividef(hmax - cl, den), 0.f);
                    }
                }
            }
            *o0 = r0;
            if (a.kind == MM_DONCHIAN) {
                *o1 = r1;
                *o2 = r2;
            }
        }
    }
}

// ---- arithmetic-progression sweeps ----------------------------------------
// Periods p_c = p_0 + c d (ascending, constant step d: the crate's range
// grids).  The window of combo c is combo c - 1's window extended by the d
// bars before it, so hmax_c(t) = max(hmax_{c-1}(t), M_d(t - p_{c-1})) with M_d
// the d-bar sliding maximum, built once per tile in shared memory (likewise
// the lows).  Per output: two shared-memory loads and two min/max (exact, so
// the same values as the sparse-table lookups) instead of four loads and the
// per-combo table set-up.  The first combo's window (of each combo group of
// the block) comes from p mod d single bars and p / d blocks of M_d.  Clean tiles only (the same test as
// k_minmax_batch); k_minmax_batch, launched after with skip_clean, computes
// the others.
template <int KIND, int THREADS, int PER>
__global__ void __launch_bounds__(THREADS) k_minmax_ap(MinMaxArgs a, int tile, int cpb) {
    extern __shared__ float sm[];
    const int cb = blockIdx.y * cpb, ce = min(a.n_combos, cb + cpb);  // this block's combos
    const int t0 = blockIdx.x * tile;
    const int lo_i = t0 - (a.pmax - 1);  // global index of slot 0
    const int nloc = tile + a.pmax - 1;
    const int d = a.ap_d;
    float* xh = sm;
    float* xl = xh + nloc;
    float* mh = xl + nloc;
    float* ml = mh + nloc;
    int any_bad = 0;
    for (int i = threadIdx.x; i < nloc; i += THREADS) {
        const int g = lo_i + i;
        float hv = -INFINITY, lv = INFINITY;
        if (g >= 0 && g < a.n) {
            const float h = __ldg(a.h + g), l = __ldg(a.l + g);
            if (!(isnan(h) || isnan(l))) {
                hv = h;
                lv = l;
            }
            if (g >= a.first && !(isfinite(h) && isfinite(l))) any_bad = 1;
            if (KIND == MM_WILLR && g >= a.first && i >= a.pmax - 1 && isnan(__ldg(a.c + g))) any_bad = 1;
        }
        xh[i] = hv;
        xl[i] = lv;
    }
    const int bad = __syncthreads_or(any_bad);
    if (blockIdx.y == 0 && threadIdx.x == 0) a.dirty[blockIdx.x] = bad ? 1 : 0;
    if (bad) return;  // k_minmax_batch computes this tile
    // M_d: the d-bar sliding max / min ending at slot i (i >= d - 1)
    for (int i = threadIdx.x; i < nloc; i += THREADS) {
        float hv = -INFINITY, lv = INFINITY;
        if (i >= d - 1)
            for (int j = 0; j < d; ++j) {
                hv = fmaxf(hv, xh[i - j]);
                lv = fminf(lv, xl[i - j]);
            }
        mh[i] = hv;
        ml[i] = lv;
    }
    __syncthreads();
    const int tid = threadIdx.x;
    const bool full = t0 + tile <= a.n;
    const int p0 = __ldg(a.periods + cb);  // the group's first period
    const int r = p0 % d, nb = p0 / d;
    float hm[PER], lm[PER], cl[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int t = t0 + tid + k * THREADS;
        const int ie = tid + k * THREADS + a.pmax - 1;  // slot of t
        cl[k] = (KIND == MM_WILLR && t < a.n) ? __ldg(a.c + t) : 0.f;
        float h = -INFINITY, l = INFINITY;
        for (int i = 0; i < r; ++i) {
            h = fmaxf(h, xh[ie - i]);
            l = fminf(l, xl[ie - i]);
        }
        for (int j = 0; j < nb; ++j) {
            h = fmaxf(h, mh[ie - r - j * d]);
            l = fminf(l, ml[ie - r - j * d]);
        }
        hm[k] = h;
        lm[k] = l;
    }
    const int ie0 = tid + a.pmax - 1;
    int p = p0;
    for (int c = cb; c < ce; ++c, p += d) {
        if (c > cb) {
            const int back = ie0 - (p - d);  // slot of t - p_{c-1} for k = 0
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                hm[k] = fmaxf(hm[k], mh[back + k * THREADS]);
                lm[k] = fminf(lm[k], ml[back + k * THREADS]);
            }
        }
        const int warm = a.first + p - 1;
        const size_t o = (size_t)c * a.n + t0 + tid;
        float* r0 = a.out0 + o;
        float* r1 = KIND == MM_DONCHIAN ? a.out1 + o : nullptr;
        float* r2 = KIND == MM_DONCHIAN ? a.out2 + o : nullptr;
        // value of slot k (finite prices: the fast divide is within 2 ulp)
        auto emit = [&](int k, bool valid) {
            if (KIND == MM_DONCHIAN) {
                r0[k * THREADS] = valid ? hm[k] : qnan();
                r1[k * THREADS] = valid ? fmaf(hm[k] - lm[k], 0.5f, lm[k]) : qnan();
                r2[k * THREADS] = valid ? lm[k] : qnan();
            } else {
                const float den = hm[k] - lm[k];
                const float v = den == 0.f ? 0.f : fmaf(-100.f, __fdividef(hm[k] - cl[k], den), 0.f);
                r0[k * THREADS] = valid ? v : qnan();
            }
        };
        if (full && t0 >= warm) {  // the whole tile is valid for this combo (uniform branch)
            bool fast = KIND == MM_WILLR;
            if (KIND == MM_WILLR) {
                bool wide = true;
#pragma unroll
                for (int k = 0; k < PER; ++k) wide = wide && willr_wide_ok(hm[k] - lm[k]);
                fast = __all_sync(0xffffffffu, wide);
            }
            if (fast) {
#pragma unroll
                for (int k = 0; k < PER; ++k) r0[k * THREADS] = willr_wide(hm[k], lm[k], cl[k]);
            } else {
#pragma unroll
                for (int k = 0; k < PER; ++k) emit(k, true);
            }
        } else {
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const int t = t0 + tid + k * THREADS;
                if (t < a.n) emit(k, t >= warm);
            }
        }
    }
}

// Direct window scan (large windows that do not fit the shared-memory table).
__global__ void k_minmax_batch_naive(MinMaxArgs a) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (t >= a.n || c >= a.n_combos) return;
    const int p = a.periods[c];
    const size_t o = (size_t)c * a.n + t;
    float r0 = qnan(), r1 = qnan(), r2 = qnan();
    if (t >= a.first + p - 1) {
        float hmax = -INFINITY, lmin = INFINITY;
        bool bad_n = false, bad_f = false;
        for (int j = t - p + 1; j <= t; ++j) {
            const float h = a.h[j], l = a.l[j];
            if (isnan(h) || isnan(l)) { bad_n = true; bad_f = true; break; }
            if (!isfinite(h) || !isfinite(l)) bad_f = true;
            hmax = fmaxf(hmax, h);
            lmin = fminf(lmin, l);
        }
        if (a.kind == MM_DONCHIAN) {
            if (!(p > 32 ? bad_f : bad_n)) { r0 = hmax; r2 = lmin; r1 = fmaf(hmax - lmin, 0.5f, lmin); }
        } else {
            const float cl = a.c[t];
            if (!isnan(cl) && !bad_n && isfinite(hmax) && isfinite(lmin)) {
                const float den = hmax - lmin;
                r0 = den == 0.f ? 0.f : fmaf(-100.f, (hmax - cl) / den, 0.f);
            }
        }
    }
    a.out0[o] = r0;
    if (a.kind == MM_DONCHIAN) { a.out1[o] = r1; a.out2[o] = r2; }
}

// ------------------------------------------------- min/max, time-major -----
constexpr int kMmTmChunk = 256;

__global__ void k_minmax_tm(MinMaxTmArgs a) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.cols) return;
    const int c0 = blockIdx.y * kMmTmChunk;
    const int c1 = min(c0 + kMmTmChunk, a.rows);
    const int p = a.period, f = a.first[s];
    const size_t S = a.cols;
    for (int t = c0; t < c1; ++t) {
        const size_t o = (size_t)t * S + s;
        float r0 = qnan(), r1 = qnan(), r2 = qnan();
        if (t >= f + p - 1) {
            float hmax = -INFINITY, lmin = INFINITY;
            bool bad_n = false, bad_f = false;
            for (int j = t - p + 1; j <= t; ++j) {
                const float h = __ldg(a.h + (size_t)j * S + s), l = __ldg(a.l + (size_t)j * S + s);
                if (isnan(h) || isnan(l)) { bad_n = true; bad_f = true; break; }
                if (!isfinite(h) || !isfinite(l)) bad_f = true;
                hmax = fmaxf(hmax, h);
                lmin = fminf(lmin, l);
            }
            if (a.kind == MM_DONCHIAN) {
                if (!(p > 32 ? bad_f : bad_n)) { r0 = hmax; r2 = lmin; r1 = fmaf(hmax - lmin, 0.5f, lmin); }
            } else {
                const float cl = a.c[o];
                if (!isnan(cl) && !bad_n && isfinite(hmax) && isfinite(lmin)) {
                    const float den = hmax - lmin;
                    r0 = den == 0.f ? 0.f : fmaf(-100.f, (hmax - cl) / den, 0.f);
                }
            }
        }
        a.out0[o] = r0;
        if (a.kind == MM_DONCHIAN) { a.out1[o] = r1; a.out2[o] = r2; }
    }
}

// ------------------------------------------------- percentile --------------
// Sorted window of the non-NaN values (percentile_nearest_rank.rs:190-266):
// binary-search removal of the value leaving and insertion of the value
// entering; out = sorted[k], k = round(p*wl) - 1 clamped.  Exact selection,
// so results are bit-identical to the crate on the same f32 inputs.
constexpr int kPnrChunk = 256;
constexpr int kPnrLocal = 64;

using pnr::rank;

__device__ __forceinline__ int lower_bound(const float* w, int n, float v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (w[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ void pnr_lane(const float* x, size_t stride, int n, int f, int len, double pf, int c0,
                         int c1, float* out, size_t ostride, float* win) {
    const int start = f + len - 1;
    int t = c0;
    for (; t < c1 && t < start; ++t) out[(size_t)t * ostride] = qnan();
    if (t >= c1) return;
    int wl = 0;
    for (int j = t - len + 1; j <= t; ++j) {
        const float v = x[(size_t)j * stride];
        if (isnan(v)) continue;
        int pos = wl;
        while (pos > 0 && win[pos - 1] > v) { win[pos] = win[pos - 1]; --pos; }
        win[pos] = v;
        ++wl;
    }
    const int kfull = rank(pf, len);
    for (;;) {
        float r = qnan();
        if (wl > 0) r = win[wl == len ? kfull : rank(pf, wl)];
        out[(size_t)t * ostride] = r;
        if (t + 1 >= c1) break;
        const float vo = x[(size_t)(t + 1 - len) * stride];
        if (!isnan(vo)) {
            int pos = lower_bound(win, wl, vo);
            if (pos < wl && win[pos] == vo) {
                for (int k = pos; k + 1 < wl; ++k) win[k] = win[k + 1];
                --wl;
            }
        }
        const float vi = x[(size_t)(t + 1) * stride];
        if (!isnan(vi)) {
            int pos = lower_bound(win, wl, vi);
            for (int k = wl; k > pos; --k) win[k] = win[k - 1];
            win[pos] = vi;
            ++wl;
        }
        ++t;
    }
}

// One lane's outputs [c0, c1) with the window sorted in W registers (len <=
// W): every lane of the warp runs one step loop over [u0, c1), u0 the warp's
// earliest window start, replacing the value leaving its window by the one
// entering (pnr_ops.cuh); a lane whose window has not started yet adds only.
template <int W>
__device__ void pnr_lane_reg(const float* x, size_t stride, int f, int len, double pf, int c0, int c1, int u0,
                             float* out, size_t ostride) {
    const int start = f + len - 1;
    const int tbeg = max(0, c0 - len + 1);  // this lane's first window value
    const int kfull = pnr::rank(pf, len);
    float w[W];
#pragma unroll
    for (int i = 0; i < W; ++i) w[i] = __int_as_float(0x7f800000);
    int wl = 0;
    for (int u = u0; u < c1; ++u) {
        const int uo = u - len;
        const float vi = u >= tbeg ? __ldg(x + (size_t)u * stride) : qnan();
        const float vo = uo >= tbeg ? __ldg(x + (size_t)uo * stride) : qnan();
        pnr::replace(w, vo, vi);
        wl += (isnan(vi) ? 0 : 1) - (isnan(vo) ? 0 : 1);
        if (u >= c0) out[(size_t)u * ostride] = u < start ? qnan() : pnr::pick(w, wl, len, kfull, pf);
    }
}

__global__ void k_percentile(PnrArgs a) {
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    const int c0 = blockIdx.y * kPnrChunk;
    const int c1 = min(c0 + kPnrChunk, a.n);
    if (c0 >= a.n) return;
    // windows of at most 64 values: the register window, sized by the
    // warp's longest window (warp-uniform); longer ones: the sorted array
    {
        const bool live = li < a.n_lanes;
        const int len = live ? (a.layout == 0 ? a.lengths[li] : a.length) : 1;
        const int wmax = __reduce_max_sync(0xffffffffu, len);
        if (wmax <= 64) {
            const int u0 = max(0, c0 - wmax + 1);
            const float* x = a.layout == 0 ? a.x : a.x + (live ? li : 0);
            const size_t stride = a.layout == 0 ? 1 : (size_t)a.cols;
            const int f = a.layout == 0 ? a.first : (live ? a.first_tm[li] : 0);
            const double pf = a.layout == 0 ? (live ? (double)a.pfrac[li] : 0.5) : (double)a.p_frac;
            float* out = a.layout == 0 ? a.out + (size_t)(live ? li : 0) * a.n : a.out + (live ? li : 0);
            const size_t ostride = a.layout == 0 ? 1 : (size_t)a.cols;
            if (!live) return;  // after the warp-wide reduction
            switch ((wmax + 7) / 8) {
                case 1: case 2: pnr_lane_reg<16>(x, stride, f, len, pf, c0, c1, u0, out, ostride); break;
                case 3: pnr_lane_reg<24>(x, stride, f, len, pf, c0, c1, u0, out, ostride); break;
                case 4: pnr_lane_reg<32>(x, stride, f, len, pf, c0, c1, u0, out, ostride); break;
                case 5: pnr_lane_reg<40>(x, stride, f, len, pf, c0, c1, u0, out, ostride); break;
                case 6: pnr_lane_reg<48>(x, stride, f, len, pf, c0, c1, u0, out, ostride); break;
                case 7: pnr_lane_reg<56>(x, stride, f, len, pf, c0, c1, u0, out, ostride); break;
                default: pnr_lane_reg<64>(x, stride, f, len, pf, c0, c1, u0, out, ostride); break;
            }
            return;
        }
    }
    if (li >= a.n_lanes) return;
    float local[kPnrLocal];
    if (a.layout == 0) {
        const int len = a.lengths[li];
        float* win = len <= kPnrLocal ? local
                                      : a.scratch + ((size_t)blockIdx.y * a.n_lanes + li) * (size_t)a.length;
        pnr_lane(a.x, 1, a.n, a.first, len, (double)a.pfrac[li], c0, c1, a.out + (size_t)li * a.n, 1, win);
    } else {
        float* win = a.length <= kPnrLocal
                         ? local
                         : a.scratch + ((size_t)blockIdx.y * a.n_lanes + li) * (size_t)a.length;
        pnr_lane(a.x + li, a.cols, a.n, a.first_tm[li], a.length, (double)a.p_frac, c0, c1, a.out + li,
                 a.cols, win);
    }
}

}  // namespace

// Combos per block for a grid of `tiles` time tiles x combo groups: the
// grid in (nearly) whole waves of the kernel's resident blocks, counting a
// group's per-tile set-up (prefix or table rebuild) as ~4 combos of work.
template <class K>
static int wave_combos(K kern, int threads, size_t smem, long long tiles, int n_combos) {
    int per_sm = 0, dev = 0, sms = kNumSMs;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        per_sm = 1;
    }
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long slots = (long long)std::max(1, per_sm) * sms;
    int best_g = 1;
    double best = 1e300;
    for (int g = 1; g <= 16 && g <= n_combos; ++g) {
        const int cpb = (n_combos + g - 1) / g;
        const long long blocks = tiles * ((n_combos + cpb - 1) / cpb);
        const double cost = (double)((blocks + slots - 1) / slots) * (cpb + 4);
        if (cost < best * 0.98) {
            best = cost;
            best_g = g;
        }
    }
    return (n_combos + best_g - 1) / best_g;
}

vta_status launch_prefix_window_batch(const PrefixWinArgs& a, int pmax, size_t smem_optin, cudaStream_t st) {
    const size_t smem = (size_t)(kPwTile + pmax) * sizeof(float2) * (a.kind == WK_SMA ? 1 : 2);
    if (smem + 2 * (kPwThreads / 32) * sizeof(DS) > smem_optin)
        return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "prefix window: period too large");
    VTA_CUDA_TRY(cudaMemsetAsync(a.bad, 0, 2 * sizeof(int), st));
    if (a.first < a.n) {
        k_first_bad<<<std::min<int>(ceil_div(a.n - a.first, 256), 4 * kNumSMs), 256, 0, st>>>(a.x, a.n, a.first, a.bad);
        VTA_TRY(check_launch("k_first_bad"));
    }
    VTA_CUDA_TRY(cudaFuncSetAttribute(k_prefix_window_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long tiles = ceil_div(a.n, kPwTile);
    const int cpb = wave_combos(k_prefix_window_batch, kPwThreads, smem, tiles, a.n_combos);
    ktimer_begin(st);
    k_prefix_window_batch<<<dim3((unsigned)tiles, (unsigned)ceil_div(a.n_combos, cpb)), kPwThreads, smem, st>>>(a, pmax,
                                                                                                              cpb);
    ktimer_end(st);
    return check_launch("k_prefix_window_batch");
}

// first_nan scratch is carved by the caller right after `first`
vta_status launch_prefix_window_tm(const PrefixWinTmArgs& a, cudaStream_t st) {
    int* first_nan = const_cast<int*>(a.first) + a.cols;
    k_first_nan_after_tm<<<ceil_div(a.cols, 128), 128, 0, st>>>(a.x_tm, a.cols, a.rows, a.first, first_nan);
    VTA_TRY(check_launch("k_first_nan_after_tm"));
    dim3 grid(ceil_div(a.cols, 128), ceil_div(a.rows, kTmChunk));
    ktimer_begin(st);
    k_prefix_window_tm<<<grid, 128, 0, st>>>(a, first_nan);
    ktimer_end(st);
    return check_launch("k_prefix_window_tm");
}

static size_t minmax_smem(const MinMaxArgs& a, int tile, int levels) {
    const size_t nloc = (size_t)tile + a.pmax - 1;
    return nloc * levels * 2 * sizeof(float) + (2 * (nloc + 1) + 4) * sizeof(int) + (size_t)a.n_combos * sizeof(int4);
}

// Candidates encoded as tile | threads << 16 | split << 28 (split: combo
// groups per tile from the wave model; without it one block per tile).
constexpr int kMmSplitBit = 1 << 28;
// bit 29: the progression kernel on clean tiles (tile kMmApTile), the
// sparse-table kernel on the rest
constexpr int kMmApBit = 1 << 29;
constexpr int kMmApThreads = 256, kMmApPer = 4, kMmApTile = kMmApThreads * kMmApPer;
static bool minmax_ap_ok(const MinMaxArgs& a, size_t smem_optin) {
    const int levels = 32 - __builtin_clz((unsigned)a.pmax);
    const size_t nloc = (size_t)kMmApTile + a.pmax - 1;
    return a.ap_d >= 1 && a.ap_d <= 64 && a.n_combos >= 2 && a.dirty && 4 * nloc * sizeof(float) <= smem_optin &&
           minmax_smem(a, kMmApTile, levels) <= smem_optin;
}
bool minmax_uses_progression(const MinMaxArgs& a, size_t smem_optin) {
    return (a.tile_hint == 0 || (a.tile_hint & kMmApBit)) && minmax_ap_ok(a, smem_optin);
}
std::vector<int> minmax_tile_candidates(const MinMaxArgs& a, size_t smem_optin) {
    const int levels = 32 - __builtin_clz((unsigned)a.pmax);
    std::vector<int> c;
    const int cfg[][2] = {{512, 512}, {512, 256}, {512, 128}, {1024, 512}, {1024, 256}, {1024, 128}};
    for (const auto& tc : cfg)
        if (minmax_smem(a, tc[0], levels) <= smem_optin && (size_t)a.n >= (size_t)tc[0] * 2 * kNumSMs)
            for (int split : {0, kMmSplitBit}) c.push_back(tc[0] | (tc[1] << 16) | split);
    if (minmax_ap_ok(a, smem_optin) && !c.empty()) c.push_back(kMmApTile | (512 << 16) | kMmApBit);
    return c.size() > 1 ? c : std::vector<int>{};
}

vta_status launch_minmax_batch(const MinMaxArgs& a_in, size_t smem_optin, cudaStream_t st) {
    MinMaxArgs a = a_in;
    a.skip_clean = 0;
    const int levels = 32 - __builtin_clz((unsigned)a.pmax);  // floor(log2 pmax) + 1
    const bool ap = minmax_uses_progression(a, smem_optin);
    if (ap) {
        // progression kernel on the clean tiles, then the sparse-table kernel
        // (same tiles) on the others
        const size_t bytes = 4 * ((size_t)kMmApTile + a.pmax - 1) * sizeof(float);
        auto kern = a.kind == MM_DONCHIAN ? k_minmax_ap<MM_DONCHIAN, kMmApThreads, kMmApPer>
                                          : k_minmax_ap<MM_WILLR, kMmApThreads, kMmApPer>;
        VTA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
        const long long tiles = ceil_div(a.n, kMmApTile);
        const int cpb = wave_combos(kern, kMmApThreads, bytes, tiles, a.n_combos);
        ktimer_begin(st);
        kern<<<dim3((unsigned)tiles, (unsigned)ceil_div(a.n_combos, cpb)), kMmApThreads, bytes, st>>>(a, kMmApTile,
                                                                                                    cpb);
        VTA_TRY(check_launch("k_minmax_ap"));
        a.skip_clean = 1;
        a.tile_hint = kMmApTile | (512 << 16);
    }
    const int hint_tile = a.tile_hint & 0xffff, hint_threads = (a.tile_hint >> 16) & 0xfff;
    for (int tile = 2048; tile >= 256; tile >>= 1) {
        const size_t bytes = minmax_smem(a, tile, levels);
        const bool pick = hint_tile > 0 ? tile == hint_tile
                                        : (tile <= 512 || (size_t)a.n >= (size_t)tile * 8 * kNumSMs);
        if (bytes <= smem_optin && pick) {
            const int threads = hint_threads == 128 ? 128 : hint_threads == 256 ? 256 : kMmThreads;
            auto kern = threads == 128 ? k_minmax_batch<128> : threads == 256 ? k_minmax_batch<256>
                                                                               : k_minmax_batch<kMmThreads>;
            VTA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
            // combo groups: as the hint says, else only when one block per
            // tile would not give two waves (the table rebuild and its
            // barriers are latency that few resident blocks do not hide)
            int cpb = a.n_combos;
            const long long tiles = ceil_div(a.n, tile);
            bool split = (a.tile_hint & kMmSplitBit) != 0;
            if (a.tile_hint == 0) {
                int per_sm = 0;
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, bytes) != cudaSuccess) {
                    cudaGetLastError();
                    per_sm = 1;
                }
                split = tiles < 2LL * std::max(1, per_sm) * kNumSMs;
            }
            if (split) cpb = wave_combos(kern, threads, bytes, tiles, a.n_combos);
            if (!ap) ktimer_begin(st);
            kern<<<dim3((unsigned)ceil_div(a.n, tile), (unsigned)ceil_div(a.n_combos, cpb)), threads, bytes, st>>>(
                a, tile, levels, cpb);
            ktimer_end(st);
            return check_launch("k_minmax_batch");
        }
    }
    dim3 grid(ceil_div(a.n, 256), a.n_combos);
    ktimer_begin(st);
    k_minmax_batch_naive<<<grid, 256, 0, st>>>(a);
    ktimer_end(st);
    return check_launch("k_minmax_batch_naive");
}

vta_status launch_minmax_tm(const MinMaxTmArgs& a, cudaStream_t st) {
    dim3 grid(ceil_div(a.cols, 128), ceil_div(a.rows, kMmTmChunk));
    ktimer_begin(st);
    k_minmax_tm<<<grid, 128, 0, st>>>(a);
    ktimer_end(st);
    return check_launch("k_minmax_tm");
}

vta_status launch_percentile(const PnrArgs& a, cudaStream_t st) {
    dim3 grid(ceil_div(a.n_lanes, 64), ceil_div(a.n, kPnrChunk));
    ktimer_begin(st);
    k_percentile<<<grid, 64, 0, st>>>(a);
    ktimer_end(st);
    return check_launch("k_percentile");
}

}  // namespace vta
