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
    WinOut r;
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

__global__ void __launch_bounds__(kPwThreads)
k_prefix_window_batch(PrefixWinArgs a, int pmax) {
    extern __shared__ float2 psm[];
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
    DS a1 = {0.f, 0.f}, a2 = {0.f, 0.f};
    for (int i = i0; i < i1; ++i) {
        const int g = base + i;
        const float v = (g >= a.first && g < a.n) ? __ldg(a.x + g) : 0.f;
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
        xt[k] = (a.kind == WK_ZSCORE && t < a.n) ? a.x[t] : 0.f;
    }
    for (int c = 0; c < a.n_combos; ++c) {
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
            const WinOut r = window_eval(a.kind, w1, w2, pf, inv_p, inv_p2, xt[k], k1, k2);
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

__global__ void __launch_bounds__(kMmThreads)
k_minmax_batch(MinMaxArgs a, int tile, int levels) {
    extern __shared__ float sm[];
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
    for (int c = threadIdx.x; c < a.n_combos; c += blockDim.x) {
        const int p = a.periods[c];
        const int k = 31 - __clz(p);
        ctab[c] = make_int4(p, a.first + p - 1, k * nloc - p + 1, k * nloc - (1 << k) + 1);
    }
    // level 0 + invalid flags
    for (int i = threadIdx.x; i < nloc; i += blockDim.x) {
        const int g = lo_i + i;
        float hv = -INFINITY, lv = INFINITY;
        int fnan = 0, ffin = 0;
        if (g >= 0 && g < a.n) {
            const float h = a.h[g], l = a.l[g];
            fnan = (isnan(h) || isnan(l)) ? 1 : 0;
            ffin = (isfinite(h) && isfinite(l)) ? 0 : 1;
            if (!fnan) { hv = h; lv = l; }
        }
        mx[i] = hv;
        mn[i] = lv;
        bad_nan[i + 1] = fnan;
        bad_fin[i + 1] = ffin;
    }
    if (threadIdx.x == 0) { bad_nan[0] = 0; bad_fin[0] = 0; }
    __syncthreads();
    // prefix counts (single warp, sequential per lane-strided segments)
    if (threadIdx.x < 32) {
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
    // a span without invalid inputs (the usual case) needs no window counts
    const bool clean = bad_nan[nloc] == 0 && bad_fin[nloc] == 0;
    for (int tt = threadIdx.x; tt < tile; tt += blockDim.x) {
        const int t = t0 + tt;
        if (t >= a.n) break;
        const float cl = a.kind == MM_WILLR ? a.c[t] : 0.f;
        const int ie = t - lo_i;  // local index of t
        float* o0 = a.out0 + t;
        float* o1 = a.out1 + t;
        float* o2 = a.out2 + t;
        for (int c = 0; c < a.n_combos; ++c, o0 += a.n, o1 += a.n, o2 += a.n) {
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

__device__ __forceinline__ int pnr_rank(double pf, int wl) {
    long long raw = (long long)round(fma(pf, (double)wl, 0.0)) - 1;
    int k = raw <= 0 ? 0 : (int)raw;
    return k >= wl ? wl - 1 : k;
}

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
    const int kfull = pnr_rank(pf, len);
    for (;;) {
        float r = qnan();
        if (wl > 0) r = win[wl == len ? kfull : pnr_rank(pf, wl)];
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

__global__ void k_percentile(PnrArgs a) {
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= a.n_lanes) return;
    const int c0 = blockIdx.y * kPnrChunk;
    const int c1 = min(c0 + kPnrChunk, a.n);
    if (c0 >= a.n) return;
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
    ktimer_begin(st);
    k_prefix_window_batch<<<ceil_div(a.n, kPwTile), kPwThreads, smem, st>>>(a, pmax);
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

vta_status launch_minmax_batch(const MinMaxArgs& a, size_t smem_optin, cudaStream_t st) {
    const int levels = 32 - __builtin_clz((unsigned)a.pmax);  // floor(log2 pmax) + 1
    for (int tile = 2048; tile >= 256; tile >>= 1) {
        const size_t nloc = (size_t)tile + a.pmax - 1;
        const size_t bytes = nloc * levels * 2 * sizeof(float) + (2 * (nloc + 1) + 4) * sizeof(int) +
                             (size_t)a.n_combos * sizeof(int4);
        if (bytes <= smem_optin && (tile <= 512 || (size_t)a.n >= (size_t)tile * 8 * kNumSMs)) {
            VTA_CUDA_TRY(cudaFuncSetAttribute(k_minmax_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)bytes));
            ktimer_begin(st);
            k_minmax_batch<<<ceil_div(a.n, tile), kMmThreads, bytes, st>>>(a, tile, levels);
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
