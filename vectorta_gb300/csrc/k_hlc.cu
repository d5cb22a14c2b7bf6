// ADX and SuperTrend: per-lane sequential scans over high/low/close.
//
// ADX is a two-level Wilder recurrence whose second level is driven by a
// non-linear function (DX) of the first; SuperTrend is a band state machine.
// Both run one lane per combo (batch, staged stores) or per series
// (time-major, coalesced) over the full series.
#include "hlc_ops.cuh"
#include "vta_internal.h"

namespace vta {
namespace {

constexpr int kWarps = 4;
__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

struct HlcBatch {
    const float *h, *l, *c;
    __device__ float H(int t) const { return __ldg(h + t); }
    __device__ float L(int t) const { return __ldg(l + t); }
    __device__ float C(int t) const { return __ldg(c + t); }
};
struct HlcTm {
    const float *h, *l, *c;
    size_t S, s;
    __device__ float H(int t) const { return __ldg(h + (size_t)t * S + s); }
    __device__ float L(int t) const { return __ldg(l + (size_t)t * S + s); }
    __device__ float C(int t) const { return __ldg(c + (size_t)t * S + s); }
};

// Emits v for time t: time-major writes directly, batch stages through
// shared memory and flushes 32 times x 32 rows per warp.
template <bool TM>
struct Emitter {
    float (*stage)[33];
    float* out;
    size_t n, cols;
    int li, lane, row0, n_lanes;
    __device__ void put(int t, float v) {
        if (TM) {
            if (li < n_lanes) out[(size_t)t * cols + li] = v;
        } else {
            stage[lane][t & 31] = v;
        }
    }
    __device__ void flush(int tb, int te) {
        if (TM) return;
        __syncwarp();
        const int t = tb + lane;
        for (int r = 0; r < 32; ++r) {
            const int row = row0 + r;
            if (row < n_lanes && t < te) out[(size_t)row * n + t] = stage[r][lane];
        }
        __syncwarp();
    }
};

__device__ __forceinline__ void dm_tr(float ch, float cl, float ph, float pl, float pc, float& tr,
                                      float& pdm, float& mdm) {
    tr = fmaxf(fmaxf(ch - cl, fabsf(ch - pc)), fabsf(cl - pc));
    const float up = ch - ph, down = pl - cl;
    pdm = (up > down && up > 0.f) ? up : 0.f;
    mdm = (down > up && down > 0.f) ? down : 0.f;
}

// adx_scalar on the slices from `first` (adx.rs:299-421): Wilder sums over
// relative indices 1..=p, DX from the smoothed DM/TR, ADX = mean of the first
// p DX values then (adx*(p-1) + dx)/p; NaN prefix [0, first+2p-1).
template <bool TM>
__global__ void __launch_bounds__(kWarps * 32) k_adx(HlcArgs a) {
    __shared__ float stage[kWarps][32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int group = blockIdx.x * kWarps + warp;
    const int li = group * 32 + lane;
    const bool valid = li < a.n_lanes;
    const int p = valid ? (TM ? a.period : a.periods[li]) : 1;
    const int f = valid ? (TM ? a.first_tm[li] : a.first) : a.n;
    typename std::conditional<TM, HlcTm, HlcBatch>::type in;
    if constexpr (TM) in = HlcTm{a.h, a.l, a.c, (size_t)a.cols, (size_t)(valid ? li : 0)};
    else in = HlcBatch{a.h, a.l, a.c};
    Emitter<TM> em{stage[warp], a.out0, (size_t)a.n, (size_t)a.cols, li, lane, group * 32, a.n_lanes};

    const float pf = (float)p, rp = (float)(1.0 / (double)p);
    const float omr = (float)(1.0 - 1.0 / (double)p), pm1 = pf - 1.f;
    float atr = 0.f, pdm = 0.f, mdm = 0.f, ph = 0.f, pl = 0.f, pc = 0.f;
    float dx_sum = 0.f, adx = 0.f;
    int dx_count = 0;
    const bool ok = valid && f < a.n && a.n - f > p;
    for (int tb = 0; tb < a.n; tb += 32) {
        const int te = min(tb + 32, a.n);
        for (int t = tb; t < te; ++t) {
            float v = qnan();
            if (ok && t >= f) {
                const int r = t - f;
                const float ch = in.H(t), cl = in.L(t), cc = in.C(t);
                if (r == 0) {
                    ph = ch; pl = cl; pc = cc;
                } else {
                    float tr, dp, dm;
                    dm_tr(ch, cl, ph, pl, pc, tr, dp, dm);
                    if (r <= p) {
                        atr += tr; pdm += dp; mdm += dm;
                        if (r == p) {
                            dx_sum = hlc::adx_dx(pdm, mdm, atr);
                            dx_count = 1;
                        }
                    } else {
                        atr = atr * omr + tr;
                        pdm = pdm * omr + dp;
                        mdm = mdm * omr + dm;
                        const float dx = hlc::adx_dx(pdm, mdm, atr);
                        if (dx_count < p) {
                            dx_sum += dx;
                            dx_count += 1;
                            if (dx_count == p) { adx = dx_sum * rp; v = adx; }
                        } else {
                            adx = (adx * pm1 + dx) * rp;
                            v = adx;
                        }
                    }
                    ph = ch; pl = cl; pc = cc;
                }
            }
            em.put(t, v);
        }
        em.flush(tb, te);
    }
}

// supertrend_scalar (supertrend.rs:457-550) with the ATR of the slice from
// `first` (atr.rs:329-460) computed inline; outputs trend and changed with a
// NaN prefix [0, first+p-1).
template <bool TM>
__global__ void __launch_bounds__(kWarps * 32) k_supertrend(HlcArgs a) {
    __shared__ float stage0[kWarps][32][33];
    __shared__ float stage1[kWarps][32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int group = blockIdx.x * kWarps + warp;
    const int li = group * 32 + lane;
    const bool valid = li < a.n_lanes;
    const int p = valid ? (TM ? a.period : a.periods[li]) : 1;
    const float fac = valid ? (TM ? a.factor : a.factors[li]) : 1.f;
    const int f = valid ? (TM ? a.first_tm[li] : a.first) : a.n;
    typename std::conditional<TM, HlcTm, HlcBatch>::type in;
    if constexpr (TM) in = HlcTm{a.h, a.l, a.c, (size_t)a.cols, (size_t)(valid ? li : 0)};
    else in = HlcBatch{a.h, a.l, a.c};
    Emitter<TM> e0{stage0[warp], a.out0, (size_t)a.n, (size_t)a.cols, li, lane, group * 32, a.n_lanes};
    Emitter<TM> e1{stage1[warp], a.out1, (size_t)a.n, (size_t)a.cols, li, lane, group * 32, a.n_lanes};

    const float alpha = (float)(1.0 / (double)p);
    const int warm = f + p - 1;
    const bool ok = valid && f < a.n && a.n - f >= p;
    double tr_sum = 0.0;
    float atr = 0.f, pub = 0.f, plb = 0.f, last_close = 0.f, pc = 0.f;
    bool upper = false;
    for (int tb = 0; tb < a.n; tb += 32) {
        const int te = min(tb + 32, a.n);
        for (int t = tb; t < te; ++t) {
            float v0 = qnan(), v1 = qnan();
            if (ok && t >= f) {
                const float hi = in.H(t), lo = in.L(t), cl = in.C(t);
                float tr;
                if (t == f) tr = hi - lo;
                else {
                    tr = hi - lo;
                    const float hc = fabsf(hi - pc);
                    if (hc > tr) tr = hc;
                    const float lc = fabsf(lo - pc);
                    if (lc > tr) tr = lc;
                }
                pc = cl;
                if (t < warm) {
                    tr_sum += (double)tr;
                } else if (t == warm) {
                    tr_sum += (double)tr;
                    atr = (float)(tr_sum / (double)p);
                    const float hl2 = (hi + lo) * 0.5f;
                    pub = hl2 + fac * atr;
                    plb = hl2 - fac * atr;
                    last_close = cl;
                    if (cl <= pub) { v0 = pub; upper = true; }
                    else { v0 = plb; upper = false; }
                    v1 = 0.f;
                } else {
                    atr = fmaf(-alpha, atr, atr) + alpha * tr;
                    const float hl2 = (hi + lo) * 0.5f;
                    const float ub = fmaf(fac, atr, hl2);
                    const float lb = fmaf(-fac, atr, hl2);
                    float cub = ub, clb = lb;
                    if (last_close <= pub) cub = fminf(cub, pub);
                    if (last_close >= plb) clb = fmaxf(clb, plb);
                    if (upper) {
                        if (cl <= cub) { v0 = cub; v1 = 0.f; }
                        else { v0 = clb; v1 = 1.f; upper = false; }
                    } else {
                        if (cl >= clb) { v0 = clb; v1 = 0.f; }
                        else { v0 = cub; v1 = 1.f; upper = true; }
                    }
                    pub = cub; plb = clb; last_close = cl;
                }
            }
            e0.put(t, v0);
            e1.put(t, v1);
        }
        e0.flush(tb, te);
        e1.flush(tb, te);
    }
}

}  // namespace

vta_status launch_adx(const HlcArgs& a, cudaStream_t st) {
    const unsigned blocks = ceil_div(ceil_div(a.n_lanes, 32), kWarps);
    ktimer_begin(st);
    if (a.layout) k_adx<true><<<blocks, kWarps * 32, 0, st>>>(a);
    else k_adx<false><<<blocks, kWarps * 32, 0, st>>>(a);
    ktimer_end(st);
    return check_launch("k_adx");
}

vta_status launch_supertrend(const HlcArgs& a, cudaStream_t st) {
    const unsigned blocks = ceil_div(ceil_div(a.n_lanes, 32), kWarps);
    ktimer_begin(st);
    if (a.layout) k_supertrend<true><<<blocks, kWarps * 32, 0, st>>>(a);
    else k_supertrend<false><<<blocks, kWarps * 32, 0, st>>>(a);
    ktimer_end(st);
    return check_launch("k_supertrend");
}

}  // namespace vta
