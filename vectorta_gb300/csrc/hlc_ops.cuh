// Lane-level sequential state machines of ATR, ADX and SuperTrend with the
// state interface that time-chunked runs use (shared by the many-series plans
// and the chunked single-series sweeps).
//
// Op interface (one series, one parameter set per lane):
//   init(period, param, f)       constants; f = first valid index
//   run_from() -> int            first t whose entering state is a running
//                                state (everything before is seeding)
//   start_exact()                state entering t = f
//   start_warm(in, t0)           guessed running state entering t0 >= run_from()
//   load(w, in, t0)              exact running state entering t0 from 8 words
//   save(w)                      running state as 8 words
//   step(in, t, o1) -> o0        process t (any phase), outputs for t
//   stepv(t, h, l, c, o1) -> o0  the same with the inputs of t given
//   step_run(h, l, c, o1) -> o0  stepv for t >= run_from() without phase checks
//   (ADX also: wide_ok(h, l, c) and step_run<true> for tiles of up to 32 steps
//   whose sums stay normal, with DX by the hardware reciprocal)
// `In` provides H(t), L(t), C(t).  The arithmetic of each op is that of the
// sequential kernels in k_hlc.cu, so a run that starts at the series start is
// bit-identical to them.
#pragma once

#include "vta_internal.h"

namespace vta {
namespace hlc {

__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

// True range with the crate's NaN-skipping comparisons (atr.rs:352-366).
__device__ __forceinline__ float true_range(float hi, float lo, float pc) {
    float tr = hi - lo;
    const float hc = fabsf(hi - pc);
    if (hc > tr) tr = hc;
    const float lc = fabsf(lo - pc);
    if (lc > tr) tr = lc;
    return tr;
}

// DX from the smoothed DM and TR sums.  The crate forms +DI = 100 pdm / atr and
// -DI = 100 mdm / atr, then DX = 100 |+DI - -DI| / (+DI + -DI); the common
// factor 100 / atr cancels, leaving one division.  atr == 0 gives 0 (both DI
// are 0) and a NaN atr gives NaN, as in the crate.  The ratio |a - b| / (a + b)
// lies in [0, 1] and is taken with the fast reciprocal-multiply divide (2 ulp;
// the ADX sweeps and plans are issue-bound and the IEEE divide was a third of
// a step); every ADX kernel shares this function, so the chunked and the
// sequential kernels stay bit-identical.
// 1 / x by the hardware approximation (relative error within about 2^-23;
// subnormal x is read as zero), one instruction
__device__ __forceinline__ float rcp_approx_ftz(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Whether up to 32 running ADX steps from this state keep atr and
// pdm + mdm normal and nonzero, given the inputs of those steps and of the
// bar before them (x*, p*): the sums shrink by at most omr^32 >= 2^-32 and
// grow by at most 32 x 2^100 when every price is within 2^98 in magnitude,
// so sums in [2^-60, 2^100] at the start stay within [2^-92, 2^106].  On such
// steps DX = |pdm - mdm| / (pdm + mdm) 100 needs none of adx_dx's guards
// (adx_dx_wide).  NaN prices or sums fail the test.
__device__ __forceinline__ bool adx_wide_ok(float atr, float pdm, float mdm, float xh, float xl, float xc,
                                            float ph, float pl, float pc) {
    const float s = pdm + mdm;
    const bool in_range = fabsf(xh) <= 0x1p98f && fabsf(xl) <= 0x1p98f && fabsf(xc) <= 0x1p98f &&
                          fabsf(ph) <= 0x1p98f && fabsf(pl) <= 0x1p98f && fabsf(pc) <= 0x1p98f;
    return in_range && atr >= 0x1p-60f && atr <= 0x1p100f && s >= 0x1p-60f && s <= 0x1p100f;
}
__device__ __forceinline__ float adx_dx_wide(float pdm, float mdm) {
    return fabsf(pdm - mdm) * rcp_approx_ftz(pdm + mdm) * 100.f;
}

__device__ __forceinline__ float adx_dx(float pdm, float mdm, float atr) {
    if (atr == 0.f) return 0.f;
    const float s = pdm + mdm;
    const float d = s != 0.f ? __fdividef(fabsf(pdm - mdm), s) * 100.f : 0.f;
    return atr == atr ? d : qnan();
}

// ATR: atr_compute_into_scalar (atr.rs:329-460); TR(f) = h - l, seed = mean
// of the first p TRs at s = f + p - 1, then rma = fma(-a, rma, rma) + a * tr.
struct PAtr {
    static constexpr bool kTwo = false;
    int p, f;
    float alpha, rma, pc;
    double tr_sum;
    __device__ void init(int period, float, int first) {
        p = period;
        f = first;
        alpha = (float)(1.0 / (double)p);
    }
    __device__ int run_from() const { return f + p; }
    __device__ void start_exact() { tr_sum = 0.0; rma = 0.f; pc = 0.f; }
    template <class In> __device__ void start_warm(const In& in, int t0) {
        pc = in.C(t0 - 1);
        rma = in.H(t0 - 1) - in.L(t0 - 1);
    }
    template <class In> __device__ void load(const float* w, const In& in, int t0) {
        rma = w[0];
        pc = in.C(t0 - 1);
    }
    __device__ void save(float* w) const {
        w[0] = rma;
        w[1] = w[2] = w[3] = w[4] = w[5] = w[6] = w[7] = 0.f;
    }
    template <class In> __device__ float step(const In& in, int t, float& o1) {
        if (t < f) return qnan();
        return stepv(t, in.H(t), in.L(t), in.C(t), o1);
    }
    __device__ float stepv(int t, float hi, float lo, float cl, float&) {
        if (t < f) return qnan();
        const float tr = (t == f) ? hi - lo : true_range(hi, lo, pc);
        pc = cl;
        const int s = f + p - 1;
        if (t < s) {
            tr_sum += (double)tr;
            return qnan();
        }
        if (t == s) {
            tr_sum += (double)tr;
            rma = (float)(tr_sum / (double)p);
            return rma;
        }
        rma = fmaf(-alpha, rma, rma) + alpha * tr;
        return rma;
    }
    // stepv for t >= run_from(): the running update alone
    template <bool WIDE = false>  // (no division: one form)
    __device__ __forceinline__ float step_run(float hi, float lo, float cl, float&) {
        const float tr = true_range(hi, lo, pc);
        pc = cl;
        rma = fmaf(-alpha, rma, rma) + alpha * tr;
        return rma;
    }
};

// ADX: adx_scalar on the slice from f (adx.rs:299-421): Wilder sums over
// relative indices 1..=p, DX from the smoothed DM/TR, ADX = mean of the
// first p DX, then (adx * (p - 1) + dx) / p; first output at f + 2p - 1.
// The arithmetic is the sequential time-major kernel's (k_adx).
struct PAdx {
    static constexpr bool kTwo = false;
    int p, f, dx_count;
    float rp, omr, pm1;
    float atr, pdm, mdm, dx_sum, adx, ph, pl, pc;
    __device__ void init(int period, float, int first) {
        p = period;
        f = first;
        rp = (float)(1.0 / (double)p);
        omr = (float)(1.0 - 1.0 / (double)p);
        pm1 = (float)p - 1.f;
    }
    __device__ int run_from() const { return f + 2 * p; }
    __device__ void start_exact() {
        atr = pdm = mdm = dx_sum = adx = ph = pl = pc = 0.f;
        dx_count = 0;
    }
    template <class In> __device__ void prev_inputs(const In& in, int t0) {
        ph = in.H(t0 - 1);
        pl = in.L(t0 - 1);
        pc = in.C(t0 - 1);
    }
    template <class In> __device__ void start_warm(const In& in, int t0) {
        prev_inputs(in, t0);
        atr = (float)p * (ph - pl);
        pdm = mdm = 0.f;
        adx = 0.f;
        dx_count = p;
    }
    template <class In> __device__ void load(const float* w, const In& in, int t0) {
        atr = w[0]; pdm = w[1]; mdm = w[2]; adx = w[3];
        dx_count = p;
        prev_inputs(in, t0);
    }
    __device__ void save(float* w) const {
        w[0] = atr; w[1] = pdm; w[2] = mdm; w[3] = adx;
        w[4] = w[5] = w[6] = w[7] = 0.f;
    }
    __device__ float dx_now() const {
        return adx_dx(pdm, mdm, atr);
    }
    template <class In> __device__ float step(const In& in, int t, float& o1) {
        if (t < f) return qnan();
        return stepv(t, in.H(t), in.L(t), in.C(t), o1);
    }
    __device__ float stepv(int t, float ch, float cl, float cc, float&) {
        if (t < f) return qnan();
        const int r = t - f;
        float v = qnan();
        if (r > 0) {
            const float tr = fmaxf(fmaxf(ch - cl, fabsf(ch - pc)), fabsf(cl - pc));
            const float up = ch - ph, down = pl - cl;
            const float dp = (up > down && up > 0.f) ? up : 0.f;
            const float dm = (down > up && down > 0.f) ? down : 0.f;
            if (r <= p) {
                atr += tr; pdm += dp; mdm += dm;
                if (r == p) {
                    dx_sum = dx_now();
                    dx_count = 1;
                }
            } else {
                atr = atr * omr + tr;
                pdm = pdm * omr + dp;
                mdm = mdm * omr + dm;
                const float dx = dx_now();
                if (dx_count < p) {
                    dx_sum += dx;
                    dx_count += 1;
                    if (dx_count == p) { adx = dx_sum * rp; v = adx; }
                } else {
                    adx = (adx * pm1 + dx) * rp;
                    v = adx;
                }
            }
        }
        ph = ch; pl = cl; pc = cc;
        return v;
    }
    // stepv for t >= run_from(): the running update alone; WIDE: the steps
    // of a tile for which wide_ok held on every lane at its start
    template <bool WIDE = false>
    __device__ __forceinline__ float step_run(float ch, float cl, float cc, float&) {
        const float tr = fmaxf(fmaxf(ch - cl, fabsf(ch - pc)), fabsf(cl - pc));
        const float up = ch - ph, down = pl - cl;
        const float dp = (up > down && up > 0.f) ? up : 0.f;
        const float dm = (down > up && down > 0.f) ? down : 0.f;
        atr = atr * omr + tr;
        pdm = pdm * omr + dp;
        mdm = mdm * omr + dm;
        adx = (adx * pm1 + (WIDE ? adx_dx_wide(pdm, mdm) : adx_dx(pdm, mdm, atr))) * rp;
        ph = ch; pl = cl; pc = cc;
        return adx;
    }
    static constexpr bool kWide = true;
    __device__ bool wide_ok(float xh, float xl, float xc) const {
        return adx_wide_ok(atr, pdm, mdm, xh, xl, xc, ph, pl, pc);
    }
};

// SuperTrend: supertrend_scalar (supertrend.rs:457-550) with the ATR of the
// slice from f computed inline; outputs trend and changed, first at f + p - 1.
// The arithmetic is the sequential time-major kernel's (k_supertrend).
struct PSuperTrend {
    static constexpr bool kTwo = true;
    int p, f;
    float alpha, fac, atr, pub, plb, last_close, pc;
    bool upper;
    double tr_sum;
    __device__ void init(int period, float factor, int first) {
        p = period;
        f = first;
        alpha = (float)(1.0 / (double)p);
        fac = factor;
    }
    __device__ int run_from() const { return f + p; }
    __device__ void start_exact() {
        tr_sum = 0.0;
        atr = pub = plb = last_close = pc = 0.f;
        upper = false;
    }
    template <class In> __device__ void start_warm(const In& in, int t0) {
        const float hi = in.H(t0 - 1), lo = in.L(t0 - 1), cl = in.C(t0 - 1);
        atr = hi - lo;
        const float hl2 = (hi + lo) * 0.5f;
        pub = hl2 + fac * atr;
        plb = hl2 - fac * atr;
        last_close = pc = cl;
        upper = cl <= pub;
    }
    template <class In> __device__ void load(const float* w, const In& in, int t0) {
        atr = w[0]; pub = w[1]; plb = w[2];
        upper = w[3] != 0.f;
        last_close = pc = in.C(t0 - 1);
    }
    __device__ void save(float* w) const {
        w[0] = atr; w[1] = pub; w[2] = plb; w[3] = upper ? 1.f : 0.f;
        w[4] = w[5] = w[6] = w[7] = 0.f;
    }
    template <class In> __device__ float step(const In& in, int t, float& v1) {
        v1 = qnan();
        if (t < f) return qnan();
        return stepv(t, in.H(t), in.L(t), in.C(t), v1);
    }
    __device__ float stepv(int t, float hi, float lo, float cl, float& v1) {
        v1 = qnan();
        if (t < f) return qnan();
        float tr = hi - lo;
        if (t != f) {
            const float hc = fabsf(hi - pc);
            if (hc > tr) tr = hc;
            const float lc = fabsf(lo - pc);
            if (lc > tr) tr = lc;
        }
        pc = cl;
        const int warm = f + p - 1;
        float v0 = qnan();
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
        return v0;
    }
    // stepv for t >= run_from(): the running update alone
    template <bool WIDE = false>  // (no division: one form)
    __device__ __forceinline__ float step_run(float hi, float lo, float cl, float& v1) {
        float tr = hi - lo;
        const float hc = fabsf(hi - pc);
        if (hc > tr) tr = hc;
        const float lc = fabsf(lo - pc);
        if (lc > tr) tr = lc;
        pc = cl;
        atr = fmaf(-alpha, atr, atr) + alpha * tr;
        const float hl2 = (hi + lo) * 0.5f;
        float cub = fmaf(fac, atr, hl2), clb = fmaf(-fac, atr, hl2);
        if (last_close <= pub) cub = fminf(cub, pub);
        if (last_close >= plb) clb = fmaxf(clb, plb);
        float v0;
        if (upper) {
            if (cl <= cub) { v0 = cub; v1 = 0.f; }
            else { v0 = clb; v1 = 1.f; upper = false; }
        } else {
            if (cl >= clb) { v0 = clb; v1 = 0.f; }
            else { v0 = cub; v1 = 1.f; upper = true; }
        }
        pub = cub; plb = clb; last_close = cl;
        return v0;
    }
};


}  // namespace hlc
}  // namespace vta
