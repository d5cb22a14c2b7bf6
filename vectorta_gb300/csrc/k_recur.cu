// Chunked linear-recurrence scans: EMA, DEMA, TEMA, RSI, Wilders, ATR.
//
// Each indicator is a linear time-invariant recurrence once seeded, so the
// time axis is cut into chunks processed in parallel:
//   pass A (k_recur<.., PASS_AGG>):  per (lane, chunk) run the recurrence from
//       a zero state (or from the exact seed inside the seed chunk) and keep
//       the chunk-end state plus the number of applied steps;
//   pass B (k_recur_carry):          per lane, compose the chunk transforms
//       (closed-form powers of the transition matrix) in double-single
//       arithmetic -> carry-in per chunk;
//   pass C (k_recur<.., PASS_EMIT>): per (lane, chunk) re-run from the carry
//       and write the outputs.
// A "lane" is one parameter combo of a single-series sweep (batch layout:
// every lane reads the same x[t], outputs are staged through shared memory so
// each store instruction writes one contiguous 256-byte row segment) or one
// series of a time-major matrix (coalesced loads and stores directly).
// The warm-up rules (seed index, NaN prefix, running-mean outputs) follow the
// crate's scalar paths cited on each op.
#include <climits>

#include "vta_internal.h"

namespace vta {
namespace {

constexpr int kWarps = 4;  // warps per block
__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

// Compensated running sum (float value + float error term, Neumaier): the
// warm-up accumulators of the crate are f64, and GB300's FP64 rate is a
// small fraction of FP32, so the per-step sums are kept in float pairs and
// turned into f64 only once, at the seed.  Sums of up to a few thousand
// terms stay within ~1e-14 relative of the f64 ones.
struct Acc {
    float hi, lo;
    __device__ void zero() { hi = 0.f; lo = 0.f; }
    // error terms of non-finite sums are dropped so that inf / NaN propagate
    // through hi exactly as through an f64 sum
    __device__ void add(float v) {
        const float sum = hi + v;
        const float bb = sum - hi;
        const float e = (hi - (sum - bb)) + (v - bb);
        lo += isfinite(e) ? e : 0.f;
        hi = sum;
    }
    // adds the exact difference a - b
    __device__ void add_diff(float a, float b) {
        const float d = a - b;
        const float bb = d - a;
        const float e = (a - (d - bb)) - (b + bb);
        add(d);
        lo += isfinite(e) ? e : 0.f;
    }
    __device__ float f() const { return hi + lo; }
    __device__ double d() const { return (double)hi + (double)lo; }
};

// ------------------------------------------------------------ inputs -------
struct InBatch {
    const float *x, *h, *l, *c;
    __device__ float X(int t) const { return __ldg(x + t); }
    __device__ float H(int t) const { return __ldg(h + t); }
    __device__ float L(int t) const { return __ldg(l + t); }
    __device__ float C(int t) const { return __ldg(c + t); }
};
struct InTm {
    const float *x, *h, *l, *c;
    size_t cols, s;
    __device__ float X(int t) const { return __ldg(x + (size_t)t * cols + s); }
    __device__ float H(int t) const { return __ldg(h + (size_t)t * cols + s); }
    __device__ float L(int t) const { return __ldg(l + (size_t)t * cols + s); }
    __device__ float C(int t) const { return __ldg(c + (size_t)t * cols + s); }
};

// One 32-step tile of a single shared series held in registers: lane l holds
// x[tb + l]; X(t) is a warp shuffle (t - 1 < tb reads the value before the
// tile).  Used by the batch fast path so each step costs no memory access.
struct InTile {
    float xv, hv, lv, cv;  // this lane's element of the tile
    float xb, cb;          // x[tb-1], c[tb-1]
    int tb;
    float4* xs;  // this warp's 2 x 32-float input scratch in shared memory
    __device__ float X(int t) const {
        const int j = t - tb;
        const float v = __shfl_sync(0xffffffffu, xv, j & 31);
        return j >= 0 ? v : xb;
    }
    __device__ float H(int t) const { return __shfl_sync(0xffffffffu, hv, (t - tb) & 31); }
    __device__ float L(int t) const { return __shfl_sync(0xffffffffu, lv, (t - tb) & 31); }
    __device__ float C(int t) const {
        const int j = t - tb;
        const float v = __shfl_sync(0xffffffffu, cv, j & 31);
        return j >= 0 ? v : cb;
    }
};

// The values of one step t of a single shared series (and of t - 1), for the
// general path: X / C at t or t - 1, H / L at t.
struct InStep {
    int t;
    float x0, x1;  // x[t], x[t-1]  (close for the high/low/close ops)
    float h0, l0;  // h[t], l[t]
    __device__ float X(int u) const { return u == t ? x0 : x1; }
    __device__ float C(int u) const { return u == t ? x0 : x1; }
    __device__ float H(int) const { return h0; }
    __device__ float L(int) const { return l0; }
};

// Double-single numbers for the carry scan and the closed-form chunk
// transitions: value = hi + lo with |lo| <= ulp(hi) / 2, about 2^-44
// relative after a few operations.  GB300 runs FP32 at many times its FP64
// rate (one FP64 warp instruction holds the SM's FP64 pipe for many cycles),
// so the scan works with FP32 error-free transformations (exact products by
// FMA, TwoSum) instead of f64.
struct D2 {
    float hi, lo;
};
__device__ __forceinline__ D2 d2_norm(float s, float e) {
    const float hi = s + e;
    return {hi, e - (hi - s)};
}
__device__ __forceinline__ D2 d2_mul(D2 a, D2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return d2_norm(p, e);
}
__device__ __forceinline__ D2 d2_add(D2 a, D2 b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    const float e = ((a.hi - (s - bb)) + (b.hi - bb)) + (a.lo + b.lo);
    return d2_norm(s, e);
}
// a * b + c
__device__ __forceinline__ D2 d2_fma(D2 a, D2 b, D2 c) { return d2_add(d2_mul(a, b), c); }
__device__ __forceinline__ D2 d2_neg(D2 a) { return {-a.hi, -a.lo}; }
// num / den for small positive integers, to double-single accuracy: the
// FP32 quotient plus its exact remainder (FMA) divided again
__device__ __forceinline__ D2 d2_ratio(int num, int den) {
    const float fn = (float)num, fd = (float)den;
    const float q = fn / fd;
    const float r = fmaf(-q, fd, fn);
    return d2_norm(q, r / fd);
}
__device__ __forceinline__ D2 d2_from_ll(long long n) {
    const float hi = (float)n;
    return {hi, (float)(n - (long long)hi)};
}
// b^n for a whole step count n >= 0 by repeated squaring
__device__ __forceinline__ D2 d2_pow(D2 b, long long n) {
    D2 r = {1.f, 0.f};
    while (n > 0) {
        if (n & 1) r = d2_mul(r, b);
        b = d2_mul(b, b);
        n >>= 1;
    }
    return r;
}
__device__ __forceinline__ D2 d2_shfl_up(D2 v, int d) {
    return {__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d)};
}

// ------------------------------------------------------------ ops ----------
// Common op interface:
//   init(p, f)            lane constants; sets f (first valid), s (seed index),
//                         warm (first non-NaN output index)
//   accum(in, t)          warm-up accumulation for t in [f, s]
//   seed()                running state from the accumulators (at t == s)
//   step(in, t) -> int    running update for t > s; returns 1 if applied
//   value(in, t)          output for t >= s
//   warm_value(t)         output for t in [f, s)
//   zero() / get(i) / set(i, v)   running state access (NS components)
//   propagate(S, n, p)    S <- M^n S in f64 (static)

// EMA: ema.rs:430-469 / 858-893.  Warm-up outputs are the running mean of the
// finite values of [f, t]; NaN prefix is [0, f); non-finite x is skipped.
struct OpEma {
    static constexpr bool kHlc = false;
    static constexpr int NS = 1;
    float alpha, beta, y;
    int f, s, warm;
    Acc wsum;
    int wcnt;
    __device__ void init(int p, int first) {
        double a = 2.0 / ((double)p + 1.0);
        alpha = (float)a;
        beta = (float)(1.0 - a);
        f = first; s = first + p - 1; warm = first;
        wsum.zero(); wcnt = 0;
    }
    template <class In> __device__ void accum(const In& in, int t) {
        float v = in.X(t);
        if (t == f || isfinite(v)) { wsum.add(v); wcnt += 1; }
    }
    __device__ float cur_mean() const { return wsum.f() / (float)wcnt; }
    __device__ void seed() { y = cur_mean(); }
    // y <- y + alpha (x - y): the fixed point is x itself whatever the f32
    // rounding of alpha.  The crate's form beta y + alpha x, with alpha and
    // beta = 1 - alpha rounded to f32 separately, has the steady-state gain
    // alpha / (1 - beta) = 1 + O(2^-25 / alpha): a bias of 1.5e-5 at p = 1000.
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        if (isfinite(v)) { y = fmaf(alpha, v - y, y); return 1; }
        return 0;
    }
    template <class In> __device__ float value(const In&, int) const { return y; }
    __device__ float warm_value(int) const { return cur_mean(); }
    __device__ void zero() { y = 0.f; }
    __device__ float get(int) const { return y; }
    __device__ void set(int, float v) { y = v; }
    // running step + output without phase checks; returns applied-step flag
    // FIN: every input of the step is known finite (no skip logic)
    template <bool FIN = false, class In> __device__ float fast(const In& in, int t, int& applied) {
        const float v = in.X(t);
        if (FIN) {
            y = fmaf(alpha, v - y, y);
            ++applied;
            return y;
        }
        const bool ok = isfinite(v);
        y = ok ? fmaf(alpha, v - y, y) : y;
        applied += ok;
        return y;
    }
    // closed-form transition of n steps (double-single): a = 2 / (p + 1),
    // an = (1 - a)^n
    static __device__ void coef(int p, D2& a, D2& b) {
        a = d2_ratio(2, p + 1);
        b = d2_add({1.f, 0.f}, d2_neg(a));
    }
    static __device__ void propagate(D2* S, D2, D2, D2 an, int) { S[0] = d2_mul(S[0], an); }
};

// DEMA: dema.rs:291-354 (x86 mul_add form).  Seed x[f] at f; NaN prefix
// [0, f+p-1); out = 2*e1 - e2.
struct OpDema {
    static constexpr bool kHlc = false;
    static constexpr int NS = 2;
    static constexpr int kShape = 1;
    float alpha, a, e1, e2, xf;
    int f, s, warm;
    __device__ void init(int p, int first) {
        double al = 2.0 / ((double)p + 1.0);
        alpha = (float)al;
        a = (float)(1.0 - al);
        f = first; s = first; warm = first + p - 1;
    }
    template <class In> __device__ void accum(const In& in, int t) { xf = in.X(t); }
    __device__ void seed() { e1 = xf; e2 = xf; }
    // gain-exact form of e <- a e + alpha x (see OpEma::step)
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        e1 = fmaf(alpha, v - e1, e1);
        e2 = fmaf(alpha, e1 - e2, e2);
        return 1;
    }
    template <class In> __device__ float value(const In&, int t) const {
        return t < warm ? qnan() : fmaf(e1, 2.f, -e2);
    }
    __device__ float warm_value(int) const { return qnan(); }
    __device__ void zero() { e1 = 0.f; e2 = 0.f; }
    __device__ float get(int i) const { return i == 0 ? e1 : e2; }
    __device__ void set(int i, float v) { if (i == 0) e1 = v; else e2 = v; }
    template <bool FIN = false, class In> __device__ float fast(const In& in, int t, int& applied) {
        const float v = in.X(t);
        e1 = fmaf(alpha, v - e1, e1);
        e2 = fmaf(alpha, e1 - e2, e2);
        ++applied;
        return fmaf(e1, 2.f, -e2);
    }
    static __device__ void coef(int p, D2& a, D2& b) { OpEma::coef(p, a, b); }
    static __device__ void propagate(D2* S, D2 n, D2 al, D2 an, int) {
        const D2 s1 = S[0];
        S[0] = d2_mul(an, s1);
        S[1] = d2_mul(an, d2_fma(d2_mul(n, al), s1, S[1]));
    }
};

// TEMA: tema.rs:228-298.  Three EMAs started at f, f+(p-1), f+2(p-1) exactly
// as the crate staggers them; running from s = f+2(p-1); NaN prefix
// [0, f+3(p-1)); out = 3*e1 - 3*e2 + e3; p == 1 copies x.
struct OpTema {
    static constexpr bool kHlc = false;
    static constexpr int NS = 3;
    static constexpr int kShape = 1;
    float per, per1, e1, e2, e3;
    int f, s, warm, start2, p1;
    __device__ void init(int p, int first) {
        double pd = 2.0 / ((double)p + 1.0);
        per = (float)pd;
        per1 = (float)(1.0 - pd);
        p1 = p - 1;
        f = first; start2 = first + p1; s = first + 2 * p1; warm = first + 3 * p1;
        e1 = e2 = e3 = 0.f;
    }
    template <class In> __device__ void accum(const In& in, int t) {
        float v = in.X(t);
        if (p1 == 0) { e1 = v; return; }
        if (t == f) e1 = v;  // ema1 = data[first]; the loop then re-applies it
        // gain-exact form of e <- per1 e + per x (see OpEma::step)
        e1 = fmaf(per, v - e1, e1);
        if (t == start2) { e2 = e1; e2 = fmaf(per, e1 - e2, e2); }
        else if (t > start2) e2 = fmaf(per, e1 - e2, e2);
        if (t == s) { e3 = e2; e3 = fmaf(per, e2 - e3, e3); }
    }
    __device__ void seed() {}
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        if (p1 == 0) { e1 = v; return 1; }
        e1 = fmaf(per, v - e1, e1);
        e2 = fmaf(per, e1 - e2, e2);
        e3 = fmaf(per, e2 - e3, e3);
        return 1;
    }
    template <class In> __device__ float value(const In& in, int t) const {
        if (p1 == 0) return e1;
        return t < warm ? qnan() : 3.f * e1 - 3.f * e2 + e3;
    }
    __device__ float warm_value(int) const { return qnan(); }
    __device__ void zero() { e1 = e2 = e3 = 0.f; }
    template <bool FIN = false, class In> __device__ float fast(const In& in, int t, int& applied) {
        const float v = in.X(t);
        ++applied;
        if (p1 == 0) { e1 = v; return v; }
        e1 = fmaf(per, v - e1, e1);
        e2 = fmaf(per, e1 - e2, e2);
        e3 = fmaf(per, e2 - e3, e3);
        return 3.f * e1 - 3.f * e2 + e3;
    }
    __device__ float get(int i) const { return i == 0 ? e1 : (i == 1 ? e2 : e3); }
    __device__ void set(int i, float v) { if (i == 0) e1 = v; else if (i == 1) e2 = v; else e3 = v; }
    // One general-path step for any t >= f: the arithmetic of accum / step
    // with the phase tests (t == f, start2, s) as selects instead of branches,
    // so the lanes of a warp in different warm-up phases do not diverge.
    static constexpr bool kUni = true;
    template <class In> __device__ float uni(const In& in, int t, int& steps) {
        const float v = in.X(t);
        steps += t > s;
        if (p1 == 0) { e1 = v; return v; }
        const float a1 = t == f ? v : e1;
        e1 = fmaf(per, v - a1, a1);
        const float a2 = t == start2 ? e1 : e2;
        const float n2 = fmaf(per, e1 - a2, a2);
        e2 = t >= start2 ? n2 : e2;
        const float a3 = t == s ? e2 : e3;
        const float n3 = fmaf(per, e2 - a3, a3);
        e3 = t >= s ? n3 : e3;
        return t < warm ? qnan() : 3.f * e1 - 3.f * e2 + e3;
    }
    static __device__ void coef(int p, D2& a, D2& b) { OpEma::coef(p, a, b); }
    static __device__ void propagate(D2* S, D2 n, D2 al, D2 an, int p) {
        if (p == 1) {  // p==1 carries nothing (out = x)
            S[0] = {0.f, 0.f};
            return;
        }
        const D2 s1 = S[0], s2 = S[1], s3 = S[2];
        const D2 nal = d2_mul(n, al);
        // n a^2 + n (n - 1) / 2 a^2 = n (n + 1) / 2 a^2
        const D2 c = d2_mul(d2_mul(d2_mul(n, d2_add(n, {1.f, 0.f})), {0.5f, 0.f}), d2_mul(al, al));
        S[0] = d2_mul(an, s1);
        S[1] = d2_mul(an, d2_fma(nal, s1, s2));
        S[2] = d2_mul(an, d2_fma(c, s1, d2_fma(nal, s2, s3)));
    }
};

// RSI: batch rows follow rsi_batch_inner (rsi.rs:568-697: non-finite deltas
// become NaN gains/losses and poison the row); time-major series follow the
// single-series rsi_compute_into_scalar (rsi.rs:327-414: a NaN delta poisons
// only inside the warm-up, later ones count as 0).  NaN prefix [0, f+p).
template <bool kBatchSem>
struct OpRsi {
    static constexpr bool kHlc = false;
    static constexpr int NS = 2;
    static constexpr int kShape = 2;
    float inv_p, beta, ag, al, xprev, pf;
    float sN, sD;  // the emit tiles' scaled state while sc (run_tile below)
    int f, s, warm;
    Acc sg, sl;
    bool wnan, sc;
    __device__ void init(int p, int first) {
        double ip = 1.0 / (double)p;
        inv_p = (float)ip;
        pf = (float)p;
        beta = (float)(1.0 - ip);
        f = first; s = first + p; warm = s;
        sg.zero(); sl.zero(); wnan = false; sc = false;
    }
    template <class In> __device__ void accum(const In& in, int t) {
        float v = in.X(t);
        if (t > f && !wnan) {
            // the f64 difference of two floats is exact; its sign is v vs xprev
            if (!(isfinite(v) && isfinite(xprev))) wnan = true;
            else if (v > xprev) sg.add_diff(v, xprev);
            else if (v < xprev) sl.add_diff(xprev, v);
        }
        xprev = v;
    }
    __device__ void seed() {
        if (wnan) { ag = qnan(); al = qnan(); }
        else { ag = (float)(sg.d() * (double)inv_p); al = (float)(sl.d() * (double)inv_p); }
        // the crate multiplies by inv_p = 1/p in f64
    }
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        float xp = (t == 0) ? v : in.X(t - 1);
        float d = v - xp;
        float g, lo;
        if (kBatchSem && !isfinite(d)) { g = qnan(); lo = qnan(); }
        else { g = d > 0.f ? d : 0.f; lo = d < 0.f ? -d : 0.f; }
        ag = fmaf(ag, beta, inv_p * g);
        al = fmaf(al, beta, inv_p * lo);
        return 1;
    }
    template <class In> __device__ float value(const In&, int) const {
        float den = ag + al;
        return den == 0.f ? 50.f : __fdividef(100.f * ag, den);
    }
    __device__ float warm_value(int) const { return qnan(); }
    __device__ void zero() { ag = 0.f; al = 0.f; }
    template <bool FIN = false, class In> __device__ float fast(const In& in, int t, int& applied) {
        const float v = in.X(t);
        const float d = v - in.X(t - 1);
        float g = d > 0.f ? d : 0.f, lo = d < 0.f ? -d : 0.f;
        if (!FIN && kBatchSem && !isfinite(d)) { g = qnan(); lo = qnan(); }
        ag = fmaf(ag, beta, inv_p * g);
        al = fmaf(al, beta, inv_p * lo);
        ++applied;
        const float den = ag + al;
        return den == 0.f ? 50.f : __fdividef(100.f * ag, den);
    }
    __device__ float get(int i) const { return i == 0 ? ag : al; }
    __device__ void set(int i, float v) { if (i == 0) ag = v; else al = v; }
    // a = 1 / p, an = (1 - 1/p)^n
    static __device__ void coef(int p, D2& a, D2& b) {
        a = d2_ratio(1, p);
        b = d2_add({1.f, 0.f}, d2_neg(a));
    }
    static __device__ void propagate(D2* S, D2, D2, D2 an, int) {
        S[0] = d2_mul(S[0], an);
        S[1] = d2_mul(S[1], an);
    }
};

// Wilders: wilders.rs:262-322.  Seed = mean of x[f..f+p); y = (x-y)*a + y;
// NaN prefix [0, f+p-1); p == 1 copies x.
struct OpWilders {
    static constexpr bool kHlc = false;
    static constexpr int NS = 1;
    float alpha, y;
    int f, s, warm, p;
    Acc wsum;
    __device__ void init(int p_, int first) {
        p = p_;
        alpha = (float)(1.0 / (double)p);
        f = first; s = first + p - 1; warm = s;
        wsum.zero();
    }
    template <class In> __device__ void accum(const In& in, int t) { wsum.add(in.X(t)); }
    __device__ void seed() { y = (float)(wsum.d() * (1.0 / (double)p)); }
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        y = (p == 1) ? v : fmaf(v - y, alpha, y);
        return 1;
    }
    template <class In> __device__ float value(const In&, int) const { return y; }
    __device__ float warm_value(int) const { return qnan(); }
    __device__ void zero() { y = 0.f; }
    __device__ float get(int) const { return y; }
    __device__ void set(int, float v) { y = v; }
    template <bool FIN = false, class In> __device__ float fast(const In& in, int t, int& applied) {
        const float v = in.X(t);
        y = (p == 1) ? v : fmaf(v - y, alpha, y);
        ++applied;
        return y;
    }
    static __device__ void coef(int p, D2& a, D2& b) { OpRsi<true>::coef(p, a, b); }
    static __device__ void propagate(D2* S, D2, D2, D2 an, int p) {
        S[0] = (p == 1) ? D2{0.f, 0.f} : d2_mul(S[0], an);
    }
};

// True range as the crate computes it (atr.rs:352-366): comparisons skip NaN.
__device__ __forceinline__ float true_range(float hi, float lo, float pc) {
    float tr = hi - lo;
    float hc = fabsf(hi - pc);
    if (hc > tr) tr = hc;
    float lc = fabsf(lo - pc);
    if (lc > tr) tr = lc;
    return tr;
}

// ATR: atr.rs:329-460.  TR(f) = h-l; seed = mean TR over [f, f+L);
// rma = (-a).mul_add(rma, rma) + a*tr; NaN prefix [0, f+L-1).
struct OpAtr {
    static constexpr int NS = 1;
    static constexpr bool kHlc = true;
    float alpha, y;
    int f, s, warm, p;
    Acc wsum;
    __device__ void init(int p_, int first) {
        p = p_;
        alpha = (float)(1.0 / (double)p);
        f = first; s = first + p - 1; warm = s;
        wsum.zero();
    }
    template <class In> __device__ void accum(const In& in, int t) {
        float hi = in.H(t), lo = in.L(t);
        if (t == f) wsum.add_diff(hi, lo);
        else wsum.add(true_range(hi, lo, in.C(t - 1)));
    }
    __device__ void seed() { y = (float)(wsum.d() / (double)p); }
    template <class In> __device__ int step(const In& in, int t) {
        float tr = true_range(in.H(t), in.L(t), in.C(t - 1));
        y = fmaf(-alpha, y, y) + alpha * tr;
        return 1;
    }
    template <class In> __device__ float value(const In&, int) const { return y; }
    __device__ float warm_value(int) const { return qnan(); }
    __device__ void zero() { y = 0.f; }
    __device__ float get(int) const { return y; }
    __device__ void set(int, float v) { y = v; }
    template <bool FIN = false, class In> __device__ float fast(const In& in, int t, int& applied) {
        const float tr = true_range(in.H(t), in.L(t), in.C(t - 1));
        y = fmaf(-alpha, y, y) + alpha * tr;
        ++applied;
        return y;
    }
    static __device__ void coef(int p, D2& a, D2& b) { OpRsi<true>::coef(p, a, b); }
    static __device__ void propagate(D2* S, D2, D2, D2 an, int) { S[0] = d2_mul(S[0], an); }
};

// ------------------------------------------------------------ kernels ------
enum { PASS_AGG = 0, PASS_EMIT = 1 };
constexpr float kBeforeSeed = -2.f, kAbsolute = -1.f;

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Staging row write at column j ^ sw (sw = 0 or 1) with no per-step address
// arithmetic once j is a compile-time constant: even columns go to row + sw,
// odd ones to row - sw.
__device__ __forceinline__ void stage_put(float* row, int sw, int j, float v) {
    (j & 1 ? row - sw : row + sw)[j] = v;
}

// One warp = 32 lanes x one time chunk.  Tiles of 32 steps where every lane
// of the warp is past its seed and warm-up take the fast path (no phase
// checks: 2-6 FP ops per step); the few tiles around warm-up take the general
// per-step state machine.
// The 32 steps of one register tile, fully unrolled so every shuffle source
// lane is a constant; EMIT stages the outputs in this lane's row.
template <bool FIN, int PASS, class Op>
__device__ __forceinline__ void run_tile(Op& op, const InTile& ti, float* row, int sw, int& steps) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const float y = op.template fast<FIN>(ti, ti.tb + j, steps);
        if (PASS == PASS_EMIT) stage_put(row, sw, j, y);
    }
}

// 1 / x by the hardware approximation (relative error within about 2^-23;
// subnormal x is read as zero), one instruction
__device__ __forceinline__ float rcp_approx_ftz(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The 32 steps of an RSI emit tile on the scaled state (see run_tile below);
// NORMAL: D stays normal over the tile.
template <bool NORMAL, bool kB>
__device__ __forceinline__ void rsi_emit_steps(OpRsi<kB>& op, const InTile& ti, float* row, int sw) {
    float N = op.sN, D = op.sD;
    const float b = op.beta;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float4 e4 = ti.xs[q], a4 = ti.xs[8 + q];
        const float ev[4] = {e4.x, e4.y, e4.z, e4.w}, av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            N = fmaf(b, N, fmaxf(ev[u], 0.f));
            D = fmaf(b, D, av[u]);
            const float y = NORMAL ? N * rcp_approx_ftz(D) : (D == 0.f ? 50.f : __fdividef(N, D));
            stage_put(row, sw, 4 * q + u, y);
        }
    }
    op.sN = N;
    op.sD = D;
}

// RSI emit tile with finite inputs.  Across consecutive such tiles the state
// is held as
//   N = 100 ag p       (the gain sum, scaled by 100 p)
//   D = (ag + al) p    (the gain + loss sum: its input is |d|)
// so a step is N <- b N + max(100 d, 0), D <- b D + |d| and the output
// 100 ag / (ag + al) = N / D: two FMAs and a max, no per-step scaling.  Each
// lane forms its step's 100 d and |d| once; the warp reads them back from
// shared memory four steps per 16-byte broadcast load.  The state goes back
// to (ag, al) only when the lane leaves these tiles (rsi_fast_exit), so the
// scale factors' roundings do not build up from tile to tile.
template <bool FIN, int PASS, bool kB>
__device__ __forceinline__ void run_tile(OpRsi<kB>& op, const InTile& ti, float* row, int sw, int& steps) {
    if constexpr (!(FIN && PASS == PASS_EMIT)) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float y = op.template fast<FIN>(ti, ti.tb + j, steps);
            if (PASS == PASS_EMIT) stage_put(row, sw, j, y);
        }
    } else {
        const int lane = threadIdx.x & 31;
        float xp = __shfl_up_sync(0xffffffffu, ti.xv, 1);
        if (lane == 0) xp = ti.xb;
        const float d = ti.xv - xp;
        float* xs = reinterpret_cast<float*>(ti.xs);
        __syncwarp();  // the previous tile's reads are done
        xs[lane] = 100.f * d;
        xs[32 + lane] = fabsf(d);
        __syncwarp();
        if (!op.sc) {
            op.sN = op.ag * (100.f * op.pf);  // 100 p is exact
            op.sD = (op.ag + op.al) * op.pf;
            op.sc = true;
        }
        // D never shrinks by more than b^32 >= 2^-32 over a tile (its inputs
        // are >= 0) nor grows past D + 32 max|d|, so a tile entered with D in
        // [2^-60, 2^100] and every |d| <= 2^100 keeps D and 1 / D normal: the
        // output is N times the hardware reciprocal, with no zero guard or
        // subnormal handling
        if (__all_sync(0xffffffffu, op.sD >= 0x1p-60f && op.sD <= 0x1p100f && fabsf(d) <= 0x1p100f))
            rsi_emit_steps<true>(op, ti, row, sw);
        else
            rsi_emit_steps<false>(op, ti, row, sw);
        steps += 32;
    }
}

// (ag, al) from the scaled emit-tile state, before any other step reads them
template <class Op> __device__ __forceinline__ void rsi_fast_exit(Op&) {}
template <bool kB> __device__ __forceinline__ void rsi_fast_exit(OpRsi<kB>& op) {
    if (op.sc) {
        op.ag = (op.sN * 0.01f) * op.inv_p;
        op.al = fmaf(op.sD, op.inv_p, -op.ag);
        op.sc = false;
    }
}

// TEMA emit tile with finite inputs: the three cascaded gain-exact EMA steps
// with shuffle-broadcast inputs and no phase checks; p == 1 copies x.
template <bool FIN, int PASS>
__device__ __forceinline__ void run_tile(OpTema& op, const InTile& ti, float* row, int sw, int& steps) {
    if constexpr (!(FIN && PASS == PASS_EMIT)) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float y = op.template fast<FIN>(ti, ti.tb + j, steps);
            if (PASS == PASS_EMIT) stage_put(row, sw, j, y);
        }
    } else {
        const float a = op.per;
        const bool copy = op.p1 == 0;
        float e1 = op.e1, e2 = op.e2, e3 = op.e3;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float v = __shfl_sync(0xffffffffu, ti.xv, j);
            e1 = fmaf(a, v - e1, e1);
            e2 = fmaf(a, e1 - e2, e2);
            e3 = fmaf(a, e2 - e3, e3);
            stage_put(row, sw, j, copy ? v : fmaf(3.f, e1 - e2, e3));
        }
        op.e1 = e1;  // (a p == 1 lane's state is never read: each step copies x)
        op.e2 = e2;
        op.e3 = e3;
        steps += 32;
    }
}

// Ops with a branch-free general-path step (Op::kUni) use it for t >= f.
template <class Op, class = void> struct HasUni : std::false_type {};
template <class Op> struct HasUni<Op, std::void_t<decltype(Op::kUni)>> : std::true_type {};

// ------------------------------------------------------- fast aggregates ---
// AGG blocks of the chunks in which every combo of a batch sweep is already
// running (EMA, DEMA, TEMA, RSI; chunk >= fast_from).  They share the launch
// with the seed chunk's general-path blocks, so the long per-step seeding run
// of chunk 0 overlaps with this work.  The block stages the chunk's inputs in
// shared memory, kAggTile steps at a time, and reads them back four steps per
// 16-byte broadcast load; each thread advances its combo from a zero state:
//   EMA / DEMA / TEMA  the emit pass's gain-exact steps e <- e + a (in - e)
//                      (a = 2 / (p + 1)), two FP ops per component;
//   RSI                zg = ag p, zl = al p: zg <- b zg + gain, zl <- b zl + loss
//                      (b = 1 - 1/p), one FMA each, scaled back at the chunk
//                      end (the output ratio is insensitive to the rounding
//                      of b, which scales gains and losses alike).
// A chunk holding a non-finite input
// (RSI: a non-finite difference) returns false and the block runs the general
// pass, which applies the skip / NaN rules.
enum FastKind { FK_NONE = -1, FK_EMA = 0, FK_DEMA = 1, FK_TEMA = 2, FK_RSI = 3 };
constexpr int kAggTile = 1024;  // steps staged per round (x, or gains + losses)

template <class Op> struct FastKindOf { static constexpr int k = FK_NONE; };
template <> struct FastKindOf<OpEma> { static constexpr int k = FK_EMA; };
template <> struct FastKindOf<OpDema> { static constexpr int k = FK_DEMA; };
template <> struct FastKindOf<OpTema> { static constexpr int k = FK_TEMA; };
template <> struct FastKindOf<OpRsi<true>> { static constexpr int k = FK_RSI; };

// smem: 2 * kAggTile floats, 16-byte aligned.  Called by the whole block.
// The EMA cascades advance kAggBlk steps at a time by their exact block
// transition: after B steps from (e1, e2, e3) with inputs x_0..x_{B-1}
// (a = 2/(p+1), b = 1 - a, j = 0 the oldest),
//   e1' = b^B e1 + sum_j a b^(B-1-j) x_j
//   e2' = b^B e2 + a B b^B e1 + sum_j a^2 (B-j) b^(B-1-j) x_j
//   e3' = b^B e3 + a B b^B e2 + a^2 b^B B(B+1)/2 e1
//         + sum_j a^3 (B-j)(B-j+1)/2 b^(B-1-j) x_j,
// evaluated in the gain-exact form e' = e + sum_i c_i (e_i - e) + (dot - W e)
// (W = the sum of the rounded x-weights; the coefficient of e is b^B in exact
// arithmetic), so a constant input stays fixed whatever the weights'
// rounding.  A block costs one FMA per input per component plus a few for
// the update: about half the work of the per-step form, whose two dependent
// FP ops per step also made each lane's chain latency-bound.
constexpr int kAggBlk = 16;

template <int NZ>
struct CascadeBlock {
    float w[NZ][kAggBlk];  // x-weights, j = 0 the oldest input of the block
    float W[NZ];           // their sums
    float c1, c2;          // a B b^B (e1 -> e2 and e2 -> e3), a^2 b^B B(B+1)/2 (e1 -> e3)
    __device__ void init(float al) {
        // b = 1 - a and its powers in f32: the weights carry relative errors
        // near 1e-6, a perturbation of the filter's time constant (the gain
        // stays exact by the update's form)
        const float be = 1.f - al;
        float pw = 1.f;  // b^(B-1-j), j from B-1 down to 0
#pragma unroll
        for (int q = 0; q < NZ; ++q) W[q] = 0.f;
#pragma unroll
        for (int j = kAggBlk - 1; j >= 0; --j) {
            const float r = (float)(kAggBlk - j);  // B - j
            w[0][j] = al * pw;
            if constexpr (NZ > 1) w[1][j] = al * al * r * pw;
            if constexpr (NZ > 2) w[2][j] = al * al * al * (r * (r + 1.f) * 0.5f) * pw;
            pw *= be;
        }
        // the sums in the order the dots accumulate (oldest first)
#pragma unroll
        for (int j = 0; j < kAggBlk; ++j)
#pragma unroll
            for (int q = 0; q < NZ; ++q) W[q] += w[q][j];
        c1 = al * (float)kAggBlk * pw;
        c2 = al * al * pw * (float)(kAggBlk * (kAggBlk + 1) / 2);
    }
    // one block of inputs x[0..B) (shared-memory broadcast reads, x 16-byte
    // aligned) advancing the first M components (the cascade's later stages
    // not yet started stay as they are)
    template <int M = NZ>
    __device__ __forceinline__ void step(float (&z)[NZ], const float* x) const {
        static_assert(M >= 1 && M <= NZ, "components");
        float d[M][2];
#pragma unroll
        for (int q = 0; q < M; ++q) d[q][0] = d[q][1] = 0.f;
#pragma unroll
        for (int j = 0; j < kAggBlk; j += 4) {
            const float4 v = *reinterpret_cast<const float4*>(x + j);
#pragma unroll
            for (int q = 0; q < M; ++q) {
                d[q][0] = fmaf(w[q][j], v.x, d[q][0]);
                d[q][1] = fmaf(w[q][j + 1], v.y, d[q][1]);
                d[q][0] = fmaf(w[q][j + 2], v.z, d[q][0]);
                d[q][1] = fmaf(w[q][j + 3], v.w, d[q][1]);
            }
        }
        const float e1 = z[0];
        z[0] = e1 + fmaf(-W[0], e1, d[0][0] + d[0][1]);
        if constexpr (M > 1) {
            const float e2 = z[1];
            z[1] = fmaf(c1, e1 - e2, e2) + fmaf(-W[1], e2, d[1][0] + d[1][1]);
            if constexpr (M > 2) {
                const float e3 = z[2];
                z[2] = fmaf(c1, e2 - e3, fmaf(c2, e1 - e3, e3)) + fmaf(-W[2], e3, d[2][0] + d[2][1]);
            }
        }
    }
    // steps t in [t0, t1) of the first M components: single gain-exact steps
    // up to a 4-aligned index, blocks of kAggBlk, single steps for the rest
    template <int M>
    __device__ __forceinline__ void run(float (&z)[NZ], const float* xs, int t0, int t1, float al) const {
        auto one = [&](float x) {
            z[0] = fmaf(al, x - z[0], z[0]);
            if constexpr (M > 1) z[1] = fmaf(al, z[0] - z[1], z[1]);
            if constexpr (M > 2) z[2] = fmaf(al, z[1] - z[2], z[2]);
        };
        int t = t0;
        for (; t < t1 && (t & 3); ++t) one(xs[t]);
        for (; t + kAggBlk <= t1; t += kAggBlk) step<M>(z, xs + t);
        for (; t < t1; ++t) one(xs[t]);
    }
};

template <int K>
__device__ bool agg_fast_block(const RecurArgs& a, int chunk, int c0, int c1, float* smem) {
    constexpr int NZ = K == FK_EMA ? 1 : (K == FK_TEMA ? 3 : 2);
    float* s0 = smem;
    float* s1 = smem + kAggTile;
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    const double p = li < a.n_lanes ? (double)a.periods[li] : 1.0;
    const float b = (float)(1.0 - 1.0 / p);       // RSI
    const float al = (float)(2.0 / (p + 1.0));   // the EMAs
    float z[NZ];
#pragma unroll
    for (int q = 0; q < NZ; ++q) z[q] = 0.f;
    CascadeBlock<NZ> cb;
    if constexpr (K != FK_RSI) cb.init(al);
    auto step = [&](float v, float w) {
        if constexpr (K == FK_RSI) {
            z[0] = fmaf(b, z[0], v);
            z[1] = fmaf(b, z[1], w);
        } else {
            // the gain-exact EMA step of the emit pass (OpEma::step)
            z[0] = fmaf(al, v - z[0], z[0]);
            if constexpr (NZ > 1) z[1] = fmaf(al, z[0] - z[1], z[1]);
            if constexpr (NZ > 2) z[2] = fmaf(al, z[1] - z[2], z[2]);
        }
    };
    for (int t0 = c0; t0 < c1; t0 += kAggTile) {
        const int m = min(kAggTile, c1 - t0);
        int bad = 0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const float v = __ldg(a.x + t0 + i);
            if (K == FK_RSI) {
                const float d = v - __ldg(a.x + t0 + i - 1);  // t0 + i >= c0 > 0
                bad |= !isfinite(d);
                s0[i] = d > 0.f ? d : 0.f;
                s1[i] = d < 0.f ? -d : 0.f;
            } else {
                bad |= !isfinite(v);
                s0[i] = v;
            }
        }
        if (__syncthreads_or(bad)) return false;
        if constexpr (K != FK_RSI) {
            const int mb = m - m % kAggBlk;
            for (int i = 0; i < mb; i += kAggBlk) cb.step(z, s0 + i);
            for (int i = mb; i < m; ++i) step(s0[i], 0.f);
            __syncthreads();
            continue;
        }
        const int m4 = m & ~3;
#pragma unroll 2
        for (int i = 0; i < m4; i += 4) {
            const float4 v = *reinterpret_cast<const float4*>(s0 + i);
            float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
            if (K == FK_RSI) w = *reinterpret_cast<const float4*>(s1 + i);
            step(v.x, w.x);
            step(v.y, w.y);
            step(v.z, w.z);
            step(v.w, w.w);
        }
        for (int i = m4; i < m; ++i) step(s0[i], K == FK_RSI ? s1[i] : 0.f);
        __syncthreads();
    }
    if (li < a.n_lanes) {
        float4 g = make_float4(0.f, 0.f, 0.f, (float)(c1 - c0));
        if constexpr (K == FK_RSI) {
            const float ip = (float)(1.0 / p);
            g.x = z[0] * ip;
            g.y = z[1] * ip;
        } else {
            g.x = z[0];
            if constexpr (NZ > 1) g.y = z[1];
            if constexpr (NZ > 2) g.z = z[2];
        }
        reinterpret_cast<float4*>(a.agg)[(size_t)chunk * a.n_lanes + li] = g;
    }
    return true;
}

// AGG record of a chunk from the tensor-core contraction's S partial sums
// (k_recur_tc.cu): per component the sum of the partials, times the row and
// column scales, plus the centring term.  One thread per lane.
template <int K>
__device__ void agg_from_partials(const RecurArgs& a, int chunk, int len) {
    constexpr int NZ = K == FK_EMA ? 1 : (K == FK_TEMA ? 3 : 2);
    const RecurTcView& v = a.tc;
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= a.n_lanes) return;
    const int j0 = chunk - v.g0;
    float z[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < NZ; ++q) {
        const int r = K == FK_RSI ? li : q * v.mpad + li;
        const int j = K == FK_RSI ? j0 + q * v.nc : j0;
        const float* p = v.part + (size_t)j * v.rows + r;
        const size_t stride = (size_t)v.npad * v.rows;
        // four independent loads in flight, summed in split order
        float acc = 0.f;
        int s = 0;
        for (; s + 4 <= v.S; s += 4) {
            const float p0 = __ldg(p + (size_t)s * stride), p1 = __ldg(p + (size_t)(s + 1) * stride);
            const float p2 = __ldg(p + (size_t)(s + 2) * stride), p3 = __ldg(p + (size_t)(s + 3) * stride);
            acc = (((acc + p0) + p1) + p2) + p3;
        }
        for (; s < v.S; ++s) acc += __ldg(p + (size_t)s * stride);
        z[q] = fmaf(acc, __ldg(v.row_scale + r) * __ldg(v.col_scale + j), __ldg(v.col_ref + j) * __ldg(v.row_sum + r));
    }
    reinterpret_cast<float4*>(a.agg)[(size_t)chunk * a.n_lanes + li] = make_float4(z[0], z[1], z[2], (float)len);
}

// ------------------------------------------------------ seed chunk, AGG ---
// The AGG pass needs only the state at the end of the seed chunk [0, c1).
// When every input in [first, c1) is finite and every lane's seed index lies
// inside the chunk, a lane gets there by plain loops instead of the per-step
// phase logic: the warm-up sum in four independent compensated partial sums
// (a short dependency chain), then the running steps from the seed on.  The
// per-step phase logic made each lane's 1,000-2,000-step walk the critical
// path of the whole AGG launch.
// Pair sum of two (hi, lo) compensated values (TwoSum of the heads).
__device__ __forceinline__ float2 pair_add(float2 a, float2 b) {
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb);
    const float lo = a.y + b.y + e;
    const float hi = s + lo;
    return make_float2(hi, lo - (hi - s));
}

// Block-wide sums of the seed chunk's warm-up terms in 32-step segments:
// segment i covers [b0 + 32 i, b0 + 32 i + 32) ∩ [b0, c1) and holds, as
// compensated (hi, lo) pairs, the sum of x (EMA: b0 = first) or of the
// exact gains and losses (RSI: b0 = first + 1; the differences to the
// previous bar).  A lane's warm-up sum over p terms from b0 is then p / 32
// segment sums plus at most 31 single terms, instead of a p-step chain.
// seg: float4 {sum hi, sum lo, loss hi, loss lo} per segment.  Called by the
// whole block; every input in [b0 - 1, c1) is finite.
template <int K>
__device__ void seed_segments(const float* xs, int b0, int c1, float4* seg) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nseg = (c1 - b0 + 31) >> 5;
    for (int i = warp; i < nseg; i += nw) {
        const int t = b0 + 32 * i + lane;
        float2 u = make_float2(0.f, 0.f), v = make_float2(0.f, 0.f);
        if (t < c1) {
            if constexpr (K == FK_RSI) {
                const float x1 = xs[t], x0 = xs[t - 1];
                const float d = x1 - x0;  // exact difference d + e (TwoDiff)
                const float bb = d - x1;
                const float e = (x1 - (d - bb)) - (x0 + bb);
                if (d > 0.f) u = make_float2(d, e);
                else if (d < 0.f) v = make_float2(-d, -e);
            } else {
                u = make_float2(xs[t], 0.f);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            u = pair_add(u, make_float2(__shfl_xor_sync(0xffffffffu, u.x, o), __shfl_xor_sync(0xffffffffu, u.y, o)));
            if constexpr (K == FK_RSI)
                v = pair_add(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o),
                                            __shfl_xor_sync(0xffffffffu, v.y, o)));
        }
        if (lane == 0) seg[i] = make_float4(u.x, u.y, v.x, v.y);
    }
}

template <int K>
__device__ bool agg_seed_fast(const RecurArgs& a, float* xs, int c1, int cap) {
    const int f = a.first;
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    const bool lane_ok = li < a.n_lanes;
    const int p = lane_ok ? a.periods[li] : 1;
    // seed index of the lane (the op's s)
    const int s = K == FK_EMA ? f + p - 1 : K == FK_RSI ? f + p : f + 2 * (p - 1);
    int bad = lane_ok && (p <= 0 || s >= c1);
    for (int t = max(f, 0) + threadIdx.x; t < c1; t += blockDim.x) bad |= !isfinite(xs[t]);
    if (__syncthreads_or(bad)) return false;
    // segment sums of the warm-up terms (EMA, RSI) when they fit beside xs
    const int b0 = K == FK_RSI ? f + 1 : f;
    const int seg_off = (c1 + 3) & ~3;
    const bool use_seg = K != FK_TEMA && f >= 0 && seg_off + 4 * ((c1 - b0 + 31) >> 5) <= cap;
    float4* seg = reinterpret_cast<float4*>(xs + seg_off);
    if (use_seg) {
        seed_segments<K>(xs, b0, c1, seg);
        __syncthreads();
    }
    if (!lane_ok) return true;
    float4 g = make_float4(0.f, 0.f, 0.f, kAbsolute);
    if constexpr (K == FK_EMA) {
        // the op's warm-up mean of x[f..s] (every value finite: count p)
        Acc acc[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q].zero();
        int t = f;
        if (use_seg) {
            const int full = p >> 5;
            for (int i = 0; i < full; ++i) {
                const float4 sv = seg[i];
                acc[i & 1].add(sv.x);
                acc[i & 1].lo += sv.y;
            }
            t = f + 32 * full;
        }
        for (; t + 3 <= s; t += 4)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q].add(xs[t + q]);
        for (; t <= s; ++t) acc[0].add(xs[t]);
        acc[0].add(acc[1].hi); acc[0].add(acc[1].lo);
        acc[2].add(acc[3].hi); acc[2].add(acc[3].lo);
        acc[0].add(acc[2].hi); acc[0].add(acc[2].lo);
        const float al = (float)(2.0 / ((double)p + 1.0));
        CascadeBlock<1> cb;
        cb.init(al);
        float y[1] = {acc[0].f() / (float)p};
        cb.run<1>(y, xs, s + 1, c1, al);  // the running steps, kAggBlk at a time
        g.x = y[0];
    } else if constexpr (K == FK_RSI) {
        // sums of the gains and losses of the p deltas in (f, s], then the
        // Wilder steps (the op's seed() and step() arithmetic)
        Acc sg[2], sl[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) { sg[q].zero(); sl[q].zero(); }
        int t = f + 1;
        if (use_seg) {
            const int full = p >> 5;
            for (int i = 0; i < full; ++i) {
                const float4 sv = seg[i];
                sg[i & 1].add(sv.x);
                sg[i & 1].lo += sv.y;
                sl[i & 1].add(sv.z);
                sl[i & 1].lo += sv.w;
            }
            t = f + 1 + 32 * full;
        }
        for (; t + 1 <= s; t += 2)
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const float v = xs[t + q], xp = xs[t + q - 1];
                if (v > xp) sg[q].add_diff(v, xp);
                else if (v < xp) sl[q].add_diff(xp, v);
            }
        for (; t <= s; ++t) {
            const float v = xs[t], xp = xs[t - 1];
            if (v > xp) sg[0].add_diff(v, xp);
            else if (v < xp) sl[0].add_diff(xp, v);
        }
        const double inv_p = (double)(float)(1.0 / (double)p);
        const float beta = (float)(1.0 - 1.0 / (double)p), ip = (float)(1.0 / (double)p);
        float ag = (float)((sg[0].d() + sg[1].d()) * inv_p);
        float al = (float)((sl[0].d() + sl[1].d()) * inv_p);
        for (t = s + 1; t < c1; ++t) {
            const float d = xs[t] - xs[t - 1];
            ag = fmaf(ag, beta, ip * (d > 0.f ? d : 0.f));
            al = fmaf(al, beta, ip * (d < 0.f ? -d : 0.f));
        }
        g.x = ag;
        g.y = al;
    } else {
        // TEMA: e1 from x[f]; e2 joins at f + p - 1 as a copy of e1, e3 at s
        // as a copy of e2 (the op's accum), then all three run (p == 1:
        // the op copies x into e1)
        const float per = (float)(2.0 / ((double)p + 1.0));
        if (p == 1) {
            g.x = xs[c1 - 1];
        } else {
            // the three phases kAggBlk steps at a time (CascadeBlock)
            const int start2 = f + p - 1;
            CascadeBlock<3> cb;
            cb.init(per);
            float z[3] = {xs[f], 0.f, 0.f};
            cb.run<1>(z, xs, f + 1, start2 + 1, per);
            z[1] = z[0];
            cb.run<2>(z, xs, start2 + 1, s + 1, per);
            z[2] = z[1];
            cb.run<3>(z, xs, s + 1, c1, per);
            g.x = z[0];
            g.y = z[1];
            g.z = z[2];
        }
    }
    reinterpret_cast<float4*>(a.agg)[li] = g;  // chunk 0
    return true;
}

// One step of the general (per-step phase) path of one lane: warm-up
// accumulation until the seed index, the seed, then running steps.
template <class Op, class In>
__device__ __forceinline__ float general_step(Op& op, bool active, bool seeded_ever, bool& running, int& steps,
                                              const In& in, int t) {
    float v = qnan();
    if constexpr (HasUni<Op>::value) {
        if (active && t >= op.f) v = op.uni(in, t, steps);
        return v;
    }
    if (active && t >= op.f && seeded_ever) {
        if (running) {
            steps += op.step(in, t);
            v = op.value(in, t);
        } else if (t <= op.s) {
            op.accum(in, t);
            if (t == op.s) {
                op.seed();
                running = true;
                v = op.value(in, t);
            } else {
                v = op.warm_value(t);
            }
        }
    } else if (active && t >= op.f && !seeded_ever) {
        op.accum(in, t);  // never seeded (s >= n): warm-up style outputs only
        v = op.warm_value(t);
    }
    return v;
}

// AGG record of one (lane, chunk): state, and applied steps or a marker for
// a chunk before the seed / holding the seed.
template <class Op>
__device__ __forceinline__ void write_agg(const RecurArgs& a, const Op& op, bool active, bool seeded_ever, int steps,
                                          int chunk, int c0, int c1, int li) {
    float4 g;
    const bool abs_chunk = active && seeded_ever && c0 <= op.s && op.s < c1;
    const bool before = !active || !seeded_ever || c1 <= op.s;
    g.x = Op::NS > 0 ? op.get(0) : 0.f;
    g.y = Op::NS > 1 ? op.get(1) : 0.f;
    g.z = Op::NS > 2 ? op.get(2) : 0.f;
    g.w = before ? kBeforeSeed : (abs_chunk ? kAbsolute : (float)steps);
    if (before) g.x = g.y = g.z = 0.f;
    reinterpret_cast<float4*>(a.agg)[(size_t)chunk * a.n_lanes + li] = g;
}


// Batch EMIT stages 64 steps per lane (two 32-step tiles) and writes each
// row's 256-byte segment with one float2 store per lane: on GB300 that write
// pattern reaches ~6.9 TB/s where 128-byte row segments reach ~6.2 TB/s.
// Staging rows are 66 floats (8-byte aligned float2 reads); rows 16..31 swap
// the two floats of each pair (column c is stored at c ^ 1), so the per-step
// scalar writes of the 32 lanes fall in 32 distinct banks.
constexpr int kSeg = 64;
constexpr int kStageW = kSeg + 2;

template <class Op, bool TM, int PASS>
__global__ void __launch_bounds__(kWarps * 32)
k_recur(RecurArgs a) {
    __shared__ __align__(16) float stage[kWarps][32][(PASS == PASS_EMIT && !TM) ? kStageW : 33];
    // per warp: a fast tile's broadcast inputs (EMIT), 2 x 32 floats
    __shared__ float4 xin[kWarps][PASS == PASS_EMIT ? 16 : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int group = blockIdx.x * kWarps + warp;
    const int li = group * 32 + lane;
    const bool valid = li < a.n_lanes;
    const int chunk = blockIdx.y;
    int c0, c1;
    recur_chunk_bounds(a, chunk, c0, c1);
    if (c0 >= a.n) return;
    if constexpr (PASS == PASS_AGG && !TM && FastKindOf<Op>::k != FK_NONE) {
        // chunks the tensor-core contraction covered: sum its partials
        const RecurTcView& v = a.tc;
        if (v.done && chunk >= v.g0 && chunk < v.g0 + v.nc && v.done[chunk] && *v.err == 0) {
            agg_from_partials<FastKindOf<Op>::k>(a, chunk, c1 - c0);
            return;
        }
        static_assert(sizeof(stage) >= 2 * kAggTile * sizeof(float), "fast AGG staging");
        if (a.fast_agg && chunk >= a.fast_from &&
            agg_fast_block<FastKindOf<Op>::k>(a, chunk, c0, c1, &stage[0][0][0]))
            return;
        __syncthreads();  // the general pass below reuses `stage`
        // the seed chunk: each thread replays its combo's warm-up and seed
        // from the chunk's inputs staged in shared memory (no per-step
        // shuffles or warp-wide tiles: the lanes run independently)
        if (a.fast_agg && chunk == 0 && c1 <= (int)(sizeof(stage) / sizeof(float))) {
            float* xs = &stage[0][0][0];
            for (int i = threadIdx.x; i < c1; i += blockDim.x) xs[i] = __ldg(a.x + i);
            __syncthreads();
            constexpr int FK = FastKindOf<Op>::k;
            if constexpr (FK == FK_EMA || FK == FK_RSI || FK == FK_TEMA) {
                if (a.first < a.n && agg_seed_fast<FK>(a, xs, c1, (int)(sizeof(stage) / sizeof(float)))) return;
            }
            const int l0 = blockIdx.x * blockDim.x + threadIdx.x;
            if (l0 < a.n_lanes) {
                const int p0 = a.periods[l0];
                Op op0;
                op0.init(p0 > 0 ? p0 : 1, a.first);
                const bool act0 = a.first < a.n && p0 > 0;
                const bool seeded0 = act0 && op0.s < a.n;
                bool run0 = false;
                int st0 = 0;
                int t = min(a.first, c1);
                // warm-up and seed through the per-step phase logic ...
                for (; t < c1 && !run0; ++t) {
                    InStep st;  // x[t] and x[t - 1] from shared memory
                    st.t = t;
                    st.x0 = xs[t];
                    st.x1 = t > 0 ? xs[t - 1] : 0.f;
                    st.h0 = st.l0 = 0.f;
                    general_step(op0, act0, seeded0, run0, st0, st, t);
                }
                // ... then the running steps without it (the same state update
                // as the op's step(); t > s >= 0 here)
                if constexpr (!HasUni<Op>::value) {
                    float xprev = t > 0 && t <= c1 ? xs[t - 1] : 0.f;
#pragma unroll 4
                    for (; t < c1; ++t) {
                        const float xv = xs[t];
                        const InStep st{t, xv, xprev, 0.f, 0.f};
                        op0.template fast<false>(st, t, st0);
                        xprev = xv;
                    }
                }
                write_agg(a, op0, act0, seeded0, st0, 0, 0, c1, l0);
            }
            return;
        }
    }
    // a warp with no valid lane has nothing to compute (whole warp leaves; the
    // kernel has no block-wide barrier)
    if (group * 32 >= a.n_lanes) return;

    Op op;
    int p = 0, first = a.n;
    if (valid) {
        p = TM ? a.period : a.periods[li];
        first = TM ? a.first_tm[li] : a.first;
    }
    op.init(p > 0 ? p : 1, first);
    const bool active = valid && first < a.n && p > 0;
    const bool seeded_ever = active && op.s < a.n;

    typename std::conditional<TM, InTm, InBatch>::type in;
    if constexpr (TM) {
        in = InTm{a.x, a.h, a.l, a.c, (size_t)a.cols, (size_t)(valid ? li : 0)};
    } else {
        in = InBatch{a.x, a.h, a.l, a.c};
    }

    // chunk entry state
    bool running = false;
    if (active) {
        if (c0 > op.s && seeded_ever) {
            if (PASS == PASS_AGG) {
                op.zero();
            } else {
                float4 cv = reinterpret_cast<const float4*>(a.carry)[(size_t)chunk * a.n_lanes + li];
                if (Op::NS > 0) op.set(0, cv.x);
                if (Op::NS > 1) op.set(1, cv.y);
                if (Op::NS > 2) op.set(2, cv.z);
            }
            running = true;
        } else if (c0 > op.f) {
            // the chunk starts inside the warm-up: accumulate [f, c0) first
            const int end = min(c0, op.s + 1);
            for (int t = op.f; t < end; ++t) op.accum(in, t);
        }
    }
    // first time index from which this lane needs no phase checks; lanes that
    // never write (invalid / all-NaN) do not hold the warp back
    const int run_from = (active && seeded_ever) ? max(op.s + 1, op.warm) : (valid ? INT_MAX : INT_MIN);
    const int warp_run_from = warp_max(run_from);

    int steps = 0;
    // this lane's staging row (batch EMIT): the current 64-step segment starts
    // at seg0, the tile at column off = tb - seg0 (0 or 32), swizzle sw
    const int sw = (lane >> 4) & 1;
    const bool vec2 = !TM && PASS == PASS_EMIT && (a.n & 1) == 0 && (c0 & 1) == 0 &&
                      (reinterpret_cast<uintptr_t>(a.out) & 7) == 0;
    for (int tb = c0; tb < c1; tb += 32) {
        const int te = min(tb + 32, c1);
        const int seg0 = c0 + ((tb - c0) & ~(kSeg - 1));
        const int off = tb - seg0;
        float* srow = &stage[warp][lane][off];
        if (tb >= warp_run_from) {
            // ---- fast path: every lane running and past warm-up
            if (!TM && te - tb == 32) {
                // the tile's inputs in registers, one coalesced load per lane
                InTile ti;
                ti.tb = tb;
                ti.xs = &xin[warp][0];
                if constexpr (Op::kHlc) {
                    ti.hv = __ldg(a.h + tb + lane);
                    ti.lv = __ldg(a.l + tb + lane);
                    ti.cv = __ldg(a.c + tb + lane);
                    ti.cb = __ldg(a.c + tb - 1);
                    ti.xv = ti.cv;
                    ti.xb = ti.cb;
                } else {
                    ti.xv = __ldg(a.x + tb + lane);
                    ti.xb = __ldg(a.x + tb - 1);
                }
                // a tile whose inputs (and the value before it) are all finite
                // runs without per-step skip / NaN logic
                bool fin;
                if constexpr (Op::kHlc) {
                    fin = __all_sync(0xffffffffu, isfinite(ti.hv) && isfinite(ti.lv) && isfinite(ti.cv) &&
                                                      isfinite(ti.cb));
                } else {
                    fin = __all_sync(0xffffffffu, isfinite(ti.xv) && isfinite(ti.xb));
                }
                if (fin) {
                    run_tile<true, PASS>(op, ti, srow, sw, steps);
                } else {
                    rsi_fast_exit(op);
                    run_tile<false, PASS>(op, ti, srow, sw, steps);
                }
            } else if (PASS == PASS_EMIT && !TM) {
                rsi_fast_exit(op);
#pragma unroll 8
                for (int t = tb; t < te; ++t) srow[(t - tb) ^ sw] = op.fast(in, t, steps);
            } else if (PASS == PASS_EMIT) {
#pragma unroll 8
                for (int t = tb; t < te; ++t) {
                    const float v = op.fast(in, t, steps);
                    if (valid) a.out[(size_t)t * a.cols + li] = v;
                }
            } else {
#pragma unroll 8
                for (int t = tb; t < te; ++t) op.fast(in, t, steps);
            }
        } else {
            // ---- general path: per-step phase logic
            rsi_fast_exit(op);  // (a no-op: general tiles come before the fast ones)
            auto gen_step = [&](const auto& in_, int t) -> float {
                return general_step(op, active, seeded_ever, running, steps, in_, t);
            };
            if constexpr (!TM) {
                // the tile's inputs in registers (one coalesced load per lane);
                // each step's values are broadcast by shuffles at the top of
                // the warp-uniform step loop, before any per-lane branch
                const int nt = te - tb;
                float xv = 0.f, hv = 0.f, lv = 0.f, pb = 0.f;
                if constexpr (Op::kHlc) {
                    if (lane < nt) {
                        hv = __ldg(a.h + tb + lane);
                        lv = __ldg(a.l + tb + lane);
                        xv = __ldg(a.c + tb + lane);
                    }
                    if (tb > 0) pb = __ldg(a.c + tb - 1);
                } else {
                    if (lane < nt) xv = __ldg(a.x + tb + lane);
                    if (tb > 0) pb = __ldg(a.x + tb - 1);
                }
                for (int j = 0; j < nt; ++j) {
                    InStep st;
                    st.t = tb + j;
                    st.x0 = __shfl_sync(0xffffffffu, xv, j);
                    const float xm = __shfl_sync(0xffffffffu, xv, (j - 1) & 31);
                    st.x1 = j > 0 ? xm : pb;
                    if constexpr (Op::kHlc) {
                        st.h0 = __shfl_sync(0xffffffffu, hv, j);
                        st.l0 = __shfl_sync(0xffffffffu, lv, j);
                    }
                    const float v = gen_step(st, tb + j);
                    if (PASS == PASS_EMIT) srow[j ^ sw] = v;
                }
            } else {
                for (int t = tb; t < te; ++t) {
                    const float v = gen_step(in, t);
                    if (PASS == PASS_EMIT && valid) a.out[(size_t)t * a.cols + li] = v;
                }
            }
        }
        if (PASS == PASS_EMIT && !TM && (off == kSeg - 32 || te == c1)) {
            // flush the segment [seg0, te) of the warp's 32 rows
            __syncwarp();
            const int row0 = group * 32;
            const int rows = min(32, a.n_lanes - row0);
            const int len = te - seg0;
            float* ob = a.out + (size_t)row0 * a.n + seg0;
            if (vec2 && len == kSeg) {
                // rows 0..15 as staged, rows 16..31 with each pair swapped back
                const int r16 = min(rows, 16);
                float* op = ob + 2 * lane;
#pragma unroll 4
                for (int r = 0; r < r16; ++r, op += a.n)
                    *reinterpret_cast<float2*>(op) = *reinterpret_cast<const float2*>(&stage[warp][r][2 * lane]);
#pragma unroll 4
                for (int r = 16; r < rows; ++r, op += a.n) {
                    const float2 v = *reinterpret_cast<const float2*>(&stage[warp][r][2 * lane]);
                    *reinterpret_cast<float2*>(op) = make_float2(v.y, v.x);
                }
            } else {
                for (int h = lane; h < len; h += 32) {
#pragma unroll 4
                    for (int r = 0; r < rows; ++r) ob[(size_t)r * a.n + h] = stage[warp][r][h ^ ((r >> 4) & 1)];
                }
            }
            __syncwarp();
        }
    }
    if (PASS == PASS_AGG && valid) write_agg(a, op, active, seeded_ever, steps, chunk, c0, c1, li);
}

// Carry-in of every chunk: an exclusive scan, over the chunks of one lane, of
// the affine chunk maps S -> M_k S + b_k.  One warp per lane: each thread
// composes a contiguous run of chunks, a Kogge-Stone scan across the warp
// combines the runs, then each thread re-walks its run writing carries.  The
// maps are N x N with N the op's state size, in double-single arithmetic.
// Structure of an op's transition matrix: every product of such matrices
// keeps it, so the f64 work skips the structural zeros (GB300's FP64 rate
// makes them count).  0 = full, 1 = lower triangular (DEMA, TEMA cascades),
// 2 = diagonal (RSI's independent gain / loss averages).
template <class Op, class = void> struct ShapeOf { static constexpr int v = 0; };
template <class Op> struct ShapeOf<Op, std::void_t<decltype(Op::kShape)>> { static constexpr int v = Op::kShape; };
__host__ __device__ constexpr bool shape_nz(int sh, int r, int c) { return sh == 0 || (sh == 1 ? c <= r : c == r); }

template <int N>
struct AffD {
    D2 m[N][N];
    D2 b[N];
};
template <int N>
__device__ __forceinline__ void affd_identity(AffD<N>& a) {
#pragma unroll
    for (int r = 0; r < N; ++r) {
#pragma unroll
        for (int c = 0; c < N; ++c) a.m[r][c] = {r == c ? 1.f : 0.f, 0.f};
        a.b[r] = {0.f, 0.f};
    }
}
// second o first (apply `first`, then `second`)
template <int N, int SH>
__device__ __forceinline__ AffD<N> affd_then(const AffD<N>& first, const AffD<N>& second) {
    AffD<N> o;
#pragma unroll
    for (int r = 0; r < N; ++r) {
        D2 br = second.b[r];
#pragma unroll
        for (int c = 0; c < N; ++c) {
            D2 mrc = {0.f, 0.f};
            if (shape_nz(SH, r, c)) {
#pragma unroll
                for (int q = 0; q < N; ++q)
                    if (shape_nz(SH, r, q) && shape_nz(SH, q, c)) mrc = d2_fma(second.m[r][q], first.m[q][c], mrc);
                br = d2_fma(second.m[r][c], first.b[c], br);
            }
            o.m[r][c] = mrc;
        }
        o.b[r] = br;
    }
    return o;
}
template <int N, int SH>
__device__ __forceinline__ AffD<N> affd_shfl_up(const AffD<N>& a, int d) {
    AffD<N> o;
#pragma unroll
    for (int r = 0; r < N; ++r) {
#pragma unroll
        for (int c = 0; c < N; ++c) o.m[r][c] = shape_nz(SH, r, c) ? d2_shfl_up(a.m[r][c], d) : D2{0.f, 0.f};
        o.b[r] = d2_shfl_up(a.b[r], d);
    }
    return o;
}

// M^n of the op's transition (n steps), column by column from propagate.
template <class Op>
__device__ void trans_pow(long long n, int p, D2 (&m)[Op::NS][Op::NS]) {
    constexpr int N = Op::NS;
    D2 al, b;
    Op::coef(p, al, b);
    const D2 an = d2_pow(b, n), nd = d2_from_ll(n);
#pragma unroll
    for (int c = 0; c < N; ++c) {
        D2 e[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        e[c] = {1.f, 0.f};
        Op::propagate(e, nd, al, an, p);
#pragma unroll
        for (int r = 0; r < N; ++r) m[r][c] = e[r];
    }
}

// The map of one chunk from its AGG record (state, applied steps or marker).
template <class Op>
__device__ void chunk_map(const float4 g, int p, int chunk, const D2 (&ml)[Op::NS][Op::NS], AffD<Op::NS>& a) {
    constexpr int N = Op::NS;
    if (g.w == kBeforeSeed) {
        affd_identity(a);
        return;
    }
    if (g.w == kAbsolute) {
#pragma unroll
        for (int r = 0; r < N; ++r)
#pragma unroll
            for (int c = 0; c < N; ++c) a.m[r][c] = {0.f, 0.f};
    } else if (g.w == (float)chunk) {
#pragma unroll
        for (int r = 0; r < N; ++r)
#pragma unroll
            for (int c = 0; c < N; ++c) a.m[r][c] = ml[r][c];
    } else {
        trans_pow<Op>((long long)g.w, p, a.m);
    }
    const float gb[3] = {g.x, g.y, g.z};
#pragma unroll
    for (int r = 0; r < N; ++r) a.b[r] = {gb[r], 0.f};
}

// Carry-in state of every (lane, chunk): one warp per lane, each thread a
// contiguous run of chunks.  Pass 1 composes the thread's chunk maps, a warp
// scan of the compositions gives each thread its entry state, pass 2 applies
// the maps chunk by chunk and writes the carries.  Full chunks share one
// linear part M (the transition of `chunk` steps), so a run of them only
// updates the offset (b <- M b + agg) and its power M^cnt is applied once
// when another map follows or the run ends: the work per chunk is a
// matrix-vector product.
template <class Op>
__global__ void k_recur_carry(RecurArgs a, int n_chunks) {
    constexpr int N = Op::NS;
    constexpr int SH = ShapeOf<Op>::v;
    const int lane = threadIdx.x & 31;
    const int li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // one warp per lane of the scan
    if (li >= a.n_lanes) return;
    const int p = a.layout ? a.period : a.periods[li];
    const float4* agg = reinterpret_cast<const float4*>(a.agg);
    float4* carry = reinterpret_cast<float4*>(a.carry);
    const int per = (n_chunks + 31) / 32;
    const int k0 = min(lane * per, n_chunks), k1 = min(k0 + per, n_chunks);
    const float full = (float)a.chunk;
    D2 ml[N][N], mper[N][N];  // transitions of one and of `per` full chunks
    trans_pow<Op>((long long)a.chunk, p, ml);
    trans_pow<Op>((long long)per * a.chunk, p, mper);
    // v <- M v + g (the map of a full chunk applied to a vector)
    auto full_step = [&](D2 (&v)[N], const float4 g) {
        const float gb[3] = {g.x, g.y, g.z};
        D2 t[N];
#pragma unroll
        for (int r = 0; r < N; ++r) {
            D2 x = {gb[r], 0.f};
#pragma unroll
            for (int c = 0; c < N; ++c)
                if (shape_nz(SH, r, c)) x = d2_fma(ml[r][c], v[c], x);
            t[r] = x;
        }
#pragma unroll
        for (int r = 0; r < N; ++r) v[r] = t[r];
    };
    AffD<N> run;
    affd_identity(run);
    int cnt = 0;          // full chunks whose linear part is not yet in run.m
    bool m_zero = false;  // run.m == 0 (after an absolute chunk): powers leave it 0
    auto flush = [&]() {
        if (cnt == 0 || m_zero) {
            cnt = 0;
            return;
        }
        D2 pw[N][N];
        if (cnt == per) {
#pragma unroll
            for (int r = 0; r < N; ++r)
#pragma unroll
                for (int c = 0; c < N; ++c) pw[r][c] = mper[r][c];
        } else {
            trans_pow<Op>((long long)cnt * a.chunk, p, pw);
        }
        D2 m2[N][N];  // run.m <- M^cnt run.m (the offset is already current)
#pragma unroll
        for (int r = 0; r < N; ++r)
#pragma unroll
            for (int c = 0; c < N; ++c) {
                D2 v = {0.f, 0.f};
                if (shape_nz(SH, r, c))
#pragma unroll
                    for (int q = 0; q < N; ++q)
                        if (shape_nz(SH, r, q) && shape_nz(SH, q, c)) v = d2_fma(pw[r][q], run.m[q][c], v);
                m2[r][c] = v;
            }
#pragma unroll
        for (int r = 0; r < N; ++r)
#pragma unroll
            for (int c = 0; c < N; ++c) run.m[r][c] = m2[r][c];
        cnt = 0;
    };
    // the chunk records in a 4-deep register queue: loads run ahead of the
    // dependent math without an unrolled batch (the scan's double-single code
    // is large, and unrolled copies of it overflowed the instruction cache)
    const float4 kNone = make_float4(0.f, 0.f, 0.f, 0.f);
    auto rec = [&](int k) { return k < k1 ? __ldg(agg + (size_t)k * a.n_lanes + li) : kNone; };
    float4 q0 = rec(k0), q1 = rec(k0 + 1), q2 = rec(k0 + 2), q3 = rec(k0 + 3);
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
        const float4 g = q0;
        q0 = q1;
        q1 = q2;
        q2 = q3;
        q3 = rec(k + 4);
        if (g.w == full) {
            full_step(run.b, g);
            ++cnt;
        } else {
            flush();
            AffD<N> ak;
            chunk_map<Op>(g, p, a.chunk, ml, ak);
            run = affd_then<N, SH>(run, ak);
            if (g.w == kAbsolute) m_zero = true;
        }
    }
    flush();
#pragma unroll 1
    for (int d = 1; d < 32; d <<= 1) {
        const AffD<N> up = affd_shfl_up<N, SH>(run, d);
        if (lane >= d) run = affd_then<N, SH>(up, run);
    }
    AffD<N> ex = affd_shfl_up<N, SH>(run, 1);
    if (lane == 0) affd_identity(ex);
    D2 S[N];  // state at the start of chunk k0
#pragma unroll
    for (int r = 0; r < N; ++r) S[r] = ex.b[r];
    q0 = rec(k0);
    q1 = rec(k0 + 1);
    q2 = rec(k0 + 2);
    q3 = rec(k0 + 3);
#pragma unroll 1
    for (int k = k0; k < k1; ++k) {
        const float4 g = q0;
        q0 = q1;
        q1 = q2;
        q2 = q3;
        q3 = rec(k + 4);
        {
            float4 cv = make_float4(0.f, 0.f, 0.f, 0.f);
            cv.x = S[0].hi + S[0].lo;
            if (N > 1) cv.y = S[N > 1 ? 1 : 0].hi + S[N > 1 ? 1 : 0].lo;
            if (N > 2) cv.z = S[N > 2 ? 2 : 0].hi + S[N > 2 ? 2 : 0].lo;
            carry[(size_t)k * a.n_lanes + li] = cv;
            if (g.w == full) {
                full_step(S, g);
            } else {
                AffD<N> ak;
                chunk_map<Op>(g, p, a.chunk, ml, ak);
                D2 t[N];
#pragma unroll
                for (int r = 0; r < N; ++r) {
                    D2 v = ak.b[r];
#pragma unroll
                    for (int c = 0; c < N; ++c)
                        if (shape_nz(SH, r, c)) v = d2_fma(ak.m[r][c], S[c], v);
                    t[r] = v;
                }
#pragma unroll
                for (int r = 0; r < N; ++r) S[r] = t[r];
            }
        }
    }
}

template <class Op, bool TM>
vta_status run(const RecurArgs& a, cudaStream_t st) {
    const int n_chunks = recur_n_chunks(a.n, a.chunk, a.chunk0);
    const int groups = (int)ceil_div(a.n_lanes, 32);
    dim3 grid(ceil_div(groups, kWarps), n_chunks);
    if (n_chunks > 65535) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "recurrence: too many time chunks");
    if (n_chunks > 1) {
        k_recur<Op, TM, PASS_AGG><<<grid, kWarps * 32, 0, st>>>(a);
        VTA_TRY(check_launch("k_recur_agg"));
        k_recur_carry<Op><<<ceil_div((size_t)a.n_lanes * 32, 128), 128, 0, st>>>(a, n_chunks);
        VTA_TRY(check_launch("k_recur_carry"));
    }
    ktimer_begin(st);
    k_recur<Op, TM, PASS_EMIT><<<grid, kWarps * 32, 0, st>>>(a);
    ktimer_end(st);
    return check_launch("k_recur_emit");
}

}  // namespace

int recur_state_dim(int kind) {
    switch (kind) {
        case RK_DEMA: return 2;
        case RK_TEMA: return 3;
        case RK_RSI: return 2;
        default: return 1;
    }
}

vta_status launch_recurrence(const RecurArgs& a, cudaStream_t st) {
    const bool tm = a.layout != 0;
    switch (a.kind) {
        case RK_EMA: return tm ? run<OpEma, true>(a, st) : run<OpEma, false>(a, st);
        case RK_DEMA: return tm ? run<OpDema, true>(a, st) : run<OpDema, false>(a, st);
        case RK_TEMA: return tm ? run<OpTema, true>(a, st) : run<OpTema, false>(a, st);
        case RK_RSI: return tm ? run<OpRsi<false>, true>(a, st) : run<OpRsi<true>, false>(a, st);
        case RK_WILDERS: return tm ? run<OpWilders, true>(a, st) : run<OpWilders, false>(a, st);
        case RK_ATR: return tm ? run<OpAtr, true>(a, st) : run<OpAtr, false>(a, st);
        default: return fail(VTA_ERR_INVALID_INPUT, "unknown recurrence kind");
    }
}

}  // namespace vta
