// Chunked linear-recurrence scans: EMA, DEMA, TEMA, RSI, Wilders, ATR.
//
// Each indicator is a linear time-invariant recurrence once seeded, so the
// time axis is cut into chunks processed in parallel:
//   pass A (k_recur<.., PASS_AGG>):  per (lane, chunk) run the recurrence from
//       a zero state (or from the exact seed inside the seed chunk) and keep
//       the chunk-end state plus the number of applied steps;
//   pass B (k_recur_carry):          per lane, compose the chunk transforms in
//       f64 (closed-form powers of the transition matrix) -> carry-in per chunk;
//   pass C (k_recur<.., PASS_EMIT>): per (lane, chunk) re-run from the carry
//       and write the outputs.
// A "lane" is one parameter combo of a single-series sweep (batch layout:
// every lane reads the same x[t], outputs are staged through shared memory so
// each store instruction writes one contiguous 128-byte row segment) or one
// series of a time-major matrix (coalesced loads and stores directly).
// The warm-up rules (seed index, NaN prefix, running-mean outputs) follow the
// crate's scalar paths cited on each op.
#include <climits>

#include "vta_internal.h"

namespace vta {
namespace {

constexpr int kWarps = 4;  // warps per block
__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }

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
    double wsum;
    int wcnt;
    __device__ void init(int p, int first) {
        double a = 2.0 / ((double)p + 1.0);
        alpha = (float)a;
        beta = (float)(1.0 - a);
        f = first; s = first + p - 1; warm = first;
        wsum = 0.0; wcnt = 0;
    }
    template <class In> __device__ void accum(const In& in, int t) {
        float v = in.X(t);
        if (t == f || isfinite(v)) { wsum += (double)v; wcnt += 1; }
    }
    __device__ float cur_mean() const { return (float)wsum / (float)wcnt; }
    __device__ void seed() { y = cur_mean(); }
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        if (isfinite(v)) { y = fmaf(beta, y, alpha * v); return 1; }
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
            y = fmaf(beta, y, alpha * v);
            ++applied;
            return y;
        }
        const bool ok = isfinite(v);
        y = ok ? fmaf(beta, y, alpha * v) : y;
        applied += ok;
        return y;
    }
    static __device__ void propagate(double* S, double n, int p) {
        double b = 1.0 - 2.0 / ((double)p + 1.0);
        S[0] *= pow(b, n);
    }
};

// DEMA: dema.rs:291-354 (x86 mul_add form).  Seed x[f] at f; NaN prefix
// [0, f+p-1); out = 2*e1 - e2.
struct OpDema {
    static constexpr bool kHlc = false;
    static constexpr int NS = 2;
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
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        e1 = fmaf(e1, a, v * alpha);
        e2 = fmaf(e2, a, e1 * alpha);
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
        e1 = fmaf(e1, a, v * alpha);
        e2 = fmaf(e2, a, e1 * alpha);
        ++applied;
        return fmaf(e1, 2.f, -e2);
    }
    static __device__ void propagate(double* S, double n, int p) {
        double al = 2.0 / ((double)p + 1.0);
        double an = pow(1.0 - al, n);
        double s1 = S[0];
        S[0] = an * s1;
        S[1] = an * (S[1] + n * al * s1);
    }
};

// TEMA: tema.rs:228-298.  Three EMAs started at f, f+(p-1), f+2(p-1) exactly
// as the crate staggers them; running from s = f+2(p-1); NaN prefix
// [0, f+3(p-1)); out = 3*e1 - 3*e2 + e3; p == 1 copies x.
struct OpTema {
    static constexpr bool kHlc = false;
    static constexpr int NS = 3;
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
        e1 = e1 * per1 + v * per;
        if (t == start2) { e2 = e1; e2 = e2 * per1 + e1 * per; }
        else if (t > start2) e2 = e2 * per1 + e1 * per;
        if (t == s) { e3 = e2; e3 = e3 * per1 + e2 * per; }
    }
    __device__ void seed() {}
    template <class In> __device__ int step(const In& in, int t) {
        float v = in.X(t);
        if (p1 == 0) { e1 = v; return 1; }
        e1 = e1 * per1 + v * per;
        e2 = e2 * per1 + e1 * per;
        e3 = e3 * per1 + e2 * per;
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
        e1 = e1 * per1 + v * per;
        e2 = e2 * per1 + e1 * per;
        e3 = e3 * per1 + e2 * per;
        return 3.f * e1 - 3.f * e2 + e3;
    }
    __device__ float get(int i) const { return i == 0 ? e1 : (i == 1 ? e2 : e3); }
    __device__ void set(int i, float v) { if (i == 0) e1 = v; else if (i == 1) e2 = v; else e3 = v; }
    static __device__ void propagate(double* S, double n, int p) {
        if (p == 1) { S[0] = 0.0; return; }  // p==1 carries nothing (out = x)
        double al = 2.0 / ((double)p + 1.0);
        double an = pow(1.0 - al, n);
        double s1 = S[0], s2 = S[1], s3 = S[2];
        double c2 = n * (n - 1.0) * 0.5;
        S[0] = an * s1;
        S[1] = an * (n * al * s1 + s2);
        S[2] = an * ((n * al * al + c2 * al * al) * s1 + n * al * s2 + s3);
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
    float inv_p, beta, ag, al, xprev;
    int f, s, warm;
    double sg, sl;
    bool wnan;
    __device__ void init(int p, int first) {
        double ip = 1.0 / (double)p;
        inv_p = (float)ip;
        beta = (float)(1.0 - ip);
        f = first; s = first + p; warm = s;
        sg = 0.0; sl = 0.0; wnan = false;
    }
    template <class In> __device__ void accum(const In& in, int t) {
        float v = in.X(t);
        if (t > f && !wnan) {
            double d = (double)v - (double)xprev;
            if (!isfinite(d)) wnan = true;
            else if (d > 0.0) sg += d;
            else if (d < 0.0) sl -= d;
        }
        xprev = v;
    }
    __device__ void seed() {
        if (wnan) { ag = qnan(); al = qnan(); }
        else { ag = (float)(sg * (double)inv_p); al = (float)(sl * (double)inv_p); }
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
    static __device__ void propagate(double* S, double n, int p) {
        double bn = pow(1.0 - 1.0 / (double)p, n);
        S[0] *= bn;
        S[1] *= bn;
    }
};

// Wilders: wilders.rs:262-322.  Seed = mean of x[f..f+p); y = (x-y)*a + y;
// NaN prefix [0, f+p-1); p == 1 copies x.
struct OpWilders {
    static constexpr bool kHlc = false;
    static constexpr int NS = 1;
    float alpha, y;
    int f, s, warm, p;
    double wsum;
    __device__ void init(int p_, int first) {
        p = p_;
        alpha = (float)(1.0 / (double)p);
        f = first; s = first + p - 1; warm = s;
        wsum = 0.0;
    }
    template <class In> __device__ void accum(const In& in, int t) { wsum += (double)in.X(t); }
    __device__ void seed() { y = (float)(wsum * (1.0 / (double)p)); }
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
    static __device__ void propagate(double* S, double n, int p) {
        S[0] = (p == 1) ? 0.0 : S[0] * pow(1.0 - 1.0 / (double)p, n);
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
    double wsum;
    __device__ void init(int p_, int first) {
        p = p_;
        alpha = (float)(1.0 / (double)p);
        f = first; s = first + p - 1; warm = s;
        wsum = 0.0;
    }
    template <class In> __device__ void accum(const In& in, int t) {
        float hi = in.H(t), lo = in.L(t);
        if (t == f) wsum += (double)hi - (double)lo;
        else wsum += (double)true_range(hi, lo, in.C(t - 1));
    }
    __device__ void seed() { y = (float)(wsum / (double)p); }
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
    static __device__ void propagate(double* S, double n, int p) {
        S[0] *= pow(1.0 - 1.0 / (double)p, n);
    }
};

// ------------------------------------------------------------ kernels ------
enum { PASS_AGG = 0, PASS_EMIT = 1 };
constexpr float kBeforeSeed = -2.f, kAbsolute = -1.f;

__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// One warp = 32 lanes x one time chunk.  Tiles of 32 steps where every lane
// of the warp is past its seed and warm-up take the fast path (no phase
// checks: 2-6 FP ops per step); the few tiles around warm-up take the general
// per-step state machine.
// The 32 steps of one register tile, fully unrolled so every shuffle source
// lane is a constant; EMIT stages the outputs in this lane's row.
template <bool FIN, int PASS, class Op>
__device__ __forceinline__ void run_tile(Op& op, const InTile& ti, float* row, int& steps) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const float y = op.template fast<FIN>(ti, ti.tb + j, steps);
        if (PASS == PASS_EMIT) row[j] = y;
    }
}

template <class Op, bool TM, int PASS>
__global__ void __launch_bounds__(kWarps * 32)
k_recur(RecurArgs a) {
    __shared__ float stage[kWarps][32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int group = blockIdx.x * kWarps + warp;
    const int li = group * 32 + lane;
    const bool valid = li < a.n_lanes;
    const int chunk = blockIdx.y;
    const int c0 = chunk * a.chunk;
    const int c1 = min(c0 + a.chunk, a.n);
    if (c0 >= a.n) return;
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
    for (int tb = c0; tb < c1; tb += 32) {
        const int te = min(tb + 32, c1);
        if (tb >= warp_run_from) {
            // ---- fast path: every lane running and past warm-up
            if (!TM && te - tb == 32) {
                // the tile's inputs in registers, one coalesced load per lane
                InTile ti;
                ti.tb = tb;
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
                if (fin) run_tile<true, PASS>(op, ti, stage[warp][lane], steps);
                else run_tile<false, PASS>(op, ti, stage[warp][lane], steps);
            } else if (PASS == PASS_EMIT && !TM) {
#pragma unroll 8
                for (int t = tb; t < te; ++t) stage[warp][lane][t - tb] = op.fast(in, t, steps);
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
            // ---- general path
            for (int t = tb; t < te; ++t) {
                float v = qnan();
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
                if (PASS == PASS_EMIT) {
                    if (TM) {
                        if (valid) a.out[(size_t)t * a.cols + li] = v;
                    } else {
                        stage[warp][lane][t - tb] = v;
                    }
                }
            }
        }
        if (PASS == PASS_EMIT && !TM) {
            __syncwarp();
            const int row0 = group * 32;
            const int t = tb + lane;
            if (t < te) {
                float* o = a.out + (size_t)row0 * a.n + t;
                const int rows = min(32, a.n_lanes - row0);
#pragma unroll 4
                for (int r = 0; r < rows; ++r) o[(size_t)r * a.n] = stage[warp][r][lane];
            }
            __syncwarp();
        }
    }
    if (PASS == PASS_AGG && valid) {
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
}

// Carry-in of every chunk: an exclusive scan, over the chunks of one lane, of
// the affine chunk maps S -> M_k S + b_k (f64).  One warp per lane: each
// thread composes a contiguous run of chunks, a Kogge-Stone scan across the
// warp combines the runs, then each thread re-walks its run writing carries.
struct Aff {
    double m[3][3];
    double b[3];
};

__device__ __forceinline__ void aff_identity(Aff& a) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) a.m[r][c] = r == c ? 1.0 : 0.0;
        a.b[r] = 0.0;
    }
}
// returns second o first (apply `first`, then `second`)
__device__ __forceinline__ Aff aff_then(const Aff& first, const Aff& second) {
    Aff o;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
            o.m[r][c] = second.m[r][0] * first.m[0][c] + second.m[r][1] * first.m[1][c] + second.m[r][2] * first.m[2][c];
        o.b[r] = second.m[r][0] * first.b[0] + second.m[r][1] * first.b[1] + second.m[r][2] * first.b[2] + second.b[r];
    }
    return o;
}
__device__ __forceinline__ Aff aff_shfl_up(const Aff& a, int d) {
    Aff o;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) o.m[r][c] = __shfl_up_sync(0xffffffffu, a.m[r][c], d);
        o.b[r] = __shfl_up_sync(0xffffffffu, a.b[r], d);
    }
    return o;
}

template <class Op>
__device__ void chunk_map(const float4 g, int p, int chunk, const double (&ml)[3][3], Aff& a) {
    if (g.w == kBeforeSeed) {
        aff_identity(a);
        return;
    }
    if (g.w == kAbsolute) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) a.m[r][c] = 0.0;
    } else if (g.w == (float)chunk) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) a.m[r][c] = ml[r][c];
    } else {
        for (int c = 0; c < 3; ++c) {
            double e[3] = {0.0, 0.0, 0.0};
            e[c] = 1.0;
            Op::propagate(e, (double)g.w, p);
            for (int r = 0; r < 3; ++r) a.m[r][c] = e[r];
        }
    }
    a.b[0] = g.x;
    a.b[1] = g.y;
    a.b[2] = g.z;
}

template <class Op>
__global__ void k_recur_carry(RecurArgs a, int n_chunks) {
    const int lane = threadIdx.x & 31;
    const int li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // one warp per lane of the scan
    if (li >= a.n_lanes) return;
    const int p = a.layout ? a.period : a.periods[li];
    double ml[3][3];  // transition of a full chunk
    for (int c = 0; c < 3; ++c) {
        double e[3] = {0.0, 0.0, 0.0};
        e[c] = 1.0;
        Op::propagate(e, (double)a.chunk, p);
        for (int r = 0; r < 3; ++r) ml[r][c] = e[r];
    }
    const float4* agg = reinterpret_cast<const float4*>(a.agg);
    float4* carry = reinterpret_cast<float4*>(a.carry);
    const int per = (n_chunks + 31) / 32;
    const int k0 = min(lane * per, n_chunks), k1 = min(k0 + per, n_chunks);
    Aff run;
    aff_identity(run);
    for (int k = k0; k < k1; ++k) {
        Aff ak;
        chunk_map<Op>(agg[(size_t)k * a.n_lanes + li], p, a.chunk, ml, ak);
        run = aff_then(run, ak);
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const Aff up = aff_shfl_up(run, d);
        if (lane >= d) run = aff_then(up, run);
    }
    Aff ex = aff_shfl_up(run, 1);
    if (lane == 0) aff_identity(ex);
    double S[3] = {ex.b[0], ex.b[1], ex.b[2]};  // state at the start of chunk k0
    for (int k = k0; k < k1; ++k) {
        carry[(size_t)k * a.n_lanes + li] = make_float4((float)S[0], (float)S[1], (float)S[2], 0.f);
        Aff ak;
        chunk_map<Op>(agg[(size_t)k * a.n_lanes + li], p, a.chunk, ml, ak);
        double t[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) t[r] = ak.m[r][0] * S[0] + ak.m[r][1] * S[1] + ak.m[r][2] * S[2] + ak.b[r];
        S[0] = t[0]; S[1] = t[1]; S[2] = t[2];
    }
}

template <class Op, bool TM>
vta_status run(const RecurArgs& a, cudaStream_t st) {
    const int n_chunks = (int)ceil_div(a.n, a.chunk);
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
