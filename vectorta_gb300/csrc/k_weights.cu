// Per-combo weight rows of the weighted-window moving averages, generated on
// the device and right-aligned into a [n_combos][kmax] f32 matrix
// (zero-padded on the left), normalised so each row sums to one.
//
// Weight definitions follow the crate:
//   ALMA   w_i = exp(-(i - m)^2 / (2 s^2)), m = offset (p-1), s = p / sigma
//          (alma.rs:1426-1437)
//   WMA    w_i = (i + 1) / (p (p + 1) / 2)                       (wma.rs:295-336)
//   SWMA   symmetric triangle = box(a) * box(b)        (swma.rs:320-400, 406-482)
//   PWMA   binomial row C(p-1, r) / sum                  (pwma.rs:1367-1408)
//   SINWMA w_k = sin((k+1) pi / (p+1)) / sum             (sinwma.rs:271-289)
//   TRIMA  box(m1) * box(m2), m1 = (p+1)/2, m2 = p - m1 + 1 (trima.rs:277-364)
//
// Arithmetic: GB300's FP64 rate is a small fraction of its FP32 rate, so the
// per-combo constants (ALMA's centre m and 1/(2 s^2)) come in f64 from the
// host and the rest is FP32.  Each weight is evaluated in
// double-single FP32 (error-free products through FMA): the ALMA exponent
// e = (i - m)^2 / (2 s^2) is carried as e_hi + e_lo and exponentiated as
// expf(-e_hi) * (1 - e_lo), and the row sum is accumulated as a double-single
// value, so the stored f32 weights stay within ~2 ulp of the f64 ones.
#include "vta_internal.h"

namespace vta {

namespace {

constexpr int kWThreads = 256;

struct DS {
    float hi, lo;
};

__device__ __forceinline__ DS two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ DS quick_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ DS ds_add(DS a, DS b) {
    const DS s = two_sum(a.hi, b.hi);
    return quick_two_sum(s.hi, s.lo + a.lo + b.lo);
}
__device__ __forceinline__ DS ds_mul(DS a, DS b) {
    const float p = a.hi * b.hi;
    const float e = fmaf(a.hi, b.hi, -p);
    return quick_two_sum(p, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e)));
}
__device__ __forceinline__ DS split(double v) {
    const float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}

struct RowConst {
    DS m;        // ALMA centre offset (p - 1)
    DS inv2s2;   // ALMA 1 / (2 s^2) = sigma^2 / (2 p^2)
    double pw;   // VPWMA power
};

__device__ DS raw_weight(int kind, int i, int p, const RowConst& rc) {
    switch (kind) {
        case WT_ALMA: {
            const DS d = ds_add(DS{(float)i, 0.f}, DS{-rc.m.hi, -rc.m.lo});
            const DS e = ds_mul(ds_mul(d, d), rc.inv2s2);
            const float w = expf(-e.hi);
            return {w, -w * e.lo};
        }
        case WT_WMA: return {(float)(i + 1), 0.f};
        case WT_SWMA: {
            int aa, bb;
            if (p & 1) { aa = bb = (p + 1) >> 1; }
            else { aa = p >> 1; bb = aa + 1; }
            return {(float)min(min(i + 1, p - i), min(aa, bb)), 0.f};
        }
        case WT_PWMA: {
            // binomial C(p-1, r): integer-valued, exact in f64 up to 2^53
            const int n = p - 1;
            const int r = min(i, n - i);
            double res = 1.0;
            for (int k = 0; k < r; ++k) {
                res *= (double)(n - k);
                res /= (double)(k + 1);
            }
            return split(res);
        }
        case WT_SINWMA: return {sinpif((float)(i + 1) / (float)(p + 1)), 0.f};
        case WT_TRIMA: {
            const int m1 = (p + 1) / 2, m2 = p - m1 + 1;
            return {(float)min(min(i + 1, p - i), min(m1, m2)), 0.f};
        }
        // the rest have window L = p (FWMA) or L = period - 1 (the others),
        // oldest first; p here is L
        case WT_CWMA: {  // (k + 2)^3, cwma.rs:246-252
            const double v = (double)(i + 2);
            return split(v * v * v);
        }
        case WT_SQWMA: {  // (k + 2)^2, sqwma.rs:222-225
            const double v = (double)(i + 2);
            return split(v * v);
        }
        case WT_SRWMA: {  // sqrt(k + 2), srwma.rs:207-211; residual by FMA
            const float v = (float)(i + 2);
            const float r = sqrtf(v);
            return {r, fmaf(-r, r, v) / (2.f * r)};
        }
        case WT_FWMA: {
            // Fibonacci F(k+1) (fwma.rs:321-331) relative to F(L): by Binet,
            // phi^(k+1-L) * (1 - (-1)^(k+1) phi^(-2(k+1))); the exponent is
            // formed as a double-single product so the ratio of weights keeps
            // f32 precision for windows of any length
            const DS l2phi = rc.m;  // log2(phi) as double-single
            const float e = (float)(i + 1 - p);
            const DS ex = ds_mul(DS{e, 0.f}, l2phi);
            float w = exp2f(ex.hi);
            w = fmaf(w, ex.lo * 0.69314718f, w);
            const DS ey = ds_mul(DS{-2.f * (float)(i + 1), 0.f}, l2phi);
            const float alt = exp2f(ey.hi) * (((i + 1) & 1) ? -1.f : 1.f);
            return {w * (1.f - alt), 0.f};
        }
        case WT_EPMA: {  // c0 + k with c0 = 2 - offset, epma.rs:346-366
            return {(float)(i + 2) - rc.inv2s2.hi, 0.f};
        }
        case WT_VPWMA: {  // (k + 2)^power, vpwma.rs:247-256 (f64 pow, once per weight)
            return split(pow((double)(i + 2), rc.pw));
        }
    }
    return {0.f, 0.f};
}

// One warp per combo (kWThreads / 32 combos per block): raw weights summed in
// double-single across the lanes, then a second pass writes raw * (1 / sum).
// The per-combo f64 constants and the reciprocal are formed by lane 0 only.
__global__ void __launch_bounds__(kWThreads) k_weights(int kind, const int* periods, const double* pa,
                                                       const double* pb, int n_combos, int kmax, float* w) {
    const int lane = threadIdx.x & 31;
    const int c = blockIdx.x * (kWThreads / 32) + (threadIdx.x >> 5);
    if (c >= n_combos) return;  // whole warp (no block-wide barrier below)
    const int p = periods[c];
    RowConst rc{};
    if (kind == WT_FWMA) {
        rc.m = split(0.69424191363061730173879026);  // log2 of the golden ratio
    } else if (kind == WT_EPMA) {
        rc.inv2s2 = DS{(float)pa[c], 0.f};  // the offset (an integer)
    } else if (kind == WT_VPWMA) {
        rc.pw = pa[c];
    } else if (kind == WT_ALMA) {
        // pa = m = offset (p - 1) and pb = 1 / (2 s^2) = sigma^2 / (2 p^2),
        // formed in f64 on the host (an f64 divide per combo on the device
        // cost more than the whole weight row)
        float m_hi = 0.f, m_lo = 0.f, q_hi = 0.f, q_lo = 0.f;
        if (lane == 0) {
            const DS m = split(pa[c]);
            const DS q = split(pb[c]);
            m_hi = m.hi; m_lo = m.lo; q_hi = q.hi; q_lo = q.lo;
        }
        rc.m = DS{__shfl_sync(0xffffffffu, m_hi, 0), __shfl_sync(0xffffffffu, m_lo, 0)};
        rc.inv2s2 = DS{__shfl_sync(0xffffffffu, q_hi, 0), __shfl_sync(0xffffffffu, q_lo, 0)};
    }
    DS s{0.f, 0.f};
    for (int i = lane; i < p; i += 32) s = ds_add(s, raw_weight(kind, i, p, rc));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const DS t{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)};
        s = ds_add(s, t);
    }
    // 1 / sum in double-single: r0 = 1 / hi, one Newton step on the residual
    // 1 - sum r0 (formed exactly with FMA), so inv = r0 + r0 e to ~1e-14
    const float r0 = 1.f / s.hi;
    const float e = fmaf(-s.lo, r0, fmaf(-s.hi, r0, 1.f));
    const DS inv = quick_two_sum(r0, r0 * e);
    float* row = w + (size_t)c * kmax;
    const int lead = kmax - p;
    for (int k = lane; k < kmax; k += 32) {
        const int i = k - lead;
        float v = 0.f;
        if (i >= 0) {
            const DS r = ds_mul(raw_weight(kind, i, p, rc), inv);
            v = r.hi + r.lo;
        }
        row[k] = v;
    }
}

}  // namespace

vta_status launch_weights(int kind, const int* periods, const double* pa, const double* pb, int n_combos,
                          int kmax, float* w, cudaStream_t st) {
    k_weights<<<ceil_div(n_combos, kWThreads / 32), kWThreads, 0, st>>>(kind, periods, pa, pb, n_combos, kmax, w);
    return check_launch("k_weights");
}

}  // namespace vta
