/*
 * vta_oracle.c -- CPU oracle for the VectorTA indicator hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * VectorTA crate's scalar f64 CPU paths (the src/indicators/ Rust files, the
 * `Kernel::Scalar` / `Kernel::ScalarBatch` row functions).  It is used by the
 * test-suite, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg
 * as the checker.  The product (vectorta_gb300/) never links or calls it.
 *
 * Arithmetic rules followed so results match the Rust code bit for bit on the
 * same host libm:
 *   - compiled with -ffp-contract=off (Rust never contracts a*b+c);
 *   - fma() exactly where the Rust source calls f64::mul_add;
 *   - the same summation order / unrolling as the cited row function;
 *   - fmax/fmin where the Rust calls f64::max/min (NaN-ignoring semantics).
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the VectorTA project root).  Status codes: 0 ok, otherwise a VTO_E* code.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define VTO_OK 0
#define VTO_E_EMPTY 1
#define VTO_E_ALL_NAN 2
#define VTO_E_INVALID_PERIOD 3
#define VTO_E_NOT_ENOUGH_VALID 4
#define VTO_E_INVALID_PARAM 5
#define VTO_E_INVALID_RANGE 6
#define VTO_E_NOT_ENOUGH_DATA 7

static const double QNAN = __builtin_nan("");

static size_t first_valid(const double *x, size_t n) {
    size_t i = 0;
    while (i < n && isnan(x[i])) i++;
    return i;
}

static void fill_nan(double *o, size_t n) {
    for (size_t i = 0; i < n; i++) o[i] = QNAN;
}

/* ------------------------------------------------------------------------ */
/* Parameter-grid expansion.                                                  */
/* Ascending ranges are identical across the crate; descending ranges differ  */
/* per indicator, so the mode is explicit.                                    */
/* ------------------------------------------------------------------------ */
enum {
    VTO_AX_DESC = 0,     /* start, start-step, ... while >= end
                            (alma.rs:1199-1222, dema.rs:780-809, sma.rs:705-...) */
    VTO_AX_SWAP = 1,     /* descending swapped to ascending
                            (ema.rs:691-702, rsi.rs:513-542, trima.rs:1024-1049) */
    VTO_AX_REV_FROM_END = 2, /* (end..=start).step_by(step) reversed (atr.rs:917-936) */
    VTO_AX_DESC_PLUS_END = 3 /* DESC then `end` appended if missing (wma.rs:552-576) */
};

/* Returns the number of values written (<= cap) or the count needed when out
 * is NULL.  0 means an empty (invalid) range. */
size_t vto_axis_usize(size_t start, size_t end, size_t step, int mode,
                      size_t *out, size_t cap) {
    size_t n = 0;
#define PUSH(v)                            \
    do {                                   \
        if (out && n < cap) out[n] = (v);  \
        n++;                               \
    } while (0)
    if (step == 0 || start == end) {
        PUSH(start);
        return n;
    }
    if (start < end) {
        for (size_t v = start; v <= end; v += step) {
            PUSH(v);
            if (v > (size_t)-1 - step) break;
        }
        return n;
    }
    switch (mode) {
    case VTO_AX_SWAP:
        for (size_t v = end; v <= start; v += step) {
            PUSH(v);
            if (v > (size_t)-1 - step) break;
        }
        break;
    case VTO_AX_REV_FROM_END: {
        size_t cnt = (start - end) / step + 1;
        for (size_t k = cnt; k-- > 0;) PUSH(end + k * step);
        break;
    }
    case VTO_AX_DESC_PLUS_END:
    case VTO_AX_DESC:
    default: {
        size_t v = start, last = start;
        for (;;) {
            PUSH(v);
            last = v;
            if (v < end + step) break; /* next would drop below end */
            v -= step;
        }
        if (mode == VTO_AX_DESC_PLUS_END && last != end) PUSH(end);
        break;
    }
    }
#undef PUSH
    return n;
}

/* f64 axis with the crate's 1e-12 slack and accumulated x += step
 * (alma.rs:1224-1260; same in stddev.rs:721, bollinger_bands.rs:1250,
 * percentile_nearest_rank.rs:945, supertrend.rs:1253, zscore.rs:964). */
size_t vto_axis_f64(double start, double end, double step, double *out, size_t cap) {
    size_t n = 0;
    if (fabs(step) < 1e-12 || fabs(start - end) < 1e-12) {
        if (out && cap) out[0] = start;
        return 1;
    }
    double st = fabs(step);
    if (start < end) {
        for (double x = start; x <= end + 1e-12; x += st) {
            if (out && n < cap) out[n] = x;
            n++;
        }
    } else {
        for (double x = start; x + 1e-12 >= end; x -= st) {
            if (out && n < cap) out[n] = x;
            n++;
        }
    }
    return n;
}

/* ------------------------------------------------------------------------ */
/* ALMA                                                                       */
/* ------------------------------------------------------------------------ */

/* alma_prepare weights (alma.rs:315-332): w_i = exp(-diff*diff*inv_s2). */
static void alma_weights_single(size_t period, double offset, double sigma,
                                double *w, double *inv_norm) {
    double m = offset * (double)(period - 1);
    double s = (double)period / sigma;
    double s2 = 2.0 * s * s;
    double inv_s2 = 1.0 / s2;
    double norm = 0.0;
    for (size_t i = 0; i < period; i++) {
        double diff = (double)i - m;
        double wi = exp(-diff * diff * inv_s2);
        w[i] = wi;
        norm += wi;
    }
    *inv_norm = 1.0 / norm;
}

/* Batch weights (alma.rs:1426-1437): w = exp(-(i-m).powi(2) / s2). */
void vto_alma_weights_batch(size_t period, double offset, double sigma,
                            double *w, double *inv_norm) {
    double m = offset * (double)(period - 1);
    double s = (double)period / sigma;
    double s2 = 2.0 * s * s;
    double norm = 0.0;
    for (size_t i = 0; i < period; i++) {
        double d = (double)i - m;
        double wi = exp(-(d * d) / s2);
        w[i] = wi;
        norm += wi;
    }
    *inv_norm = 1.0 / norm;
}

/* alma_scalar / alma_row_scalar (alma.rs:426-463, alma.rs:1505-1527):
 * 4-wide unrolled dot, sum += ((d0w0 + d1w1) + d2w2) + d3w3, no FMA. */
static void alma_row(const double *x, size_t n, size_t first, size_t period,
                     const double *w, double inv_n, double *out) {
    size_t p4 = period & ~(size_t)3;
    for (size_t i = first + period - 1; i < n; i++) {
        size_t start = i + 1 - period;
        double sum = 0.0;
        for (size_t k = 0; k < p4; k += 4) {
            const double *d = x + start + k;
            sum += d[0] * w[k] + d[1] * w[k + 1] + d[2] * w[k + 2] + d[3] * w[k + 3];
        }
        for (size_t k = p4; k < period; k++) sum += x[start + k] * w[k];
        out[i] = sum * inv_n;
    }
}

/* alma() single series (alma.rs:236-347). */
int vto_alma(const double *x, size_t n, size_t period, double offset, double sigma,
             double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    if (!(sigma > 0.0)) return VTO_E_INVALID_PARAM;
    if (!(offset >= 0.0 && offset <= 1.0)) return VTO_E_INVALID_PARAM;
    double *w = (double *)malloc(sizeof(double) * period);
    double inv_n;
    alma_weights_single(period, offset, sigma, w, &inv_n);
    fill_nan(out, first + period - 1);
    alma_row(x, n, first, period, w, inv_n, out);
    free(w);
    return VTO_OK;
}

/* alma_batch_with_kernel(ScalarBatch) row semantics (alma.rs:1368-1527).
 * periods/offsets/sigmas give the expanded grid (period-major). */
int vto_alma_batch(const double *x, size_t n, size_t rows, const size_t *periods,
                   const double *offsets, const double *sigmas, double *out) {
    if (n == 0) return VTO_E_ALL_NAN;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    size_t max_p = 0;
    for (size_t r = 0; r < rows; r++) {
        size_t p8 = (periods[r] + 7) & ~(size_t)7;
        if (p8 > max_p) max_p = p8;
    }
    if (n - first < max_p) return VTO_E_NOT_ENOUGH_VALID;
    double *w = (double *)malloc(sizeof(double) * (max_p ? max_p : 1));
    for (size_t r = 0; r < rows; r++) {
        size_t p = periods[r];
        if (!(sigmas[r] > 0.0)) { free(w); return VTO_E_INVALID_PARAM; }
        if (!(offsets[r] >= 0.0 && offsets[r] <= 1.0)) { free(w); return VTO_E_INVALID_PARAM; }
        double inv_n;
        vto_alma_weights_batch(p, offsets[r], sigmas[r], w, &inv_n);
        double *o = out + r * n;
        fill_nan(o, first + p - 1);
        alma_row(x, n, first, p, w, inv_n, o);
    }
    free(w);
    return VTO_OK;
}

/* One row of vto_alma_batch evaluated only at the end indices idx[0..nidx)
 * (same batch weights, same 4-wide dot as alma_row; NaN before the row's
 * warm-up end first + p - 1).  Lets a test check every row of a large grid
 * on a time sample without computing the whole row. */
int vto_alma_batch_row_at(const double *x, size_t n, size_t period, double offset, double sigma,
                          const size_t *idx, size_t nidx, double *out) {
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    double *w = (double *)malloc(sizeof(double) * period);
    double inv_n;
    vto_alma_weights_batch(period, offset, sigma, w, &inv_n);
    size_t p4 = period & ~(size_t)3;
    for (size_t k = 0; k < nidx; k++) {
        size_t i = idx[k];
        if (i >= n) { free(w); return VTO_E_INVALID_RANGE; }
        if (i < first + period - 1) { out[k] = QNAN; continue; }
        size_t start = i + 1 - period;
        double sum = 0.0;
        for (size_t j = 0; j < p4; j += 4) {
            const double *d = x + start + j;
            sum += d[0] * w[j] + d[1] * w[j + 1] + d[2] * w[j + 2] + d[3] * w[j + 3];
        }
        for (size_t j = p4; j < period; j++) sum += x[start + j] * w[j];
        out[k] = sum * inv_n;
    }
    free(w);
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* EMA / DEMA / TEMA                                                          */
/* ------------------------------------------------------------------------ */

static int is_finite_bits(double v) { return isfinite(v); }

/* ema_scalar_into / ema_row_scalar (ema.rs:430-469, ema.rs:858-893).
 * Warmup: running mean over [first, first+p) of finite values; then
 * prev = beta.mul_add(prev, alpha*x), non-finite x skipped.  NaN prefix =
 * first only (ema.rs:362). */
int vto_ema(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    double alpha = 2.0 / ((double)period + 1.0);
    double beta = 1.0 - alpha;
    fill_nan(out, first);
    double mean = x[first];
    out[first] = mean;
    size_t vc = 1;
    size_t wend = first + period < n ? first + period : n;
    for (size_t i = first + 1; i < wend; i++) {
        double v = x[i];
        if (is_finite_bits(v)) {
            vc++;
            double fvc = (double)vc;
            mean = ((fvc - 1.0) * mean + v) / fvc;
        }
        out[i] = mean;
    }
    double prev = mean;
    for (size_t i = wend; i < n; i++) {
        double v = x[i];
        if (is_finite_bits(v)) prev = fma(beta, prev, alpha * v);
        out[i] = prev;
    }
    return VTO_OK;
}

/* dema_scalar, x86_64 variant (dema.rs:291-354): ema1 = ema2 = x[first],
 * ema1 = ema1.mul_add(a, x*alpha); ema2 = ema2.mul_add(a, ema1*alpha);
 * out = ema1.mul_add(2, -ema2).  NaN prefix first+p-1 (dema.rs:235).
 * Needs len-first >= 2(p-1) (dema.rs:215-223). */
static void dema_row(const double *x, size_t n, size_t first, size_t period, double *out) {
    double alpha = 2.0 / ((double)period + 1.0);
    double a = 1.0 - alpha;
    double e1 = x[first], e2 = e1;
    out[first] = e1;
    for (size_t i = first + 1; i < n; i++) {
        e1 = fma(e1, a, x[i] * alpha);
        e2 = fma(e2, a, e1 * alpha);
        out[i] = fma(e1, 2.0, -e2);
    }
    fill_nan(out, first + period - 1);
}

int vto_dema(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period < 1 || period > n) return VTO_E_INVALID_PERIOD;
    size_t needed = 2 * (period - 1);
    if (n < needed) return VTO_E_NOT_ENOUGH_DATA;
    if (n - first < needed) return VTO_E_NOT_ENOUGH_VALID;
    dema_row(x, n, first, period, out);
    return VTO_OK;
}

/* tema_scalar (tema.rs:228-298): three cascaded EMAs started at first,
 * first+(p-1), first+2(p-1); out = 3*e1 - 3*e2 + e3 from first+3(p-1). */
static void tema_row(const double *x, size_t n, size_t first, size_t period, double *out) {
    size_t warm = first + (period - 1) * 3;
    fill_nan(out, warm < n ? warm : n);
    double per = 2.0 / ((double)period + 1.0);
    double per1 = 1.0 - per;
    size_t p1 = period - 1;
    size_t start2 = first + p1, start3 = first + 2 * p1, start_out = first + 3 * p1;
    if (period == 1) {
        for (size_t i = first; i < n; i++) out[i] = x[i];
        return;
    }
    double e1 = x[first], e2 = 0.0, e3 = 0.0;
    size_t end0 = start2 < n ? start2 : n;
    for (size_t i = first; i < end0; i++) e1 = e1 * per1 + x[i] * per;
    if (start2 < n) {
        e1 = e1 * per1 + x[start2] * per;
        e2 = e1;
        e2 = e2 * per1 + e1 * per;
        size_t end1 = start3 < n ? start3 : n;
        for (size_t i = start2 + 1; i < end1; i++) {
            e1 = e1 * per1 + x[i] * per;
            e2 = e2 * per1 + e1 * per;
        }
        if (start3 < n) {
            e1 = e1 * per1 + x[start3] * per;
            e2 = e2 * per1 + e1 * per;
            e3 = e2;
            e3 = e3 * per1 + e2 * per;
            size_t end2 = start_out < n ? start_out : n;
            for (size_t i = start3 + 1; i < end2; i++) {
                e1 = e1 * per1 + x[i] * per;
                e2 = e2 * per1 + e1 * per;
                e3 = e3 * per1 + e2 * per;
            }
            for (size_t i = start_out; i < n; i++) {
                e1 = e1 * per1 + x[i] * per;
                e2 = e2 * per1 + e1 * per;
                e3 = e3 * per1 + e2 * per;
                out[i] = 3.0 * e1 - 3.0 * e2 + e3;
            }
        }
    }
}

/* tema_prepare (tema.rs:1396-1435). */
int vto_tema(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    tema_row(x, n, first, period, out);
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* RSI / Wilders                                                              */
/* ------------------------------------------------------------------------ */

static double rsi_val(double g, double l) {
    double d = g + l;
    return d == 0.0 ? 50.0 : 100.0 * g / d;
}

/* rsi_compute_into_scalar (rsi.rs:327-414).  Single-series path: a NaN delta
 * in the warmup poisons the row; later NaN deltas count as 0 gain/loss. */
int vto_rsi(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm = first + period;
    fill_nan(out, warm < n ? warm : n);
    double inv_p = 1.0 / (double)period, beta = 1.0 - inv_p;
    double ag = 0.0, al = 0.0;
    int has_nan = 0;
    size_t warm_last = first + period < n - 1 ? first + period : (n ? n - 1 : 0);
    for (size_t i = first + 1; i <= warm_last; i++) {
        double d = x[i] - x[i - 1];
        if (!isfinite(d)) { has_nan = 1; break; }
        if (d > 0.0) ag += d;
        else if (d < 0.0) al -= d;
    }
    size_t idx0 = first + period;
    if (has_nan) {
        ag = QNAN; al = QNAN;
        if (idx0 < n) out[idx0] = QNAN;
    } else {
        ag *= inv_p; al *= inv_p;
        if (idx0 < n) out[idx0] = rsi_val(ag, al);
    }
    for (size_t j = idx0 + 1; j < n; j++) {
        double d = x[j] - x[j - 1];
        double g = d > 0.0 ? d : 0.0;
        double l = d < 0.0 ? -d : 0.0;
        ag = fma(ag, beta, inv_p * g);
        al = fma(al, beta, inv_p * l);
        out[j] = rsi_val(ag, al);
    }
    return VTO_OK;
}

/* rsi_batch_inner (rsi.rs:568-697): shared gains/losses (NaN for non-finite
 * deltas, so any later NaN delta poisons the row) and prefix sums pg/pl; the
 * warmup average is (pg[idx0]-pg[first])*inv_p. */
int vto_rsi_batch(const double *x, size_t n, size_t rows, const size_t *periods, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    size_t max_p = 0;
    for (size_t r = 0; r < rows; r++) if (periods[r] > max_p) max_p = periods[r];
    if (n - first < max_p) return VTO_E_NOT_ENOUGH_VALID;
    double *gains = (double *)calloc(n, sizeof(double));
    double *losses = (double *)calloc(n, sizeof(double));
    double *pg = (double *)calloc(n, sizeof(double));
    double *pl = (double *)calloc(n, sizeof(double));
    for (size_t i = first + 1; i < n; i++) {
        double d = x[i] - x[i - 1];
        if (isfinite(d)) {
            if (d > 0.0) gains[i] = d;
            else if (d < 0.0) losses[i] = -d;
        } else {
            gains[i] = QNAN; losses[i] = QNAN;
        }
    }
    for (size_t i = 1; i < n; i++) {
        pg[i] = pg[i - 1] + gains[i];
        pl[i] = pl[i - 1] + losses[i];
    }
    for (size_t r = 0; r < rows; r++) {
        size_t period = periods[r];
        double *o = out + r * n;
        size_t idx0 = first + period;
        fill_nan(o, idx0 < n ? idx0 : n);
        if (idx0 >= n) continue;
        double inv_p = 1.0 / (double)period, beta = 1.0 - inv_p;
        double sg = pg[idx0] - pg[first], sl = pl[idx0] - pl[first];
        double ag = sg * inv_p, al = sl * inv_p;
        if (isnan(sg) || isnan(sl)) {
            ag = QNAN; al = QNAN; o[idx0] = QNAN;
        } else {
            o[idx0] = rsi_val(ag, al);
        }
        for (size_t j = idx0 + 1; j < n; j++) {
            ag = fma(ag, beta, inv_p * gains[j]);
            al = fma(al, beta, inv_p * losses[j]);
            o[j] = rsi_val(ag, al);
        }
    }
    free(gains); free(losses); free(pg); free(pl);
    return VTO_OK;
}

/* wilders_scalar (wilders.rs:262-322): seed = mean of the first p values
 * (4-way chunked sum), then y = (x - y).mul_add(alpha, y).  The first p values
 * must be finite (wilders.rs:223-230). */
int vto_wilders(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    for (size_t i = 0; i < period; i++)
        if (!isfinite(x[first + i])) return VTO_E_NOT_ENOUGH_VALID;
    size_t ws = first + period - 1;
    fill_nan(out, ws);
    const double *p = x + first;
    double sum = 0.0;
    size_t c4 = period / 4;
    for (size_t c = 0; c < c4; c++, p += 4) sum += p[0] + p[1] + p[2] + p[3];
    switch (period - c4 * 4) {
    case 3: sum += p[0] + p[1] + p[2]; break;
    case 2: sum += p[0] + p[1]; break;
    case 1: sum += p[0]; break;
    default: break;
    }
    double inv_n = 1.0 / (double)period;
    double y = sum * inv_n;
    out[ws] = y;
    if (period == 1) {
        for (size_t i = ws + 1; i < n; i++) out[i] = x[i];
        return VTO_OK;
    }
    for (size_t i = ws + 1; i < n; i++) {
        y = fma(x[i] - y, inv_n, y);
        out[i] = y;
    }
    return VTO_OK;
}

/* wilders_batch_inner_into (wilders.rs:997-1110): seed from a prefix sum of
 * data[first..] (sum = pref[period] - pref[0]); rows otherwise as scalar. */
int vto_wilders_batch(const double *x, size_t n, size_t rows, const size_t *periods, double *out) {
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    size_t max_p = 0;
    for (size_t r = 0; r < rows; r++) if (periods[r] > max_p) max_p = periods[r];
    if (n - first < max_p) return VTO_E_NOT_ENOUGH_VALID;
    double *pref = (double *)malloc(sizeof(double) * (n - first + 1));
    pref[0] = 0.0;
    double acc = 0.0;
    for (size_t i = first; i < n; i++) { acc += x[i]; pref[i - first + 1] = acc; }
    for (size_t r = 0; r < rows; r++) {
        size_t period = periods[r];
        double *o = out + r * n;
        size_t ws = first + period - 1;
        fill_nan(o, ws);
        double sum = pref[period] - pref[0];
        double inv_n = 1.0 / (double)period;
        double y = sum * inv_n;
        o[ws] = y;
        if (period == 1) {
            for (size_t i = ws + 1; i < n; i++) o[i] = x[i];
            continue;
        }
        for (size_t i = ws + 1; i < n; i++) {
            y = fma(x[i] - y, inv_n, y);
            o[i] = y;
        }
    }
    free(pref);
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* ATR / ADX / SuperTrend                                                     */
/* ------------------------------------------------------------------------ */

static size_t first_valid_hlc(const double *h, const double *l, const double *c, size_t n) {
    size_t i = 0;
    while (i < n && (isnan(h[i]) || isnan(l[i]) || isnan(c[i]))) i++;
    return i;
}

/* atr_compute_into_scalar (atr.rs:329-460): seed = mean TR over
 * [first, first+len), TR(first) = h-l; rma = (-alpha).mul_add(rma, rma) +
 * alpha*tr.  NaN prefix first+len-1 (atr.rs:229). */
int vto_atr(const double *h, const double *l, const double *c, size_t n, size_t length,
            double *out) {
    if (n == 0) return VTO_E_EMPTY;
    if (length == 0) return VTO_E_INVALID_PERIOD;
    size_t first = first_valid_hlc(h, l, c, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (n - first < length) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm = first + length - 1;
    fill_nan(out, warm);
    double alpha = 1.0 / (double)length;
    double sum_tr = h[first] - l[first];
    if (warm > first) {
        double pc = c[first];
        for (size_t i = first + 1; i <= warm; i++) {
            double tr = h[i] - l[i];
            double hc = fabs(h[i] - pc);
            if (hc > tr) tr = hc;
            double lc = fabs(l[i] - pc);
            if (lc > tr) tr = lc;
            sum_tr += tr;
            pc = c[i];
        }
    }
    double rma = sum_tr / (double)length;
    out[warm] = rma;
    for (size_t i = warm + 1; i < n; i++) {
        double pc = c[i - 1];
        double tr = h[i] - l[i];
        double hc = fabs(h[i] - pc);
        if (hc > tr) tr = hc;
        double lc = fabs(l[i] - pc);
        if (lc > tr) tr = lc;
        rma = fma(-alpha, rma, rma) + alpha * tr;
        out[i] = rma;
    }
    return VTO_OK;
}

/* adx_scalar on the slices from first (adx.rs:299-421, called at
 * adx.rs:265-272).  first = max of the per-field first valid indices
 * (adx.rs:190-198); needs len-first >= p+1; NaN prefix first+2p-1. */
int vto_adx(const double *h, const double *l, const double *c, size_t n, size_t period,
            double *out) {
    if (n == 0) return VTO_E_EMPTY;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    size_t fh = first_valid(h, n), fl = first_valid(l, n), fc = first_valid(c, n);
    if (fh >= n || fl >= n || fc >= n) return VTO_E_ALL_NAN;
    size_t first = fh > fl ? fh : fl;
    if (fc > first) first = fc;
    if (n - first < period + 1) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm_end = first + 2 * period - 1;
    fill_nan(out, warm_end < n ? warm_end : n);
    const double *H = h + first, *L = l + first, *C = c + first;
    double *O = out + first;
    size_t len = n - first;
    if (len <= period) return VTO_OK;
    double pf = (double)period, rp = 1.0 / pf, omr = 1.0 - rp, pm1 = pf - 1.0;
    double tr_sum = 0.0, pdm_sum = 0.0, mdm_sum = 0.0;
    double ph = H[0], pl = L[0], pc = C[0];
    for (size_t i = 1; i <= period; i++) {
        double ch = H[i], cl = L[i];
        double tr = fmax(fmax(ch - cl, fabs(ch - pc)), fabs(cl - pc));
        double up = ch - ph, down = pl - cl;
        if (up > down && up > 0.0) pdm_sum += up;
        if (down > up && down > 0.0) mdm_sum += down;
        tr_sum += tr;
        ph = ch; pl = cl; pc = C[i];
    }
    double atr = tr_sum, pdm = pdm_sum, mdm = mdm_sum;
    double pdi0 = 0.0, mdi0 = 0.0;
    if (atr != 0.0) { pdi0 = (pdm / atr) * 100.0; mdi0 = (mdm / atr) * 100.0; }
    double sdi0 = pdi0 + mdi0;
    double dx_sum = sdi0 != 0.0 ? (fabs(pdi0 - mdi0) / sdi0) * 100.0 : 0.0;
    size_t dx_count = 1;
    double last_adx = 0.0;
    ph = H[period]; pl = L[period]; pc = C[period];
    for (size_t i = period + 1; i < len; i++) {
        double ch = H[i], cl = L[i];
        double tr = fmax(fmax(ch - cl, fabs(ch - pc)), fabs(cl - pc));
        double up = ch - ph, down = pl - cl;
        double pdmv = (up > down && up > 0.0) ? up : 0.0;
        double mdmv = (down > up && down > 0.0) ? down : 0.0;
        atr = atr * omr + tr;
        pdm = pdm * omr + pdmv;
        mdm = mdm * omr + mdmv;
        double pdi = 0.0, mdi = 0.0;
        if (atr != 0.0) { pdi = (pdm / atr) * 100.0; mdi = (mdm / atr) * 100.0; }
        double sdi = pdi + mdi;
        double dx = sdi != 0.0 ? (fabs(pdi - mdi) / sdi) * 100.0 : 0.0;
        if (dx_count < period) {
            dx_sum += dx;
            dx_count++;
            if (dx_count == period) {
                last_adx = dx_sum * rp;
                O[i] = last_adx;
            }
        } else {
            last_adx = (last_adx * pm1 + dx) * rp;
            O[i] = last_adx;
        }
        ph = ch; pl = cl; pc = C[i];
    }
    return VTO_OK;
}

/* supertrend_prepare + supertrend_scalar (supertrend.rs:223-302,
 * supertrend.rs:457-550).  ATR is taken on the slices from first
 * (atr() on &high[first..] etc.); outputs trend and changed with a NaN prefix
 * first+p-1. */
int vto_supertrend(const double *h, const double *l, const double *c, size_t n,
                   size_t period, double factor, double *trend, double *changed) {
    if (n == 0) return VTO_E_EMPTY;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    size_t first = first_valid_hlc(h, l, c, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t m = n - first;
    double *atr = (double *)malloc(sizeof(double) * m);
    int st = vto_atr(h + first, l + first, c + first, m, period, atr);
    if (st) { free(atr); return st; }
    size_t warm = first + period - 1;
    fill_nan(trend, warm);
    fill_nan(changed, warm);
    size_t start = first + period;
    if (start > n) { free(atr); return VTO_OK; }
    double hl2w = (h[warm] + l[warm]) * 0.5;
    double atrw = atr[period - 1];
    double pub = hl2w + factor * atrw;
    double plb = hl2w - factor * atrw;
    double last_close = c[warm];
    int upper_state;
    if (last_close <= pub) { trend[warm] = pub; upper_state = 1; }
    else { trend[warm] = plb; upper_state = 0; }
    changed[warm] = 0.0;
    size_t ai = warm + 1 - first;
    for (size_t i = warm + 1; i < n; i++, ai++) {
        double a = atr[ai];
        double hl2 = (h[i] + l[i]) * 0.5;
        double ub = fma(factor, a, hl2);
        double lb = fma(-factor, a, hl2);
        double pcl = last_close;
        double cub = ub;
        if (pcl <= pub) cub = fmin(cub, pub);
        double clb = lb;
        if (pcl >= plb) clb = fmax(clb, plb);
        double cc = c[i];
        if (upper_state) {
            if (cc <= cub) { trend[i] = cub; changed[i] = 0.0; }
            else { trend[i] = clb; changed[i] = 1.0; upper_state = 0; }
        } else {
            if (cc >= clb) { trend[i] = clb; changed[i] = 0.0; }
            else { trend[i] = cub; changed[i] = 1.0; upper_state = 1; }
        }
        pub = cub; plb = clb; last_close = cc;
    }
    free(atr);
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* SMA / StdDev / Z-score / Bollinger                                         */
/* ------------------------------------------------------------------------ */

/* sma_scalar (sma.rs:302-330): running sum. */
int vto_sma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    fill_nan(out, first + period - 1);
    if (period == 1) {
        for (size_t i = first; i < n; i++) out[i] = x[i];
        return VTO_OK;
    }
    double sum = 0.0;
    for (size_t k = 0; k < period; k++) sum += x[first + k];
    double inv = 1.0 / (double)period;
    out[first + period - 1] = sum * inv;
    for (size_t i = first + period; i < n; i++) {
        sum += x[i] - x[i - period];
        out[i] = sum * inv;
    }
    return VTO_OK;
}

/* sma_batch_inner_into (sma.rs:909-1020): inclusive prefix ps starting at
 * first; out[i] = (ps[i] - ps[i-p]) * inv. */
int vto_sma_batch(const double *x, size_t n, size_t rows, const size_t *periods, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    size_t max_p = 0;
    for (size_t r = 0; r < rows; r++) if (periods[r] > max_p) max_p = periods[r];
    if (n - first < max_p) return VTO_E_NOT_ENOUGH_VALID;
    double *ps = (double *)calloc(n, sizeof(double));
    ps[first] = x[first];
    for (size_t i = first + 1; i < n; i++) ps[i] = ps[i - 1] + x[i];
    for (size_t r = 0; r < rows; r++) {
        size_t p = periods[r];
        double *o = out + r * n;
        size_t warm = first + p - 1;
        fill_nan(o, warm < n ? warm : n);
        if (warm >= n) continue;
        double inv = 1.0 / (double)p;
        for (size_t i = warm; i < n; i++) {
            double lo = i >= p ? ps[i - p] : 0.0;
            o[i] = (ps[i] - lo) * inv;
        }
    }
    free(ps);
    return VTO_OK;
}

/* stddev_scalar (stddev.rs:358-409): population variance from running sum
 * and sum of squares; var <= 0 -> 0; result * nbdev.  Same for batch rows
 * (stddev.rs:1097-1105). */
static void stddev_row(const double *x, size_t n, size_t first, size_t period, double nbdev,
                       double *out) {
    double inv = 1.0 / (double)period;
    double sum = 0.0, sq = 0.0;
    for (size_t k = 0; k < period; k++) {
        double v = x[first + k];
        sum += v;
        sq += v * v;
    }
    size_t i0 = first + period - 1;
    fill_nan(out, i0);
    double mean = sum * inv;
    double var = (sq * inv) - (mean * mean);
    out[i0] = var <= 0.0 ? 0.0 : sqrt(var) * nbdev;
    for (size_t j = first + period; j < n; j++) {
        double old = x[j - period], nw = x[j];
        sum += nw - old;
        sq += nw * nw - old * old;
        double m = sum * inv;
        double v = (sq * inv) - (m * m);
        out[j] = v <= 0.0 ? 0.0 : sqrt(v) * nbdev;
    }
}

int vto_stddev(const double *x, size_t n, size_t period, double nbdev, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (!isfinite(nbdev) || nbdev < 0.0) return VTO_E_INVALID_PARAM;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    stddev_row(x, n, first, period, nbdev, out);
    return VTO_OK;
}

/* The crate's batch StdDev row (stddev_batch_inner with Kernel::Scalar,
 * stddev.rs:822-1060): f64 prefixes ps, ps2 of x and x^2 and a NaN-count
 * prefix over the WHOLE series (build_std_prefixes, stddev.rs:878-897), then
 * per output sum = ps[i+1] - ps[i+1-p], sum2 likewise and
 * var = sum2.mul_add(1/p, -(sum*sum) * (1/p)^2) (stddev_from_prefix_scalar,
 * stddev.rs:899-935, called per row at stddev.rs:1043-1050); a window holding
 * a NaN gives NaN. */
int vto_stddev_batch_prefix(const double *x, size_t n, size_t period, double nbdev, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    double *ps = (double *)malloc(sizeof(double) * (n + 1));
    double *ps2 = (double *)malloc(sizeof(double) * (n + 1));
    int *pn = (int *)malloc(sizeof(int) * (n + 1));
    ps[0] = ps2[0] = 0.0;
    pn[0] = 0;
    for (size_t i = 0; i < n; i++) {
        double v = x[i];
        if (isnan(v)) {
            ps[i + 1] = ps[i];
            ps2[i + 1] = ps2[i];
            pn[i + 1] = pn[i] + 1;
        } else {
            ps[i + 1] = ps[i] + v;
            ps2[i + 1] = ps2[i] + v * v;
            pn[i + 1] = pn[i];
        }
    }
    size_t we = first + period - 1;
    fill_nan(out, we < n ? we : n);
    double inv = 1.0 / (double)period, inv2 = inv * inv;
    for (size_t i = we; i < n; i++) {
        if (pn[i + 1] - pn[i + 1 - period] > 0) {
            out[i] = QNAN;
            continue;
        }
        double s = ps[i + 1] - ps[i + 1 - period];
        double s2 = ps2[i + 1] - ps2[i + 1 - period];
        double var = fma(s2, inv, -(s * s) * inv2);
        out[i] = var <= 0.0 ? 0.0 : sqrt(var) * nbdev;
    }
    free(ps);
    free(ps2);
    free(pn);
    return VTO_OK;
}

/* NOT a restatement of the crate: the exact window statistics that the
 * crate's StdDev / Z-score paths approximate, used to measure how far the
 * crate's own running f64 sums drift on long series.  For each requested end
 * index i (window [i-p+1, i], all values finite) it returns the mean and the
 * population standard deviation by the corrected two-pass algorithm in f64
 * (Chan, Golub and LeVeque 1983: mean by a compensated sum, then
 * sum (x-m)^2 - (sum (x-m))^2 / p), whose relative error is a few f64 ulps
 * for windows of up to thousands of values. */
int vto_window_exact(const double *x, size_t n, size_t period, const size_t *idx, size_t nidx,
                     double *mean, double *sd) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    for (size_t k = 0; k < nidx; k++) {
        size_t i = idx[k];
        if (i >= n || i + 1 < period) return VTO_E_INVALID_RANGE;
        const double *w = x + (i + 1 - period);
        double s = 0.0, c = 0.0; /* Neumaier compensated sum */
        for (size_t j = 0; j < period; j++) {
            double t = s + w[j];
            c += fabs(s) >= fabs(w[j]) ? (s - t) + w[j] : (w[j] - t) + s;
            s = t;
        }
        double m = (s + c) / (double)period;
        double d1 = 0.0, d2 = 0.0;
        for (size_t j = 0; j < period; j++) {
            double d = w[j] - m;
            d1 += d;
            d2 += d * d;
        }
        double var = (d2 - d1 * d1 / (double)period) / (double)period;
        mean[k] = m;
        sd[k] = var > 0.0 ? sqrt(var) : 0.0;
    }
    return VTO_OK;
}

/* zscore_scalar_classic_sma (zscore.rs:359-431), single-series path with
 * mul_add: sum_sqr = v.mul_add(v, sum_sqr); variance = (-mean).mul_add(mean,
 * sum_sqr*inv); sd==0 or NaN -> NaN. */
int vto_zscore(const double *x, size_t n, size_t period, double nbdev, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t we = first + period - 1;
    fill_nan(out, we);
    double inv = 1.0 / (double)period;
    double sum = 0.0, sq = 0.0;
    for (size_t j = first; j <= we; j++) {
        double v = x[j];
        sum += v;
        sq = fma(v, v, sq);
    }
    double mean = sum * inv;
    double var = fma(-mean, mean, sq * inv);
    if (var < 0.0) var = 0.0;
    double sd = var == 0.0 ? 0.0 : sqrt(var) * nbdev;
    out[we] = (sd == 0.0 || isnan(sd)) ? QNAN : (x[we] - mean) / sd;
    for (size_t i = we + 1; i < n; i++) {
        double ov = x[i - period], nv = x[i];
        double dd = nv - ov;
        sum += dd;
        sq = fma(nv + ov, dd, sq);
        mean = sum * inv;
        var = fma(-mean, mean, sq * inv);
        if (var < 0.0) var = 0.0;
        sd = var == 0.0 ? 0.0 : sqrt(var) * nbdev;
        out[i] = (sd == 0.0 || isnan(sd)) ? QNAN : (nv - mean) / sd;
    }
    return VTO_OK;
}

/* zscore_row_scalar_classic_sma (zscore.rs:1344-1403): batch row, no FMA. */
int vto_zscore_batch_row(const double *x, size_t n, size_t period, double nbdev, double *out) {
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (n - first < period || period == 0) return VTO_E_NOT_ENOUGH_VALID;
    size_t we = first + period - 1;
    fill_nan(out, we);
    double sum = 0.0, sq = 0.0;
    for (size_t j = first; j <= we; j++) { sum += x[j]; sq += x[j] * x[j]; }
    double mean = sum / (double)period;
    double var = (sq / (double)period) - (mean * mean);
    double sd = var <= 0.0 ? 0.0 : sqrt(var) * nbdev;
    out[we] = (sd == 0.0 || isnan(sd)) ? QNAN : (x[we] - mean) / sd;
    for (size_t i = we + 1; i < n; i++) {
        double ov = x[i - period], nv = x[i];
        sum += nv - ov;
        sq += nv * nv - ov * ov;
        mean = sum / (double)period;
        var = (sq / (double)period) - (mean * mean);
        sd = var <= 0.0 ? 0.0 : sqrt(var) * nbdev;
        out[i] = (sd == 0.0 || isnan(sd)) ? QNAN : (nv - mean) / sd;
    }
    return VTO_OK;
}

/* bb_row_scalar_classic_sma, devtype 0 (bollinger_bands.rs:566-670):
 * population std; upper = m + devup*sd; lower = m - devdn*sd. */
int vto_bollinger(const double *x, size_t n, size_t period, double devup, double devdn,
                  double *up, double *mid, double *lo) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm = first + period - 1;
    fill_nan(up, warm); fill_nan(mid, warm); fill_nan(lo, warm);
    double inv_n = 1.0 / (double)period;
    double sum = 0.0, sq = 0.0;
    for (size_t k = 0; k < period; k++) {
        double v = x[first + k];
        sum += v;
        sq += v * v;
    }
    double mean = sum * inv_n;
    double var0 = (sq * inv_n) - (mean * mean);
    double sd0 = sqrt(fmax(var0, 0.0));
    mid[warm] = mean;
    up[warm] = mean + devup * sd0;
    lo[warm] = mean - devdn * sd0;
    for (size_t i = warm + 1; i < n; i++) {
        double nw = x[i], old = x[i - period];
        sum += nw - old;
        sq = (sq - old * old) + nw * nw;
        double m = sum * inv_n;
        double var = (sq * inv_n) - (m * m);
        double sd = sqrt(fmax(var, 0.0));
        mid[i] = m;
        up[i] = m + devup * sd;
        lo[i] = m - devdn * sd;
    }
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* Donchian / WillR / Percentile                                              */
/* ------------------------------------------------------------------------ */

/* donchian_scalar (donchian.rs:278-517).  Max/min are exact selections, so a
 * direct window scan gives the same bits as the crate's block-prefix path.
 * Window validity: p <= 32 uses is_nan, p > 32 uses is_finite. */
int vto_donchian(const double *h, const double *l, size_t n, size_t period,
                 double *up, double *mid, double *lo) {
    if (n == 0) return VTO_E_EMPTY;
    size_t fh = first_valid(h, n), fl = first_valid(l, n);
    if (fh >= n || fl >= n) return VTO_E_ALL_NAN;
    size_t first = fh > fl ? fh : fl;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm = first + period - 1;
    fill_nan(up, warm); fill_nan(mid, warm); fill_nan(lo, warm);
    int finite_rule = period > 32;
    for (size_t i = warm; i < n; i++) {
        double mx = -INFINITY, mn = INFINITY;
        int bad = 0;
        for (size_t j = i + 1 - period; j <= i; j++) {
            double hv = h[j], lv = l[j];
            if (finite_rule ? !(isfinite(hv) && isfinite(lv)) : (isnan(hv) || isnan(lv))) {
                bad = 1;
                break;
            }
            if (hv > mx) mx = hv;
            if (lv < mn) mn = lv;
        }
        if (bad) { up[i] = mid[i] = lo[i] = QNAN; }
        else { up[i] = mx; lo[i] = mn; mid[i] = fma(mx - mn, 0.5, mn); }
    }
    return VTO_OK;
}

/* willr_scalar (willr.rs:327-445) and willr_row_shared_core
 * (willr.rs:1386-1425): window containing a NaN high/low -> NaN, NaN close
 * -> NaN, denom == 0 -> 0, else (-100).mul_add((h-c)/denom, 0). */
int vto_willr(const double *h, const double *l, const double *c, size_t n, size_t period,
              double *out) {
    if (n == 0) return VTO_E_EMPTY;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    size_t first = first_valid_hlc(h, l, c, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm = first + period - 1;
    fill_nan(out, warm);
    for (size_t i = warm; i < n; i++) {
        double cv = c[i];
        if (isnan(cv)) { out[i] = QNAN; continue; }
        double hh = -INFINITY, ll = INFINITY;
        int bad = 0;
        for (size_t j = i + 1 - period; j <= i; j++) {
            if (isnan(h[j]) || isnan(l[j])) { bad = 1; break; }
            if (h[j] > hh) hh = h[j];
            if (l[j] < ll) ll = l[j];
        }
        if (bad || !(isfinite(hh) && isfinite(ll))) { out[i] = QNAN; continue; }
        double den = hh - ll;
        out[i] = den == 0.0 ? 0.0 : fma(-100.0, (hh - cv) / den, 0.0);
    }
    return VTO_OK;
}

static int cmp_dbl(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* nearest-rank index: round(p_frac.mul_add(wl, 0)) - 1 clamped to [0, wl-1]
 * (percentile_nearest_rank.rs:221-229); Rust round = C round(). */
static size_t pnr_rank(double p_frac, size_t wl) {
    double raw_f = round(fma(p_frac, (double)wl, 0.0));
    long long raw = (long long)raw_f - 1;
    size_t k = raw <= 0 ? 0 : (size_t)raw;
    if (k >= wl) k = wl - 1;
    return k;
}

/* pnr_compute_into (percentile_nearest_rank.rs:190-266): sorted window of the
 * non-NaN values; out = sorted[k]; empty window -> NaN. */
int vto_percentile_nearest_rank(const double *x, size_t n, size_t length, double percentage,
                                double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (length == 0 || length > n) return VTO_E_INVALID_PERIOD;
    if (!(percentage >= 0.0 && percentage <= 100.0)) return VTO_E_INVALID_PARAM;
    if (n - first < length) return VTO_E_NOT_ENOUGH_VALID;
    size_t start_i = first + length - 1;
    fill_nan(out, start_i);
    double p_frac = percentage * 0.01;
    double *buf = (double *)malloc(sizeof(double) * length);
    for (size_t i = start_i; i < n; i++) {
        size_t wl = 0;
        for (size_t j = i + 1 - length; j <= i; j++)
            if (!isnan(x[j])) buf[wl++] = x[j];
        if (wl == 0) { out[i] = QNAN; continue; }
        qsort(buf, wl, sizeof(double), cmp_dbl);
        out[i] = buf[pnr_rank(p_frac, wl)];
    }
    free(buf);
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* Weighted-window moving averages                                            */
/* ------------------------------------------------------------------------ */

/* wma_scalar (wma.rs:295-336): running weighted sum; p >= 2 (wma.rs:260). */
int vto_wma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period < 2 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    fill_nan(out, first + period - 1);
    size_t lb = period - 1;
    double pf = (double)period;
    double weights = pf * (pf + 1.0) * 0.5;
    const double *base = x + first;
    double sum = 0.0, ws = 0.0;
    for (size_t k = 0; k < lb; k++) {
        double v = base[k];
        ws += v * ((double)k + 1.0);
        sum += v;
    }
    for (size_t i = first + lb, old = first; i < n; i++, old++) {
        double v = x[i];
        ws += v * pf;
        sum += v;
        out[i] = ws / weights;
        ws -= sum;
        sum -= x[old];
    }
    return VTO_OK;
}

/* swma_scalar (swma.rs:406-482): triangle = SMA(a) of SMA(b) via a ring of
 * running sums; a,b from the parity of p; p==1 copy, p==2 pairwise mean. */
int vto_swma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    fill_nan(out, first + period - 1);
    size_t a, b;
    if (period & 1) { a = b = (period + 1) >> 1; }
    else { a = period >> 1; b = a + 1; }
    if (period == 1) {
        for (size_t i = first; i < n; i++) out[i] = x[i];
        return VTO_OK;
    }
    if (period == 2) {
        for (size_t i = first + 1; i < n; i++) out[i] = (x[i - 1] + x[i]) * 0.5;
        return VTO_OK;
    }
    double inv_ab = 1.0 / ((double)a * (double)b);
    size_t sfa = first + a - 1, sfab = first + period - 1;
    double *ring = (double *)calloc(b, sizeof(double));
    size_t rb = 0;
    double s1 = 0.0, s2 = 0.0;
    for (size_t i = first; i < n; i++) {
        s1 += x[i];
        if (i >= sfa) {
            double old = ring[rb];
            s2 = s2 + (s1 - old);
            ring[rb] = s1;
            if (++rb == b) rb = 0;
            if (i >= sfab) out[i] = s2 * inv_ab;
            s1 -= x[i + 1 - a];
        }
    }
    free(ring);
    return VTO_OK;
}

/* combination_f64 / pascal_weights (pwma.rs:1367-1408). */
void vto_pwma_weights(size_t period, double *w) {
    size_t nn = period - 1;
    double sum = 0.0;
    for (size_t r = 0; r <= nn; r++) {
        size_t rr = r < nn - r ? r : nn - r;
        double res = 1.0;
        for (size_t i = 0; i < rr; i++) {
            res *= (double)(nn - i);
            res /= (double)(i + 1);
        }
        w[r] = res;
    }
    for (size_t r = 0; r <= nn; r++) sum += w[r];
    for (size_t r = 0; r <= nn; r++) w[r] /= sum;
}

/* pwma_scalar (pwma.rs:345-400): 4 FMA accumulators, (s0+s1)+(s2+s3), tail
 * by mul_add.  `batch` selects pwma_row_scalar's 8 accumulators
 * (pwma.rs:1126-1196). */
static void pwma_row(const double *x, size_t n, size_t first, size_t period, const double *w,
                     int batch, double *out) {
    for (size_t i = first + period - 1; i < n; i++) {
        const double *d = x + i + 1 - period;
        double sum;
        size_t k = 0;
        if (!batch) {
            double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            size_t ke = period & ~(size_t)3;
            for (; k < ke; k += 4) {
                s0 = fma(d[k], w[k], s0);
                s1 = fma(d[k + 1], w[k + 1], s1);
                s2 = fma(d[k + 2], w[k + 2], s2);
                s3 = fma(d[k + 3], w[k + 3], s3);
            }
            sum = (s0 + s1) + (s2 + s3);
        } else {
            double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            size_t ke = period & ~(size_t)7;
            for (; k < ke; k += 8)
                for (int u = 0; u < 8; u++) s[u] = fma(d[k + u], w[k + u], s[u]);
            sum = (((s[0] + s[1]) + (s[2] + s[3])) + (s[4] + s[5])) + (s[6] + s[7]);
        }
        for (; k < period; k++) sum = fma(d[k], w[k], sum);
        out[i] = sum;
    }
}

int vto_pwma(const double *x, size_t n, size_t period, int batch, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    double *w = (double *)malloc(sizeof(double) * period);
    vto_pwma_weights(period, w);
    fill_nan(out, first + period - 1);
    pwma_row(x, n, first, period, w, batch, out);
    free(w);
    return VTO_OK;
}

/* sinwma_prepare weights (sinwma.rs:271-289) and sinwma_scalar
 * (sinwma.rs:353-389, same 4-wide unrolled dot as ALMA, no inv_norm). */
void vto_sinwma_weights(size_t period, double *w) {
    double sum = 0.0;
    for (size_t k = 0; k < period; k++) {
        double ang = ((double)k + 1.0) * M_PI / ((double)period + 1.0);
        w[k] = sin(ang);
        sum += w[k];
    }
    double inv = 1.0 / sum;
    for (size_t k = 0; k < period; k++) w[k] *= inv;
}

int vto_sinwma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    double *w = (double *)malloc(sizeof(double) * period);
    vto_sinwma_weights(period, w);
    fill_nan(out, first + period - 1);
    size_t p4 = period & ~(size_t)3;
    for (size_t i = first + period - 1; i < n; i++) {
        const double *d = x + i + 1 - period;
        double sum = 0.0;
        for (size_t k = 0; k < p4; k += 4)
            sum += d[k] * w[k] + d[k + 1] * w[k + 1] + d[k + 2] * w[k + 2] + d[k + 3] * w[k + 3];
        for (size_t k = p4; k < period; k++) sum += d[k] * w[k];
        out[i] = sum;
    }
    free(w);
    return VTO_OK;
}

/* trima_scalar_optimized (trima.rs:277-364): SMA(m1) then SMA(m2) over a
 * ring of SMA1 values; m1 = (p+1)/2, m2 = p - m1 + 1; p > 3. */
int vto_trima(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (period <= 3) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t m1 = (period + 1) / 2, m2 = period - m1 + 1;
    size_t warm = first + period - 1;
    fill_nan(out, warm);
    double inv1 = 1.0 / (double)m1, inv2 = 1.0 / (double)m2;
    const double *base = x + first;
    double sum1 = 0.0;
    size_t j = 0, eu = m1 & ~(size_t)3;
    for (; j < eu; j += 4) sum1 += base[j] + base[j + 1] + base[j + 2] + base[j + 3];
    for (; j < m1; j++) sum1 += base[j];
    double *ring = (double *)malloc(sizeof(double) * m2);
    size_t rl = 0;
    double sum2 = 0.0;
    size_t t = first + m1 - 1;
    size_t pn = first + m1, po = first;
    double s1 = sum1 * inv1;
    ring[rl++] = s1;
    sum2 += s1;
    while (rl < m2) {
        t++;
        sum1 += x[pn++] - x[po++];
        s1 = sum1 * inv1;
        ring[rl++] = s1;
        sum2 += s1;
    }
    out[warm] = sum2 * inv2;
    size_t head = 0;
    for (t = t + 1; t < n; t++) {
        sum1 += x[pn++] - x[po++];
        double ns1 = sum1 * inv1;
        double os1 = ring[head];
        sum2 += ns1 - os1;
        ring[head] = ns1;
        if (++head == m2) head = 0;
        out[t] = sum2 * inv2;
    }
    free(ring);
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* Fast min/max windows with the crate's own algorithms (used to time the    */
/* CPU baseline).  Max/min are exact selections, so these return the same    */
/* bits as vto_donchian / vto_willr.                                         */
/* ------------------------------------------------------------------------ */

/* donchian_scalar p > 32 (donchian.rs:413-517): block-prefix maxima g_max /
 * minima g_min over blocks of p, reverse running block-suffix extrema, and a
 * valid-count prefix; p <= 32 falls back to the direct scan. */
int vto_donchian_fast(const double *h, const double *l, size_t n, size_t period,
                      double *up, double *mid, double *lo) {
    if (period <= 32) return vto_donchian(h, l, n, period, up, mid, lo);
    if (n == 0) return VTO_E_EMPTY;
    size_t fh = first_valid(h, n), fl = first_valid(l, n);
    if (fh >= n || fl >= n) return VTO_E_ALL_NAN;
    size_t first = fh > fl ? fh : fl;
    if (period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm = first + period - 1;
    fill_nan(up, warm); fill_nan(mid, warm); fill_nan(lo, warm);
    double *gmax = (double *)malloc(sizeof(double) * n);
    double *gmin = (double *)malloc(sizeof(double) * n);
    unsigned *ps = (unsigned *)malloc(sizeof(unsigned) * (n + 1));
    double amax = -INFINITY, amin = INFINITY;
    size_t k = 0;
    ps[0] = 0;
    for (size_t i = 0; i < n; i++) {
        int ok = isfinite(h[i]) && isfinite(l[i]);
        double hv = ok ? h[i] : -INFINITY, lv = ok ? l[i] : INFINITY;
        if (k == 0) { amax = hv; amin = lv; }
        else { if (hv > amax) amax = hv; if (lv < amin) amin = lv; }
        gmax[i] = amax; gmin[i] = amin;
        if (++k == period) k = 0;
        ps[i + 1] = ps[i] + (unsigned)ok;
    }
    amax = -INFINITY; amin = INFINITY;
    for (size_t j = n; j-- > 0;) {
        int ok = isfinite(h[j]) && isfinite(l[j]);
        double hv = ok ? h[j] : -INFINITY, lv = ok ? l[j] : INFINITY;
        if (j == n - 1 || ((j + 1) % period) == 0) { amax = hv; amin = lv; }
        else { if (hv > amax) amax = hv; if (lv < amin) amin = lv; }
        size_t i = j + period - 1;
        if (i >= n || i < warm) continue;
        if (ps[i + 1] - ps[i + 1 - period] == (unsigned)period) {
            double mx = amax > gmax[i] ? amax : gmax[i];
            double mn = amin < gmin[i] ? amin : gmin[i];
            up[i] = mx; lo[i] = mn; mid[i] = fma(mx - mn, 0.5, mn);
        } else {
            up[i] = mid[i] = lo[i] = QNAN;
        }
    }
    free(gmax); free(gmin); free(ps);
    return VTO_OK;
}

/* willr_scalar p > 32 (willr.rs:447-622): monotonic deques of indices for the
 * window max of high and min of low plus a NaN counter; p <= 32 falls back to
 * the direct scan. */
int vto_willr_fast(const double *h, const double *l, const double *c, size_t n, size_t period,
                   double *out) {
    if (period <= 32) return vto_willr(h, l, c, n, period, out);
    if (n == 0) return VTO_E_EMPTY;
    if (period > n) return VTO_E_INVALID_PERIOD;
    size_t first = first_valid_hlc(h, l, c, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    size_t warm = first + period - 1;
    fill_nan(out, warm);
    size_t *dqx = (size_t *)malloc(sizeof(size_t) * (period + 1));
    size_t *dqn = (size_t *)malloc(sizeof(size_t) * (period + 1));
    size_t hx = 0, tx = 0, hn = 0, tn = 0; /* deque = [head, tail) in a ring of period+1 */
    size_t cap = period + 1, nan_cnt = 0;
    for (size_t i = warm + 1 - period; i < n; i++) {
        /* push i */
        if (isnan(h[i]) || isnan(l[i])) nan_cnt++;
        else {
            while (hx != tx && h[dqx[(tx + cap - 1) % cap]] <= h[i]) tx = (tx + cap - 1) % cap;
            dqx[tx] = i; tx = (tx + 1) % cap;
            while (hn != tn && l[dqn[(tn + cap - 1) % cap]] >= l[i]) tn = (tn + cap - 1) % cap;
            dqn[tn] = i; tn = (tn + 1) % cap;
        }
        if (i < warm) continue;
        size_t lo_i = i + 1 - period;
        while (hx != tx && dqx[hx] < lo_i) hx = (hx + 1) % cap;
        while (hn != tn && dqn[hn] < lo_i) hn = (hn + 1) % cap;
        double cv = c[i];
        if (isnan(cv) || nan_cnt > 0 || hx == tx || hn == tn) out[i] = QNAN;
        else {
            double hh = h[dqx[hx]], ll = l[dqn[hn]];
            if (!(isfinite(hh) && isfinite(ll))) out[i] = QNAN;
            else {
                double den = hh - ll;
                out[i] = den == 0.0 ? 0.0 : fma(-100.0, (hh - cv) / den, 0.0);
            }
        }
        /* pop the element leaving next step */
        if (isnan(h[lo_i]) || isnan(l[lo_i])) nan_cnt--;
    }
    free(dqx); free(dqn);
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* The remaining weighted-window moving averages.                             */
/* ------------------------------------------------------------------------ */

/* cwma_prepare (cwma.rs:205-263): weights (p - i)^3, i < p - 1 (newest
 * first), inv_norm = 1 / sum; cwma_scalar x86 form (cwma.rs:331-451): eight
 * mul_add accumulators over blocks of 8, summed pairwise, then a sequential
 * mul_add tail; first output first + p - 1. */
int vto_cwma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n || period == 1) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    const size_t wlen = period - 1;
    double *w = (double *)malloc(sizeof(double) * wlen);
    double norm = 0.0;
    for (size_t i = 0; i < wlen; i++) {
        double v = (double)(period - i);
        w[i] = v * v * v;
        norm += w[i];
    }
    double inv = 1.0 / norm;
    fill_nan(out, first + wlen);
    for (size_t i = first + wlen; i < n; i++) {
        const double *d = x + i;
        double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        size_t k = 0;
        while (k + 7 < wlen) {
            for (int j = 0; j < 8; j++) {
                s[j] = fma(*d, w[k + j], s[j]);
                d--;
            }
            k += 8;
        }
        double sum = (s[0] + s[1]) + (s[2] + s[3]) + (s[4] + s[5]) + (s[6] + s[7]);
        for (; k < wlen; k++) {
            sum = fma(*d, w[k], sum);
            d--;
        }
        out[i] = sum * inv;
    }
    free(w);
    return VTO_OK;
}

/* fwma_prepare (fwma.rs:293-339): Fibonacci weights fib[0] = fib[1] = 1
 * (oldest first), each divided by their sum; fwma_scalar (fwma.rs:428-454):
 * per group of 4 `sum += d0 w0 + d1 w1 + d2 w2 + d3 w3`, then the tail;
 * first output first + p - 1. */
int vto_fwma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period == 0 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    double *w = (double *)malloc(sizeof(double) * period);
    for (size_t i = 0; i < period; i++) w[i] = 1.0;
    for (size_t i = 2; i < period; i++) w[i] = w[i - 1] + w[i - 2];
    double sum_w = 0.0;
    for (size_t i = 0; i < period; i++) sum_w += w[i];
    for (size_t i = 0; i < period; i++) w[i] /= sum_w;
    fill_nan(out, first + period - 1);
    const size_t p4 = period & ~(size_t)3;
    for (size_t i = first + period - 1; i < n; i++) {
        const double *d = x + i + 1 - period;
        double sum = 0.0;
        for (size_t k = 0; k < p4; k += 4)
            sum += d[k] * w[k] + d[k + 1] * w[k + 1] + d[k + 2] * w[k + 2] + d[k + 3] * w[k + 3];
        for (size_t k = p4; k < period; k++) sum += d[k] * w[k];
        out[i] = sum;
    }
    free(w);
    return VTO_OK;
}

/* srwma_with_kernel (srwma.rs:174-246): weights sqrt(p - i), i < p - 1
 * (newest first), inv_norm = 1 / sum, first output first + p + 1; needs
 * len - first >= p + 1.  srwma_scalar (srwma.rs:275-379): eight mul_add
 * accumulators over blocks of 8, then four over blocks of 4, then s0; the
 * accumulators summed as ((s0+s1)+(s2+s3)) + ((s4+s5)+(s6+s7)).  Periods
 * below 2 are rejected here (the crate's p = 1 has an empty weight row). */
int vto_srwma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period < 2 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period + 1) return VTO_E_NOT_ENOUGH_VALID;
    const size_t wlen = period - 1;
    double *w = (double *)malloc(sizeof(double) * wlen);
    double norm = 0.0;
    for (size_t i = 0; i < wlen; i++) {
        w[i] = sqrt((double)(period - i));
        norm += w[i];
    }
    double inv = 1.0 / norm;
    const size_t start = first + period + 1;
    fill_nan(out, start < n ? start : n);
    for (size_t i = start; i < n; i++) {
        const double *dp = x + i;
        double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        size_t k = 0;
        while (k + 8 <= wlen) {
            for (int j = 0; j < 8; j++) s[j] = fma(*(dp - (k + j)), w[k + j], s[j]);
            k += 8;
        }
        while (k + 4 <= wlen) {
            for (int j = 0; j < 4; j++) s[j] = fma(*(dp - (k + j)), w[k + j], s[j]);
            k += 4;
        }
        while (k < wlen) {
            s[0] = fma(*(dp - k), w[k], s[0]);
            k++;
        }
        double sum = ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
        out[i] = sum * inv;
    }
    free(w);
    return VTO_OK;
}

/* sqwma_with_kernel (sqwma.rs:195-251): weights (p - i)^2, i < p - 1 (newest
 * first), first output first + p + 1; sqwma_scalar (sqwma.rs:254-300): one
 * sequential mul_add chain, times 1 / weight_sum. */
int vto_sqwma(const double *x, size_t n, size_t period, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period < 2 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    const size_t wlen = period - 1;
    double *w = (double *)malloc(sizeof(double) * wlen);
    double ws = 0.0;
    for (size_t i = 0; i < wlen; i++) {
        double v = (double)period - (double)i;
        w[i] = v * v;
        ws += w[i];
    }
    double inv = 1.0 / ws;
    const size_t start = first + period + 1;
    fill_nan(out, start < n ? start : n);
    for (size_t j = start; j < n; j++) {
        double sum = 0.0;
        for (size_t k = 0; k < wlen; k++) sum = fma(x[j - k], w[k], sum);
        out[j] = sum * inv;
    }
    free(w);
    return VTO_OK;
}

/* epma_prepare (epma.rs:205-250) and epma_scalar (epma.rs:333-366): window
 * of p - 1 values x[j-p+2 .. j] with weights c0, c0 + 1, ... (oldest first),
 * c0 = 2 - offset; weight_sum = mul_add(p1, c0, 0.5 (p1 - 1) p1); one
 * sequential mul_add chain times 1 / weight_sum; first output
 * first + p + offset + 1; needs offset < p, p >= 2 and len - first >= p + offset + 1. */
int vto_epma(const double *x, size_t n, size_t period, size_t offset, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (offset >= period) return VTO_E_INVALID_PARAM;
    if (period < 2 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period + offset + 1) return VTO_E_NOT_ENOUGH_VALID;
    const size_t p1 = period - 1;
    const double c0 = 2.0 - (double)offset;
    const double p1f = (double)p1;
    const double weight_sum = fma(p1f, c0, 0.5 * (p1f - 1.0) * p1f);
    const double inv = 1.0 / weight_sum;
    const size_t start = first + period + offset + 1;
    fill_nan(out, start < n ? start : n);
    for (size_t j = start; j < n; j++) {
        const size_t s0 = j + 1 - p1;
        double sum = 0.0, wi = c0;
        for (size_t i = 0; i < p1; i++, wi += 1.0) sum = fma(x[s0 + i], wi, sum);
        out[j] = sum * inv;
    }
    return VTO_OK;
}

/* ------------------------------------------------------------------------ */
/* Streaming updates (the crate's XStream structs): x[t] is fed to update()   */
/* in order; out[t] is the returned value, NaN where update() returns None.   */
/* ------------------------------------------------------------------------ */

/* EmaStream (ema.rs:519-585): running mean over the first `period` finite
 * values (mean += (x - mean) / c by mul_add), then beta*mean + alpha*x by
 * mul_add; non-finite x leaves the state alone and returns the mean once
 * filled. */
int vto_ema_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const double alpha = 2.0 / ((double)period + 1.0), beta = 1.0 - alpha;
    size_t count = 0;
    double mean = QNAN;
    int filled = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        if (!isfinite(v)) {
            out[t] = filled ? mean : QNAN;
            continue;
        }
        count++;
        if (count == 1) mean = v;
        else if (count <= period) mean = fma(v - mean, 1.0 / (double)count, mean);
        else mean = fma(beta, mean, alpha * v);
        if (!filled && count >= period) filled = 1;
        out[t] = filled ? mean : QNAN;
    }
    return VTO_OK;
}

/* SmaStream (sma.rs: SmaStream::update): ring buffer and running sum,
 * sum += value - old once full; period 1 copies the value. */
int vto_sma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    double *buf = (double *)calloc(period, sizeof(double));
    size_t head = 0, count = 0;
    double sum = 0.0, inv = 1.0 / (double)period;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        if (period == 1) { out[t] = v; continue; }
        if (count < period) {
            sum += v;
            buf[head] = v;
            head = head + 1 == period ? 0 : head + 1;
            count++;
            out[t] = count == period ? sum * inv : QNAN;
            continue;
        }
        double old = buf[head];
        sum += v - old;
        buf[head] = v;
        head = head + 1 == period ? 0 : head + 1;
        out[t] = sum * inv;
    }
    free(buf);
    return VTO_OK;
}

/* AlmaStream (alma.rs:865-964): weights exp(-(i-m)^2 / (2 s^2)) with
 * m = offset (p-1), s = p / sigma (no FMA); every value (NaN included) enters
 * the ring; once `period` values were seen, the window oldest first is
 * dotted with 4 accumulators (dot_scalar_unrolled_safe) times 1 / norm. */
void vto_alma_stream_weights(size_t period, double offset, double sigma, double *w, double *inv_norm) {
    const double m = offset * (double)(period - 1);
    const double s = (double)period / sigma;
    const double s2 = 2.0 * s * s;
    double norm = 0.0;
    for (size_t i = 0; i < period; i++) {
        double diff = (double)i - m;
        w[i] = exp(-(diff * diff) / s2);
        norm += w[i];
    }
    *inv_norm = 1.0 / norm;
}

int vto_alma_stream(const double *x, size_t n, size_t period, double offset, double sigma, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    if (!(offset >= 0.0 && offset <= 1.0)) return VTO_E_INVALID_PARAM;
    if (!(sigma > 0.0)) return VTO_E_INVALID_PARAM;
    double *w = (double *)malloc(sizeof(double) * period);
    double inv_norm;
    vto_alma_stream_weights(period, offset, sigma, w, &inv_norm);
    double *ring = (double *)malloc(sizeof(double) * period);
    double *win = (double *)malloc(sizeof(double) * period);
    size_t head = 0, filled = 0;
    for (size_t t = 0; t < n; t++) {
        ring[head] = x[t];
        head = head + 1 == period ? 0 : head + 1;
        if (filled < period) {
            filled++;
            if (filled < period) { out[t] = QNAN; continue; }
        }
        for (size_t i = 0; i < period; i++) win[i] = ring[(head + i) % period];
        size_t n4 = period & ~(size_t)3, i = 0;
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (; i < n4; i += 4) {
            s0 += win[i] * w[i];
            s1 += win[i + 1] * w[i + 1];
            s2 += win[i + 2] * w[i + 2];
            s3 += win[i + 3] * w[i + 3];
        }
        double sum = (s0 + s1) + (s2 + s3);
        for (; i < period; i++) sum += win[i] * w[i];
        out[t] = sum * inv_norm;
    }
    free(w);
    free(ring);
    free(win);
    return VTO_OK;
}

/* RsiStream (rsi.rs: RsiStream::update): the first value only primes prev;
 * gains / losses (f64::max against 0) summed over `period` deltas, a
 * non-finite delta there poisons the seed (NaN); then Wilder mul_add. */
int vto_rsi_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const double inv_p = 1.0 / (double)period, beta = 1.0 - inv_p;
    int has_prev = 0, poisoned = 0, seeded = 0;
    size_t seed_count = 0;
    double prev = QNAN, sg = 0.0, sl = 0.0, ag = 0.0, al = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        if (!has_prev) { prev = v; has_prev = 1; out[t] = QNAN; continue; }
        double d = v - prev;
        prev = v;
        if (!seeded) {
            if (!isfinite(d)) poisoned = 1;
            sg += fmax(d, 0.0);
            sl += fmax(-d, 0.0);
            seed_count++;
            if (seed_count == period) {
                seeded = 1;
                if (poisoned) { ag = al = QNAN; out[t] = QNAN; }
                else {
                    ag = sg * inv_p;
                    al = sl * inv_p;
                    double den = ag + al;
                    out[t] = den == 0.0 ? 50.0 : 100.0 * ag / den;
                }
            } else {
                out[t] = QNAN;
            }
            continue;
        }
        ag = fma(ag, beta, inv_p * fmax(d, 0.0));
        al = fma(al, beta, inv_p * fmax(-d, 0.0));
        double den = ag + al;
        out[t] = den == 0.0 ? 50.0 : 100.0 * ag / den;
    }
    return VTO_OK;
}

/* AtrStream (atr.rs: AtrStream::update): TR = h - l while prev_close is NaN,
 * else max(h, pc) - min(l, pc) by comparisons; seed = sum of the first
 * `length` TRs times 1/length; then rma = mul_add(alpha, tr - rma, rma). */
int vto_atr_stream(const double *h, const double *l, const double *c, size_t n, size_t length, double *out) {
    if (length == 0) return VTO_E_INVALID_PERIOD;
    const double alpha = 1.0 / (double)length;
    double pc = QNAN, rma = QNAN, warm_sum = 0.0;
    size_t warm_count = 0;
    int seeded = 0;
    for (size_t t = 0; t < n; t++) {
        double tr;
        if (isnan(pc)) tr = h[t] - l[t];
        else {
            double up = h[t] > pc ? h[t] : pc;
            double dn = l[t] < pc ? l[t] : pc;
            tr = up - dn;
        }
        pc = c[t];
        if (!seeded) {
            warm_sum += tr;
            warm_count++;
            if (warm_count == length) {
                rma = warm_sum * alpha;
                seeded = 1;
                out[t] = rma;
            } else {
                out[t] = QNAN;
            }
            continue;
        }
        rma = fma(alpha, tr - rma, rma);
        out[t] = rma;
    }
    return VTO_OK;
}

/* WildersStream (wilders.rs: WildersStream::update): a non-finite value
 * during warm-up restarts it; seed = sum / period; then
 * mul_add(value - last, alpha, last). */
int vto_wilders_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const double alpha = 1.0 / (double)period;
    double warm_sum = 0.0, last = QNAN;
    size_t warm_count = 0;
    int started = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        if (!started) {
            if (!isfinite(v)) { warm_sum = 0.0; warm_count = 0; out[t] = QNAN; continue; }
            warm_sum += v;
            warm_count++;
            if (warm_count < period) { out[t] = QNAN; continue; }
            last = warm_sum / (double)period;
            started = 1;
            out[t] = last;
            continue;
        }
        last = fma(v - last, alpha, last);
        out[t] = last;
    }
    return VTO_OK;
}

/* DemaStream (dema.rs:615-690): the first value seeds both EMAs (output if
 * period 1); then ema = fmadd(ema, 1 - a, x a), ema2 = fmadd(ema2, 1 - a,
 * ema a), y = fmadd(ema, 2, -ema2), output once more than period - 1 values
 * were seen.  fmadd is mul_add on x86 targets (separate operations elsewhere);
 * this follows x86. */
int vto_dema_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const double a = 2.0 / ((double)period + 1.0), a1 = 1.0 - 2.0 / ((double)period + 1.0);
    double e1 = QNAN, e2 = QNAN;
    size_t filled = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        if (filled == 0) {
            e1 = e2 = v;
            filled = 1;
            out[t] = period == 1 ? v : QNAN;
            continue;
        }
        e1 = fma(e1, a1, v * a);
        e2 = fma(e2, a1, e1 * a);
        double y = fma(e1, 2.0, -e2);
        filled++;
        out[t] = filled > period - 1 ? y : QNAN;
    }
    return VTO_OK;
}

/* TemaStream (tema.rs:324-425): NaN before the first value is skipped; the
 * first value seeds ema1; ema2 starts at count == period (copy of ema1),
 * ema3 at count == 2 period - 1; output once count > 3 (period - 1); all
 * updates e = e (1 - a) + v a without FMA; y = 3 e1 - 3 e2 + e3. */
int vto_tema_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const double a = 2.0 / ((double)period + 1.0), om = 1.0 - a;
    const size_t start2 = period, start3 = 2 * period - 1, lookback = 3 * (period - 1);
    double e1 = QNAN, e2 = 0.0, e3 = 0.0;
    size_t count = 0;
    int ready = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        if (ready) {
            e1 = e1 * om + v * a;
            e2 = e2 * om + e1 * a;
            e3 = e3 * om + e2 * a;
            out[t] = 3.0 * e1 - 3.0 * e2 + e3;
            continue;
        }
        if (count == 0) {
            out[t] = QNAN;
            if (isnan(v)) continue;
            e1 = v;
            count = 1;
            if (period == 1) { e2 = e1; e3 = e2; ready = 1; out[t] = e1; }
            continue;
        }
        e1 = e1 * om + v * a;
        count++;
        if (count == start2) e2 = e1;
        else if (count > start2) e2 = e2 * om + e1 * a;
        if (count == start3) e3 = e2;
        else if (count > start3) e3 = e3 * om + e2 * a;
        if (count > lookback) { ready = 1; out[t] = 3.0 * e1 - 3.0 * e2 + e3; }
        else out[t] = QNAN;
    }
    return VTO_OK;
}

/* WmaStream (wma.rs:384-460): ring of `period` values; when it first fills,
 * weighted and plain sums are formed oldest first (weights 1..p) and the
 * output is wsum / (p (p + 1) / 2); then the sums are updated in O(1):
 * wsum += p v, ssum += v, out, wsum -= ssum, ssum -= oldest. */
int vto_wma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period < 2) return VTO_E_INVALID_PERIOD;
    double *buf = (double *)malloc(sizeof(double) * period);
    for (size_t i = 0; i < period; i++) buf[i] = QNAN;
    const double inv_div = 1.0 / ((double)(period * (period + 1)) * 0.5), pf = (double)period;
    size_t head = 0;
    int filled = 0;
    double plain = 0.0, wsum = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        buf[head] = v;
        head = head + 1 == period ? 0 : head + 1;
        if (!filled) {
            if (head != 0) { out[t] = QNAN; continue; }
            double ws = 0.0, ss = 0.0;
            size_t idx = head;
            for (size_t w = 1; w <= period; w++) {
                double b = buf[idx];
                ss += b;
                ws += (double)w * b;
                idx = idx + 1 == period ? 0 : idx + 1;
            }
            out[t] = ws * inv_div;
            wsum = ws - ss;
            plain = ss - buf[head];
            filled = 1;
            continue;
        }
        double oldest = buf[head];
        wsum += pf * v;
        plain += v;
        out[t] = wsum * inv_div;
        wsum -= plain;
        plain -= oldest;
    }
    free(buf);
    return VTO_OK;
}

/* SwmaStream (swma.rs:536-630): the triangle as two box sums, a = b = (p+1)/2
 * for odd p, a = p/2, b = a + 1 for even p: s1 = sum of the last a values,
 * s2 = sum of the last b values of s1, output s2 / (a b). */
int vto_swma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    size_t a, b;
    if (period & 1) { a = b = (period + 1) >> 1; }
    else { a = period >> 1; b = a + 1; }
    double *ra = (double *)calloc(a, sizeof(double)), *rb = (double *)calloc(b, sizeof(double));
    const double inv_ab = 1.0 / ((double)a * (double)b);
    size_t ia = 0, ca = 0, ib = 0, cb = 0;
    double s1 = 0.0, s2 = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        out[t] = QNAN;
        double old_a = ra[ia];
        if (ca == a) s1 -= old_a; else ca++;
        ra[ia] = v;
        s1 += v;
        ia = ia + 1 == a ? 0 : ia + 1;
        if (ca == a) {
            double old_b = rb[ib];
            if (cb == b) s2 -= old_b; else cb++;
            rb[ib] = s1;
            s2 += s1;
            ib = ib + 1 == b ? 0 : ib + 1;
            if (cb == b) out[t] = s2 * inv_ab;
        }
    }
    free(ra);
    free(rb);
    return VTO_OK;
}

/* PwmaStream (pwma.rs:675-720): Pascal weights as a cascade of p - 1 running
 * pairwise sums (prev starts NaN), output times 2^-(p-1) once p values were
 * seen; period 1 returns the value. */
int vto_pwma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const size_t m = period - 1;
    double *prev = (double *)malloc(sizeof(double) * (m ? m : 1));
    for (size_t i = 0; i < m; i++) prev[i] = QNAN;
    const double norm = ldexp(1.0, -(int)(m > 2000 ? 2000 : m));
    size_t seen = 0;
    for (size_t t = 0; t < n; t++) {
        if (m == 0) { out[t] = x[t]; continue; }
        double acc = x[t];
        for (size_t k = 0; k < m; k++) {
            double o = acc + prev[k];
            prev[k] = acc;
            acc = o;
        }
        if (seen < m) { seen++; out[t] = QNAN; continue; }
        out[t] = acc * norm;
    }
    free(prev);
    return VTO_OK;
}

/* StdDevStream (stddev.rs:451-570): ring with NaN count; sums skip NaN
 * values; while the window holds a NaN the output is NaN; else
 * var = sum_sq / p - mean^2, sqrt(var) * nbdev (0 if var <= 0). */
int vto_stddev_stream(const double *x, size_t n, size_t period, double nbdev, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    if (!isfinite(nbdev) || nbdev < 0.0) return VTO_E_INVALID_PARAM;
    double *buf = (double *)malloc(sizeof(double) * period);
    for (size_t i = 0; i < period; i++) buf[i] = QNAN;
    const double inv = 1.0 / (double)period;
    size_t head = 0, nanc = 0;
    int filled = 0;
    double sum = 0.0, sq = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        if (!filled) {
            if (isnan(v)) nanc++;
            else { sum += v; sq += v * v; }
            buf[head] = v;
            if (head + 1 != period) { head++; out[t] = QNAN; continue; }
            head = 0;
            filled = 1;
        } else {
            double old = buf[head];
            int on = isnan(old), nn = isnan(v);
            if (!on && !nn) { sum += v - old; sq += (v * v) - (old * old); }
            else if (!on && nn) { sum -= old; sq -= old * old; nanc++; }
            else if (on && !nn) { if (nanc > 0) nanc--; sum += v; sq += v * v; }
            else { if (nanc > 0) nanc--; nanc++; }
            buf[head] = v;
            head = head + 1 == period ? 0 : head + 1;
        }
        if (nanc > 0) { out[t] = QNAN; continue; }
        double mean = sum * inv;
        double var = (sq * inv) - (mean * mean);
        out[t] = var <= 0.0 ? 0.0 : sqrt(var) * nbdev;
    }
    free(buf);
    return VTO_OK;
}

/* ZscoreStream (zscore.rs:567-735) with ma_type "sma", devtype 0: NaN-zeroed
 * running sums; once filled and with no NaN in the window and nbdev != 0,
 * z = (last - mean) / (sqrt(max(ex2 - mean^2, 0)) nbdev), NaN when the
 * deviation is 0 or not finite.  A window holding a NaN, or nbdev == 0, goes
 * through the crate's slow path, whose result is NaN for this MA. */
int vto_zscore_stream(const double *x, size_t n, size_t period, double nbdev, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    double *buf = (double *)malloc(sizeof(double) * period);
    for (size_t i = 0; i < period; i++) buf[i] = QNAN;
    const double inv = 1.0 / (double)period;
    size_t head = 0, nanc = period;
    int filled = 0;
    double sum = 0.0, sum2 = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        double old = buf[head];
        buf[head] = v;
        head = (head + 1) % period;
        if (!filled && head == 0) filled = 1;
        if (isnan(old) && nanc > 0) nanc--;
        if (isnan(v)) nanc++;
        double oc = isnan(old) ? 0.0 : old, nc = isnan(v) ? 0.0 : v;
        sum = sum + nc - oc;
        sum2 = sum2 + nc * nc - oc * oc;
        if (!filled) { out[t] = QNAN; continue; }
        if (nbdev == 0.0 || nanc != 0) { out[t] = QNAN; continue; }
        double mean = sum * inv, ex2 = sum2 * inv;
        double var = ex2 - mean * mean;
        if (var < 0.0) var = 0.0;
        double sd = sqrt(var);
        if (sd == 0.0 || !isfinite(sd)) { out[t] = QNAN; continue; }
        double last = buf[head == 0 ? period - 1 : head - 1];
        out[t] = (last - mean) / (sd * nbdev);
    }
    free(buf);
    return VTO_OK;
}

/* BollingerBandsStream (bollinger_bands.rs:884-1075), devtype 0 with ma "sma"
 * (ema = 0) or "ema" (ema = 1): a non-finite value resets the stream; the
 * ring keeps sum and sum of squares (x mul_add x); sd = sqrt(max(sq/p -
 * mean^2, 0)); the EMA middle is seeded with the window mean, then
 * mul_add(a, x, (1 - a) ema); bands mul_add(+-dev, sd, middle). */
int vto_bollinger_stream(const double *x, size_t n, size_t period, double devup, double devdn, int ema,
                         double *up, double *mid, double *lo) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    double *buf = (double *)calloc(period, sizeof(double));
    const double inv = 1.0 / (double)period, alpha = 2.0 / ((double)period + 1.0);
    size_t idx = 0, len = 0;
    double sum = 0.0, sq = 0.0, e = 0.0;
    int seeded = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        up[t] = mid[t] = lo[t] = QNAN;
        if (!isfinite(v)) { idx = len = 0; sum = sq = e = 0.0; seeded = 0; continue; }
        if (len < period) {
            buf[idx] = v;
            idx = idx + 1 == period ? 0 : idx + 1;
            len++;
            sum += v;
            sq = fma(v, v, sq);
        } else {
            double old = buf[idx];
            buf[idx] = v;
            idx = idx + 1 == period ? 0 : idx + 1;
            sum += v - old;
            double tmp = sq - old * old;
            sq = fma(v, v, tmp);
        }
        if (len < period) continue;
        double mean = sum * inv;
        double var = (sq * inv) - mean * mean;
        double sd = sqrt(var > 0.0 ? var : 0.0);
        double m = mean;
        if (ema) {
            if (!seeded) { e = sum * inv; seeded = 1; }
            else e = fma(alpha, v, (1.0 - alpha) * e);
            m = e;
        }
        up[t] = fma(devup, sd, m);
        mid[t] = m;
        lo[t] = fma(-devdn, sd, m);
    }
    free(buf);
    return VTO_OK;
}

/* DonchianStream (donchian.rs:1251-1340): once `period` bars were seen, NaN
 * bands while any bar of the window has a non-finite high or low; else the
 * window's highest high and lowest low (the monotone deques' fronts) and
 * middle mul_add(max - min, 0.5, min). */
int vto_donchian_stream(const double *h, const double *l, size_t n, size_t period, double *up, double *mid,
                        double *lo) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    for (size_t t = 0; t < n; t++) {
        up[t] = mid[t] = lo[t] = QNAN;
        if (t + 1 < period) continue;
        int ok = 1;
        double mx = -INFINITY, mn = INFINITY;
        for (size_t k = t + 1 - period; k <= t; k++) {
            if (!isfinite(h[k]) || !isfinite(l[k])) { ok = 0; break; }
            if (h[k] > mx) mx = h[k];
            if (l[k] < mn) mn = l[k];
        }
        if (!ok) continue;
        up[t] = mx;
        lo[t] = mn;
        mid[t] = fma(mx - mn, 0.5, mn);
    }
    return VTO_OK;
}

/* WillrStream (willr.rs:1657-1820): once `period` bars were seen, NaN when
 * the close is NaN or any bar of the window has a NaN high or low, or the
 * window extremes are not finite; else 0 for a flat window and
 * mul_add(-100, (hh - close) / (hh - ll), 0). */
int vto_willr_stream(const double *h, const double *l, const double *c, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    for (size_t t = 0; t < n; t++) {
        out[t] = QNAN;
        if (t + 1 < period) continue;
        int ok = !isnan(c[t]);
        double hh = -INFINITY, ll = INFINITY;
        for (size_t k = t + 1 - period; ok && k <= t; k++) {
            if (isnan(h[k]) || isnan(l[k])) { ok = 0; break; }
            if (h[k] > hh) hh = h[k];
            if (l[k] < ll) ll = l[k];
        }
        if (!ok || !(isfinite(hh) && isfinite(ll))) continue;
        double den = hh - ll;
        out[t] = den == 0.0 ? 0.0 : fma(-100.0, (hh - c[t]) / den, 0.0);
    }
    return VTO_OK;
}

/* AdxStream (adx.rs:1949-2085): TR = max(h, pc) - min(l, pc) (f64::max /
 * min, NaN-ignoring), +DM / -DM; the first `period` moves are summed and give
 * the first DX; then Wilder smoothing s (1 - 1/p) + m, DX from
 * 100 / ATR; ADX = mean of the first `period` DX values, then
 * (adx (p - 1) + dx) / p. */
int vto_adx_stream(const double *h, const double *l, const double *c, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    double atr = 0.0, pdm_s = 0.0, mdm_s = 0.0, dx_sum = 0.0, last = 0.0, ph = QNAN, pl = QNAN, pc = QNAN;
    size_t count = 0, dx_count = 0;
    const double rp = 1.0 / (double)period, omr = 1.0 - rp, pm1 = (double)period - 1.0;
    for (size_t t = 0; t < n; t++) {
        out[t] = QNAN;
        if (count == 0) { ph = h[t]; pl = l[t]; pc = c[t]; count = 1; continue; }
        double tr = fmax(h[t], pc) - fmin(l[t], pc);
        double upm = h[t] - ph, dnm = pl - l[t];
        double pdm = (upm > dnm && upm > 0.0) ? upm : 0.0;
        double mdm = (dnm > upm && dnm > 0.0) ? dnm : 0.0;
        count++;
        if (count <= period + 1) {
            atr += tr;
            pdm_s += pdm;
            mdm_s += mdm;
            if (count == period + 1) {
                double inv = atr != 0.0 ? 100.0 / atr : 0.0;
                double pdi = pdm_s * inv, mdi = mdm_s * inv, sdi = pdi + mdi;
                dx_sum = sdi != 0.0 ? (fabs(pdi - mdi) / sdi) * 100.0 : 0.0;
                dx_count = 1;
            }
            ph = h[t]; pl = l[t]; pc = c[t];
            continue;
        }
        atr = atr * omr + tr;
        pdm_s = pdm_s * omr + pdm;
        mdm_s = mdm_s * omr + mdm;
        double inv = atr != 0.0 ? 100.0 / atr : 0.0;
        double pdi = pdm_s * inv, mdi = mdm_s * inv, sdi = pdi + mdi;
        double dx = sdi != 0.0 ? (fabs(pdi - mdi) / sdi) * 100.0 : 0.0;
        if (dx_count < period) {
            dx_sum += dx;
            dx_count++;
            if (dx_count == period) { last = dx_sum * rp; out[t] = last; }
        } else {
            last = (last * pm1 + dx) * rp;
            out[t] = last;
        }
        ph = h[t]; pl = l[t]; pc = c[t];
    }
    return VTO_OK;
}

/* SuperTrendStream (supertrend.rs:798-885): AtrStream(length = period), then
 * basic bands mul_add(+-factor, atr, (h + l) / 2); the first ATR bar picks
 * the side (close <= upper) with changed 0; later bands ratchet with
 * f64::min / max against the previous bands while the previous close was
 * inside, and the side flips when the close crosses (changed 1). */
int vto_supertrend_stream(const double *h, const double *l, const double *c, size_t n, size_t period,
                          double factor, double *trend, double *changed) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    double *atr = (double *)malloc(sizeof(double) * (n ? n : 1));
    int code = vto_atr_stream(h, l, c, n, period, atr);
    if (code != VTO_OK) { free(atr); return code; }
    double pu = QNAN, pl = QNAN, pc = QNAN;
    int upper = 0, warmed = 0;
    for (size_t t = 0; t < n; t++) {
        trend[t] = changed[t] = QNAN;
        if (t + 1 < period) continue; /* AtrStream::update returned None */
        double hl2 = (h[t] + l[t]) * 0.5;
        double ub = fma(factor, atr[t], hl2), lb = fma(-factor, atr[t], hl2);
        if (!warmed) {
            pu = ub; pl = lb;
            upper = c[t] <= pu;
            trend[t] = upper ? pu : pl;
            changed[t] = 0.0;
            pc = c[t];
            warmed = 1;
            continue;
        }
        double cu = ub, cl = lb;
        if (pc <= pu) cu = fmin(cu, pu);
        if (pc >= pl) cl = fmax(cl, pl);
        double ch = 0.0, tv;
        if (upper) {
            if (c[t] <= cu) tv = cu;
            else { ch = 1.0; upper = 0; tv = cl; }
        } else {
            if (c[t] >= cl) tv = cl;
            else { ch = 1.0; upper = 1; tv = cu; }
        }
        pu = cu; pl = cl; pc = c[t];
        trend[t] = tv;
        changed[t] = ch;
    }
    free(atr);
    return VTO_OK;
}

/* SinWmaStream (sinwma.rs:586-750): sine weights through the rotation
 * z = sum_j r^j x_(newest - j), r = e^(i alpha), alpha = pi / (p + 1):
 * rebuilt from the ring (mul_add chain) when the window becomes NaN-free,
 * then advanced in O(1): z' = r z + x_new - r^p x_old; output
 * mul_add(sin(p alpha), Re z, -cos(p alpha) Im z) / sum of sines.
 * Constants with the C library's sin / cos, as the crate's try_new. */
static void sinwma_rebuild(const double *buf, size_t p, size_t head, double r_re, double r_im, double *zr,
                           double *zi) {
    size_t newest = (head + p - 1) % p;
    double rj_re = 1.0, rj_im = 0.0, a = 0.0, b = 0.0;
    for (size_t j = 0; j < p; j++) {
        double xv = buf[(newest + p - j) % p];
        a = fma(rj_re, xv, a);
        b = fma(rj_im, xv, b);
        double nr = fma(rj_re, r_re, -rj_im * r_im);
        double ni = fma(rj_re, r_im, rj_im * r_re);
        rj_re = nr;
        rj_im = ni;
    }
    *zr = a;
    *zi = b;
}

int vto_sinwma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const double pi = 3.14159265358979323846;
    const double alpha = pi / ((double)period + 1.0);
    const double sina = sin(alpha), cosa = cos(alpha);
    const double sinp = sin(alpha * (double)period), cosp = cos(alpha * (double)period);
    const double denom = sin(0.5 * alpha);
    if (fabs(denom) < 2.220446049250313e-16) return VTO_E_INVALID_PARAM;
    const double sum_sines = sin(0.5 * alpha * (double)period) / denom;
    if (fabs(sum_sines) < 2.220446049250313e-16) return VTO_E_INVALID_PARAM;
    const double inv_sum = 1.0 / sum_sines;
    double *buf = (double *)malloc(sizeof(double) * period);
    for (size_t i = 0; i < period; i++) buf[i] = QNAN;
    size_t head = 0, nanc = period;
    int filled = 0, zvalid = 0;
    double zr = 0.0, zi = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        out[t] = QNAN;
        double old = buf[head];
        buf[head] = v;
        head = (head + 1) % period;
        if (isnan(old) && nanc > 0) nanc--;
        if (isnan(v)) nanc++;
        if (!filled) {
            if (head != 0) continue;
            filled = 1;
            if (nanc != 0) { zvalid = 0; continue; }
            sinwma_rebuild(buf, period, head, cosa, sina, &zr, &zi);
            zvalid = 1;
        } else {
            if (nanc != 0) { zvalid = 0; continue; }
            if (!zvalid) {
                sinwma_rebuild(buf, period, head, cosa, sina, &zr, &zi);
                zvalid = 1;
            } else {
                double rr = fma(cosa, zr, -sina * zi);
                double ri = fma(cosa, zi, sina * zr);
                zr = rr + v - cosp * old;
                zi = ri - sinp * old;
            }
        }
        out[t] = fma(sinp, zr, -cosp * zi) * inv_sum;
    }
    free(buf);
    return VTO_OK;
}

/* TrimaStream (trima.rs:826-905): SMA(m1) of the values (NaN values left out
 * of the running sum), then SMA(m2) of those means, m1 = (p + 1) / 2,
 * m2 = p - m1 + 1; period > 3. */
int vto_trima_stream(const double *x, size_t n, size_t period, double *out) {
    if (period <= 3) return VTO_E_INVALID_PERIOD;
    const size_t m1 = (period + 1) / 2, m2 = period - m1 + 1;
    const double inv1 = 1.0 / (double)m1, inv2 = 1.0 / (double)m2;
    double *b1 = (double *)malloc(sizeof(double) * m1), *b2 = (double *)malloc(sizeof(double) * m2);
    for (size_t i = 0; i < m1; i++) b1[i] = QNAN;
    for (size_t i = 0; i < m2; i++) b2[i] = QNAN;
    size_t h1 = 0, h2 = 0;
    int f1 = 0, f2 = 0;
    double s1 = 0.0, s2 = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        out[t] = QNAN;
        double o1 = b1[h1];
        b1[h1] = v;
        if (++h1 == m1) { h1 = 0; f1 = 1; }
        if (!isnan(o1)) s1 -= o1;
        if (!isnan(v)) s1 += v;
        if (!f1) continue;
        double mean1 = s1 * inv1;
        double o2 = b2[h2];
        b2[h2] = mean1;
        if (++h2 == m2) { h2 = 0; f2 = 1; }
        if (!isnan(o2)) s2 -= o2;
        s2 += mean1;
        if (f2) out[t] = s2 * inv2;
    }
    free(b1);
    free(b2);
    return VTO_OK;
}

/* CwmaStream (cwma.rs:792-1040): leading NaNs are skipped; a ring of the last
 * n = p - 1 values; the first n values give None, then NaN while the window
 * holds a NaN, else the direct sum (sum_weighted: mul_add chain newest
 * first, weights (p + 1 - r)^3, r = 1..n) over sum_{j=2..p} j^3.  The
 * crate's running moments do not enter the output. */
int vto_cwma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period <= 1) return VTO_E_INVALID_PERIOD;
    const size_t m = period - 1;
    double norm = 0.0;
    for (size_t j = 2; j <= period; j++) {
        double jf = (double)j;
        norm += jf * jf * jf;
    }
    const double inv_norm = 1.0 / norm, a = (double)(m + 2);
    double *ring = (double *)malloc(sizeof(double) * m);
    for (size_t i = 0; i < m; i++) ring[i] = QNAN;
    size_t head = 0, filled = 0, nanc = 0;
    int found = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        out[t] = QNAN;
        if (!found) {
            if (isnan(v)) continue;
            found = 1;
        }
        double old = filled >= m ? ring[head] : QNAN;
        size_t new_nan = isnan(v) ? 1 : 0, old_nan = (filled >= m && isnan(old)) ? 1 : 0;
        ring[head] = v;
        head = (head + 1) % m;
        if (filled <= m) {
            filled++;
            nanc += new_nan;
            if (filled == m + 1) nanc -= old_nan;
            if (filled <= m) continue;
        } else {
            nanc = nanc + new_nan - old_nan;
        }
        if (nanc > 0) continue;
        double s = 0.0;
        for (size_t r = 1; r <= m; r++) {
            double tv = a - (double)r;
            s = fma(ring[(head + m - r) % m], tv * tv * tv, s);
        }
        out[t] = s * inv_norm;
    }
    free(ring);
    return VTO_OK;
}

/* FwmaStream (fwma.rs:750-890): Fibonacci weights 1, 1, 2, 3, ... divided
 * by their sum; once `period` values were seen, NaN while the window holds
 * a NaN, else the dot of the window (oldest first) with the weights. */
int vto_fwma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    double *w = (double *)malloc(sizeof(double) * period), *buf = (double *)malloc(sizeof(double) * period);
    for (size_t i = 0; i < period; i++) { w[i] = 1.0; buf[i] = QNAN; }
    for (size_t i = 2; i < period; i++) w[i] = w[i - 1] + w[i - 2];
    double sum = 0.0;
    for (size_t i = 0; i < period; i++) sum += w[i];
    for (size_t i = 0; i < period; i++) w[i] /= sum;
    size_t head = 0, nanc = 0;
    int filled = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        out[t] = QNAN;
        double old = buf[head];
        if (filled && isnan(old) && nanc > 0) nanc--;
        buf[head] = v;
        if (isnan(v)) nanc++;
        head = head + 1 == period ? 0 : head + 1;
        if (!filled) {
            if (head != 0) continue;
            filled = 1;
        }
        if (nanc != 0) continue;
        double s = 0.0;
        size_t idx = head;
        for (size_t j = 0; j < period; j++) {
            s += w[j] * buf[idx];
            idx = idx + 1 == period ? 0 : idx + 1;
        }
        out[t] = s;
    }
    free(w);
    free(buf);
    return VTO_OK;
}

/* SrwmaStream (srwma.rs:1183-1290): weights sqrt(p - k), k = 0..p-2, newest
 * first; output once more than p + 1 values were seen: four mul_add
 * accumulators over blocks of 4, the tail into the first, times 1 / sum of
 * weights.  Period 1 passes the value through after two bars. */
int vto_srwma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period == 0) return VTO_E_INVALID_PERIOD;
    const size_t m = period - 1;
    double *w = (double *)malloc(sizeof(double) * (m ? m : 1)), *ring = (double *)calloc(m ? m : 1, sizeof(double));
    double sumw = 0.0;
    for (size_t k = 0; k < m; k++) { w[k] = sqrt((double)(period - k)); sumw += w[k]; }
    const double inv = sumw == 0.0 ? 0.0 : 1.0 / sumw;
    size_t head = 0, count = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        out[t] = QNAN;
        count++;
        if (m == 0) { if (count > period + 1) out[t] = v; continue; }
        ring[head] = v;
        head = head + 1 == m ? 0 : head + 1;
        if (count <= period + 1) continue;
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        size_t k = 0;
        /* newest first: ring[(head - 1 - k) mod m] */
        for (; k + 4 <= m; k += 4) {
            s0 = fma(ring[(head + 2 * m - 1 - k) % m], w[k], s0);
            s1 = fma(ring[(head + 2 * m - 2 - k) % m], w[k + 1], s1);
            s2 = fma(ring[(head + 2 * m - 3 - k) % m], w[k + 2], s2);
            s3 = fma(ring[(head + 2 * m - 4 - k) % m], w[k + 3], s3);
        }
        for (; k < m; k++) s0 = fma(ring[(head + 2 * m - 1 - k) % m], w[k], s0);
        out[t] = ((s0 + s1) + (s2 + s3)) * inv;
    }
    free(w);
    free(ring);
    return VTO_OK;
}

/* SqwmaStream (sqwma.rs:360-545): weights (p - i)^2, i = 0..p-2, newest
 * first; output once p + 2 values were seen; REBASE_MASK = 0 rebuilds the
 * sum from the ring on every bar (one mul_add chain), so that sum is the
 * output, times 1 / sum of weights. */
int vto_sqwma_stream(const double *x, size_t n, size_t period, double *out) {
    if (period < 2) return VTO_E_INVALID_PERIOD;
    const size_t m = period - 1;
    double *w = (double *)malloc(sizeof(double) * m), *ring = (double *)calloc(period, sizeof(double));
    double ws = 0.0;
    for (size_t i = 0; i < m; i++) { double d = (double)period - (double)i; w[i] = d * d; ws += w[i]; }
    const double inv = 1.0 / ws;
    size_t head = 0, count = 0;
    for (size_t t = 0; t < n; t++) {
        out[t] = QNAN;
        ring[head] = x[t];
        head = head + 1 == period ? 0 : head + 1;
        count++;
        if (count < period + 2) continue;
        double r = 0.0;
        for (size_t i = 0; i < m; i++) r = fma(ring[(head + period - 1 - i) % period], w[i], r);
        out[t] = r * inv;
    }
    free(w);
    free(ring);
    return VTO_OK;
}

/* EpmaStream (epma.rs:635-735): Kahan-compensated running sum and ramp of
 * the last p - 1 values; during the first p + offset + 1 bars update()
 * returns the value itself; then mul_add(c0, sum, ramp) / wsum with
 * c0 = 2 - offset, wsum = mul_add(p - 1, c0, (p - 2)(p - 1) / 2). */
static void kahan(double *s, double *c, double v) {
    double y = v - *c;
    double t = *s + y;
    *c = (t - *s) - y;
    *s = t;
}

int vto_epma_stream(const double *x, size_t n, size_t period, size_t offset, double *out) {
    if (period < 2) return VTO_E_INVALID_PERIOD;
    if (offset >= period) return VTO_E_INVALID_PARAM;
    const size_t p1 = period - 1;
    const double c0 = 2.0 - (double)offset, p1f = (double)p1, p1m1 = (double)(p1 - 1);
    const double inv_wsum = 1.0 / fma(p1f, c0, 0.5 * (p1f - 1.0) * p1f);
    double *buf = (double *)calloc(period, sizeof(double));
    size_t head = 0, seen = 0, inc = 0;
    double sum = 0.0, sc = 0.0, ramp = 0.0, rc = 0.0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        double xo = inc == p1 ? buf[(head + 1) % period] : 0.0;
        buf[head] = v;
        head = (head + 1) % period;
        seen++;
        if (inc < p1) {
            double mm = (double)inc;
            kahan(&sum, &sc, v);
            kahan(&ramp, &rc, mm * v);
            inc++;
        } else {
            double s_old = sum;
            kahan(&sum, &sc, v - xo);
            kahan(&ramp, &rc, fma(p1m1, v, xo - s_old));
        }
        out[t] = seen <= period + offset + 1 ? v : fma(c0, sum, ramp) * inv_wsum;
    }
    free(buf);
    return VTO_OK;
}

/* VpwmaStream (vpwma.rs:583-884): weights (p - k)^power, k = 0..p-2, newest
 * first, over 1 / their sum; output once p values were seen.  A power within
 * 1e-12 of an integer deg in 0..8 runs the crate's PolyInt mode: moments
 * m_j = sum k^j x (k = age, 0 newest) built from the ring on the first
 * output, then shifted each bar by binomial sums, output dot(coeff, m) with
 * coeff_j = (-1)^j C(deg, j) p^(deg - j); any other power the ExactDot mode:
 * the window oldest first against the reversed weights as two ring segments,
 * each with four mul_add accumulators.  Integer powers of p by binary
 * exponentiation (the LLVM runtime's powi). */
static double powi_bin(double a, int b) {
    double r = 1.0;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return r;
}

static double binom_f(size_t n, size_t k) {
    if (k == 0 || k == n) return 1.0;
    if (k > n - k) k = n - k;
    unsigned long long num = 1, den = 1;
    for (size_t i = 1; i <= k; i++) { num *= (unsigned long long)(n + 1 - i); den *= (unsigned long long)i; }
    return (double)num / (double)den;
}

static double dot4(const double *a, const double *b, size_t n) {
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    size_t i = 0, p4 = n & ~(size_t)3;
    for (; i < p4; i += 4) {
        s0 = fma(a[i], b[i], s0);
        s1 = fma(a[i + 1], b[i + 1], s1);
        s2 = fma(a[i + 2], b[i + 2], s2);
        s3 = fma(a[i + 3], b[i + 3], s3);
    }
    for (; i < n; i++) s0 = fma(a[i], b[i], s0);
    return (s0 + s1) + (s2 + s3);
}

int vto_vpwma_stream(const double *x, size_t n, size_t period, double power, double *out) {
    if (period < 2) return VTO_E_INVALID_PERIOD;
    if (isnan(power) || isinf(power)) return VTO_E_INVALID_PARAM;
    const size_t m = period - 1;
    double *w = (double *)malloc(sizeof(double) * m), *buf = (double *)malloc(sizeof(double) * period);
    double norm = 0.0;
    for (size_t k = 0; k < m; k++) { w[k] = pow((double)period - (double)k, power); norm += w[k]; }
    const double inv_norm = 1.0 / norm;
    for (size_t i = 0; i < period; i++) buf[i] = QNAN;
    const double pr = round(power);
    const int poly = fabs(power - pr) <= 1e-12 && pr >= 0.0 && pr <= 8.0;
    const size_t deg = poly ? (size_t)pr : 0;
    double coeff[9], bv[45], pm1[9], mom[9], nxt[9];
    size_t rs[10];
    if (poly) {
        for (size_t j = 0; j <= deg; j++)
            coeff[j] = ((j & 1) ? -1.0 : 1.0) * binom_f(deg, j) * powi_bin((double)period, (int)(deg - j));
        size_t c = 0;
        for (size_t j = 0; j <= deg; j++) {
            rs[j] = c;
            for (size_t q = 0; q <= j; q++) bv[c++] = binom_f(j, q);
        }
        double pp = 1.0, mm1 = (double)(m - 1);
        for (size_t q = 0; q <= deg; q++) { pm1[q] = pp; pp *= mm1; }
    }
    size_t head = 0;
    int filled = 0, ready = 0;
    for (size_t t = 0; t < n; t++) {
        double v = x[t];
        out[t] = QNAN;
        buf[head] = v;
        head = (head + 1) % period;
        if (!filled && head == 0) filled = 1;
        if (!filled) continue;
        const size_t oldest = (head + 1) % period;
        const size_t left = period - oldest < m ? period - oldest : m, right = m - left;
        if (poly) {
            double xo = buf[head];
            if (!ready) {
                for (size_t j = 0; j <= deg; j++) mom[j] = 0.0;
                for (size_t pos = 0; pos < left; pos++) {
                    double xv = buf[oldest + pos], kk = (double)(m - 1 - pos), kp = 1.0;
                    for (size_t j = 0; j <= deg; j++) { mom[j] += kp * xv; kp *= kk; }
                }
                for (size_t pos = 0; pos < right; pos++) {
                    double xv = buf[pos], kk = (double)(right - 1 - pos), kp = 1.0;
                    for (size_t j = 0; j <= deg; j++) { mom[j] += kp * xv; kp *= kk; }
                }
                ready = 1;
            } else {
                nxt[0] = mom[0] + v - xo;
                for (size_t j = 1; j <= deg; j++) {
                    double s = 0.0;
                    for (size_t q = 0; q <= j; q++) s += bv[rs[j] + q] * (mom[q] - pm1[q] * xo);
                    nxt[j] = s;
                }
                for (size_t j = 0; j <= deg; j++) mom[j] = nxt[j];
            }
            out[t] = dot4(coeff, mom, deg + 1) * inv_norm;
        } else {
            /* weights_rev[i] = w[m - 1 - i] */
            double s0 = 0, s1 = 0, s2 = 0, s3 = 0, sum;
            size_t k = 0, p4 = left & ~(size_t)3;
            for (; k < p4; k += 4) {
                s0 = fma(buf[oldest + k], w[m - 1 - k], s0);
                s1 = fma(buf[oldest + k + 1], w[m - 2 - k], s1);
                s2 = fma(buf[oldest + k + 2], w[m - 3 - k], s2);
                s3 = fma(buf[oldest + k + 3], w[m - 4 - k], s3);
            }
            for (; k < left; k++) s0 = fma(buf[oldest + k], w[m - 1 - k], s0);
            sum = (s0 + s1) + (s2 + s3);
            if (right) {
                s0 = s1 = s2 = s3 = 0;
                k = 0;
                p4 = right & ~(size_t)3;
                for (; k < p4; k += 4) {
                    s0 = fma(buf[k], w[m - 1 - (left + k)], s0);
                    s1 = fma(buf[k + 1], w[m - 2 - (left + k)], s1);
                    s2 = fma(buf[k + 2], w[m - 3 - (left + k)], s2);
                    s3 = fma(buf[k + 3], w[m - 4 - (left + k)], s3);
                }
                for (; k < right; k++) s0 = fma(buf[k], w[m - 1 - (left + k)], s0);
                sum += (s0 + s1) + (s2 + s3);
            }
            out[t] = sum * inv_norm;
        }
    }
    free(w);
    free(buf);
    return VTO_OK;
}

/* PercentileNearestRankStream (percentile_nearest_rank.rs:468-665): two
 * heaps with lazy deletion keep the window's valid (non-NaN) values split at
 * the target rank; the output is the left heap's top, i.e. the k-th smallest
 * valid value, k = nearest_rank(p / 100, valid) + 1 with
 * nearest_rank(f, n) = clamp(trunc(mul_add(f, n, 0.5)) - 1, 0, n - 1);
 * NaN when the window has no valid value.  Restated here by sorting. */
static int cmp_d(const void *a, const void *b) {
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y ? 1 : 0;
}

int vto_percentile_nearest_rank_stream(const double *x, size_t n, size_t length, double percentage, double *out) {
    if (length == 0) return VTO_E_INVALID_PERIOD;
    if (!(percentage >= 0.0 && percentage <= 100.0)) return VTO_E_INVALID_PARAM;
    const double pf = percentage * 0.01;
    double *buf = (double *)malloc(sizeof(double) * length), *tmp = (double *)malloc(sizeof(double) * length);
    for (size_t i = 0; i < length; i++) buf[i] = QNAN;
    size_t head = 0;
    int filled = 0;
    for (size_t t = 0; t < n; t++) {
        out[t] = QNAN;
        buf[head] = x[t];
        head = (head + 1) % length;
        if (!filled && head == 0) filled = 1;
        if (!filled) continue;
        size_t valid = 0;
        for (size_t i = 0; i < length; i++)
            if (!isnan(buf[i])) tmp[valid++] = buf[i];
        if (valid == 0) continue;
        double kf = fma(pf, (double)valid, 0.5);
        size_t k = kf > 0.0 ? (size_t)kf : 0;
        k = k == 0 ? 0 : (k - 1 >= valid ? valid - 1 : k - 1);
        qsort(tmp, valid, sizeof(double), cmp_d);
        out[t] = tmp[k];
    }
    free(buf);
    free(tmp);
    return VTO_OK;
}

/* vpwma_with_kernel (vpwma.rs:215-290): weights (p - k)^power, k < p - 1
 * (newest first), inv_norm = 1 / sum, first output first + p - 1;
 * vpwma_scalar (vpwma.rs:296-360): four mul_add accumulators, two rounds per
 * block of 8, then a block of 4, then up to three more (one per
 * accumulator), summed as (s0 + s1) + (s2 + s3). */
int vto_vpwma(const double *x, size_t n, size_t period, double power, double *out) {
    if (n == 0) return VTO_E_EMPTY;
    size_t first = first_valid(x, n);
    if (first >= n) return VTO_E_ALL_NAN;
    if (period < 2 || period > n) return VTO_E_INVALID_PERIOD;
    if (n - first < period) return VTO_E_NOT_ENOUGH_VALID;
    if (!isfinite(power)) return VTO_E_INVALID_PARAM;
    const size_t wl = period - 1;
    double *w = (double *)malloc(sizeof(double) * wl);
    double norm = 0.0;
    for (size_t k = 0; k < wl; k++) {
        w[k] = pow((double)period - (double)k, power);
        norm += w[k];
    }
    const double inv = 1.0 / norm;
    fill_nan(out, first + wl < n ? first + wl : n);
    const size_t p8 = wl & ~(size_t)7, p4 = wl & ~(size_t)3;
    for (size_t i = first + wl; i < n; i++) {
        double s[4] = {0, 0, 0, 0};
        size_t k = 0;
        for (; k < p8; k += 8)
            for (int j = 0; j < 8; j++) s[j & 3] = fma(x[i - (k + j)], w[k + j], s[j & 3]);
        for (; k < p4; k += 4)
            for (int j = 0; j < 4; j++) s[j] = fma(x[i - (k + j)], w[k + j], s[j]);
        for (int j = 0; k + j < wl; j++) s[j] = fma(x[i - (k + j)], w[k + j], s[j]);
        out[i] = ((s[0] + s[1]) + (s[2] + s[3])) * inv;
    }
    free(w);
    return VTO_OK;
}
