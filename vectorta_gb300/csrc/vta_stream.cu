// Banks of streaming indicators on the device (vta_streams_*): S independent
// streams of one indicator and parameter set, advanced together by one bar
// per call, one thread per stream.  Each stream follows the update rule of
// the crate's XStream struct bar for bar (cited per kind) in f64, with the
// crate's rounding: explicit __dadd_rn / __dmul_rn where the Rust code has
// separate operations (so nothing is contracted into an FMA), fma() where it
// calls mul_add.  The outputs are the f64 values rounded to f32, NaN where the
// crate's update() returns None.  The step after the batch entry points for
// live data: the state stays resident between calls.
//
// State is structure-of-arrays: eight f64 and four int slots per stream
// ([slot][stream]) whose meaning depends on the kind, plus a ring of
// ring_slots f64 values per stream ([slot][stream]) for the windowed kinds.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "vta_internal.h"

namespace {

enum StreamKind {
    SK_EMA = 0,
    SK_SMA,
    SK_ALMA,
    SK_RSI,
    SK_ATR,
    SK_WILDERS,
    SK_DEMA,
    SK_TEMA,
    SK_WMA,
    SK_SWMA,
    SK_PWMA,
    SK_STDDEV,
    SK_ZSCORE,
    SK_BOLLINGER,
    SK_DONCHIAN,
    SK_WILLR,
    SK_ADX,
    SK_SUPERTREND,
    SK_SINWMA,
    SK_TRIMA,
    SK_CWMA,
    SK_FWMA,
    SK_SRWMA,
    SK_SQWMA,
    SK_EPMA,
    SK_VPWMA,
    SK_PERCENTILE,
    SK_COUNT
};

struct KindInfo {
    const char* name;
    int n_in, n_out;
    double period;  // the crate's default period (XParams / XStream::try_new)
};

// inputs: 1 = value; 2 = (high, low); 3 = (high, low, close)
constexpr KindInfo kKinds[SK_COUNT] = {
    {"ema", 1, 1, 9},
    {"sma", 1, 1, 9},
    {"alma", 1, 1, 9},
    {"rsi", 1, 1, 14},
    {"atr", 3, 1, 14},
    {"wilders", 1, 1, 5},
    {"dema", 1, 1, 30},
    {"tema", 1, 1, 9},
    {"wma", 1, 1, 30},
    {"swma", 1, 1, 5},
    {"pwma", 1, 1, 5},
    {"stddev", 1, 1, 5},
    {"zscore", 1, 1, 14},
    {"bollinger_bands", 1, 3, 20},
    {"donchian", 2, 3, 20},
    {"willr", 3, 1, 14},
    {"adx", 3, 1, 14},
    {"supertrend", 3, 2, 10},
    {"sinwma", 1, 1, 14},
    {"trima", 1, 1, 30},
    {"cwma", 1, 1, 14},
    {"fwma", 1, 1, 5},
    {"srwma", 1, 1, 14},
    {"sqwma", 1, 1, 14},
    {"epma", 1, 1, 11},
    {"vpwma", 1, 1, 14},
    {"percentile_nearest_rank", 1, 1, 15},
};

constexpr int kD = 10, kI = 4;

// VPWMA integer-power constants in the weight array: coeff at 0, (m - 1)^q at
// kVpPow, binomial row j at kVpBinom + j (j + 1) / 2
constexpr int kVpPow = 9, kVpBinom = 18, kVpConsts = kVpBinom + 45;

struct StreamState {
    int kind, n, period, n_out;
    int ka, kb;   // SWMA box lengths; TRIMA m1, m2
    int offset;   // EPMA offset
    int deg;      // VPWMA: integer power (moment mode), -1 = exact dot
    int ema_mid;  // Bollinger: EMA middle band (else SMA)
    int ring_slots;
    double alpha, beta, inv_p, inv_norm;
    double nbdev, devup, devdn, factor;
    double k[5];  // SINWMA cos a, sin a, cos pa, sin pa, 1 / sum of sines; EPMA c0, 1 / wsum,
                  // p - 2; percentile p / 100
    const double* w;  // ALMA weights (device)
    double* d[kD];    // per-stream f64 state
    int* iv[kI];      // per-stream int state
    double* ring;     // [ring_slots][n]
};

__device__ __forceinline__ double dnan() { return __longlong_as_double(0x7ff8000000000000ll); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }

__global__ void k_stream_init(StreamState s) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= s.n) return;
    const double nan = dnan();
    for (int k = 0; k < kI; ++k) s.iv[k][j] = 0;
    for (int k = 0; k < kD; ++k) s.d[k][j] = 0.0;
    switch (s.kind) {
        case SK_EMA:  // mean
        case SK_RSI:  // prev
        case SK_TEMA:  // ema1
            s.d[0][j] = nan;
            break;
        case SK_ATR:         // prev_close, rma
        case SK_DEMA:        // ema, ema2
        case SK_SUPERTREND:  // (ATR) prev_close, rma
            s.d[0][j] = nan;
            s.d[1][j] = nan;
            if (s.kind == SK_SUPERTREND) s.d[3][j] = s.d[4][j] = s.d[5][j] = nan;  // previous bands, close
            break;
        case SK_WILDERS: s.d[1][j] = nan; break;                       // last
        case SK_ADX: s.d[5][j] = s.d[6][j] = s.d[7][j] = nan; break;  // previous high, low, close
        case SK_ZSCORE:  // nan_count
        case SK_SINWMA:
            s.iv[2][j] = s.period;
            break;
        default: break;
    }
    if (s.ring) {
        const bool zero = s.kind == SK_SWMA || s.kind == SK_BOLLINGER || s.kind == SK_SRWMA || s.kind == SK_SQWMA ||
                          s.kind == SK_EPMA;
        const double fill = zero ? 0.0 : nan;
        for (int k = 0; k < s.ring_slots; ++k) s.ring[(size_t)k * s.n + j] = fill;
    }
}

// AtrStream::update (atr.rs): TR = h - l while prev_close is NaN, else
// max(h, pc) - min(l, pc) by comparisons; seed = sum of the first `length`
// TRs times 1/length; then mul_add(alpha, tr - rma, rma).  Slots d0
// prev_close, d1 rma, d2 warm_sum, i0 warm_count, i1 seeded.  Returns false
// while update() returns None.
__device__ __forceinline__ bool atr_step(const StreamState& s, int j, double h, double l, double cl, double& y) {
    const double pc = s.d[0][j];
    double tr;
    if (isnan(pc)) {
        tr = dsub(h, l);
    } else {
        const double up = h > pc ? h : pc;
        const double dn = l < pc ? l : pc;
        tr = dsub(up, dn);
    }
    s.d[0][j] = cl;
    if (!s.iv[1][j]) {
        s.d[2][j] = dadd(s.d[2][j], tr);
        const int cnt = s.iv[0][j] + 1;
        s.iv[0][j] = cnt;
        if (cnt == s.period) {
            const double rma = dmul(s.d[2][j], s.alpha);
            s.d[1][j] = rma;
            s.iv[1][j] = 1;
            y = rma;
            return true;
        }
        return false;
    }
    const double rma = fma(s.alpha, dsub(tr, s.d[1][j]), s.d[1][j]);
    s.d[1][j] = rma;
    y = rma;
    return true;
}

template <int K>
__global__ void k_stream_update(StreamState s, const float* __restrict__ a, const float* __restrict__ b,
                                const float* __restrict__ c, float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= s.n) return;
    const int p = s.period;
    const double nan = dnan();
    double y = nan, y1 = nan, y2 = nan;  // outputs 0..2
#define D(k) s.d[k][j]
#define IV(k) s.iv[k][j]
#define RING(k) s.ring[(size_t)(k) * s.n + j]
    if constexpr (K == SK_EMA) {  // EmaStream::update, ema.rs:560-585
        const double v = (double)a[j];
        if (!isfinite(v)) {
            y = IV(1) ? D(0) : nan;
        } else {
            const int cnt = IV(0) + 1;
            IV(0) = cnt;
            double mean = D(0);
            if (cnt == 1) mean = v;
            else if (cnt <= p) mean = fma(dsub(v, mean), ddiv(1.0, (double)cnt), mean);
            else mean = fma(s.beta, mean, dmul(s.alpha, v));
            D(0) = mean;
            if (!IV(1) && cnt >= p) IV(1) = 1;
            y = IV(1) ? mean : nan;
        }
    } else if constexpr (K == SK_SMA) {  // SmaStream::update (sma.rs)
        const double v = (double)a[j];
        if (p == 1) {
            y = v;
        } else {
            int head = IV(1);
            const int cnt = IV(0);
            double sum = D(0);
            if (cnt < p) {
                sum = dadd(sum, v);
                RING(head) = v;
                head = head + 1 == p ? 0 : head + 1;
                IV(0) = cnt + 1;
                y = cnt + 1 == p ? dmul(sum, s.inv_p) : nan;
            } else {
                const double old = RING(head);
                sum = dadd(sum, dsub(v, old));
                RING(head) = v;
                head = head + 1 == p ? 0 : head + 1;
                y = dmul(sum, s.inv_p);
            }
            D(0) = sum;
            IV(1) = head;
        }
    } else if constexpr (K == SK_ALMA) {  // AlmaStream::update / dot_at_head, alma.rs:865-964
        const double v = (double)a[j];
        int head = IV(1);
        RING(head) = v;
        head = head + 1 == p ? 0 : head + 1;
        IV(1) = head;
        int filled = IV(0);
        if (filled < p) IV(0) = ++filled;
        if (filled >= p) {
            // window oldest first = ring[(head + i) % p]; four accumulators
            // over blocks of 4, then the tail (dot_scalar_unrolled_safe)
            double acc[4] = {0.0, 0.0, 0.0, 0.0};
            const int p4 = p & ~3;
            int i = 0;
            for (; i < p4; i += 4)
                for (int q = 0; q < 4; ++q) {
                    int slot = head + i + q;
                    if (slot >= p) slot -= p;
                    acc[q] = dadd(acc[q], dmul(RING(slot), s.w[i + q]));
                }
            double sum = dadd(dadd(acc[0], acc[1]), dadd(acc[2], acc[3]));
            for (; i < p; ++i) {
                int slot = head + i;
                if (slot >= p) slot -= p;
                sum = dadd(sum, dmul(RING(slot), s.w[i]));
            }
            y = dmul(sum, s.inv_norm);
        }
    } else if constexpr (K == SK_RSI) {  // RsiStream::update (rsi.rs)
        const double v = (double)a[j];
        if (!IV(1)) {
            D(0) = v;
            IV(1) = 1;
        } else {
            const double d = dsub(v, D(0));
            D(0) = v;
            const double g = fmax(d, 0.0), l = fmax(-d, 0.0);  // f64::max ignores NaN
            const bool seeded = (IV(2) & 2) != 0;                  // i2: bit 0 poisoned, bit 1 seeded
            if (!seeded) {
                int poisoned = IV(2) & 1;
                if (!isfinite(d)) poisoned = 1;
                D(1) = dadd(D(1), g);
                D(2) = dadd(D(2), l);
                const int cnt = IV(0) + 1;
                IV(0) = cnt;
                if (cnt == p) {
                    if (poisoned) {
                        D(3) = nan;
                        D(4) = nan;
                        y = nan;
                    } else {
                        const double ag = dmul(D(1), s.inv_p), al = dmul(D(2), s.inv_p);
                        D(3) = ag;
                        D(4) = al;
                        const double den = dadd(ag, al);
                        y = den == 0.0 ? 50.0 : ddiv(dmul(100.0, ag), den);
                    }
                    IV(2) = poisoned | 2;
                } else {
                    IV(2) = poisoned;
                }
            } else {
                const double ag = fma(D(3), s.beta, dmul(s.inv_p, g));
                const double al = fma(D(4), s.beta, dmul(s.inv_p, l));
                D(3) = ag;
                D(4) = al;
                const double den = dadd(ag, al);
                y = den == 0.0 ? 50.0 : ddiv(dmul(100.0, ag), den);
            }
        }
    } else if constexpr (K == SK_ATR) {
        atr_step(s, j, (double)a[j], (double)b[j], (double)c[j], y);
    } else if constexpr (K == SK_WILDERS) {  // WildersStream::update (wilders.rs)
        const double v = (double)a[j];
        if (!IV(1)) {
            if (!isfinite(v)) {
                D(0) = 0.0;
                IV(0) = 0;
            } else {
                const double sum = dadd(D(0), v);
                D(0) = sum;
                const int cnt = IV(0) + 1;
                IV(0) = cnt;
                if (cnt >= p) {
                    const double y0 = ddiv(sum, (double)p);
                    D(1) = y0;
                    IV(1) = 1;
                    y = y0;
                }
            }
        } else {
            const double last = fma(dsub(v, D(1)), s.alpha, D(1));
            D(1) = last;
            y = last;
        }
    } else if constexpr (K == SK_DEMA) {
        // DemaStream::update (dema.rs:657-687), fmadd = mul_add (x86
        // targets): d0 ema, d1 ema2, i0 filled
        const double v = (double)a[j];
        if (IV(0) == 0) {
            D(0) = v;
            D(1) = v;
            IV(0) = 1;
            y = p == 1 ? v : nan;
        } else {
            const double e1 = fma(D(0), s.beta, dmul(v, s.alpha));
            const double e2 = fma(D(1), s.beta, dmul(e1, s.alpha));
            D(0) = e1;
            D(1) = e2;
            const double yy = fma(e1, 2.0, -e2);
            const int f = IV(0) < INT32_MAX ? IV(0) + 1 : IV(0);
            IV(0) = f;
            y = f > p - 1 ? yy : nan;
        }
    } else if constexpr (K == SK_TEMA) {
        // TemaStream::update (tema.rs:378-424): d0..d2 ema1..ema3, i0 count,
        // i1 ready; e = e (1 - a) + v a without FMA
        const double v = (double)a[j];
        double e1 = D(0), e2 = D(1), e3 = D(2);
        if (IV(1)) {
            e1 = dadd(dmul(e1, s.beta), dmul(v, s.alpha));
            e2 = dadd(dmul(e2, s.beta), dmul(e1, s.alpha));
            e3 = dadd(dmul(e3, s.beta), dmul(e2, s.alpha));
            y = dadd(dsub(dmul(3.0, e1), dmul(3.0, e2)), e3);
        } else if (IV(0) == 0) {
            if (!isnan(v)) {
                e1 = v;
                IV(0) = 1;
                if (p == 1) {
                    e2 = e1;
                    e3 = e2;
                    IV(1) = 1;
                    y = e1;
                }
            }
        } else {
            e1 = dadd(dmul(e1, s.beta), dmul(v, s.alpha));
            const int cnt = IV(0) + 1;
            IV(0) = cnt;
            const int start2 = p, start3 = 2 * p - 1, lookback = 3 * (p - 1);
            if (cnt == start2) e2 = e1;
            else if (cnt > start2) e2 = dadd(dmul(e2, s.beta), dmul(e1, s.alpha));
            if (cnt == start3) e3 = e2;
            else if (cnt > start3) e3 = dadd(dmul(e3, s.beta), dmul(e2, s.alpha));
            if (cnt > lookback) {
                IV(1) = 1;
                y = dadd(dsub(dmul(3.0, e1), dmul(3.0, e2)), e3);
            }
        }
        D(0) = e1;
        D(1) = e2;
        D(2) = e3;
    } else if constexpr (K == SK_WMA) {
        // WmaStream::update (wma.rs:420-459): ring of p values, i0 head,
        // i1 filled, d0 plain_sum, d1 weighted_sum
        const double v = (double)a[j];
        int head = IV(0);
        RING(head) = v;
        head = head + 1 == p ? 0 : head + 1;
        IV(0) = head;
        if (!IV(1)) {
            if (head == 0) {
                double ws = 0.0, ss = 0.0;
                for (int w = 1; w <= p; ++w) {  // oldest first from slot 0
                    const double bv = RING(w - 1);
                    ss = dadd(ss, bv);
                    ws = dadd(ws, dmul((double)w, bv));
                }
                y = dmul(ws, s.inv_norm);
                D(1) = dsub(ws, ss);
                D(0) = dsub(ss, RING(0));
                IV(1) = 1;
            }
        } else {
            const double oldest = RING(head);
            const double ws = dadd(D(1), dmul((double)p, v));
            const double ps = dadd(D(0), v);
            y = dmul(ws, s.inv_norm);
            D(1) = dsub(ws, ps);
            D(0) = dsub(ps, oldest);
        }
    } else if constexpr (K == SK_SWMA) {
        // SwmaStream::update (swma.rs:595-630): ring_a = ring slots [0, a),
        // ring_b = [a, a + b); i0 idx_a, i1 cnt_a, i2 idx_b, i3 cnt_b,
        // d0 s1_sum, d1 s2_sum
        const double v = (double)a[j];
        const int ka = s.ka, kb = s.kb;
        const int ia = IV(0);
        const double old_a = RING(ia);
        double s1 = D(0);
        int ca = IV(1);
        if (ca == ka) s1 = dsub(s1, old_a);
        else IV(1) = ++ca;
        RING(ia) = v;
        s1 = dadd(s1, v);
        D(0) = s1;
        IV(0) = ia + 1 == ka ? 0 : ia + 1;
        if (ca == ka) {
            const int ib = IV(2);
            const double old_b = RING(ka + ib);
            double s2 = D(1);
            int cb = IV(3);
            if (cb == kb) s2 = dsub(s2, old_b);
            else IV(3) = ++cb;
            RING(ka + ib) = s1;
            s2 = dadd(s2, s1);
            D(1) = s2;
            IV(2) = ib + 1 == kb ? 0 : ib + 1;
            if (cb == kb) y = dmul(s2, s.inv_norm);
        }
    } else if constexpr (K == SK_PWMA) {
        // PwmaStream::update (pwma.rs:712-733): cascade of p - 1 pairwise
        // running sums in the ring (prev, NaN at start), i0 seen
        const double v = (double)a[j];
        const int m = p - 1;
        if (m == 0) {
            y = v;
        } else {
            double acc = v;
            for (int k = 0; k < m; ++k) {
                const double o = dadd(acc, RING(k));
                RING(k) = acc;
                acc = o;
            }
            if (IV(0) < m) ++IV(0);
            else y = dmul(acc, s.inv_norm);
        }
    } else if constexpr (K == SK_STDDEV) {
        // StdDevStream::update (stddev.rs:490-569): ring, i0 head, i1 filled,
        // i2 nan_count, d0 sum, d1 sum_sqr
        const double v = (double)a[j];
        const int head = IV(0);
        bool emit = true;
        if (!IV(1)) {
            if (isnan(v)) {
                ++IV(2);
            } else {
                D(0) = dadd(D(0), v);
                D(1) = dadd(D(1), dmul(v, v));
            }
            RING(head) = v;
            if (head + 1 == p) {
                IV(0) = 0;
                IV(1) = 1;
            } else {
                IV(0) = head + 1;
                emit = false;
            }
        } else {
            const double old = RING(head);
            const bool nn = isnan(v), on = isnan(old);
            if (!on && !nn) {
                D(0) = dadd(D(0), dsub(v, old));
                D(1) = dadd(D(1), dsub(dmul(v, v), dmul(old, old)));
            } else if (!on && nn) {
                D(0) = dsub(D(0), old);
                D(1) = dsub(D(1), dmul(old, old));
                ++IV(2);
            } else if (on && !nn) {
                if (IV(2) > 0) --IV(2);
                D(0) = dadd(D(0), v);
                D(1) = dadd(D(1), dmul(v, v));
            } else {
                if (IV(2) > 0) --IV(2);
                ++IV(2);
            }
            RING(head) = v;
            IV(0) = head + 1 == p ? 0 : head + 1;
        }
        if (emit) {
            if (IV(2) > 0) {
                y = nan;
            } else {
                const double mean = dmul(D(0), s.inv_p);
                const double var = dsub(dmul(D(1), s.inv_p), dmul(mean, mean));
                y = var <= 0.0 ? 0.0 : dmul(dsqrt(var), s.nbdev);
            }
        }
    } else if constexpr (K == SK_ZSCORE) {
        // ZscoreStream::update (zscore.rs:657-735), MA "sma", devtype 0:
        // ring, i0 head, i1 filled, i2 nan_count (starts at p), d0 sum,
        // d1 sum2.  A window holding a NaN, or nbdev == 0, takes the crate's
        // slow path, whose result is NaN for this MA.
        const double v = (double)a[j];
        int head = IV(0);
        const double old = RING(head);
        RING(head) = v;
        head = head + 1 == p ? 0 : head + 1;
        IV(0) = head;
        if (!IV(1) && head == 0) IV(1) = 1;
        if (isnan(old) && IV(2) > 0) --IV(2);
        if (isnan(v)) ++IV(2);
        const double oc = isnan(old) ? 0.0 : old, nc = isnan(v) ? 0.0 : v;
        D(0) = dsub(dadd(D(0), nc), oc);
        D(1) = dsub(dadd(D(1), dmul(nc, nc)), dmul(oc, oc));
        if (IV(1) && s.nbdev != 0.0 && IV(2) == 0) {
            const double mean = dmul(D(0), s.inv_p), ex2 = dmul(D(1), s.inv_p);
            double var = dsub(ex2, dmul(mean, mean));
            if (var < 0.0) var = 0.0;
            const double sd = dsqrt(var);
            if (sd != 0.0 && isfinite(sd)) {
                const double last = RING(head == 0 ? p - 1 : head - 1);
                y = ddiv(dsub(last, mean), dmul(sd, s.nbdev));
            }
        }
    } else if constexpr (K == SK_BOLLINGER) {
        // BollingerBandsStream::update (bollinger_bands.rs:1022-1060), devtype
        // 0, SMA or EMA middle: ring, i0 idx, i1 len, i2 ema_seeded, d0 sum,
        // d1 sum_sq, d2 ema.  A non-finite value resets the stream.
        const double v = (double)a[j];
        if (!isfinite(v)) {
            IV(0) = IV(1) = IV(2) = 0;
            D(0) = D(1) = D(2) = 0.0;
        } else {
            const int idx = IV(0);
            const int len = IV(1);
            if (len < p) {
                RING(idx) = v;
                IV(1) = len + 1;
                D(0) = dadd(D(0), v);
                D(1) = fma(v, v, D(1));
            } else {
                const double old = RING(idx);
                RING(idx) = v;
                D(0) = dadd(D(0), dsub(v, old));
                const double tmp = dsub(D(1), dmul(old, old));
                D(1) = fma(v, v, tmp);
            }
            IV(0) = idx + 1 == p ? 0 : idx + 1;
            if (IV(1) >= p) {
                const double mean = dmul(D(0), s.inv_p);
                const double var = dsub(dmul(D(1), s.inv_p), dmul(mean, mean));
                const double sd = dsqrt(var > 0.0 ? var : 0.0);
                double mid = mean;
                if (s.ema_mid) {
                    if (!IV(2)) {
                        D(2) = dmul(D(0), s.inv_p);
                        IV(2) = 1;
                    } else {
                        D(2) = fma(s.alpha, v, dmul(s.beta, D(2)));
                    }
                    mid = D(2);
                }
                y = fma(s.devup, sd, mid);
                y1 = mid;
                y2 = fma(-s.devdn, sd, mid);
            }
        }
    } else if constexpr (K == SK_DONCHIAN) {
        // DonchianStream::update (donchian.rs:1302-1340): once p bars were
        // seen, NaN while the window holds a non-finite high or low, else the
        // window's highest high / lowest low (the monotone deques' fronts).
        // Ring slots [0, p) highs, [p, 2p) lows; i0 head, i1 seen (capped).
        const double h = (double)a[j], l = (double)b[j];
        const int head = IV(0);
        RING(head) = h;
        RING(p + head) = l;
        IV(0) = head + 1 == p ? 0 : head + 1;
        if (IV(1) < p) ++IV(1);
        if (IV(1) >= p) {
            bool ok = true;
            double mx = -INFINITY, mn = INFINITY;
            for (int k = 0; k < p; ++k) {
                const double hk = RING(k), lk = RING(p + k);
                ok = ok && isfinite(hk) && isfinite(lk);
                mx = hk > mx ? hk : mx;
                mn = lk < mn ? lk : mn;
            }
            if (ok) {
                y = mx;
                y1 = fma(dsub(mx, mn), 0.5, mn);
                y2 = mn;
            }
        }
    } else if constexpr (K == SK_WILLR) {
        // WillrStream::update (willr.rs:1709-1820): once p bars were seen,
        // NaN when the close is NaN or the window holds a NaN high or low or
        // its extremes are not finite; 0 for a flat window; else
        // mul_add(-100, (hh - close) / (hh - ll), 0).  Ring slots as Donchian.
        const double h = (double)a[j], l = (double)b[j], cl = (double)c[j];
        const int head = IV(0);
        RING(head) = h;
        RING(p + head) = l;
        IV(0) = head + 1 == p ? 0 : head + 1;
        if (IV(1) < p) ++IV(1);
        if (IV(1) >= p) {
            bool ok = !isnan(cl);
            double hh = -INFINITY, ll = INFINITY;
            for (int k = 0; k < p; ++k) {
                const double hk = RING(k), lk = RING(p + k);
                ok = ok && !isnan(hk) && !isnan(lk);
                hh = hk > hh ? hk : hh;
                ll = lk < ll ? lk : ll;
            }
            if (ok && isfinite(hh) && isfinite(ll)) {
                const double den = dsub(hh, ll);
                y = den == 0.0 ? 0.0 : fma(-100.0, ddiv(dsub(hh, cl), den), 0.0);
            }
        }
    } else if constexpr (K == SK_ADX) {
        // AdxStream::update (adx.rs:1988-2084): d0 atr, d1 +DM, d2 -DM
        // (smoothed), d3 dx_sum, d4 last_adx, d5..d7 previous high / low /
        // close; i0 count (capped at p + 2), i1 dx_count
        const double h = (double)a[j], l = (double)b[j], cl = (double)c[j];
        if (IV(0) == 0) {
            IV(0) = 1;
        } else {
            const double tr = dsub(fmax(h, D(7)), fmin(l, D(7)));
            const double upm = dsub(h, D(5)), dnm = dsub(D(6), l);
            const double pdm = (upm > dnm && upm > 0.0) ? upm : 0.0;
            const double mdm = (dnm > upm && dnm > 0.0) ? dnm : 0.0;
            const int cnt = IV(0) + 1;
            IV(0) = cnt < p + 2 ? cnt : p + 2;
            if (cnt <= p + 1) {
                D(0) = dadd(D(0), tr);
                D(1) = dadd(D(1), pdm);
                D(2) = dadd(D(2), mdm);
                if (cnt == p + 1) {
                    const double inv = D(0) != 0.0 ? ddiv(100.0, D(0)) : 0.0;
                    const double pdi = dmul(D(1), inv), mdi = dmul(D(2), inv), sdi = dadd(pdi, mdi);
                    D(3) = sdi != 0.0 ? dmul(ddiv(fabs(dsub(pdi, mdi)), sdi), 100.0) : 0.0;
                    IV(1) = 1;
                }
            } else {
                D(0) = dadd(dmul(D(0), s.beta), tr);
                D(1) = dadd(dmul(D(1), s.beta), pdm);
                D(2) = dadd(dmul(D(2), s.beta), mdm);
                const double inv = D(0) != 0.0 ? ddiv(100.0, D(0)) : 0.0;
                const double pdi = dmul(D(1), inv), mdi = dmul(D(2), inv), sdi = dadd(pdi, mdi);
                const double dx = sdi != 0.0 ? dmul(ddiv(fabs(dsub(pdi, mdi)), sdi), 100.0) : 0.0;
                if (IV(1) < p) {
                    D(3) = dadd(D(3), dx);
                    const int dc = IV(1) + 1;
                    IV(1) = dc;
                    if (dc == p) {
                        D(4) = dmul(D(3), s.inv_p);
                        y = D(4);
                    }
                } else {
                    D(4) = dmul(dadd(dmul(D(4), (double)p - 1.0), dx), s.inv_p);
                    y = D(4);
                }
            }
        }
        D(5) = h;
        D(6) = l;
        D(7) = cl;
    } else if constexpr (K == SK_SUPERTREND) {
        // SuperTrendStream::update (supertrend.rs:831-884) over the AtrStream
        // slots (d0..d2, i0, i1): d3 / d4 previous upper / lower band, d5
        // previous close, i2 upper_state, i3 warmed.  Outputs trend, changed.
        const double h = (double)a[j], l = (double)b[j], cl = (double)c[j];
        double atr;
        if (atr_step(s, j, h, l, cl, atr)) {
            const double hl2 = dmul(dadd(h, l), 0.5);
            const double ub = fma(s.factor, atr, hl2), lb = fma(-s.factor, atr, hl2);
            if (!IV(3)) {
                D(3) = ub;
                D(4) = lb;
                IV(2) = cl <= ub;
                y = IV(2) ? ub : lb;
                y1 = 0.0;
                D(5) = cl;
                IV(3) = 1;
            } else {
                double cu = ub, cb = lb;
                if (D(5) <= D(3)) cu = fmin(cu, D(3));
                if (D(5) >= D(4)) cb = fmax(cb, D(4));
                double ch = 0.0, tv;
                if (IV(2)) {
                    if (cl <= cu) {
                        tv = cu;
                    } else {
                        ch = 1.0;
                        IV(2) = 0;
                        tv = cb;
                    }
                } else {
                    if (cl >= cb) {
                        tv = cb;
                    } else {
                        ch = 1.0;
                        IV(2) = 1;
                        tv = cu;
                    }
                }
                D(3) = cu;
                D(4) = cb;
                D(5) = cl;
                y = tv;
                y1 = ch;
            }
        }
    } else if constexpr (K == SK_SINWMA) {
        // SinWmaStream::update (sinwma.rs:654-718): z = sum_j r^j x(newest - j)
        // with r = e^(i alpha); ring, i0 head, i1 filled, i2 nan_count (starts
        // at p), i3 z_valid, d0 / d1 z.  Rebuilt from the ring when the window
        // becomes NaN-free, else z' = r z + x_new - r^p x_old.
        const double v = (double)a[j];
        const double cosa = s.k[0], sina = s.k[1], cosp = s.k[2], sinp = s.k[3];
        int head = IV(0);
        const double old = RING(head);
        RING(head) = v;
        head = head + 1 == p ? 0 : head + 1;
        IV(0) = head;
        if (isnan(old) && IV(2) > 0) --IV(2);
        if (isnan(v)) ++IV(2);
        bool rebuild = false, emit = false;
        if (!IV(1)) {
            if (head == 0) {
                IV(1) = 1;
                if (IV(2) != 0) IV(3) = 0;
                else rebuild = emit = true;
            }
        } else if (IV(2) != 0) {
            IV(3) = 0;
        } else if (!IV(3)) {
            rebuild = emit = true;
        } else {
            const double zr = D(0), zi = D(1);
            const double rr = fma(cosa, zr, dmul(-sina, zi));
            const double ri = fma(cosa, zi, dmul(sina, zr));
            D(0) = dsub(dadd(rr, v), dmul(cosp, old));
            D(1) = dsub(ri, dmul(sinp, old));
            emit = true;
        }
        if (rebuild) {
            const int newest = head == 0 ? p - 1 : head - 1;
            double rj_re = 1.0, rj_im = 0.0, zr = 0.0, zi = 0.0;
            for (int q = 0; q < p; ++q) {
                int idx = newest - q;
                if (idx < 0) idx += p;
                const double xv = RING(idx);
                zr = fma(rj_re, xv, zr);
                zi = fma(rj_im, xv, zi);
                const double nr = fma(rj_re, cosa, dmul(-rj_im, sina));
                const double ni = fma(rj_re, sina, dmul(rj_im, cosa));
                rj_re = nr;
                rj_im = ni;
            }
            D(0) = zr;
            D(1) = zi;
            IV(3) = 1;
        }
        if (emit) y = dmul(fma(sinp, D(0), dmul(-cosp, D(1))), s.k[4]);
    } else if constexpr (K == SK_TRIMA) {
        // TrimaStream::update (trima.rs:876-905): SMA(m1) of the values (NaN
        // left out of the sum) in ring slots [0, m1), SMA(m2) of those means
        // in [m1, m1 + m2); i0 / i1 head1 / filled1, i2 / i3 head2 / filled2,
        // d0 / d1 sum1 / sum2
        const double v = (double)a[j];
        const int m1 = s.ka, m2 = s.kb;
        int h1 = IV(0);
        const double o1 = RING(h1);
        RING(h1) = v;
        if (++h1 == m1) {
            h1 = 0;
            IV(1) = 1;
        }
        IV(0) = h1;
        double s1 = D(0);
        if (!isnan(o1)) s1 = dsub(s1, o1);
        if (!isnan(v)) s1 = dadd(s1, v);
        D(0) = s1;
        if (IV(1)) {
            const double mean1 = dmul(s1, s.inv_p);
            int h2 = IV(2);
            const double o2 = RING(m1 + h2);
            RING(m1 + h2) = mean1;
            if (++h2 == m2) {
                h2 = 0;
                IV(3) = 1;
            }
            IV(2) = h2;
            double s2 = D(1);
            if (!isnan(o2)) s2 = dsub(s2, o2);
            s2 = dadd(s2, mean1);
            D(1) = s2;
            if (IV(3)) y = dmul(s2, s.inv_norm);
        }
    } else if constexpr (K == SK_CWMA) {
        // CwmaStream::update (cwma.rs:893-980): leading NaNs skipped; ring of
        // the last m = p - 1 values; i0 head, i1 filled (to m + 1), i2
        // nan_count, i3 found_first.  Output: NaN while the window holds a NaN,
        // else sum_weighted (mul_add chain newest first, weights (p + 1 - r)^3
        // in w) / sum of j^3; the crate's moments do not enter it.
        const double v = (double)a[j];
        const int m = p - 1;
        bool go = true;
        if (!IV(3)) {
            if (isnan(v)) go = false;
            else IV(3) = 1;
        }
        if (go) {
            int filled = IV(1), head = IV(0);
            const double old = filled >= m ? RING(head) : nan;
            const int new_nan = isnan(v) ? 1 : 0, old_nan = (filled >= m && isnan(old)) ? 1 : 0;
            RING(head) = v;
            head = head + 1 == m ? 0 : head + 1;
            IV(0) = head;
            bool emit = true;
            if (filled <= m) {
                IV(1) = ++filled;
                int nc = IV(2) + new_nan;
                if (filled == m + 1) nc -= old_nan;
                IV(2) = nc;
                emit = filled > m;
            } else {
                IV(2) = IV(2) + new_nan - old_nan;
            }
            if (emit && IV(2) == 0) {
                double acc = 0.0;
                int idx = head;
                for (int r = 1; r <= m; ++r) {  // newest first
                    idx = idx == 0 ? m - 1 : idx - 1;
                    acc = fma(RING(idx), s.w[r - 1], acc);
                }
                y = dmul(acc, s.inv_norm);
            }
        }
    } else if constexpr (K == SK_FWMA) {
        // FwmaStream::update (fwma.rs:814-875): ring, i0 head, i1 filled,
        // i2 nan_count; output the dot of the window (oldest first) with the
        // normalised Fibonacci weights in w, NaN while it holds a NaN
        const double v = (double)a[j];
        int head = IV(0);
        const double old = RING(head);
        if (IV(1) && isnan(old) && IV(2) > 0) --IV(2);
        RING(head) = v;
        if (isnan(v)) ++IV(2);
        head = head + 1 == p ? 0 : head + 1;
        IV(0) = head;
        bool emit = true;
        if (!IV(1)) {
            if (head != 0) emit = false;
            else IV(1) = 1;
        }
        if (emit && IV(2) == 0) {
            double acc = 0.0;
            int idx = head;
            for (int q = 0; q < p; ++q) {
                acc = dadd(acc, dmul(s.w[q], RING(idx)));
                idx = idx + 1 == p ? 0 : idx + 1;
            }
            y = acc;
        }
    } else if constexpr (K == SK_SRWMA) {
        // SrwmaStream::update (srwma.rs:1242-1290): ring of m = p - 1 values,
        // i0 head, i1 count (capped at p + 2); output once count > p + 1:
        // four mul_add accumulators newest first over blocks of 4, the tail in
        // the first; weights sqrt(p - k) in w
        const double v = (double)a[j];
        const int m = p - 1;
        const int cnt = IV(1) < p + 2 ? IV(1) + 1 : p + 2;
        IV(1) = cnt;
        if (m == 0) {
            if (cnt > p + 1) y = v;
        } else {
            int head = IV(0);
            RING(head) = v;
            head = head + 1 == m ? 0 : head + 1;
            IV(0) = head;
            if (cnt > p + 1) {
                double acc[4] = {0.0, 0.0, 0.0, 0.0};
                int idx = head, k = 0;  // idx walks newest first
                for (; k + 4 <= m; k += 4)
                    for (int q = 0; q < 4; ++q) {
                        idx = idx == 0 ? m - 1 : idx - 1;
                        acc[q] = fma(RING(idx), s.w[k + q], acc[q]);
                    }
                for (; k < m; ++k) {
                    idx = idx == 0 ? m - 1 : idx - 1;
                    acc[0] = fma(RING(idx), s.w[k], acc[0]);
                }
                y = dmul(dadd(dadd(acc[0], acc[1]), dadd(acc[2], acc[3])), s.inv_norm);
            }
        }
    } else if constexpr (K == SK_SQWMA) {
        // SqwmaStream::update (sqwma.rs:495-530) with REBASE_MASK = 0: every
        // output is the ring's mul_add chain newest first over the p - 1 most
        // recent values, weights (p - i)^2 in w; ring of p, i0 head, i1 count
        // (capped at p + 2), output once count >= p + 2
        const double v = (double)a[j];
        int head = IV(0);
        RING(head) = v;
        head = head + 1 == p ? 0 : head + 1;
        IV(0) = head;
        const int cnt = IV(1) < p + 2 ? IV(1) + 1 : p + 2;
        IV(1) = cnt;
        if (cnt >= p + 2) {
            double r = 0.0;
            int idx = head;
            for (int i = 0; i < p - 1; ++i) {
                idx = idx == 0 ? p - 1 : idx - 1;
                r = fma(RING(idx), s.w[i], r);
            }
            y = dmul(r, s.inv_norm);
        }
    } else if constexpr (K == SK_EPMA) {
        // EpmaStream::update (epma.rs:707-735): Kahan-compensated sum (d0, d1)
        // and ramp (d2, d3) of the last p - 1 values; ring of p, i0 head, i1
        // seen (capped), i2 included; the value itself during the first
        // p + offset + 1 bars, then mul_add(c0, sum, ramp) / wsum
        const double v = (double)a[j];
        const int p1 = p - 1;
        const int head = IV(0), inc = IV(2);
        int nx = head + 1 == p ? 0 : head + 1;
        const double xo = inc == p1 ? RING(nx) : 0.0;
        RING(head) = v;
        IV(0) = nx;
        const int cap = p + s.offset + 2;
        const int seen = IV(1) < cap ? IV(1) + 1 : cap;
        IV(1) = seen;
        auto kahan = [&](int si, int ci, double x) {
            const double yk = dsub(x, D(ci));
            const double tk = dadd(D(si), yk);
            D(ci) = dsub(dsub(tk, D(si)), yk);
            D(si) = tk;
        };
        if (inc < p1) {
            kahan(0, 1, v);
            kahan(2, 3, dmul((double)inc, v));
            IV(2) = inc + 1;
        } else {
            const double s_old = D(0);
            kahan(0, 1, dsub(v, xo));
            kahan(2, 3, fma(s.k[2], v, dsub(xo, s_old)));
        }
        y = seen <= p + s.offset + 1 ? v : dmul(fma(s.k[0], D(0), D(2)), s.k[1]);
    } else if constexpr (K == SK_VPWMA) {
        // VpwmaStream::update (vpwma.rs:684-750): ring of p (NaN at start), i0
        // head, i1 filled, i2 moments_ready; output once p values were seen.
        // deg >= 0: PolyInt moments d0..d_deg (age powers), shifted by
        // binomial sums; else ExactDot: the window oldest first against the
        // reversed weights as two ring segments of four accumulators each.
        const double v = (double)a[j];
        int head = IV(0);
        RING(head) = v;
        head = head + 1 == p ? 0 : head + 1;
        IV(0) = head;
        if (!IV(1) && head == 0) IV(1) = 1;
        if (IV(1)) {
            const int m = p - 1;
            const int oldest = head + 1 == p ? 0 : head + 1;
            const int left = min(p - oldest, m), right = m - left;
            if (s.deg >= 0) {
                const int dg = s.deg;
                double mo[9];
                if (!IV(2)) {
                    for (int q = 0; q <= dg; ++q) mo[q] = 0.0;
                    for (int pos = 0; pos < m; ++pos) {
                        const double xv = pos < left ? RING(oldest + pos) : RING(pos - left);
                        const double kk = pos < left ? (double)(m - 1 - pos) : (double)(right - 1 - (pos - left));
                        double kp = 1.0;
                        for (int q = 0; q <= dg; ++q) {
                            mo[q] = dadd(mo[q], dmul(kp, xv));
                            kp = dmul(kp, kk);
                        }
                    }
                    IV(2) = 1;
                } else {
                    const double xo = RING(head);
                    double nx[9];
                    for (int q = 0; q <= dg; ++q) mo[q] = D(q);
                    nx[0] = dsub(dadd(mo[0], v), xo);
                    for (int jj = 1; jj <= dg; ++jj) {
                        double acc = 0.0;
                        for (int q = 0; q <= jj; ++q)
                            acc = dadd(acc, dmul(s.w[kVpBinom + jj * (jj + 1) / 2 + q],
                                                 dsub(mo[q], dmul(s.w[kVpPow + q], xo))));
                        nx[jj] = acc;
                    }
                    for (int q = 0; q <= dg; ++q) mo[q] = nx[q];
                }
                for (int q = 0; q <= dg; ++q) D(q) = mo[q];
                double acc[4] = {0.0, 0.0, 0.0, 0.0};
                const int n4 = (dg + 1) & ~3;
                int i = 0;
                for (; i < n4; i += 4)
                    for (int q = 0; q < 4; ++q) acc[q] = fma(s.w[i + q], mo[i + q], acc[q]);
                for (; i <= dg; ++i) acc[0] = fma(s.w[i], mo[i], acc[0]);
                y = dmul(dadd(dadd(acc[0], acc[1]), dadd(acc[2], acc[3])), s.inv_norm);
            } else {
                // weights_rev[i] = w[m - 1 - i]
                double sum = 0.0;
                for (int seg = 0; seg < 2; ++seg) {
                    const int len = seg == 0 ? left : right, base = seg == 0 ? oldest : 0, wo = seg == 0 ? 0 : left;
                    if (seg == 1 && len == 0) break;
                    double acc[4] = {0.0, 0.0, 0.0, 0.0};
                    const int n4 = len & ~3;
                    int k = 0;
                    for (; k < n4; k += 4)
                        for (int q = 0; q < 4; ++q)
                            acc[q] = fma(RING(base + k + q), s.w[m - 1 - (wo + k + q)], acc[q]);
                    for (; k < len; ++k) acc[0] = fma(RING(base + k), s.w[m - 1 - (wo + k)], acc[0]);
                    const double part = dadd(dadd(acc[0], acc[1]), dadd(acc[2], acc[3]));
                    sum = seg == 0 ? part : dadd(sum, part);
                }
                y = dmul(sum, s.inv_norm);
            }
        }
    } else if constexpr (K == SK_PERCENTILE) {
        // PercentileNearestRankStream::update (percentile_nearest_rank.rs:
        // 665-700): once `length` values were seen, the k-th smallest valid
        // (non-NaN) value of the window, k = nearest_rank(p / 100, valid) + 1,
        // NaN with no valid value.  The crate's two heaps hold exactly that
        // value on top; here it is selected by counting (O(length^2)).
        const double v = (double)a[j];
        int head = IV(0);
        RING(head) = v;
        head = head + 1 == p ? 0 : head + 1;
        IV(0) = head;
        if (!IV(1) && head == 0) IV(1) = 1;
        if (IV(1)) {
            int valid = 0;
            for (int q = 0; q < p; ++q) valid += isnan(RING(q)) ? 0 : 1;
            if (valid > 0) {
                const double kf = fma(s.k[0], (double)valid, 0.5);
                long long k = kf > 0.0 ? (long long)kf : 0;  // kf <= valid + 0.5
                k = k == 0 ? 0 : (k - 1 >= valid ? valid - 1 : k - 1);
                for (int q = 0; q < p; ++q) {
                    const double xq = RING(q);
                    if (isnan(xq)) continue;
                    int less = 0, eq = 0;
                    for (int r = 0; r < p; ++r) {
                        const double xr = RING(r);
                        less += xr < xq ? 1 : 0;
                        eq += xr == xq ? 1 : 0;
                    }
                    if (less <= k && k < less + eq) {
                        y = xq;
                        break;
                    }
                }
            }
        }
    }
#undef D
#undef IV
#undef RING
    out[j] = (float)y;
    if (s.n_out > 1) out[(size_t)s.n + j] = (float)y1;
    if (s.n_out > 2) out[2 * (size_t)s.n + j] = (float)y2;
}

int kind_of(const char* name) {
    if (!name) return -1;
    std::string s(name);
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    if (s == "bollinger" || s == "bb") s = "bollinger_bands";
    for (int k = 0; k < SK_COUNT; ++k)
        if (s == kKinds[k].name) return k;
    return -1;
}

double param(const char* const* keys, const double* vals, size_t n, const char* key, double dflt) {
    for (size_t i = 0; i < n; ++i)
        if (keys && keys[i] && vals && std::strcmp(keys[i], key) == 0) return vals[i];
    return dflt;
}

template <int K>
void launch_update(const StreamState& s, cudaStream_t st, const float* a, const float* b, const float* c,
                   float* out) {
    k_stream_update<K><<<vta::ceil_div(s.n, 256), 256, 0, st>>>(s, a, b, c, out);
}

template <int... Ks>
void dispatch_update(std::integer_sequence<int, Ks...>, const StreamState& s, cudaStream_t st, const float* a,
                     const float* b, const float* c, float* out) {
    ((s.kind == Ks ? launch_update<Ks>(s, st, a, b, c, out) : void()), ...);
}

}  // namespace

struct vta_streams {
    vta_ctx* ctx = nullptr;
    StreamState s{};
    void* block = nullptr;  // one device allocation for all state
    float* d_io = nullptr;  // staging of the host-buffer update: inputs (3 n) + outputs (n_out n)
};

using namespace vta;

namespace {

vta_status enqueue_update(vta_streams* S, const float* a, const float* b, const float* c, float* out) {
    dispatch_update(std::make_integer_sequence<int, SK_COUNT>{}, S->s, S->ctx->stream, a, b, c, out);
    return check_launch("k_stream_update");
}

bool inputs_ok(const vta_streams* S, const float* a, const float* b, const float* c) {
    const int n_in = kKinds[S->s.kind].n_in;
    return a && (n_in < 2 || b) && (n_in < 3 || c);
}

}  // namespace

extern "C" {

vta_status vta_streams_create(vta_ctx* ctx, const char* indicator, const char* const* param_keys,
                              const double* param_values, size_t n_params, size_t n_streams, vta_streams** out) {
    if (!out) return fail(VTA_ERR_INVALID_INPUT, "streams: null out");
    *out = nullptr;
    VTA_TRY(enter_call(ctx));
    const int kind = kind_of(indicator);
    if (kind < 0) return fail(VTA_ERR_NOT_IMPLEMENTED, std::string("streams: no streaming kernel for ") +
                                                           (indicator ? indicator : "(null)"));
    if (n_streams == 0 || n_streams > (size_t)INT32_MAX) return fail(VTA_ERR_INVALID_INPUT, "streams: bad count");
    const KindInfo& info = kKinds[kind];
    auto P = [&](const char* key, double dflt) { return param(param_keys, param_values, n_params, key, dflt); };
    double pd = P("period", info.period);
    if (kind == SK_ATR || kind == SK_PERCENTILE) pd = P("length", pd);
    if (!(pd >= 1.0) || pd != std::floor(pd) || pd > 1e6)
        return fail(VTA_ERR_INVALID_INPUT, "streams: invalid period (must be a positive integer)");
    const int p = (int)pd;
    if (kind == SK_WMA && p < 2) return fail(VTA_ERR_INVALID_INPUT, "streams: wma period must be >= 2");

    StreamState s{};
    s.kind = kind;
    s.n = (int)n_streams;
    s.period = p;
    s.n_out = info.n_out;
    std::vector<double> w;
    int ring_slots = 0;
    switch (kind) {
        case SK_EMA:
            s.alpha = 2.0 / ((double)p + 1.0);
            s.beta = 1.0 - s.alpha;
            break;
        case SK_RSI:
            s.inv_p = 1.0 / (double)p;
            s.beta = 1.0 - s.inv_p;
            break;
        case SK_SMA:
            s.inv_p = 1.0 / (double)p;
            ring_slots = p;
            break;
        case SK_ALMA: {
            const double offset = P("offset", 0.85), sigma = P("sigma", 6.0);
            if (!(offset >= 0.0 && offset <= 1.0)) return fail(VTA_ERR_INVALID_INPUT, "streams: alma offset");
            if (!(sigma > 0.0)) return fail(VTA_ERR_INVALID_INPUT, "streams: alma sigma");
            // weights on the host with the C library's exp, as the crate's
            // AlmaStream::try_new forms them (alma.rs:883-899)
            const double m = offset * (double)(p - 1);
            const double sg = (double)p / sigma;
            const double s2 = 2.0 * sg * sg;
            double norm = 0.0;
            w.resize(p);
            for (int i = 0; i < p; ++i) {
                const double diff = (double)i - m;
                w[i] = std::exp(-(diff * diff) / s2);
                norm += w[i];
            }
            s.inv_norm = 1.0 / norm;
            ring_slots = p;
            break;
        }
        case SK_ATR:
        case SK_WILDERS:
            s.alpha = 1.0 / (double)p;
            break;
        case SK_SUPERTREND:
            // AtrStream(length = period) inside (supertrend.rs:810-818)
            s.alpha = 1.0 / (double)p;
            s.factor = P("factor", 3.0);
            break;
        case SK_DEMA:
            // DemaStream::try_new (dema.rs:625-640)
            s.alpha = 2.0 / ((double)p + 1.0);
            s.beta = 1.0 - 2.0 / ((double)p + 1.0);
            break;
        case SK_TEMA:
            s.alpha = 2.0 / ((double)p + 1.0);
            s.beta = 1.0 - s.alpha;
            break;
        case SK_WMA:
            // 1 / (p (p + 1) / 2), the product formed in integers (wma.rs:406)
            s.inv_norm = 1.0 / ((double)((long long)p * (p + 1)) * 0.5);
            ring_slots = p;
            break;
        case SK_SWMA:
            if (p & 1) {
                s.ka = s.kb = (p + 1) >> 1;
            } else {
                s.ka = p >> 1;
                s.kb = s.ka + 1;
            }
            s.inv_norm = 1.0 / ((double)s.ka * (double)s.kb);
            ring_slots = s.ka + s.kb;
            break;
        case SK_PWMA:
            // 2^-(p-1) exactly (fast_pow2_neg_i32, pwma.rs:738-750); 0 below
            // the subnormal range
            s.inv_norm = std::ldexp(1.0, -(p - 1 > 2000 ? 2000 : p - 1));
            ring_slots = p - 1;
            break;
        case SK_STDDEV:
        case SK_ZSCORE:
            s.nbdev = P("nbdev", 1.0);
            if (kind == SK_STDDEV && !(std::isfinite(s.nbdev) && s.nbdev >= 0.0))
                return fail(VTA_ERR_INVALID_INPUT, "streams: stddev nbdev must be finite and >= 0");
            if (kind == SK_ZSCORE && (P("ma_type", 0.0) != 0.0 || P("devtype", 0.0) != 0.0))
                return fail(VTA_ERR_NOT_IMPLEMENTED, "streams: zscore supports ma_type sma (0), devtype 0");
            s.inv_p = 1.0 / (double)p;
            ring_slots = p;
            break;
        case SK_BOLLINGER: {
            s.devup = P("devup", 2.0);
            s.devdn = P("devdn", 2.0);
            const double mt = P("matype", 0.0);
            if ((mt != 0.0 && mt != 1.0) || P("devtype", 0.0) != 0.0)
                return fail(VTA_ERR_NOT_IMPLEMENTED,
                            "streams: bollinger_bands supports matype sma (0) / ema (1), devtype 0");
            s.ema_mid = mt == 1.0;
            s.inv_p = 1.0 / (double)p;
            s.alpha = 2.0 / ((double)p + 1.0);
            s.beta = 1.0 - s.alpha;
            ring_slots = p;
            break;
        }
        case SK_DONCHIAN:
        case SK_WILLR:
            ring_slots = 2 * p;
            break;
        case SK_ADX:
            s.inv_p = 1.0 / (double)p;
            s.beta = 1.0 - s.inv_p;
            break;
        case SK_SINWMA: {
            // SinWmaStream::try_new (sinwma.rs:610-650), the C library's sin / cos
            const double pi = 3.14159265358979323846;
            const double al = pi / ((double)p + 1.0);
            s.k[0] = std::cos(al);
            s.k[1] = std::sin(al);
            s.k[2] = std::cos(al * (double)p);
            s.k[3] = std::sin(al * (double)p);
            const double den = std::sin(0.5 * al);
            const double eps = 2.220446049250313e-16;
            if (std::fabs(den) < eps) return fail(VTA_ERR_INVALID_INPUT, "streams: sinwma zero sum of sines");
            const double sum_sines = std::sin(0.5 * al * (double)p) / den;
            if (std::fabs(sum_sines) < eps) return fail(VTA_ERR_INVALID_INPUT, "streams: sinwma zero sum of sines");
            s.k[4] = 1.0 / sum_sines;
            ring_slots = p;
            break;
        }
        case SK_TRIMA:
            if (p <= 3) return fail(VTA_ERR_INVALID_INPUT, "streams: trima period must be > 3");
            s.ka = (p + 1) / 2;
            s.kb = p - s.ka + 1;
            s.inv_p = 1.0 / (double)s.ka;
            s.inv_norm = 1.0 / (double)s.kb;
            ring_slots = s.ka + s.kb;
            break;
        case SK_CWMA: {
            // CwmaStream::try_new (cwma.rs:832-870): weights (p + 1 - r)^3,
            // r = 1..p-1 (newest first), norm = sum_{j=2..p} j^3
            if (p <= 1) return fail(VTA_ERR_INVALID_INPUT, "streams: cwma period must be > 1");
            double norm = 0.0;
            for (int jj = 2; jj <= p; ++jj) {
                const double jf = (double)jj;
                norm += jf * jf * jf;
            }
            s.inv_norm = 1.0 / norm;
            const double av = (double)(p + 1);
            w.resize(p - 1);
            for (int r = 1; r <= p - 1; ++r) {
                const double t = av - (double)r;
                w[r - 1] = t * t * t;
            }
            ring_slots = p - 1;
            break;
        }
        case SK_FWMA: {
            // FwmaStream::try_new (fwma.rs:771-800): 1, 1, 2, 3, ... / sum
            w.assign(p, 1.0);
            for (int i = 2; i < p; ++i) w[i] = w[i - 1] + w[i - 2];
            double sum = 0.0;
            for (int i = 0; i < p; ++i) sum += w[i];
            for (int i = 0; i < p; ++i) w[i] /= sum;
            ring_slots = p;
            break;
        }
        case SK_SRWMA: {
            // SrwmaStream::try_new (srwma.rs:1208-1235): sqrt(p - k), k < p - 1
            double sumw = 0.0;
            w.resize(p > 1 ? p - 1 : 0);
            for (int k = 0; k < p - 1; ++k) {
                w[k] = std::sqrt((double)(p - k));
                sumw += w[k];
            }
            s.inv_norm = sumw == 0.0 ? 0.0 : 1.0 / sumw;
            ring_slots = p > 1 ? p - 1 : 0;
            break;
        }
        case SK_SQWMA: {
            // SqwmaStream::try_new (sqwma.rs:383-420): (p - i)^2, i < p - 1
            if (p < 2) return fail(VTA_ERR_INVALID_INPUT, "streams: sqwma period must be >= 2");
            double ws = 0.0;
            w.resize(p - 1);
            for (int i = 0; i < p - 1; ++i) {
                const double d = (double)p - (double)i;
                w[i] = d * d;
                ws += w[i];
            }
            s.inv_norm = 1.0 / ws;
            ring_slots = p;
            break;
        }
        case SK_EPMA: {
            // EpmaStream::try_new (epma.rs:667-700)
            const double off = P("offset", 4.0);
            if (p < 2) return fail(VTA_ERR_INVALID_INPUT, "streams: epma period must be >= 2");
            if (!(off >= 0.0) || off != std::floor(off) || off >= (double)p)
                return fail(VTA_ERR_INVALID_INPUT, "streams: epma offset must be an integer in [0, period)");
            s.offset = (int)off;
            const double p1f = (double)(p - 1);
            s.k[0] = 2.0 - off;
            s.k[1] = 1.0 / std::fma(p1f, s.k[0], 0.5 * (p1f - 1.0) * p1f);
            s.k[2] = (double)(p - 2);
            ring_slots = p;
            break;
        }
        case SK_VPWMA: {
            // VpwmaStream::try_new (vpwma.rs:595-680)
            const double power = P("power", 0.382);
            if (p < 2) return fail(VTA_ERR_INVALID_INPUT, "streams: vpwma period must be >= 2");
            if (!std::isfinite(power)) return fail(VTA_ERR_INVALID_INPUT, "streams: vpwma power must be finite");
            const int m = p - 1;
            std::vector<double> wt(m);
            double norm = 0.0;
            for (int k = 0; k < m; ++k) {
                wt[k] = std::pow((double)p - (double)k, power);
                norm += wt[k];
            }
            s.inv_norm = 1.0 / norm;
            const double pr = std::round(power);
            if (std::fabs(power - pr) <= 1e-12 && pr >= 0.0 && pr <= 8.0) {
                const int dg = (int)pr;
                s.deg = dg;
                w.assign(kVpConsts, 0.0);
                // integer powers by binary exponentiation (the LLVM runtime's
                // powi); binomials as exact integer ratios
                auto powi = [](double base, int e) {
                    double r = 1.0;
                    for (;;) {
                        if (e & 1) r *= base;
                        e /= 2;
                        if (e == 0) break;
                        base *= base;
                    }
                    return r;
                };
                auto binom = [](int nn, int kk) {
                    if (kk == 0 || kk == nn) return 1.0;
                    if (kk > nn - kk) kk = nn - kk;
                    unsigned long long num = 1, den = 1;
                    for (int i = 1; i <= kk; ++i) {
                        num *= (unsigned long long)(nn + 1 - i);
                        den *= (unsigned long long)i;
                    }
                    return (double)num / (double)den;
                };
                for (int jj = 0; jj <= dg; ++jj)
                    w[jj] = ((jj & 1) ? -1.0 : 1.0) * binom(dg, jj) * powi((double)p, dg - jj);
                double pp = 1.0;
                for (int q = 0; q <= dg; ++q) {
                    w[kVpPow + q] = pp;
                    pp *= (double)(m - 1);
                }
                for (int jj = 0; jj <= dg; ++jj)
                    for (int q = 0; q <= jj; ++q) w[kVpBinom + jj * (jj + 1) / 2 + q] = binom(jj, q);
            } else {
                s.deg = -1;
                w = wt;
            }
            ring_slots = p;
            break;
        }
        case SK_PERCENTILE: {
            const double pct = P("percentage", 50.0);
            if (!(pct >= 0.0 && pct <= 100.0))
                return fail(VTA_ERR_INVALID_INPUT, "streams: percentage must be in [0, 100]");
            s.k[0] = pct * 0.01;
            ring_slots = p;
            break;
        }
        default: break;
    }
    s.ring_slots = ring_slots;

    auto* S = new vta_streams();
    S->ctx = ctx;
    const size_t n = n_streams;
    const size_t bytes = kI * n * sizeof(int) + kD * n * sizeof(double) + (size_t)ring_slots * n * sizeof(double) +
                         w.size() * sizeof(double) + (3 + (size_t)info.n_out) * n * sizeof(float) + 64 * 24;
    vta_status st = vram_check(bytes);
    if (st == VTA_OK) {
        const cudaError_t e = cudaMalloc(&S->block, bytes);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMalloc(streams)");
    }
    if (st != VTA_OK) {
        delete S;
        return st;
    }
    char* q = static_cast<char*>(S->block);
    auto take = [&](size_t b) {
        char* r = q;
        q += (b + 63) & ~size_t(63);
        return r;
    };
    for (int k = 0; k < kD; ++k) s.d[k] = reinterpret_cast<double*>(take(n * sizeof(double)));
    s.ring = ring_slots ? reinterpret_cast<double*>(take((size_t)ring_slots * n * sizeof(double))) : nullptr;
    double* dw = w.empty() ? nullptr : reinterpret_cast<double*>(take(w.size() * sizeof(double)));
    s.w = dw;
    for (int k = 0; k < kI; ++k) s.iv[k] = reinterpret_cast<int*>(take(n * sizeof(int)));
    S->d_io = reinterpret_cast<float*>(take((3 + (size_t)info.n_out) * n * sizeof(float)));
    S->s = s;
    cudaStream_t cs = ctx->stream;
    if (dw) st = upload_async(ctx, dw, w.data(), w.size() * sizeof(double), cs);
    if (st == VTA_OK) {
        k_stream_init<<<ceil_div(n, 256), 256, 0, cs>>>(S->s);
        st = check_launch("k_stream_init");
    }
    if (st == VTA_OK) {
        const cudaError_t e = cudaStreamSynchronize(cs);
        if (e != cudaSuccess) st = cuda_fail(e, "streams init");
    }
    if (st != VTA_OK) {
        cudaFree(S->block);
        delete S;
        return st;
    }
    *out = S;
    return VTA_OK;
}

vta_status vta_streams_shape(const vta_streams* S, int* n_inputs, int* n_outputs) {
    if (!S) return fail(VTA_ERR_INVALID_INPUT, "streams: null handle");
    if (n_inputs) *n_inputs = kKinds[S->s.kind].n_in;
    if (n_outputs) *n_outputs = S->s.n_out;
    return VTA_OK;
}

vta_status vta_streams_update_device(vta_streams* S, const float* d_a, const float* d_b, const float* d_c,
                                     float* d_out) {
    if (!S) return fail(VTA_ERR_INVALID_INPUT, "streams: null handle");
    VTA_TRY(enter_call(S->ctx));
    if (!inputs_ok(S, d_a, d_b, d_c) || !d_out)
        return fail(VTA_ERR_INVALID_INPUT, "streams: null input/output pointer");
    VTA_TRY(enqueue_update(S, d_a, d_b, d_c, d_out));
    VTA_CUDA_TRY(cudaStreamSynchronize(S->ctx->stream));
    return check_async("stream");
}

vta_status vta_streams_update_host(vta_streams* S, const float* a, const float* b, const float* c, float* out) {
    if (!S) return fail(VTA_ERR_INVALID_INPUT, "streams: null handle");
    VTA_TRY(enter_call(S->ctx));
    if (!inputs_ok(S, a, b, c) || !out) return fail(VTA_ERR_INVALID_INPUT, "streams: null input/output pointer");
    const size_t n = (size_t)S->s.n;
    const int n_in = kKinds[S->s.kind].n_in;
    cudaStream_t cs = S->ctx->stream;
    float* da = S->d_io;
    float* db = da + n;
    float* dc = db + n;
    float* dout = dc + n;
    VTA_TRY(upload_async(S->ctx, da, a, n * sizeof(float), cs));
    if (n_in >= 2) VTA_TRY(upload_async(S->ctx, db, b, n * sizeof(float), cs));
    if (n_in >= 3) VTA_TRY(upload_async(S->ctx, dc, c, n * sizeof(float), cs));
    VTA_TRY(enqueue_update(S, da, db, dc, dout));
    VTA_CUDA_TRY(cudaMemcpyAsync(out, dout, (size_t)S->s.n_out * n * sizeof(float), cudaMemcpyDeviceToHost, cs));
    VTA_CUDA_TRY(cudaStreamSynchronize(cs));
    return check_async("stream");
}

vta_status vta_streams_reset(vta_streams* S) {
    if (!S) return fail(VTA_ERR_INVALID_INPUT, "streams: null handle");
    VTA_TRY(enter_call(S->ctx));
    k_stream_init<<<ceil_div(S->s.n, 256), 256, 0, S->ctx->stream>>>(S->s);
    VTA_TRY(check_launch("k_stream_init"));
    VTA_CUDA_TRY(cudaStreamSynchronize(S->ctx->stream));
    return VTA_OK;
}

vta_status vta_streams_destroy(vta_streams* S) {
    if (!S) return VTA_OK;
    cudaSetDevice(S->ctx->device);
    cudaStreamSynchronize(S->ctx->stream);
    if (S->block) cudaFree(S->block);
    delete S;
    return VTA_OK;
}

}  // extern "C"
