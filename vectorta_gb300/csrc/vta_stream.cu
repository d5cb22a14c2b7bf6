// Banks of streaming indicators on the device (vta_streams_*): S independent
// streams of one indicator and parameter set, advanced together by one bar
// per call, one thread per stream.  Each stream follows the update rule of
// the crate's XStream struct bar for bar (cited per kind) in f64, with the
// crate's rounding: explicit __dadd_rn / __dmul_rn where the Rust code has
// separate operations (so nothing is contracted into an FMA), fma() where it
// calls mul_add.  The outputs are the f64 values rounded to f32, NaN where the
// crate's update() returns None.  The step after the batch entry points for
// live data: the state stays resident between calls.
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "vta_internal.h"

namespace {

enum StreamKind { SK_EMA = 0, SK_SMA = 1, SK_ALMA = 2, SK_RSI = 3, SK_ATR = 4, SK_WILDERS = 5 };

// Per-stream state, structure of arrays ([slot][stream] for the rings).
struct StreamState {
    int kind, n, period;
    double alpha, beta, inv_p, inv_norm;
    const double* w;  // ALMA weights (device)
    int* i0;          // count / head / seed_count / warm_count
    int* i1;          // filled / has_prev / seeded / started / ring head
    int* i2;          // poisoned
    double* d0;       // mean / sum / prev / prev_close / warm_sum
    double* d1;       // sum_gain / rma / last
    double* d2;       // sum_loss
    double* d3;       // avg_gain
    double* d4;       // avg_loss
    double* ring;     // [period][n] (SMA, ALMA)
};

__device__ __forceinline__ double dnan() { return __longlong_as_double(0x7ff8000000000000ll); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

__global__ void k_stream_init(StreamState s) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= s.n) return;
    s.i0[j] = 0;
    s.i1[j] = 0;
    s.i2[j] = 0;
    const double nan = dnan();
    // EMA mean NaN, RSI prev NaN, ATR prev_close NaN, Wilders last NaN
    s.d0[j] = (s.kind == SK_EMA || s.kind == SK_RSI || s.kind == SK_ATR) ? nan : 0.0;
    s.d1[j] = (s.kind == SK_ATR || s.kind == SK_WILDERS) ? nan : 0.0;
    s.d2[j] = 0.0;
    s.d3[j] = 0.0;
    s.d4[j] = 0.0;
    if (s.ring)
        for (int k = 0; k < s.period; ++k) s.ring[(size_t)k * s.n + j] = nan;
}

template <int K>
__global__ void k_stream_update(StreamState s, const float* __restrict__ a, const float* __restrict__ b,
                                const float* __restrict__ c, float* __restrict__ out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= s.n) return;
    const int p = s.period;
    const double nan = dnan();
    double y = nan;
    if constexpr (K == SK_EMA) {  // EmaStream::update, ema.rs:560-585
        const double v = (double)a[j];
        if (!isfinite(v)) {
            y = s.i1[j] ? s.d0[j] : nan;
        } else {
            const int cnt = s.i0[j] + 1;
            s.i0[j] = cnt;
            double mean = s.d0[j];
            if (cnt == 1) mean = v;
            else if (cnt <= p) mean = fma(dsub(v, mean), ddiv(1.0, (double)cnt), mean);
            else mean = fma(s.beta, mean, dmul(s.alpha, v));
            s.d0[j] = mean;
            if (!s.i1[j] && cnt >= p) s.i1[j] = 1;
            y = s.i1[j] ? mean : nan;
        }
    } else if constexpr (K == SK_SMA) {  // SmaStream::update (sma.rs)
        const double v = (double)a[j];
        if (p == 1) {
            y = v;
        } else {
            int head = s.i1[j];
            const int cnt = s.i0[j];
            double sum = s.d0[j];
            if (cnt < p) {
                sum = dadd(sum, v);
                s.ring[(size_t)head * s.n + j] = v;
                head = head + 1 == p ? 0 : head + 1;
                s.i0[j] = cnt + 1;
                y = cnt + 1 == p ? dmul(sum, s.inv_p) : nan;
            } else {
                const double old = s.ring[(size_t)head * s.n + j];
                sum = dadd(sum, dsub(v, old));
                s.ring[(size_t)head * s.n + j] = v;
                head = head + 1 == p ? 0 : head + 1;
                y = dmul(sum, s.inv_p);
            }
            s.d0[j] = sum;
            s.i1[j] = head;
        }
    } else if constexpr (K == SK_ALMA) {  // AlmaStream::update / dot_at_head, alma.rs:865-964
        const double v = (double)a[j];
        int head = s.i1[j];
        s.ring[(size_t)head * s.n + j] = v;
        head = head + 1 == p ? 0 : head + 1;
        s.i1[j] = head;
        int filled = s.i0[j];
        if (filled < p) s.i0[j] = ++filled;
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
                    acc[q] = dadd(acc[q], dmul(s.ring[(size_t)slot * s.n + j], s.w[i + q]));
                }
            double sum = dadd(dadd(acc[0], acc[1]), dadd(acc[2], acc[3]));
            for (; i < p; ++i) {
                int slot = head + i;
                if (slot >= p) slot -= p;
                sum = dadd(sum, dmul(s.ring[(size_t)slot * s.n + j], s.w[i]));
            }
            y = dmul(sum, s.inv_norm);
        }
    } else if constexpr (K == SK_RSI) {  // RsiStream::update (rsi.rs)
        const double v = (double)a[j];
        if (!s.i1[j]) {
            s.d0[j] = v;
            s.i1[j] = 1;
        } else {
            const double d = dsub(v, s.d0[j]);
            s.d0[j] = v;
            const double g = fmax(d, 0.0), l = fmax(-d, 0.0);  // f64::max ignores NaN
            const bool seeded = (s.i2[j] & 2) != 0;                 // i2: bit 0 poisoned, bit 1 seeded
            if (!seeded) {
                int poisoned = s.i2[j] & 1;
                if (!isfinite(d)) poisoned = 1;
                s.d1[j] = dadd(s.d1[j], g);
                s.d2[j] = dadd(s.d2[j], l);
                const int cnt = s.i0[j] + 1;
                s.i0[j] = cnt;
                if (cnt == p) {
                    if (poisoned) {
                        s.d3[j] = nan;
                        s.d4[j] = nan;
                        y = nan;
                    } else {
                        const double ag = dmul(s.d1[j], s.inv_p), al = dmul(s.d2[j], s.inv_p);
                        s.d3[j] = ag;
                        s.d4[j] = al;
                        const double den = dadd(ag, al);
                        y = den == 0.0 ? 50.0 : ddiv(dmul(100.0, ag), den);
                    }
                    s.i2[j] = poisoned | 2;
                } else {
                    s.i2[j] = poisoned;
                }
            } else {
                const double ag = fma(s.d3[j], s.beta, dmul(s.inv_p, g));
                const double al = fma(s.d4[j], s.beta, dmul(s.inv_p, l));
                s.d3[j] = ag;
                s.d4[j] = al;
                const double den = dadd(ag, al);
                y = den == 0.0 ? 50.0 : ddiv(dmul(100.0, ag), den);
            }
        }
    } else if constexpr (K == SK_ATR) {  // AtrStream::update (atr.rs)
        const double h = (double)a[j], l = (double)b[j], cl = (double)c[j];
        const double pc = s.d0[j];
        double tr;
        if (isnan(pc)) {
            tr = dsub(h, l);
        } else {
            const double up = h > pc ? h : pc;
            const double dn = l < pc ? l : pc;
            tr = dsub(up, dn);
        }
        s.d0[j] = cl;
        if (!s.i1[j]) {
            s.d2[j] = dadd(s.d2[j], tr);
            const int cnt = s.i0[j] + 1;
            s.i0[j] = cnt;
            if (cnt == p) {
                const double rma = dmul(s.d2[j], s.alpha);
                s.d1[j] = rma;
                s.i1[j] = 1;
                y = rma;
            }
        } else {
            const double rma = fma(s.alpha, dsub(tr, s.d1[j]), s.d1[j]);
            s.d1[j] = rma;
            y = rma;
        }
    } else if constexpr (K == SK_WILDERS) {  // WildersStream::update (wilders.rs)
        const double v = (double)a[j];
        if (!s.i1[j]) {
            if (!isfinite(v)) {
                s.d0[j] = 0.0;
                s.i0[j] = 0;
            } else {
                const double sum = dadd(s.d0[j], v);
                s.d0[j] = sum;
                const int cnt = s.i0[j] + 1;
                s.i0[j] = cnt;
                if (cnt >= p) {
                    const double y0 = ddiv(sum, (double)p);
                    s.d1[j] = y0;
                    s.i1[j] = 1;
                    y = y0;
                }
            }
        } else {
            const double last = fma(dsub(v, s.d1[j]), s.alpha, s.d1[j]);
            s.d1[j] = last;
            y = last;
        }
    }
    out[j] = (float)y;
}

int kind_of(const char* name) {
    if (!name) return -1;
    std::string s(name);
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    if (s == "ema") return SK_EMA;
    if (s == "sma") return SK_SMA;
    if (s == "alma") return SK_ALMA;
    if (s == "rsi") return SK_RSI;
    if (s == "atr") return SK_ATR;
    if (s == "wilders") return SK_WILDERS;
    return -1;
}

double param(const char* const* keys, const double* vals, size_t n, const char* key, double dflt) {
    for (size_t i = 0; i < n; ++i)
        if (keys && keys[i] && vals && std::strcmp(keys[i], key) == 0) return vals[i];
    return dflt;
}

}  // namespace

struct vta_streams {
    vta_ctx* ctx = nullptr;
    StreamState s{};
    void* block = nullptr;  // one device allocation for all state
    float* d_io = nullptr;  // staging of the host-buffer update: inputs (3 n) + output (n)
};

using namespace vta;

namespace {

vta_status enqueue_update(vta_streams* S, const float* a, const float* b, const float* c, float* out) {
    cudaStream_t st = S->ctx->stream;
    const unsigned blocks = ceil_div(S->s.n, 256);
    switch (S->s.kind) {
        case SK_EMA: k_stream_update<SK_EMA><<<blocks, 256, 0, st>>>(S->s, a, b, c, out); break;
        case SK_SMA: k_stream_update<SK_SMA><<<blocks, 256, 0, st>>>(S->s, a, b, c, out); break;
        case SK_ALMA: k_stream_update<SK_ALMA><<<blocks, 256, 0, st>>>(S->s, a, b, c, out); break;
        case SK_RSI: k_stream_update<SK_RSI><<<blocks, 256, 0, st>>>(S->s, a, b, c, out); break;
        case SK_ATR: k_stream_update<SK_ATR><<<blocks, 256, 0, st>>>(S->s, a, b, c, out); break;
        default: k_stream_update<SK_WILDERS><<<blocks, 256, 0, st>>>(S->s, a, b, c, out); break;
    }
    return check_launch("k_stream_update");
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
    // the crate's defaults (EmaParams 9, SmaParams 9, AlmaParams 9 / 0.85 /
    // 6.0, RsiParams 14, AtrParams 14, WildersParams 5)
    const double dflt = kind == SK_RSI || kind == SK_ATR ? 14.0 : kind == SK_WILDERS ? 5.0 : 9.0;
    double pd = param(param_keys, param_values, n_params, "period", dflt);
    if (kind == SK_ATR) pd = param(param_keys, param_values, n_params, "length", pd);
    if (!(pd >= 1.0) || pd != std::floor(pd) || pd > 1e7)
        return fail(VTA_ERR_INVALID_INPUT, "streams: invalid period (must be a positive integer)");
    const int p = (int)pd;
    const double offset = param(param_keys, param_values, n_params, "offset", 0.85);
    const double sigma = param(param_keys, param_values, n_params, "sigma", 6.0);
    if (kind == SK_ALMA && !(offset >= 0.0 && offset <= 1.0)) return fail(VTA_ERR_INVALID_INPUT, "streams: alma offset");
    if (kind == SK_ALMA && !(sigma > 0.0)) return fail(VTA_ERR_INVALID_INPUT, "streams: alma sigma");

    auto* S = new vta_streams();
    S->ctx = ctx;
    StreamState& s = S->s;
    s.kind = kind;
    s.n = (int)n_streams;
    s.period = p;
    if (kind == SK_EMA) {
        s.alpha = 2.0 / ((double)p + 1.0);
        s.beta = 1.0 - s.alpha;
    } else if (kind == SK_RSI) {
        s.inv_p = 1.0 / (double)p;
        s.beta = 1.0 - s.inv_p;
    } else if (kind == SK_SMA) {
        s.inv_p = 1.0 / (double)p;
    } else {
        s.alpha = 1.0 / (double)p;
    }
    // ALMA weights on the host with the C library's exp, as the crate's
    // AlmaStream::try_new forms them (alma.rs:883-899)
    std::vector<double> w;
    if (kind == SK_ALMA) {
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
    }
    const size_t n = n_streams;
    const bool ring = kind == SK_SMA || kind == SK_ALMA;
    const size_t bytes = 3 * n * sizeof(int) + 5 * n * sizeof(double) + (ring ? (size_t)p * n * sizeof(double) : 0) +
                         w.size() * sizeof(double) + 4 * n * sizeof(float) + 64 * 8;
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
    s.d0 = reinterpret_cast<double*>(take(n * sizeof(double)));
    s.d1 = reinterpret_cast<double*>(take(n * sizeof(double)));
    s.d2 = reinterpret_cast<double*>(take(n * sizeof(double)));
    s.d3 = reinterpret_cast<double*>(take(n * sizeof(double)));
    s.d4 = reinterpret_cast<double*>(take(n * sizeof(double)));
    s.ring = ring ? reinterpret_cast<double*>(take((size_t)p * n * sizeof(double))) : nullptr;
    double* dw = w.empty() ? nullptr : reinterpret_cast<double*>(take(w.size() * sizeof(double)));
    s.w = dw;
    s.i0 = reinterpret_cast<int*>(take(n * sizeof(int)));
    s.i1 = reinterpret_cast<int*>(take(n * sizeof(int)));
    s.i2 = reinterpret_cast<int*>(take(n * sizeof(int)));
    S->d_io = reinterpret_cast<float*>(take(4 * n * sizeof(float)));
    cudaStream_t cs = ctx->stream;
    if (dw) st = upload_async(ctx, dw, w.data(), w.size() * sizeof(double), cs);
    if (st == VTA_OK) {
        k_stream_init<<<ceil_div(n, 256), 256, 0, cs>>>(s);
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

vta_status vta_streams_update_device(vta_streams* S, const float* d_a, const float* d_b, const float* d_c,
                                     float* d_out) {
    if (!S) return fail(VTA_ERR_INVALID_INPUT, "streams: null handle");
    VTA_TRY(enter_call(S->ctx));
    if (!d_a || !d_out || (S->s.kind == SK_ATR && (!d_b || !d_c)))
        return fail(VTA_ERR_INVALID_INPUT, "streams: null input/output pointer");
    VTA_TRY(enqueue_update(S, d_a, d_b, d_c, d_out));
    VTA_CUDA_TRY(cudaStreamSynchronize(S->ctx->stream));
    return check_launch("stream");
}

vta_status vta_streams_update_host(vta_streams* S, const float* a, const float* b, const float* c, float* out) {
    if (!S) return fail(VTA_ERR_INVALID_INPUT, "streams: null handle");
    VTA_TRY(enter_call(S->ctx));
    if (!a || !out || (S->s.kind == SK_ATR && (!b || !c)))
        return fail(VTA_ERR_INVALID_INPUT, "streams: null input/output pointer");
    const size_t n = (size_t)S->s.n;
    cudaStream_t cs = S->ctx->stream;
    float* da = S->d_io;
    float* db = da + n;
    float* dc = db + n;
    float* dout = dc + n;
    VTA_TRY(upload_async(S->ctx, da, a, n * sizeof(float), cs));
    if (S->s.kind == SK_ATR) {
        VTA_TRY(upload_async(S->ctx, db, b, n * sizeof(float), cs));
        VTA_TRY(upload_async(S->ctx, dc, c, n * sizeof(float), cs));
    }
    VTA_TRY(enqueue_update(S, da, db, dc, dout));
    VTA_CUDA_TRY(cudaMemcpyAsync(out, dout, n * sizeof(float), cudaMemcpyDeviceToHost, cs));
    VTA_CUDA_TRY(cudaStreamSynchronize(cs));
    return check_launch("stream");
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
