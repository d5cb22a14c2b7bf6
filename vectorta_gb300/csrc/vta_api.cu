// Host side of the C ABI: contexts, device arrays, parameter grids, input
// validation and kernel orchestration for every indicator.
//
// Each public entry point funnels into one of two internal drivers:
//   run_batch(ctx, ind, device inputs, len, first, combos, device outputs)
//   run_tm(ctx, ind, device inputs, cols, rows, params, device outputs)
// which enqueue kernels on the context stream.  The *_dev / *_into_host_f32
// / *_many_series_*_dev forms add the crate's host-side validation, the
// host->device copies and the output allocation around them.
#include <algorithm>
#include <cctype>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>

#include "vta_internal.h"

// ============================================================ errors =======
namespace vta {

static thread_local std::string g_err;
// status of the last failure on this thread and, for VTA_ERR_OUT_OF_MEMORY,
// its byte counts (required, free, headroom)
static thread_local vta_status g_err_status = VTA_OK;
static thread_local size_t g_oom[3] = {0, 0, 0};

void set_error(const std::string& msg) { g_err = msg; }
vta_status fail(vta_status st, const std::string& msg) {
    g_err = msg;
    g_err_status = st;
    return st;
}
vta_status cuda_fail(cudaError_t e, const char* what) {
    g_err = std::string("cuda error: ") + cudaGetErrorString(e) + " (" + what + ")";
    return VTA_ERR_CUDA;
}
static std::atomic<uint64_t> g_launches{0};
static thread_local vta_ctx* g_cur = nullptr;  // context of the call in progress

void ktimer_begin(cudaStream_t st) {
    if (g_cur && g_cur->timing && g_cur->ev0) {
        cudaEventRecord(g_cur->ev0, st);
        g_cur->timed = false;
    }
}
void ktimer_end(cudaStream_t st) {
    if (g_cur && g_cur->timing && g_cur->ev1) {
        cudaEventRecord(g_cur->ev1, st);
        g_cur->timed = true;
    }
}

vta_status check_launch(const char* kernel) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, kernel);
    return VTA_OK;
}
vta_status check_async(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, what);
    return VTA_OK;
}

vta_status Arena::commit() {
    if (total_ <= ctx_->scratch_bytes) return VTA_OK;
    size_t want = std::max(total_, size_t(1) << 20);
    want = (want + (size_t(1) << 20) - 1) & ~((size_t(1) << 20) - 1);
    if (ctx_->async_alloc) {
        // server slots: stream-ordered, so growing never waits for other streams
        if (ctx_->scratch) VTA_CUDA_TRY(cudaFreeAsync(ctx_->scratch, ctx_->stream));
        ctx_->scratch = nullptr;
        ctx_->scratch_bytes = 0;
        VTA_CUDA_TRY(ctx_->pool ? cudaMallocFromPoolAsync(&ctx_->scratch, want, ctx_->pool, ctx_->stream)
                                : cudaMallocAsync(&ctx_->scratch, want, ctx_->stream));
        ctx_->scratch_bytes = want;
        return VTA_OK;
    }
    if (ctx_->scratch) {
        VTA_CUDA_TRY(cudaStreamSynchronize(ctx_->stream));
        cudaFree(ctx_->scratch);
        ctx_->scratch = nullptr;
        ctx_->scratch_bytes = 0;
    }
    VTA_TRY(vram_check(want));
    VTA_CUDA_TRY(cudaMalloc(&ctx_->scratch, want));
    ctx_->scratch_bytes = want;
    return VTA_OK;
}

vta_status vram_check(size_t required) {
    const char* env = std::getenv("VTA_MEM_CHECK");
    if (env && (env[0] == '0' || env[0] == 'f' || env[0] == 'F')) return VTA_OK;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return VTA_OK;
    const size_t headroom = size_t(64) << 20;
    if (required + headroom > free_b) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "out of memory: required=%zu free=%zu headroom=%zu", required, free_b,
                      headroom);
        const vta_status st = fail(VTA_ERR_OUT_OF_MEMORY, buf);
        g_oom[0] = required;
        g_oom[1] = free_b;
        g_oom[2] = headroom;
        return st;
    }
    return VTA_OK;
}

// ============================================================ grids ========
enum AxisMode { AX_DESC = 0, AX_SWAP = 1, AX_REV_FROM_END = 2, AX_DESC_PLUS_END = 3 };

// usize axis of the crate's expand_grid functions.  Ascending ranges are the
// same everywhere; descending ones differ per indicator (see AxisMode users).
static std::vector<size_t> axis_usize(vta_range_usize r, int mode) {
    std::vector<size_t> v;
    if (r.step == 0 || r.start == r.end) return {r.start};
    if (r.start < r.end) {
        for (size_t x = r.start; x <= r.end; x += r.step) {
            v.push_back(x);
            if (x > SIZE_MAX - r.step) break;
        }
        return v;
    }
    switch (mode) {
        case AX_SWAP:
            for (size_t x = r.end; x <= r.start; x += r.step) {
                v.push_back(x);
                if (x > SIZE_MAX - r.step) break;
            }
            break;
        case AX_REV_FROM_END: {
            const size_t cnt = (r.start - r.end) / r.step + 1;
            for (size_t k = cnt; k-- > 0;) v.push_back(r.end + k * r.step);
            break;
        }
        default: {
            size_t x = r.start;
            for (;;) {
                v.push_back(x);
                if (x < r.end + r.step) break;
                x -= r.step;
            }
            if (mode == AX_DESC_PLUS_END && v.back() != r.end) v.push_back(r.end);
        }
    }
    return v;
}

// f64 axis: accumulated x += step with the crate's 1e-12 slack
// (alma.rs:1224-1260 and the same helper in the other indicators).
static std::vector<double> axis_f64(vta_range_f64 r) {
    std::vector<double> v;
    if (std::fabs(r.step) < 1e-12 || std::fabs(r.start - r.end) < 1e-12) return {r.start};
    const double st = std::fabs(r.step);
    if (r.start < r.end) {
        for (double x = r.start; x <= r.end + 1e-12; x += st) v.push_back(x);
    } else {
        for (double x = r.start; x + 1e-12 >= r.end; x -= st) v.push_back(x);
    }
    return v;
}

// ============================================================ indicators ===
enum Ind {
    I_ALMA, I_EMA, I_DEMA, I_TEMA, I_RSI, I_WILDERS, I_SMA, I_WMA, I_SWMA, I_PWMA, I_SINWMA, I_TRIMA,
    I_STDDEV, I_ZSCORE, I_BB, I_ATR, I_ADX, I_SUPERTREND, I_DONCHIAN, I_WILLR, I_PNR,
    I_CWMA, I_FWMA, I_SRWMA, I_SQWMA, I_EPMA, I_VPWMA
};
enum InKind { IN_X = 1, IN_HL = 2, IN_HLC = 3 };

struct IndInfo {
    const char* name;
    int in;       // InKind == number of input series
    int n_out;
    int axis;     // AxisMode of the period axis
};
static const IndInfo kInfo[] = {
    {"alma", IN_X, 1, AX_DESC},        {"ema", IN_X, 1, AX_SWAP},         {"dema", IN_X, 1, AX_DESC},
    {"tema", IN_X, 1, AX_DESC},        {"rsi", IN_X, 1, AX_SWAP},         {"wilders", IN_X, 1, AX_DESC},
    {"sma", IN_X, 1, AX_DESC},         {"wma", IN_X, 1, AX_DESC_PLUS_END}, {"swma", IN_X, 1, AX_DESC},
    {"pwma", IN_X, 1, AX_DESC},        {"sinwma", IN_X, 1, AX_DESC},      {"trima", IN_X, 1, AX_SWAP},
    {"stddev", IN_X, 1, AX_DESC},      {"zscore", IN_X, 1, AX_DESC},      {"bollinger_bands", IN_X, 3, AX_DESC},
    {"atr", IN_HLC, 1, AX_REV_FROM_END}, {"adx", IN_HLC, 1, AX_DESC},     {"supertrend", IN_HLC, 2, AX_DESC},
    {"donchian", IN_HL, 3, AX_DESC},   {"willr", IN_HLC, 1, AX_DESC},     {"percentile_nearest_rank", IN_X, 1, AX_DESC},
    {"cwma", IN_X, 1, AX_SWAP},        {"fwma", IN_X, 1, AX_SWAP},        {"srwma", IN_X, 1, AX_DESC},
    {"sqwma", IN_X, 1, AX_DESC},       {"epma", IN_X, 1, AX_SWAP},        {"vpwma", IN_X, 1, AX_DESC},
};

// One parameter set: period plus up to two f64 parameters
// (alma: offset, sigma; stddev/zscore: nbdev; bb: devup, devdn;
//  supertrend: factor; percentile: percentage; epma: offset; vpwma: power).
struct Combo {
    size_t period;
    double a, b;
};

static bool is_wwma(Ind i) {
    return i == I_ALMA || i == I_WMA || i == I_SWMA || i == I_PWMA || i == I_SINWMA || i == I_TRIMA ||
           i == I_CWMA || i == I_FWMA || i == I_SRWMA || i == I_SQWMA || i == I_EPMA || i == I_VPWMA;
}

// Weighted-window geometry of a combo: window length L (the weight row) and
// the extra warm-up past first + L - 1 of its first output.
//   CWMA  L = p - 1, first output first + p - 1   (cwma.rs:243-253, 453-466)
//   SRWMA L = p - 1, first output first + p + 1   (srwma.rs:204-215, 288-292)
//   SQWMA L = p - 1, first output first + p + 1   (sqwma.rs:222-228, 270-272)
//   EPMA  L = p - 1, first output first + p + o + 1 (epma.rs:247, 341-352)
//   VPWMA L = p - 1, first output first + p - 1   (vpwma.rs:246-262, 296-312)
//   others L = p, first output first + p - 1
static int wwma_len(Ind i, const Combo& c) {
    return (i == I_CWMA || i == I_SRWMA || i == I_SQWMA || i == I_EPMA || i == I_VPWMA) ? (int)c.period - 1
                                                                                        : (int)c.period;
}
static int wwma_warm_extra(Ind i, const Combo& c) {
    switch (i) {
        case I_CWMA: case I_VPWMA: return 1;
        case I_SRWMA: case I_SQWMA: return 3;
        case I_EPMA: return (int)c.a + 3;
        default: return 0;
    }
}
static int wwma_weight_kind(Ind i) {
    switch (i) {
        case I_WMA: return WT_WMA;
        case I_SWMA: return WT_SWMA;
        case I_PWMA: return WT_PWMA;
        case I_SINWMA: return WT_SINWMA;
        case I_TRIMA: return WT_TRIMA;
        case I_CWMA: return WT_CWMA;
        case I_FWMA: return WT_FWMA;
        case I_SRWMA: return WT_SRWMA;
        case I_SQWMA: return WT_SQWMA;
        case I_EPMA: return WT_EPMA;
        case I_VPWMA: return WT_VPWMA;
        default: return WT_ALMA;
    }
}

// minimum valid length after `first` a combo needs (the crate's checks)
static size_t needed_len(Ind ind, size_t p, double a = 0.0) {
    switch (ind) {
        case I_DEMA: return p > 0 ? 2 * (p - 1) : 0;
        case I_ADX: return p + 1;
        case I_EPMA: return p + (size_t)a + 1;  // epma.rs:235
        default: return p;
    }
}

static vta_status validate_combo(Ind ind, const Combo& c, size_t len) {
    const IndInfo& in = kInfo[ind];
    char buf[200];
    auto bad = [&](const char* why) {
        std::snprintf(buf, sizeof buf, "%s: invalid params: period=%zu a=%g b=%g (%s)", in.name, c.period, c.a,
                      c.b, why);
        return fail(VTA_ERR_INVALID_INPUT, buf);
    };
    if (c.period == 0) return bad("period must be > 0");
    if (c.period > len) return bad("period exceeds data length");
    if (c.period > (size_t)INT32_MAX) return bad("period too large");
    switch (ind) {
        case I_ALMA:
            if (!(c.b > 0.0)) return bad("sigma must be > 0");
            if (!(c.a >= 0.0 && c.a <= 1.0)) return bad("offset must be in [0, 1]");
            break;
        case I_WMA: case I_CWMA: case I_SRWMA: case I_SQWMA:
            if (c.period < 2) return bad("period must be >= 2");
            break;
        case I_VPWMA:
            if (c.period < 2) return bad("period must be >= 2");
            if (!std::isfinite(c.a)) return bad("power must be finite");
            break;
        case I_EPMA:
            if (c.period < 2) return bad("period must be >= 2");
            if (!(c.a < (double)c.period)) return bad("offset must be < period");
            break;
        case I_TRIMA:
            if (c.period <= 3) return bad("period must be > 3");
            break;
        case I_STDDEV:
            if (!std::isfinite(c.a) || c.a < 0.0) return bad("nbdev must be finite and >= 0");
            break;
        case I_PNR:
            if (!(c.a >= 0.0 && c.a <= 100.0)) return bad("percentage must be in [0, 100]");
            break;
        default:
            break;
    }
    return VTA_OK;
}

static vta_status validate_combos(Ind ind, const std::vector<Combo>& cs, size_t len, size_t first) {
    if (cs.empty()) return fail(VTA_ERR_INVALID_INPUT, std::string(kInfo[ind].name) + ": no parameter combinations");
    size_t need = 0;
    for (const Combo& c : cs) {
        VTA_TRY(validate_combo(ind, c, len));
        need = std::max(need, needed_len(ind, c.period, c.a));
    }
    if (first >= len) return fail(VTA_ERR_INVALID_INPUT, std::string(kInfo[ind].name) + ": all values are NaN");
    if (len - first < need) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "%s: not enough valid data (needed >= %zu, valid = %zu)", kInfo[ind].name,
                      need, len - first);
        return fail(VTA_ERR_INVALID_INPUT, buf);
    }
    return VTA_OK;
}

// first valid index as each indicator defines it
static size_t host_first(Ind ind, const float* const* in, size_t n, size_t stride = 1, size_t off = 0) {
    auto at = [&](int k, size_t t) { return in[k][t * stride + off]; };
    if (kInfo[ind].in == IN_X) {
        size_t t = 0;
        while (t < n && std::isnan(at(0, t))) ++t;
        return t;
    }
    if (ind == I_ADX || ind == I_DONCHIAN) {  // max of the per-field firsts (adx.rs:190-198)
        size_t f = 0;
        for (int k = 0; k < kInfo[ind].in; ++k) {
            size_t t = 0;
            while (t < n && std::isnan(at(k, t))) ++t;
            if (t >= n) return n;
            f = std::max(f, t);
        }
        return f;
    }
    size_t t = 0;  // first index where h, l, c are all non-NaN (atr.rs:197-207)
    while (t < n && (std::isnan(at(0, t)) || std::isnan(at(1, t)) || std::isnan(at(2, t)))) ++t;
    return t;
}

// ------------------------------------------------------------ batch run ----
struct DevIn {
    const float* p[3];
};

// `warps_per_sm`: how many lane-warps x time chunks the chunked scan aims to
// have in flight per SM (the autotuner's recurrence knob; 64 untuned).
static int pick_chunk(vta_ctx* ctx, int n, int lanes, int warps_per_sm = 64) {
    const int pol = ctx->policy.recur_chunk;
    if (pol == 1) return ((n + 31) / 32) * 32;
    if (pol > 1) return pol;
    const long lane_warps = (lanes + 31) / 32;
    const long target = (long)ctx->num_sms * warps_per_sm;  // warps in flight we aim for
    long chunks = std::max(1L, target / std::max(1L, lane_warps));
    long len = (n + chunks - 1) / chunks;
    len = std::max<long>(len, kChunkMin);
    // a multiple of 64 steps: with the first chunk also one, every 64-step
    // row segment of the emit pass starts on a 256-byte boundary of its row
    // (a segment 128 bytes off one wrote about 10% slower)
    len = ((len + 63) / 64) * 64;
    while ((n + len - 1) / len > 65535) len *= 2;
    return (int)len;
}

// ------------------------------------------------------ sweep autotuner ---
// The launch knobs of the batch sweeps are picked by timing: the first call
// with a new (indicator, log2 length, log2 sweep size, knob) runs the sweep
// once per candidate (CUDA events around the call's kernels), keeps the
// fastest, and leaves the outputs of a run with that choice.  The choice is
// cached for the process and, with VTA_TUNE_CACHE=<file>, in <file>.sweeps
// ("indicator len_bucket combos_bucket knob value" per line).  Knobs:
//   TK_RECUR   chunked scans: lane-warps x chunks in flight per SM (32, 64, 128)
//   TK_MINMAX  sliding min/max: output tile (512, 1024 times per block)
//   TK_RECUR_TC  TK_RECUR where the chunk aggregates may take the tensor cores
// Policy "tune" = on (default) | off (untuned defaults) | cached (use cached
// choices, never time); server slots never time.
enum TuneKnob { TK_RECUR = 1, TK_MINMAX = 2, TK_RECUR_TC = 3 };
constexpr int kMmApLabel = -1;  // last_kernel marker: the min/max progression kernel ran
// ADX groups whose warm-restart run would exceed this many steps take the
// exact chunked scan; its chunks are at least kAdxScanMinL steps long
constexpr long long kAdxExactWarm = 4096;
constexpr long long kAdxScanMinL = 1024;
using SweepTuneKey = std::tuple<int, int, int, int>;
static std::mutex g_stune_mu;
static std::map<SweepTuneKey, int> g_stune;
static bool g_stune_loaded = false;

static int log2_bucket(long long v) {
    int b = 0;
    while ((1LL << b) < v) ++b;
    return b;
}

static std::string stune_path() {
    const char* p = std::getenv("VTA_TUNE_CACHE");
    return p && *p ? std::string(p) + ".sweeps" : std::string();
}

static bool stune_lookup(const SweepTuneKey& k, int* v) {
    std::lock_guard<std::mutex> lock(g_stune_mu);
    if (!g_stune_loaded) {
        g_stune_loaded = true;
        const std::string path = stune_path();
        if (!path.empty())
            if (FILE* f = std::fopen(path.c_str(), "r")) {
                int a, b, c, d, e;
                while (std::fscanf(f, "%d %d %d %d %d", &a, &b, &c, &d, &e) == 5)
                    if (e > 0) g_stune[SweepTuneKey{a, b, c, d}] = e;
                std::fclose(f);
            }
    }
    auto it = g_stune.find(k);
    if (it == g_stune.end()) return false;
    *v = it->second;
    return true;
}

static void stune_store(const SweepTuneKey& k, int v) {
    std::lock_guard<std::mutex> lock(g_stune_mu);
    g_stune[k] = v;
    const std::string path = stune_path();
    if (!path.empty())
        if (FILE* f = std::fopen(path.c_str(), "a")) {
            std::fprintf(f, "%d %d %d %d %d\n", std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k), v);
            std::fclose(f);
        }
}

// Weights of the tensor-core recurrence aggregates for (kind, L, periods):
// the context keeps up to kRwCap bytes of them across calls.  *build = 1 when
// the buffer does not hold them yet (the caller launches the weights kernel
// and then marks the entry valid).
constexpr size_t kRwCap = size_t(256) << 20;
static vta_status rw_get(vta_ctx* ctx, int kind, int L, const std::vector<int>& periods, size_t bytes,
                         vta_ctx::RwEntry** out, int* build) {
    for (auto& e : ctx->rw)
        if (e.kind == kind && e.L == L && e.bytes >= bytes && e.periods == periods) {
            e.tick = ++ctx->rw_tick;
            *out = &e;
            *build = e.valid ? 0 : 1;
            return VTA_OK;
        }
    size_t total = bytes;
    for (auto& e : ctx->rw) total += e.bytes;
    if (total > kRwCap) VTA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));  // buffers may be in use
    while (total > kRwCap && !ctx->rw.empty()) {
        size_t lru = 0;
        for (size_t i = 1; i < ctx->rw.size(); ++i)
            if (ctx->rw[i].tick < ctx->rw[lru].tick) lru = i;
        total -= ctx->rw[lru].bytes;
        cudaFree(ctx->rw[lru].dev);
        ctx->rw.erase(ctx->rw.begin() + (long)lru);
    }
    VTA_TRY(vram_check(bytes));
    void* dev = nullptr;
    VTA_CUDA_TRY(cudaMalloc(&dev, bytes));
    ctx->rw.push_back(vta_ctx::RwEntry{kind, L, periods, dev, bytes, ++ctx->rw_tick, false});
    *out = &ctx->rw.back();
    *build = 1;
    return VTA_OK;
}

// Runs `launch(candidate)` for every candidate, keeps the fastest and makes
// sure the outputs left behind are that candidate's.  `tag` gets the choice
// and whether it was timed now ("tuned") or taken from the cache ("cached").
template <class F>
static vta_status tuned_launch(vta_ctx* ctx, int ind, long long n, long long combos, int knob,
                               const std::vector<int>& cand, int dflt, F launch, int* chosen, const char** tag) {
    const SweepTuneKey key{ind, log2_bucket(n), log2_bucket(combos), knob};
    int v = 0;
    if (ctx->policy.tune != 1 && cand.size() > 1 && stune_lookup(key, &v) &&
        std::find(cand.begin(), cand.end(), v) != cand.end()) {
        *chosen = v;
        *tag = "cached";
        return launch(v);
    }
    if (ctx->policy.tune != 0 || ctx->async_alloc || cand.size() < 2) {
        *chosen = dflt;
        *tag = "default";
        return launch(dflt);
    }
    cudaStream_t st = ctx->stream;
    cudaEvent_t e0, e1;
    VTA_CUDA_TRY(cudaEventCreate(&e0));
    VTA_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_v = dflt;
    vta_status s = VTA_OK;
    // each candidate runs twice and keeps its faster time (the first launch
    // of a kernel variant pays one-time costs that say nothing of its speed)
    for (size_t i = 0; i < cand.size() && s == VTA_OK; ++i) {
        for (int rep = 0; rep < 2 && s == VTA_OK; ++rep) {
            cudaEventRecord(e0, st);
            s = launch(cand[i]);
            cudaEventRecord(e1, st);
            if (s == VTA_OK && cudaStreamSynchronize(st) != cudaSuccess) s = check_async("sweep tuning");
            float ms = 0.f;
            if (s == VTA_OK) cudaEventElapsedTime(&ms, e0, e1);
            if (s == VTA_OK && ms < best) {
                best = ms;
                best_v = cand[i];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != VTA_OK) return s;
    stune_store(key, best_v);
    *chosen = best_v;
    *tag = "tuned";
    // the last run's outputs stand unless another candidate won
    return best_v == cand.back() ? VTA_OK : launch(best_v);
}

vta_status upload_async(vta_ctx* ctx, void* dst, const void* src, size_t bytes, cudaStream_t st) {
    if (!bytes) return VTA_OK;
    const size_t off = (ctx->host_stage_off + 255) & ~size_t(255);
    if (ctx->host_stage && off + bytes <= ctx->host_stage_bytes) {
        // the staging region is reused by the next call only after the event
        // recorded behind this copy (check_ctx)
        char* h = static_cast<char*>(ctx->host_stage) + off;
        std::memcpy(h, src, bytes);
        ctx->host_stage_off = off + bytes;
        VTA_CUDA_TRY(cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, st));
        if (!ctx->stage_ev) VTA_CUDA_TRY(cudaEventCreateWithFlags(&ctx->stage_ev, cudaEventDisableTiming));
        VTA_CUDA_TRY(cudaEventRecord(ctx->stage_ev, st));
        ctx->stage_pending = true;
        return VTA_OK;
    }
    VTA_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return VTA_OK;
}

// Constant cache of a context (see vta_ctx::cc_*): a device buffer filled
// front to back by uploads; an upload whose bytes match an earlier one (hash,
// then a full compare with the host copy) reuses it.  When the buffer is full
// it starts over: the uploads are stream-ordered copies on the context's
// stream, behind every kernel of the earlier calls that reads the buffer
// (a stream switch waits for the old stream).  Server slots bypass it.
static constexpr size_t kConstCacheBytes = size_t(4) << 20;
static constexpr size_t kConstCacheMaxItem = size_t(256) << 10;

static uint64_t bytes_hash(const void* src, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(src);
    uint64_t h = 0x9E3779B97F4A7C15ull ^ n;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        std::memcpy(&w, b + i, 8);
        h = (h ^ w) * 0xff51afd7ed558ccdull;
        h ^= h >> 32;
    }
    for (; i < n; ++i) h = (h ^ b[i]) * 0x100000001b3ull;
    return h;
}

vta_status const_upload_bytes(vta_ctx* ctx, const void* src, size_t bytes, void* fallback, const void** out) {
    if (bytes == 0) {
        *out = fallback;
        return VTA_OK;
    }
    if (ctx->async_alloc || bytes > kConstCacheMaxItem) {
        VTA_TRY(upload_async(ctx, fallback, src, bytes, ctx->stream));
        *out = fallback;
        return VTA_OK;
    }
    const uint64_t h = bytes_hash(src, bytes);
    for (const auto& e : ctx->cc)
        if (e.hash == h && e.bytes == bytes && std::memcmp(ctx->cc_host.data() + e.off, src, bytes) == 0) {
            *out = static_cast<const char*>(ctx->cc_dev) + e.off;
            return VTA_OK;
        }
    if (!ctx->cc_dev) {
        if (vram_check(kConstCacheBytes) != VTA_OK || cudaMalloc(&ctx->cc_dev, kConstCacheBytes) != cudaSuccess) {
            cudaGetLastError();
            ctx->cc_dev = nullptr;
            VTA_TRY(upload_async(ctx, fallback, src, bytes, ctx->stream));
            *out = fallback;
            return VTA_OK;
        }
        ctx->cc_cap = kConstCacheBytes;
        ctx->cc_host.resize(kConstCacheBytes);
    }
    const size_t need = (bytes + 255) & ~size_t(255);
    if (ctx->cc_used + need > ctx->cc_cap) {
        ctx->cc_used = 0;
        ctx->cc.clear();
    }
    const size_t off = ctx->cc_used;
    std::memcpy(ctx->cc_host.data() + off, src, bytes);
    char* dst = static_cast<char*>(ctx->cc_dev) + off;
    VTA_TRY(upload_async(ctx, dst, src, bytes, ctx->stream));
    ctx->cc.push_back({h, off, bytes});
    ctx->cc_used = off + need;
    *out = dst;
    return VTA_OK;
}

vta_status ctx_aux(vta_ctx* ctx, size_t bytes, void** out) {
    if (bytes > ctx->aux_bytes && ctx->async_alloc) {
        if (ctx->aux) VTA_CUDA_TRY(cudaFreeAsync(ctx->aux, ctx->stream));
        ctx->aux = nullptr;
        ctx->aux_bytes = 0;
        VTA_CUDA_TRY(ctx->pool ? cudaMallocFromPoolAsync(&ctx->aux, bytes, ctx->pool, ctx->stream)
                               : cudaMallocAsync(&ctx->aux, bytes, ctx->stream));
        ctx->aux_bytes = bytes;
    }
    if (bytes > ctx->aux_bytes) {
        if (ctx->aux) {
            VTA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
            cudaFree(ctx->aux);
            ctx->aux = nullptr;
            ctx->aux_bytes = 0;
        }
        VTA_TRY(vram_check(bytes));
        VTA_CUDA_TRY(cudaMalloc(&ctx->aux, bytes));
        ctx->aux_bytes = bytes;
    }
    *out = ctx->aux;
    return VTA_OK;
}

static vta_status upload(vta_ctx* ctx, void* dst, const void* src, size_t bytes) {
    return upload_async(ctx, dst, src, bytes, ctx->stream);
}

static vta_status run_batch(vta_ctx* ctx, Ind ind, const DevIn& in, size_t len, size_t first,
                            const std::vector<Combo>& cs, float* const* out) {
    cudaStream_t st = ctx->stream;
    const int n = (int)len;
    const int nc = (int)cs.size();
    if (len > (size_t)INT32_MAX) return fail(VTA_ERR_INVALID_INPUT, "series longer than 2^31-1");
    std::vector<int> periods(nc);
    std::vector<double> pa(nc), pb(nc);
    std::vector<float> fa(nc), fb(nc);
    int pmax = 0;
    for (int i = 0; i < nc; ++i) {
        periods[i] = (int)cs[i].period;
        pa[i] = cs[i].a;
        pb[i] = cs[i].b;
        fa[i] = (float)cs[i].a;
        fb[i] = (float)cs[i].b;
        pmax = std::max(pmax, periods[i]);
    }
    Arena ar(ctx);
    ar.need(nc * sizeof(int));
    ar.need(nc * sizeof(double));
    ar.need(nc * sizeof(double));
    ar.need(nc * sizeof(float));
    ar.need(nc * sizeof(float));

    if (is_wwma(ind)) {
        // rows are window lengths from here on (the weight rows' length)
        std::vector<int> wextra(nc);
        bool any_extra = false;
        int kmax = 1;
        for (int i = 0; i < nc; ++i) {
            periods[i] = wwma_len(ind, cs[i]);
            wextra[i] = wwma_warm_extra(ind, cs[i]);
            any_extra = any_extra || wextra[i] != 0;
            kmax = std::max(kmax, periods[i]);
        }
        const int ntile = (nc + 15) / 16;
        ar.need((size_t)nc * kmax * sizeof(float));
        ar.need(ntile * sizeof(int));
        ar.need(len * sizeof(double));
        ar.need(prefix_tmp_doubles(n) * sizeof(double));
        ar.need(nc * sizeof(int));
        VTA_TRY(ar.commit());
        int* d_per = ar.take<int>(nc);
        double* d_pa = ar.take<double>(nc);
        double* d_pb = ar.take<double>(nc);
        ar.take<float>(nc);
        ar.take<float>(nc);
        float* d_w = ar.take<float>((size_t)nc * kmax);
        int* d_tk = ar.take<int>(ntile);
        double* d_nanp = ar.take<double>(len);
        double* d_tmp = ar.take<double>(prefix_tmp_doubles(n));
        int* d_wx = ar.take<int>(nc);
        if (ind == I_ALMA)  // the weight kernel takes m = offset (p - 1) and 1 / (2 s^2) = sigma^2 / (2 p^2)
            for (int i = 0; i < nc; ++i) {
                const double pd = (double)periods[i];
                pa[i] = pa[i] * (pd - 1.0);
                pb[i] = pb[i] * pb[i] / (2.0 * pd * pd);
            }
        std::vector<int> tk(ntile, 0);
        for (int i = 0; i < nc; ++i) tk[i / 16] = std::max(tk[i / 16], periods[i]);
        VTA_TRY(upload(ctx, d_per, periods.data(), nc * sizeof(int)));
        VTA_TRY(upload(ctx, d_pa, pa.data(), nc * sizeof(double)));
        VTA_TRY(upload(ctx, d_pb, pb.data(), nc * sizeof(double)));
        VTA_TRY(upload(ctx, d_tk, tk.data(), ntile * sizeof(int)));
        if (any_extra) VTA_TRY(upload(ctx, d_wx, wextra.data(), nc * sizeof(int)));
        VTA_TRY(launch_weights(wwma_weight_kind(ind), d_per, d_pa, d_pb, nc, kmax, d_w, st));
        VTA_TRY(launch_prefix_f64(in.p[0], n, (int)first, PK_NAN, d_nanp, nullptr, d_tmp, st));
        WwmaBatchArgs a{};
        a.x = in.p[0];
        a.n = n;
        a.first = (int)first;
        a.w = d_w;
        a.periods = d_per;
        a.periods_host = periods.data();
        a.tile_kmax = d_tk;
        a.kmax = kmax;
        a.n_combos = nc;
        // running-sum indicators (WMA, SWMA, TRIMA) keep a NaN forever
        a.nan_mode = (ind == I_WMA || ind == I_SWMA || ind == I_TRIMA) ? 1 : 0;
        a.nanp = d_nanp;
        a.warm_extra = any_extra ? d_wx : nullptr;
        a.out = out[0];
        const int pol = ctx->policy.wma_batch;
        if (pol == 0 || pol >= 2) {
            const vta_status s = launch_wwma_batch_tc(a, pol == 3 ? 1 : 0, ctx, st);
            if (s == VTA_OK) {
                ctx->last_kernel = pol == 3 ? "wwma_tc_bf16x3" : "wwma_tc_fp16x3";
                return VTA_OK;
            }
            if (s != VTA_ERR_NOT_IMPLEMENTED || pol >= 2) return s;
        }
        ctx->last_kernel = "wwma_plain_f32";
        return launch_wwma_batch_plain(a, st);
    }

    switch (ind) {
        case I_EMA: case I_DEMA: case I_TEMA: case I_RSI: case I_WILDERS: case I_ATR: {
            // EMA/DEMA/TEMA/RSI: the last seed index of the sweep; chunks that
            // start past it run the fast aggregate pass.  With the automatic
            // policy chunk 0 ends just past it, so that only one short chunk
            // takes the general seeding path.
            const bool fast_kind = ind == I_EMA || ind == I_DEMA || ind == I_TEMA || ind == I_RSI;
            long long s_max = 0;
            for (int i = 0; i < nc; ++i) {
                const long long p = periods[i];
                const long long s = ind == I_EMA ? (long long)first + p - 1
                                    : ind == I_DEMA ? (long long)first
                                    : ind == I_TEMA ? (long long)first + 2 * (p - 1)
                                    : (long long)first + p;
                s_max = std::max(s_max, s);
            }
            // chunking for a target of `wps` lane-warps x chunks per SM
            struct Chunking {
                int chunk, chunk0, nch, fast_from;
                int tc_nc;  // full-length chunks from fast_from on (tensor-core aggregates)
            };
            auto chunking = [&](int wps) {
                Chunking c{};
                c.chunk = pick_chunk(ctx, n, nc, wps);
                c.chunk0 = c.chunk;
                if (fast_kind && ctx->policy.recur_chunk == 0 && s_max + 1 < n)
                    c.chunk0 = (int)std::max<long long>(64, ((s_max + 1 + 63) / 64) * 64);
                c.nch = recur_n_chunks(n, c.chunk, c.chunk0);
                c.fast_from = c.nch;
                for (int k = 1; k < c.nch; ++k) {
                    int c0 = 0, c1 = 0;
                    RecurArgs tmp{};
                    tmp.n = n;
                    tmp.chunk = c.chunk;
                    tmp.chunk0 = c.chunk0;
                    recur_chunk_bounds(tmp, k, c0, c1);
                    if (c0 > s_max) {
                        c.fast_from = k;
                        break;
                    }
                }
                c.tc_nc = 0;
                if (c.fast_from < c.nch) {
                    int c0 = 0, c1 = 0;
                    RecurArgs tmp{};
                    tmp.n = n;
                    tmp.chunk = c.chunk;
                    tmp.chunk0 = c.chunk0;
                    recur_chunk_bounds(tmp, c.nch - 1, c0, c1);
                    c.tc_nc = c.nch - c.fast_from - (c1 - c0 < c.chunk ? 1 : 0);
                }
                return c;
            };
            // tensor-core chunk aggregates: EMA / DEMA / TEMA / RSI with at
            // least a few full chunks past every seed and a workspace (the
            // packed weights and inputs) of at most 1 GiB
            const int tc_kind = ind == I_EMA ? RK_EMA : ind == I_DEMA ? RK_DEMA : ind == I_TEMA ? RK_TEMA : RK_RSI;
            constexpr size_t kTcWsCap = size_t(1) << 30;
            auto tc_geo = [&](const Chunking& c) { return recur_agg_tc_geo(tc_kind, nc, c.chunk, c.tc_nc, ctx->num_sms); };
            auto tc_ok = [&](const Chunking& c) {
                if (!(fast_kind && ctx->policy.recur_agg != 1 && c.nch > 1 && c.tc_nc >= 2 && c.chunk % 32 == 0 &&
                      ctx->smem_optin >= recur_agg_tc_smem()))
                    return false;
                const RecurTcGeo g = tc_geo(c);
                return g.ws_bytes + g.w_bytes <= kTcWsCap && g.w_bytes <= kRwCap;
            };
            const std::vector<int> cand = ctx->policy.recur_chunk == 0 ? std::vector<int>{32, 64, 128}
                                                                       : std::vector<int>{64};
            int max_nch = 1;
            size_t tc_ws = 0, tc_w = 0;
            bool tc_any = false;
            for (int w : cand) {
                const Chunking c = chunking(w);
                max_nch = std::max(max_nch, c.nch);
                if (tc_ok(c)) {
                    tc_any = true;
                    const RecurTcGeo g = tc_geo(c);
                    tc_ws = std::max(tc_ws, g.ws_bytes);
                    tc_w = std::max(tc_w, g.w_bytes);
                }
            }
            // server slots (stream-ordered workspaces) rebuild the weights per call
            const bool tc_cache = !ctx->async_alloc;
            if (ctx->policy.recur_agg == 2 && !tc_any)
                return fail(VTA_ERR_NOT_IMPLEMENTED, "recur_agg=tc: this sweep has no tensor-core chunk aggregates");
            ar.need((size_t)max_nch * nc * 16);
            ar.need((size_t)max_nch * nc * 16);
            if (tc_any) {
                ar.need(tc_ws);
                if (!tc_cache) ar.need(tc_w);
                ar.need((size_t)max_nch * sizeof(int));
                ar.need(sizeof(int));
            }
            VTA_TRY(ar.commit());
            const int* d_per = nullptr;
            VTA_TRY(const_upload(ctx, periods.data(), nc, ar.take<int>(nc), &d_per));
            ar.take<double>(nc);
            ar.take<double>(nc);
            ar.take<float>(nc);
            ar.take<float>(nc);
            float* d_agg = ar.take<float>((size_t)max_nch * nc * 4);
            float* d_carry = ar.take<float>((size_t)max_nch * nc * 4);
            void* d_tc_ws = tc_any ? ar.take<char>(tc_ws) : nullptr;
            void* d_tc_w = tc_any && !tc_cache ? ar.take<char>(tc_w) : nullptr;
            int* d_tc_done = tc_any ? ar.take<int>(max_nch) : nullptr;
            int* d_tc_err = tc_any ? ar.take<int>(1) : nullptr;
            RecurArgs a{};
            a.kind = ind == I_EMA ? RK_EMA : ind == I_DEMA ? RK_DEMA : ind == I_TEMA ? RK_TEMA
                   : ind == I_RSI ? RK_RSI : ind == I_WILDERS ? RK_WILDERS : RK_ATR;
            a.layout = 0;
            a.x = in.p[0];
            if (ind == I_ATR) { a.h = in.p[0]; a.l = in.p[1]; a.c = in.p[2]; a.x = in.p[2]; }
            a.n = n;
            a.first = (int)first;
            a.periods = d_per;
            a.n_lanes = nc;
            a.out = out[0];
            a.agg = d_agg;
            a.carry = d_carry;
            int nch_used = 1;
            bool tc_used = false;
            auto launch = [&](int wps) {
                const Chunking c = chunking(wps);
                a.chunk = c.chunk;
                a.chunk0 = c.chunk0;
                a.fast_from = c.fast_from;
                a.fast_agg = (fast_kind && c.nch > 1 && c.fast_from < c.nch) ? 1 : 0;
                nch_used = c.nch;
                a.tc = RecurTcView{};
                tc_used = false;
                if (a.fast_agg && tc_ok(c)) {
                    RecurTcArgs t{};
                    t.kind = tc_kind;
                    t.x = a.x;
                    t.periods = d_per;
                    t.n_lanes = nc;
                    t.L = c.chunk;
                    t.chunk0 = c.chunk0;
                    t.g0 = c.fast_from;
                    t.nc = c.tc_nc;
                    t.geo = tc_geo(c);
                    vta_ctx::RwEntry* ent = nullptr;
                    if (tc_cache) {
                        VTA_TRY(rw_get(ctx, tc_kind, c.chunk, periods, t.geo.w_bytes, &ent, &t.build_weights));
                        t.wts = ent->dev;
                    } else {
                        t.wts = d_tc_w;
                        t.build_weights = 1;
                    }
                    t.ws = d_tc_ws;
                    t.done = d_tc_done;
                    t.err = d_tc_err;
                    VTA_TRY(launch_recur_agg_tc(t, ctx->smem_optin, st));
                    if (ent) ent->valid = true;
                    RecurTcView& v = a.tc;
                    v.done = d_tc_done;
                    v.err = d_tc_err;
                    v.g0 = t.g0;
                    v.nc = t.nc;
                    const char* ws = static_cast<const char*>(t.ws);
                    const char* wb = static_cast<const char*>(t.wts);
                    v.part = reinterpret_cast<const float*>(ws + t.geo.part_off);
                    v.S = t.geo.S;
                    v.npad = t.geo.npad;
                    v.rows = t.geo.rows;
                    v.mpad = t.geo.mpad;
                    v.row_scale = reinterpret_cast<const float*>(wb + t.geo.row_scale_off);
                    v.row_sum = reinterpret_cast<const float*>(wb + t.geo.row_sum_off);
                    v.col_scale = reinterpret_cast<const float*>(ws + t.geo.col_scale_off);
                    v.col_ref = reinterpret_cast<const float*>(ws + t.geo.col_ref_off);
                    tc_used = true;
                }
                return launch_recurrence(a, st);
            };
            int wps = 64;
            const char* tag = "default";
            const int knob = (fast_kind && ctx->policy.recur_agg != 1) ? TK_RECUR_TC : TK_RECUR;
            VTA_TRY(tuned_launch(ctx, (int)ind, n, nc, knob, cand, 64, launch, &wps, &tag));
            ctx->last_kernel = nch_used > 1 ? "recurrence_chunked" : "recurrence_sequential";
            if (nch_used > 1 && ctx->policy.recur_chunk == 0)
                ctx->last_kernel += "(chunk=" + std::to_string(a.chunk) + ", " + std::to_string(wps) + " warps/SM, " +
                                    (tc_used ? "tc aggregates, " : "") + tag + ")";
            else if (tc_used)
                ctx->last_kernel += "(tc aggregates)";
            return VTA_OK;
        }
        case I_ADX: case I_SUPERTREND: {
            // time-chunked with verified warm restarts unless the policy asks
            // for the sequential kernel; per 32-combo group a chunk of at least
            // the warm length (else the group runs as one chunk)
            const int G = (nc + 31) / 32;
            std::vector<int> gchunk(G), gwarm(G);
            std::vector<int2> items;
            int max_nch = 1;
            bool chunked = false;
            std::vector<int> adx_groups, adx_s0;  // groups on the exact scan and their s0
            int adx_L = 0;
            if (ctx->policy.recur_chunk != 1) {
                // warm length per group: 32 p steps shrink the guessed state's
                // error by (1 - 1/p)^(32 p) < e^-32, far below an f32 ulp, so the
                // warm run (almost always) lands on the exact state; the fix-up
                // pass covers the rest
                auto warm_of = [&](int g) {
                    int pm = 1;
                    for (int i = g * 32; i < std::min(nc, g * 32 + 32); ++i) pm = std::max(pm, periods[i]);
                    long long w = ((32LL * pm + 64) + 31) & ~31LL;
                    if (ctx->policy.tm_warm > 0) w = ((long long)ctx->policy.tm_warm + 31) & ~31LL;
                    return w;
                };
                // ADX groups whose warm run would be long take the exact
                // chunked scan (k_adx_scan.cu) after a seeding chunk [0, s0)
                // run here as the group's only item
                if (ind == I_ADX && ctx->policy.tm_warm == 0) {
                    std::vector<int> cand_g, cand_s0;
                    for (int g = 0; g < G; ++g) {
                        int pm = 1;
                        for (int i = g * 32; i < std::min(nc, g * 32 + 32); ++i) pm = std::max(pm, periods[i]);
                        const long long s0 = (((long long)first + 2LL * pm) + 31) & ~31LL;
                        if (32LL * pm + 64 > kAdxExactWarm && s0 + 2LL * kAdxScanMinL <= n) {
                            cand_g.push_back(g);
                            cand_s0.push_back((int)s0);
                        }
                    }
                    if (!cand_g.empty()) {
                        // chunk length: about 2,400 warp items over the scan
                        long long work = 0;
                        for (int s0v : cand_s0) work += n - s0v;
                        long long L = ((work / 2400) + 31) & ~31LL;
                        L = std::max<long long>(kAdxScanMinL, std::min<long long>(16384, L));
                        if (ctx->policy.scan_chunk > 0) L = ctx->policy.scan_chunk;
                        adx_L = (int)L;
                        adx_groups = cand_g;
                        adx_s0 = cand_s0;
                    }
                }
                auto is_scan = [&](int g) {
                    return std::find(adx_groups.begin(), adx_groups.end(), g) != adx_groups.end();
                };
                long long w_max = 0;
                for (int g = 0; g < G; ++g)
                    if (!is_scan(g)) w_max = std::max(w_max, warm_of(g));
                // an item runs warm + chunk steps; the items of every group are
                // made about equally long (1.5 x the longest warm), so the
                // large-period groups' items do not form the critical path
                const long long item_len = w_max + w_max / 2;
                for (int g = 0; g < G; ++g) {
                    if (is_scan(g)) {
                        const size_t gi = (size_t)(std::find(adx_groups.begin(), adx_groups.end(), g) -
                                                   adx_groups.begin());
                        gchunk[g] = adx_s0[gi];  // chunk 0 = the seeding run; the scan does the rest
                        gwarm[g] = 0;
                        items.push_back(make_int2(g, 0));
                        chunked = true;
                        continue;
                    }
                    const long long w = warm_of(g);
                    long long c = std::max<long long>(1024, item_len - w);
                    if (ctx->policy.recur_chunk > 1) c = std::max<long long>(ctx->policy.recur_chunk, w);
                    c = (c + 31) & ~31LL;
                    if (2 * c > n) c = ((long long)n + 31) & ~31LL;  // one chunk: the sequential run
                    gchunk[g] = (int)c;
                    gwarm[g] = (int)std::min<long long>(w, INT32_MAX / 2);
                    const int nch = (int)((n + c - 1) / c);
                    max_nch = std::max(max_nch, nch);
                    chunked = chunked || nch > 1;
                    for (int k = 0; k < nch; ++k) items.push_back(make_int2(g, k));
                }
                // longest items first (chunk + warm steps), so the long warm
                // runs of large-period groups do not trail at the end
                std::stable_sort(items.begin(), items.end(), [&](const int2& x, const int2& y) {
                    return (long long)gchunk[x.x] + gwarm[x.x] > (long long)gchunk[y.x] + gwarm[y.x];
                });
            }
            // the exact scan's items and state slots
            std::vector<int2> scan_items;
            int scan_nch = 1;
            for (size_t gi = 0; gi < adx_groups.size(); ++gi) {
                const int nch_g = 1 + (int)((n - adx_s0[gi] + adx_L - 1) / adx_L);
                scan_nch = std::max(scan_nch, nch_g);
                for (int k = 1; k < nch_g; ++k) scan_items.push_back(make_int2((int)gi, k));
            }
            const size_t scan_slots = adx_groups.size() * 32;
            if (chunked) {
                const size_t states = (size_t)max_nch * nc;
                ar.need(G * sizeof(int));
                ar.need(G * sizeof(int));
                ar.need(items.size() * sizeof(int2));
                ar.need(states * 8 * sizeof(float));
                ar.need(states * 8 * sizeof(float));
                ar.need(states);
                ar.need(sizeof(int));
                ar.need(nc * sizeof(int));
                if (!adx_groups.empty()) {
                    ar.need(adx_groups.size() * sizeof(int));
                    ar.need(adx_groups.size() * sizeof(int));
                    ar.need(scan_items.size() * sizeof(int2));
                    ar.need((size_t)scan_nch * scan_slots * sizeof(float4));
                    ar.need((size_t)scan_nch * scan_slots * sizeof(float4));
                    ar.need((size_t)scan_nch * scan_slots * sizeof(float));
                    ar.need((size_t)scan_nch * scan_slots * sizeof(float));
                }
            }
            VTA_TRY(ar.commit());
            int* d_per = ar.take<int>(nc);
            ar.take<double>(nc);
            ar.take<double>(nc);
            float* d_fa = ar.take<float>(nc);
            ar.take<float>(nc);
            VTA_TRY(upload(ctx, d_per, periods.data(), nc * sizeof(int)));
            VTA_TRY(upload(ctx, d_fa, fa.data(), nc * sizeof(float)));
            if (chunked) {
                const size_t states = (size_t)max_nch * nc;
                HlcChunkArgs c{};
                c.kind = ind == I_ADX ? 0 : 1;
                c.h = in.p[0]; c.l = in.p[1]; c.c = in.p[2];
                c.n = n;
                c.first = (int)first;
                c.periods = d_per;
                c.factors = ind == I_SUPERTREND ? d_fa : nullptr;
                c.n_combos = nc;
                int* d_gc = ar.take<int>(G);
                int* d_gw = ar.take<int>(G);
                int2* d_items = ar.take<int2>(items.size());
                c.st_start = ar.take<float>(states * 8);
                c.st_end = ar.take<float>(states * 8);
                c.exact = ar.take<unsigned char>(states);
                c.fixups = ar.take<int>(1);
                c.need = ar.take<int>(nc);
                c.max_chunks = max_nch;
                VTA_CUDA_TRY(cudaMemsetAsync(c.need, 0, nc * sizeof(int), st));
                // chunks the warm-restart kernel does not write (the exact
                // scan's groups) read as exact, so the fix-up leaves them alone
                if (!adx_groups.empty()) VTA_CUDA_TRY(cudaMemsetAsync(c.exact, 1, states, st));
                VTA_TRY(upload(ctx, d_gc, gchunk.data(), G * sizeof(int)));
                VTA_TRY(upload(ctx, d_gw, gwarm.data(), G * sizeof(int)));
                VTA_TRY(upload(ctx, d_items, items.data(), items.size() * sizeof(int2)));
                VTA_CUDA_TRY(cudaMemsetAsync(c.fixups, 0, sizeof(int), st));
                c.group_chunk = d_gc;
                c.group_warm = d_gw;
                c.items = d_items;
                c.n_items = (int)items.size();
                c.out0 = out[0];
                c.out1 = ind == I_SUPERTREND ? out[1] : nullptr;
                ctx->last_kernel = ind == I_ADX ? "adx_chunked" : "supertrend_chunked";
                VTA_TRY(launch_hlc_chunk(c, st));
                if (adx_groups.empty()) return VTA_OK;
                AdxScanArgs x{};
                x.h = in.p[0]; x.l = in.p[1]; x.c = in.p[2];
                x.n = n;
                x.periods = d_per;
                x.n_combos = nc;
                int* d_sg = ar.take<int>(adx_groups.size());
                int* d_ss = ar.take<int>(adx_groups.size());
                int2* d_si = ar.take<int2>(scan_items.size());
                VTA_TRY(upload(ctx, d_sg, adx_groups.data(), adx_groups.size() * sizeof(int)));
                VTA_TRY(upload(ctx, d_ss, adx_s0.data(), adx_s0.size() * sizeof(int)));
                if (!scan_items.empty())
                    VTA_TRY(upload(ctx, d_si, scan_items.data(), scan_items.size() * sizeof(int2)));
                x.groups = d_sg;
                x.group_s0 = d_ss;
                x.n_groups = (int)adx_groups.size();
                x.n_slots = (int)scan_slots;
                x.L = adx_L;
                x.items = d_si;
                x.n_items = (int)scan_items.size();
                x.seed_state = c.st_end;
                x.agg1 = ar.take<float4>((size_t)scan_nch * scan_slots);
                x.carry1 = ar.take<float4>((size_t)scan_nch * scan_slots);
                x.agg2 = ar.take<float>((size_t)scan_nch * scan_slots);
                x.carry2 = ar.take<float>((size_t)scan_nch * scan_slots);
                x.out = out[0];
                VTA_TRY(launch_adx_scan(x, st));
                ktimer_end(st);  // the call's timing covers the scan too
                ctx->last_kernel = "adx_chunked(" + std::to_string(adx_groups.size()) + " of " + std::to_string(G) +
                                   " groups on the exact scan, L=" + std::to_string(adx_L) + ")";
                return VTA_OK;
            }
            HlcArgs a{};
            a.layout = 0;
            a.h = in.p[0]; a.l = in.p[1]; a.c = in.p[2];
            a.n = n;
            a.first = (int)first;
            a.periods = d_per;
            a.factors = d_fa;
            a.n_lanes = nc;
            a.out0 = out[0];
            a.out1 = ind == I_SUPERTREND ? out[1] : nullptr;
            ctx->last_kernel = ind == I_ADX ? "adx_sequential" : "supertrend_sequential";
            return ind == I_ADX ? launch_adx(a, st) : launch_supertrend(a, st);
        }
        case I_SMA: case I_STDDEV: case I_ZSCORE: case I_BB: {
            ar.need(2 * sizeof(int));
            VTA_TRY(ar.commit());
            const int* d_per = nullptr;
            VTA_TRY(const_upload(ctx, periods.data(), nc, ar.take<int>(nc), &d_per));
            ar.take<double>(nc);
            ar.take<double>(nc);
            float* fa_slot = ar.take<float>(nc);
            float* fb_slot = ar.take<float>(nc);
            int* d_bad = ar.take<int>(2);
            // per-combo scales: nbdev (StdDev / Z-score), devup and devdn (BB);
            // SMA has none
            const float* d_fa = nullptr;
            const float* d_fb = nullptr;
            if (ind != I_SMA) VTA_TRY(const_upload(ctx, fa.data(), nc, fa_slot, &d_fa));
            if (ind == I_BB) VTA_TRY(const_upload(ctx, fb.data(), nc, fb_slot, &d_fb));
            PrefixWinArgs a{};
            a.kind = ind == I_SMA ? WK_SMA : ind == I_STDDEV ? WK_STDDEV : ind == I_ZSCORE ? WK_ZSCORE : WK_BB;
            a.x = in.p[0];
            a.bad = d_bad;
            a.n = n;
            a.first = (int)first;
            a.periods = d_per;
            a.k1 = d_fa;
            a.k2 = d_fb;
            a.n_combos = nc;
            a.out0 = out[0];
            if (ind == I_BB) { a.out0 = out[0]; a.out1 = out[1]; a.out2 = out[2]; }
            ctx->last_kernel = "prefix_window_ds";
            return launch_prefix_window_batch(a, pmax, ctx->smem_optin, st);
        }
        case I_DONCHIAN: case I_WILLR: {
            ar.need(((size_t)n + 1023) / 1024 * sizeof(int));  // per-tile flags of the progression kernel
            VTA_TRY(ar.commit());
            const int* d_per = nullptr;
            VTA_TRY(const_upload(ctx, periods.data(), nc, ar.take<int>(nc), &d_per));
            MinMaxArgs a{};
            a.dirty = ar.take<int>(((size_t)n + 1023) / 1024);
            a.kind = ind == I_DONCHIAN ? MM_DONCHIAN : MM_WILLR;
            a.tile_hint = 0;
            a.h = in.p[0]; a.l = in.p[1];
            a.c = ind == I_WILLR ? in.p[2] : nullptr;
            a.n = n;
            a.first = (int)first;
            a.periods = d_per;
            a.n_combos = nc;
            a.pmax = pmax;
            a.out0 = out[0];
            if (ind == I_DONCHIAN) { a.out1 = out[1]; a.out2 = out[2]; }
            // an ascending arithmetic progression of periods (range grids)
            a.ap_d = 0;
            if (nc >= 2 && periods[1] > periods[0]) {
                const int d = periods[1] - periods[0];
                bool ap = d <= 64;
                for (int i = 2; i < nc && ap; ++i) ap = periods[i] - periods[i - 1] == d;
                if (ap) a.ap_d = d;
            }
            int tile = 0;
            const char* tag = "default";
            auto launch = [&](int t) {
                a.tile_hint = t;
                return launch_minmax_batch(a, ctx->smem_optin, st);
            };
            VTA_TRY(tuned_launch(ctx, (int)ind, n, nc, TK_MINMAX, minmax_tile_candidates(a, ctx->smem_optin), 0,
                                 launch, &tile, &tag));
            const int thr = (tile >> 16) & 0xfff;
            a.tile_hint = tile;
            if (minmax_uses_progression(a, ctx->smem_optin)) tile = kMmApLabel;
            ctx->last_kernel = std::string("minmax_sparse_table(") +
                               (tile == kMmApLabel ? std::string("progression, tile=1024")
                                : tile ? "tile=" + std::to_string(tile & 0xffff) + ", threads=" +
                                             std::to_string(thr ? thr : 512) + ((tile >> 28) & 1 ? ", split" : "")
                                       : std::string("tile=auto")) +
                               ", " + tag + ")";
            return VTA_OK;
        }
        case I_PNR: {
            const int nchunk = (n + 255) / 256;
            const size_t sc = pmax > 64 ? (size_t)nchunk * nc * pmax : 0;
            ar.need(sc * sizeof(float));
            VTA_TRY(ar.commit());
            int* d_per = ar.take<int>(nc);
            ar.take<double>(nc);
            ar.take<double>(nc);
            float* d_fa = ar.take<float>(nc);
            ar.take<float>(nc);
            float* d_sc = sc ? ar.take<float>(sc) : nullptr;
            std::vector<float> pf(nc);
            // p_frac = percentage * 0.01 in f64 (percentile_nearest_rank.rs:213)
            std::vector<double> pfd(nc);
            for (int i = 0; i < nc; ++i) pf[i] = (float)(cs[i].a * 0.01);
            VTA_TRY(upload(ctx, d_per, periods.data(), nc * sizeof(int)));
            VTA_TRY(upload(ctx, d_fa, pf.data(), nc * sizeof(float)));
            PnrArgs a{};
            a.layout = 0;
            a.x = in.p[0];
            a.n = n;
            a.first = (int)first;
            a.lengths = d_per;
            a.pfrac = d_fa;
            a.length = pmax;
            a.n_lanes = nc;
            a.out = out[0];
            a.scratch = d_sc;
            ctx->last_kernel = "percentile_sorted_window";
            return launch_percentile(a, st);
        }
        default:
            return fail(VTA_ERR_NOT_IMPLEMENTED, "indicator not implemented");
    }
}

// ------------------------------------------------------------ tm run -------
static vta_status run_tm(vta_ctx* ctx, Ind ind, const DevIn& in, size_t cols, size_t rows, const Combo& c,
                         float* const* out) {
    cudaStream_t st = ctx->stream;
    if (rows > (size_t)INT32_MAX || cols > (size_t)INT32_MAX)
        return fail(VTA_ERR_INVALID_INPUT, "matrix too large");
    const int C = (int)cols, R = (int)rows;
    const int p = (int)c.period;
    // ADX, SuperTrend and the percentile (window <= 64) run on the many-series
    // work-list kernels (time-chunked, bit-identical to the sequential kernels
    // below, which the "sequential" policy keeps)
    if (ctx->policy.recur_chunk != 1 &&
        (ind == I_ADX || ind == I_SUPERTREND || (ind == I_PNR && c.period <= 64))) {
        const int kind = ind == I_ADX ? 1 : ind == I_SUPERTREND ? 2 : 3;
        ctx->last_kernel = ind == I_ADX ? "adx_tm_chunked" : ind == I_SUPERTREND ? "supertrend_tm_chunked"
                                                                               : "percentile_tm_register";
        if (ind == I_PNR)
            return tm_job_enqueue(ctx, kind, p, c.a, nullptr, nullptr, in.p[0], C, R, out[0], nullptr, st);
        return tm_job_enqueue(ctx, kind, p, c.a, in.p[0], in.p[1], in.p[2], C, R, out[0],
                              ind == I_SUPERTREND ? out[1] : nullptr, st);
    }
    Arena ar(ctx);
    ar.need(2 * cols * sizeof(int));  // first + first_nan
    const bool recur = ind == I_EMA || ind == I_DEMA || ind == I_TEMA || ind == I_RSI || ind == I_WILDERS ||
                       ind == I_ATR;
    int chunk = 0, nch = 0;
    if (recur) {
        chunk = pick_chunk(ctx, R, C);
        nch = (R + chunk - 1) / chunk;
        ar.need((size_t)nch * cols * 16);
        ar.need((size_t)nch * cols * 16);
    }
    const int pw = is_wwma(ind) ? wwma_len(ind, c) : 0;
    ar.need(pw * sizeof(float));
    ar.need(sizeof(int));
    ar.need(2 * sizeof(double));
    const size_t pnr_sc = (ind == I_PNR && p > 64) ? (size_t)((R + 255) / 256) * cols * p : 0;
    ar.need(pnr_sc * sizeof(float));
    VTA_TRY(ar.commit());
    int* d_first = ar.take<int>(2 * cols);
    float* d_agg = recur ? ar.take<float>((size_t)nch * cols * 4) : nullptr;
    float* d_carry = recur ? ar.take<float>((size_t)nch * cols * 4) : nullptr;
    float* d_w = ar.take<float>(pw);
    int* d_p1 = ar.take<int>(1);
    double* d_ab = ar.take<double>(2);
    float* d_sc = pnr_sc ? ar.take<float>(pnr_sc) : nullptr;

    if (kInfo[ind].in == IN_X) VTA_TRY(launch_first_valid_tm(in.p[0], C, R, d_first, st));
    else if (ind == I_DONCHIAN) VTA_TRY(launch_first_valid_tm_hlc(in.p[0], in.p[1], in.p[1], C, R, d_first, st));
    else VTA_TRY(launch_first_valid_tm_hlc(in.p[0], in.p[1], in.p[2], C, R, d_first, st));

    if (is_wwma(ind)) {
        double ab[2] = {c.a, c.b};
        if (ind == I_ALMA) {  // m and 1 / (2 s^2), as in the batch path
            ab[0] = c.a * ((double)pw - 1.0);
            ab[1] = c.b * c.b / (2.0 * (double)pw * (double)pw);
        }
        VTA_TRY(upload(ctx, d_p1, &pw, sizeof(int)));
        VTA_TRY(upload(ctx, d_ab, ab, sizeof ab));
        VTA_TRY(launch_weights(wwma_weight_kind(ind), d_p1, d_ab, d_ab + 1, 1, pw, d_w, st));
        WwmaTmArgs a{};
        a.x_tm = in.p[0];
        a.cols = C;
        a.rows = R;
        a.first = d_first;
        a.w = d_w;
        a.period = pw;
        a.warm_extra = wwma_warm_extra(ind, c);
        a.nan_mode = (ind == I_WMA || ind == I_SWMA || ind == I_TRIMA) ? 1 : 0;
        a.out_tm = out[0];
        ctx->last_kernel = "wwma_tm_f32";
        return launch_wwma_tm(a, st);
    }
    if (recur) {
        RecurArgs a{};
        a.kind = ind == I_EMA ? RK_EMA : ind == I_DEMA ? RK_DEMA : ind == I_TEMA ? RK_TEMA
               : ind == I_RSI ? RK_RSI : ind == I_WILDERS ? RK_WILDERS : RK_ATR;
        a.layout = 1;
        a.x = in.p[0];
        if (ind == I_ATR) { a.h = in.p[0]; a.l = in.p[1]; a.c = in.p[2]; a.x = in.p[2]; }
        a.n = R;
        a.cols = C;
        a.first_tm = d_first;
        a.period = p;
        a.n_lanes = C;
        a.chunk = chunk;
        a.out = out[0];
        a.agg = d_agg;
        a.carry = d_carry;
        ctx->last_kernel = "recurrence_tm";
        return launch_recurrence(a, st);
    }
    switch (ind) {
        case I_ADX: case I_SUPERTREND: {
            HlcArgs a{};
            a.layout = 1;
            a.h = in.p[0]; a.l = in.p[1]; a.c = in.p[2];
            a.n = R;
            a.cols = C;
            a.first_tm = d_first;
            a.period = p;
            a.factor = (float)c.a;
            a.n_lanes = C;
            a.out0 = out[0];
            a.out1 = ind == I_SUPERTREND ? out[1] : nullptr;
            ctx->last_kernel = ind == I_ADX ? "adx_tm" : "supertrend_tm";
            return ind == I_ADX ? launch_adx(a, st) : launch_supertrend(a, st);
        }
        case I_SMA: case I_STDDEV: case I_ZSCORE: case I_BB: {
            PrefixWinTmArgs a{};
            a.kind = ind == I_SMA ? WK_SMA : ind == I_STDDEV ? WK_STDDEV : ind == I_ZSCORE ? WK_ZSCORE : WK_BB;
            a.x_tm = in.p[0];
            a.cols = C;
            a.rows = R;
            a.first = d_first;
            a.period = p;
            a.k1 = (float)c.a;
            a.k2 = (float)c.b;
            a.out0 = out[0];
            if (ind == I_BB) { a.out1 = out[1]; a.out2 = out[2]; }
            ctx->last_kernel = "prefix_window_tm";
            return launch_prefix_window_tm(a, st);
        }
        case I_DONCHIAN: case I_WILLR: {
            MinMaxTmArgs a{};
            a.kind = ind == I_DONCHIAN ? MM_DONCHIAN : MM_WILLR;
            a.h = in.p[0]; a.l = in.p[1];
            a.c = ind == I_WILLR ? in.p[2] : nullptr;
            a.cols = C;
            a.rows = R;
            a.first = d_first;
            a.period = p;
            a.out0 = out[0];
            if (ind == I_DONCHIAN) { a.out1 = out[1]; a.out2 = out[2]; }
            ctx->last_kernel = "minmax_tm";
            return launch_minmax_tm(a, st);
        }
        case I_PNR: {
            PnrArgs a{};
            a.layout = 1;
            a.x = in.p[0];
            a.n = R;
            a.cols = C;
            a.first_tm = d_first;
            a.length = p;
            a.p_frac = (float)(c.a * 0.01);
            a.n_lanes = C;
            a.out = out[0];
            a.scratch = d_sc;
            ctx->last_kernel = "percentile_tm";
            return launch_percentile(a, st);
        }
        default:
            return fail(VTA_ERR_NOT_IMPLEMENTED, "indicator not implemented");
    }
}

// ------------------------------------------------------------ drivers ------
static vta_status check_ctx(vta_ctx* ctx) {
    if (!ctx) return fail(VTA_ERR_INVALID_INPUT, "null context");
    VTA_CUDA_TRY(cudaSetDevice(ctx->device));
    g_cur = ctx;
    ctx->timed = false;
    // the pinned staging buffer is reused once the copies of the calls that
    // staged through it (device entry points return without waiting) are done
    if (ctx->stage_pending) {
        VTA_CUDA_TRY(cudaEventSynchronize(ctx->stage_ev));
        ctx->stage_pending = false;
    }
    ctx->host_stage_off = 0;
    return VTA_OK;
}

static vta_status sync(vta_ctx* ctx) {
    VTA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return check_async("stream");
}

// Blocks from vta_pinned_alloc are mapped into every device's address space;
// the registry lets the into-host calls recognise an output buffer that lies
// wholly inside one and have the kernels store into it directly.
struct PinnedBlock {
    size_t bytes;
    char* dev;
};
static std::mutex g_pin_mu;
static std::map<uintptr_t, PinnedBlock> g_pin;

float* pinned_device_view(const void* p, size_t bytes) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pin.upper_bound(a);
    if (it == g_pin.begin()) return nullptr;
    --it;
    const uintptr_t off = a - it->first;
    if (off > it->second.bytes || bytes > it->second.bytes - off) return nullptr;
    return reinterpret_cast<float*>(it->second.dev + off);
}

// host inputs -> device outputs (`out_dev` non-null: caller's device buffers;
// `out_host` non-null: copy results into host buffers of out_len floats)
static vta_status batch_host(vta_ctx* ctx, Ind ind, const float* const* hin, size_t len,
                             const std::vector<Combo>& cs, vta_device_array* const* out_arr, float* const* out_host,
                             size_t out_len, size_t* rows, size_t* cols) {
    VTA_TRY(check_ctx(ctx));
    const int nin = kInfo[ind].in, nout = kInfo[ind].n_out;
    if (len == 0) return fail(VTA_ERR_INVALID_INPUT, std::string(kInfo[ind].name) + ": empty data");
    for (int k = 0; k < nin; ++k)
        if (!hin[k]) return fail(VTA_ERR_INVALID_INPUT, "null input pointer");
    const size_t first = host_first(ind, hin, len);
    VTA_TRY(validate_combos(ind, cs, len, first));
    const size_t nc = cs.size();
    if (nc > SIZE_MAX / len) return fail(VTA_ERR_INVALID_INPUT, "rows*cols overflow");
    const size_t out_elems = nc * len;
    if (out_host && out_len < out_elems) return fail(VTA_ERR_INVALID_INPUT, "output buffer too small");
    const size_t in_bytes = len * sizeof(float) * nin;
    const size_t out_bytes = out_elems * sizeof(float);
    // an output buffer from vta_pinned_alloc takes the kernels' stores
    // directly (one pass over the host link instead of a device buffer and a
    // copy); the others go through device buffers and a copy
    float* direct[3] = {nullptr, nullptr, nullptr};
    int n_staged = nout;
    if (out_host && ctx->policy.host_out == 0) {
        n_staged = 0;
        for (int k = 0; k < nout; ++k) {
            direct[k] = pinned_device_view(out_host[k], out_bytes);
            if (!direct[k]) ++n_staged;
        }
    }
    // into-host calls with the cached policy keep one device buffer for the
    // inputs and outputs in the context (grown when too small), so repeated
    // calls do not pay a cudaMalloc / cudaFree of their outputs each time
    const bool cached = out_host && ctx->policy.host_io == 0;
    float* d_in = nullptr;
    float* d_out[3] = {nullptr, nullptr, nullptr};
    std::unique_ptr<void, void (*)(void*)> in_guard(nullptr, [](void* p) { cudaFree(p); });
    if (cached) {
        const size_t in_al = (in_bytes + 255) & ~size_t(255);
        const size_t out_al = (out_bytes + 255) & ~size_t(255);
        const size_t need = in_al + out_al * n_staged;
        if (need > ctx->io_bytes) {
            VTA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
            if (ctx->io) cudaFree(ctx->io);
            ctx->io = nullptr;
            ctx->io_bytes = 0;
            VTA_TRY(vram_check(need));
            VTA_CUDA_TRY(cudaMalloc(&ctx->io, need));
            ctx->io_bytes = need;
        }
        char* base = static_cast<char*>(ctx->io);
        d_in = reinterpret_cast<float*>(base);
        for (int k = 0, j = 0; k < nout; ++k)
            if (!direct[k]) d_out[k] = reinterpret_cast<float*>(base + in_al + out_al * j++);
    } else {
        VTA_TRY(vram_check(out_bytes * n_staged + in_bytes));
        VTA_CUDA_TRY(cudaMalloc((void**)&d_in, in_bytes));
        in_guard.reset(d_in);
        for (int k = 0; k < nout; ++k) {
            if (direct[k]) continue;
            cudaError_t e = cudaMalloc((void**)&d_out[k], out_bytes);
            if (e != cudaSuccess) {
                for (int j = 0; j < k; ++j) cudaFree(d_out[j]);
                return cuda_fail(e, "cudaMalloc(output)");
            }
        }
    }
    float* k_out[3] = {nullptr, nullptr, nullptr};  // where the kernels write
    for (int k = 0; k < nout; ++k) k_out[k] = direct[k] ? direct[k] : d_out[k];
    // inputs -> device
    DevIn din{};
    for (int k = 0; k < nin; ++k) {
        din.p[k] = d_in + (size_t)k * len;
        VTA_TRY(upload(ctx, d_in + (size_t)k * len, hin[k], len * sizeof(float)));
    }
    vta_status s = run_batch(ctx, ind, din, len, first, cs, k_out);
    if (s == VTA_OK && out_host) {
        for (int k = 0; k < nout && s == VTA_OK; ++k) {
            if (direct[k]) continue;
            cudaError_t e = cudaMemcpyAsync(out_host[k], d_out[k], out_elems * sizeof(float),
                                            cudaMemcpyDeviceToHost, ctx->stream);
            if (e != cudaSuccess) s = cuda_fail(e, "cudaMemcpyAsync(D2H)");
        }
    }
    if (s == VTA_OK) s = sync(ctx);
    cudaStreamSynchronize(ctx->stream);
    if (s != VTA_OK || out_host) {
        if (!cached)
            for (int k = 0; k < nout; ++k)
                if (d_out[k]) cudaFree(d_out[k]);
        if (s != VTA_OK) return s;
    } else {
        for (int k = 0; k < nout; ++k) *out_arr[k] = vta_device_array{d_out[k], nc, len, ctx->device};
    }
    if (rows) *rows = nc;
    if (cols) *cols = len;
    return VTA_OK;
}

static vta_status batch_device(vta_ctx* ctx, Ind ind, const float* const* din_p, size_t len, size_t first,
                               const std::vector<Combo>& cs, float* const* d_out) {
    VTA_TRY(check_ctx(ctx));
    const int nin = kInfo[ind].in, nout = kInfo[ind].n_out;
    if (len == 0) return fail(VTA_ERR_INVALID_INPUT, std::string(kInfo[ind].name) + ": empty data");
    for (int k = 0; k < nin; ++k)
        if (!din_p[k]) return fail(VTA_ERR_INVALID_INPUT, "null input pointer");
    for (int k = 0; k < nout; ++k)
        if (!d_out[k]) return fail(VTA_ERR_INVALID_INPUT, "null output pointer");
    VTA_TRY(validate_combos(ind, cs, len, first));
    DevIn din{};
    for (int k = 0; k < nin; ++k) din.p[k] = din_p[k];
    VTA_TRY(run_batch(ctx, ind, din, len, first, cs, d_out));
    // stream-ordered, not waited for (the crate's x_batch_device returns
    // after the launch too); vta_ctx_synchronize waits
    return check_async("batch_device");
}

static vta_status tm_validate_host(Ind ind, const float* const* hin, size_t cols, size_t rows, const Combo& c) {
    VTA_TRY(validate_combo(ind, c, rows));
    for (size_t s = 0; s < cols; ++s) {
        const size_t f = host_first(ind, hin, rows, cols, s);
        char buf[160];
        if (f >= rows) {
            std::snprintf(buf, sizeof buf, "%s: series %zu all NaN", kInfo[ind].name, s);
            return fail(VTA_ERR_INVALID_INPUT, buf);
        }
        const size_t need = needed_len(ind, c.period, c.a);
        if (rows - f < need) {
            std::snprintf(buf, sizeof buf, "%s: series %zu not enough valid data (needed >= %zu, valid = %zu)",
                          kInfo[ind].name, s, need, rows - f);
            return fail(VTA_ERR_INVALID_INPUT, buf);
        }
    }
    return VTA_OK;
}

static vta_status tm_host(vta_ctx* ctx, Ind ind, const float* const* hin, size_t cols, size_t rows, const Combo& c,
                          vta_device_array* const* out_arr) {
    VTA_TRY(check_ctx(ctx));
    const int nin = kInfo[ind].in, nout = kInfo[ind].n_out;
    if (cols == 0 || rows == 0) return fail(VTA_ERR_INVALID_INPUT, "empty matrix");
    if (cols > SIZE_MAX / rows) return fail(VTA_ERR_INVALID_INPUT, "rows*cols overflow");
    for (int k = 0; k < nin; ++k)
        if (!hin[k]) return fail(VTA_ERR_INVALID_INPUT, "null input pointer");
    VTA_TRY(tm_validate_host(ind, hin, cols, rows, c));
    const size_t elems = cols * rows;
    VTA_TRY(vram_check(elems * sizeof(float) * (nin + nout)));
    float* d_in = nullptr;
    VTA_CUDA_TRY(cudaMalloc((void**)&d_in, elems * sizeof(float) * nin));
    std::unique_ptr<void, void (*)(void*)> in_guard(d_in, [](void* p) { cudaFree(p); });
    DevIn din{};
    for (int k = 0; k < nin; ++k) {
        din.p[k] = d_in + (size_t)k * elems;
        VTA_TRY(upload(ctx, d_in + (size_t)k * elems, hin[k], elems * sizeof(float)));
    }
    float* d_out[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < nout; ++k) {
        cudaError_t e = cudaMalloc((void**)&d_out[k], elems * sizeof(float));
        if (e != cudaSuccess) {
            for (int j = 0; j < k; ++j) cudaFree(d_out[j]);
            return cuda_fail(e, "cudaMalloc(output)");
        }
    }
    vta_status s = run_tm(ctx, ind, din, cols, rows, c, d_out);
    if (s == VTA_OK) s = sync(ctx);
    cudaStreamSynchronize(ctx->stream);
    if (s != VTA_OK) {
        for (int k = 0; k < nout; ++k) cudaFree(d_out[k]);
        return s;
    }
    for (int k = 0; k < nout; ++k) *out_arr[k] = vta_device_array{d_out[k], rows, cols, ctx->device};
    return VTA_OK;
}

static vta_status tm_device(vta_ctx* ctx, Ind ind, const float* const* din_p, size_t cols, size_t rows,
                            const Combo& c, float* const* d_out) {
    VTA_TRY(check_ctx(ctx));
    const int nin = kInfo[ind].in, nout = kInfo[ind].n_out;
    if (cols == 0 || rows == 0) return fail(VTA_ERR_INVALID_INPUT, "empty matrix");
    for (int k = 0; k < nin; ++k)
        if (!din_p[k]) return fail(VTA_ERR_INVALID_INPUT, "null input pointer");
    for (int k = 0; k < nout; ++k)
        if (!d_out[k]) return fail(VTA_ERR_INVALID_INPUT, "null output pointer");
    VTA_TRY(validate_combo(ind, c, rows));
    DevIn din{};
    for (int k = 0; k < nin; ++k) din.p[k] = din_p[k];
    VTA_TRY(run_tm(ctx, ind, din, cols, rows, c, d_out));
    return check_async("many_series_device");  // stream-ordered, like batch_device
}

// ------------------------------------------------------------ grids --------
static std::vector<Combo> grid_period(Ind ind, const vta_period_batch_range* r) {
    std::vector<Combo> cs;
    for (size_t p : axis_usize(r->period, kInfo[ind].axis)) cs.push_back({p, 0.0, 0.0});
    return cs;
}
// (each axis is expanded once, outside the loops: a grid of 17,920 ALMA
// combos took 0.7 ms of host time per call when the inner axes were rebuilt
// per outer value)
static std::vector<Combo> grid_alma(const vta_alma_batch_range* r) {
    const std::vector<size_t> ps = axis_usize(r->period, AX_DESC);
    const std::vector<double> os = axis_f64(r->offset), ss = axis_f64(r->sigma);
    std::vector<Combo> cs;
    cs.reserve(ps.size() * os.size() * ss.size());
    for (size_t p : ps)
        for (double o : os)
            for (double s : ss) cs.push_back({p, o, s});
    return cs;
}
static std::vector<Combo> grid_p1(Ind ind, vta_range_usize pr, vta_range_f64 ar_) {
    const std::vector<size_t> ps = axis_usize(pr, kInfo[ind].axis);
    const std::vector<double> as = axis_f64(ar_);
    std::vector<Combo> cs;
    cs.reserve(ps.size() * as.size());
    for (size_t p : ps)
        for (double a : as) cs.push_back({p, a, 0.0});
    return cs;
}
static std::vector<Combo> grid_bb(const vta_bollinger_batch_range* r) {
    const std::vector<size_t> ps = axis_usize(r->period, AX_DESC);
    const std::vector<double> us = axis_f64(r->devup), ds = axis_f64(r->devdn);
    std::vector<Combo> cs;
    cs.reserve(ps.size() * us.size() * ds.size());
    for (size_t p : ps)
        for (double u : us)
            for (double d : ds) cs.push_back({p, u, d});
    return cs;
}

static std::vector<Combo> grid_of(Ind, const vta_alma_batch_range* r) { return grid_alma(r); }
static std::vector<Combo> grid_of(Ind ind, const vta_period_batch_range* r) { return grid_period(ind, r); }
static std::vector<Combo> grid_of(Ind ind, const vta_stddev_batch_range* r) { return grid_p1(ind, r->period, r->nbdev); }
static std::vector<Combo> grid_of(Ind ind, const vta_zscore_batch_range* r) { return grid_p1(ind, r->period, r->nbdev); }
static std::vector<Combo> grid_of(Ind, const vta_bollinger_batch_range* r) { return grid_bb(r); }
static std::vector<Combo> grid_of(Ind ind, const vta_supertrend_batch_range* r) { return grid_p1(ind, r->period, r->factor); }
static std::vector<Combo> grid_of(Ind ind, const vta_percentile_batch_range* r) { return grid_p1(ind, r->length, r->percentage); }
// EpmaBatchRange: period outer, offset inner, both axes ascending after a swap
// (epma.rs:835-859)
static std::vector<Combo> grid_of(Ind ind, const vta_vpwma_batch_range* r) { return grid_p1(ind, r->period, r->power); }
static std::vector<Combo> grid_of(Ind, const vta_epma_batch_range* r) {
    const std::vector<size_t> ps = axis_usize(r->period, AX_SWAP), os = axis_usize(r->offset, AX_SWAP);
    std::vector<Combo> cs;
    cs.reserve(ps.size() * os.size());
    for (size_t p : ps)
        for (size_t o : os) cs.push_back({p, (double)o, 0.0});
    return cs;
}

static Combo combo_of(const vta_alma_params* p) { return {p->period, p->offset, p->sigma}; }
static Combo combo_of(const vta_period_params* p) { return {p->period, 0.0, 0.0}; }
static Combo combo_of(const vta_stddev_params* p) { return {p->period, p->nbdev, 0.0}; }
static Combo combo_of(const vta_zscore_params* p) { return {p->period, p->nbdev, 0.0}; }
static Combo combo_of(const vta_bollinger_params* p) { return {p->period, p->devup, p->devdn}; }
static Combo combo_of(const vta_supertrend_params* p) { return {p->period, p->factor, 0.0}; }
static Combo combo_of(const vta_percentile_params* p) { return {p->length, p->percentage, 0.0}; }
static Combo combo_of(const vta_epma_params* p) { return {p->period, (double)p->offset, 0.0}; }
static Combo combo_of(const vta_vpwma_params* p) { return {p->period, p->power, 0.0}; }

static void params_of(const Combo& c, vta_alma_params* p) { *p = {c.period, c.a, c.b}; }
static void params_of(const Combo& c, vta_period_params* p) { *p = {c.period}; }
static void params_of(const Combo& c, vta_stddev_params* p) { *p = {c.period, c.a}; }
static void params_of(const Combo& c, vta_zscore_params* p) { *p = {c.period, c.a}; }
static void params_of(const Combo& c, vta_bollinger_params* p) { *p = {c.period, c.a, c.b}; }
static void params_of(const Combo& c, vta_supertrend_params* p) { *p = {c.period, c.a}; }
static void params_of(const Combo& c, vta_percentile_params* p) { *p = {c.period, c.a}; }
static void params_of(const Combo& c, vta_epma_params* p) { *p = {c.period, (size_t)c.a}; }
static void params_of(const Combo& c, vta_vpwma_params* p) { *p = {c.period, c.a}; }

template <class R, class P>
static vta_status expand(Ind ind, const R* r, P* out, size_t cap, size_t* n) {
    if (!r) return fail(VTA_ERR_INVALID_INPUT, "null sweep");
    std::vector<Combo> cs = grid_of(ind, r);
    if (n) *n = cs.size();
    if (out)
        for (size_t i = 0; i < cs.size() && i < cap; ++i) params_of(cs[i], &out[i]);
    return cs.empty() ? fail(VTA_ERR_INVALID_INPUT, "empty range") : VTA_OK;
}

// ---- MA computer over a device-resident series (VramMaComputer) ----------
// The crate's VramMaComputer (vram_ma.rs:87-160) dispatches an MA name and an
// arbitrary period list to the batch kernels (compute_period_ma_into,
// vram_ma.rs:574; time-major output: compute_period_ma_tm_into, :2153).
static int ma_ind(const char* name) {
    if (!name) return -1;
    std::string s(name);
    while (!s.empty() && std::isspace((unsigned char)s.back())) s.pop_back();
    size_t b = 0;
    while (b < s.size() && std::isspace((unsigned char)s[b])) ++b;
    s = s.substr(b);
    for (char& ch : s) ch = (char)std::tolower((unsigned char)ch);
    static const struct { const char* n; Ind i; } kMa[] = {
        {"sma", I_SMA},     {"ema", I_EMA},       {"wma", I_WMA},     {"alma", I_ALMA},   {"dema", I_DEMA},
        {"tema", I_TEMA},   {"swma", I_SWMA},     {"trima", I_TRIMA}, {"sinwma", I_SINWMA}, {"epma", I_EPMA},
        {"wilders", I_WILDERS}, {"cwma", I_CWMA}, {"fwma", I_FWMA},   {"pwma", I_PWMA},   {"srwma", I_SRWMA},
        {"sqwma", I_SQWMA}, {"vpwma", I_VPWMA},
    };
    for (const auto& m : kMa)
        if (s == m.n) return m.i;
    // names the crate's computer also serves (supports_vram_kernel_ma,
    // vram_ma.rs:68-76) whose kernels are not part of this library
    static const char* kOther[] = {"jsa", "smma", "highpass", "maaq", "mwdx", "supersmoother",
                                   "supersmoother_3_pole", "zlema", "nma", "hma", "jma", "edcf",
                                   "ehlers_itrend", "cora_wave", "vwma", "frama"};
    for (const char* o : kOther)
        if (s == o) return -2;
    return -1;
}

static double ma_param(const char* const* keys, const double* vals, size_t n, const char* key, double dflt) {
    for (size_t i = 0; i < n; ++i)
        if (keys && keys[i] && vals && std::strcmp(keys[i], key) == 0 && std::isfinite(vals[i])) return vals[i];
    return dflt;  // vram_ma.rs:521-523: missing or non-finite -> default
}

static vta_status ma_periods_device(vta_ctx* ctx, const char* ma_type, const char* const* keys, const double* vals,
                                    size_t n_params, const float* d_prices, size_t len, size_t first_valid,
                                    const int* periods, size_t n_periods, int time_major, float* d_out) {
    VTA_TRY(check_ctx(ctx));
    const int mi = ma_ind(ma_type);
    if (mi == -2) return fail(VTA_ERR_NOT_IMPLEMENTED, std::string("ma computer: no kernel for ") + ma_type);
    if (mi < 0) return fail(VTA_ERR_INVALID_INPUT, std::string("ma computer: unknown ma_type ") +
                                                       (ma_type ? ma_type : "(null)"));
    const Ind ind = (Ind)mi;
    if (!d_prices || !d_out) return fail(VTA_ERR_INVALID_INPUT, "ma computer: null device pointer");
    if (!periods || n_periods == 0) return fail(VTA_ERR_INVALID_INPUT, "ma computer: empty period list");
    if (len == 0) return fail(VTA_ERR_INVALID_INPUT, "ma computer: empty series");
    if (len > (size_t)INT32_MAX) return fail(VTA_ERR_INVALID_INPUT, "series longer than 2^31-1");
    const double offset = ma_param(keys, vals, n_params, "offset", ind == I_ALMA ? 0.85 : 0.0);
    const double sigma = ma_param(keys, vals, n_params, "sigma", 6.0);
    const double power = ma_param(keys, vals, n_params, "power", 0.382);
    std::vector<Combo> cs;
    cs.reserve(n_periods);
    for (size_t i = 0; i < n_periods; ++i) {
        if (periods[i] <= 0) return fail(VTA_ERR_INVALID_INPUT, "ma computer: periods must be > 0");
        const size_t p = (size_t)periods[i];
        if (ind == I_ALMA) cs.push_back({p, offset, sigma});
        else if (ind == I_EPMA) cs.push_back({p, std::max(0.0, std::round(offset)), 0.0});
        else if (ind == I_VPWMA) cs.push_back({p, power, 0.0});
        else cs.push_back({p, 0.0, 0.0});
    }
    VTA_TRY(validate_combos(ind, cs, len, first_valid));
    DevIn din{};
    din.p[0] = d_prices;
    if (!time_major) {
        float* outs[1] = {d_out};
        VTA_TRY(run_batch(ctx, ind, din, len, first_valid, cs, outs));
        return sync(ctx);
    }
    // rows are produced row-major into the context's staging buffer, then
    // transposed into d_out[t][combo]
    const size_t bytes = n_periods * len * sizeof(float);
    if (bytes > ctx->tmp_bytes) {
        VTA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        if (ctx->tmp) cudaFree(ctx->tmp);
        ctx->tmp = nullptr;
        ctx->tmp_bytes = 0;
        VTA_TRY(vram_check(bytes));
        VTA_CUDA_TRY(cudaMalloc(&ctx->tmp, bytes));
        ctx->tmp_bytes = bytes;
    }
    float* rowmajor = static_cast<float*>(ctx->tmp);
    float* outs[1] = {rowmajor};
    VTA_TRY(run_batch(ctx, ind, din, len, first_valid, cs, outs));
    VTA_TRY(launch_transpose(rowmajor, (int)n_periods, (int)len, d_out, ctx->stream));
    return sync(ctx);
}

// The crate's CudaMaSelector (ma_selector.rs:194-1820): the same by-name
// dispatch from host prices, one period (ma_to_device, :935) or a period
// range (ma_sweep_to_device, :1712; its own range rule, :1037-1061).
static std::vector<size_t> selector_periods(size_t start, size_t end, size_t step) {
    std::vector<size_t> v;
    if (step == 0 || start == end) return {start};
    if (start < end) {
        for (size_t x = start; x <= end; x += step) {
            v.push_back(x);
            if (x > SIZE_MAX - step) break;
        }
        return v;
    }
    size_t cur = start;
    while (cur >= end) {
        v.push_back(cur);
        if (cur == 0) break;
        const size_t next = cur >= step ? cur - step : 0;
        if (next == cur) break;
        cur = next;
        if (cur < end) break;
    }
    return v;
}

static vta_status ma_select(vta_ctx* ctx, const char* ma_type, const char* const* keys, const double* vals,
                            size_t n_params, const float* prices, size_t len, size_t start, size_t end, size_t step,
                            vta_device_array* out_arr, float* out_host, size_t out_len, size_t* rows, size_t* cols) {
    const int mi = ma_ind(ma_type);
    if (mi == -2) return fail(VTA_ERR_NOT_IMPLEMENTED, std::string("ma selector: no kernel for ") + ma_type);
    if (mi < 0) return fail(VTA_ERR_INVALID_INPUT, std::string("ma selector: unknown ma_type ") +
                                                       (ma_type ? ma_type : "(null)"));
    const Ind ind = (Ind)mi;
    if (len == 0) return fail(VTA_ERR_INVALID_INPUT, "ma selector: empty price input");
    const double offset = ma_param(keys, vals, n_params, "offset", ind == I_ALMA ? 0.85 : 0.0);
    const double sigma = ma_param(keys, vals, n_params, "sigma", 6.0);
    const double power = ma_param(keys, vals, n_params, "power", 0.382);
    std::vector<Combo> cs;
    for (size_t p : selector_periods(start, end, step)) {
        if (p == 0 || p > len) {
            char buf[120];
            std::snprintf(buf, sizeof buf, "ma selector: invalid period: %zu for length %zu", p, len);
            return fail(VTA_ERR_INVALID_INPUT, buf);
        }
        if (ind == I_ALMA) cs.push_back({p, offset, sigma});
        else if (ind == I_EPMA) cs.push_back({p, std::max(0.0, std::round(offset)), 0.0});
        else if (ind == I_VPWMA) cs.push_back({p, power, 0.0});
        else cs.push_back({p, 0.0, 0.0});
    }
    const float* in[1] = {prices};
    vta_device_array* oa[1] = {out_arr};
    float* oh[1] = {out_host};
    return batch_host(ctx, ind, in, len, cs, out_arr ? oa : nullptr, out_host ? oh : nullptr, out_len, rows, cols);
}

// ---- hooks for the request server (vta_server.cu) -------------------------
int ind_by_name(const char* name) {
    if (!name) return -1;
    for (int i = 0; i < (int)(sizeof(kInfo) / sizeof(kInfo[0])); ++i)
        if (std::strcmp(kInfo[i].name, name) == 0) return i;
    return -1;
}
int ind_inputs(int ind) { return kInfo[ind].in; }
int ind_outputs(int ind) { return kInfo[ind].n_out; }
// Device time per output relative to an HBM-bound sweep (EMA, SMA, ALMA):
// the sequential high/low/close recurrences and the percentile window run
// well below the write bandwidth (measured bench figures, rounded).
double ind_cost(int ind) {
    switch (ind) {
        case I_ADX: return 12.0;
        case I_SUPERTREND: return 8.0;
        case I_PNR: return 10.0;
        case I_ATR: return 2.0;
        default: return 1.0;
    }
}

// first valid index from the per-field firsts of a stored series, as
// host_first defines it per indicator
size_t ind_first(int ind, size_t fh, size_t fl, size_t fc, size_t fall) {
    if (kInfo[ind].in == IN_X) return fc;
    if (ind == I_DONCHIAN) return std::max(fh, fl);
    if (ind == I_ADX) return std::max(fh, std::max(fl, fc));
    return fall;
}

static std::vector<Combo> grid_generic(Ind ind, const vta_sweep* sw) {
    switch (ind) {
        case I_ALMA: { const vta_alma_batch_range r{sw->period, sw->p1, sw->p2}; return grid_of(ind, &r); }
        case I_STDDEV: { const vta_stddev_batch_range r{sw->period, sw->p1}; return grid_of(ind, &r); }
        case I_ZSCORE: { const vta_zscore_batch_range r{sw->period, sw->p1}; return grid_of(ind, &r); }
        case I_BB: { const vta_bollinger_batch_range r{sw->period, sw->p1, sw->p2}; return grid_of(ind, &r); }
        case I_SUPERTREND: { const vta_supertrend_batch_range r{sw->period, sw->p1}; return grid_of(ind, &r); }
        case I_PNR: { const vta_percentile_batch_range r{sw->period, sw->p1}; return grid_of(ind, &r); }
        case I_VPWMA: { const vta_vpwma_batch_range r{sw->period, sw->p1}; return grid_of(ind, &r); }
        case I_EPMA: {  // offsets from p1 (rounded to integers)
            const vta_range_usize o{(size_t)std::llround(sw->p1.start), (size_t)std::llround(sw->p1.end),
                                    (size_t)std::llround(sw->p1.step)};
            const vta_epma_batch_range r{sw->period, o};
            return grid_of(ind, &r);
        }
        default: { const vta_period_batch_range r{sw->period}; return grid_of(ind, &r); }
    }
}

vta_status batch_check(int ind, const vta_sweep* sw, size_t len, size_t first, size_t* rows) {
    const std::vector<Combo> cs = grid_generic((Ind)ind, sw);
    VTA_TRY(validate_combos((Ind)ind, cs, len, first));
    if (cs.size() > SIZE_MAX / len) return fail(VTA_ERR_INVALID_INPUT, "rows*cols overflow");
    *rows = cs.size();
    return VTA_OK;
}

vta_status batch_enqueue(vta_ctx* ctx, int ind, const float* const* d_in, size_t len, size_t first,
                         const vta_sweep* sw, float* const* d_out) {
    VTA_CUDA_TRY(cudaSetDevice(ctx->device));
    ctx->host_stage_off = 0;  // the slot's previous request has completed
    const std::vector<Combo> cs = grid_generic((Ind)ind, sw);
    VTA_TRY(validate_combos((Ind)ind, cs, len, first));
    DevIn din{};
    for (int k = 0; k < kInfo[ind].in; ++k) din.p[k] = d_in[k];
    return run_batch(ctx, (Ind)ind, din, len, first, cs, d_out);
}

// ---- hooks for the no-allocation SMA entry point (vta_noalloc.cu) --------
vta_status enter_call(vta_ctx* ctx) { return check_ctx(ctx); }

// Number of periods of an SMA sweep, counted the way axis_usize expands it
// (SMA's descending ranges run start, start - step, ... while >= end), so the
// caller can reject an oversized sweep before expanding it.
size_t sma_period_count(vta_range_usize r) {
    if (r.step == 0 || r.start == r.end) return 1;
    if (r.start < r.end) return (r.end - r.start) / r.step + 1;
    return (r.start - r.end) / r.step + 1;  // kInfo[I_SMA].axis is AX_DESC
}

// Period k of an SMA sweep (k < sma_period_count(r)): the same values as
// axis_usize(r, SMA's mode), without building a vector.
size_t sma_period_at(vta_range_usize r, size_t k) {
    if (r.step == 0 || r.start == r.end) return r.start;
    return r.start < r.end ? r.start + k * r.step : r.start - k * r.step;
}

// The checks of validate_combos for the n periods of an SMA sweep.
vta_status validate_sma_range(vta_range_usize r, size_t n, size_t len, size_t first) {
    if (n == 0) return fail(VTA_ERR_INVALID_INPUT, "sma: no parameter combinations");
    size_t need = 0;
    for (size_t i = 0; i < n; ++i) {
        const size_t p = sma_period_at(r, i);
        VTA_TRY(validate_combo(I_SMA, Combo{p, 0.0, 0.0}, len));
        need = std::max(need, needed_len(I_SMA, p));
    }
    if (first >= len) return fail(VTA_ERR_INVALID_INPUT, "sma: all values are NaN");
    if (len - first < need) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "sma: not enough valid data (needed >= %zu, valid = %zu)", need, len - first);
        return fail(VTA_ERR_INVALID_INPUT, buf);
    }
    return VTA_OK;
}

}  // namespace vta

using namespace vta;

// ============================================================ C ABI ========
extern "C" {

const char* vta_last_error(void) { return g_err.c_str(); }

vta_status vta_last_error_oom(size_t* required, size_t* free_bytes, size_t* headroom) {
    const bool oom = g_err_status == VTA_ERR_OUT_OF_MEMORY;
    if (required) *required = oom ? g_oom[0] : 0;
    if (free_bytes) *free_bytes = oom ? g_oom[1] : 0;
    if (headroom) *headroom = oom ? g_oom[2] : 0;
    return oom ? VTA_OK : VTA_ERR_INVALID_INPUT;
}
const char* vta_version(void) { return "vta_gb300 0.1.0 (sm_103a)"; }

int vta_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

vta_status vta_ctx_create(int device_id, vta_ctx** out) {
    if (!out) return fail(VTA_ERR_INVALID_INPUT, "null out");
    *out = nullptr;
    int n = 0;
    VTA_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device_id < 0 || device_id >= n) return fail(VTA_ERR_INVALID_INPUT, "device id out of range");
    VTA_CUDA_TRY(cudaSetDevice(device_id));
    auto* c = new vta_ctx();
    c->device = device_id;
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device_id) == cudaSuccess) {
        c->num_sms = prop.multiProcessorCount;
        c->smem_optin = prop.sharedMemPerBlockOptin;
        if (prop.major != 10 || prop.minor != 3) {
            // the kernels are built for sm_103a only
            char buf[128];
            std::snprintf(buf, sizeof buf, "device %d is sm_%d%d; this library is built for sm_103a", device_id,
                          prop.major, prop.minor);
            delete c;
            return fail(VTA_ERR_MISSING_KERNEL_SYMBOL, buf);
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaStreamCreate");
    }
    if (cudaHostAlloc(&c->host_stage, size_t(1) << 20, cudaHostAllocDefault) == cudaSuccess) {
        c->host_stage_bytes = size_t(1) << 20;
    } else {
        c->host_stage = nullptr;  // uploads fall back to pageable copies
        cudaGetLastError();
    }
    const char* pol = std::getenv("VTA_WMA_BATCH");
    if (pol) vta_ctx_set_policy(c, "wma_batch", pol);
    *out = c;
    return VTA_OK;
}

vta_status vta_ctx_destroy(vta_ctx* ctx) {
    if (!ctx) return VTA_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->scratch) ctx->async_alloc ? (void)cudaFreeAsync(ctx->scratch, ctx->stream) : (void)cudaFree(ctx->scratch);
    if (ctx->aux) ctx->async_alloc ? (void)cudaFreeAsync(ctx->aux, ctx->stream) : (void)cudaFree(ctx->aux);
    if (ctx->io) cudaFree(ctx->io);
    if (ctx->tmp) cudaFree(ctx->tmp);
    if (ctx->cc_dev) cudaFree(ctx->cc_dev);
    for (auto& e : ctx->rw) cudaFree(e.dev);
    if (ctx->async_alloc) cudaStreamSynchronize(ctx->stream);
    if (ctx->err_host) cudaFreeHost(ctx->err_host);
    if (ctx->host_stage) cudaFreeHost(ctx->host_stage);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stage_ev) cudaEventDestroy(ctx->stage_ev);
    if (g_cur == ctx) g_cur = nullptr;
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return VTA_OK;
}

vta_status vta_ctx_synchronize(vta_ctx* ctx) {
    // not a compute call: the last call's timing stays readable
    if (!ctx) return fail(VTA_ERR_INVALID_INPUT, "null context");
    VTA_CUDA_TRY(cudaSetDevice(ctx->device));
    VTA_TRY(sync(ctx));
    ctx->stage_pending = false;
    return VTA_OK;
}

vta_status vta_ctx_set_stream(vta_ctx* ctx, void* stream) {
    VTA_TRY(check_ctx(ctx));
    // work already queued on the old stream (device entry points do not wait)
    // finishes before the context's buffers are used from another stream
    if (ctx->stream) VTA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (stream) {
        if (ctx->own_stream && ctx->stream) {
            cudaStreamSynchronize(ctx->stream);
            cudaStreamDestroy(ctx->stream);
        }
        ctx->stream = (cudaStream_t)stream;
        ctx->own_stream = false;
    } else if (!ctx->own_stream) {
        VTA_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return VTA_OK;
}

void* vta_ctx_get_stream(vta_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

vta_status vta_ctx_set_policy(vta_ctx* ctx, const char* key, const char* value) {
    if (!ctx || !key || !value) return fail(VTA_ERR_INVALID_POLICY, "null policy argument");
    const std::string k(key), v(value);
    if (k == "wma_batch") {
        if (v == "auto") ctx->policy.wma_batch = 0;
        else if (v == "plain") ctx->policy.wma_batch = 1;
        else if (v == "tc_fp16x3") ctx->policy.wma_batch = 2;
        else if (v == "tc_bf16x3") ctx->policy.wma_batch = 3;
        else return fail(VTA_ERR_INVALID_POLICY, "wma_batch: auto|plain|tc_fp16x3|tc_bf16x3");
        return VTA_OK;
    }
    if (k == "timing") {
        if (v == "on") {
            if (!ctx->ev0) {
                VTA_CUDA_TRY(cudaSetDevice(ctx->device));
                VTA_CUDA_TRY(cudaEventCreate(&ctx->ev0));
                VTA_CUDA_TRY(cudaEventCreate(&ctx->ev1));
            }
            ctx->timing = true;
        } else if (v == "off") {
            ctx->timing = false;
        } else {
            return fail(VTA_ERR_INVALID_POLICY, "timing: on|off");
        }
        return VTA_OK;
    }
    if (k == "recur_chunk") {
        if (v == "auto") ctx->policy.recur_chunk = 0;
        else if (v == "sequential") ctx->policy.recur_chunk = 1;
        else {
            char* end = nullptr;
            long x = std::strtol(v.c_str(), &end, 10);
            if (!end || *end || x < 32 || x % 32) return fail(VTA_ERR_INVALID_POLICY, "recur_chunk: multiple of 32");
            ctx->policy.recur_chunk = (int)x;
        }
        return VTA_OK;
    }
    if (k == "host_io") {
        if (v == "cached") {
            ctx->policy.host_io = 0;
        } else if (v == "per_call") {
            ctx->policy.host_io = 1;
            if (ctx->io) {
                VTA_CUDA_TRY(cudaSetDevice(ctx->device));
                VTA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
                cudaFree(ctx->io);
                ctx->io = nullptr;
                ctx->io_bytes = 0;
            }
        } else {
            return fail(VTA_ERR_INVALID_POLICY, "host_io: cached|per_call");
        }
        return VTA_OK;
    }
    if (k == "host_out") {
        // *_batch_into_host_f32 outputs in vta_pinned_alloc buffers: "direct"
        // (the kernels store into them) or "copy" (device buffer + copy)
        if (v == "direct") ctx->policy.host_out = 0;
        else if (v == "copy") ctx->policy.host_out = 1;
        else return fail(VTA_ERR_INVALID_POLICY, "host_out: direct|copy");
        return VTA_OK;
    }
    if (k == "recur_agg") {
        if (v == "auto") ctx->policy.recur_agg = 0;
        else if (v == "cuda") ctx->policy.recur_agg = 1;
        else if (v == "tc") ctx->policy.recur_agg = 2;
        else return fail(VTA_ERR_INVALID_POLICY, "recur_agg: auto|cuda|tc");
        return VTA_OK;
    }
    if (k == "tune") {
        if (v == "on") ctx->policy.tune = 0;
        else if (v == "off") ctx->policy.tune = 1;
        else if (v == "cached") ctx->policy.tune = 2;
        else return fail(VTA_ERR_INVALID_POLICY, "tune: on|off|cached");
        return VTA_OK;
    }
    if (k == "scan_chunk") {
        // chunk length of the exact ADX scan: "auto" or a multiple of 32 of
        // at least 1,024 steps
        if (v == "auto") {
            ctx->policy.scan_chunk = 0;
            return VTA_OK;
        }
        char* end = nullptr;
        long x = std::strtol(v.c_str(), &end, 10);
        if (!end || *end || x < kAdxScanMinL || x > (1L << 24) || x % 32)
            return fail(VTA_ERR_INVALID_POLICY, "scan_chunk: auto | multiple of 32 >= 1024");
        ctx->policy.scan_chunk = (int)x;
        return VTA_OK;
    }
    if (k == "tm_chunk" || k == "tm_warm") {
        // many-series plans: time-chunk length ("sequential" = one chunk per
        // series) and warm-restart steps; "auto" = timed / derived
        int& dst = k == "tm_chunk" ? ctx->policy.tm_chunk : ctx->policy.tm_warm;
        if (v == "auto") dst = 0;
        else if (k == "tm_chunk" && v == "sequential") dst = -1;
        else {
            char* end = nullptr;
            long x = std::strtol(v.c_str(), &end, 10);
            if (!end || *end || x < 1 || x > (1L << 30)) return fail(VTA_ERR_INVALID_POLICY, (k + ": positive integer").c_str());
            dst = (int)x;
        }
        return VTA_OK;
    }
    return fail(VTA_ERR_INVALID_POLICY, "unknown policy key");
}

const char* vta_ctx_last_kernel(vta_ctx* ctx) { return ctx ? ctx->last_kernel.c_str() : ""; }

float vta_ctx_kernel_ms(vta_ctx* ctx) {
    if (!ctx || !ctx->timing || !ctx->timed) return -1.f;
    float ms = -1.f;
    if (cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) != cudaSuccess) {
        cudaGetLastError();
        return -1.f;
    }
    return ms;
}

uint64_t vta_launch_count(void) { return g_launches.load(); }
size_t vta_ctx_scratch_bytes(vta_ctx* ctx) { return ctx ? ctx->scratch_bytes : 0; }

vta_status vta_device_array_free(vta_device_array* a) {
    if (!a || !a->ptr) return VTA_OK;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(a->device);
    cudaError_t e = cudaFree(a->ptr);
    cudaSetDevice(cur);
    a->ptr = nullptr;
    a->rows = a->cols = 0;
    if (e != cudaSuccess) return cuda_fail(e, "cudaFree");
    return VTA_OK;
}

vta_status vta_device_array_copy_to_host(vta_ctx* ctx, const vta_device_array* a, float* host, size_t n) {
    VTA_TRY(check_ctx(ctx));
    if (!a || !host) return fail(VTA_ERR_INVALID_INPUT, "null argument");
    if (a->device != ctx->device) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "device mismatch: buf=%d current=%d", a->device, ctx->device);
        return fail(VTA_ERR_DEVICE_MISMATCH, buf);
    }
    if (n < a->rows * a->cols) return fail(VTA_ERR_INVALID_INPUT, "host buffer too small");
    VTA_CUDA_TRY(cudaMemcpyAsync(host, a->ptr, a->rows * a->cols * sizeof(float), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    return sync(ctx);
}

vta_status vta_pinned_alloc(size_t bytes, void** out) {
    if (!out) return fail(VTA_ERR_INVALID_INPUT, "null out");
    *out = nullptr;
    VTA_CUDA_TRY(cudaHostAlloc(out, bytes, cudaHostAllocMapped | cudaHostAllocPortable));
    void* dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, *out, 0) != cudaSuccess) {
        cudaGetLastError();
        dev = nullptr;  // copies only
    }
    if (dev) {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        g_pin[reinterpret_cast<uintptr_t>(*out)] = PinnedBlock{bytes, static_cast<char*>(dev)};
    }
    return VTA_OK;
}
vta_status vta_pinned_free(void* p) {
    if (!p) return VTA_OK;
    {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        g_pin.erase(reinterpret_cast<uintptr_t>(p));
    }
    VTA_CUDA_TRY(cudaFreeHost(p));
    return VTA_OK;
}
vta_status vta_device_alloc(vta_ctx* ctx, size_t bytes, void** out) {
    VTA_TRY(check_ctx(ctx));
    if (!out) return fail(VTA_ERR_INVALID_INPUT, "null out");
    VTA_TRY(vram_check(bytes));
    VTA_CUDA_TRY(cudaMalloc(out, bytes));
    return VTA_OK;
}
vta_status vta_device_free(vta_ctx* ctx, void* p) {
    VTA_TRY(check_ctx(ctx));
    if (p) VTA_CUDA_TRY(cudaFree(p));
    return VTA_OK;
}
vta_status vta_memcpy_h2d(vta_ctx* ctx, void* dst, const void* src, size_t bytes) {
    VTA_TRY(check_ctx(ctx));
    VTA_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return sync(ctx);
}
vta_status vta_memcpy_d2h(vta_ctx* ctx, void* dst, const void* src, size_t bytes) {
    VTA_TRY(check_ctx(ctx));
    VTA_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return sync(ctx);
}

// ---------------------------------------------------- per-indicator ABI ----
int vta_ma_supported(const char* ma_type) { return ma_ind(ma_type) >= 0 ? 1 : 0; }

vta_status vta_ma_periods_device(vta_ctx* ctx, const char* ma_type, const char* const* param_keys,
                                 const double* param_values, size_t n_params, const float* d_prices, size_t len,
                                 size_t first_valid, const int* periods, size_t n_periods, int time_major,
                                 float* d_out) {
    return ma_periods_device(ctx, ma_type, param_keys, param_values, n_params, d_prices, len, first_valid,
                             periods, n_periods, time_major, d_out);
}

vta_status vta_ma_select_dev(vta_ctx* ctx, const char* ma_type, const char* const* param_keys,
                             const double* param_values, size_t n_params, const float* prices, size_t len,
                             size_t period_start, size_t period_end, size_t period_step, vta_device_array* out) {
    if (!prices || !out) return fail(VTA_ERR_INVALID_INPUT, "ma selector: null pointer");
    return ma_select(ctx, ma_type, param_keys, param_values, n_params, prices, len, period_start, period_end,
                     period_step, out, nullptr, 0, nullptr, nullptr);
}

vta_status vta_ma_select_into_host_f32(vta_ctx* ctx, const char* ma_type, const char* const* param_keys,
                                       const double* param_values, size_t n_params, const float* prices, size_t len,
                                       size_t period_start, size_t period_end, size_t period_step, float* out,
                                       size_t out_len, size_t* rows, size_t* cols) {
    if (!prices || !out) return fail(VTA_ERR_INVALID_INPUT, "ma selector: null pointer");
    return ma_select(ctx, ma_type, param_keys, param_values, n_params, prices, len, period_start, period_end,
                     period_step, nullptr, out, out_len, rows, cols);
}

#include "vta_abi_gen.inc"

}  // extern "C"
