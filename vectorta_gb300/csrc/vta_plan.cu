// Many-series work-list plans (vta_tm_plan_*): host side.
//
// A plan binds device OHLC inputs, per-series lengths and a list of jobs
// (indicator + parameters + outputs), picks each job's time-chunk length
// (timed on the plan's own data unless the context policy fixes it; results
// cached per indicator, period, length and series count), builds the work
// list and captures one run -- first-valid scans, the persistent work-list
// kernel, the fix-up pass and the read-back of its counters -- in a CUDA
// graph that vta_tm_plan_run replays.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "vta_internal.h"
#include "vta_plan.h"

using namespace vta;

struct vta_tm_plan {
    vta_ctx* ctx = nullptr;
    const float* h = nullptr;
    const float* l = nullptr;
    const float* c = nullptr;
    int cols = 0, rows = 0;
    std::vector<int> lens;      // host copy of the series lengths
    std::vector<int> tile_max;  // longest series of each 32-series tile
    std::vector<PlanJob> jobs;  // device pointers inside
    std::vector<size_t> state_cap;  // chunks the state buffers of each job hold
    std::vector<void*> allocs;  // every device allocation of the plan
    int* d_len = nullptr;
    int* d_first_hlc = nullptr;
    int* d_first_c = nullptr;
    PlanJob* d_jobs = nullptr;
    int4* d_items = nullptr;
    size_t items_cap = 0;
    int n_items = 0;
    int* d_ctr = nullptr;   // [0] work-list head, [1] fix-up count
    int* h_stats = nullptr; // pinned copy of d_ctr after each run
    int blocks = 0;
    bool tuned = false;
    size_t fixups = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

vta_status plan_alloc(vta_tm_plan* P, size_t bytes, void** out) {
    VTA_TRY(vram_check(bytes));
    VTA_CUDA_TRY(cudaMalloc(out, bytes));
    P->allocs.push_back(*out);
    return VTA_OK;
}

void plan_free(vta_tm_plan* P, void* p) {
    auto it = std::find(P->allocs.begin(), P->allocs.end(), p);
    if (it != P->allocs.end()) {
        cudaFree(p);
        P->allocs.erase(it);
    }
}

int n_chunks_of(int rows, int chunk) { return (rows + chunk - 1) / chunk; }

// State buffers of job j for `chunk` (grown when too small).
vta_status plan_states(vta_tm_plan* P, int j, int chunk) {
    PlanJob& J = P->jobs[j];
    J.chunk = chunk;
    if (!plan_job_recurrent(J.kind)) return VTA_OK;
    const size_t nch = (size_t)n_chunks_of(P->rows, chunk);
    if (nch <= P->state_cap[j]) return VTA_OK;
    plan_free(P, J.st_start);
    plan_free(P, J.st_end);
    plan_free(P, J.exact);
    void *a = nullptr, *b = nullptr, *e = nullptr;
    const size_t words = nch * (size_t)P->cols * 8;
    VTA_TRY(plan_alloc(P, words * sizeof(float), &a));
    VTA_TRY(plan_alloc(P, words * sizeof(float), &b));
    VTA_TRY(plan_alloc(P, nch * (size_t)P->cols, &e));
    J.st_start = static_cast<float*>(a);
    J.st_end = static_cast<float*>(b);
    J.exact = static_cast<unsigned char*>(e);
    P->state_cap[j] = nch;
    return VTA_OK;
}

// Work list of the jobs in `which` (indices into P->jobs; the item's job field
// is the position in `which`), ordered by chunk start so that the jobs and
// tiles working on the same rows run together and share the inputs in L2.
vta_status plan_items(vta_tm_plan* P, const std::vector<int>& which) {
    struct Key {
        int c0, tile, job, k;
    };
    std::vector<Key> keys;
    for (size_t q = 0; q < which.size(); ++q) {
        const PlanJob& J = P->jobs[which[q]];
        for (size_t g = 0; g < P->tile_max.size(); ++g)
            for (int k = 0; (long long)k * J.chunk < P->tile_max[g]; ++k)
                keys.push_back({k * J.chunk, (int)g, (int)q, k});
    }
    std::sort(keys.begin(), keys.end(), [](const Key& a, const Key& b) {
        return std::tie(a.c0, a.tile, a.job) < std::tie(b.c0, b.tile, b.job);
    });
    if (keys.size() > (size_t)INT32_MAX) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "tm plan: too many work items");
    if (keys.size() > P->items_cap) {
        plan_free(P, P->d_items);
        void* p = nullptr;
        VTA_TRY(plan_alloc(P, std::max<size_t>(keys.size(), 1) * sizeof(int4), &p));
        P->d_items = static_cast<int4*>(p);
        P->items_cap = keys.size();
    }
    std::vector<int4> items(keys.size());
    for (size_t i = 0; i < keys.size(); ++i) items[i] = make_int4(keys[i].job, keys[i].tile, keys[i].k, 0);
    if (!items.empty())
        VTA_CUDA_TRY(cudaMemcpy(P->d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    P->n_items = (int)items.size();
    return VTA_OK;
}

// Device copy of the jobs in `which`, at d_jobs[0 ..).
vta_status plan_upload_jobs(vta_tm_plan* P, const std::vector<int>& which) {
    std::vector<PlanJob> js;
    for (int j : which) js.push_back(P->jobs[j]);
    VTA_CUDA_TRY(cudaMemcpy(P->d_jobs, js.data(), js.size() * sizeof(PlanJob), cudaMemcpyHostToDevice));
    return VTA_OK;
}

PlanArgs plan_args(const vta_tm_plan* P, int n_jobs) {
    PlanArgs a{};
    a.h = P->h;
    a.l = P->l;
    a.c = P->c;
    a.cols = P->cols;
    a.rows = P->rows;
    a.len = P->d_len;
    a.first_hlc = P->d_first_hlc;
    a.first_c = P->d_first_c;
    a.jobs = P->d_jobs;
    a.n_jobs = n_jobs;
    a.items = P->d_items;
    a.n_items = P->n_items;
    a.counter = P->d_ctr;
    a.stats = P->d_ctr + 1;
    return a;
}

// One run on stream st: first-valid scans, work list, fix-up, counters back.
vta_status plan_enqueue(vta_tm_plan* P, int n_jobs, cudaStream_t st, bool with_first) {
    VTA_CUDA_TRY(cudaMemsetAsync(P->d_ctr, 0, 2 * sizeof(int), st));
    const PlanArgs a = plan_args(P, n_jobs);
    if (with_first) VTA_TRY(launch_plan_first(a, P->d_first_hlc, P->d_first_c, st));
    VTA_TRY(launch_tm_plan(a, P->blocks, st));
    VTA_TRY(launch_tm_fixup(a, st));
    VTA_CUDA_TRY(cudaMemcpyAsync(P->h_stats, P->d_ctr, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    return VTA_OK;
}

// ---------------------------------------------------------------- tuning ----
// Chunk length per (indicator, period, length bucket, series-count bucket),
// for the process; with VTA_TUNE_CACHE=<file> also read from and appended to
// that file ("kind period len_bucket cols_bucket chunk" per line).
using TuneKey = std::tuple<int, int, int, int>;
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;
bool g_tune_loaded = false;

int log2_bucket(long long v) {
    int b = 0;
    while ((1LL << b) < v) ++b;
    return b;
}

void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = std::getenv("VTA_TUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    int k, p, lb, cb, ch;
    while (std::fscanf(f, "%d %d %d %d %d", &k, &p, &lb, &cb, &ch) == 5)
        if (ch > 0) g_tune[TuneKey{k, p, lb, cb}] = ch;
    std::fclose(f);
}

void tune_store_locked(const TuneKey& key, int chunk) {
    g_tune[key] = chunk;
    const char* path = std::getenv("VTA_TUNE_CACHE");
    if (!path || !*path) return;
    if (FILE* f = std::fopen(path, "a")) {
        std::fprintf(f, "%d %d %d %d %d\n", std::get<0>(key), std::get<1>(key), std::get<2>(key), std::get<3>(key),
                     chunk);
        std::fclose(f);
    }
}

// Times job j alone with each candidate chunk length (second of two runs)
// and returns the fastest.
vta_status tune_job(vta_tm_plan* P, int j, int* best) {
    static const int kRec[] = {1024, 2048, 4096, 8192, 16384};
    static const int kPnr[] = {128, 256, 512, 1024};
    const bool rec = plan_job_recurrent(P->jobs[j].kind);
    const int* cand = rec ? kRec : kPnr;
    const int nc = rec ? 5 : 4;
    const int maxlen = *std::max_element(P->lens.begin(), P->lens.end());
    cudaStream_t st = P->ctx->stream;
    cudaEvent_t e0, e1;
    VTA_CUDA_TRY(cudaEventCreate(&e0));
    VTA_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 1e30f;
    *best = cand[0];
    vta_status s = VTA_OK;
    for (int i = 0; i < nc && s == VTA_OK; ++i) {
        if (i > 0 && cand[i - 1] >= maxlen) break;  // one chunk per series already
        s = plan_states(P, j, cand[i]);
        if (s == VTA_OK) s = plan_items(P, {j});
        if (s == VTA_OK) s = plan_upload_jobs(P, {j});
        float ms = 0.f;
        for (int rep = 0; rep < 2 && s == VTA_OK; ++rep) {
            cudaEventRecord(e0, st);
            s = plan_enqueue(P, 1, st, false);
            cudaEventRecord(e1, st);
            if (s == VTA_OK && cudaStreamSynchronize(st) != cudaSuccess) s = check_launch("tm plan tuning");
            if (s == VTA_OK) cudaEventElapsedTime(&ms, e0, e1);
        }
        if (s == VTA_OK && ms < best_ms) {
            best_ms = ms;
            *best = cand[i];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return s;
}

void plan_release(vta_tm_plan* P) {
    if (!P) return;
    if (P->ctx) cudaSetDevice(P->ctx->device);
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    for (void* p : P->allocs) cudaFree(p);
    if (P->h_stats) cudaFreeHost(P->h_stats);
    delete P;
}

vta_status plan_create(vta_ctx* ctx, const float* h, const float* l, const float* c, size_t cols, size_t rows,
                       const size_t* lengths, const vta_tm_job* jobs, size_t n_jobs, vta_tm_plan* P) {
    if (!h || !l || !c) return fail(VTA_ERR_INVALID_INPUT, "tm plan: null input pointer");
    if (cols == 0 || rows == 0) return fail(VTA_ERR_INVALID_INPUT, "tm plan: empty matrix");
    if (cols > (size_t)INT32_MAX / 2 || rows > (size_t)INT32_MAX / 2 || cols * rows > (size_t)1 << 40)
        return fail(VTA_ERR_INVALID_INPUT, "tm plan: matrix too large");
    if (!jobs || n_jobs == 0) return fail(VTA_ERR_INVALID_INPUT, "tm plan: no jobs");
    if (n_jobs > 64) return fail(VTA_ERR_INVALID_INPUT, "tm plan: at most 64 jobs");
    P->ctx = ctx;
    P->h = h;
    P->l = l;
    P->c = c;
    P->cols = (int)cols;
    P->rows = (int)rows;
    P->lens.resize(cols);
    for (size_t s = 0; s < cols; ++s) {
        const size_t L = lengths ? lengths[s] : rows;
        if (L > rows) return fail(VTA_ERR_INVALID_INPUT, "tm plan: a series length exceeds rows");
        P->lens[s] = (int)L;
    }
    for (size_t g = 0; g < (cols + 31) / 32; ++g) {
        int mx = 0;
        for (size_t s = g * 32; s < std::min(cols, g * 32 + 32); ++s) mx = std::max(mx, P->lens[s]);
        P->tile_max.push_back(mx);
    }
    for (size_t j = 0; j < n_jobs; ++j) {
        const vta_tm_job& in = jobs[j];
        char buf[160];
        auto bad = [&](const char* why) {
            std::snprintf(buf, sizeof buf, "tm plan: job %zu: %s", j, why);
            return fail(VTA_ERR_INVALID_INPUT, buf);
        };
        if (in.kind < VTA_TM_ATR || in.kind > VTA_TM_PERCENTILE) return bad("unknown kind");
        if (in.period == 0 || in.period > (size_t)(1 << 20)) return bad("period must be in 1..2^20");
        if (!in.d_out0) return bad("null output");
        if (in.kind == VTA_TM_SUPERTREND && !in.d_out1) return bad("SuperTrend needs d_out1 (changed)");
        if (in.kind == VTA_TM_SUPERTREND && !std::isfinite(in.param)) return bad("factor must be finite");
        if (in.kind == VTA_TM_PERCENTILE) {
            if (in.period > (size_t)kPlanMaxPnrWindow) {
                std::snprintf(buf, sizeof buf,
                              "tm plan: job %zu: percentile length above %d (use the many-series entry point)", j,
                              kPlanMaxPnrWindow);
                return fail(VTA_ERR_NOT_IMPLEMENTED, buf);
            }
            if (!(in.param >= 0.0 && in.param <= 100.0)) return bad("percentage must be in [0, 100]");
        }
        PlanJob J{};
        J.kind = in.kind;  // vta_tm_kind and PlanKind share their values
        J.period = (int)in.period;
        J.param = (float)in.param;
        J.pfrac = in.param * 0.01;
        J.out0 = in.d_out0;
        J.out1 = in.d_out1;
        // (1 - 1/p)^(32 p) < e^-32: the guessed state's error decays far below an
        // f32 ulp, with room for the last ulp of difference to round away
        J.warm = ctx->policy.tm_warm > 0 ? ctx->policy.tm_warm : 32 * J.period + 64;
        P->jobs.push_back(J);
    }
    P->state_cap.assign(n_jobs, 0);
    void* p = nullptr;
    VTA_TRY(plan_alloc(P, cols * sizeof(int), &p));
    P->d_len = static_cast<int*>(p);
    VTA_TRY(plan_alloc(P, cols * sizeof(int), &p));
    P->d_first_hlc = static_cast<int*>(p);
    VTA_TRY(plan_alloc(P, cols * sizeof(int), &p));
    P->d_first_c = static_cast<int*>(p);
    VTA_TRY(plan_alloc(P, n_jobs * sizeof(PlanJob), &p));
    P->d_jobs = static_cast<PlanJob*>(p);
    VTA_TRY(plan_alloc(P, 2 * sizeof(int), &p));
    P->d_ctr = static_cast<int*>(p);
    VTA_CUDA_TRY(cudaHostAlloc((void**)&P->h_stats, 2 * sizeof(int), cudaHostAllocDefault));
    VTA_CUDA_TRY(cudaMemcpy(P->d_len, P->lens.data(), cols * sizeof(int), cudaMemcpyHostToDevice));
    P->blocks = tm_plan_blocks(ctx->num_sms);

    cudaStream_t st = ctx->stream;
    const PlanArgs a0 = plan_args(P, 0);
    VTA_TRY(launch_plan_first(a0, P->d_first_hlc, P->d_first_c, st));
    // chunk length per job: policy, cache, or timed now
    const int maxlen = *std::max_element(P->lens.begin(), P->lens.end());
    for (size_t j = 0; j < n_jobs; ++j) {
        int chunk = ctx->policy.tm_chunk;
        if (chunk < 0) chunk = std::max(maxlen, 1);
        if (chunk == 0) {
            const TuneKey key{P->jobs[j].kind, P->jobs[j].period, log2_bucket(maxlen), log2_bucket((long long)cols)};
            {
                std::lock_guard<std::mutex> lock(g_tune_mu);
                tune_load_locked();
                auto it = g_tune.find(key);
                if (it != g_tune.end()) chunk = it->second;
            }
            if (chunk == 0) {
                VTA_TRY(tune_job(P, (int)j, &chunk));
                P->tuned = true;
                std::lock_guard<std::mutex> lock(g_tune_mu);
                tune_store_locked(key, chunk);
            }
        }
        VTA_TRY(plan_states(P, (int)j, chunk));
    }
    std::vector<int> all(n_jobs);
    for (size_t j = 0; j < n_jobs; ++j) all[j] = (int)j;
    VTA_TRY(plan_items(P, all));
    VTA_TRY(plan_upload_jobs(P, all));
    VTA_CUDA_TRY(cudaStreamSynchronize(st));

    // capture one full run
    VTA_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const vta_status cs = plan_enqueue(P, (int)n_jobs, st, true);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (cs != VTA_OK) {
        if (g) cudaGraphDestroy(g);
        return cs;
    }
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture(tm plan)");
    P->graph = g;
    VTA_CUDA_TRY(cudaGraphInstantiate(&P->exec, P->graph, 0));
    return VTA_OK;
}

}  // namespace

extern "C" {

vta_status vta_tm_plan_create(vta_ctx* ctx, const float* d_high, const float* d_low, const float* d_close,
                              size_t cols, size_t rows, const size_t* lengths, const vta_tm_job* jobs,
                              size_t n_jobs, vta_tm_plan** out) {
    if (!out) return fail(VTA_ERR_INVALID_INPUT, "null out");
    *out = nullptr;
    VTA_TRY(enter_call(ctx));
    auto* P = new vta_tm_plan();
    const vta_status s = plan_create(ctx, d_high, d_low, d_close, cols, rows, lengths, jobs, n_jobs, P);
    if (s != VTA_OK) {
        cudaStreamSynchronize(ctx->stream);
        plan_release(P);
        return s;
    }
    ctx->last_kernel = "tm_plan";
    *out = P;
    return VTA_OK;
}

vta_status vta_tm_plan_run(vta_tm_plan* plan) {
    if (!plan) return fail(VTA_ERR_INVALID_INPUT, "null plan");
    VTA_TRY(enter_call(plan->ctx));
    cudaStream_t st = plan->ctx->stream;
    ktimer_begin(st);
    VTA_CUDA_TRY(cudaGraphLaunch(plan->exec, st));
    ktimer_end(st);
    VTA_CUDA_TRY(cudaStreamSynchronize(st));
    VTA_TRY(check_launch("tm plan graph"));
    plan->fixups = (size_t)plan->h_stats[1];
    plan->ctx->last_kernel = "tm_plan";
    return VTA_OK;
}

vta_status vta_tm_plan_info_get(const vta_tm_plan* plan, vta_tm_plan_info* info) {
    if (!plan || !info) return fail(VTA_ERR_INVALID_INPUT, "null argument");
    *info = vta_tm_plan_info{};
    info->n_items = (size_t)plan->n_items;
    for (size_t j = 0; j < plan->jobs.size() && j < 8; ++j) info->chunk[j] = (size_t)plan->jobs[j].chunk;
    info->fixups = plan->fixups;
    info->tuned = plan->tuned ? 1 : 0;
    return VTA_OK;
}

vta_status vta_tm_plan_destroy(vta_tm_plan* plan) {
    if (!plan) return VTA_OK;
    if (plan->ctx) cudaStreamSynchronize(plan->ctx->stream);
    plan_release(plan);
    return VTA_OK;
}

}  // extern "C"

namespace vta {

// One job of the plan kernels over a rectangular time-major matrix (every
// series `rows` long): the many-series entry points of ATR, ADX, SuperTrend
// and percentile use it.  Workspace from the context arena, chunk length
// fixed (1,024 steps; 512 for the percentile) unless the policy sets it.
vta_status tm_job_enqueue(vta_ctx* ctx, int kind, int period, double param, const float* h, const float* l,
                          const float* c, int cols, int rows, float* out0, float* out1, cudaStream_t st) {
    const bool rec = plan_job_recurrent(kind);
    int chunk = rec ? 1024 : 512;
    if (ctx->policy.tm_chunk > 0) chunk = ctx->policy.tm_chunk;
    if (ctx->policy.tm_chunk < 0 || 2LL * chunk > rows) chunk = rows;  // one chunk per series
    const int tiles = (cols + 31) / 32;
    const int nch = (rows + chunk - 1) / chunk;
    const size_t n_items = (size_t)tiles * nch;
    if (n_items > (size_t)INT32_MAX) return fail(VTA_ERR_LAUNCH_CONFIG_TOO_LARGE, "too many work items");
    const size_t states = rec ? (size_t)nch * cols : 0;
    Arena ar(ctx);
    ar.need(cols * sizeof(int));
    ar.need(cols * sizeof(int));
    ar.need(cols * sizeof(int));
    ar.need(sizeof(PlanJob));
    ar.need(n_items * sizeof(int4));
    ar.need(2 * sizeof(int));
    ar.need(states * 8 * sizeof(float));
    ar.need(states * 8 * sizeof(float));
    ar.need(states);
    VTA_TRY(ar.commit());
    int* d_len = ar.take<int>(cols);
    int* d_fh = ar.take<int>(cols);
    int* d_fc = ar.take<int>(cols);
    PlanJob* d_job = ar.take<PlanJob>(1);
    int4* d_items = ar.take<int4>(n_items);
    int* d_ctr = ar.take<int>(2);
    PlanJob J{};
    J.kind = kind;
    J.period = period;
    J.param = (float)param;
    J.pfrac = param * 0.01;
    J.chunk = chunk;
    J.warm = ctx->policy.tm_warm > 0 ? ctx->policy.tm_warm : 32 * period + 64;
    J.out0 = out0;
    J.out1 = out1;
    J.st_start = ar.take<float>(states * 8);
    J.st_end = ar.take<float>(states * 8);
    J.exact = ar.take<unsigned char>(states);
    const std::vector<int> lens(cols, rows);
    std::vector<int4> items;
    items.reserve(n_items);
    for (int k = 0; k < nch; ++k)
        for (int g = 0; g < tiles; ++g) items.push_back(make_int4(0, g, k, 0));
    VTA_TRY(upload_async(ctx, d_len, lens.data(), cols * sizeof(int), st));
    VTA_TRY(upload_async(ctx, d_job, &J, sizeof(PlanJob), st));
    VTA_TRY(upload_async(ctx, d_items, items.data(), n_items * sizeof(int4), st));
    VTA_CUDA_TRY(cudaMemsetAsync(d_ctr, 0, 2 * sizeof(int), st));
    PlanArgs a{};
    a.h = h ? h : c;  // close-only jobs: the high/low scan sees close
    a.l = l ? l : c;
    a.c = c;
    a.cols = cols;
    a.rows = rows;
    a.len = d_len;
    a.first_hlc = d_fh;
    a.first_c = d_fc;
    a.jobs = d_job;
    a.n_jobs = 1;
    a.items = d_items;
    a.n_items = (int)n_items;
    a.counter = d_ctr;
    a.stats = d_ctr + 1;
    VTA_TRY(launch_plan_first(a, d_fh, d_fc, st));
    ktimer_begin(st);
    VTA_TRY(launch_tm_plan(a, tm_plan_blocks(ctx->num_sms), st));
    VTA_TRY(launch_tm_fixup(a, st));
    ktimer_end(st);
    return VTA_OK;
}

}  // namespace vta
