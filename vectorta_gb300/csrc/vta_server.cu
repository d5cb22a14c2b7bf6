// Request server: continuous batching of single-series parameter sweeps over a
// device-resident store of series (vta_server_*).
//
// One server thread owns the device work.  It
//   * collects finished requests (an event per slot, polled without waiting),
//   * admits queued requests while a slot is free and the request's outputs
//     fit the memory budget (a request that has to wait for budget is counted
//     once as deferred), and
//   * enqueues each admitted request's kernels on its slot's stream through
//     the same driver the vta_X_batch_device entry points use, with outputs
//     from a stream-ordered memory pool.
// Slots run concurrently, so requests that arrive while others are on the
// device overlap with them.  Submitting, polling and releasing only take the
// server lock; none of them waits for the device.
//
// Requests are small or large by their estimated device time (outputs times
// ind_cost).  Each class has its own arrival-order queue.  A quarter of the
// slots (at least one) take small requests only and run on the device's
// highest-priority streams, so a burst of large sweeps neither holds every
// slot nor delays the blocks of the small ones; the other slots take small
// requests first and large ones otherwise, and a large request that has
// waited kLargeMaxWait goes before the small ones on those slots.  A large
// request waiting for memory budget does not hold back the small queue.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "vta_internal.h"

using namespace vta;

namespace {

struct Series {
    float* d[3] = {nullptr, nullptr, nullptr};  // high, low, close
    size_t len = 0;
    size_t fh = 0, fl = 0, fc = 0, fall = 0;     // first valid: high, low, close, all three
    bool hl = false;
};

struct Req {
    uint64_t ticket = 0;
    int ind = 0;
    uint32_t series = 0;
    vta_sweep sw{};
    size_t rows = 0;
    int n_out = 1;
    size_t bytes = 0;
    double t_submit = 0.0;
    bool deferred = false;
    bool large = false;  // estimated device time above kLargeWork
};

// a request with more than this many cost-weighted outputs is large (about a
// millisecond of device time at the write bandwidth)
constexpr double kLargeWork = 32e6;
constexpr double kLargeMaxWait = 0.05;  // seconds

struct Slot {
    vta_ctx* ctx = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    bool small_only = false;         // reserved for small requests (high-priority stream)
    cudaStream_t prio = nullptr;     // that stream (owned here)
    Req req;
    float* out[3] = {nullptr, nullptr, nullptr};
    double t_start = 0.0;
    vta_status launch_status = VTA_OK;
    std::string msg;
};

struct Result {
    vta_completion c{};
    size_t bytes = 0;
    std::string msg;
};

}  // namespace

struct vta_server {
    int device = 0;
    std::deque<Series> store;  // a deque: push_back keeps references to stored series valid
    std::vector<Slot> slots;
    cudaMemPool_t pool = nullptr;
    cudaStream_t aux_stream = nullptr;  // store uploads and releases
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> queue;                      // small requests, in arrival order
    std::deque<Req> q_large;                    // large requests, in arrival order
    int running_large = 0;
    std::deque<Result> ready;                   // finished, not yet polled
    std::unordered_map<uint64_t, Result> held;  // polled, not yet released
    size_t budget = 0, in_use = 0, running = 0;
    uint64_t next_ticket = 1, n_sub = 0, n_adm = 0, n_def = 0, n_done = 0, n_fail = 0;
    bool stop = false, draining = false;
    std::thread worker;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

// Inputs of indicator `ind` from a stored series, in the order the batch
// driver expects (close; high, low; high, low, close).
void inputs_of(const Series& se, int ind, const float* in[3]) {
    const int n = ind_inputs(ind);
    if (n == 1) {
        in[0] = se.d[2];
    } else {
        in[0] = se.d[0];
        in[1] = se.d[1];
        in[2] = n == 3 ? se.d[2] : nullptr;
    }
}

// Enqueues request r on slot sl (called by the server thread, lock released).
void launch(vta_server* S, Slot& sl, const Req& r) {
    sl.busy = true;
    sl.req = r;
    sl.t_start = S->now();
    sl.launch_status = VTA_OK;
    sl.msg.clear();
    *sl.ctx->err_host = 0;
    const Series& se = S->store[r.series];
    cudaStream_t st = sl.ctx->stream;
    for (int k = 0; k < 3; ++k) sl.out[k] = nullptr;
    vta_status s = VTA_OK;
    const size_t elems = r.rows * se.len;
    for (int k = 0; k < r.n_out && s == VTA_OK; ++k) {
        void* p = nullptr;
        const cudaError_t e = cudaMallocFromPoolAsync(&p, elems * sizeof(float), S->pool, st);
        if (e != cudaSuccess) s = cuda_fail(e, "cudaMallocFromPoolAsync(request output)");
        sl.out[k] = static_cast<float*>(p);
    }
    if (s == VTA_OK) {
        const float* in[3] = {nullptr, nullptr, nullptr};
        inputs_of(se, r.ind, in);
        const size_t first = ind_first(r.ind, se.fh, se.fl, se.fc, se.fall);
        s = batch_enqueue(sl.ctx, r.ind, in, se.len, first, &r.sw, sl.out);
    }
    if (s != VTA_OK) {
        sl.launch_status = s;
        sl.msg = vta_last_error();
    }
    cudaEventRecord(sl.done, st);
}

// Slot sl's request has finished (q = its event status): record the result.
void finish(vta_server* S, Slot& sl, cudaError_t q) {
    Result res;
    vta_completion& c = res.c;
    c.ticket = sl.req.ticket;
    c.status = sl.launch_status;
    res.msg = sl.msg;
    if (c.status == VTA_OK && q != cudaSuccess) {
        c.status = VTA_ERR_CUDA;
        res.msg = std::string("cuda error: ") + cudaGetErrorString(q);
    }
    if (c.status == VTA_OK && *sl.ctx->err_host) {
        c.status = VTA_ERR_CUDA;
        res.msg = "tcgen05 contraction: pipeline wait timed out";
    }
    c.rows = sl.req.rows;
    c.cols = S->store[sl.req.series].len;
    c.n_out = sl.req.n_out;
    c.t_submit = sl.req.t_submit;
    c.t_start = sl.t_start;
    c.t_done = S->now();
    res.bytes = sl.req.bytes;
    if (c.status == VTA_OK) {
        for (int k = 0; k < 3; ++k) c.d_out[k] = sl.out[k];
    } else {
        for (int k = 0; k < 3; ++k)
            if (sl.out[k]) cudaFreeAsync(sl.out[k], sl.ctx->stream);
        S->in_use -= res.bytes;
        res.bytes = 0;
        ++S->n_fail;
    }
    ++S->n_done;
    --S->running;
    if (sl.req.large) --S->running_large;
    sl.busy = false;
    S->ready.push_back(std::move(res));
    S->cv_done.notify_all();
}

void worker_main(vta_server* S) {
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (!S->stop) {
        bool progress = false;
        for (Slot& sl : S->slots) {
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaErrorNotReady) continue;
            finish(S, sl, q);
            progress = true;
        }
        // the head of queue q when it fits the memory budget (else it is
        // counted as deferred, once)
        auto fits = [&](std::deque<Req>& q) {
            if (q.empty()) return false;
            Req& f = q.front();
            if (S->in_use == 0 || S->in_use + f.bytes <= S->budget) return true;
            if (!f.deferred) {
                f.deferred = true;
                ++S->n_def;
            }
            return false;
        };
        const int large_cap = (int)S->slots.size() - (int)std::count_if(S->slots.begin(), S->slots.end(),
                                                                         [](const Slot& x) { return x.small_only; });
        for (bool again = true; again && !S->draining;) {
            again = false;
            for (Slot& sl : S->slots) {
                if (sl.busy) continue;
                const bool large_ok = !sl.small_only && S->running_large < large_cap;
                const bool large_due = large_ok && !S->q_large.empty() &&
                                       S->now() - S->q_large.front().t_submit > kLargeMaxWait;
                std::deque<Req>* q = nullptr;
                if (large_due && fits(S->q_large)) q = &S->q_large;
                else if (fits(S->queue)) q = &S->queue;
                else if (large_ok && fits(S->q_large)) q = &S->q_large;
                if (!q) continue;
                const Req r = q->front();
                q->pop_front();
                S->in_use += r.bytes;
                ++S->n_adm;
                ++S->running;
                if (r.large) ++S->running_large;
                sl.busy = true;
                lk.unlock();
                launch(S, sl, r);
                lk.lock();
                progress = again = true;
            }
        }
        if (!progress) S->cv_work.wait_for(lk, std::chrono::microseconds(S->running ? 20 : 2000));
    }
}

Result* find_result(vta_server* S, uint64_t ticket) {
    auto it = S->held.find(ticket);
    if (it != S->held.end()) return &it->second;
    for (Result& r : S->ready)
        if (r.c.ticket == ticket) return &r;
    return nullptr;
}

}  // namespace

extern "C" {

vta_status vta_server_create(int device_id, const vta_server_config* config, vta_server** out) {
    if (!out) return fail(VTA_ERR_INVALID_INPUT, "null out");
    *out = nullptr;
    int n = 0;
    VTA_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device_id < 0 || device_id >= n) return fail(VTA_ERR_INVALID_INPUT, "device id out of range");
    VTA_CUDA_TRY(cudaSetDevice(device_id));
    const int n_slots = config && config->slots > 0 ? config->slots : 8;
    if (n_slots > 64) return fail(VTA_ERR_INVALID_INPUT, "at most 64 slots");
    auto* S = new vta_server();
    S->device = device_id;
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    S->budget = config && config->memory_budget ? config->memory_budget : free_b / 2;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device_id;
    vta_status s = VTA_OK;
    cudaError_t e = cudaMemPoolCreate(&S->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = UINT64_MAX;  // keep freed blocks for reuse instead of returning them at each sync
        cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        e = cudaStreamCreateWithFlags(&S->aux_stream, cudaStreamNonBlocking);
    }
    if (e != cudaSuccess) s = cuda_fail(e, "server pool / stream");
    S->slots.resize(n_slots);
    const int reserve = n_slots >= 2 ? std::max(1, n_slots / 4) : 0;
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    for (int i = 0; i < n_slots && s == VTA_OK; ++i) {
        Slot& sl = S->slots[i];
        s = vta_ctx_create(device_id, &sl.ctx);
        if (s != VTA_OK) break;
        if (i < reserve) {
            sl.small_only = true;
            e = cudaStreamCreateWithPriority(&sl.prio, cudaStreamNonBlocking, prio_hi);
            if (e != cudaSuccess) {
                s = cuda_fail(e, "server slot stream");
                break;
            }
            s = vta_ctx_set_stream(sl.ctx, sl.prio);
            if (s != VTA_OK) break;
        }
        sl.ctx->async_alloc = true;
        sl.ctx->pool = S->pool;
        e = cudaHostAlloc((void**)&sl.ctx->err_host, sizeof(int), cudaHostAllocDefault);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e != cudaSuccess) s = cuda_fail(e, "server slot");
    }
    if (s != VTA_OK) {
        for (Slot& sl : S->slots) {
            if (sl.done) cudaEventDestroy(sl.done);
            if (sl.ctx) vta_ctx_destroy(sl.ctx);
            if (sl.prio) cudaStreamDestroy(sl.prio);
        }
        if (S->aux_stream) cudaStreamDestroy(S->aux_stream);
        if (S->pool) cudaMemPoolDestroy(S->pool);
        delete S;
        return s;
    }
    S->worker = std::thread(worker_main, S);
    *out = S;
    return VTA_OK;
}

static vta_status add_series(vta_server* S, const float* h, const float* l, const float* c, size_t len, uint32_t* id,
                             cudaMemcpyKind kind) {
    if (!S || !id) return fail(VTA_ERR_INVALID_INPUT, "null argument");
    if (!c) return fail(VTA_ERR_INVALID_INPUT, "close is required");
    if ((h == nullptr) != (l == nullptr)) return fail(VTA_ERR_INVALID_INPUT, "high and low go together");
    if (len == 0 || len > (size_t)INT32_MAX) return fail(VTA_ERR_INVALID_INPUT, "series length out of range");
    VTA_CUDA_TRY(cudaSetDevice(S->device));
    Series se;
    se.len = len;
    se.hl = h != nullptr;
    const float* src[3] = {h, l, c};
    for (int k = 0; k < 3; ++k) {
        if (!src[k]) continue;
        VTA_TRY(vram_check(len * sizeof(float)));
        VTA_CUDA_TRY(cudaMalloc((void**)&se.d[k], len * sizeof(float)));
        VTA_CUDA_TRY(cudaMemcpyAsync(se.d[k], src[k], len * sizeof(float), kind, S->aux_stream));
    }
    // first valid index per field and of all three (device scans)
    int* d_f = nullptr;
    VTA_CUDA_TRY(cudaMallocAsync((void**)&d_f, 4 * sizeof(int), S->aux_stream));
    VTA_TRY(launch_first_valid_tm(se.d[2], 1, (int)len, d_f + 2, S->aux_stream));
    if (se.hl) {
        VTA_TRY(launch_first_valid_tm(se.d[0], 1, (int)len, d_f + 0, S->aux_stream));
        VTA_TRY(launch_first_valid_tm(se.d[1], 1, (int)len, d_f + 1, S->aux_stream));
        VTA_TRY(launch_first_valid_tm_hlc(se.d[0], se.d[1], se.d[2], 1, (int)len, d_f + 3, S->aux_stream));
    }
    int f[4] = {0, 0, 0, 0};
    VTA_CUDA_TRY(cudaMemcpyAsync(f, d_f, sizeof f, cudaMemcpyDeviceToHost, S->aux_stream));
    VTA_CUDA_TRY(cudaFreeAsync(d_f, S->aux_stream));
    VTA_CUDA_TRY(cudaStreamSynchronize(S->aux_stream));
    se.fc = (size_t)f[2];
    se.fh = se.hl ? (size_t)f[0] : len;
    se.fl = se.hl ? (size_t)f[1] : len;
    se.fall = se.hl ? (size_t)f[3] : len;
    std::lock_guard<std::mutex> lock(S->mu);
    *id = (uint32_t)S->store.size();
    S->store.push_back(se);
    return VTA_OK;
}

vta_status vta_server_add_series(vta_server* s, const float* high, const float* low, const float* close, size_t len,
                                 uint32_t* id) {
    return add_series(s, high, low, close, len, id, cudaMemcpyHostToDevice);
}

vta_status vta_server_add_series_device(vta_server* s, const float* d_high, const float* d_low, const float* d_close,
                                        size_t len, uint32_t* id) {
    return add_series(s, d_high, d_low, d_close, len, id, cudaMemcpyDeviceToDevice);
}

vta_status vta_server_submit(vta_server* S, const vta_request* req, uint64_t* ticket) {
    if (!S || !req || !ticket) return fail(VTA_ERR_INVALID_INPUT, "null argument");
    const int ind = ind_by_name(req->indicator);
    if (ind < 0) return fail(VTA_ERR_INVALID_INPUT, std::string("unknown indicator: ") + (req->indicator ? req->indicator : "(null)"));
    Series se;
    {
        std::lock_guard<std::mutex> lock(S->mu);
        if (req->series >= S->store.size()) return fail(VTA_ERR_INVALID_INPUT, "unknown series id");
        se = S->store[req->series];
    }
    if (ind_inputs(ind) > 1 && !se.hl) return fail(VTA_ERR_INVALID_INPUT, "series has no high/low");
    Req r;
    r.ind = ind;
    r.series = req->series;
    r.sw = req->sweep;
    r.n_out = ind_outputs(ind);
    const size_t first = ind_first(ind, se.fh, se.fl, se.fc, se.fall);
    VTA_TRY(batch_check(ind, &r.sw, se.len, first, &r.rows));
    r.bytes = r.rows * se.len * sizeof(float) * (size_t)r.n_out;
    r.large = (double)r.rows * (double)se.len * r.n_out * ind_cost(ind) > kLargeWork;
    std::lock_guard<std::mutex> lock(S->mu);
    if (r.bytes > S->budget) return fail(VTA_ERR_OUT_OF_MEMORY, "request outputs exceed the server's memory budget");
    r.ticket = S->next_ticket++;
    r.t_submit = S->now();
    (r.large ? S->q_large : S->queue).push_back(r);
    ++S->n_sub;
    *ticket = r.ticket;
    S->cv_work.notify_one();
    return VTA_OK;
}

vta_status vta_server_poll(vta_server* S, vta_completion* out, size_t cap, size_t* n, int wait_ms) {
    if (!S || !n || (cap && !out)) return fail(VTA_ERR_INVALID_INPUT, "null argument");
    std::unique_lock<std::mutex> lk(S->mu);
    if (S->ready.empty() && wait_ms > 0)
        S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !S->ready.empty(); });
    size_t k = 0;
    while (k < cap && !S->ready.empty()) {
        Result r = std::move(S->ready.front());
        S->ready.pop_front();
        out[k++] = r.c;
        if (r.c.status != VTA_OK) set_error(r.msg);
        S->held.emplace(r.c.ticket, std::move(r));
    }
    *n = k;
    return VTA_OK;
}

vta_status vta_server_copy_out(vta_server* S, uint64_t ticket, int k, float* host, size_t n_floats) {
    if (!S || !host) return fail(VTA_ERR_INVALID_INPUT, "null argument");
    float* src = nullptr;
    size_t elems = 0;
    {
        std::lock_guard<std::mutex> lock(S->mu);
        Result* r = find_result(S, ticket);
        if (!r) return fail(VTA_ERR_INVALID_INPUT, "no completed, unreleased request with this ticket");
        if (r->c.status != VTA_OK) return fail(VTA_ERR_INVALID_INPUT, "the request failed: " + r->msg);
        if (k < 0 || k >= r->c.n_out) return fail(VTA_ERR_INVALID_INPUT, "output index out of range");
        src = r->c.d_out[k];
        elems = r->c.rows * r->c.cols;
    }
    if (n_floats < elems) return fail(VTA_ERR_INVALID_INPUT, "host buffer too small");
    VTA_CUDA_TRY(cudaSetDevice(S->device));
    VTA_CUDA_TRY(cudaMemcpy(host, src, elems * sizeof(float), cudaMemcpyDeviceToHost));
    return VTA_OK;
}

vta_status vta_server_release(vta_server* S, uint64_t ticket) {
    if (!S) return fail(VTA_ERR_INVALID_INPUT, "null server");
    std::lock_guard<std::mutex> lock(S->mu);
    Result r;
    auto it = S->held.find(ticket);
    if (it != S->held.end()) {
        r = std::move(it->second);
        S->held.erase(it);
    } else {
        auto jt = std::find_if(S->ready.begin(), S->ready.end(), [&](const Result& x) { return x.c.ticket == ticket; });
        if (jt == S->ready.end()) return fail(VTA_ERR_INVALID_INPUT, "no completed, unreleased request with this ticket");
        r = std::move(*jt);
        S->ready.erase(jt);
    }
    if (r.bytes) {
        VTA_CUDA_TRY(cudaSetDevice(S->device));
        for (int k = 0; k < r.c.n_out; ++k)
            if (r.c.d_out[k]) cudaFreeAsync(r.c.d_out[k], S->aux_stream);
        S->in_use -= r.bytes;
        S->cv_work.notify_one();
    }
    return VTA_OK;
}

vta_status vta_server_get_stats(vta_server* S, vta_server_stats* st) {
    if (!S || !st) return fail(VTA_ERR_INVALID_INPUT, "null argument");
    std::lock_guard<std::mutex> lock(S->mu);
    st->submitted = S->n_sub;
    st->admitted = S->n_adm;
    st->deferred = S->n_def;
    st->completed = S->n_done;
    st->failed = S->n_fail;
    st->queued = S->queue.size() + S->q_large.size();
    st->running = S->running;
    st->bytes_in_use = S->in_use;
    st->memory_budget = S->budget;
    return VTA_OK;
}

vta_status vta_server_destroy(vta_server* S) {
    if (!S) return VTA_OK;
    {
        std::unique_lock<std::mutex> lk(S->mu);
        S->draining = true;  // admit nothing more; let the running requests finish
        S->cv_work.notify_all();
        while (S->running > 0) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(200));
            lk.lock();
        }
        S->stop = true;
        S->cv_work.notify_all();
    }
    S->worker.join();
    cudaSetDevice(S->device);
    for (auto& kv : S->held)
        for (int k = 0; k < kv.second.c.n_out; ++k)
            if (kv.second.c.d_out[k]) cudaFreeAsync(kv.second.c.d_out[k], S->aux_stream);
    for (Result& r : S->ready)
        for (int k = 0; k < r.c.n_out; ++k)
            if (r.c.d_out[k]) cudaFreeAsync(r.c.d_out[k], S->aux_stream);
    cudaStreamSynchronize(S->aux_stream);
    for (Slot& sl : S->slots) {
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.ctx) vta_ctx_destroy(sl.ctx);
        if (sl.prio) cudaStreamDestroy(sl.prio);
    }
    for (Series& se : S->store)
        for (float* p : se.d)
            if (p) cudaFree(p);
    cudaStreamDestroy(S->aux_stream);
    cudaMemPoolDestroy(S->pool);
    delete S;
    return VTA_OK;
}

}  // extern "C"
