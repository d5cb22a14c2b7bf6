// Internal declarations shared by the host API (vta_api.cu) and the kernel
// translation units.  Nothing here is part of the C ABI (include/vta_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstddef>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/vta_gb300.h"

namespace vta {

// ---------------------------------------------------------------- errors ---
void set_error(const std::string& msg);
vta_status fail(vta_status st, const std::string& msg);
vta_status cuda_fail(cudaError_t e, const char* what);

#define VTA_CUDA_TRY(expr)                                         \
    do {                                                           \
        cudaError_t _e = (expr);                                   \
        if (_e != cudaSuccess) return ::vta::cuda_fail(_e, #expr); \
    } while (0)

#define VTA_TRY(expr)                        \
    do {                                     \
        vta_status _s = (expr);              \
        if (_s != VTA_OK) return _s;         \
    } while (0)

// Checks the launch that was just enqueued (and counts it).
vta_status check_launch(const char* kernel);
// The sticky / asynchronous error state after non-kernel work (a stream
// synchronize, a copy); not counted as a launch.
vta_status check_async(const char* what);

// Event timer around a call's main output kernel, on the launching stream;
// active only when the current context has policy "timing" = "on".
void ktimer_begin(cudaStream_t st);
void ktimer_end(cudaStream_t st);

// ---------------------------------------------------------------- launch ---
constexpr int kNumSMs = 152;     // GB300: 2 dies x 76 SMs (re-read at ctx create)
constexpr int kChunkMin = 256;   // smallest time chunk of the chunked scans

struct Policy {
    // weighted-window batch kernel: 0 = auto, 1 = plain FP32, 2 = tcgen05 fp16x3,
    // 3 = tcgen05 bf16x3
    int wma_batch = 0;
    // recurrence time-chunk length (0 = auto); 1 = whole series (plain
    // sequential per-combo kernel)
    int recur_chunk = 0;
    // many-series plans: time-chunk length (0 = timed at plan creation,
    // -1 = one chunk per series) and warm-restart steps (0 = 32 p + 64)
    int tm_chunk = 0;
    int tm_warm = 0;
    // *_batch_into_host_f32: 0 = keep the device input/output buffers in the
    // context between calls ("cached"), 1 = allocate and free them per call
    int host_io = 0;
    // batch-sweep autotuner: 0 = on (time candidates on the first call per
    // key), 1 = off (untuned defaults), 2 = cached choices only
    int tune = 0;
    // chunk aggregates of the EMA / DEMA / TEMA / RSI batch sweeps: 0 = auto
    // (tensor-core contraction where the sweep is eligible), 1 = CUDA cores
    // only, 2 = tensor cores required (an ineligible sweep is an error)
    int recur_agg = 0;
    // chunk length of the exact ADX scan (0 = auto: about 2,400 warp items)
    int scan_chunk = 0;
    // *_batch_into_host_f32 outputs in vta_pinned_alloc buffers: 0 = the
    // kernels store into them directly, 1 = device buffer and a copy
    int host_out = 0;
};

}  // namespace vta

// The opaque context of the C ABI.
struct vta_ctx {
    int device = 0;
    int num_sms = vta::kNumSMs;
    size_t smem_optin = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = true;
    void* scratch = nullptr;  // growing device workspace, owned by the ctx
    size_t scratch_bytes = 0;
    void* aux = nullptr;      // second growing device workspace (operands a launcher
    size_t aux_bytes = 0;     // builds after the call's arena pieces are taken)
    void* io = nullptr;       // device inputs + outputs of *_batch_into_host_f32 (host_io cached)
    size_t io_bytes = 0;
    void* tmp = nullptr;      // row-major staging of time-major MA-computer outputs
    size_t tmp_bytes = 0;
    void* host_stage = nullptr;  // pinned staging of small uploads, reused per call
    size_t host_stage_bytes = 0;
    size_t host_stage_off = 0;
    cudaEvent_t stage_ev = nullptr;  // recorded behind the last staged copy
    bool stage_pending = false;
    vta::Policy policy;
    std::string last_kernel;
    bool timing = false;
    bool timed = false;  // the last call recorded both events
    // server slots: workspaces grow stream-ordered and calls never wait for
    // the device; the tensor-core path leaves its error word in err_host
    bool async_alloc = false;
    int* err_host = nullptr;         // pinned
    cudaMemPool_t pool = nullptr;    // stream-ordered allocations of async slots
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // constant cache: small per-sweep arrays (period lists, per-combo
    // constants) uploaded once and reused by later calls with the same bytes
    void* cc_dev = nullptr;
    size_t cc_cap = 0, cc_used = 0;
    std::vector<unsigned char> cc_host;  // host copy of cc_dev[0, cc_used)
    struct CcEntry {
        uint64_t hash;
        size_t off, bytes;
    };
    std::vector<CcEntry> cc;
    // packed weights of the tensor-core recurrence aggregates, kept across
    // calls per (kind, chunk length, periods); least recently used evicted
    struct RwEntry {
        int kind, L;
        std::vector<int> periods;
        void* dev;
        size_t bytes;
        uint64_t tick;
        bool valid;  // the weights kernel ran on this buffer
    };
    std::vector<RwEntry> rw;
    uint64_t rw_tick = 0;
};

namespace vta {

// Bump allocator over the ctx workspace.  Usage: first `need()` every piece,
// then `commit()` (grows the workspace with cudaMalloc when too small), then
// `take()` the pieces in the same order.  Pieces are 256-byte aligned.
class Arena {
   public:
    explicit Arena(vta_ctx* c) : ctx_(c) {}
    void need(size_t bytes) { total_ += align(bytes); }
    vta_status commit();
    template <class T>
    T* take(size_t count) {
        char* p = static_cast<char*>(ctx_->scratch) + off_;
        off_ += align(count * sizeof(T));
        return reinterpret_cast<T*>(p);
    }
    size_t total() const { return total_; }

   private:
    static size_t align(size_t b) { return (b + 255) & ~size_t(255); }
    vta_ctx* ctx_;
    size_t total_ = 0;
    size_t off_ = 0;
};

// Device workspace of at least `bytes` in ctx->aux (grown with cudaMalloc;
// valid until the next ctx_aux call on the same context).
vta_status ctx_aux(vta_ctx* ctx, size_t bytes, void** out);
// Host -> device copy on `st`, staged through the context's pinned buffer when
// it fits (the copy is then fully asynchronous), else a pageable copy.
vta_status upload_async(vta_ctx* ctx, void* dst, const void* src, size_t bytes, cudaStream_t st);

// Device copy of `bytes` constant bytes for this call: from the context's
// constant cache when an earlier call uploaded the same bytes, else uploaded
// into the cache (or, for server slots and large arrays, into `fallback`).
vta_status const_upload_bytes(vta_ctx* ctx, const void* src, size_t bytes, void* fallback, const void** out);
// The device address of [p, p + bytes) when it lies inside one block from
// vta_pinned_alloc, else null
float* pinned_device_view(const void* p, size_t bytes);
template <class T>
inline vta_status const_upload(vta_ctx* ctx, const T* src, size_t count, T* fallback, const T** out) {
    const void* p = nullptr;
    const vta_status st = const_upload_bytes(ctx, src, count * sizeof(T), fallback, &p);
    *out = static_cast<const T*>(p);
    return st;
}

// VRAM admission check mirroring the crate's wrappers: required + 64 MiB
// headroom must fit in free memory (disabled with VTA_MEM_CHECK=0).
vta_status vram_check(size_t required_bytes);

inline unsigned ceil_div(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// ------------------------------------------------------- kernel launchers ---
// Every launcher enqueues on `st` and returns the launch status.

// First valid (non-NaN) index of each time-major series; rows if all NaN.
vta_status launch_first_valid_tm(const float* x_tm, int cols, int rows, int* first, cudaStream_t st);
// Same over the three HLC inputs (first index where all three are non-NaN).
vta_status launch_first_valid_tm_hlc(const float* h, const float* l, const float* c, int cols,
                                     int rows, int* first, cudaStream_t st);

// Inclusive f64 prefix of f(x[i]) for i >= first (0 before first), with
// f selected by `kind`; optionally packed to double-single float2.
enum PrefixKind { PK_X = 0, PK_X2 = 1, PK_GAIN = 2, PK_LOSS = 3, PK_NAN = 4 };
vta_status launch_prefix_f64(const float* x, int n, int first, int kind, double* out_f64,
                             float2* out_ds, double* block_tmp, cudaStream_t st);
size_t prefix_tmp_doubles(int n);
// out[c][r] = in[r][c] for a [rows][cols] f32 matrix.
vta_status launch_transpose(const float* in, int rows, int cols, float* out, cudaStream_t st);

// --- weighted-window moving averages (ALMA/WMA/SWMA/PWMA/SINWMA/TRIMA,
// CWMA/FWMA/SRWMA/SQWMA/EPMA/VPWMA) ----------------------------------------
// Row weights are right-aligned into a [n_combos][kmax] f32 matrix.  A row's
// "period" here is its window length L; its first output is at
// first + L - 1 + warm_extra (the crate's warm-up of each indicator).
struct WwmaBatchArgs {
    const float* x;        // series (device)
    int n;                 // series length
    int first;             // first valid index
    const float* w;        // [n_combos][kmax] normalised weights, right-aligned
    const int* periods;    // [n_combos]
    const int* periods_host;  // [n_combos] host copy (tile sizing)
    const int* tile_kmax;  // per 16-combo tile: max period (K of the tile)
    int kmax;
    int n_combos;
    int nan_mode;          // 0: window NaN -> NaN; 1: NaN poisons all later outputs
    const double* nanp;    // [n] count of NaN in x[first..i] (null: series has none)
    const int* warm_extra; // [n_combos] extra warm-up steps (device; null: 0)
    float* out;            // [n_combos][n]
};
enum WeightKind {
    WT_ALMA = 0, WT_WMA = 1, WT_SWMA = 2, WT_PWMA = 3, WT_SINWMA = 4, WT_TRIMA = 5,
    WT_CWMA = 6, WT_FWMA = 7, WT_SRWMA = 8, WT_SQWMA = 9, WT_EPMA = 10, WT_VPWMA = 11
};
vta_status launch_weights(int kind, const int* periods, const double* pa, const double* pb, int n_combos,
                          int kmax, float* w, cudaStream_t st);
vta_status launch_wwma_batch_plain(const WwmaBatchArgs& a, cudaStream_t st);
// tcgen05 split-precision contraction; returns VTA_ERR_NOT_IMPLEMENTED when
// the shape is unsupported (caller falls back to the plain kernel).
vta_status launch_wwma_batch_tc(const WwmaBatchArgs& a, int variant, vta_ctx* ctx,
                                cudaStream_t st);

struct WwmaTmArgs {
    const float* x_tm;
    int cols, rows;
    const int* first;      // per-series first valid
    const float* w;        // [period] normalised weights
    int period;            // window length
    int warm_extra;        // first output of series s at first[s] + period - 1 + warm_extra
    int nan_mode;
    float* out_tm;
};
vta_status launch_wwma_tm(const WwmaTmArgs& a, cudaStream_t st);

// ------------------------------------------------- chunked recurrences -----
enum RecurKind { RK_EMA = 0, RK_DEMA = 1, RK_TEMA = 2, RK_RSI = 3, RK_WILDERS = 4, RK_ATR = 5 };

// Shape of the tensor-core chunk-aggregate contraction (k_recur_tc.cu):
// weight rows (component, lane) x columns (chunk; RSI: gains | losses), K
// split S ways; byte offsets of the pieces in the weight and work buffers.
struct RecurTcGeo {
    int nsr;               // weight rows per lane: 1 (EMA, RSI), 2 (DEMA), 3 (TEMA)
    int mpad;              // lanes rounded up to 128
    int rows;              // nsr * mpad
    int ncol;              // columns: nc (RSI: 2 nc)
    int npad;              // ncol rounded up to 128
    int S;                 // K splits
    size_t w_bytes, row_scale_off, row_sum_off;
    size_t ws_bytes, col_scale_off, col_ref_off, part_off;
};
// What the AGG pass reads of a finished contraction: for a chunk c in
// [g0, g0 + nc) with done[c] and *err == 0, component q of lane li is
//   (sum over s < S of part[s][j][r]) * row_scale[r] * col_scale[j] + col_ref[j] * row_sum[r]
// with r = q mpad + li, j = c - g0 (RSI: component 1 at j + nc, r = li).
struct RecurTcView {
    const int* done;
    const int* err;
    int g0, nc;
    const float* part;     // [S][npad][rows]
    int S, npad, rows, mpad;
    const float* row_scale;
    const float* row_sum;
    const float* col_scale;
    const float* col_ref;
};

struct RecurArgs {
    int kind;
    int layout;            // 0 = batch (one series, lane = combo), 1 = time-major
    // inputs: batch -> x[n] (or h,l,c); tm -> x_tm[t*cols+s]
    const float* x;
    const float* h;
    const float* l;
    const float* c;
    int n;                 // series length (batch) / rows (tm)
    int cols;              // tm: number of series
    int first;             // batch: first valid index
    const int* first_tm;   // tm: per-series first valid
    const int* periods;    // batch: per combo period; tm: null
    int period;            // tm: the single period
    int n_lanes;           // batch: n_combos; tm: cols
    // f64 prefixes for seeds (batch): EMA/Wilders: x; RSI: gains, losses
    const double* p0;
    const double* p1;
    int chunk;             // time chunk length (multiple of 32)
    int chunk0;            // length of chunk 0 (multiple of 32; 0 = chunk); later chunks are `chunk` long
    // batch EMA/DEMA/TEMA/RSI with fast_agg != 0: chunks >= fast_from start
    // with every lane past its seed, and their AGG blocks take the scaled
    // one-FMA-per-component path unless the chunk holds a non-finite input
    int fast_from;
    int fast_agg;
    float* out;            // batch [n_combos][n]; tm [n][cols]
    // scratch
    float* agg;            // [n_chunks][n_lanes] float4 (state, applied steps)
    float* carry;          // [n_chunks][n_lanes] float4 (carry-in state)
    // tensor-core partial sums of the full chunks (k_recur_tc.cu); done ==
    // null: none
    RecurTcView tc;
};
vta_status launch_recurrence(const RecurArgs& a, cudaStream_t st);

// Chunk aggregates of a batch EMA / DEMA / TEMA / RSI sweep as one
// split-precision tcgen05 contraction over the full-length chunks
// [g0, g0 + nc) (k_recur_tc.cu).
struct RecurTcArgs {
    int kind;              // RK_EMA, RK_DEMA, RK_TEMA or RK_RSI
    const float* x;        // the series
    const int* periods;    // per lane
    int n_lanes;
    int L;                 // chunk length (multiple of 32)
    int chunk0;            // length of chunk 0: chunk c >= 1 starts at chunk0 + (c - 1) L
    int g0, nc;            // g0 >= 1; every chunk of the range is L long
    RecurTcGeo geo;        // recur_agg_tc_geo(kind, n_lanes, L, nc, SMs)
    void* wts;             // geo.w_bytes: packed weights (a function of kind, periods, L)
    int build_weights;     // 0: wts already holds this sweep's weights
    void* ws;              // geo.ws_bytes: packed inputs, column scales, partial sums
    int* done;             // [n_chunks]: 1 = the chunk's inputs are finite (partials valid)
    int* err;              // raised on a pipeline wait timeout (partials then unusable)
};
RecurTcGeo recur_agg_tc_geo(int kind, int n_lanes, int L, int nc, int num_sms);
size_t recur_agg_tc_smem();
vta_status launch_recur_agg_tc(const RecurTcArgs& a, size_t smem_optin, cudaStream_t st);
int recur_state_dim(int kind);
// Time range [c0, c1) of chunk k (chunk 0 is chunk0 long, the rest chunk).
__host__ __device__ inline void recur_chunk_bounds(const RecurArgs& a, int k, int& c0, int& c1) {
    const int f0 = a.chunk0 > 0 ? a.chunk0 : a.chunk;
    c0 = k == 0 ? 0 : f0 + (k - 1) * a.chunk;
    const int e = k == 0 ? f0 : c0 + a.chunk;
    c1 = e < a.n ? e : a.n;
}
inline int recur_n_chunks(int n, int chunk, int chunk0) {
    const int f0 = chunk0 > 0 ? chunk0 : chunk;
    return f0 >= n ? 1 : 1 + (n - f0 + chunk - 1) / chunk;
}

// ADX (two-level recurrence) and SuperTrend (state machine).
struct HlcArgs {
    int layout;
    const float* h;
    const float* l;
    const float* c;
    int n, cols, first;
    const int* first_tm;
    const int* periods;    // batch
    const float* factors;  // supertrend batch
    int period;
    float factor;
    int n_lanes;
    float* out0;           // adx / trend
    float* out1;           // changed
};
vta_status launch_adx(const HlcArgs& a, cudaStream_t st);
// Batch ADX (kind 0) / SuperTrend (kind 1) cut into time chunks with verified
// warm restarts (k_hlc_chunk.cu); bit-identical to the sequential kernels.
struct HlcChunkArgs {
    int kind;
    const float* h;
    const float* l;
    const float* c;
    int n, first;
    const int* periods;
    const float* factors;   // supertrend
    int n_combos;
    const int2* items;      // {32-combo group, chunk}
    int n_items;
    const int* group_chunk; // chunk length per group (n: one chunk)
    const int* group_warm;  // warm-restart steps per group (multiple of 32)
    float* out0;
    float* out1;
    float* st_start;        // [max chunks][n_combos][8]
    float* st_end;
    unsigned char* exact;   // [max chunks][n_combos]
    int* fixups;
    int* need;              // [n_combos] mismatches found (zeroed before the launch)
    int max_chunks;
};
vta_status launch_hlc_chunk(const HlcChunkArgs& a, cudaStream_t st);
// Exact chunked scan of batch ADX for 32-combo groups with long periods
// (k_adx_scan.cu).  Group gi (combos groups[gi] * 32 ..) is seeded by
// k_hlc_chunk's exact chunk-0 item over [0, group_s0[gi]); its chunks k >= 1
// start at group_s0[gi] + (k - 1) L.  State slots: [chunk][n_slots], slot =
// gi * 32 + lane.
struct AdxScanArgs {
    const float* h;
    const float* l;
    const float* c;
    int n;
    const int* periods;
    int n_combos;
    const int* groups;      // [n_groups] 32-combo group ids
    const int* group_s0;    // [n_groups] start of chunk 1 (multiple of 32, past every lane's seeding)
    int n_groups;
    int n_slots;            // n_groups * 32
    int L;                  // chunk length, multiple of 32
    const int2* items;      // {group index, chunk >= 1}
    int n_items;
    const float* seed_state;  // [n_combos][8]: the chunk-0 end state (atr, +DM, -DM, adx)
    float4* agg1;
    float* agg2;
    float4* carry1;
    float* carry2;
    float* out;             // [n_combos][n]
};
vta_status launch_adx_scan(const AdxScanArgs& a, cudaStream_t st);
vta_status launch_supertrend(const HlcArgs& a, cudaStream_t st);

// ------------------------------------------------- prefix-sum windows ------
enum WinKind { WK_SMA = 0, WK_STDDEV = 1, WK_ZSCORE = 2, WK_BB = 3 };
struct PrefixWinArgs {
    int kind;
    const float* x;
    // int[2] scratch: the first NaN / infinite input at or after `first`,
    // filled by launch_prefix_window_batch
    int* bad;
    int n, first;
    const int* periods;
    const float* k1;       // stddev/zscore nbdev; bb devup
    const float* k2;       // bb devdn
    int n_combos;
    float* out0;           // sma/stddev/zscore/bb upper
    float* out1;           // bb middle
    float* out2;           // bb lower
};
vta_status launch_prefix_window_batch(const PrefixWinArgs& a, int pmax, size_t smem_optin, cudaStream_t st);

struct PrefixWinTmArgs {
    int kind;
    const float* x_tm;
    int cols, rows;
    const int* first;
    int period;
    float k1, k2;
    float* out0;
    float* out1;
    float* out2;
};
vta_status launch_prefix_window_tm(const PrefixWinTmArgs& a, cudaStream_t st);

// ------------------------------------------------- min/max windows ---------
enum MinMaxKind { MM_DONCHIAN = 0, MM_WILLR = 1 };
struct MinMaxArgs {
    int kind;
    const float* h;
    const float* l;
    const float* c;        // willr only
    int n, first;
    const int* periods;
    int n_combos;
    int pmax;
    float* out0;           // donchian upper / willr
    float* out1;           // donchian middle
    float* out2;           // donchian lower
    int tile_hint;         // output times per block (0 = the launcher's choice)
    // periods[c] = periods[0] + c * ap_d for every combo (an ascending
    // arithmetic progression, 1 <= ap_d <= 64); 0 = not known to be one
    int ap_d;
    int skip_clean;        // (set by the launcher) leave clean tiles to the progression kernel
    int* dirty;            // scratch, one int per 1024-bar tile: the tiles the progression kernel left
};
vta_status launch_minmax_batch(const MinMaxArgs& a, size_t smem_optin, cudaStream_t st);
// Tiles launch_minmax_batch can run for `a` (the autotuner's candidates;
// empty when only the launcher's own choice applies).
std::vector<int> minmax_tile_candidates(const MinMaxArgs& a, size_t smem_optin);
// Whether launch_minmax_batch runs the progression kernel for `a` (as hinted).
bool minmax_uses_progression(const MinMaxArgs& a, size_t smem_optin);

struct MinMaxTmArgs {
    int kind;
    const float* h;
    const float* l;
    const float* c;
    int cols, rows;
    const int* first;
    int period;
    float* out0;
    float* out1;
    float* out2;
};
vta_status launch_minmax_tm(const MinMaxTmArgs& a, cudaStream_t st);

// ------------------------------------------------- nearest-rank percentile -
struct PnrArgs {
    int layout;
    const float* x;
    int n, cols, first;
    const int* first_tm;
    const int* lengths;     // batch per combo
    const float* pfrac;     // batch per combo (percentage * 0.01)
    int length;             // tm
    float p_frac;           // tm
    int n_lanes;
    float* out;
    float* scratch;         // batch: per-thread sorted windows
    size_t scratch_floats;
};
vta_status launch_percentile(const PnrArgs& a, cudaStream_t st);

// One ATR (0) / ADX (1) / SuperTrend (2) / percentile (3) job of the plan
// kernels over a rectangular time-major matrix, enqueued on st (vta_plan.cu).
vta_status tm_job_enqueue(vta_ctx* ctx, int kind, int period, double param, const float* h, const float* l,
                          const float* c, int cols, int rows, float* out0, float* out1, cudaStream_t st);

// ------------------------------------------------- request server ---------
int ind_by_name(const char* name);  // -1 if unknown
int ind_inputs(int ind);            // 1: close, 2: high, low, 3: high, low, close
int ind_outputs(int ind);
double ind_cost(int ind);           // device time per output relative to an HBM-bound sweep
size_t ind_first(int ind, size_t fh, size_t fl, size_t fc, size_t fall);
// grid expansion + the crate's checks for a series of len with first valid `first`
vta_status batch_check(int ind, const vta_sweep* sw, size_t len, size_t first, size_t* rows);
// the same plus the kernels of the sweep enqueued on ctx's stream (no wait)
vta_status batch_enqueue(vta_ctx* ctx, int ind, const float* const* d_in, size_t len, size_t first,
                         const vta_sweep* sw, float* const* d_out);

// ------------------------------------------------- no-allocation SMA -------
// Binds a call to `ctx` (device current, timing events), as every entry does.
vta_status enter_call(vta_ctx* ctx);
// The allocating SMA entry points' parameter and length checks, same messages.
size_t sma_period_count(vta_range_usize r);
size_t sma_period_at(vta_range_usize r, size_t k);
vta_status validate_sma_range(vta_range_usize r, size_t n, size_t len, size_t first);

}  // namespace vta
