"""Generates the C ABI of the library from one table of indicators:

* include/vta_gb300.h                      -- the public declarations;
* vectorta_gb300/csrc/vta_abi_gen.inc      -- the extern "C" definitions that
  forward each entry point to the generic drivers in vta_api.cu.

Run from the repository root after changing the table:
    python vectorta_gb300/csrc/gen_abi.py
"""
IND = [
 # name, wrapper file, input kind, outputs, range type, params type, cites (new, batch_dev, batch_device, into_host, tm_dev, tm_device)
 ("alma","src/cuda/moving_averages/alma_wrapper.rs","x",["out"],"alma","alma",(133,625,671,783,819,1521)),
 ("ema","src/cuda/moving_averages/ema_wrapper.rs","x",["out"],"period","period",(125,193,256,309,325,381)),
 ("dema","src/cuda/moving_averages/dema_wrapper.rs","x",["out"],"period","period",(115,219,305,379,516,554)),
 ("tema","src/cuda/moving_averages/tema_wrapper.rs","x",["out"],"period","period",(159,336,367,345,430,397)),
 ("rsi","src/cuda/rsi_wrapper.rs","x",["out"],"period","period",(62,152,None,None,271,None)),
 ("wilders","src/cuda/moving_averages/wilders_wrapper.rs","x",["out"],"period","period",(101,134,252,None,600,662)),
 ("sma","src/cuda/moving_averages/sma_wrapper.rs","x",["out"],"period","period",(56,548,830,558,750,982)),
 ("wma","src/cuda/moving_averages/wma_wrapper.rs","x",["out"],"period","period",(151,713,747,723,1014,1049)),
 ("swma","src/cuda/moving_averages/swma_wrapper.rs","x",["out"],"period","period",(121,678,663,None,825,787)),
 ("pwma","src/cuda/moving_averages/pwma_wrapper.rs","x",["out"],"period","period",(93,385,369,None,723,696)),
 ("sinwma","src/cuda/moving_averages/sinwma_wrapper.rs","x",["out"],"period","period",(116,609,643,619,841,873)),
 ("trima","src/cuda/moving_averages/trima_wrapper.rs","x",["out"],"period","period",(123,722,707,None,855,829)),
 ("stddev","src/cuda/stddev_wrapper.rs","x",["out"],"stddev","stddev",(101,509,None,606,630,None)),
 ("zscore","src/cuda/zscore_wrapper.rs","x",["out"],"zscore","zscore",(86,620,None,663,720,None)),
 ("bollinger_bands","src/cuda/bollinger_bands_wrapper.rs","x",["out_upper","out_middle","out_lower"],"bollinger","bollinger",(85,567,None,None,605,None)),
 ("atr","src/cuda/atr_wrapper.rs","hlc",["out"],"period","period",(110,270,626,None,834,None)),
 ("adx","src/cuda/adx_wrapper.rs","hlc",["out"],"period","period",(88,199,None,253,340,None)),
 ("supertrend","src/cuda/supertrend_wrapper.rs","hlc",["out_trend","out_changed"],"supertrend","supertrend",(88,179,None,None,337,None)),
 ("donchian","src/cuda/donchian_wrapper.rs","hl",["out_upper","out_middle","out_lower"],"period","period",(128,344,None,None,593,None)),
 ("willr","src/cuda/willr_wrapper.rs","hlc",["out"],"period","period",(75,132,236,None,583,642)),
 ("percentile_nearest_rank","src/cuda/percentile_nearest_rank_wrapper.rs","x",["out"],"percentile","percentile",(99,365,None,None,623,None)),
 ("cwma","src/cuda/moving_averages/cwma_wrapper.rs","x",["out"],"period","period",(118,767,737,850,1208,1180)),
 ("fwma","src/cuda/moving_averages/fwma_wrapper.rs","x",["out"],"period","period",(132,491,475,None,760,734)),
 ("srwma","src/cuda/moving_averages/srwma_wrapper.rs","x",["out"],"period","period",(176,328,420,None,485,572)),
 ("sqwma","src/cuda/moving_averages/sqwma_wrapper.rs","x",["out"],"period","period",(62,157,190,166,255,222)),
 ("epma","src/cuda/moving_averages/epma_wrapper.rs","x",["out"],"epma","epma",(110,485,574,495,773,805)),
 ("vpwma","src/cuda/moving_averages/vpwma_wrapper.rs","x",["out"],"vpwma","vpwma",(126,720,751,730,851,823)),
]
RANGES = {
 "alma": ("vta_alma_batch_range", "vta_alma_params"),
 "period": ("vta_period_batch_range", "vta_period_params"),
 "stddev": ("vta_stddev_batch_range", "vta_stddev_params"),
 "zscore": ("vta_zscore_batch_range", "vta_zscore_params"),
 "bollinger": ("vta_bollinger_batch_range", "vta_bollinger_params"),
 "supertrend": ("vta_supertrend_batch_range", "vta_supertrend_params"),
 "percentile": ("vta_percentile_batch_range", "vta_percentile_params"),
 "epma": ("vta_epma_batch_range", "vta_epma_params"),
 "vpwma": ("vta_vpwma_batch_range", "vta_vpwma_params"),
}
def inputs(kind, dev, tm):
    pre = "d_" if dev else ""
    suf = "_tm" if tm else ""
    if kind == "x": return [f"const float* {pre}data{suf}"]
    if kind == "hl": return [f"const float* {pre}high{suf}", f"const float* {pre}low{suf}"]
    return [f"const float* {pre}high{suf}", f"const float* {pre}low{suf}", f"const float* {pre}close{suf}"]

out = []
w = out.append
w("""/*
 * vta_gb300.h -- C ABI of the GB300-native VectorTA indicator hot path.
 *
 * One shared library (libvta_gb300.so) replaces the crate's per-indicator CUDA
 * wrappers (the src/cuda X_wrapper.rs files: `CudaX` structs driving PTX through
 * `cust`).  Every entry point is plain C: host or device pointers, sizes and
 * small parameter structs; no CUDA, torch or Rust types cross the boundary.
 *
 * Conventions (the crate's, kept so existing callers port one-to-one):
 *   - batch ("one series, many params"): output is row-major
 *     [n_combos][len], rows in the crate's expand_grid order (period-major);
 *   - many-series ("time-major"): input and output are [rows][cols] with
 *     element (t, s) at t*cols + s; one parameter set for all series;
 *   - warm-up cells are quiet NaN at exactly the crate's positions;
 *   - *_dev functions take host inputs and return device arrays owned by the
 *     caller (free with vta_device_array_free); *_device functions take device
 *     inputs and write into caller-provided device outputs (the crate's
 *     x_batch_device / x_many_series_one_param_device); *_into_host_f32
 *     writes host outputs (the crate's x_batch_into_host_f32);
 *   - every call is stream-ordered on the context's stream and synchronous on
 *     return, like the crate's wrappers (which end with stream.synchronize()).
 * Thread safety: a vta_ctx is used by one thread at a time (as a CudaX is).
 */
#ifndef VTA_GB300_H
#define VTA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes map the crate's CudaXError variants one-to-one
 * (src/cuda/moving_averages/alma_wrapper.rs:72-101). */
typedef enum vta_status {
    VTA_OK = 0,
    VTA_ERR_CUDA = 1,                   /* Cuda(CudaError) */
    VTA_ERR_OUT_OF_MEMORY = 2,          /* OutOfMemory{required, free, headroom} */
    VTA_ERR_MISSING_KERNEL_SYMBOL = 3,  /* MissingKernelSymbol{name} */
    VTA_ERR_INVALID_INPUT = 4,          /* InvalidInput(String) */
    VTA_ERR_INVALID_POLICY = 5,         /* InvalidPolicy(&str) */
    VTA_ERR_LAUNCH_CONFIG_TOO_LARGE = 6,/* LaunchConfigTooLarge{grid, block} */
    VTA_ERR_DEVICE_MISMATCH = 7,        /* DeviceMismatch{buf, current} */
    VTA_ERR_NOT_IMPLEMENTED = 8         /* NotImplemented */
} vta_status;

/* Message of the last failure on the calling thread (the Display text of the
 * crate's error enums). */
const char* vta_last_error(void);
const char* vta_version(void);

/* Number of CUDA devices (crate: cuda_device_count, src/cuda/mod.rs:560-575);
 * 0 when no driver or device is present. */
int vta_device_count(void);

/* ---- context: CudaX::new(device_id) (alma_wrapper.rs:133-169) ---------- */
typedef struct vta_ctx vta_ctx;
vta_status vta_ctx_create(int device_id, vta_ctx** out);
vta_status vta_ctx_destroy(vta_ctx* ctx);
/* CudaX::synchronize (alma_wrapper.rs:171-173). */
vta_status vta_ctx_synchronize(vta_ctx* ctx);
/* Run on a caller-owned cudaStream_t instead of the context's own stream
 * (NULL restores the context stream). */
vta_status vta_ctx_set_stream(vta_ctx* ctx, void* cuda_stream);
void* vta_ctx_get_stream(vta_ctx* ctx);
/* CudaXPolicy / set_policy (alma_wrapper.rs:18-70): keys
 *   "wma_batch"   = "auto" | "plain" | "tc_fp16x3" | "tc_bf16x3"
 *   "recur_chunk" = "auto" | "sequential" | <positive multiple of 32>
 *   "tm_chunk"    = "auto" | "sequential" | <steps>   (many-series plans)
 *   "tm_warm"     = "auto" | <steps>   (plans; chunked ADX/SuperTrend sweeps)
 *   "timing"      = "on" | "off"
 *   "host_io"     = "cached" | "per_call": *_batch_into_host_f32 keeps its
 *                   device input/output buffer in the context between calls
 *                   (cached, the default; freed by per_call or ctx destroy) */
vta_status vta_ctx_set_policy(vta_ctx* ctx, const char* key, const char* value);
/* selected_batch_kernel() (alma_wrapper.rs:239-245): name of the last kernel
 * path used by this context. */
const char* vta_ctx_last_kernel(vta_ctx* ctx);
/* Device workspace currently held by the context (bytes). */
size_t vta_ctx_scratch_bytes(vta_ctx* ctx);
/* With policy "timing" = "on", each call records CUDA events on the context
 * stream around its main output kernel; this returns that kernel's duration
 * in ms for the last call (-1 when not recorded). */
float vta_ctx_kernel_ms(vta_ctx* ctx);
/* Number of kernels this library has launched in the process. */
uint64_t vta_launch_count(void);

/* ---- device arrays: DeviceArrayF32 (alma_wrapper.rs:103-117) ----------- */
typedef struct vta_device_array {
    float* ptr;     /* device pointer, rows*cols floats, owned */
    size_t rows;
    size_t cols;
    int device;
} vta_device_array;
vta_status vta_device_array_free(vta_device_array* arr);
vta_status vta_device_array_copy_to_host(vta_ctx* ctx, const vta_device_array* arr,
                                         float* host, size_t n);
/* DeviceArrayF32Py::__dlpack__ (src/utilities/dlpack_cuda.rs:265-374): moves
 * arr's buffer into a new DLPack managed tensor (2-D f32, kDLCUDA, row-major
 * strides in elements) and empties arr.  versioned != 0 gives a
 * DLManagedTensorVersioned (DLPack 1.0, for a "dltensor_versioned" capsule),
 * else a DLManagedTensor ("dltensor").  Its deleter frees the buffer on the
 * array's device; vta_dlpack_delete calls it for a tensor nobody consumed. */
vta_status vta_device_array_to_dlpack(vta_device_array* arr, int versioned, void** out_managed);
vta_status vta_dlpack_delete(void* managed, int versioned);

/* ---- MA computer: VramMaComputer (src/cuda/moving_averages/vram_ma.rs) -- */
/* supports_vram_kernel_ma (vram_ma.rs:68-76), for the MAs this library has
 * kernels for: sma ema wma alma dema tema swma trima sinwma epma wilders cwma
 * fwma pwma srwma sqwma vpwma (trimmed, case-insensitive); 1 if supported. */
int vta_ma_supported(const char* ma_type);
/* compute_period_ma_into (vram_ma.rs:574) / compute_period_ma_tm_into (:2153):
 * one MA over a device-resident series for an arbitrary list of periods.
 * Optional parameters as key/value pairs like the crate's HashMap (ALMA
 * "offset" (0.85) and "sigma" (6.0); EPMA "offset" (0, rounded); VPWMA
 * "power" (0.382); missing or non-finite values take the default).  d_out holds n_periods x len floats:
 * [period][t] when time_major == 0, else [t][period].  The other names the
 * crate's computer serves (jsa, smma, hma, ...) give VTA_ERR_NOT_IMPLEMENTED. */
vta_status vta_ma_periods_device(vta_ctx* ctx, const char* ma_type, const char* const* param_keys,
    const double* param_values, size_t n_params, const float* d_prices, size_t len, size_t first_valid,
    const int* periods, size_t n_periods, int time_major, float* d_out);
/* CudaMaSelector (src/cuda/moving_averages/ma_selector.rs): the same dispatch
 * from host prices.  ma_to_device / ma_sweep_to_device (ma_selector.rs:935,
 * 1712): period_start == period_end (or step 0) is the single-period call;
 * otherwise the selector's own range rule (ma_selector.rs:1037-1061).  out:
 * rows = periods, cols = len, owned by the caller (vta_device_array_free). */
vta_status vta_ma_select_dev(vta_ctx* ctx, const char* ma_type, const char* const* param_keys,
    const double* param_values, size_t n_params, const float* prices, size_t len, size_t period_start,
    size_t period_end, size_t period_step, vta_device_array* out);
/* ma_to_host_f32 / ma_sweep_to_host_f32 (ma_selector.rs:954, 1735). */
vta_status vta_ma_select_into_host_f32(vta_ctx* ctx, const char* ma_type, const char* const* param_keys,
    const double* param_values, size_t n_params, const float* prices, size_t len, size_t period_start,
    size_t period_end, size_t period_step, float* out, size_t out_len, size_t* rows, size_t* cols);

/* ---- streaming: banks of the crate's XStream structs ----------------- */
/* n_streams independent streams of one indicator and parameter set on the
 * device, advanced together by one bar per update, each bar for bar as the
 * crate's XStream::update (EmaStream ema.rs:519-585, SmaStream sma.rs,
 * AlmaStream alma.rs:865-964, RsiStream rsi.rs, AtrStream atr.rs,
 * WildersStream wilders.rs, DemaStream dema.rs:615-690, TemaStream
 * tema.rs:324-425, WmaStream wma.rs:384-460, SwmaStream swma.rs:536-630,
 * PwmaStream pwma.rs:675-720, StdDevStream stddev.rs:451-570, ZscoreStream
 * zscore.rs:567-780, BollingerBandsStream bollinger_bands.rs:884-1075,
 * DonchianStream donchian.rs:1251-1340, WillrStream willr.rs:1657-1820,
 * AdxStream adx.rs:1949-2085, SuperTrendStream supertrend.rs:798-885,
 * SinWmaStream sinwma.rs:586-750, TrimaStream trima.rs:826-905, CwmaStream
 * cwma.rs:792-1040, FwmaStream fwma.rs:750-890, SrwmaStream
 * srwma.rs:1183-1290, SqwmaStream sqwma.rs:360-545, EpmaStream
 * epma.rs:635-735, VpwmaStream vpwma.rs:583-884,
 * PercentileNearestRankStream percentile_nearest_rank.rs:468-700), f64
 * state, f32 in and out; outputs are NaN where update() returns None.
 * indicator: "ema" "sma" "alma" "rsi" "atr" "wilders" "dema" "tema" "wma"
 * "swma" "pwma" "stddev" "zscore" "bollinger_bands" "donchian" "willr" "adx"
 * "supertrend" "sinwma" "trima" "cwma" "fwma" "srwma" "sqwma" "epma" "vpwma"
 * "percentile_nearest_rank".  Parameters as key/value pairs, the crate's
 * defaults when absent: "period" (ATR and percentile also "length"), ALMA
 * "offset" / "sigma", StdDev and Z-score "nbdev", Bollinger "devup" /
 * "devdn" / "matype" (0 sma, 1 ema), SuperTrend "factor", EPMA "offset",
 * VPWMA "power", percentile "percentage"; Z-score takes ma_type sma,
 * Bollinger and Z-score devtype 0 (others: VTA_ERR_NOT_IMPLEMENTED).
 * Inputs: one series in a (b, c NULL); Donchian (high, low) in (a, b); ATR,
 * WillR, ADX, SuperTrend (high, low, close).  Outputs: out holds n_outputs
 * rows of n_streams values: Bollinger and Donchian upper / middle / lower,
 * SuperTrend trend / changed. */
typedef struct vta_streams vta_streams;
vta_status vta_streams_create(vta_ctx* ctx, const char* indicator, const char* const* param_keys,
    const double* param_values, size_t n_params, size_t n_streams, vta_streams** out);
vta_status vta_streams_shape(const vta_streams* s, int* n_inputs, int* n_outputs);
vta_status vta_streams_update_device(vta_streams* s, const float* d_a, const float* d_b, const float* d_c,
    float* d_out);
vta_status vta_streams_update_host(vta_streams* s, const float* a, const float* b, const float* c, float* out);
vta_status vta_streams_reset(vta_streams* s);
vta_status vta_streams_destroy(vta_streams* s);

/* Page-locked host buffers for fast copies (the crate's LockedBuffer,
 * alma_wrapper.rs:810-815). */
vta_status vta_pinned_alloc(size_t bytes, void** out);
vta_status vta_pinned_free(void* p);
/* Plain device buffers for callers without their own allocator. */
vta_status vta_device_alloc(vta_ctx* ctx, size_t bytes, void** out);
vta_status vta_device_free(vta_ctx* ctx, void* p);
vta_status vta_memcpy_h2d(vta_ctx* ctx, void* dst, const void* src, size_t bytes);
vta_status vta_memcpy_d2h(vta_ctx* ctx, void* dst, const void* src, size_t bytes);

/* ---- parameter sweeps: (start, end, step) like the crate's BatchRange --- */
typedef struct vta_range_usize { size_t start, end, step; } vta_range_usize;
typedef struct vta_range_f64 { double start, end, step; } vta_range_f64;

/* AlmaBatchRange / AlmaParams (alma.rs:66-80, 1068-1082) */
typedef struct vta_alma_batch_range { vta_range_usize period; vta_range_f64 offset, sigma; } vta_alma_batch_range;
typedef struct vta_alma_params { size_t period; double offset, sigma; } vta_alma_params;
/* period-only sweeps: EMA, DEMA, TEMA, RSI, Wilders, SMA, WMA, SWMA, PWMA,
 * SINWMA, TRIMA, ATR (`length`), ADX, Donchian, WillR, CWMA, FWMA, SRWMA,
 * SQWMA */
typedef struct vta_period_batch_range { vta_range_usize period; } vta_period_batch_range;
typedef struct vta_period_params { size_t period; } vta_period_params;
/* StdDevBatchRange (stddev.rs:573-585) */
typedef struct vta_stddev_batch_range { vta_range_usize period; vta_range_f64 nbdev; } vta_stddev_batch_range;
typedef struct vta_stddev_params { size_t period; double nbdev; } vta_stddev_params;
/* ZscoreBatchRange (zscore.rs:786-802), ma_type "sma" and devtype 0 */
typedef struct vta_zscore_batch_range { vta_range_usize period; vta_range_f64 nbdev; } vta_zscore_batch_range;
typedef struct vta_zscore_params { size_t period; double nbdev; } vta_zscore_params;
/* BollingerBandsBatchRange (bollinger_bands.rs:1087-1104), matype "sma", devtype 0 */
typedef struct vta_bollinger_batch_range { vta_range_usize period; vta_range_f64 devup, devdn; } vta_bollinger_batch_range;
typedef struct vta_bollinger_params { size_t period; double devup, devdn; } vta_bollinger_params;
/* SuperTrendBatchRange (supertrend.rs:1223-1300) */
typedef struct vta_supertrend_batch_range { vta_range_usize period; vta_range_f64 factor; } vta_supertrend_batch_range;
typedef struct vta_supertrend_params { size_t period; double factor; } vta_supertrend_params;
/* PercentileNearestRankBatchRange (percentile_nearest_rank.rs:815-827) */
typedef struct vta_percentile_batch_range { vta_range_usize length; vta_range_f64 percentage; } vta_percentile_batch_range;
typedef struct vta_percentile_params { size_t length; double percentage; } vta_percentile_params;
/* EpmaBatchRange / EpmaParams (epma.rs:750-753; offset < period) */
typedef struct vta_epma_batch_range { vta_range_usize period, offset; } vta_epma_batch_range;
typedef struct vta_epma_params { size_t period, offset; } vta_epma_params;
/* VpwmaBatchRange / VpwmaParams (vpwma.rs:887-899; power finite) */
typedef struct vta_vpwma_batch_range { vta_range_usize period; vta_range_f64 power; } vta_vpwma_batch_range;
typedef struct vta_vpwma_params { size_t period; double power; } vta_vpwma_params;
""")
for (name, wf, kind, outs, rng, prm, cites) in IND:
    R, P = RANGES[rng]
    c_new, c_bd, c_bdev, c_ih, c_tm, c_tmd = cites
    wn = wf.split("/")[-1]
    w(f"/* ==== {name} ({wf}) ==== */")
    w(f"/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */")
    w(f"vta_status vta_{name}_expand_grid(const {R}* sweep, {P}* out, size_t cap, size_t* n_combos);")
    outs_dev = ", ".join(f"vta_device_array* {o}" for o in outs)
    w(f"/* {name}_batch_dev ({wn}:{c_bd}) */")
    w(f"vta_status vta_{name}_batch_dev(vta_ctx* ctx, {', '.join(inputs(kind, False, False))}, size_t len,\n    const {R}* sweep, {outs_dev});")
    cite = f"{wn}:{c_bdev}" if c_bdev else f"device-input form of {wn}:{c_bd}"
    outs_d = ", ".join(f"float* d_{o}" for o in outs)
    w(f"/* {name}_batch_device / _from_device_prices ({cite}); first_valid as in the crate. */")
    w(f"vta_status vta_{name}_batch_device(vta_ctx* ctx, {', '.join(inputs(kind, True, False))}, size_t len,\n    size_t first_valid, const {R}* sweep, {outs_d});")
    cite = f"{wn}:{c_ih}" if c_ih else f"host-output form of {wn}:{c_bd}"
    outs_h = ", ".join(f"float* {o}" for o in outs)
    w(f"/* {name}_batch_into_host_f32 ({cite}); each output holds out_len >= rows*cols floats. */")
    w(f"vta_status vta_{name}_batch_into_host_f32(vta_ctx* ctx, {', '.join(inputs(kind, False, False))}, size_t len,\n    const {R}* sweep, {outs_h}, size_t out_len, size_t* rows, size_t* cols);")
    w(f"/* {name}_many_series_one_param_time_major_dev ({wn}:{c_tm}) */")
    w(f"vta_status vta_{name}_many_series_one_param_time_major_dev(vta_ctx* ctx, {', '.join(inputs(kind, False, True))},\n    size_t cols, size_t rows, const {P}* params, {outs_dev});")
    cite = f"{wn}:{c_tmd}" if c_tmd else f"device-input form of {wn}:{c_tm}"
    w(f"/* {name}_many_series_one_param_device ({cite}) */")
    w(f"vta_status vta_{name}_many_series_one_param_device(vta_ctx* ctx, {', '.join(inputs(kind, True, True))},\n    size_t cols, size_t rows, const {P}* params, {outs_d});")
    w("")
w("""/* ==== many-series work-list plans ====
 * No counterpart in the crate, whose many-series entry points run one
 * indicator per call over a rectangular time-major matrix.  A plan runs
 * several indicators over one set of time-major OHLC series [rows][cols]
 * whose lengths differ: series s has lengths[s] <= rows valid rows (rows
 * past it are neither read nor written, in inputs and outputs alike).  All
 * jobs run in one persistent launch over a work list of (job, 32 series,
 * time chunk) items, captured once in a CUDA graph at creation and replayed
 * by vta_tm_plan_run.  The time-chunk length of each job is picked by timing
 * candidates on the plan's own data at creation (cached per indicator,
 * period, length and series count for the process); the context policies
 * "tm_chunk" and "tm_warm" override it.  Results are bit-identical to one
 * sequential pass per series (the chunking is verified and repaired on the
 * device), and per cell they follow the crate's many-series semantics:
 *   ATR    atr.rs:329-460             out0 = atr            (period = length)
 *   ADX    adx.rs:299-421             out0 = adx
 *   ST     supertrend.rs:457-550      out0 = trend, out1 = changed (param = factor)
 *   PNR    percentile_nearest_rank.rs:190-266 on close, out0 (period = length
 *          <= 64, param = percentage)
 * The input and output buffers are bound at creation; to run on new data,
 * write it into the same buffers and call vta_tm_plan_run again. */
typedef enum vta_tm_kind { VTA_TM_ATR = 0, VTA_TM_ADX = 1, VTA_TM_SUPERTREND = 2, VTA_TM_PERCENTILE = 3 } vta_tm_kind;
typedef struct vta_tm_job {
    int kind;          /* vta_tm_kind */
    size_t period;
    double param;      /* SuperTrend factor / percentile percentage; else 0 */
    float* d_out0;     /* [rows][cols] device */
    float* d_out1;     /* SuperTrend changed [rows][cols]; else NULL */
} vta_tm_job;
typedef struct vta_tm_plan vta_tm_plan;
typedef struct vta_tm_plan_info {
    size_t n_items;      /* work items of one run */
    size_t chunk[8];     /* time-chunk length per job (first 8 jobs) */
    size_t fixups;       /* chunks recomputed by the last run's verification */
    int tuned;           /* 1 if the chunk lengths were timed at creation */
} vta_tm_plan_info;
/* lengths: host array of cols series lengths, or NULL (every series has rows). */
vta_status vta_tm_plan_create(vta_ctx* ctx, const float* d_high, const float* d_low, const float* d_close,
    size_t cols, size_t rows, const size_t* lengths, const vta_tm_job* jobs, size_t n_jobs, vta_tm_plan** out);
/* Replays the plan's graph on the context stream; synchronous. */
vta_status vta_tm_plan_run(vta_tm_plan* plan);
vta_status vta_tm_plan_info_get(const vta_tm_plan* plan, vta_tm_plan_info* info);
vta_status vta_tm_plan_destroy(vta_tm_plan* plan);
""")
w("""/* ==== request server (continuous batching over a device-resident store) ====
 * No counterpart in the crate.  A server owns a store of series resident on
 * one device and a pool of slots (each a stream with its own workspace).
 * Requests -- one single-series parameter sweep of any batch indicator above
 * over one stored series -- are queued by vta_server_submit and admitted in
 * arrival order by a server thread as soon as a slot is free and their output
 * fits the memory budget; admitted requests run concurrently, each on its
 * slot's stream, with the same kernels and results as the corresponding
 * vta_X_batch_device call.  Completed requests are collected with
 * vta_server_poll; their device outputs stay valid until vta_server_release.
 * Times are seconds since the server was created. */
typedef struct vta_sweep {      /* generic sweep: the fields each indicator reads */
    vta_range_usize period;     /* period / length */
    vta_range_f64 p1;           /* alma offset, stddev/zscore nbdev, bb devup, supertrend factor, percentile %, epma offset, vpwma power */
    vta_range_f64 p2;           /* alma sigma, bb devdn */
} vta_sweep;
typedef struct vta_server_config {
    int slots;                  /* concurrent requests (streams); 0 = 8 */
    size_t memory_budget;       /* bytes of request outputs held at once; 0 = half the free memory */
} vta_server_config;
typedef struct vta_request {
    const char* indicator;      /* "alma", "ema", "rsi", "adx", "bollinger_bands", ... */
    uint32_t series;            /* id from vta_server_add_series */
    vta_sweep sweep;
} vta_request;
typedef struct vta_completion {
    uint64_t ticket;
    int status;                 /* vta_status of the request */
    size_t rows, cols;          /* combos x series length */
    int n_out;
    float* d_out[3];            /* device [rows][cols] outputs (valid until released) */
    double t_submit, t_start, t_done;
} vta_completion;
typedef struct vta_server_stats {
    uint64_t submitted, admitted, deferred, completed, failed;
    size_t queued, running, bytes_in_use, memory_budget;
} vta_server_stats;
typedef struct vta_server vta_server;
vta_status vta_server_create(int device_id, const vta_server_config* config, vta_server** out);
/* Copies a host series into the store (high/low may be NULL: close-only). */
vta_status vta_server_add_series(vta_server* s, const float* high, const float* low, const float* close,
    size_t len, uint32_t* id);
/* Same from device buffers (copied; the caller keeps its buffers). */
vta_status vta_server_add_series_device(vta_server* s, const float* d_high, const float* d_low,
    const float* d_close, size_t len, uint32_t* id);
/* Validates and queues a request; never waits for the device. */
vta_status vta_server_submit(vta_server* s, const vta_request* req, uint64_t* ticket);
/* Up to cap completed requests (waits up to wait_ms for at least one). */
vta_status vta_server_poll(vta_server* s, vta_completion* out, size_t cap, size_t* n, int wait_ms);
/* Copies output k of a completed, unreleased request to host memory. */
vta_status vta_server_copy_out(vta_server* s, uint64_t ticket, int k, float* host, size_t n_floats);
/* Frees a completed request's outputs (returns their bytes to the budget). */
vta_status vta_server_release(vta_server* s, uint64_t ticket);
vta_status vta_server_get_stats(vta_server* s, vta_server_stats* st);
/* Waits for running requests, then frees everything. */
vta_status vta_server_destroy(vta_server* s);
""")
w("""/* ==== sma without device allocation ====
 * No counterpart in the crate: its wrappers allocate device memory on every
 * call (sma_batch_dev_from_device, sma_wrapper.rs:830-841, allocates the
 * period list, the prefix and the output), and so do the other entry points
 * here.  vta_sma_batch_device_noalloc returns what vta_sma_batch_device
 * returns (same arguments, checks and errors) but never allocates device
 * memory: its working buffers live in one fixed scratch area of the library's
 * static device memory (VTA_NOALLOC_SCRATCH_BYTES, about 16 KiB per device,
 * reserved on a device when the function is first called there).
 * It is for callers that may not allocate once running: cudaMalloc and
 * cudaFree can synchronise the whole device and take unbounded time, which a
 * latency-bound loop (re-running a sweep on every new bar of a live feed)
 * cannot absorb, and a process whose own memory pool already holds the
 * device's free memory would see a mid-session allocation fail.
 *   - At most VTA_NOALLOC_MAX_LEN bars and VTA_NOALLOC_MAX_COMBOS periods;
 *     larger requests fail with VTA_ERR_INVALID_INPUT and a message naming
 *     the limit (vta_sma_batch_device has no such limit).
 *   - The first call on each device does one-time setup (it looks up the
 *     scratch address, which loads the library's device code there); make
 *     that first call before any stream capture on that device.
 *   - There is one scratch area per device per process.  Calls that overlap
 *     in time on the same device (from several host threads, whatever their
 *     contexts or streams) race on it and corrupt each other's results:
 *     serialise them.  Each call returns only when its work has finished, so
 *     consecutive calls from one thread never overlap.
 *   - Nothing in the scratch has to start at zero; each call writes every
 *     scratch cell it reads. */
#define VTA_NOALLOC_MAX_LEN 1048576
#define VTA_NOALLOC_MAX_COMBOS 4096
#define VTA_NOALLOC_SCRATCH_BYTES 16640
vta_status vta_sma_batch_device_noalloc(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
""")
w("""#ifdef __cplusplus
}
#endif

#endif /* VTA_GB300_H */""")
open("include/vta_gb300.h","w").write("\n".join(out)+"\n")

# ---------------------------------------------------------------- .inc ----
ENUM = {"alma":"I_ALMA","ema":"I_EMA","dema":"I_DEMA","tema":"I_TEMA","rsi":"I_RSI","wilders":"I_WILDERS",
        "sma":"I_SMA","wma":"I_WMA","swma":"I_SWMA","pwma":"I_PWMA","sinwma":"I_SINWMA","trima":"I_TRIMA",
        "stddev":"I_STDDEV","zscore":"I_ZSCORE","bollinger_bands":"I_BB","atr":"I_ATR","adx":"I_ADX",
        "supertrend":"I_SUPERTREND","donchian":"I_DONCHIAN","willr":"I_WILLR",
        "percentile_nearest_rank":"I_PNR","cwma":"I_CWMA","fwma":"I_FWMA","srwma":"I_SRWMA",
        "sqwma":"I_SQWMA","epma":"I_EPMA","vpwma":"I_VPWMA"}
def names(kind, dev, tm):
    return [a.split()[-1] for a in inputs(kind, dev, tm)]
inc = ["// Generated by gen_abi.py: extern \"C\" entry points forwarding to the drivers of",
       "// vta_api.cu (included inside its extern \"C\" block).  Do not edit by hand.", ""]
for (name, wf, kind, outs, rng, prm, cites) in IND:
    R, P = RANGES[rng]
    E = ENUM[name]
    ih = ", ".join(inputs(kind, False, False)); id_ = ", ".join(inputs(kind, True, False))
    ith = ", ".join(inputs(kind, False, True)); itd = ", ".join(inputs(kind, True, True))
    nh = ", ".join(names(kind, False, False)); nd = ", ".join(names(kind, True, False))
    nth = ", ".join(names(kind, False, True)); ntd = ", ".join(names(kind, True, True))
    oa = ", ".join(f"vta_device_array* {o}" for o in outs)
    od = ", ".join(f"float* d_{o}" for o in outs)
    oh = ", ".join(f"float* {o}" for o in outs)
    on = ", ".join(outs); odn = ", ".join(f"d_{o}" for o in outs)
    inc.append(f"vta_status vta_{name}_expand_grid(const {R}* sweep, {P}* out, size_t cap, size_t* n_combos) {{")
    inc.append(f"    return expand({E}, sweep, out, cap, n_combos);\n}}")
    inc.append(f"vta_status vta_{name}_batch_dev(vta_ctx* ctx, {ih}, size_t len, const {R}* sweep, {oa}) {{")
    inc.append(f"    if (!sweep) return fail(VTA_ERR_INVALID_INPUT, \"null sweep\");")
    inc.append(f"    const float* in[] = {{{nh}}};\n    vta_device_array* outs[] = {{{on}}};")
    inc.append(f"    for (vta_device_array* o : outs) if (!o) return fail(VTA_ERR_INVALID_INPUT, \"null output\");")
    inc.append(f"    return batch_host(ctx, {E}, in, len, grid_of({E}, sweep), outs, nullptr, 0, nullptr, nullptr);\n}}")
    inc.append(f"vta_status vta_{name}_batch_device(vta_ctx* ctx, {id_}, size_t len, size_t first_valid, const {R}* sweep, {od}) {{")
    inc.append(f"    if (!sweep) return fail(VTA_ERR_INVALID_INPUT, \"null sweep\");")
    inc.append(f"    const float* in[] = {{{nd}}};\n    float* outs[] = {{{odn}}};")
    inc.append(f"    return batch_device(ctx, {E}, in, len, first_valid, grid_of({E}, sweep), outs);\n}}")
    inc.append(f"vta_status vta_{name}_batch_into_host_f32(vta_ctx* ctx, {ih}, size_t len, const {R}* sweep, {oh}, size_t out_len, size_t* rows, size_t* cols) {{")
    inc.append(f"    if (!sweep) return fail(VTA_ERR_INVALID_INPUT, \"null sweep\");")
    inc.append(f"    const float* in[] = {{{nh}}};\n    float* outs[] = {{{on}}};")
    inc.append(f"    for (float* o : outs) if (!o) return fail(VTA_ERR_INVALID_INPUT, \"null output\");")
    inc.append(f"    return batch_host(ctx, {E}, in, len, grid_of({E}, sweep), nullptr, outs, out_len, rows, cols);\n}}")
    inc.append(f"vta_status vta_{name}_many_series_one_param_time_major_dev(vta_ctx* ctx, {ith}, size_t cols, size_t rows, const {P}* params, {oa}) {{")
    inc.append(f"    if (!params) return fail(VTA_ERR_INVALID_INPUT, \"null params\");")
    inc.append(f"    const float* in[] = {{{nth}}};\n    vta_device_array* outs[] = {{{on}}};")
    inc.append(f"    for (vta_device_array* o : outs) if (!o) return fail(VTA_ERR_INVALID_INPUT, \"null output\");")
    inc.append(f"    return tm_host(ctx, {E}, in, cols, rows, combo_of(params), outs);\n}}")
    inc.append(f"vta_status vta_{name}_many_series_one_param_device(vta_ctx* ctx, {itd}, size_t cols, size_t rows, const {P}* params, {od}) {{")
    inc.append(f"    if (!params) return fail(VTA_ERR_INVALID_INPUT, \"null params\");")
    inc.append(f"    const float* in[] = {{{ntd}}};\n    float* outs[] = {{{odn}}};")
    inc.append(f"    return tm_device(ctx, {E}, in, cols, rows, combo_of(params), outs);\n}}")
    inc.append("")
open("vectorta_gb300/csrc/vta_abi_gen.inc","w").write("\n".join(inc)+"\n")
print("ok")
