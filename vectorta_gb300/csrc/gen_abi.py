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
 *   - every call is stream-ordered on the context's stream.  Calls that take
 *     host data or return host results wait for their work before returning,
 *     like the crate's x_batch_dev / *_into_host_f32 (which end with
 *     stream.synchronize()); the device-pointer entry points that write into
 *     caller device buffers (*_batch_device, *_many_series_one_param_device)
 *     return once their work is queued, like the crate's x_batch_device /
 *     x_many_series_one_param_device: read their outputs after
 *     vta_ctx_synchronize (CudaX::synchronize) or from work queued behind them
 *     on the same stream.
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
/* The fields of CudaXError::OutOfMemory{required, free, headroom}
 * (alma_wrapper.rs:72-101, raised at alma_wrapper.rs:300-310): when the last
 * failure on the calling thread was VTA_ERR_OUT_OF_MEMORY, writes its byte
 * counts (any pointer may be null) and returns VTA_OK; otherwise writes zeros
 * and returns VTA_ERR_INVALID_INPUT. */
vta_status vta_last_error_oom(size_t* required, size_t* free_bytes, size_t* headroom);
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
 * alma_wrapper.rs:810-815).  They are mapped into the device address space:
 * a *_batch_into_host_f32 output buffer that lies inside one takes the
 * kernels' stores directly, with no device buffer or copy (policy "host_out"
 * = "direct", the default; "copy" stages through the device). */
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
 * returns (same arguments and parameter checks) but never allocates device
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
 *     that first call before any stream capture on that device.  No call can
 *     be captured: each uploads its period list from host memory and waits
 *     for its stream.
 *   - The period count is taken from the range arithmetic before anything
 *     is expanded, so an oversized sweep is refused at once; the periods
 *     live on the caller's stack (16 KiB at the limit).
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

# ---------------------------------------------------------------- Rust ----
# A thin Rust binding crate (vectorta_gb300/rust/vta_sys): the C ABI's
# declarations plus CudaX-shaped safe wrappers with the crate's method names,
# so the crate's src/cuda callers can switch their backend to the library.
# No Rust toolchain exists in the environment that builds this repository, so
# the generated crate is not compiled here.
RFIELDS = {
    "alma": ([("period", "VtaRangeUsize"), ("offset", "VtaRangeF64"), ("sigma", "VtaRangeF64")],
             [("period", "usize"), ("offset", "f64"), ("sigma", "f64")]),
    "period": ([("period", "VtaRangeUsize")], [("period", "usize")]),
    "stddev": ([("period", "VtaRangeUsize"), ("nbdev", "VtaRangeF64")], [("period", "usize"), ("nbdev", "f64")]),
    "zscore": ([("period", "VtaRangeUsize"), ("nbdev", "VtaRangeF64")], [("period", "usize"), ("nbdev", "f64")]),
    "bollinger": ([("period", "VtaRangeUsize"), ("devup", "VtaRangeF64"), ("devdn", "VtaRangeF64")],
                  [("period", "usize"), ("devup", "f64"), ("devdn", "f64")]),
    "supertrend": ([("period", "VtaRangeUsize"), ("factor", "VtaRangeF64")], [("period", "usize"), ("factor", "f64")]),
    "percentile": ([("length", "VtaRangeUsize"), ("percentage", "VtaRangeF64")],
                   [("length", "usize"), ("percentage", "f64")]),
    "epma": ([("period", "VtaRangeUsize"), ("offset", "VtaRangeUsize")], [("period", "usize"), ("offset", "usize")]),
    "vpwma": ([("period", "VtaRangeUsize"), ("power", "VtaRangeF64")], [("period", "usize"), ("power", "f64")]),
}


def camel(s):
    return "".join(p[:1].upper() + p[1:] for p in s.split("_"))


def rtypes(rng):
    R, P = RANGES[rng]
    return camel(R), camel(P)


def rin(kind, dev, tm):
    """Rust parameters of the input series (slices, or raw device pointers)."""
    nm = {"x": ["data"], "hl": ["high", "low"], "hlc": ["high", "low", "close"]}[kind]
    suf = "_tm" if tm else ""
    return [(f"{'d_' if dev else ''}{n}{suf}", "*const f32" if dev else "&[f32]") for n in nm]


rs = []
r = rs.append
r("""//! vta_sys -- Rust binding of libvta_gb300.so (include/vta_gb300.h).
//!
//! Generated by vectorta_gb300/csrc/gen_abi.py; do not edit by hand.  NOT
//! COMPILED in the environment that builds this repository (it has no Rust
//! toolchain): the declarations follow the C header one to one and the safe
//! layer mirrors the crate's src/cuda wrappers (`CudaX::new`,
//! `x_batch_dev`, `x_batch_into_host_f32`, `x_many_series_one_param_time_major_dev`,
//! `x_batch_device`, `DeviceArrayF32`, `CudaXError`), so a caller switches by
//! replacing its `use crate::cuda::...` imports.  Link with
//! `-L <repo>/vectorta_gb300/_lib -lvta_gb300` (see build.rs).
#![allow(non_camel_case_types, clippy::too_many_arguments)]

use std::ffi::{CStr, CString};
use std::os::raw::{c_char, c_int, c_void};

pub type VtaStatus = c_int;

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaRangeUsize { pub start: usize, pub end: usize, pub step: usize }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaRangeF64 { pub start: f64, pub end: f64, pub step: f64 }
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct VtaDeviceArray { pub ptr: *mut f32, pub rows: usize, pub cols: usize, pub device: c_int }
impl Default for VtaDeviceArray {
    fn default() -> Self { VtaDeviceArray { ptr: std::ptr::null_mut(), rows: 0, cols: 0, device: -1 } }
}
#[repr(C)]
pub struct VtaCtx { _private: [u8; 0] }
""")
for rng, (rf, pf) in RFIELDS.items():
    RT, PT = rtypes(rng)
    r("#[repr(C)]\n#[derive(Clone, Copy, Debug, Default)]")
    r(f"pub struct {RT} {{ " + ", ".join(f"pub {n}: {t}" for n, t in rf) + " }")
    r("#[repr(C)]\n#[derive(Clone, Copy, Debug, Default)]")
    r(f"pub struct {PT} {{ " + ", ".join(f"pub {n}: {t}" for n, t in pf) + " }")
r("""
#[link(name = "vta_gb300")]
extern "C" {
    pub fn vta_last_error() -> *const c_char;
    pub fn vta_last_error_oom(required: *mut usize, free_bytes: *mut usize, headroom: *mut usize) -> VtaStatus;
    pub fn vta_version() -> *const c_char;
    pub fn vta_device_count() -> c_int;
    pub fn vta_ctx_create(device_id: c_int, out: *mut *mut VtaCtx) -> VtaStatus;
    pub fn vta_ctx_destroy(ctx: *mut VtaCtx) -> VtaStatus;
    pub fn vta_ctx_synchronize(ctx: *mut VtaCtx) -> VtaStatus;
    pub fn vta_ctx_set_stream(ctx: *mut VtaCtx, stream: *mut c_void) -> VtaStatus;
    pub fn vta_ctx_set_policy(ctx: *mut VtaCtx, key: *const c_char, value: *const c_char) -> VtaStatus;
    pub fn vta_ctx_last_kernel(ctx: *mut VtaCtx) -> *const c_char;
    pub fn vta_device_array_free(a: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_device_array_copy_to_host(ctx: *mut VtaCtx, a: *const VtaDeviceArray, host: *mut f32, n: usize) -> VtaStatus;""")
for (name, wf, kind, outs, rng, prm, cites) in IND:
    RT, PT = rtypes(rng)
    hin = ", ".join(f"{n.replace('&[f32]','')}: *const f32" for n, _ in rin(kind, False, False))
    din = ", ".join(f"{n}: *const f32" for n, _ in rin(kind, True, False))
    thin = ", ".join(f"{n}: *const f32" for n, _ in rin(kind, False, True))
    tdin = ", ".join(f"{n}: *const f32" for n, _ in rin(kind, True, True))
    oa = ", ".join(f"{o}: *mut VtaDeviceArray" for o in outs)
    od = ", ".join(f"d_{o}: *mut f32" for o in outs)
    oh = ", ".join(f"{o}: *mut f32" for o in outs)
    r(f"    pub fn vta_{name}_expand_grid(sweep: *const {RT}, out: *mut {PT}, cap: usize, n_combos: *mut usize) -> VtaStatus;")
    r(f"    pub fn vta_{name}_batch_dev(ctx: *mut VtaCtx, {hin}, len: usize, sweep: *const {RT}, {oa}) -> VtaStatus;")
    r(f"    pub fn vta_{name}_batch_device(ctx: *mut VtaCtx, {din}, len: usize, first_valid: usize, sweep: *const {RT}, {od}) -> VtaStatus;")
    r(f"    pub fn vta_{name}_batch_into_host_f32(ctx: *mut VtaCtx, {hin}, len: usize, sweep: *const {RT}, {oh}, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;")
    r(f"    pub fn vta_{name}_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, {thin}, cols: usize, rows: usize, params: *const {PT}, {oa}) -> VtaStatus;")
    r(f"    pub fn vta_{name}_many_series_one_param_device(ctx: *mut VtaCtx, {tdin}, cols: usize, rows: usize, params: *const {PT}, {od}) -> VtaStatus;")
r("}")
r("""
/// The crate's CudaXError variants (alma_wrapper.rs:72-101), one per status.
#[derive(Debug, Clone)]
pub enum CudaError {
    Cuda(String),
    OutOfMemory { required: usize, free: usize, headroom: usize },
    MissingKernelSymbol(String),
    InvalidInput(String),
    InvalidPolicy(String),
    LaunchConfigTooLarge(String),
    DeviceMismatch(String),
    NotImplemented(String),
}

impl std::fmt::Display for CudaError {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result { write!(f, "{:?}", self) }
}
impl std::error::Error for CudaError {}

fn check(st: VtaStatus) -> Result<(), CudaError> {
    if st == 0 {
        return Ok(());
    }
    let msg = unsafe {
        let p = vta_last_error();
        if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
    };
    Err(match st {
        2 => {
            let (mut r, mut f, mut h) = (0usize, 0usize, 0usize);
            unsafe { vta_last_error_oom(&mut r, &mut f, &mut h) };
            CudaError::OutOfMemory { required: r, free: f, headroom: h }
        }
        3 => CudaError::MissingKernelSymbol(msg),
        4 => CudaError::InvalidInput(msg),
        5 => CudaError::InvalidPolicy(msg),
        6 => CudaError::LaunchConfigTooLarge(msg),
        7 => CudaError::DeviceMismatch(msg),
        8 => CudaError::NotImplemented(msg),
        _ => CudaError::Cuda(msg),
    })
}

/// One context: a device and a private non-blocking stream (CudaX::new).
pub struct Context { raw: *mut VtaCtx }
impl Context {
    pub fn new(device_id: usize) -> Result<Self, CudaError> {
        let mut raw = std::ptr::null_mut();
        check(unsafe { vta_ctx_create(device_id as c_int, &mut raw) })?;
        Ok(Context { raw })
    }
    pub fn raw(&self) -> *mut VtaCtx { self.raw }
    pub fn synchronize(&self) -> Result<(), CudaError> { check(unsafe { vta_ctx_synchronize(self.raw) }) }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> {
        let (k, v) = (CString::new(key).unwrap(), CString::new(value).unwrap());
        check(unsafe { vta_ctx_set_policy(self.raw, k.as_ptr(), v.as_ptr()) })
    }
    pub fn selected_kernel(&self) -> String {
        unsafe { CStr::from_ptr(vta_ctx_last_kernel(self.raw)).to_string_lossy().into_owned() }
    }
}
impl Drop for Context {
    fn drop(&mut self) { unsafe { vta_ctx_destroy(self.raw); } }
}

/// A device-resident f32 matrix owned by the caller (the crate's DeviceArrayF32,
/// alma_wrapper.rs:103-117): row-major rows x cols, freed on drop.
pub struct DeviceArrayF32 { pub raw: VtaDeviceArray }
impl DeviceArrayF32 {
    pub fn rows(&self) -> usize { self.raw.rows }
    pub fn cols(&self) -> usize { self.raw.cols }
    pub fn len(&self) -> usize { self.raw.rows * self.raw.cols }
    pub fn is_empty(&self) -> bool { self.len() == 0 }
    pub fn device_ptr(&self) -> *mut f32 { self.raw.ptr }
    pub fn copy_to_host(&self, ctx: &Context, out: &mut [f32]) -> Result<(), CudaError> {
        check(unsafe { vta_device_array_copy_to_host(ctx.raw(), &self.raw, out.as_mut_ptr(), out.len()) })
    }
}
impl Drop for DeviceArrayF32 {
    fn drop(&mut self) { unsafe { vta_device_array_free(&mut self.raw); } }
}
""")
for (name, wf, kind, outs, rng, prm, cites) in IND:
    RT, PT = rtypes(rng)
    cls = "Cuda" + camel(name)
    ins = rin(kind, False, False)
    ins_tm = rin(kind, False, True)
    dins = rin(kind, True, False)
    dins_tm = rin(kind, True, True)
    no = len(outs)
    ret = "DeviceArrayF32" if no == 1 else "(" + ", ".join(["DeviceArrayF32"] * no) + ")"
    mk = ("DeviceArrayF32 { raw: o[0] }" if no == 1 else
          "(" + ", ".join(f"DeviceArrayF32 {{ raw: o[{i}] }}" for i in range(no)) + ")")
    optrs = ", ".join(f"&mut o[{i}]" for i in range(no))
    r(f"/// {name}: replaces {wf} (CudaX::new at line {cites[0]}).")
    r(f"pub struct {cls} {{ pub ctx: Context }}")
    r(f"impl {cls} {{")
    r(f"    pub fn new(device_id: usize) -> Result<Self, CudaError> {{ Ok({cls} {{ ctx: Context::new(device_id)? }}) }}")
    r(f"    pub fn synchronize(&self) -> Result<(), CudaError> {{ self.ctx.synchronize() }}")
    r(f"    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> {{ self.ctx.set_policy(key, value) }}")
    r(f"    pub fn expand_grid(sweep: &{RT}) -> Result<Vec<{PT}>, CudaError> {{")
    r(f"        let mut n = 0usize;")
    r(f"        unsafe {{ vta_{name}_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) }};")
    r(f"        let mut v = vec![{PT}::default(); n];")
    r(f"        check(unsafe {{ vta_{name}_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) }})?;")
    r(f"        Ok(v)")
    r(f"    }}")
    a_in = ", ".join(f"{n}: {t}" for n, t in ins)
    lens = ins[0][0]
    checks = "".join(f"        if {n}.len() != {lens}.len() {{ return Err(CudaError::InvalidInput(\"inconsistent input lengths\".into())); }}\n"
                     for n, _ in ins[1:])
    p_in = ", ".join(f"{n}.as_ptr()" for n, _ in ins)
    r(f"    pub fn {name}_batch_dev(&self, {a_in}, sweep: &{RT}) -> Result<{ret}, CudaError> {{")
    if checks: r(checks.rstrip("\n"))
    r(f"        let mut o = [VtaDeviceArray::default(); {no}];")
    r(f"        check(unsafe {{ vta_{name}_batch_dev(self.ctx.raw(), {p_in}, {lens}.len(), sweep, {optrs}) }})?;")
    r(f"        Ok({mk})")
    r(f"    }}")
    on_ = [o if o.startswith("out") else "out_" + o for o in outs]
    o_mut = ", ".join(f"{o}: &mut [f32]" for o in on_)
    o_ptr = ", ".join(f"{o}.as_mut_ptr()" for o in on_)
    r(f"    /// Returns (rows, cols); every output slice holds at least rows * cols values.")
    r(f"    pub fn {name}_batch_into_host_f32(&self, {a_in}, sweep: &{RT}, {o_mut}) -> Result<(usize, usize), CudaError> {{")
    if checks: r(checks.rstrip("\n"))
    r(f"        let out_len = {on_[0]}.len();")
    for o in on_[1:]:
        r(f"        if {o}.len() < out_len {{ return Err(CudaError::InvalidInput(\"output slices of different lengths\".into())); }}")
    r(f"        let (mut rows, mut cols) = (0usize, 0usize);")
    r(f"        check(unsafe {{ vta_{name}_batch_into_host_f32(self.ctx.raw(), {p_in}, {lens}.len(), sweep, {o_ptr}, out_len, &mut rows, &mut cols) }})?;")
    r(f"        Ok((rows, cols))")
    r(f"    }}")
    a_tm = ", ".join(f"{n}: {t}" for n, t in ins_tm)
    p_tm = ", ".join(f"{n}.as_ptr()" for n, _ in ins_tm)
    r(f"    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).")
    r(f"    pub fn {name}_many_series_one_param_time_major_dev(&self, {a_tm}, cols: usize, rows: usize, params: &{PT}) -> Result<{ret}, CudaError> {{")
    for n, _ in ins_tm:
        r(f"        if {n}.len() < cols * rows {{ return Err(CudaError::InvalidInput(\"input shorter than cols * rows\".into())); }}")
    r(f"        let mut o = [VtaDeviceArray::default(); {no}];")
    r(f"        check(unsafe {{ vta_{name}_many_series_one_param_time_major_dev(self.ctx.raw(), {p_tm}, cols, rows, params, {optrs}) }})?;")
    r(f"        Ok({mk})")
    r(f"    }}")
    a_d = ", ".join(f"{n}: {t}" for n, t in dins)
    n_d = ", ".join(n for n, _ in dins)
    od_a = ", ".join(f"d_{o}: *mut f32" for o in outs)
    od_n = ", ".join(f"d_{o}" for o in outs)
    r(f"    /// Device inputs and caller-provided device outputs (x_batch_device).")
    r(f"    /// # Safety: the pointers address device buffers of len and n_combos * len floats.")
    r(f"    pub unsafe fn {name}_batch_device(&self, {a_d}, len: usize, first_valid: usize, sweep: &{RT}, {od_a}) -> Result<(), CudaError> {{")
    r(f"        check(vta_{name}_batch_device(self.ctx.raw(), {n_d}, len, first_valid, sweep, {od_n}))")
    r(f"    }}")
    a_dt = ", ".join(f"{n}: {t}" for n, t in dins_tm)
    n_dt = ", ".join(n for n, _ in dins_tm)
    r(f"    /// # Safety: the pointers address device buffers of cols * rows floats.")
    r(f"    pub unsafe fn {name}_many_series_one_param_device(&self, {a_dt}, cols: usize, rows: usize, params: &{PT}, {od_a}) -> Result<(), CudaError> {{")
    r(f"        check(vta_{name}_many_series_one_param_device(self.ctx.raw(), {n_dt}, cols, rows, params, {od_n}))")
    r(f"    }}")
    r("}")
    r("")
import os as _os
_os.makedirs("vectorta_gb300/rust/vta_sys/src", exist_ok=True)
open("vectorta_gb300/rust/vta_sys/src/lib.rs", "w").write("\n".join(rs) + "\n")
open("vectorta_gb300/rust/vta_sys/Cargo.toml", "w").write("""[package]
name = "vta_sys"
version = "0.1.0"
edition = "2021"
description = "Rust binding of libvta_gb300 (GB300-native VectorTA indicator hot path); generated by gen_abi.py"
publish = false

[lib]
path = "src/lib.rs"
""")
open("vectorta_gb300/rust/vta_sys/build.rs", "w").write("""// Links libvta_gb300.so from the repository's build folder, or from
// VTA_GB300_LIB_DIR when set.  Generated by gen_abi.py.
fn main() {
    let dir = std::env::var("VTA_GB300_LIB_DIR").unwrap_or_else(|_| {
        let here = std::env::var("CARGO_MANIFEST_DIR").unwrap();
        format!("{}/../../_lib", here)
    });
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=vta_gb300");
    println!("cargo:rerun-if-env-changed=VTA_GB300_LIB_DIR");
}
""")
print("rust ok")
