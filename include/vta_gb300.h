/*
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

/* ==== alma (src/cuda/moving_averages/alma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_alma_expand_grid(const vta_alma_batch_range* sweep, vta_alma_params* out, size_t cap, size_t* n_combos);
/* alma_batch_dev (alma_wrapper.rs:625) */
vta_status vta_alma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_alma_batch_range* sweep, vta_device_array* out);
/* alma_batch_device / _from_device_prices (alma_wrapper.rs:671); first_valid as in the crate. */
vta_status vta_alma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_alma_batch_range* sweep, float* d_out);
/* alma_batch_into_host_f32 (alma_wrapper.rs:783); each output holds out_len >= rows*cols floats. */
vta_status vta_alma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_alma_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* alma_many_series_one_param_time_major_dev (alma_wrapper.rs:819) */
vta_status vta_alma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_alma_params* params, vta_device_array* out);
/* alma_many_series_one_param_device (alma_wrapper.rs:1521) */
vta_status vta_alma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_alma_params* params, float* d_out);

/* ==== ema (src/cuda/moving_averages/ema_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_ema_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* ema_batch_dev (ema_wrapper.rs:193) */
vta_status vta_ema_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* ema_batch_device / _from_device_prices (ema_wrapper.rs:256); first_valid as in the crate. */
vta_status vta_ema_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* ema_batch_into_host_f32 (ema_wrapper.rs:309); each output holds out_len >= rows*cols floats. */
vta_status vta_ema_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* ema_many_series_one_param_time_major_dev (ema_wrapper.rs:325) */
vta_status vta_ema_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* ema_many_series_one_param_device (ema_wrapper.rs:381) */
vta_status vta_ema_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== dema (src/cuda/moving_averages/dema_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_dema_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* dema_batch_dev (dema_wrapper.rs:219) */
vta_status vta_dema_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* dema_batch_device / _from_device_prices (dema_wrapper.rs:305); first_valid as in the crate. */
vta_status vta_dema_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* dema_batch_into_host_f32 (dema_wrapper.rs:379); each output holds out_len >= rows*cols floats. */
vta_status vta_dema_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* dema_many_series_one_param_time_major_dev (dema_wrapper.rs:516) */
vta_status vta_dema_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* dema_many_series_one_param_device (dema_wrapper.rs:554) */
vta_status vta_dema_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== tema (src/cuda/moving_averages/tema_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_tema_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* tema_batch_dev (tema_wrapper.rs:336) */
vta_status vta_tema_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* tema_batch_device / _from_device_prices (tema_wrapper.rs:367); first_valid as in the crate. */
vta_status vta_tema_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* tema_batch_into_host_f32 (tema_wrapper.rs:345); each output holds out_len >= rows*cols floats. */
vta_status vta_tema_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* tema_many_series_one_param_time_major_dev (tema_wrapper.rs:430) */
vta_status vta_tema_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* tema_many_series_one_param_device (tema_wrapper.rs:397) */
vta_status vta_tema_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== rsi (src/cuda/rsi_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_rsi_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* rsi_batch_dev (rsi_wrapper.rs:152) */
vta_status vta_rsi_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* rsi_batch_device / _from_device_prices (device-input form of rsi_wrapper.rs:152); first_valid as in the crate. */
vta_status vta_rsi_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* rsi_batch_into_host_f32 (host-output form of rsi_wrapper.rs:152); each output holds out_len >= rows*cols floats. */
vta_status vta_rsi_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* rsi_many_series_one_param_time_major_dev (rsi_wrapper.rs:271) */
vta_status vta_rsi_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* rsi_many_series_one_param_device (device-input form of rsi_wrapper.rs:271) */
vta_status vta_rsi_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== wilders (src/cuda/moving_averages/wilders_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_wilders_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* wilders_batch_dev (wilders_wrapper.rs:134) */
vta_status vta_wilders_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* wilders_batch_device / _from_device_prices (wilders_wrapper.rs:252); first_valid as in the crate. */
vta_status vta_wilders_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* wilders_batch_into_host_f32 (host-output form of wilders_wrapper.rs:134); each output holds out_len >= rows*cols floats. */
vta_status vta_wilders_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* wilders_many_series_one_param_time_major_dev (wilders_wrapper.rs:600) */
vta_status vta_wilders_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* wilders_many_series_one_param_device (wilders_wrapper.rs:662) */
vta_status vta_wilders_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== sma (src/cuda/moving_averages/sma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_sma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* sma_batch_dev (sma_wrapper.rs:548) */
vta_status vta_sma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* sma_batch_device / _from_device_prices (sma_wrapper.rs:830); first_valid as in the crate. */
vta_status vta_sma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* sma_batch_into_host_f32 (sma_wrapper.rs:558); each output holds out_len >= rows*cols floats. */
vta_status vta_sma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* sma_many_series_one_param_time_major_dev (sma_wrapper.rs:750) */
vta_status vta_sma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* sma_many_series_one_param_device (sma_wrapper.rs:982) */
vta_status vta_sma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== wma (src/cuda/moving_averages/wma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_wma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* wma_batch_dev (wma_wrapper.rs:713) */
vta_status vta_wma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* wma_batch_device / _from_device_prices (wma_wrapper.rs:747); first_valid as in the crate. */
vta_status vta_wma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* wma_batch_into_host_f32 (wma_wrapper.rs:723); each output holds out_len >= rows*cols floats. */
vta_status vta_wma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* wma_many_series_one_param_time_major_dev (wma_wrapper.rs:1014) */
vta_status vta_wma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* wma_many_series_one_param_device (wma_wrapper.rs:1049) */
vta_status vta_wma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== swma (src/cuda/moving_averages/swma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_swma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* swma_batch_dev (swma_wrapper.rs:678) */
vta_status vta_swma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* swma_batch_device / _from_device_prices (swma_wrapper.rs:663); first_valid as in the crate. */
vta_status vta_swma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* swma_batch_into_host_f32 (host-output form of swma_wrapper.rs:678); each output holds out_len >= rows*cols floats. */
vta_status vta_swma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* swma_many_series_one_param_time_major_dev (swma_wrapper.rs:825) */
vta_status vta_swma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* swma_many_series_one_param_device (swma_wrapper.rs:787) */
vta_status vta_swma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== pwma (src/cuda/moving_averages/pwma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_pwma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* pwma_batch_dev (pwma_wrapper.rs:385) */
vta_status vta_pwma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* pwma_batch_device / _from_device_prices (pwma_wrapper.rs:369); first_valid as in the crate. */
vta_status vta_pwma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* pwma_batch_into_host_f32 (host-output form of pwma_wrapper.rs:385); each output holds out_len >= rows*cols floats. */
vta_status vta_pwma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* pwma_many_series_one_param_time_major_dev (pwma_wrapper.rs:723) */
vta_status vta_pwma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* pwma_many_series_one_param_device (pwma_wrapper.rs:696) */
vta_status vta_pwma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== sinwma (src/cuda/moving_averages/sinwma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_sinwma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* sinwma_batch_dev (sinwma_wrapper.rs:609) */
vta_status vta_sinwma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* sinwma_batch_device / _from_device_prices (sinwma_wrapper.rs:643); first_valid as in the crate. */
vta_status vta_sinwma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* sinwma_batch_into_host_f32 (sinwma_wrapper.rs:619); each output holds out_len >= rows*cols floats. */
vta_status vta_sinwma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* sinwma_many_series_one_param_time_major_dev (sinwma_wrapper.rs:841) */
vta_status vta_sinwma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* sinwma_many_series_one_param_device (sinwma_wrapper.rs:873) */
vta_status vta_sinwma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== trima (src/cuda/moving_averages/trima_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_trima_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* trima_batch_dev (trima_wrapper.rs:722) */
vta_status vta_trima_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* trima_batch_device / _from_device_prices (trima_wrapper.rs:707); first_valid as in the crate. */
vta_status vta_trima_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* trima_batch_into_host_f32 (host-output form of trima_wrapper.rs:722); each output holds out_len >= rows*cols floats. */
vta_status vta_trima_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* trima_many_series_one_param_time_major_dev (trima_wrapper.rs:855) */
vta_status vta_trima_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* trima_many_series_one_param_device (trima_wrapper.rs:829) */
vta_status vta_trima_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== stddev (src/cuda/stddev_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_stddev_expand_grid(const vta_stddev_batch_range* sweep, vta_stddev_params* out, size_t cap, size_t* n_combos);
/* stddev_batch_dev (stddev_wrapper.rs:509) */
vta_status vta_stddev_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_stddev_batch_range* sweep, vta_device_array* out);
/* stddev_batch_device / _from_device_prices (device-input form of stddev_wrapper.rs:509); first_valid as in the crate. */
vta_status vta_stddev_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_stddev_batch_range* sweep, float* d_out);
/* stddev_batch_into_host_f32 (stddev_wrapper.rs:606); each output holds out_len >= rows*cols floats. */
vta_status vta_stddev_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_stddev_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* stddev_many_series_one_param_time_major_dev (stddev_wrapper.rs:630) */
vta_status vta_stddev_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_stddev_params* params, vta_device_array* out);
/* stddev_many_series_one_param_device (device-input form of stddev_wrapper.rs:630) */
vta_status vta_stddev_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_stddev_params* params, float* d_out);

/* ==== zscore (src/cuda/zscore_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_zscore_expand_grid(const vta_zscore_batch_range* sweep, vta_zscore_params* out, size_t cap, size_t* n_combos);
/* zscore_batch_dev (zscore_wrapper.rs:620) */
vta_status vta_zscore_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_zscore_batch_range* sweep, vta_device_array* out);
/* zscore_batch_device / _from_device_prices (device-input form of zscore_wrapper.rs:620); first_valid as in the crate. */
vta_status vta_zscore_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_zscore_batch_range* sweep, float* d_out);
/* zscore_batch_into_host_f32 (zscore_wrapper.rs:663); each output holds out_len >= rows*cols floats. */
vta_status vta_zscore_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_zscore_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* zscore_many_series_one_param_time_major_dev (zscore_wrapper.rs:720) */
vta_status vta_zscore_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_zscore_params* params, vta_device_array* out);
/* zscore_many_series_one_param_device (device-input form of zscore_wrapper.rs:720) */
vta_status vta_zscore_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_zscore_params* params, float* d_out);

/* ==== bollinger_bands (src/cuda/bollinger_bands_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_bollinger_bands_expand_grid(const vta_bollinger_batch_range* sweep, vta_bollinger_params* out, size_t cap, size_t* n_combos);
/* bollinger_bands_batch_dev (bollinger_bands_wrapper.rs:567) */
vta_status vta_bollinger_bands_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_bollinger_batch_range* sweep, vta_device_array* out_upper, vta_device_array* out_middle, vta_device_array* out_lower);
/* bollinger_bands_batch_device / _from_device_prices (device-input form of bollinger_bands_wrapper.rs:567); first_valid as in the crate. */
vta_status vta_bollinger_bands_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_bollinger_batch_range* sweep, float* d_out_upper, float* d_out_middle, float* d_out_lower);
/* bollinger_bands_batch_into_host_f32 (host-output form of bollinger_bands_wrapper.rs:567); each output holds out_len >= rows*cols floats. */
vta_status vta_bollinger_bands_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_bollinger_batch_range* sweep, float* out_upper, float* out_middle, float* out_lower, size_t out_len, size_t* rows, size_t* cols);
/* bollinger_bands_many_series_one_param_time_major_dev (bollinger_bands_wrapper.rs:605) */
vta_status vta_bollinger_bands_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_bollinger_params* params, vta_device_array* out_upper, vta_device_array* out_middle, vta_device_array* out_lower);
/* bollinger_bands_many_series_one_param_device (device-input form of bollinger_bands_wrapper.rs:605) */
vta_status vta_bollinger_bands_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_bollinger_params* params, float* d_out_upper, float* d_out_middle, float* d_out_lower);

/* ==== atr (src/cuda/atr_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_atr_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* atr_batch_dev (atr_wrapper.rs:270) */
vta_status vta_atr_batch_dev(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* atr_batch_device / _from_device_prices (atr_wrapper.rs:626); first_valid as in the crate. */
vta_status vta_atr_batch_device(vta_ctx* ctx, const float* d_high, const float* d_low, const float* d_close, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* atr_batch_into_host_f32 (host-output form of atr_wrapper.rs:270); each output holds out_len >= rows*cols floats. */
vta_status vta_atr_batch_into_host_f32(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* atr_many_series_one_param_time_major_dev (atr_wrapper.rs:834) */
vta_status vta_atr_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* high_tm, const float* low_tm, const float* close_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* atr_many_series_one_param_device (device-input form of atr_wrapper.rs:834) */
vta_status vta_atr_many_series_one_param_device(vta_ctx* ctx, const float* d_high_tm, const float* d_low_tm, const float* d_close_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== adx (src/cuda/adx_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_adx_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* adx_batch_dev (adx_wrapper.rs:199) */
vta_status vta_adx_batch_dev(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* adx_batch_device / _from_device_prices (device-input form of adx_wrapper.rs:199); first_valid as in the crate. */
vta_status vta_adx_batch_device(vta_ctx* ctx, const float* d_high, const float* d_low, const float* d_close, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* adx_batch_into_host_f32 (adx_wrapper.rs:253); each output holds out_len >= rows*cols floats. */
vta_status vta_adx_batch_into_host_f32(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* adx_many_series_one_param_time_major_dev (adx_wrapper.rs:340) */
vta_status vta_adx_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* high_tm, const float* low_tm, const float* close_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* adx_many_series_one_param_device (device-input form of adx_wrapper.rs:340) */
vta_status vta_adx_many_series_one_param_device(vta_ctx* ctx, const float* d_high_tm, const float* d_low_tm, const float* d_close_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== supertrend (src/cuda/supertrend_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_supertrend_expand_grid(const vta_supertrend_batch_range* sweep, vta_supertrend_params* out, size_t cap, size_t* n_combos);
/* supertrend_batch_dev (supertrend_wrapper.rs:179) */
vta_status vta_supertrend_batch_dev(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_supertrend_batch_range* sweep, vta_device_array* out_trend, vta_device_array* out_changed);
/* supertrend_batch_device / _from_device_prices (device-input form of supertrend_wrapper.rs:179); first_valid as in the crate. */
vta_status vta_supertrend_batch_device(vta_ctx* ctx, const float* d_high, const float* d_low, const float* d_close, size_t len,
    size_t first_valid, const vta_supertrend_batch_range* sweep, float* d_out_trend, float* d_out_changed);
/* supertrend_batch_into_host_f32 (host-output form of supertrend_wrapper.rs:179); each output holds out_len >= rows*cols floats. */
vta_status vta_supertrend_batch_into_host_f32(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_supertrend_batch_range* sweep, float* out_trend, float* out_changed, size_t out_len, size_t* rows, size_t* cols);
/* supertrend_many_series_one_param_time_major_dev (supertrend_wrapper.rs:337) */
vta_status vta_supertrend_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* high_tm, const float* low_tm, const float* close_tm,
    size_t cols, size_t rows, const vta_supertrend_params* params, vta_device_array* out_trend, vta_device_array* out_changed);
/* supertrend_many_series_one_param_device (device-input form of supertrend_wrapper.rs:337) */
vta_status vta_supertrend_many_series_one_param_device(vta_ctx* ctx, const float* d_high_tm, const float* d_low_tm, const float* d_close_tm,
    size_t cols, size_t rows, const vta_supertrend_params* params, float* d_out_trend, float* d_out_changed);

/* ==== donchian (src/cuda/donchian_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_donchian_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* donchian_batch_dev (donchian_wrapper.rs:344) */
vta_status vta_donchian_batch_dev(vta_ctx* ctx, const float* high, const float* low, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out_upper, vta_device_array* out_middle, vta_device_array* out_lower);
/* donchian_batch_device / _from_device_prices (device-input form of donchian_wrapper.rs:344); first_valid as in the crate. */
vta_status vta_donchian_batch_device(vta_ctx* ctx, const float* d_high, const float* d_low, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out_upper, float* d_out_middle, float* d_out_lower);
/* donchian_batch_into_host_f32 (host-output form of donchian_wrapper.rs:344); each output holds out_len >= rows*cols floats. */
vta_status vta_donchian_batch_into_host_f32(vta_ctx* ctx, const float* high, const float* low, size_t len,
    const vta_period_batch_range* sweep, float* out_upper, float* out_middle, float* out_lower, size_t out_len, size_t* rows, size_t* cols);
/* donchian_many_series_one_param_time_major_dev (donchian_wrapper.rs:593) */
vta_status vta_donchian_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* high_tm, const float* low_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out_upper, vta_device_array* out_middle, vta_device_array* out_lower);
/* donchian_many_series_one_param_device (device-input form of donchian_wrapper.rs:593) */
vta_status vta_donchian_many_series_one_param_device(vta_ctx* ctx, const float* d_high_tm, const float* d_low_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out_upper, float* d_out_middle, float* d_out_lower);

/* ==== willr (src/cuda/willr_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_willr_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* willr_batch_dev (willr_wrapper.rs:132) */
vta_status vta_willr_batch_dev(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* willr_batch_device / _from_device_prices (willr_wrapper.rs:236); first_valid as in the crate. */
vta_status vta_willr_batch_device(vta_ctx* ctx, const float* d_high, const float* d_low, const float* d_close, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* willr_batch_into_host_f32 (host-output form of willr_wrapper.rs:132); each output holds out_len >= rows*cols floats. */
vta_status vta_willr_batch_into_host_f32(vta_ctx* ctx, const float* high, const float* low, const float* close, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* willr_many_series_one_param_time_major_dev (willr_wrapper.rs:583) */
vta_status vta_willr_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* high_tm, const float* low_tm, const float* close_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* willr_many_series_one_param_device (willr_wrapper.rs:642) */
vta_status vta_willr_many_series_one_param_device(vta_ctx* ctx, const float* d_high_tm, const float* d_low_tm, const float* d_close_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== percentile_nearest_rank (src/cuda/percentile_nearest_rank_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_percentile_nearest_rank_expand_grid(const vta_percentile_batch_range* sweep, vta_percentile_params* out, size_t cap, size_t* n_combos);
/* percentile_nearest_rank_batch_dev (percentile_nearest_rank_wrapper.rs:365) */
vta_status vta_percentile_nearest_rank_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_percentile_batch_range* sweep, vta_device_array* out);
/* percentile_nearest_rank_batch_device / _from_device_prices (device-input form of percentile_nearest_rank_wrapper.rs:365); first_valid as in the crate. */
vta_status vta_percentile_nearest_rank_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_percentile_batch_range* sweep, float* d_out);
/* percentile_nearest_rank_batch_into_host_f32 (host-output form of percentile_nearest_rank_wrapper.rs:365); each output holds out_len >= rows*cols floats. */
vta_status vta_percentile_nearest_rank_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_percentile_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* percentile_nearest_rank_many_series_one_param_time_major_dev (percentile_nearest_rank_wrapper.rs:623) */
vta_status vta_percentile_nearest_rank_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_percentile_params* params, vta_device_array* out);
/* percentile_nearest_rank_many_series_one_param_device (device-input form of percentile_nearest_rank_wrapper.rs:623) */
vta_status vta_percentile_nearest_rank_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_percentile_params* params, float* d_out);

/* ==== cwma (src/cuda/moving_averages/cwma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_cwma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* cwma_batch_dev (cwma_wrapper.rs:767) */
vta_status vta_cwma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* cwma_batch_device / _from_device_prices (cwma_wrapper.rs:737); first_valid as in the crate. */
vta_status vta_cwma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* cwma_batch_into_host_f32 (cwma_wrapper.rs:850); each output holds out_len >= rows*cols floats. */
vta_status vta_cwma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* cwma_many_series_one_param_time_major_dev (cwma_wrapper.rs:1208) */
vta_status vta_cwma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* cwma_many_series_one_param_device (cwma_wrapper.rs:1180) */
vta_status vta_cwma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== fwma (src/cuda/moving_averages/fwma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_fwma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* fwma_batch_dev (fwma_wrapper.rs:491) */
vta_status vta_fwma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* fwma_batch_device / _from_device_prices (fwma_wrapper.rs:475); first_valid as in the crate. */
vta_status vta_fwma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* fwma_batch_into_host_f32 (host-output form of fwma_wrapper.rs:491); each output holds out_len >= rows*cols floats. */
vta_status vta_fwma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* fwma_many_series_one_param_time_major_dev (fwma_wrapper.rs:760) */
vta_status vta_fwma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* fwma_many_series_one_param_device (fwma_wrapper.rs:734) */
vta_status vta_fwma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== srwma (src/cuda/moving_averages/srwma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_srwma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* srwma_batch_dev (srwma_wrapper.rs:328) */
vta_status vta_srwma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* srwma_batch_device / _from_device_prices (srwma_wrapper.rs:420); first_valid as in the crate. */
vta_status vta_srwma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* srwma_batch_into_host_f32 (host-output form of srwma_wrapper.rs:328); each output holds out_len >= rows*cols floats. */
vta_status vta_srwma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* srwma_many_series_one_param_time_major_dev (srwma_wrapper.rs:485) */
vta_status vta_srwma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* srwma_many_series_one_param_device (srwma_wrapper.rs:572) */
vta_status vta_srwma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== sqwma (src/cuda/moving_averages/sqwma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_sqwma_expand_grid(const vta_period_batch_range* sweep, vta_period_params* out, size_t cap, size_t* n_combos);
/* sqwma_batch_dev (sqwma_wrapper.rs:157) */
vta_status vta_sqwma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, vta_device_array* out);
/* sqwma_batch_device / _from_device_prices (sqwma_wrapper.rs:190); first_valid as in the crate. */
vta_status vta_sqwma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_period_batch_range* sweep, float* d_out);
/* sqwma_batch_into_host_f32 (sqwma_wrapper.rs:166); each output holds out_len >= rows*cols floats. */
vta_status vta_sqwma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_period_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* sqwma_many_series_one_param_time_major_dev (sqwma_wrapper.rs:255) */
vta_status vta_sqwma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_period_params* params, vta_device_array* out);
/* sqwma_many_series_one_param_device (sqwma_wrapper.rs:222) */
vta_status vta_sqwma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_period_params* params, float* d_out);

/* ==== epma (src/cuda/moving_averages/epma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_epma_expand_grid(const vta_epma_batch_range* sweep, vta_epma_params* out, size_t cap, size_t* n_combos);
/* epma_batch_dev (epma_wrapper.rs:485) */
vta_status vta_epma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_epma_batch_range* sweep, vta_device_array* out);
/* epma_batch_device / _from_device_prices (epma_wrapper.rs:574); first_valid as in the crate. */
vta_status vta_epma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_epma_batch_range* sweep, float* d_out);
/* epma_batch_into_host_f32 (epma_wrapper.rs:495); each output holds out_len >= rows*cols floats. */
vta_status vta_epma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_epma_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* epma_many_series_one_param_time_major_dev (epma_wrapper.rs:773) */
vta_status vta_epma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_epma_params* params, vta_device_array* out);
/* epma_many_series_one_param_device (epma_wrapper.rs:805) */
vta_status vta_epma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_epma_params* params, float* d_out);

/* ==== vpwma (src/cuda/moving_averages/vpwma_wrapper.rs) ==== */
/* expand_grid: the crate's combo order; n_combos always set; out may be NULL. */
vta_status vta_vpwma_expand_grid(const vta_vpwma_batch_range* sweep, vta_vpwma_params* out, size_t cap, size_t* n_combos);
/* vpwma_batch_dev (vpwma_wrapper.rs:720) */
vta_status vta_vpwma_batch_dev(vta_ctx* ctx, const float* data, size_t len,
    const vta_vpwma_batch_range* sweep, vta_device_array* out);
/* vpwma_batch_device / _from_device_prices (vpwma_wrapper.rs:751); first_valid as in the crate. */
vta_status vta_vpwma_batch_device(vta_ctx* ctx, const float* d_data, size_t len,
    size_t first_valid, const vta_vpwma_batch_range* sweep, float* d_out);
/* vpwma_batch_into_host_f32 (vpwma_wrapper.rs:730); each output holds out_len >= rows*cols floats. */
vta_status vta_vpwma_batch_into_host_f32(vta_ctx* ctx, const float* data, size_t len,
    const vta_vpwma_batch_range* sweep, float* out, size_t out_len, size_t* rows, size_t* cols);
/* vpwma_many_series_one_param_time_major_dev (vpwma_wrapper.rs:851) */
vta_status vta_vpwma_many_series_one_param_time_major_dev(vta_ctx* ctx, const float* data_tm,
    size_t cols, size_t rows, const vta_vpwma_params* params, vta_device_array* out);
/* vpwma_many_series_one_param_device (vpwma_wrapper.rs:823) */
vta_status vta_vpwma_many_series_one_param_device(vta_ctx* ctx, const float* d_data_tm,
    size_t cols, size_t rows, const vta_vpwma_params* params, float* d_out);

/* ==== many-series work-list plans ====
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

/* ==== request server (continuous batching over a device-resident store) ====
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

/* ==== sma without device allocation ====
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

#ifdef __cplusplus
}
#endif

#endif /* VTA_GB300_H */
