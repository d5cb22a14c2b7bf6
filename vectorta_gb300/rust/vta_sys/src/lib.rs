//! vta_sys -- Rust binding of libvta_gb300.so (include/vta_gb300.h).
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

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaAlmaBatchRange { pub period: VtaRangeUsize, pub offset: VtaRangeF64, pub sigma: VtaRangeF64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaAlmaParams { pub period: usize, pub offset: f64, pub sigma: f64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaPeriodBatchRange { pub period: VtaRangeUsize }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaPeriodParams { pub period: usize }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaStddevBatchRange { pub period: VtaRangeUsize, pub nbdev: VtaRangeF64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaStddevParams { pub period: usize, pub nbdev: f64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaZscoreBatchRange { pub period: VtaRangeUsize, pub nbdev: VtaRangeF64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaZscoreParams { pub period: usize, pub nbdev: f64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaBollingerBatchRange { pub period: VtaRangeUsize, pub devup: VtaRangeF64, pub devdn: VtaRangeF64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaBollingerParams { pub period: usize, pub devup: f64, pub devdn: f64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaSupertrendBatchRange { pub period: VtaRangeUsize, pub factor: VtaRangeF64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaSupertrendParams { pub period: usize, pub factor: f64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaPercentileBatchRange { pub length: VtaRangeUsize, pub percentage: VtaRangeF64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaPercentileParams { pub length: usize, pub percentage: f64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaEpmaBatchRange { pub period: VtaRangeUsize, pub offset: VtaRangeUsize }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaEpmaParams { pub period: usize, pub offset: usize }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaVpwmaBatchRange { pub period: VtaRangeUsize, pub power: VtaRangeF64 }
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct VtaVpwmaParams { pub period: usize, pub power: f64 }

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
    pub fn vta_device_array_copy_to_host(ctx: *mut VtaCtx, a: *const VtaDeviceArray, host: *mut f32, n: usize) -> VtaStatus;
    pub fn vta_alma_expand_grid(sweep: *const VtaAlmaBatchRange, out: *mut VtaAlmaParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_alma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaAlmaBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_alma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaAlmaBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_alma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaAlmaBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_alma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaAlmaParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_alma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaAlmaParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_ema_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_ema_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_ema_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_ema_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_ema_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_ema_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_dema_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_dema_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_dema_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_dema_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_dema_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_dema_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_tema_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_tema_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_tema_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_tema_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_tema_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_tema_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_rsi_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_rsi_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_rsi_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_rsi_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_rsi_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_rsi_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_wilders_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_wilders_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_wilders_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_wilders_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_wilders_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_wilders_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_sma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_sma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_sma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_sma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_sma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_sma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_wma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_wma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_wma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_wma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_wma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_wma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_swma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_swma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_swma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_swma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_swma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_swma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_pwma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_pwma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_pwma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_pwma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_pwma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_pwma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_sinwma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_sinwma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_sinwma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_sinwma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_sinwma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_sinwma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_trima_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_trima_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_trima_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_trima_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_trima_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_trima_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_stddev_expand_grid(sweep: *const VtaStddevBatchRange, out: *mut VtaStddevParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_stddev_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaStddevBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_stddev_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaStddevBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_stddev_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaStddevBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_stddev_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaStddevParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_stddev_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaStddevParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_zscore_expand_grid(sweep: *const VtaZscoreBatchRange, out: *mut VtaZscoreParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_zscore_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaZscoreBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_zscore_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaZscoreBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_zscore_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaZscoreBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_zscore_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaZscoreParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_zscore_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaZscoreParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_bollinger_bands_expand_grid(sweep: *const VtaBollingerBatchRange, out: *mut VtaBollingerParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_bollinger_bands_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaBollingerBatchRange, out_upper: *mut VtaDeviceArray, out_middle: *mut VtaDeviceArray, out_lower: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_bollinger_bands_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaBollingerBatchRange, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> VtaStatus;
    pub fn vta_bollinger_bands_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaBollingerBatchRange, out_upper: *mut f32, out_middle: *mut f32, out_lower: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_bollinger_bands_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaBollingerParams, out_upper: *mut VtaDeviceArray, out_middle: *mut VtaDeviceArray, out_lower: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_bollinger_bands_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaBollingerParams, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> VtaStatus;
    pub fn vta_atr_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_atr_batch_dev(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_atr_batch_device(ctx: *mut VtaCtx, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_atr_batch_into_host_f32(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_atr_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, high_tm: *const f32, low_tm: *const f32, close_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_atr_many_series_one_param_device(ctx: *mut VtaCtx, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_adx_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_adx_batch_dev(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_adx_batch_device(ctx: *mut VtaCtx, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_adx_batch_into_host_f32(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_adx_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, high_tm: *const f32, low_tm: *const f32, close_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_adx_many_series_one_param_device(ctx: *mut VtaCtx, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_supertrend_expand_grid(sweep: *const VtaSupertrendBatchRange, out: *mut VtaSupertrendParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_supertrend_batch_dev(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaSupertrendBatchRange, out_trend: *mut VtaDeviceArray, out_changed: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_supertrend_batch_device(ctx: *mut VtaCtx, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: *const VtaSupertrendBatchRange, d_out_trend: *mut f32, d_out_changed: *mut f32) -> VtaStatus;
    pub fn vta_supertrend_batch_into_host_f32(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaSupertrendBatchRange, out_trend: *mut f32, out_changed: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_supertrend_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, high_tm: *const f32, low_tm: *const f32, close_tm: *const f32, cols: usize, rows: usize, params: *const VtaSupertrendParams, out_trend: *mut VtaDeviceArray, out_changed: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_supertrend_many_series_one_param_device(ctx: *mut VtaCtx, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: *const VtaSupertrendParams, d_out_trend: *mut f32, d_out_changed: *mut f32) -> VtaStatus;
    pub fn vta_donchian_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_donchian_batch_dev(ctx: *mut VtaCtx, high: *const f32, low: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out_upper: *mut VtaDeviceArray, out_middle: *mut VtaDeviceArray, out_lower: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_donchian_batch_device(ctx: *mut VtaCtx, d_high: *const f32, d_low: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> VtaStatus;
    pub fn vta_donchian_batch_into_host_f32(ctx: *mut VtaCtx, high: *const f32, low: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out_upper: *mut f32, out_middle: *mut f32, out_lower: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_donchian_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, high_tm: *const f32, low_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out_upper: *mut VtaDeviceArray, out_middle: *mut VtaDeviceArray, out_lower: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_donchian_many_series_one_param_device(ctx: *mut VtaCtx, d_high_tm: *const f32, d_low_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> VtaStatus;
    pub fn vta_willr_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_willr_batch_dev(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_willr_batch_device(ctx: *mut VtaCtx, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_willr_batch_into_host_f32(ctx: *mut VtaCtx, high: *const f32, low: *const f32, close: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_willr_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, high_tm: *const f32, low_tm: *const f32, close_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_willr_many_series_one_param_device(ctx: *mut VtaCtx, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_percentile_nearest_rank_expand_grid(sweep: *const VtaPercentileBatchRange, out: *mut VtaPercentileParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_percentile_nearest_rank_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPercentileBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_percentile_nearest_rank_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPercentileBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_percentile_nearest_rank_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPercentileBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_percentile_nearest_rank_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPercentileParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_percentile_nearest_rank_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPercentileParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_cwma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_cwma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_cwma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_cwma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_cwma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_cwma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_fwma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_fwma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_fwma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_fwma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_fwma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_fwma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_srwma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_srwma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_srwma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_srwma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_srwma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_srwma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_sqwma_expand_grid(sweep: *const VtaPeriodBatchRange, out: *mut VtaPeriodParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_sqwma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_sqwma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaPeriodBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_sqwma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaPeriodBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_sqwma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_sqwma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaPeriodParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_epma_expand_grid(sweep: *const VtaEpmaBatchRange, out: *mut VtaEpmaParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_epma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaEpmaBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_epma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaEpmaBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_epma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaEpmaBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_epma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaEpmaParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_epma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaEpmaParams, d_out: *mut f32) -> VtaStatus;
    pub fn vta_vpwma_expand_grid(sweep: *const VtaVpwmaBatchRange, out: *mut VtaVpwmaParams, cap: usize, n_combos: *mut usize) -> VtaStatus;
    pub fn vta_vpwma_batch_dev(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaVpwmaBatchRange, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_vpwma_batch_device(ctx: *mut VtaCtx, d_data: *const f32, len: usize, first_valid: usize, sweep: *const VtaVpwmaBatchRange, d_out: *mut f32) -> VtaStatus;
    pub fn vta_vpwma_batch_into_host_f32(ctx: *mut VtaCtx, data: *const f32, len: usize, sweep: *const VtaVpwmaBatchRange, out: *mut f32, out_len: usize, rows: *mut usize, cols: *mut usize) -> VtaStatus;
    pub fn vta_vpwma_many_series_one_param_time_major_dev(ctx: *mut VtaCtx, data_tm: *const f32, cols: usize, rows: usize, params: *const VtaVpwmaParams, out: *mut VtaDeviceArray) -> VtaStatus;
    pub fn vta_vpwma_many_series_one_param_device(ctx: *mut VtaCtx, d_data_tm: *const f32, cols: usize, rows: usize, params: *const VtaVpwmaParams, d_out: *mut f32) -> VtaStatus;
}

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

/// alma: replaces src/cuda/moving_averages/alma_wrapper.rs (CudaX::new at line 133).
pub struct CudaAlma { pub ctx: Context }
impl CudaAlma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaAlma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaAlmaBatchRange) -> Result<Vec<VtaAlmaParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_alma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaAlmaParams::default(); n];
        check(unsafe { vta_alma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn alma_batch_dev(&self, data: &[f32], sweep: &VtaAlmaBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_alma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn alma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaAlmaBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_alma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn alma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaAlmaParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_alma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn alma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaAlmaBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_alma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn alma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaAlmaParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_alma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// ema: replaces src/cuda/moving_averages/ema_wrapper.rs (CudaX::new at line 125).
pub struct CudaEma { pub ctx: Context }
impl CudaEma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaEma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_ema_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_ema_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn ema_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_ema_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn ema_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_ema_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn ema_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_ema_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn ema_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_ema_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn ema_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_ema_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// dema: replaces src/cuda/moving_averages/dema_wrapper.rs (CudaX::new at line 115).
pub struct CudaDema { pub ctx: Context }
impl CudaDema {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaDema { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_dema_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_dema_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn dema_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_dema_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn dema_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_dema_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn dema_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_dema_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn dema_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_dema_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn dema_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_dema_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// tema: replaces src/cuda/moving_averages/tema_wrapper.rs (CudaX::new at line 159).
pub struct CudaTema { pub ctx: Context }
impl CudaTema {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaTema { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_tema_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_tema_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn tema_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_tema_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn tema_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_tema_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn tema_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_tema_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn tema_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_tema_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn tema_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_tema_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// rsi: replaces src/cuda/rsi_wrapper.rs (CudaX::new at line 62).
pub struct CudaRsi { pub ctx: Context }
impl CudaRsi {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaRsi { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_rsi_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_rsi_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn rsi_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_rsi_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn rsi_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_rsi_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn rsi_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_rsi_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn rsi_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_rsi_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn rsi_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_rsi_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// wilders: replaces src/cuda/moving_averages/wilders_wrapper.rs (CudaX::new at line 101).
pub struct CudaWilders { pub ctx: Context }
impl CudaWilders {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaWilders { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_wilders_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_wilders_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn wilders_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_wilders_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn wilders_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_wilders_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn wilders_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_wilders_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn wilders_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_wilders_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn wilders_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_wilders_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// sma: replaces src/cuda/moving_averages/sma_wrapper.rs (CudaX::new at line 56).
pub struct CudaSma { pub ctx: Context }
impl CudaSma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaSma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_sma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_sma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn sma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_sma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn sma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_sma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn sma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_sma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn sma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_sma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn sma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_sma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// wma: replaces src/cuda/moving_averages/wma_wrapper.rs (CudaX::new at line 151).
pub struct CudaWma { pub ctx: Context }
impl CudaWma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaWma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_wma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_wma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn wma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_wma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn wma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_wma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn wma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_wma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn wma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_wma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn wma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_wma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// swma: replaces src/cuda/moving_averages/swma_wrapper.rs (CudaX::new at line 121).
pub struct CudaSwma { pub ctx: Context }
impl CudaSwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaSwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_swma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_swma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn swma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_swma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn swma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_swma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn swma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_swma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn swma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_swma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn swma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_swma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// pwma: replaces src/cuda/moving_averages/pwma_wrapper.rs (CudaX::new at line 93).
pub struct CudaPwma { pub ctx: Context }
impl CudaPwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaPwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_pwma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_pwma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn pwma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_pwma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn pwma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_pwma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn pwma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_pwma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn pwma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_pwma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn pwma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_pwma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// sinwma: replaces src/cuda/moving_averages/sinwma_wrapper.rs (CudaX::new at line 116).
pub struct CudaSinwma { pub ctx: Context }
impl CudaSinwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaSinwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_sinwma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_sinwma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn sinwma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_sinwma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn sinwma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_sinwma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn sinwma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_sinwma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn sinwma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_sinwma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn sinwma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_sinwma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// trima: replaces src/cuda/moving_averages/trima_wrapper.rs (CudaX::new at line 123).
pub struct CudaTrima { pub ctx: Context }
impl CudaTrima {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaTrima { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_trima_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_trima_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn trima_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_trima_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn trima_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_trima_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn trima_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_trima_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn trima_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_trima_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn trima_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_trima_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// stddev: replaces src/cuda/stddev_wrapper.rs (CudaX::new at line 101).
pub struct CudaStddev { pub ctx: Context }
impl CudaStddev {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaStddev { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaStddevBatchRange) -> Result<Vec<VtaStddevParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_stddev_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaStddevParams::default(); n];
        check(unsafe { vta_stddev_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn stddev_batch_dev(&self, data: &[f32], sweep: &VtaStddevBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_stddev_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn stddev_batch_into_host_f32(&self, data: &[f32], sweep: &VtaStddevBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_stddev_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn stddev_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaStddevParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_stddev_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn stddev_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaStddevBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_stddev_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn stddev_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaStddevParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_stddev_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// zscore: replaces src/cuda/zscore_wrapper.rs (CudaX::new at line 86).
pub struct CudaZscore { pub ctx: Context }
impl CudaZscore {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaZscore { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaZscoreBatchRange) -> Result<Vec<VtaZscoreParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_zscore_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaZscoreParams::default(); n];
        check(unsafe { vta_zscore_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn zscore_batch_dev(&self, data: &[f32], sweep: &VtaZscoreBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_zscore_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn zscore_batch_into_host_f32(&self, data: &[f32], sweep: &VtaZscoreBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_zscore_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn zscore_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaZscoreParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_zscore_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn zscore_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaZscoreBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_zscore_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn zscore_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaZscoreParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_zscore_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// bollinger_bands: replaces src/cuda/bollinger_bands_wrapper.rs (CudaX::new at line 85).
pub struct CudaBollingerBands { pub ctx: Context }
impl CudaBollingerBands {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaBollingerBands { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaBollingerBatchRange) -> Result<Vec<VtaBollingerParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_bollinger_bands_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaBollingerParams::default(); n];
        check(unsafe { vta_bollinger_bands_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn bollinger_bands_batch_dev(&self, data: &[f32], sweep: &VtaBollingerBatchRange) -> Result<(DeviceArrayF32, DeviceArrayF32, DeviceArrayF32), CudaError> {
        let mut o = [VtaDeviceArray::default(); 3];
        check(unsafe { vta_bollinger_bands_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0], &mut o[1], &mut o[2]) })?;
        Ok((DeviceArrayF32 { raw: o[0] }, DeviceArrayF32 { raw: o[1] }, DeviceArrayF32 { raw: o[2] }))
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn bollinger_bands_batch_into_host_f32(&self, data: &[f32], sweep: &VtaBollingerBatchRange, out_upper: &mut [f32], out_middle: &mut [f32], out_lower: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out_upper.len();
        if out_middle.len() < out_len { return Err(CudaError::InvalidInput("output slices of different lengths".into())); }
        if out_lower.len() < out_len { return Err(CudaError::InvalidInput("output slices of different lengths".into())); }
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_bollinger_bands_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out_upper.as_mut_ptr(), out_middle.as_mut_ptr(), out_lower.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn bollinger_bands_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaBollingerParams) -> Result<(DeviceArrayF32, DeviceArrayF32, DeviceArrayF32), CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 3];
        check(unsafe { vta_bollinger_bands_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0], &mut o[1], &mut o[2]) })?;
        Ok((DeviceArrayF32 { raw: o[0] }, DeviceArrayF32 { raw: o[1] }, DeviceArrayF32 { raw: o[2] }))
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn bollinger_bands_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaBollingerBatchRange, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> Result<(), CudaError> {
        check(vta_bollinger_bands_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out_upper, d_out_middle, d_out_lower))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn bollinger_bands_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaBollingerParams, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> Result<(), CudaError> {
        check(vta_bollinger_bands_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out_upper, d_out_middle, d_out_lower))
    }
}

/// atr: replaces src/cuda/atr_wrapper.rs (CudaX::new at line 110).
pub struct CudaAtr { pub ctx: Context }
impl CudaAtr {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaAtr { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_atr_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_atr_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn atr_batch_dev(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_atr_batch_dev(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn atr_batch_into_host_f32(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_atr_batch_into_host_f32(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn atr_many_series_one_param_time_major_dev(&self, high_tm: &[f32], low_tm: &[f32], close_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if high_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if low_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if close_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_atr_many_series_one_param_time_major_dev(self.ctx.raw(), high_tm.as_ptr(), low_tm.as_ptr(), close_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn atr_batch_device(&self, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_atr_batch_device(self.ctx.raw(), d_high, d_low, d_close, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn atr_many_series_one_param_device(&self, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_atr_many_series_one_param_device(self.ctx.raw(), d_high_tm, d_low_tm, d_close_tm, cols, rows, params, d_out))
    }
}

/// adx: replaces src/cuda/adx_wrapper.rs (CudaX::new at line 88).
pub struct CudaAdx { pub ctx: Context }
impl CudaAdx {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaAdx { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_adx_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_adx_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn adx_batch_dev(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_adx_batch_dev(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn adx_batch_into_host_f32(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_adx_batch_into_host_f32(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn adx_many_series_one_param_time_major_dev(&self, high_tm: &[f32], low_tm: &[f32], close_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if high_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if low_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if close_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_adx_many_series_one_param_time_major_dev(self.ctx.raw(), high_tm.as_ptr(), low_tm.as_ptr(), close_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn adx_batch_device(&self, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_adx_batch_device(self.ctx.raw(), d_high, d_low, d_close, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn adx_many_series_one_param_device(&self, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_adx_many_series_one_param_device(self.ctx.raw(), d_high_tm, d_low_tm, d_close_tm, cols, rows, params, d_out))
    }
}

/// supertrend: replaces src/cuda/supertrend_wrapper.rs (CudaX::new at line 88).
pub struct CudaSupertrend { pub ctx: Context }
impl CudaSupertrend {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaSupertrend { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaSupertrendBatchRange) -> Result<Vec<VtaSupertrendParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_supertrend_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaSupertrendParams::default(); n];
        check(unsafe { vta_supertrend_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn supertrend_batch_dev(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaSupertrendBatchRange) -> Result<(DeviceArrayF32, DeviceArrayF32), CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let mut o = [VtaDeviceArray::default(); 2];
        check(unsafe { vta_supertrend_batch_dev(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, &mut o[0], &mut o[1]) })?;
        Ok((DeviceArrayF32 { raw: o[0] }, DeviceArrayF32 { raw: o[1] }))
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn supertrend_batch_into_host_f32(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaSupertrendBatchRange, out_trend: &mut [f32], out_changed: &mut [f32]) -> Result<(usize, usize), CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let out_len = out_trend.len();
        if out_changed.len() < out_len { return Err(CudaError::InvalidInput("output slices of different lengths".into())); }
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_supertrend_batch_into_host_f32(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, out_trend.as_mut_ptr(), out_changed.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn supertrend_many_series_one_param_time_major_dev(&self, high_tm: &[f32], low_tm: &[f32], close_tm: &[f32], cols: usize, rows: usize, params: &VtaSupertrendParams) -> Result<(DeviceArrayF32, DeviceArrayF32), CudaError> {
        if high_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if low_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if close_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 2];
        check(unsafe { vta_supertrend_many_series_one_param_time_major_dev(self.ctx.raw(), high_tm.as_ptr(), low_tm.as_ptr(), close_tm.as_ptr(), cols, rows, params, &mut o[0], &mut o[1]) })?;
        Ok((DeviceArrayF32 { raw: o[0] }, DeviceArrayF32 { raw: o[1] }))
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn supertrend_batch_device(&self, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: &VtaSupertrendBatchRange, d_out_trend: *mut f32, d_out_changed: *mut f32) -> Result<(), CudaError> {
        check(vta_supertrend_batch_device(self.ctx.raw(), d_high, d_low, d_close, len, first_valid, sweep, d_out_trend, d_out_changed))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn supertrend_many_series_one_param_device(&self, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: &VtaSupertrendParams, d_out_trend: *mut f32, d_out_changed: *mut f32) -> Result<(), CudaError> {
        check(vta_supertrend_many_series_one_param_device(self.ctx.raw(), d_high_tm, d_low_tm, d_close_tm, cols, rows, params, d_out_trend, d_out_changed))
    }
}

/// donchian: replaces src/cuda/donchian_wrapper.rs (CudaX::new at line 128).
pub struct CudaDonchian { pub ctx: Context }
impl CudaDonchian {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaDonchian { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_donchian_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_donchian_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn donchian_batch_dev(&self, high: &[f32], low: &[f32], sweep: &VtaPeriodBatchRange) -> Result<(DeviceArrayF32, DeviceArrayF32, DeviceArrayF32), CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let mut o = [VtaDeviceArray::default(); 3];
        check(unsafe { vta_donchian_batch_dev(self.ctx.raw(), high.as_ptr(), low.as_ptr(), high.len(), sweep, &mut o[0], &mut o[1], &mut o[2]) })?;
        Ok((DeviceArrayF32 { raw: o[0] }, DeviceArrayF32 { raw: o[1] }, DeviceArrayF32 { raw: o[2] }))
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn donchian_batch_into_host_f32(&self, high: &[f32], low: &[f32], sweep: &VtaPeriodBatchRange, out_upper: &mut [f32], out_middle: &mut [f32], out_lower: &mut [f32]) -> Result<(usize, usize), CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let out_len = out_upper.len();
        if out_middle.len() < out_len { return Err(CudaError::InvalidInput("output slices of different lengths".into())); }
        if out_lower.len() < out_len { return Err(CudaError::InvalidInput("output slices of different lengths".into())); }
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_donchian_batch_into_host_f32(self.ctx.raw(), high.as_ptr(), low.as_ptr(), high.len(), sweep, out_upper.as_mut_ptr(), out_middle.as_mut_ptr(), out_lower.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn donchian_many_series_one_param_time_major_dev(&self, high_tm: &[f32], low_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<(DeviceArrayF32, DeviceArrayF32, DeviceArrayF32), CudaError> {
        if high_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if low_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 3];
        check(unsafe { vta_donchian_many_series_one_param_time_major_dev(self.ctx.raw(), high_tm.as_ptr(), low_tm.as_ptr(), cols, rows, params, &mut o[0], &mut o[1], &mut o[2]) })?;
        Ok((DeviceArrayF32 { raw: o[0] }, DeviceArrayF32 { raw: o[1] }, DeviceArrayF32 { raw: o[2] }))
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn donchian_batch_device(&self, d_high: *const f32, d_low: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> Result<(), CudaError> {
        check(vta_donchian_batch_device(self.ctx.raw(), d_high, d_low, len, first_valid, sweep, d_out_upper, d_out_middle, d_out_lower))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn donchian_many_series_one_param_device(&self, d_high_tm: *const f32, d_low_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out_upper: *mut f32, d_out_middle: *mut f32, d_out_lower: *mut f32) -> Result<(), CudaError> {
        check(vta_donchian_many_series_one_param_device(self.ctx.raw(), d_high_tm, d_low_tm, cols, rows, params, d_out_upper, d_out_middle, d_out_lower))
    }
}

/// willr: replaces src/cuda/willr_wrapper.rs (CudaX::new at line 75).
pub struct CudaWillr { pub ctx: Context }
impl CudaWillr {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaWillr { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_willr_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_willr_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn willr_batch_dev(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_willr_batch_dev(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn willr_batch_into_host_f32(&self, high: &[f32], low: &[f32], close: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        if low.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        if close.len() != high.len() { return Err(CudaError::InvalidInput("inconsistent input lengths".into())); }
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_willr_batch_into_host_f32(self.ctx.raw(), high.as_ptr(), low.as_ptr(), close.as_ptr(), high.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn willr_many_series_one_param_time_major_dev(&self, high_tm: &[f32], low_tm: &[f32], close_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if high_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if low_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        if close_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_willr_many_series_one_param_time_major_dev(self.ctx.raw(), high_tm.as_ptr(), low_tm.as_ptr(), close_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn willr_batch_device(&self, d_high: *const f32, d_low: *const f32, d_close: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_willr_batch_device(self.ctx.raw(), d_high, d_low, d_close, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn willr_many_series_one_param_device(&self, d_high_tm: *const f32, d_low_tm: *const f32, d_close_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_willr_many_series_one_param_device(self.ctx.raw(), d_high_tm, d_low_tm, d_close_tm, cols, rows, params, d_out))
    }
}

/// percentile_nearest_rank: replaces src/cuda/percentile_nearest_rank_wrapper.rs (CudaX::new at line 99).
pub struct CudaPercentileNearestRank { pub ctx: Context }
impl CudaPercentileNearestRank {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaPercentileNearestRank { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPercentileBatchRange) -> Result<Vec<VtaPercentileParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_percentile_nearest_rank_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPercentileParams::default(); n];
        check(unsafe { vta_percentile_nearest_rank_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn percentile_nearest_rank_batch_dev(&self, data: &[f32], sweep: &VtaPercentileBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_percentile_nearest_rank_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn percentile_nearest_rank_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPercentileBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_percentile_nearest_rank_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn percentile_nearest_rank_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPercentileParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_percentile_nearest_rank_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn percentile_nearest_rank_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPercentileBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_percentile_nearest_rank_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn percentile_nearest_rank_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPercentileParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_percentile_nearest_rank_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// cwma: replaces src/cuda/moving_averages/cwma_wrapper.rs (CudaX::new at line 118).
pub struct CudaCwma { pub ctx: Context }
impl CudaCwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaCwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_cwma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_cwma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn cwma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_cwma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn cwma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_cwma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn cwma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_cwma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn cwma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_cwma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn cwma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_cwma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// fwma: replaces src/cuda/moving_averages/fwma_wrapper.rs (CudaX::new at line 132).
pub struct CudaFwma { pub ctx: Context }
impl CudaFwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaFwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_fwma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_fwma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn fwma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_fwma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn fwma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_fwma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn fwma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_fwma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn fwma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_fwma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn fwma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_fwma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// srwma: replaces src/cuda/moving_averages/srwma_wrapper.rs (CudaX::new at line 176).
pub struct CudaSrwma { pub ctx: Context }
impl CudaSrwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaSrwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_srwma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_srwma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn srwma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_srwma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn srwma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_srwma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn srwma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_srwma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn srwma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_srwma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn srwma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_srwma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// sqwma: replaces src/cuda/moving_averages/sqwma_wrapper.rs (CudaX::new at line 62).
pub struct CudaSqwma { pub ctx: Context }
impl CudaSqwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaSqwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaPeriodBatchRange) -> Result<Vec<VtaPeriodParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_sqwma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaPeriodParams::default(); n];
        check(unsafe { vta_sqwma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn sqwma_batch_dev(&self, data: &[f32], sweep: &VtaPeriodBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_sqwma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn sqwma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaPeriodBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_sqwma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn sqwma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaPeriodParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_sqwma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn sqwma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaPeriodBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_sqwma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn sqwma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaPeriodParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_sqwma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// epma: replaces src/cuda/moving_averages/epma_wrapper.rs (CudaX::new at line 110).
pub struct CudaEpma { pub ctx: Context }
impl CudaEpma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaEpma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaEpmaBatchRange) -> Result<Vec<VtaEpmaParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_epma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaEpmaParams::default(); n];
        check(unsafe { vta_epma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn epma_batch_dev(&self, data: &[f32], sweep: &VtaEpmaBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_epma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn epma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaEpmaBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_epma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn epma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaEpmaParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_epma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn epma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaEpmaBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_epma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn epma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaEpmaParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_epma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

/// vpwma: replaces src/cuda/moving_averages/vpwma_wrapper.rs (CudaX::new at line 126).
pub struct CudaVpwma { pub ctx: Context }
impl CudaVpwma {
    pub fn new(device_id: usize) -> Result<Self, CudaError> { Ok(CudaVpwma { ctx: Context::new(device_id)? }) }
    pub fn synchronize(&self) -> Result<(), CudaError> { self.ctx.synchronize() }
    pub fn set_policy(&self, key: &str, value: &str) -> Result<(), CudaError> { self.ctx.set_policy(key, value) }
    pub fn expand_grid(sweep: &VtaVpwmaBatchRange) -> Result<Vec<VtaVpwmaParams>, CudaError> {
        let mut n = 0usize;
        unsafe { vta_vpwma_expand_grid(sweep, std::ptr::null_mut(), 0, &mut n) };
        let mut v = vec![VtaVpwmaParams::default(); n];
        check(unsafe { vta_vpwma_expand_grid(sweep, v.as_mut_ptr(), n, &mut n) })?;
        Ok(v)
    }
    pub fn vpwma_batch_dev(&self, data: &[f32], sweep: &VtaVpwmaBatchRange) -> Result<DeviceArrayF32, CudaError> {
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_vpwma_batch_dev(self.ctx.raw(), data.as_ptr(), data.len(), sweep, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Returns (rows, cols); every output slice holds at least rows * cols values.
    pub fn vpwma_batch_into_host_f32(&self, data: &[f32], sweep: &VtaVpwmaBatchRange, out: &mut [f32]) -> Result<(usize, usize), CudaError> {
        let out_len = out.len();
        let (mut rows, mut cols) = (0usize, 0usize);
        check(unsafe { vta_vpwma_batch_into_host_f32(self.ctx.raw(), data.as_ptr(), data.len(), sweep, out.as_mut_ptr(), out_len, &mut rows, &mut cols) })?;
        Ok((rows, cols))
    }
    /// Time-major [rows][cols] input (element (t, s) at t * cols + s).
    pub fn vpwma_many_series_one_param_time_major_dev(&self, data_tm: &[f32], cols: usize, rows: usize, params: &VtaVpwmaParams) -> Result<DeviceArrayF32, CudaError> {
        if data_tm.len() < cols * rows { return Err(CudaError::InvalidInput("input shorter than cols * rows".into())); }
        let mut o = [VtaDeviceArray::default(); 1];
        check(unsafe { vta_vpwma_many_series_one_param_time_major_dev(self.ctx.raw(), data_tm.as_ptr(), cols, rows, params, &mut o[0]) })?;
        Ok(DeviceArrayF32 { raw: o[0] })
    }
    /// Device inputs and caller-provided device outputs (x_batch_device).
    /// # Safety: the pointers address device buffers of len and n_combos * len floats.
    pub unsafe fn vpwma_batch_device(&self, d_data: *const f32, len: usize, first_valid: usize, sweep: &VtaVpwmaBatchRange, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_vpwma_batch_device(self.ctx.raw(), d_data, len, first_valid, sweep, d_out))
    }
    /// # Safety: the pointers address device buffers of cols * rows floats.
    pub unsafe fn vpwma_many_series_one_param_device(&self, d_data_tm: *const f32, cols: usize, rows: usize, params: &VtaVpwmaParams, d_out: *mut f32) -> Result<(), CudaError> {
        check(vta_vpwma_many_series_one_param_device(self.ctx.raw(), d_data_tm, cols, rows, params, d_out))
    }
}

