//! Raw bindings of the C ABI in `include/fuelg.h`, one declaration per
//! exported symbol.  Every function returns `FUELG_OK` (0) or a status code;
//! `fuelg_last_error()` then holds a message for the calling thread.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const FUELG_OK: c_int = 0;
pub const FUELG_EINVAL: c_int = 1;
pub const FUELG_ENOMEM: c_int = 2;
pub const FUELG_ECUDA: c_int = 3;
pub const FUELG_ECANCELLED: c_int = 4;
pub const FUELG_ENOTSUP: c_int = 5;
pub const FUELG_ENODEV: c_int = 6;
pub const FUELG_ETIMEOUT: c_int = 7;

pub const FUELG_METRIC_SQEUCLIDEAN: i32 = 0;
pub const FUELG_METRIC_EUCLIDEAN: i32 = 1;
pub const FUELG_ORDER_ARM: i32 = 0;
pub const FUELG_ORDER_X86: i32 = 1;
pub const FUELG_EXCLUDE_NONE: i32 = 0;
pub const FUELG_EXCLUDE_LINEAR: i32 = 1;
pub const FUELG_EXCLUDE_KPLUS1: i32 = 2;
pub const FUELG_PREC_AUTO: i32 = -1;
pub const FUELG_PREC_FP32: i32 = 0;
pub const FUELG_PREC_BF16: i32 = 1;
pub const FUELG_PREC_SPLIT_BF16: i32 = 2;
pub const FUELG_PREC_SPLIT_BF16_SCALED: i32 = 3;
pub const FUELG_PREC_F16: i32 = 4;
/// Reported by the float64 calls (the exact FP64 scan); not a request value.
pub const FUELG_PREC_FP64: i32 = 5;
pub const FUELG_LLOYD_FIXED_ITERS: i32 = 1;
pub const FUELG_PAIRWISE_CONDENSED: i32 = 0;
pub const FUELG_PAIRWISE_SQUARE: i32 = 1;

/// The summation profile fuel compiles for the host this crate is built for.
pub const FUELG_ORDER_HOST: i32 = if cfg!(target_arch = "x86_64") { FUELG_ORDER_X86 } else { FUELG_ORDER_ARM };

#[repr(C)]
pub struct fuelg_index {
    _p: [u8; 0],
}
#[repr(C)]
pub struct fuelg_range_result {
    _p: [u8; 0],
}
#[repr(C)]
pub struct fuelg_server {
    _p: [u8; 0],
}

#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct fuelg_stats {
    pub device_ms: f64,
    pub h2d_bytes: i64,
    pub d2h_bytes: i64,
    pub distance_evals: i64,
    pub rescored: i64,
    pub iterations: i32,
    pub precision_used: i32,
    pub hot_kernel_ms: f64,
    pub hot_kernel_launches: i32,
    pub kernel_launches: i32,
}

#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct fuelg_error_report {
    pub max_abs_err: f64,
    pub max_rel_err: f64,
    pub pairs: i64,
    pub near_ties: i64,
    pub order_flips: i64,
}

#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct fuelg_kmeans_problem {
    pub data: *const f32,
    pub n: i64,
    pub d: i32,
    pub k: i32,
    pub init: *const f32,
    pub out_centers: *mut f32,
    pub out_labels: *mut i64,
    pub out_iters: i32,
    pub status: i32,
    pub out_inertia: f64,
}

#[repr(C)]
#[derive(Debug, Clone, Copy)]
pub struct fuelg_knn_set {
    pub data: *const f32,
    pub n: i64,
    pub d: i32,
    pub metric: i32,
    pub queries: *const f32,
    pub m: i64,
    pub k: i32,
    pub exclude_mode: i32,
    pub out_idx: *mut i64,
    pub out_dist: *mut f32,
    pub status: i32,
    pub reserved: i32,
}

#[link(name = "fuelg")]
unsafe extern "C" {
    pub fn fuelg_last_error() -> *const c_char;
    pub fn fuelg_version() -> *const c_char;
    pub fn fuelg_device_count(out_count: *mut i32) -> c_int;

    pub fn fuelg_index_create(data: *const f32, n: i64, d: i32, metric: i32, order: i32,
                              out: *mut *mut fuelg_index) -> c_int;
    pub fn fuelg_index_destroy(index: *mut fuelg_index) -> c_int;
    pub fn fuelg_index_info(index: *const fuelg_index, n: *mut i64, d: *mut i32, metric: *mut i32,
                            order: *mut i32) -> c_int;

    pub fn fuelg_knn(index: *mut fuelg_index, queries: *const f32, m: i64, k: i32, exclude_mode: i32,
                     precision: i32, out_idx: *mut i64, out_dist: *mut f32, stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_knn_ties(index: *mut fuelg_index, queries: *const f32, m: i64, k: i32, exclude_mode: i32,
                          precision: i32, out: *mut *mut fuelg_range_result, stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_knn_batched(sets: *mut fuelg_knn_set, count: i32, order: i32, precision: i32,
                             stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_knn_error(index: *mut fuelg_index, queries: *const f32, m: i64, k: i32, idx: *const i64,
                           dist: *const f32, out: *mut fuelg_error_report) -> c_int;
    pub fn fuelg_fp32_rate(tera_fma_per_s: *mut f64) -> c_int;

    pub fn fuelg_range(index: *mut fuelg_index, queries: *const f32, m: i64, radius: f64, exclude_self: i32,
                       out: *mut *mut fuelg_range_result, stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_range_size(res: *const fuelg_range_result, m: *mut i64, total: *mut i64) -> c_int;
    pub fn fuelg_range_copy(res: *const fuelg_range_result, offsets: *mut i64, idx: *mut i64,
                            dist: *mut f32) -> c_int;
    pub fn fuelg_range_free(res: *mut fuelg_range_result) -> c_int;

    pub fn fuelg_pairwise(x: *const f32, n: i64, d: i32, metric: i32, order: i32, form: i32, out: *mut f32,
                          stats: *mut fuelg_stats) -> c_int;

    // float64 data (build_linear_scan_f64, python/search.rs:1371-1389): the exact FP64 scan
    pub fn fuelg_index_create_f64(data: *const f64, n: i64, d: i32, metric: i32, order: i32,
                                  out: *mut *mut fuelg_index) -> c_int;
    pub fn fuelg_knn_f64(index: *mut fuelg_index, queries: *const f64, m: i64, k: i32, exclude_mode: i32,
                         out_idx: *mut i64, out_dist: *mut f64, stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_knn_ties_f64(index: *mut fuelg_index, queries: *const f64, m: i64, k: i32, exclude_mode: i32,
                              out: *mut *mut fuelg_range_result, stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_range_f64(index: *mut fuelg_index, queries: *const f64, m: i64, radius: f64, exclude_self: i32,
                           out: *mut *mut fuelg_range_result, stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_range_copy_f64(res: *const fuelg_range_result, offsets: *mut i64, idx: *mut i64,
                                dist: *mut f64) -> c_int;
    pub fn fuelg_pairwise_f64(x: *const f64, n: i64, d: i32, metric: i32, order: i32, form: i32, out: *mut f64,
                              stats: *mut fuelg_stats) -> c_int;

    pub fn fuelg_kmeans_lloyd(data: *const f32, n: i64, d: i32, k: i32, init_centers: *const f32,
                              max_iter: i32, tol: f64, precision: i32, order: i32, flags: i32,
                              out_centers: *mut f32, out_labels: *mut i64, out_iters: *mut i32,
                              out_inertia: *mut f64, stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_lloyd_assign(data: *const f32, n: i64, d: i32, centers: *const f32, k: i32, initial: i32,
                              order: i32, out_labels: *mut i64, out_best: *mut f32,
                              stats: *mut fuelg_stats) -> c_int;
    pub fn fuelg_kmeans_batched(problems: *mut fuelg_kmeans_problem, count: i32, max_iter: i32, order: i32,
                                precision: i32, flags: i32, stats: *mut fuelg_stats) -> c_int;

    pub fn fuelg_server_create(index: *mut fuelg_index, precision: i32, max_batch_queries: i64,
                               budget_bytes: i64, workers: i32, out: *mut *mut fuelg_server) -> c_int;
    pub fn fuelg_server_submit(s: *mut fuelg_server, queries: *const f32, m: i64, k: i32, out_idx: *mut i64,
                               out_dist: *mut f32, request_id: *mut i64) -> c_int;
    pub fn fuelg_server_wait(s: *mut fuelg_server, request_id: i64, timeout_ms: i32,
                             latency_ms: *mut f64) -> c_int;
    pub fn fuelg_server_stats(s: *mut fuelg_server, batches: *mut i64, queries: *mut i64,
                              max_batch_rows: *mut i64, max_batch_requests: *mut i64,
                              device_ms: *mut f64) -> c_int;
    pub fn fuelg_server_destroy(s: *mut fuelg_server) -> c_int;

    pub fn fuelg_knn_noalloc(data: *const f32, n: i64, d: i32, queries: *const f32, m: i64, k: i32,
                             metric: i32, order: i32, exclude_mode: i32, out_idx: *mut i64,
                             out_dist: *mut f32, stream: *mut c_void) -> c_int;

    pub fn fuelg_cancel() -> c_int;
    pub fn fuelg_reset_cancel() -> c_int;
    pub fn fuelg_release() -> c_int;
}

/// The message of the calling thread's last failing call.
pub fn last_error() -> String {
    unsafe {
        let p = fuelg_last_error();
        if p.is_null() { String::new() } else { std::ffi::CStr::from_ptr(p).to_string_lossy().into_owned() }
    }
}

/// `Ok(())` for FUELG_OK, else the status with its message.
pub fn check(rc: c_int) -> Result<(), String> {
    if rc == FUELG_OK { Ok(()) } else { Err(format!("fuelg error {rc}: {}", last_error())) }
}
