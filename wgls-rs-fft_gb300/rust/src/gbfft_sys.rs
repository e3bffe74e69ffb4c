//! Raw bindings: one `extern "C"` declaration per function of include/gbfft.h, in the
//! header's order, and its constants.  tests/test_rust_crate.py parses this file and
//! checks every declaration and constant against the header, so the two cannot drift.
#![allow(dead_code)]
use std::os::raw::{c_char, c_int, c_void};

pub const GBFFT_FORWARD: c_int = -1;
pub const GBFFT_INVERSE: c_int = 1;

pub const GBFFT_OK: c_int = 0;
pub const GBFFT_ERR_INVALID_SIZE: c_int = 1;
pub const GBFFT_ERR_LENGTH_MISMATCH: c_int = 2;
pub const GBFFT_ERR_INVALID_ARGUMENT: c_int = 3;
pub const GBFFT_ERR_NO_DEVICE: c_int = 4;
pub const GBFFT_ERR_OUT_OF_MEMORY: c_int = 5;
pub const GBFFT_ERR_CUDA: c_int = 6;
pub const GBFFT_ERR_TIMEOUT: c_int = 7;
pub const GBFFT_ERR_UNSUPPORTED: c_int = 8;

pub const GBFFT_PREC_FP32: c_int = 0;
pub const GBFFT_PREC_TC_FP16: c_int = 1;
pub const GBFFT_PREC_TC_BF16X3: c_int = 2;
pub const GBFFT_PREC_TC_TF32: c_int = 3;
pub const GBFFT_PREC_TC_BF16X6: c_int = 4;

pub const GBFFT_RAGGED_OPT_SPIN_LIMIT: c_int = 1;
pub const GBFFT_RAGGED_OPT_TEST_DROP_PRODUCERS: c_int = 2;
pub const GBFFT_RAGGED_OPT_LAG: c_int = 3;

pub const GBFFT_WINDOW_NONE: c_int = 0;
pub const GBFFT_WINDOW_HANN: c_int = 1;

/// Opaque `gbfft_ctx`.
#[repr(C)]
pub struct GbfftCtx {
    _p: [u8; 0],
}

/// Opaque `gbfft_ragged_plan`.
#[repr(C)]
pub struct GbfftRaggedPlan {
    _p: [u8; 0],
}

/// `gbfft_ragged_desc`: one transform of a ragged batch.
#[repr(C)]
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub struct GbfftRaggedDesc {
    pub offset: u64,
    pub log2n: u32,
    pub direction: i32,
}

extern "C" {
    pub fn gbfft_is_available() -> c_int;
    pub fn gbfft_create(device: c_int, out_ctx: *mut *mut GbfftCtx) -> c_int;
    pub fn gbfft_destroy(ctx: *mut GbfftCtx);
    pub fn gbfft_last_error(ctx: *const GbfftCtx) -> *const c_char;
    pub fn gbfft_status_string(status: c_int) -> *const c_char;
    pub fn gbfft_c2c_host(ctx: *mut GbfftCtx, input: *const f32, out: *mut f32, n: u64, batch: u64,
                          direction: c_int) -> c_int;
    pub fn gbfft_c2c_host_rows(ctx: *mut GbfftCtx, in_rows: *const *const f32, row_lengths: *const u64,
                               out_rows: *const *mut f32, batch: u64, direction: c_int) -> c_int;
    pub fn gbfft_c2c_device(ctx: *mut GbfftCtx, d_in: *const c_void, d_out: *mut c_void, n: u64, batch: u64,
                            direction: c_int, stream: *mut c_void) -> c_int;
    pub fn gbfft_c2c_device_noalloc(d_in: *const c_void, d_out: *mut c_void, n: u64, batch: u64,
                                    direction: c_int, stream: *mut c_void) -> c_int;
    pub fn gbfft_ragged_plan_create(ctx: *mut GbfftCtx, descs: *const GbfftRaggedDesc, count: u32,
                                    out_plan: *mut *mut GbfftRaggedPlan) -> c_int;
    pub fn gbfft_ragged_plan_set(plan: *mut GbfftRaggedPlan, option: c_int, value: u64) -> c_int;
    pub fn gbfft_ragged_execute(plan: *mut GbfftRaggedPlan, d_in: *const c_void, d_out: *mut c_void,
                                capacity: u64, use_graph: c_int, stream: *mut c_void) -> c_int;
    pub fn gbfft_ragged_wait(plan: *mut GbfftRaggedPlan, stream: *mut c_void) -> c_int;
    pub fn gbfft_ragged_launch_count(plan: *const GbfftRaggedPlan) -> u64;
    pub fn gbfft_ragged_plan_destroy(plan: *mut GbfftRaggedPlan);
    pub fn gbfft_ragged_device(ctx: *mut GbfftCtx, d_in: *const c_void, d_out: *mut c_void, capacity: u64,
                               descs: *const GbfftRaggedDesc, count: u32, stream: *mut c_void) -> c_int;
    pub fn gbfft_bench_device(ctx: *mut GbfftCtx, n: u64, batch: u64, direction: c_int, warmup: c_int,
                              iters: c_int, seconds_per_iter: *mut f64) -> c_int;
    pub fn gbfft_set_precision(ctx: *mut GbfftCtx, precision: c_int) -> c_int;
    pub fn gbfft_set_window(ctx: *mut GbfftCtx, window: c_int) -> c_int;
    pub fn gbfft_set_noise(ctx: *mut GbfftCtx, seed: u32, sigma: f32) -> c_int;
    pub fn gbfft_autotune(ctx: *mut GbfftCtx, n: u64, batch: u64, direction: c_int,
                          best_seconds: *mut f64) -> c_int;
    pub fn gbfft_launch_count(ctx: *const GbfftCtx) -> u64;
    pub fn gbfft_version() -> *const c_char;
}
