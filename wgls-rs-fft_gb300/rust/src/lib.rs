//! GB300-native drop-in for wgls-rs-fft's `GpuFft`.
//!
//! The public surface is the reference's (src/lib.rs): the `FftExecutor` trait
//! (:32-45), `GpuFft::new` (:285-330), `GpuFft::is_gpu_available` (:381-389),
//! `GpuFft::fft` / `GpuFft::ifft` over `&[Vec<Complex<f32>>]` with the 1/N-scaled
//! inverse (:433-438, 483-488), and `Default` (:946-950).  Errors carry the
//! reference's own messages ("Transform length must be a non-zero power of two",
//! "All input vectors in a batch must have the same length"), and an empty batch
//! returns an empty result (:522-524).
//!
//! Everything runs in libgbfft.so (CUDA kernels for sm_103a) through the C ABI of
//! include/gbfft.h; there is no CPU path.  `GpuFftTrait` (:48-68) exposes wgpu types
//! and has no counterpart; its GPU-only timer is `GpuFft::benchmark_gpu_only`, and
//! the device-resident and ragged entries are new.
use num_complex::Complex;
use std::any::Any;
use std::error::Error;
use std::ffi::CStr;
use std::os::raw::c_void;

pub mod gbfft_sys;
use gbfft_sys::*;

/// Butterfly arithmetic (`gbfft_set_precision`).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum Precision {
    /// Plain FP32 Stockham form (every size).
    Fp32,
    /// Radix-16 sub-DFTs on tcgen05 tensor cores, FP16 hi+lo operands, FP32 accumulation.
    TcFp16,
    /// The same with BF16 hi+lo operands.
    TcBf16x3,
    /// The same with TF32 hi+lo operands.
    TcTf32,
    /// BF16 operands split in three (hi + mid + lo), six products.
    TcBf16x6,
}

impl Precision {
    fn code(self) -> i32 {
        match self {
            Precision::Fp32 => GBFFT_PREC_FP32,
            Precision::TcFp16 => GBFFT_PREC_TC_FP16,
            Precision::TcBf16x3 => GBFFT_PREC_TC_BF16X3,
            Precision::TcTf32 => GBFFT_PREC_TC_TF32,
            Precision::TcBf16x6 => GBFFT_PREC_TC_BF16X6,
        }
    }
}

/// Trait for FFT implementations that can be benchmarked (the reference's
/// `FftExecutor`, src/lib.rs:32-45, unchanged).
pub trait FftExecutor {
    fn name(&self) -> &str;
    fn fft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>>;
    fn ifft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>>;
    fn as_any(&self) -> &dyn Any;
}

/// GPU FFT engine on GB300.  Like the reference (a `RefCell` plan cache) it is
/// `!Sync`: use one instance per thread.
pub struct GpuFft {
    ctx: *mut GbfftCtx,
}

fn status_msg(st: i32) -> String {
    unsafe { CStr::from_ptr(gbfft_status_string(st)) }.to_string_lossy().into_owned()
}

impl GpuFft {
    /// Opens device 0 (src/lib.rs:285-330 picks the high-performance adapter).
    pub fn new() -> Result<Self, Box<dyn Error>> {
        Self::on_device(0)
    }

    /// Opens the given CUDA device.
    pub fn on_device(device: i32) -> Result<Self, Box<dyn Error>> {
        let mut ctx = std::ptr::null_mut();
        let st = unsafe { gbfft_create(device, &mut ctx) };
        if st != GBFFT_OK {
            return Err(status_msg(st).into());
        }
        Ok(Self { ctx })
    }

    /// True when a usable GB300 (sm_103) device is present.
    pub fn is_gpu_available() -> bool {
        unsafe { gbfft_is_available() != 0 }
    }

    /// Forward FFT of each row, unscaled: X_k = sum_n x_n e^{-2 pi i k n / N}.
    pub fn fft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>> {
        self.transform_rows(inputs, GBFFT_FORWARD)
    }

    /// Inverse FFT of each row, scaled by 1/N.
    pub fn ifft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>> {
        self.transform_rows(inputs, GBFFT_INVERSE)
    }

    fn transform_rows(
        &self,
        inputs: &[Vec<Complex<f32>>],
        direction: i32,
    ) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>> {
        if inputs.is_empty() {
            return Ok(Vec::new());
        }
        // Output rows are allocated at the input lengths; the library checks the
        // lengths (power of two, all equal) in the reference's order before it
        // touches anything.
        let mut out: Vec<Vec<Complex<f32>>> =
            inputs.iter().map(|r| vec![Complex::new(0.0, 0.0); r.len()]).collect();
        let ins: Vec<*const f32> = inputs.iter().map(|r| r.as_ptr() as *const f32).collect();
        let lens: Vec<u64> = inputs.iter().map(|r| r.len() as u64).collect();
        let outs: Vec<*mut f32> = out.iter_mut().map(|r| r.as_mut_ptr() as *mut f32).collect();
        let st = unsafe {
            gbfft_c2c_host_rows(self.ctx, ins.as_ptr(), lens.as_ptr(), outs.as_ptr(), inputs.len() as u64, direction)
        };
        self.check(st)?;
        Ok(out)
    }

    /// `fft` (or, with `inverse`, `ifft`) into caller-provided rows of the
    /// inputs' lengths; `outputs[i]` may be `inputs[i]`'s length-matched
    /// buffer from an earlier call.  Reused output rows stay resident, so the
    /// GPU writes them at the host link's rate; a freshly allocated row of
    /// 128 KB or more has its absent pages populated by the library first.
    pub fn transform_into(
        &self,
        inputs: &[Vec<Complex<f32>>],
        outputs: &mut [Vec<Complex<f32>>],
        inverse: bool,
    ) -> Result<(), Box<dyn Error>> {
        if outputs.len() != inputs.len() || inputs.iter().zip(outputs.iter()).any(|(a, b)| a.len() != b.len()) {
            return Err(status_msg(GBFFT_ERR_INVALID_ARGUMENT).into());
        }
        if inputs.is_empty() {
            return Ok(());
        }
        let dir = if inverse { GBFFT_INVERSE } else { GBFFT_FORWARD };
        let ins: Vec<*const f32> = inputs.iter().map(|r| r.as_ptr() as *const f32).collect();
        let lens: Vec<u64> = inputs.iter().map(|r| r.len() as u64).collect();
        let outs: Vec<*mut f32> = outputs.iter_mut().map(|r| r.as_mut_ptr() as *mut f32).collect();
        let st = unsafe {
            gbfft_c2c_host_rows(self.ctx, ins.as_ptr(), lens.as_ptr(), outs.as_ptr(), inputs.len() as u64, dir)
        };
        self.check(st)
    }

    /// A contiguous batch (`batch` rows of `n` samples, row-major) in one call.
    pub fn fft_contiguous(
        &self,
        input: &[Complex<f32>],
        output: &mut [Complex<f32>],
        n: usize,
        inverse: bool,
    ) -> Result<(), Box<dyn Error>> {
        if n == 0 || input.len() % n != 0 || output.len() != input.len() {
            return Err(status_msg(GBFFT_ERR_INVALID_ARGUMENT).into());
        }
        let dir = if inverse { GBFFT_INVERSE } else { GBFFT_FORWARD };
        let st = unsafe {
            gbfft_c2c_host(self.ctx, input.as_ptr() as *const f32, output.as_mut_ptr() as *mut f32, n as u64,
                           (input.len() / n) as u64, dir)
        };
        self.check(st)
    }

    /// Device-resident transform: `d_in` / `d_out` are device pointers to
    /// `batch * n` interleaved complex<f32> (8-byte aligned; they may alias),
    /// enqueued on `stream` (a cudaStream_t, null for the default stream).
    ///
    /// # Safety
    /// The pointers must be valid device allocations of that size on the
    /// context's device, and must stay alive until the stream has run the work.
    pub unsafe fn fft_device(
        &self,
        d_in: *const c_void,
        d_out: *mut c_void,
        n: u64,
        batch: u64,
        inverse: bool,
        stream: *mut c_void,
    ) -> Result<(), Box<dyn Error>> {
        let dir = if inverse { GBFFT_INVERSE } else { GBFFT_FORWARD };
        self.check(gbfft_c2c_device(self.ctx, d_in, d_out, n, batch, dir, stream))
    }

    /// GPU-only timing (replaces `GpuFftTrait::benchmark_gpu_only`,
    /// src/lib.rs:673-707): mean seconds per forward transform of an
    /// `n` x `batch` device batch, CUDA events, after `warmup` untimed ones.
    pub fn benchmark_gpu_only(&self, n: usize, batch: usize, warmup: usize, iters: usize) -> Result<f64, Box<dyn Error>> {
        let mut sec = 0.0f64;
        let st = unsafe {
            gbfft_bench_device(self.ctx, n as u64, batch as u64, GBFFT_FORWARD, warmup as i32, iters as i32, &mut sec)
        };
        self.check(st)?;
        Ok(sec)
    }

    /// Select the butterfly arithmetic for later calls.
    pub fn set_precision(&self, precision: Precision) -> Result<(), Box<dyn Error>> {
        self.check(unsafe { gbfft_set_precision(self.ctx, precision.code()) })
    }

    /// Hann window fused into every transform's load (`false` turns it off).
    pub fn set_hann_window(&self, on: bool) -> Result<(), Box<dyn Error>> {
        let w = if on { GBFFT_WINDOW_HANN } else { GBFFT_WINDOW_NONE };
        self.check(unsafe { gbfft_set_window(self.ctx, w) })
    }

    /// The pipeline's PCG/Box-Muller noise added on load (sigma 0 turns it off).
    pub fn set_noise(&self, seed: u32, sigma: f32) -> Result<(), Box<dyn Error>> {
        self.check(unsafe { gbfft_set_noise(self.ctx, seed, sigma) })
    }

    /// Time every plan variant for the shape; the fastest serves later calls.
    pub fn autotune(&self, n: usize, batch: usize, inverse: bool) -> Result<f64, Box<dyn Error>> {
        let dir = if inverse { GBFFT_INVERSE } else { GBFFT_FORWARD };
        let mut sec = 0.0f64;
        self.check(unsafe { gbfft_autotune(self.ctx, n as u64, batch as u64, dir, &mut sec) })?;
        Ok(sec)
    }

    /// A ragged batch (mixed sizes and directions) planned for one persistent launch.
    pub fn ragged_plan(&self, descs: &[GbfftRaggedDesc]) -> Result<RaggedPlan<'_>, Box<dyn Error>> {
        let mut plan = std::ptr::null_mut();
        let st = unsafe { gbfft_ragged_plan_create(self.ctx, descs.as_ptr(), descs.len() as u32, &mut plan) };
        self.check(st)?;
        Ok(RaggedPlan { owner: self, plan })
    }

    /// Kernel launches issued by this instance so far.
    pub fn launch_count(&self) -> u64 {
        unsafe { gbfft_launch_count(self.ctx) }
    }

    fn check(&self, st: i32) -> Result<(), Box<dyn Error>> {
        if st == GBFFT_OK {
            return Ok(());
        }
        let m = unsafe { CStr::from_ptr(gbfft_last_error(self.ctx)) }.to_string_lossy().into_owned();
        Err(if m.is_empty() { status_msg(st) } else { m }.into())
    }
}

impl Drop for GpuFft {
    fn drop(&mut self) {
        unsafe { gbfft_destroy(self.ctx) }
    }
}

impl Default for GpuFft {
    fn default() -> Self {
        Self::new().expect("No GPU available for default GpuFft instance")
    }
}

impl FftExecutor for GpuFft {
    fn name(&self) -> &str {
        "GB300 (sm_103a Stockham radix-16)"
    }
    fn fft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>> {
        GpuFft::fft(self, inputs)
    }
    fn ifft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>> {
        GpuFft::ifft(self, inputs)
    }
    fn as_any(&self) -> &dyn Any {
        self
    }
}

/// A `gbfft_ragged_plan` tied to the `GpuFft` that made it.
pub struct RaggedPlan<'a> {
    owner: &'a GpuFft,
    plan: *mut GbfftRaggedPlan,
}

impl RaggedPlan<'_> {
    /// Enqueue the plan (optionally as a CUDA graph replay) on `stream`.
    ///
    /// # Safety
    /// `d_in` / `d_out` must be device buffers of `capacity` complex samples.
    pub unsafe fn execute(
        &self,
        d_in: *const c_void,
        d_out: *mut c_void,
        capacity: u64,
        use_graph: bool,
        stream: *mut c_void,
    ) -> Result<(), Box<dyn Error>> {
        self.owner.check(gbfft_ragged_execute(self.plan, d_in, d_out, capacity, use_graph as i32, stream))
    }

    /// Wait for the stream; reports a dependency wait that gave up.
    pub fn wait(&self, stream: *mut c_void) -> Result<(), Box<dyn Error>> {
        self.owner.check(unsafe { gbfft_ragged_wait(self.plan, stream) })
    }
}

impl Drop for RaggedPlan<'_> {
    fn drop(&mut self) {
        unsafe { gbfft_ragged_plan_destroy(self.plan) }
    }
}

#[cfg(test)]
mod tests {
    //! The reference's own unit checks (src/lib.rs:207-227; tests/gpu_fft_test.rs;
    //! tests/ifft_test.rs), run on a GB300.
    use super::*;

    #[test]
    fn roundtrip_within_1e_4() {
        let fft = GpuFft::new().expect("GPU required");
        let x: Vec<Complex<f32>> = (0..1024).map(|i| Complex::new(i as f32 / 1024.0, 0.0)).collect();
        let spec = fft.fft(&[x.clone()]).unwrap();
        let back = fft.ifft(&spec).unwrap();
        for (a, b) in back[0].iter().zip(&x) {
            assert!((a - b).norm() < 1e-4);
        }
    }

    #[test]
    fn impulse_has_flat_spectrum() {
        let fft = GpuFft::new().expect("GPU required");
        let mut x = vec![Complex::new(0.0f32, 0.0); 256];
        x[0] = Complex::new(1.0, 0.0);
        for v in &fft.fft(&[x]).unwrap()[0] {
            assert!((v.norm() - 1.0).abs() < 1e-3);
        }
    }

    #[test]
    fn errors_and_empty_batch() {
        let fft = GpuFft::new().expect("GPU required");
        assert!(fft.fft(&[]).unwrap().is_empty());
        let e = fft.fft(&[vec![Complex::new(0.0f32, 0.0); 6]]).unwrap_err();
        assert_eq!(e.to_string(), "Transform length must be a non-zero power of two");
        let e = fft
            .fft(&[vec![Complex::new(0.0f32, 0.0); 8], vec![Complex::new(0.0f32, 0.0); 16]])
            .unwrap_err();
        assert_eq!(e.to_string(), "All input vectors in a batch must have the same length");
    }
}
