//! Forward and inverse transform of a small batch through the drop-in `GpuFft`,
//! the way the reference's examples use it (examples/test_batch_processing.rs).
use num_complex::Complex;
use wgls_rs_fft::{FftExecutor, GpuFft};

fn main() -> Result<(), Box<dyn std::error::Error>> {
    if !GpuFft::is_gpu_available() {
        eprintln!("no GB300 device");
        return Ok(());
    }
    let fft = GpuFft::new()?;
    let n = 4096;
    let rows: Vec<Vec<Complex<f32>>> = (0..8)
        .map(|r| (0..n).map(|i| Complex::new(((i * (r + 1)) as f32 * 0.01).sin(), 0.0)).collect())
        .collect();
    let spec = fft.fft(&rows)?;
    let back = fft.ifft(&spec)?;
    let err = back
        .iter()
        .zip(&rows)
        .flat_map(|(a, b)| a.iter().zip(b).map(|(u, v)| (u - v).norm()))
        .fold(0.0f32, f32::max);
    println!("{}: {} rows of {}, roundtrip max error {:.2e}", fft.name(), rows.len(), n, err);
    Ok(())
}
