//! Builds libgbfft.so from the CUDA sources with nvcc for sm_103a and links it.
//!
//! GBFFT_LIB_DIR=<dir> skips the build and links an existing libgbfft.so from <dir>
//! (for example wgls-rs-fft_gb300/lib, where the Python build puts it).
//! NVCC=<path> selects the compiler (default: nvcc on PATH, then /usr/local/cuda/bin/nvcc).
use std::env;
use std::path::{Path, PathBuf};
use std::process::Command;

fn main() {
    println!("cargo:rerun-if-env-changed=GBFFT_LIB_DIR");
    println!("cargo:rerun-if-env-changed=NVCC");
    if let Ok(dir) = env::var("GBFFT_LIB_DIR") {
        link(Path::new(&dir));
        return;
    }
    let crate_dir = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
    let pkg = crate_dir.parent().unwrap(); // wgls-rs-fft_gb300/
    let csrc = pkg.join("csrc");
    let include = pkg.parent().unwrap().join("include");
    let out = PathBuf::from(env::var("OUT_DIR").unwrap());
    let nvcc = env::var("NVCC").unwrap_or_else(|_| {
        if Command::new("nvcc").arg("--version").output().is_ok() {
            "nvcc".to_string()
        } else {
            "/usr/local/cuda/bin/nvcc".to_string()
        }
    });

    let mut sources: Vec<PathBuf> = std::fs::read_dir(&csrc)
        .expect("wgls-rs-fft_gb300/csrc not found")
        .filter_map(|e| e.ok().map(|e| e.path()))
        .filter(|p| p.extension().map_or(false, |x| x == "cu"))
        .collect();
    sources.sort();
    for entry in std::fs::read_dir(&csrc).unwrap().flatten() {
        println!("cargo:rerun-if-changed={}", entry.path().display());
    }
    println!("cargo:rerun-if-changed={}", include.join("gbfft.h").display());

    // One object per translation unit, then one shared library (the same flags as
    // the Python build: sm_103a only, C++20, relaxed constexpr, position independent).
    let mut objects = Vec::new();
    for src in &sources {
        let obj = out.join(src.file_stem().unwrap()).with_extension("o");
        let status = Command::new(&nvcc)
            .args(["-gencode", "arch=compute_103a,code=sm_103a", "-std=c++20", "-O3", "-lineinfo"])
            .args(["-Xcompiler", "-fPIC", "--expt-relaxed-constexpr", "-I"])
            .arg(&include)
            .arg("-c")
            .arg(src)
            .arg("-o")
            .arg(&obj)
            .status()
            .expect("failed to run nvcc");
        assert!(status.success(), "nvcc failed on {}", src.display());
        objects.push(obj);
    }
    let lib = out.join("libgbfft.so");
    let status = Command::new(&nvcc)
        .args(["-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o"])
        .arg(&lib)
        .args(&objects)
        .arg("-lcudart")
        .status()
        .expect("failed to run nvcc");
    assert!(status.success(), "linking libgbfft.so failed");
    link(&out);
}

fn link(dir: &Path) {
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=gbfft");
    // let binaries find the library without LD_LIBRARY_PATH
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", dir.display());
}
