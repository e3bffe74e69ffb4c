"""CPU: the Rust drop-in crate (wgls-rs-fft_gb300/rust) against the C header.

There is no cargo here, so the crate is not compiled; this test keeps its
hand-written `extern "C"` block and constants in step with include/gbfft.h:
every function the header declares is declared in the crate with the same
parameter count, the Rust type each C type maps to, and the same return
type; every status, precision, window and ragged-option constant has the
header's value; and the crate keeps the reference's public surface
(FftExecutor, GpuFft::new / fft / ifft / is_gpu_available, Default).
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gbfft.h")
CRATE = os.path.join(ROOT, "wgls-rs-fft_gb300", "rust")

# C parameter / return types of the header -> the Rust FFI type that binds them
C_TO_RUST = {
    "int": "c_int",
    "void": None,
    "uint64_t": "u64",
    "uint32_t": "u32",
    "float": "f32",
    "void *": "*mut c_void",
    "const void *": "*const c_void",
    "float *": "*mut f32",
    "const float *": "*const f32",
    "const float *const *": "*const *const f32",
    "float *const *": "*const *mut f32",
    "const uint64_t *": "*const u64",
    "double *": "*mut f64",
    "const char *": "*const c_char",
    "gbfft_ctx *": "*mut GbfftCtx",
    "const gbfft_ctx *": "*const GbfftCtx",
    "gbfft_ctx **": "*mut *mut GbfftCtx",
    "gbfft_ragged_plan *": "*mut GbfftRaggedPlan",
    "const gbfft_ragged_plan *": "*const GbfftRaggedPlan",
    "gbfft_ragged_plan **": "*mut *mut GbfftRaggedPlan",
    "const gbfft_ragged_desc *": "*const GbfftRaggedDesc",
}


def _strip_c_comments(s):
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return re.sub(r"//[^\n]*", " ", s)


def _norm_ctype(t):
    t = re.sub(r"\s+", " ", t.strip())
    t = re.sub(r"\s*\*\s*", " *", t)          # "float*" / "float *" -> "float *"
    t = re.sub(r"\*\s+\*", "**", t)
    t = t.replace("* const", "*const")
    return t.strip()


def header_functions():
    src = _strip_c_comments(open(HEADER).read())
    src = "\n".join(line for line in src.splitlines() if not line.lstrip().startswith("#"))
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(gbfft_\w+)\s*\(([^;{}]*?)\)\s*;", src, flags=re.S):
        ret, name, params = m.group(1), m.group(2), m.group(3).strip()
        ret = _norm_ctype(ret.replace("typedef", ""))
        args = []
        if params and params != "void":
            for p in params.split(","):
                p = re.sub(r"\s+", " ", p.strip())
                pm = re.match(r"(.*?)(\w+)$", p)
                args.append(_norm_ctype(pm.group(1)))
        out[name] = (ret, args)
    return out


def header_constants():
    src = open(HEADER).read()
    consts = {}
    for m in re.finditer(r"#define\s+(GBFFT_\w+)\s+\(?([+-]?\d+)\)?", src):
        consts[m.group(1)] = int(m.group(2))
    for m in re.finditer(r"\b(GBFFT_(?:OK|ERR_\w+|PREC_\w+))\s*=\s*(-?\d+)", src):
        consts[m.group(1)] = int(m.group(2))
    return consts


def rust_functions():
    src = open(os.path.join(CRATE, "src", "gbfft_sys.rs")).read()
    block = src[src.index('extern "C" {'):]
    block = block[:block.index("\n}")]
    out = {}
    for m in re.finditer(r"pub fn (gbfft_\w+)\s*\((.*?)\)\s*(->\s*([^;]+))?;", block, flags=re.S):
        name, params, ret = m.group(1), m.group(2), m.group(4)
        args = []
        for p in [q for q in params.split(",") if q.strip()]:
            args.append(re.sub(r"\s+", " ", p.split(":", 1)[1].strip()))
        out[name] = ((ret or "").strip() or None, args)
    return out


def rust_constants():
    src = open(os.path.join(CRATE, "src", "gbfft_sys.rs")).read()
    return {m.group(1): int(m.group(2))
            for m in re.finditer(r"pub const (GBFFT_\w+): c_int = (-?\d+);", src)}


def test_every_header_function_is_bound_with_matching_types():
    h = header_functions()
    r = rust_functions()
    assert len(h) >= 20, sorted(h)
    assert set(h) == set(r), (set(h) ^ set(r))
    for name, (ret, args) in h.items():
        rret, rargs = r[name]
        assert C_TO_RUST[ret] == rret, (name, ret, rret)
        assert len(args) == len(rargs), (name, args, rargs)
        for ca, ra in zip(args, rargs):
            assert C_TO_RUST[ca] == ra, (name, ca, ra)


def test_constants_match_header():
    h = header_constants()
    r = rust_constants()
    for name in ("GBFFT_FORWARD", "GBFFT_INVERSE", "GBFFT_OK", "GBFFT_ERR_UNSUPPORTED", "GBFFT_PREC_TC_TF32",
                 "GBFFT_RAGGED_OPT_LAG", "GBFFT_WINDOW_HANN"):
        assert name in h and name in r, name
    for name, v in r.items():
        assert h.get(name) == v, (name, h.get(name), v)
    assert set(k for k in h if not k.startswith("GBFFT_H")) <= set(r), set(h) - set(r)


def test_ragged_desc_layout_matches_header():
    src = _strip_c_comments(open(HEADER).read())
    m = re.search(r"typedef struct gbfft_ragged_desc\s*\{(.*?)\}", src, flags=re.S)
    fields = [re.sub(r"\s+", " ", f.strip()) for f in m.group(1).split(";") if f.strip()]
    assert fields == ["uint64_t offset", "uint32_t log2n", "int32_t direction"]
    rs = open(os.path.join(CRATE, "src", "gbfft_sys.rs")).read()
    m = re.search(r"pub struct GbfftRaggedDesc \{(.*?)\}", rs, flags=re.S)
    rfields = [re.sub(r"\s+", " ", f.strip()) for f in m.group(1).split(",") if f.strip()]
    assert rfields == ["pub offset: u64", "pub log2n: u32", "pub direction: i32"]


def test_crate_keeps_the_reference_surface_and_builds_for_sm_103a():
    lib = open(os.path.join(CRATE, "src", "lib.rs")).read()
    for needle in ("pub trait FftExecutor", "fn name(&self) -> &str", "fn as_any(&self) -> &dyn Any",
                   "pub fn new() -> Result<Self, Box<dyn Error>>", "pub fn is_gpu_available() -> bool",
                   "pub fn fft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>>",
                   "pub fn ifft(&self, inputs: &[Vec<Complex<f32>>]) -> Result<Vec<Vec<Complex<f32>>>, Box<dyn Error>>",
                   "impl Default for GpuFft", "impl FftExecutor for GpuFft",
                   "Transform length must be a non-zero power of two",
                   "All input vectors in a batch must have the same length"):
        assert needle in lib, needle
    build = open(os.path.join(CRATE, "build.rs")).read()
    assert "arch=compute_103a,code=sm_103a" in build and "csrc" in build
    toml = open(os.path.join(CRATE, "Cargo.toml")).read()
    assert 'name = "wgls_rs_fft"' in toml and "wgpu" not in toml.split("[dependencies]")[1]
