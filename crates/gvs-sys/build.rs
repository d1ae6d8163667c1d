//! Builds libgvs from its CUDA C++ sources with nvcc for sm_103a and links it
//! statically (with the static CUDA runtime), so a binary that depends on this
//! crate needs only the NVIDIA driver at run time.
//!
//! The flags are the ones gravis_gb300/build.py uses for the in-tree Python
//! build: one `-gencode arch=compute_103a,code=sm_103a`, `-O3 -lineinfo`,
//! `-ffp-contract=off` for host code (the initial conditions follow the
//! reference's unfused f64 arithmetic), and `--fmad=false` for sph.cu (its f64
//! kernels restate sim-core's SPH arithmetic statement by statement).
//!
//! Environment: GVS_CSRC (the csrc folder; default: this repository's
//! gravis_gb300/csrc), NVCC (default: nvcc on PATH, then $CUDA_HOME/bin/nvcc),
//! CUDA_HOME (default /usr/local/cuda).
use std::env;
use std::path::{Path, PathBuf};
use std::process::Command;

const ARCH: &[&str] = &["-gencode", "arch=compute_103a,code=sm_103a"];
const NVCC_FLAGS: &[&str] = &[
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills", "-diag-suppress", "1444,177",
];
/// Per-file flags, as in gravis_gb300/build.py's FILE_FLAGS.
const FILE_FLAGS: &[(&str, &[&str])] = &[("sph.cu", &["--fmad=false"]), ("ics_dev.cu", &["--fmad=false"])];

fn nvcc(cuda_home: &Path) -> PathBuf {
    if let Ok(p) = env::var("NVCC") {
        return PathBuf::from(p);
    }
    let on_path = Command::new("nvcc").arg("--version").output().map(|o| o.status.success()).unwrap_or(false);
    if on_path { PathBuf::from("nvcc") } else { cuda_home.join("bin").join("nvcc") }
}

fn main() {
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("CARGO_MANIFEST_DIR"));
    let csrc = env::var("GVS_CSRC")
        .map(PathBuf::from)
        .unwrap_or_else(|_| manifest.join("..").join("..").join("gravis_gb300").join("csrc"));
    let cuda_home = PathBuf::from(env::var("CUDA_HOME").unwrap_or_else(|_| "/usr/local/cuda".into()));
    let out = PathBuf::from(env::var("OUT_DIR").expect("OUT_DIR"));
    let nvcc = nvcc(&cuda_home);

    let mut srcs: Vec<PathBuf> = std::fs::read_dir(&csrc)
        .unwrap_or_else(|e| panic!("cannot read {} (set GVS_CSRC): {e}", csrc.display()))
        .filter_map(|e| e.ok().map(|e| e.path()))
        .filter(|p| matches!(p.extension().and_then(|x| x.to_str()), Some("cu") | Some("cpp")))
        .collect();
    srcs.sort();
    assert!(!srcs.is_empty(), "no .cu/.cpp sources in {}", csrc.display());

    let mut objs = Vec::new();
    for src in &srcs {
        let name = src.file_name().unwrap().to_string_lossy().into_owned();
        let obj = out.join(format!("{name}.o"));
        let mut cmd = Command::new(&nvcc);
        cmd.args(ARCH).args(NVCC_FLAGS);
        for (file, flags) in FILE_FLAGS {
            if *file == name {
                cmd.args(*flags);
            }
        }
        cmd.arg("-c").arg(src).arg("-o").arg(&obj);
        let st = cmd.status().unwrap_or_else(|e| panic!("cannot run {}: {e}", nvcc.display()));
        assert!(st.success(), "nvcc failed on {name}");
        println!("cargo:rerun-if-changed={}", src.display());
        objs.push(obj);
    }
    for entry in std::fs::read_dir(&csrc).unwrap().filter_map(|e| e.ok()) {
        let p = entry.path();
        if p.extension().and_then(|x| x.to_str()) == Some("cuh") {
            println!("cargo:rerun-if-changed={}", p.display());
        }
    }
    let lib = out.join("libgvs.a");
    let _ = std::fs::remove_file(&lib);
    let st = Command::new("ar").arg("crs").arg(&lib).args(&objs).status().expect("cannot run ar");
    assert!(st.success(), "ar failed");

    println!("cargo:rustc-link-search=native={}", out.display());
    println!("cargo:rustc-link-lib=static=gvs");
    for sub in ["lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"] {
        let d = cuda_home.join(sub);
        if d.is_dir() {
            println!("cargo:rustc-link-search=native={}", d.display());
        }
    }
    println!("cargo:rustc-link-lib=static=cudart_static");
    for l in ["stdc++", "dl", "rt", "pthread"] {
        println!("cargo:rustc-link-lib=dylib={l}");
    }
    println!("cargo:rerun-if-env-changed=GVS_CSRC");
    println!("cargo:rerun-if-env-changed=NVCC");
    println!("cargo:rerun-if-env-changed=CUDA_HOME");
}
