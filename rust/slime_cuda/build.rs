//! Links libslime_gb300.so, the CUDA library built from this repository's
//! `slime-mold_gb300/csrc` for sm_103a.
//!
//! The library is looked up in `$SLIME_GB300_LIB_DIR`, else in
//! `slime-mold_gb300/lib` of the repository this crate sits in.  With
//! `SLIME_GB300_BUILD=1` a missing library is built first by
//! `python3 slime-mold_gb300/build.py` (nvcc for sm_103a).  The run-time
//! search path of the final binary gets the same directory.
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR"));
    let repo = manifest.join("..").join("..");
    let lib_dir = match env::var("SLIME_GB300_LIB_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => repo.join("slime-mold_gb300").join("lib"),
    };
    let lib = lib_dir.join("libslime_gb300.so");
    if !lib.exists() && env::var("SLIME_GB300_BUILD").map(|v| v == "1").unwrap_or(false) {
        let status = Command::new("python3")
            .arg(repo.join("slime-mold_gb300").join("build.py"))
            .status()
            .expect("running slime-mold_gb300/build.py");
        assert!(status.success(), "slime-mold_gb300/build.py failed");
    }
    if !lib.exists() {
        panic!(
            "{} not found: build it with `python3 slime-mold_gb300/build.py` or point SLIME_GB300_LIB_DIR at it",
            lib.display()
        );
    }
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=slime_gb300");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
    println!("cargo:rerun-if-env-changed=SLIME_GB300_LIB_DIR");
    println!("cargo:rerun-if-env-changed=SLIME_GB300_BUILD");
    println!("cargo:rerun-if-changed={}", repo.join("include").join("slime.h").display());
    println!("cargo:rerun-if-changed={}", lib.display());
}
