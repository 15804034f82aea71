//! Builds libtessgpu.so (nvcc, sm_103a) from this repository and links it.
//! TESS_GB300_DIR may point at the repository root; by default it is the
//! parent of this crate.
use std::{env, path::PathBuf, process::Command};

fn main() {
    let dir = match env::var("TESS_GB300_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join(".."),
    };
    let status = Command::new("python3")
        .arg(dir.join("the-tessellator_gb300/build_lib.py"))
        .status()
        .expect("python3 and nvcc are needed to build libtessgpu.so");
    assert!(status.success(), "building libtessgpu.so failed");
    let lib = dir.join("the-tessellator_gb300/tessellator");
    println!("cargo:rustc-link-search=native={}", lib.display());
    println!("cargo:rustc-link-lib=dylib=tessgpu");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib.display());
    println!("cargo:rerun-if-env-changed=TESS_GB300_DIR");
    println!("cargo:rerun-if-changed={}", dir.join("include/tessellator.h").display());
}
