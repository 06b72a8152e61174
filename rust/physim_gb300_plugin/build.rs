//! Build script: the plugin ABI string physim checks, and the link to
//! libphysim_gb300.so.
//!
//! physim compares a Rust plugin's `get_plugin_abi_info()` with its own
//! `rustc:<version>|target:<triple>` string (physim-core/src/plugin/
//! discover.rs:327-351); the string is made here exactly as physim's own
//! plugins make it (astro/build.rs:3-9).  The CUDA library is found in
//! $PHYSIM_GB300_LIB_DIR, else in the repository's build output next to this
//! crate (physim_gb300/_lib, made by `python -c "import __graft_entry__ as g;
//! g.build()"`); its directory is also written into the plugin's run path, so
//! copying both .so files into one plugin directory is enough.

use std::env;
use std::path::PathBuf;

fn main() {
    let rustc = rustc_version::version().expect("Failed to get rustc version");
    let target = env::var("TARGET").expect("Cargo did not set TARGET");
    println!("cargo:rustc-env=ABI_INFO=rustc:{}|target:{}", rustc, target);

    let lib_dir = match env::var("PHYSIM_GB300_LIB_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap())
            .join("../../physim_gb300/_lib"),
    };
    println!("cargo:rerun-if-env-changed=PHYSIM_GB300_LIB_DIR");
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=physim_gb300");
    println!("cargo:rustc-link-arg=-Wl,-rpath,$ORIGIN");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
}
