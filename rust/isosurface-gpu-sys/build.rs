//! Links libisosurface_gpu.so.  The library is built by
//! `python -m isosurface_gb300.build` into isosurface_gb300/_build/;
//! ISOSURFACE_GPU_LIB_DIR overrides where it is looked for.

use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("ISOSURFACE_GPU_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap())
            .join("../../isosurface_gb300/_build"),
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=isosurface_gpu");
    println!("cargo:rerun-if-env-changed=ISOSURFACE_GPU_LIB_DIR");
}
