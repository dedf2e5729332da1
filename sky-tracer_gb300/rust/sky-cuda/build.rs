//! Links libsky_cuda.so (built by `python sky-tracer_gb300/build.py`).

fn main() {
    let dir = std::env::var("SKY_CUDA_LIB_DIR")
        .expect("set SKY_CUDA_LIB_DIR to the directory holding libsky_cuda.so");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=sky_cuda");
    // the loader finds the library next to the binaries without LD_LIBRARY_PATH
    println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    println!("cargo:rerun-if-env-changed=SKY_CUDA_LIB_DIR");
}
