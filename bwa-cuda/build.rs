//! Links libbwacuda.so.  The library is built outside cargo (nvcc, sm_103a):
//! `python bwa-mem4_gb300/build.py` in the bwa-cuda source tree writes
//! `bwa-mem4_gb300/libbwacuda.so`; point BWACUDA_LIB_DIR at that directory.

fn main() {
    let dir = match std::env::var("BWACUDA_LIB_DIR") {
        Ok(d) => d,
        Err(_) => panic!("set BWACUDA_LIB_DIR to the directory holding libbwacuda.so"),
    };
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=bwacuda");
    // the loader finds the library at run time without LD_LIBRARY_PATH
    println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    println!("cargo:rerun-if-env-changed=BWACUDA_LIB_DIR");
}
