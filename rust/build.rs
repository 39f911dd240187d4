// Links libaqua.so. AQUA_LIB_DIR names the folder that holds it (built by
// `python aqua-engine_gb300/build.py`); the default is that build's output
// folder next to this crate.
fn main() {
    let dir = std::env::var("AQUA_LIB_DIR").unwrap_or_else(|_| {
        let here = std::env::var("CARGO_MANIFEST_DIR").unwrap();
        format!("{}/../aqua-engine_gb300", here)
    });
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=aqua");
    println!("cargo:rerun-if-env-changed=AQUA_LIB_DIR");
}
