// Links librtcore.so, built by `python -c "import __graft_entry__ as g; g.build()"` into
// ray-tracing-gallery_gb300/_build/ (or the folder named by RTCORE_LIB_DIR).
fn main() {
    let dir = std::env::var("RTCORE_LIB_DIR").unwrap_or_else(|_| {
        let manifest = std::env::var("CARGO_MANIFEST_DIR").expect("CARGO_MANIFEST_DIR");
        format!("{}/../_build", manifest)
    });
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=rtcore");
    println!("cargo:rerun-if-env-changed=RTCORE_LIB_DIR");
}
