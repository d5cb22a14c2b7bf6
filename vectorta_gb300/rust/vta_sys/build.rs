// Links libvta_gb300.so from the repository's build folder, or from
// VTA_GB300_LIB_DIR when set.  Generated by gen_abi.py.
fn main() {
    let dir = std::env::var("VTA_GB300_LIB_DIR").unwrap_or_else(|_| {
        let here = std::env::var("CARGO_MANIFEST_DIR").unwrap();
        format!("{}/../../_lib", here)
    });
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=vta_gb300");
    println!("cargo:rerun-if-env-changed=VTA_GB300_LIB_DIR");
}
