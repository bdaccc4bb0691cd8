// Links libfuelg.so.  FUELG_LIB_DIR names the folder that holds it (the
// engine's own build puts it next to fuel_gb300/__init__.py); the library
// loads the CUDA runtime itself, so nothing else is linked here.
fn main() {
    println!("cargo:rerun-if-env-changed=FUELG_LIB_DIR");
    if let Ok(dir) = std::env::var("FUELG_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
    }
    println!("cargo:rustc-link-lib=dylib=fuelg");
}
