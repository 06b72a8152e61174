//! The part of libphysim_gb300's C ABI this crate calls.  Each declaration
//! mirrors one in include/physim_gb300.h (same name, argument order and
//! types); a test of the repository checks the two against each other.

use std::ffi::{c_char, c_int, c_void};

use physim_core::{Acceleration, Entity};

/// `PhysimAccFn`: the library calls back into physim's `acc_fn` through it.
pub type AccFn =
    unsafe extern "C" fn(user: *mut c_void, state: *const Entity, n: usize, acc: *mut Acceleration);

/// `PhysimDiagnostics` (f64 whole-system sums).
#[repr(C)]
#[derive(Default, Clone, Copy, Debug)]
pub struct Diagnostics {
    pub mass: f64,
    pub centre_of_mass: [f64; 3],
    pub momentum: [f64; 3],
    pub kinetic: f64,
    pub potential: f64,
    pub energy: f64,
}

/// `PhysimIntegratorKind`.
pub const INTEGRATOR_VERLET: u32 = 0;
pub const INTEGRATOR_EULER: u32 = 1;
pub const INTEGRATOR_RK4: u32 = 2;

unsafe extern "C" {
    pub fn physim_gpu_last_error() -> *const c_char;

    pub fn physim_gpu_integrator_create(kind: u32, device: i32, out: *mut *mut c_void) -> c_int;
    pub fn physim_gpu_integrator_integrate(
        it: *mut c_void,
        entities: *const Entity,
        new_state: *mut Entity,
        n: usize,
        acc_fn: AccFn,
        user: *mut c_void,
        dt: f64,
    ) -> c_int;
    pub fn physim_gpu_integrator_destroy(it: *mut c_void);

    pub fn physim_gpu_energy_create(device: i32, out: *mut *mut c_void) -> c_int;
    pub fn physim_gpu_energy_compute(
        energy: *mut c_void,
        state: *const Entity,
        n: usize,
        e: f64,
        with_potential: c_int,
        out: *mut Diagnostics,
    ) -> c_int;
    pub fn physim_gpu_energy_destroy(energy: *mut c_void);
}

/// The library's message for the last failed call on this thread.
pub fn last_error() -> String {
    let p = unsafe { physim_gpu_last_error() };
    if p.is_null() {
        return String::new();
    }
    unsafe { std::ffi::CStr::from_ptr(p) }.to_string_lossy().into_owned()
}

/// physim's plugins have one error channel across the FFI boundary: a panic
/// caught by the element macro aborts the process (physim-attribute/src/
/// lib.rs:94-97).  A failed GPU call does the same after saying why.
pub fn check(rc: c_int, what: &str) {
    if rc != 0 {
        eprintln!("physim_gb300: {what} failed with status {rc}: {}", last_error());
        std::process::abort();
    }
}
