//! `verlet`, `euler` and `rk4` integrator elements over the GPU steppers.
//!
//! Each element has physim's integrator contract (physim-core/src/plugin/
//! integrator.rs:5-13): given the state, the new state's buffer, `acc_fn`
//! (every transform adding into zeroed accelerations, pipeline.rs:137-141)
//! and dt, it fills the new state.  physim_gpu_integrator_integrate calls
//! back into `acc_fn` once (verlet, euler) or four times at the stage states
//! (rk4), and does the update on the GPU in f64 with the reference's
//! operation order (integrators/src/verlet.rs:24-107, euler.rs:17-49,
//! rk4.rs:24-178): given the same accelerations, the new state is
//! bit-identical to the CPU integrators'.  verlet keeps its previous state on
//! the device and takes the Taylor first step whenever the body count
//! changes, as verlet.rs:102-106 does.

use std::collections::HashMap;
use std::ffi::c_void;
use std::sync::Mutex;

use physim_attribute::integrator_element;
use physim_core::messages::MessageClient;
use physim_core::plugin::integrator::IntegratorElement;
use physim_core::plugin::{Element, ElementCreator};
use physim_core::{Acceleration, Entity};
use serde_json::Value;

use crate::ffi;

type AccClosure<'a> = &'a dyn Fn(&[Entity], &mut [Acceleration]);

/// Calls physim's `acc_fn` for the library (`user` points at the closure).
unsafe extern "C" fn call_acc_fn(
    user: *mut c_void,
    state: *const Entity,
    n: usize,
    acc: *mut Acceleration,
) {
    let f = unsafe { &*(user as *const AccClosure) };
    let (state, acc) = if n == 0 {
        (&[][..], &mut [][..])
    } else {
        unsafe { (std::slice::from_raw_parts(state, n), std::slice::from_raw_parts_mut(acc, n)) }
    };
    f(state, acc);
}

/// One GPU stepper of the library (a `PhysimIntegrator*`), used by one
/// pipeline thread at a time.
struct Stepper {
    handle: Mutex<usize>,
}

impl Stepper {
    fn new(kind: u32, properties: &HashMap<String, Value>) -> Self {
        // optional: the CUDA device (physim's own integrators have no properties)
        let device = properties.get("device").and_then(|v| v.as_i64()).unwrap_or(0) as i32;
        let mut h: *mut c_void = std::ptr::null_mut();
        ffi::check(
            unsafe { ffi::physim_gpu_integrator_create(kind, device, &mut h) },
            "physim_gpu_integrator_create",
        );
        Stepper { handle: Mutex::new(h as usize) }
    }

    fn integrate(&self, entities: &[Entity], new_state: &mut [Entity], acc_fn: AccClosure, dt: f64) {
        let h = match self.handle.lock() {
            Ok(h) => h,
            Err(_) => {
                eprintln!("physim_gb300: integrator mutex poisoned");
                std::process::exit(1)
            }
        };
        assert_eq!(entities.len(), new_state.len(), "state and new state differ in length");
        let user = &acc_fn as *const AccClosure as *mut c_void;
        let rc = unsafe {
            ffi::physim_gpu_integrator_integrate(
                *h as *mut c_void,
                entities.as_ptr(),
                new_state.as_mut_ptr(),
                entities.len(),
                call_acc_fn,
                user,
                dt,
            )
        };
        ffi::check(rc, "physim_gpu_integrator_integrate");
    }
}

impl Drop for Stepper {
    fn drop(&mut self) {
        if let Ok(h) = self.handle.lock() {
            unsafe { ffi::physim_gpu_integrator_destroy(*h as *mut c_void) };
        }
    }
}

fn descriptions() -> Result<HashMap<String, String>, Box<dyn std::error::Error>> {
    Ok(HashMap::from([(
        String::from("device"),
        String::from("CUDA device of the GPU stepper (default 0)"),
    )]))
}

#[integrator_element(name = "verlet", blurb = "Verlet integration on the GPU")]
pub struct GpuVerlet {
    stepper: Stepper,
}

impl IntegratorElement for GpuVerlet {
    fn integrate(
        &self,
        entities: &[Entity],
        new_state: &mut [Entity],
        acc_fn: &dyn Fn(&[Entity], &mut [Acceleration]),
        dt: f64,
    ) {
        self.stepper.integrate(entities, new_state, acc_fn, dt);
    }
}

impl ElementCreator for GpuVerlet {
    fn create_element(properties: HashMap<String, Value>) -> Box<Self> {
        Box::new(GpuVerlet { stepper: Stepper::new(ffi::INTEGRATOR_VERLET, &properties) })
    }
}

impl Element for GpuVerlet {
    fn get_property_descriptions(
        &self,
    ) -> Result<HashMap<String, String>, Box<dyn std::error::Error>> {
        descriptions()
    }
}

impl MessageClient for GpuVerlet {}

#[integrator_element(name = "euler", blurb = "Euler integration on the GPU")]
pub struct GpuEuler {
    stepper: Stepper,
}

impl IntegratorElement for GpuEuler {
    fn integrate(
        &self,
        entities: &[Entity],
        new_state: &mut [Entity],
        acc_fn: &dyn Fn(&[Entity], &mut [Acceleration]),
        dt: f64,
    ) {
        self.stepper.integrate(entities, new_state, acc_fn, dt);
    }
}

impl ElementCreator for GpuEuler {
    fn create_element(properties: HashMap<String, Value>) -> Box<Self> {
        Box::new(GpuEuler { stepper: Stepper::new(ffi::INTEGRATOR_EULER, &properties) })
    }
}

impl Element for GpuEuler {
    fn get_property_descriptions(
        &self,
    ) -> Result<HashMap<String, String>, Box<dyn std::error::Error>> {
        descriptions()
    }
}

impl MessageClient for GpuEuler {}

#[integrator_element(name = "rk4", blurb = "RK4 integration on the GPU")]
pub struct GpuRk4 {
    stepper: Stepper,
}

impl IntegratorElement for GpuRk4 {
    fn integrate(
        &self,
        entities: &[Entity],
        new_state: &mut [Entity],
        acc_fn: &dyn Fn(&[Entity], &mut [Acceleration]),
        dt: f64,
    ) {
        self.stepper.integrate(entities, new_state, acc_fn, dt);
    }
}

impl ElementCreator for GpuRk4 {
    fn create_element(properties: HashMap<String, Value>) -> Box<Self> {
        Box::new(GpuRk4 { stepper: Stepper::new(ffi::INTEGRATOR_RK4, &properties) })
    }
}

impl Element for GpuRk4 {
    fn get_property_descriptions(
        &self,
    ) -> Result<HashMap<String, String>, Box<dyn std::error::Error>> {
        descriptions()
    }
}

impl MessageClient for GpuRk4 {}
