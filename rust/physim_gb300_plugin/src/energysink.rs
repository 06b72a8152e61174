//! `energysink`: physim's energy-printing render element (debug/src/
//! energysink.rs) with its sums on the GPU in f64.
//!
//! It receives the initial state and every new state (pipeline.rs:128-181)
//! and prints `{i:>5} :: K = .. :: V = .. :: E = .. :: Delta E ..` for every
//! `print_n`-th state (energysink.rs:38-58).  The potential is off until a
//! gravity element posts ("energysink", "gravity") (energysink.rs:112-117,
//! astro/src/transformers.rs:107-111,198-203,266-270).  Two differences from
//! the reference sink, both its bugs: V sums every pair (energysink.rs:86
//! assigns `=` where it means `+=`, keeping the last pair only) and the first
//! line's E is K + V (the reference prints V there).  With `e` = 0 (the
//! default) the pair potential is the reference sink's -m_a m_b / r; with
//! `e` > 0 it is the potential whose gradient is the gravity elements'
//! softened force.

use std::collections::HashMap;
use std::ffi::c_void;
use std::sync::Mutex;
use std::sync::atomic::{AtomicBool, AtomicUsize, Ordering};

use physim_attribute::render_element;
use physim_core::Entity;
use physim_core::messages::MessageClient;
use physim_core::plugin::render::RenderElement;
use physim_core::plugin::{Element, ElementCreator};
use serde_json::Value;

use crate::ffi;

#[render_element(name = "energysink", blurb = "Kinetic and potential energy of every state, on the GPU")]
pub struct GpuEnergySink {
    iteration: AtomicUsize,
    print_n: usize,
    e: f64,
    calc_gpe: AtomicBool,
    handle: Mutex<usize>,
}

impl ElementCreator for GpuEnergySink {
    fn create_element(properties: HashMap<String, Value>) -> Box<Self> {
        let print_n = properties.get("print_n").and_then(|v| v.as_u64()).unwrap_or(1).max(1) as usize;
        let e = properties.get("e").and_then(|v| v.as_f64()).unwrap_or(0.0).abs();
        let device = properties.get("device").and_then(|v| v.as_i64()).unwrap_or(0) as i32;
        let mut h: *mut c_void = std::ptr::null_mut();
        ffi::check(unsafe { ffi::physim_gpu_energy_create(device, &mut h) }, "physim_gpu_energy_create");
        Box::new(GpuEnergySink {
            iteration: AtomicUsize::new(0),
            print_n,
            e,
            calc_gpe: AtomicBool::new(false),
            handle: Mutex::new(h as usize),
        })
    }
}

impl GpuEnergySink {
    /// (potential, kinetic) of one state.
    fn energy(&self, state: &[Entity]) -> (f64, f64) {
        let gpe = self.calc_gpe.load(Ordering::Relaxed);
        let mut d = ffi::Diagnostics::default();
        let h = self.handle.lock().unwrap_or_else(|_| std::process::abort());
        let rc = unsafe {
            ffi::physim_gpu_energy_compute(
                *h as *mut c_void,
                state.as_ptr(),
                state.len(),
                self.e,
                gpe as i32,
                &mut d,
            )
        };
        ffi::check(rc, "physim_gpu_energy_compute");
        (if gpe { d.potential } else { 0.0 }, d.kinetic)
    }
}

impl RenderElement for GpuEnergySink {
    fn render(&self, state_recv: std::sync::mpsc::Receiver<Vec<Entity>>) {
        let mut initial_energy = None;
        while let Ok(state) = state_recv.recv() {
            let (potential, kinetic) = self.energy(&state);
            let energy = kinetic + potential;
            let initial = *initial_energy.get_or_insert(energy);
            let delta = initial - energy;
            let iteration = self.iteration.fetch_add(1, Ordering::Relaxed);
            if iteration.rem_euclid(self.print_n) == 0 {
                println!(
                    "{iteration:>5} :: K = {kinetic:1.6} :: V = {potential:1.6} :: E = {energy:1.6} :: Delta E {delta:1.6}"
                );
            }
        }
    }
}

impl Element for GpuEnergySink {
    fn get_property_descriptions(&self) -> Result<HashMap<String, String>, Box<dyn std::error::Error>> {
        Ok(HashMap::from([
            (String::from("print_n"), String::from("print every n iterations")),
            (String::from("e"), String::from("easing of the potential (0: -m_a m_b / r)")),
            (String::from("device"), String::from("CUDA device (default 0)")),
        ]))
    }
}

impl MessageClient for GpuEnergySink {
    fn recv_message(&self, message: &physim_core::messages::Message) {
        if message.topic == "energysink" && message.message == "gravity" {
            self.calc_gpe.store(true, Ordering::Relaxed);
        }
    }
}

impl Drop for GpuEnergySink {
    fn drop(&mut self) {
        if let Ok(h) = self.handle.lock() {
            unsafe { ffi::physim_gpu_energy_destroy(*h as *mut c_void) };
        }
    }
}
