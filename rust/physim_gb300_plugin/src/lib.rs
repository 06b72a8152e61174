//! physim plugin: the `verlet`, `euler` and `rk4` integrators and the
//! `energysink` render element, computed on a GB300 GPU by libphysim_gb300.
//!
//! Element names are physim's own (integrators/src/lib.rs:3,
//! debug/src/lib.rs), so pipeline TOML files and CLI strings run unchanged.
//! physim keys elements by name, the last library scanned winning
//! (physim-core/src/plugin/discover.rs:256-259): install this plugin's
//! directory after (or instead of) the stock integrators library.  The
//! gravity transforms (astro, astro2, simple_astro) are exported by
//! libphysim_gb300.so itself through physim's C plugin ABI.
//!
//! Not built here: this crate needs physim's nightly toolchain and crates.

use physim_core::register_plugin;

register_plugin!("verlet", "euler", "rk4", "energysink");

mod energysink;
mod ffi;
mod integrators;
