//! The reference crate's public API (`src/interface.rs`: `Diagram`, `Cell`,
//! `VoronoiFace`, plus `Polyhedron::new` for the container) over the GB300
//! library's C ABI (`include/tessellator.h`).  `gpu_ffi` is the raw binding,
//! one `extern "C"` item per function of the header; `interface` is the safe
//! wrapper with the reference's method names.
pub mod gpu_ffi;
pub mod interface;

pub use interface::{Batch, Cell, Diagram, Error, Polyhedron, Precision, VoronoiFace};
