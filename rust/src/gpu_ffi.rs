//! Raw binding of include/tessellator.h: one `extern "C"` item per function,
//! and the `#[repr(C)]` structs with the header's field order.  Every call
//! returns a `tess_status` (0 = TESS_OK); `tess_last_error` gives the message.
#![allow(non_camel_case_types)]
#![allow(dead_code)]
use std::os::raw::{c_char, c_int, c_void};

#[repr(C)] pub struct tess_diagram { _p: [u8; 0] }
#[repr(C)] pub struct tess_batch { _p: [u8; 0] }
pub type tess_status = c_int;
pub const TESS_OK: tess_status = 0;
pub const TESS_E_INVALID: tess_status = 1;
pub const TESS_E_CUDA: tess_status = 2;
pub const TESS_E_CAPACITY: tess_status = 3;   // buffer too small: the size needed is reported
pub const TESS_E_OVERFLOW: tess_status = 4;  // a cell exceeded the largest capacity
pub const TESS_E_STATE: tess_status = 5;     // results asked for before compute
pub const TESS_E_NOMEM: tess_status = 6;
pub const TESS_E_LIMIT: tess_status = 7;
pub const TESS_E_CHECK: tess_status = 8;
pub const TESS_PRECISION_FP64: c_int = 0;
pub const TESS_PRECISION_FP32_GUARD: c_int = 1;
pub const TESS_PRECISION_MIXED: c_int = 2;   // FP32 clipping, FP64-accurate results
pub const TESS_FLAG_TIMING: u32 = 1;
pub const TESS_FLAG_COUNTERS: u32 = 2;
pub const TESS_FLAG_SMALL_FACE_POOL: u32 = 4;
pub const TESS_FLAG_NO_CAPACITY_RERUN: u32 = 8;
pub const TESS_FLAG_AUTOTUNE: u32 = 16;

#[repr(C)] #[derive(Clone, Copy)]
pub struct tess_config {
    pub guard_rel: f64, pub verify_rel: f64, pub bin_density: f64,
    pub table_gaps: i32, pub warps_per_block: i32, pub slots_per_lane: i32, pub device: i32,
    pub stream: *mut c_void, pub flags: u32, pub crowded_bin: i32,
}

#[repr(C)] #[derive(Clone, Copy, Default)]
pub struct tess_stats {
    pub cells: u64, pub faces: u64, pub rerun_fp64: u64, pub rerun_capacity: u64, pub failed: u64,
    pub table_entries: u64, pub ms_grid: f64, pub ms_clip: f64, pub ms_rerun: f64, pub ms_csr: f64,
    pub launches: u64, pub rerun_guard: u64, pub rerun_verify: u64, pub rerun_degenerate: u64,
    pub candidates_tested: u64, pub cuts: u64, pub new_vertices: u64, pub windows: u64, pub batches: u64,
    pub ms_query_count: f64, pub ms_query_fill: f64, pub rerun_fp64_full: u64, pub dense_cells: u64, pub face_pool_regrows: u64,
}

#[repr(C)] #[derive(Clone, Copy, Default, Debug)]
pub struct tess_tuning {
    pub warps_per_block: i32, pub crowded_bin: i32, pub bin_density: f64, pub ms_chosen: f64,
    pub ms_default: f64, pub sample_cells: u64, pub trials: i32, pub from_cache: i32,
    pub max_bin_points: u32, pub crowded_fraction: f64,
}

#[repr(C)]
pub struct tess_cell_geometry {
    pub volume: f64, pub nvertices: i32, pub nfaces: i32,
    pub vertices: [f64; 768], pub face_neighbor: [i32; 256], pub face_area: [f64; 256],
    pub face_offset: [i32; 257], pub face_vertex: [i32; 768],
}

extern "C" {
    pub fn tess_config_default(cfg: *mut tess_config);
    pub fn tess_last_error(buf: *mut c_char, cap: usize) -> usize;
    pub fn tess_version() -> *const c_char;
    // Diagram (interface.rs:25-84; the reference has no public constructor)
    pub fn tess_diagram_create(xyz: *const f64, n: usize, groups: *const u32, lo: *const f64,
                               hi: *const f64, cfg: *const tess_config,
                               out: *mut *mut tess_diagram) -> tess_status;
    pub fn tess_diagram_create_device(d_xyz: *const f64, n: usize, groups: *const u32, lo: *const f64,
                                      hi: *const f64, cfg: *const tess_config,
                                      out: *mut *mut tess_diagram) -> tess_status;
    pub fn tess_diagram_rebuild(d: *mut tess_diagram) -> tess_status;
    pub fn tess_diagram_update_points(d: *mut tess_diagram, xyz: *const f64, on_device: c_int) -> tess_status;
    pub fn tess_diagram_celery(d: *const tess_diagram, cells: *mut u32, sorted_indices: *mut u32,
                               delimiters: *mut u32) -> tess_status;
    pub fn tess_diagram_destroy(d: *mut tess_diagram) -> tess_status;
    pub fn tess_diagram_compute_all(d: *mut tess_diagram, precision: c_int, search_radius: f64,
                                    target_group: i64) -> tess_status;
    pub fn tess_diagram_stats(d: *const tess_diagram, out: *mut tess_stats) -> tess_status;
    pub fn tess_diagram_grid(d: *const tess_diagram, cpd: *mut i64, bounds: *mut f64) -> tess_status;
    // Cell / VoronoiFace (interface.rs:186-416)
    pub fn tess_cell_volume(d: *const tess_diagram, i: usize, volume: *mut f64) -> tess_status;
    pub fn tess_cell_neighbors(d: *const tess_diagram, i: usize, nbr: *mut i32, cap: usize,
                               count: *mut usize) -> tess_status;
    pub fn tess_cell_faces(d: *const tess_diagram, i: usize, nbr: *mut i32, area: *mut f64,
                           cap: usize, count: *mut usize) -> tess_status;
    pub fn tess_cell_vertices(d: *mut tess_diagram, i: usize, xyz: *mut f64, cap: usize,
                              count: *mut usize) -> tess_status;
    pub fn tess_cell_face_vertices(d: *mut tess_diagram, i: usize, face: usize, xyz: *mut f64, cap: usize,
                                   count: *mut usize) -> tess_status;
    pub fn tess_cell_original_index(d: *const tess_diagram, i: usize, original: *mut usize) -> tess_status;
    pub fn tess_cell_compute(d: *mut tess_diagram, i: usize, precision: c_int, search_radius: f64,
                             target_group: i64, lo: *const f64, hi: *const f64,
                             out: *mut tess_cell_geometry) -> tess_status;
    pub fn tess_cell_compute_at(d: *mut tess_diagram, p: *const f64, precision: c_int,
                                search_radius: f64, target_group: i64, lo: *const f64,
                                hi: *const f64, out: *mut tess_cell_geometry) -> tess_status;
    // bulk results
    pub fn tess_volumes(d: *mut tess_diagram, volumes: *mut f64) -> tess_status;
    pub fn tess_neighbors_csr(d: *mut tess_diagram, offs: *mut u64, nbr: *mut i32, area: *mut f64,
                              cap: usize, total: *mut usize) -> tess_status;
    pub fn tess_results_device(d: *mut tess_diagram, volumes: *mut *const f64, offs: *mut *const u64,
                               nbr: *mut *const i32, area: *mut *const f64, total: *mut usize) -> tess_status;
    pub fn tess_diagram_compute_all_to_host(d: *mut tess_diagram, precision: c_int, search_radius: f64,
                                            target_group: i64, volumes: *mut f64, face_start: *mut u64,
                                            face_count: *mut u32, face_nbr: *mut i32, face_area: *mut f64,
                                            face_cap: usize, faces_used: *mut usize) -> tess_status;
    pub fn tess_host_alloc(bytes: usize, ptr: *mut *mut c_void) -> tess_status;
    pub fn tess_host_free(ptr: *mut c_void) -> tess_status;
    // fixed-radius queries (celery.rs:753-855, interface.rs:348-365)
    pub fn tess_find_cells_in_radius(d: *mut tess_diagram, xyz: *const f64, nq: usize, radius: f64,
                                     on_device: c_int, offs: *mut u64, cells: *mut u32, cap: usize,
                                     total: *mut usize) -> tess_status;
    pub fn tess_find_neighbors_in_radius(d: *mut tess_diagram, xyz: *const f64, nq: usize, radius: f64,
                                         real_radius: c_int, on_device: c_int, offs: *mut u64, ids: *mut u32,
                                         cap: usize, total: *mut usize) -> tess_status;
    pub fn tess_neighbor_cloud(d: *mut tess_diagram, cells: *const u32, ncells: usize, radius: f64,
                               target_group: i64, on_device: c_int, offs: *mut u64, ids: *mut u32,
                               cap: usize, total: *mut usize) -> tess_status;
    pub fn tess_neighbor_cloud_at(d: *mut tess_diagram, xyz: *const f64, nq: usize, radius: f64,
                                  target_group: i64, on_device: c_int, offs: *mut u64, ids: *mut u32,
                                  cap: usize, total: *mut usize) -> tess_status;
    // many diagrams in one CUDA-graph launch
    pub fn tess_batch_create(ndiag: usize, pt_offsets: *const u64, xyz: *const f64, boxes: *const f64,
                             cfg: *const tess_config, out: *mut *mut tess_batch) -> tess_status;
    pub fn tess_batch_compute(b: *mut tess_batch, precision: c_int) -> tess_status;
    pub fn tess_batch_compute_to_host(b: *mut tess_batch, precision: c_int, volumes: *mut f64, face_start: *mut u64,
                                      face_count: *mut u32, face_nbr: *mut i32, face_area: *mut f64,
                                      face_cap: usize, faces_used: *mut usize) -> tess_status;
    pub fn tess_batch_update_points(b: *mut tess_batch, xyz: *const f64, on_device: c_int) -> tess_status;
    pub fn tess_batch_stats(b: *const tess_batch, out: *mut tess_stats) -> tess_status;
    pub fn tess_batch_volumes(b: *mut tess_batch, volumes: *mut f64) -> tess_status;
    pub fn tess_batch_neighbors_csr(b: *mut tess_batch, offs: *mut u64, nbr: *mut i32, area: *mut f64,
                                    cap: usize, total: *mut usize) -> tess_status;
    pub fn tess_batch_results_device(b: *mut tess_batch, volumes: *mut *const f64, offs: *mut *const u64,
                                     nbr: *mut *const i32, area: *mut *const f64, total: *mut usize) -> tess_status;
    pub fn tess_batch_destroy(b: *mut tess_batch) -> tess_status;
    // autotuning of the launch knobs (sample-timed, cached)
    pub fn tess_diagram_autotune(d: *mut tess_diagram, precision: c_int, cache_path: *const c_char,
                                 out: *mut tess_tuning) -> tess_status;
    pub fn tess_batch_autotune(b: *mut tess_batch, precision: c_int, cache_path: *const c_char,
                               out: *mut tess_tuning) -> tess_status;
    // CSR offsets from device face counts, allocating nothing
    pub fn tess_csr_offsets_noalloc(d_counts: *const u32, n: usize, d_offs: *mut u64,
                                    stream: *mut c_void) -> tess_status;
}
