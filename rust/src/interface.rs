//! Safe wrapper with the reference's public names (`src/interface.rs`).
//!
//! * `Diagram::new` is the constructor the reference lacks
//!   (`add_particle_with_group` x n + `initialize`, interface.rs:52-84).
//! * `Diagram::get_cell_at_index` / `get_cell_at_particle` (interface.rs:186-232)
//!   take the container by value, as the reference's `Polyhedron` argument, and
//!   return a `Cell`; `Cell::compute_voronoi_cell` (interface.rs:257-313) runs
//!   the cell on the GPU.
//! * `Cell::compute_volume`, `compute_neighbors`, `compute_vertices`,
//!   `compute_faces`, `original_index`, `compute_neighbor_cloud`
//!   (interface.rs:337-389) and `VoronoiFace::compute_vertices`,
//!   `compute_area`, `compute_neighbor` (interface.rs:403-416) read its result.
//! * Bulk use, the path the GPU is built for: `Diagram::compute_all`, then
//!   `volumes` and `neighbors_csr`.
//!
//! Differences a caller sees: errors come back as `Result` instead of panics;
//! box walls are neighbours -1..-6 (x_min, x_max, y_min, y_max, z_min, z_max)
//! where the reference panics (polyhedron.rs:877); vertices are relative to
//! the cell's site, as the reference leaves its polyhedron translated.
use crate::gpu_ffi::*;
use std::ffi::CStr;
use std::os::raw::{c_char, c_void};
use std::ptr;

/// A failed call: its status code and the library's message.
#[derive(Debug, Clone)]
pub struct Error {
    pub status: i32,
    pub message: String,
}

fn last_error() -> String {
    let mut buf = vec![0u8; 512];
    unsafe { tess_last_error(buf.as_mut_ptr() as *mut c_char, buf.len()) };
    let s = unsafe { CStr::from_ptr(buf.as_ptr() as *const c_char) };
    s.to_string_lossy().into_owned()
}

fn check(st: tess_status) -> Result<(), Error> {
    if st == TESS_OK {
        Ok(())
    } else {
        Err(Error { status: st, message: last_error() })
    }
}

/// Arithmetic of the clipping: plain FP64 (the reference's type), FP32 with
/// FP64 guard-band re-runs (volumes to about 1e-7), or FP32 clipping with an
/// FP64-accurate finish (volumes within 1e-11 of FP64).  Neighbour lists are
/// the same.
#[derive(Clone, Copy, Debug, PartialEq)]
pub enum Precision {
    Fp64,
    Fp32Guard,
    Mixed,
}

impl Precision {
    fn code(self) -> i32 {
        match self {
            Precision::Fp64 => TESS_PRECISION_FP64,
            Precision::Fp32Guard => TESS_PRECISION_FP32_GUARD,
            Precision::Mixed => TESS_PRECISION_MIXED,
        }
    }
}

/// The container box (`Polyhedron::new`, polyhedron.rs:226-244).
#[derive(Clone, Copy, Debug)]
pub struct Polyhedron {
    lo: [f64; 3],
    hi: [f64; 3],
}

impl Polyhedron {
    pub fn new(x_min: f64, y_min: f64, z_min: f64, x_max: f64, y_max: f64, z_max: f64) -> Polyhedron {
        Polyhedron { lo: [x_min, y_min, z_min], hi: [x_max, y_max, z_max] }
    }
}

fn box_ptrs(p: Option<&Polyhedron>) -> (*const f64, *const f64) {
    p.map_or((ptr::null(), ptr::null()), |p| (p.lo.as_ptr(), p.hi.as_ptr()))
}

fn radius_arg(r: Option<f64>) -> f64 {
    r.unwrap_or(-1.0)
}

fn group_arg(g: Option<usize>) -> i64 {
    g.map_or(-1, |g| g as i64)
}

/// Points, groups and the GPU bin grid (Diagram, interface.rs:25-84).
pub struct Diagram {
    h: *mut tess_diagram,
    n: usize,
    precision: Precision,
}

impl Diagram {
    /// `container` None: the reference's Diagram bounding box (grown from the
    /// origin to contain every point, interface.rs:53-54).
    pub fn new(points: &[[f64; 3]], groups: Option<&[u32]>, container: Option<&Polyhedron>) -> Result<Diagram, Error> {
        Diagram::with_config(points, groups, container, None)
    }

    pub fn with_config(points: &[[f64; 3]], groups: Option<&[u32]>, container: Option<&Polyhedron>,
                       config: Option<&tess_config>) -> Result<Diagram, Error> {
        if let Some(g) = groups {
            if g.len() != points.len() {
                return Err(Error { status: TESS_E_INVALID, message: "one group per point".into() });
            }
        }
        let mut h = ptr::null_mut();
        let (lo, hi) = box_ptrs(container);
        let g = groups.map_or(ptr::null(), |g| g.as_ptr());
        let cfg = config.map_or(ptr::null(), |c| c as *const tess_config);
        check(unsafe { tess_diagram_create(points.as_ptr() as *const f64, points.len(), g, lo, hi, cfg, &mut h) })?;
        Ok(Diagram { h, n: points.len(), precision: Precision::Fp64 })
    }

    pub fn len(&self) -> usize {
        self.n
    }

    /// Precision used by the cells `get_cell_at_*` make (FP64 by default).
    pub fn set_cell_precision(&mut self, p: Precision) {
        self.precision = p;
    }

    /// Every cell: get_cell_at_index(i) + compute_voronoi_cell() for all i.
    pub fn compute_all(&mut self, precision: Precision, search_radius: Option<f64>,
                       target_group: Option<usize>) -> Result<(), Error> {
        check(unsafe { tess_diagram_compute_all(self.h, precision.code(), radius_arg(search_radius),
                                                group_arg(target_group)) })
    }

    /// Volume of every cell after `compute_all`.
    pub fn volumes(&self) -> Result<Vec<f64>, Error> {
        let mut v = vec![0.0; self.n];
        check(unsafe { tess_volumes(self.h, v.as_mut_ptr()) })?;
        Ok(v)
    }

    /// Faces of every cell after `compute_all`, as CSR: offsets[n + 1],
    /// neighbour ids (walls -1..-6) and areas, each cell's faces sorted by id.
    pub fn neighbors_csr(&self) -> Result<(Vec<u64>, Vec<i32>, Vec<f64>), Error> {
        let mut offs = vec![0u64; self.n + 1];
        let mut total = 0usize;
        check(unsafe { tess_neighbors_csr(self.h, offs.as_mut_ptr(), ptr::null_mut(), ptr::null_mut(), 0, &mut total) })?;
        let mut nbr = vec![0i32; total];
        let mut area = vec![0.0f64; total];
        check(unsafe { tess_neighbors_csr(self.h, ptr::null_mut(), nbr.as_mut_ptr(), area.as_mut_ptr(), total, &mut total) })?;
        Ok((offs, nbr, area))
    }

    /// Pick the clipping launch knobs for these points (timed on a sample of
    /// the cells, cached on disk); later computes use them.
    pub fn autotune(&mut self, precision: Precision) -> Result<tess_tuning, Error> {
        let mut t = tess_tuning::default();
        check(unsafe { tess_diagram_autotune(self.h, precision.code(), ptr::null(), &mut t) })?;
        Ok(t)
    }

    /// `compute_all` with every cell's faces written into a pinned host pool
    /// while the cells finish (tess_diagram_compute_all_to_host).  `face_cap`
    /// sizes the pool; a pool too small is grown once to the size the call
    /// reports.
    pub fn compute_all_to_host(&mut self, precision: Precision, search_radius: Option<f64>,
                               target_group: Option<usize>, face_cap: usize) -> Result<HostResults, Error> {
        let (h, p, r, g) = (self.h, precision.code(), radius_arg(search_radius), group_arg(target_group));
        to_host(self.n, face_cap, |v, fs, fc, nb, ar, cap, used| unsafe {
            tess_diagram_compute_all_to_host(h, p, r, g, v, fs, fc, nb, ar, cap, used)
        })
    }

    /// get_cell_at_index (interface.rs:186-208).
    pub fn get_cell_at_index(&self, index: usize, polyhedron: Polyhedron, search_radius: Option<f64>,
                             target_group: Option<usize>) -> Cell {
        Cell::new(self, Some(index), [0.0; 3], polyhedron, search_radius, target_group)
    }

    /// get_cell_at_particle (interface.rs:211-232): a cell for a position
    /// that is not a point of the diagram.
    pub fn get_cell_at_particle(&self, point: [f64; 3], polyhedron: Polyhedron, search_radius: Option<f64>,
                                target_group: Option<usize>) -> Cell {
        Cell::new(self, None, point, polyhedron, search_radius, target_group)
    }

    fn radius_query(&self, p: [f64; 3], radius: f64, real: Option<bool>) -> Result<Vec<usize>, Error> {
        let mut offs = [0u64; 2];
        let mut total = 0usize;
        let call = |ids: *mut u32, cap: usize, total: &mut usize, offs: &mut [u64; 2]| unsafe {
            match real {
                None => tess_find_cells_in_radius(self.h, p.as_ptr(), 1, radius, 0, offs.as_mut_ptr(), ids, cap, total),
                Some(r) => tess_find_neighbors_in_radius(self.h, p.as_ptr(), 1, radius, r as i32, 0, offs.as_mut_ptr(),
                                                         ids, cap, total),
            }
        };
        check(call(ptr::null_mut(), 0, &mut total, &mut offs))?;
        let mut ids = vec![0u32; total];
        check(call(ids.as_mut_ptr(), total, &mut total, &mut offs))?;
        Ok(ids.into_iter().map(|i| i as usize).collect())
    }

    /// Celery::find_cells_in_radius (celery.rs:753-796): bin ids.
    pub fn find_cells_in_radius(&self, x: f64, y: f64, z: f64, radius: f64) -> Result<Vec<usize>, Error> {
        self.radius_query([x, y, z], radius, None)
    }

    /// Celery::find_neighbors_in_cell_radius (celery.rs:802-818).
    pub fn find_neighbors_in_cell_radius(&self, x: f64, y: f64, z: f64, radius: f64) -> Result<Vec<usize>, Error> {
        self.radius_query([x, y, z], radius, Some(false))
    }

    /// Celery::find_neighbors_in_real_radius (celery.rs:825-855).
    pub fn find_neighbors_in_real_radius(&self, x: f64, y: f64, z: f64, radius: f64) -> Result<Vec<usize>, Error> {
        self.radius_query([x, y, z], radius, Some(true))
    }
}

impl Drop for Diagram {
    fn drop(&mut self) {
        unsafe { tess_diagram_destroy(self.h) };
    }
}

/// Runs a to-host compute into fresh per-cell arrays and a pinned face pool
/// of `face_cap`, grown once to the size a TESS_E_CAPACITY reports.
fn to_host<F>(n: usize, face_cap: usize, call: F) -> Result<HostResults, Error>
where
    F: Fn(*mut f64, *mut u64, *mut u32, *mut i32, *mut f64, usize, *mut usize) -> tess_status,
{
    let mut cap = face_cap.max(1);
    for _ in 0..2 {
        let nbr = PinnedBuf::<i32>::new(cap)?;
        let area = PinnedBuf::<f64>::new(cap)?;
        let mut volumes = vec![0.0f64; n];
        let mut face_start = vec![0u64; n];
        let mut face_count = vec![0u32; n];
        let mut used = 0usize;
        let st = call(volumes.as_mut_ptr(), face_start.as_mut_ptr(), face_count.as_mut_ptr(), nbr.ptr, area.ptr, cap,
                      &mut used);
        if st == TESS_E_CAPACITY {
            cap = used;
            continue;
        }
        check(st)?;
        return Ok(HostResults { volumes, face_start, face_count, face_nbr: nbr, face_area: area, faces_used: used });
    }
    Err(Error { status: TESS_E_CAPACITY, message: last_error() })
}

/// Pinned, device-mapped host memory (tess_host_alloc).
pub struct PinnedBuf<T: Copy> {
    ptr: *mut T,
    len: usize,
}

impl<T: Copy> PinnedBuf<T> {
    pub fn new(len: usize) -> Result<Self, Error> {
        let mut p: *mut c_void = ptr::null_mut();
        check(unsafe { tess_host_alloc(len * std::mem::size_of::<T>(), &mut p) })?;
        Ok(PinnedBuf { ptr: p as *mut T, len })
    }

    pub fn as_slice(&self) -> &[T] {
        if self.len == 0 {
            &[]
        } else {
            unsafe { std::slice::from_raw_parts(self.ptr, self.len) }
        }
    }
}

impl<T: Copy> Drop for PinnedBuf<T> {
    fn drop(&mut self) {
        unsafe { tess_host_free(self.ptr as *mut c_void) };
    }
}

/// Every cell's results from `compute_all_to_host`: cell i's faces are
/// `face_nbr` / `face_area` at `face_start[i] .. face_start[i] + face_count[i]`
/// (sorted by neighbour id, walls -1..-6).
pub struct HostResults {
    pub volumes: Vec<f64>,
    pub face_start: Vec<u64>,
    pub face_count: Vec<u32>,
    pub face_nbr: PinnedBuf<i32>,
    pub face_area: PinnedBuf<f64>,
    pub faces_used: usize,
}

impl HostResults {
    /// Neighbour ids and areas of cell i.
    pub fn faces(&self, i: usize) -> (&[i32], &[f64]) {
        let a = self.face_start[i] as usize;
        let b = a + self.face_count[i] as usize;
        (&self.face_nbr.as_slice()[a..b], &self.face_area.as_slice()[a..b])
    }
}

/// A Voronoi cell (Cell, interface.rs:237-253).
pub struct Cell<'a> {
    diagram: &'a Diagram,
    index: Option<usize>,
    position: [f64; 3],
    polyhedron: Polyhedron,
    search_radius: Option<f64>,
    target_group: Option<usize>,
    geom: Option<Box<tess_cell_geometry>>,
}

impl<'a> Cell<'a> {
    fn new(diagram: &'a Diagram, index: Option<usize>, position: [f64; 3], polyhedron: Polyhedron,
           search_radius: Option<f64>, target_group: Option<usize>) -> Cell<'a> {
        Cell { diagram, index, position, polyhedron, search_radius, target_group, geom: None }
    }

    /// Clip the container by the bisectors of the nearby points
    /// (compute_voronoi_cell, interface.rs:257-313).
    pub fn compute_voronoi_cell(&mut self) -> Result<(), Error> {
        let mut g: Box<tess_cell_geometry> = Box::new(unsafe { std::mem::zeroed() });
        let (lo, hi) = (self.polyhedron.lo.as_ptr(), self.polyhedron.hi.as_ptr());
        let p = self.diagram.precision.code();
        let r = radius_arg(self.search_radius);
        let tg = group_arg(self.target_group);
        let st = unsafe {
            match self.index {
                Some(i) => tess_cell_compute(self.diagram.h, i, p, r, tg, lo, hi, &mut *g),
                None => tess_cell_compute_at(self.diagram.h, self.position.as_ptr(), p, r, tg, lo, hi, &mut *g),
            }
        };
        check(st)?;
        self.geom = Some(g);
        Ok(())
    }

    fn geom(&self) -> &tess_cell_geometry {
        self.geom.as_ref().expect("compute_voronoi_cell has not run")
    }

    pub fn compute_volume(&self) -> f64 {
        self.geom().volume
    }

    /// Neighbour ids (original indices) sorted ascending; walls are -1..-6.
    pub fn compute_neighbors(&self) -> Vec<i64> {
        let g = self.geom();
        g.face_neighbor[..g.nfaces as usize].iter().map(|&x| x as i64).collect()
    }

    /// Vertices relative to the cell's site.
    pub fn compute_vertices(&self) -> Vec<[f64; 3]> {
        let g = self.geom();
        (0..g.nvertices as usize).map(|v| [g.vertices[3 * v], g.vertices[3 * v + 1], g.vertices[3 * v + 2]]).collect()
    }

    pub fn compute_faces(&self) -> Vec<VoronoiFace<'_, 'a>> {
        (0..self.geom().nfaces as usize).map(|f| VoronoiFace { face_index: f, cell: self }).collect()
    }

    pub fn original_index(&self) -> Option<usize> {
        self.index
    }

    /// compute_neighbor_cloud (interface.rs:348-365): the points of every bin
    /// up to the first search-order key above `radius`, in search order.
    pub fn compute_neighbor_cloud(&self, radius: f64, target_group: Option<usize>) -> Result<Vec<usize>, Error> {
        let mut offs = [0u64; 2];
        let mut total = 0usize;
        let tg = group_arg(target_group);
        let h = self.diagram.h;
        let st = match self.index {
            Some(i) => {
                let cell = [i as u32];
                unsafe { tess_neighbor_cloud(h, cell.as_ptr(), 1, radius, tg, 0, offs.as_mut_ptr(), ptr::null_mut(), 0, &mut total) }
            }
            None => unsafe {
                tess_neighbor_cloud_at(h, self.position.as_ptr(), 1, radius, tg, 0, offs.as_mut_ptr(), ptr::null_mut(), 0,
                                       &mut total)
            },
        };
        check(st)?;
        let mut ids = vec![0u32; total];
        let st = match self.index {
            Some(i) => {
                let cell = [i as u32];
                unsafe { tess_neighbor_cloud(h, cell.as_ptr(), 1, radius, tg, 0, offs.as_mut_ptr(), ids.as_mut_ptr(), total, &mut total) }
            }
            None => unsafe {
                tess_neighbor_cloud_at(h, self.position.as_ptr(), 1, radius, tg, 0, offs.as_mut_ptr(), ids.as_mut_ptr(), total,
                                       &mut total)
            },
        };
        check(st)?;
        Ok(ids.into_iter().map(|i| i as usize).collect())
    }
}

/// One face of a cell (VoronoiFace, interface.rs:393-416).
pub struct VoronoiFace<'a, 'b: 'a> {
    face_index: usize,
    cell: &'a Cell<'b>,
}

impl<'a, 'b> VoronoiFace<'a, 'b> {
    /// The face's vertex cycle, counter-clockwise seen from outside the cell.
    pub fn compute_vertices(&self) -> Vec<[f64; 3]> {
        let g = self.cell.geom();
        let (b, e) = (g.face_offset[self.face_index] as usize, g.face_offset[self.face_index + 1] as usize);
        g.face_vertex[b..e]
            .iter()
            .map(|&v| {
                let v = v as usize;
                [g.vertices[3 * v], g.vertices[3 * v + 1], g.vertices[3 * v + 2]]
            })
            .collect()
    }

    pub fn compute_area(&self) -> f64 {
        self.cell.geom().face_area[self.face_index]
    }

    /// The neighbour across the face (a wall: -1..-6).
    pub fn compute_neighbor(&self) -> i64 {
        self.cell.geom().face_neighbor[self.face_index] as i64
    }
}

/// Many independent diagrams, each in its own box, computed in one CUDA-graph
/// launch (no reference counterpart: the reference builds one diagram at a time).
pub struct Batch {
    h: *mut tess_batch,
    n: usize,
}

impl Batch {
    /// `offsets`: ndiag + 1 point offsets into `points`; `boxes`:
    /// {x_min, y_min, z_min, x_max, y_max, z_max} per diagram.
    pub fn new(points: &[[f64; 3]], offsets: &[u64], boxes: &[[f64; 6]], config: Option<&tess_config>) -> Result<Batch, Error> {
        if offsets.len() != boxes.len() + 1 {
            return Err(Error { status: TESS_E_INVALID, message: "one box per diagram".into() });
        }
        let mut h = ptr::null_mut();
        let cfg = config.map_or(ptr::null(), |c| c as *const tess_config);
        check(unsafe { tess_batch_create(boxes.len(), offsets.as_ptr(), points.as_ptr() as *const f64,
                                         boxes.as_ptr() as *const f64, cfg, &mut h) })?;
        Ok(Batch { h, n: points.len() })
    }

    pub fn compute(&mut self, precision: Precision) -> Result<(), Error> {
        check(unsafe { tess_batch_compute(self.h, precision.code()) })
    }

    /// `compute` with the faces written into a pinned host pool as the cells
    /// finish (tess_batch_compute_to_host); neighbour ids are local to each
    /// diagram.
    pub fn compute_to_host(&mut self, precision: Precision, face_cap: usize) -> Result<HostResults, Error> {
        let (h, p) = (self.h, precision.code());
        to_host(self.n, face_cap, |v, fs, fc, nb, ar, cap, used| unsafe {
            tess_batch_compute_to_host(h, p, v, fs, fc, nb, ar, cap, used)
        })
    }

    /// As Diagram::autotune, with the batch's grid density among the knobs.
    pub fn autotune(&mut self, precision: Precision) -> Result<tess_tuning, Error> {
        let mut t = tess_tuning::default();
        check(unsafe { tess_batch_autotune(self.h, precision.code(), ptr::null(), &mut t) })?;
        Ok(t)
    }

    /// New positions for every diagram (same sizes and boxes).
    pub fn update_points(&mut self, points: &[[f64; 3]]) -> Result<(), Error> {
        if points.len() != self.n {
            return Err(Error { status: TESS_E_INVALID, message: "update_points keeps the point count".into() });
        }
        check(unsafe { tess_batch_update_points(self.h, points.as_ptr() as *const f64, 0) })
    }

    pub fn volumes(&self) -> Result<Vec<f64>, Error> {
        let mut v = vec![0.0; self.n];
        check(unsafe { tess_batch_volumes(self.h, v.as_mut_ptr()) })?;
        Ok(v)
    }

    /// CSR over all points; neighbour ids are local to each diagram.
    pub fn neighbors_csr(&self) -> Result<(Vec<u64>, Vec<i32>, Vec<f64>), Error> {
        let mut offs = vec![0u64; self.n + 1];
        let mut total = 0usize;
        check(unsafe { tess_batch_neighbors_csr(self.h, offs.as_mut_ptr(), ptr::null_mut(), ptr::null_mut(), 0, &mut total) })?;
        let mut nbr = vec![0i32; total];
        let mut area = vec![0.0f64; total];
        check(unsafe { tess_batch_neighbors_csr(self.h, ptr::null_mut(), nbr.as_mut_ptr(), area.as_mut_ptr(), total, &mut total) })?;
        Ok((offs, nbr, area))
    }
}

impl Drop for Batch {
    fn drop(&mut self) {
        unsafe { tess_batch_destroy(self.h) };
    }
}
