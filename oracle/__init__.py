"""CPU oracle for the Voronoi cell path: a ctypes binding of ``tess_oracle.c``.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import this package; the library in
``the-tessellator_gb300/`` never does.

The C code restates the reference algorithm (mcomstock/the-tessellator:
``src/celery.rs``, ``src/vector3.rs``, ``src/polyhedron.rs``,
``src/interface.rs``); each C function cites the lines it follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "tess_oracle.c")

MODE_SECURE, MODE_BRUTE, MODE_RADIUS = 0, 1, 2
TOLERANCE = 1e-12


def build(force: bool = False) -> str:
    """Compile ``liboracle.so`` next to its source (gcc, OpenMP, no FMA contraction)."""
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "tess_oracle.h"))
    ):
        return LIB_PATH
    cmd = [
        "gcc", "-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
        "-Wall", "-o", LIB_PATH + ".tmp", SRC, "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class GridInfo(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax", "sx", "sy", "sz", "ix", "iy", "iz")] + [
        ("cpd", C.c_int64)]


class CellStats(C.Structure):
    _fields_ = [("candidates", C.c_int64), ("classified", C.c_int64), ("cuts", C.c_int64),
                ("new_vertices", C.c_int64), ("fan_triangles", C.c_int64), ("faces", C.c_int64),
                ("min_abs_sd_rel", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        d3 = C.POINTER(C.c_double)
        u32p = C.POINTER(C.c_uint32)
        L.or_dot.restype = C.c_double
        L.or_dot.argtypes = [d3, d3]
        L.or_cross.argtypes = [d3, d3, d3]
        L.or_halfway_from_origin_to.argtypes = [d3, d3]
        L.or_plane_from_normal_and_point.argtypes = [d3, d3, d3]
        L.or_vector_location.restype = C.c_int
        L.or_vector_location.argtypes = [d3, d3, C.c_double]
        L.or_intersection.argtypes = [d3, d3, d3, d3]
        L.or_cells_per_dimension.restype = C.c_int64
        L.or_cells_per_dimension.argtypes = [C.c_size_t]
        L.or_grid_info_compute.argtypes = [d3, C.c_size_t, C.POINTER(GridInfo)]
        L.or_axis_index.restype = C.c_int64
        L.or_axis_index.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double, C.c_int64]
        L.or_bin_ids.argtypes = [d3, C.c_size_t, C.POINTER(GridInfo), u32p]
        L.or_sort_bins.argtypes = [u32p, C.c_size_t, C.c_uint64, u32p, u32p]
        L.or_search_order.restype = C.c_size_t
        L.or_search_order.argtypes = [C.POINTER(GridInfo), C.POINTER(C.c_int32), d3]
        L.or_gap_key.restype = C.c_double
        L.or_gap_key.argtypes = [C.POINTER(GridInfo), C.c_int32, C.c_int32, C.c_int32]
        L.or_diagram_create.restype = C.c_void_p
        L.or_diagram_create.argtypes = [d3, C.c_size_t, u32p, d3, d3]
        L.or_diagram_destroy.argtypes = [C.c_void_p]
        L.or_diagram_grid.argtypes = [C.c_void_p, C.POINTER(GridInfo)]
        L.or_diagram_box.argtypes = [C.c_void_p, d3, d3]
        for f in ("or_diagram_sorted", "or_diagram_delims", "or_diagram_bins"):
            getattr(L, f).restype = u32p
            getattr(L, f).argtypes = [C.c_void_p]
        L.or_cell_compute.restype = C.c_void_p
        L.or_cell_compute.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_double, C.c_int64]
        L.or_cell_compute_at.restype = C.c_void_p
        L.or_cell_compute_at.argtypes = [C.c_void_p, d3, C.c_int, C.c_double, C.c_int64]
        L.or_cell_destroy.argtypes = [C.c_void_p]
        L.or_cell_volume.restype = C.c_double
        L.or_cell_volume.argtypes = [C.c_void_p]
        L.or_cell_nfaces.restype = C.c_int
        L.or_cell_nfaces.argtypes = [C.c_void_p]
        L.or_cell_faces.argtypes = [C.c_void_p, C.POINTER(C.c_int64), d3, C.POINTER(C.c_int32)]
        L.or_cell_nvertices.restype = C.c_int
        L.or_cell_nvertices.argtypes = [C.c_void_p]
        L.or_cell_vertices.argtypes = [C.c_void_p, d3]
        L.or_cell_face_vertices.restype = C.c_int
        L.or_cell_face_vertices.argtypes = [C.c_void_p, C.c_int, d3, C.c_int]
        L.or_cell_get_stats.argtypes = [C.c_void_p, C.POINTER(CellStats)]
        L.or_compute_all.restype = C.c_void_p
        L.or_compute_all.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int64, C.c_int, u32p, C.c_size_t]
        L.or_all_destroy.argtypes = [C.c_void_p]
        L.or_all_total_faces.restype = C.c_size_t
        L.or_all_total_faces.argtypes = [C.c_void_p]
        L.or_all_results.argtypes = [C.c_void_p, d3, C.POINTER(C.c_int64), C.POINTER(C.c_int64), d3]
        L.or_all_stats.argtypes = [C.c_void_p, C.POINTER(CellStats)]
        L.or_all_seconds.restype = C.c_double
        L.or_all_seconds.argtypes = [C.c_void_p]
        u64p = C.POINTER(C.c_uint64)
        L.or_check_cell_in_range.restype = C.c_int
        L.or_check_cell_in_range.argtypes = [C.c_void_p, d3, C.c_double, C.c_int64, C.c_int64, C.c_int64]
        L.or_find_cells_in_radius.restype = C.c_size_t
        L.or_find_cells_in_radius.argtypes = [C.c_void_p, d3, C.c_size_t, C.c_double, u64p, u32p, C.c_size_t]
        L.or_find_neighbors_in_radius.restype = C.c_size_t
        L.or_find_neighbors_in_radius.argtypes = [C.c_void_p, d3, C.c_size_t, C.c_double, C.c_int, u64p, u32p,
                                                  C.c_size_t]
        L.or_neighbor_cloud.restype = C.c_size_t
        L.or_neighbor_cloud.argtypes = [C.c_void_p, d3, C.c_size_t, C.c_double, C.c_int64, u64p, u32p,
                                        C.c_size_t]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _u32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _v(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


# ---- plane / vector math (vector3.rs) --------------------------------------
def dot(a, b) -> float:
    a, b = _v(a), _v(b)
    return lib().or_dot(_dp(a), _dp(b))


def cross(a, b):
    a, b, o = _v(a), _v(b), np.zeros(3)
    lib().or_cross(_dp(a), _dp(b), _dp(o))
    return o


def halfway_from_origin_to(p):
    p, o = _v(p), np.zeros(4)
    lib().or_halfway_from_origin_to(_dp(p), _dp(o))
    return o


def plane_from_non_unit_normal_and_point(n, p):
    n, p, o = _v(n), _v(p), np.zeros(4)
    lib().or_plane_from_normal_and_point(_dp(n), _dp(p), _dp(o))
    return o


def vector_location(plane, v, tol) -> int:
    plane, v = _v(plane), _v(v)
    return lib().or_vector_location(_dp(plane), _dp(v), tol)


def intersection(plane, a, b):
    plane, a, b, o = _v(plane), _v(a), _v(b), np.zeros(3)
    lib().or_intersection(_dp(plane), _dp(a), _dp(b), _dp(o))
    return o


# ---- grid (celery.rs) -------------------------------------------------------
def cells_per_dimension(n: int) -> int:
    return lib().or_cells_per_dimension(n)


def grid_info(xyz) -> GridInfo:
    xyz = _v(xyz).reshape(-1, 3)
    g = GridInfo()
    lib().or_grid_info_compute(_dp(xyz), len(xyz), C.byref(g))
    return g


def axis_index(x, lo, hi, inv, cpd) -> int:
    return lib().or_axis_index(x, lo, hi, inv, cpd)


def bin_ids(xyz, g: GridInfo):
    xyz = _v(xyz).reshape(-1, 3)
    out = np.zeros(len(xyz), dtype=np.uint32)
    lib().or_bin_ids(_dp(xyz), len(xyz), C.byref(g), _u32p(out))
    return out


def sort_bins(bins, nbins):
    bins = np.ascontiguousarray(bins, dtype=np.uint32)
    s = np.zeros(len(bins), dtype=np.uint32)
    dl = np.zeros(nbins + 1, dtype=np.uint32)
    lib().or_sort_bins(_u32p(bins), len(bins), nbins, _u32p(s), _u32p(dl))
    return s, dl


def search_order(g: GridInfo):
    m = (2 * g.cpd - 1) ** 3
    ijk = np.zeros((m, 3), dtype=np.int32)
    dist = np.zeros(m)
    k = lib().or_search_order(C.byref(g), ijk.ctypes.data_as(C.POINTER(C.c_int32)), _dp(dist))
    return ijk[:k], dist[:k]


def gap_key(g: GridInfo, i, j, k) -> float:
    return lib().or_gap_key(C.byref(g), i, j, k)


# ---- diagram ---------------------------------------------------------------
@dataclass
class CellResult:
    volume: float
    ids: np.ndarray
    areas: np.ndarray
    degrees: np.ndarray
    vertices: np.ndarray
    face_vertices: list
    stats: CellStats


class Diagram:
    """FP64 CPU diagram: the oracle counterpart of the library's Diagram."""

    def __init__(self, xyz, groups=None, lo=None, hi=None):
        L = lib()
        self.xyz = _v(xyz).reshape(-1, 3).copy()
        self.n = len(self.xyz)
        g = None if groups is None else np.ascontiguousarray(groups, dtype=np.uint32)
        self._groups = g
        lo_a = None if lo is None else _v(lo)
        hi_a = None if hi is None else _v(hi)
        self._h = L.or_diagram_create(_dp(self.xyz), self.n, None if g is None else _u32p(g),
                                      None if lo_a is None else _dp(lo_a),
                                      None if hi_a is None else _dp(hi_a))
        if not self._h:
            raise ValueError("oracle diagram: invalid input")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().or_diagram_destroy(h)
            self._h = None

    def grid(self) -> GridInfo:
        g = GridInfo()
        lib().or_diagram_grid(self._h, C.byref(g))
        return g

    def box(self):
        lo, hi = np.zeros(3), np.zeros(3)
        lib().or_diagram_box(self._h, _dp(lo), _dp(hi))
        return lo, hi

    def _u32(self, fn, count):
        p = fn(self._h)
        return np.ctypeslib.as_array(p, shape=(count,)).copy()

    def sorted_indices(self):
        return self._u32(lib().or_diagram_sorted, self.n)

    def bins(self):
        return self._u32(lib().or_diagram_bins, self.n)

    def delimiters(self):
        c = self.grid().cpd
        return self._u32(lib().or_diagram_delims, c ** 3 + 1)

    def _read_cell(self, h) -> CellResult:
        L = lib()
        nf = L.or_cell_nfaces(h)
        ids = np.zeros(nf, dtype=np.int64)
        areas = np.zeros(nf)
        deg = np.zeros(nf, dtype=np.int32)
        L.or_cell_faces(h, ids.ctypes.data_as(C.POINTER(C.c_int64)), _dp(areas),
                        deg.ctypes.data_as(C.POINTER(C.c_int32)))
        nv = L.or_cell_nvertices(h)
        verts = np.zeros((max(nv, 1), 3))
        if nv:
            L.or_cell_vertices(h, _dp(verts))
        fv = []
        for f in range(nf):
            buf = np.zeros((int(deg[f]), 3))
            L.or_cell_face_vertices(h, f, _dp(buf), int(deg[f]))
            fv.append(buf)
        st = CellStats()
        L.or_cell_get_stats(h, C.byref(st))
        vol = L.or_cell_volume(h)
        L.or_cell_destroy(h)
        return CellResult(vol, ids, areas, deg, verts[:nv], fv, st)

    def cell(self, i: int, mode=MODE_SECURE, radius=-1.0, target_group=-1) -> CellResult:
        return self._read_cell(lib().or_cell_compute(self._h, i, mode, radius, target_group))

    def cell_at(self, p, mode=MODE_SECURE, radius=-1.0, target_group=-1) -> CellResult:
        p = _v(p)
        return self._read_cell(lib().or_cell_compute_at(self._h, _dp(p), mode, radius, target_group))

    def compute_all(self, mode=MODE_SECURE, radius=-1.0, target_group=-1, nthreads=0, subset=None):
        """Returns (volumes, offsets, ids, areas, stats, seconds)."""
        L = lib()
        sub = None if subset is None else np.ascontiguousarray(subset, dtype=np.uint32)
        a = L.or_compute_all(self._h, mode, radius, target_group, nthreads,
                             None if sub is None else _u32p(sub), 0 if sub is None else len(sub))
        ncell = self.n if sub is None else len(sub)
        tot = L.or_all_total_faces(a)
        vol = np.zeros(ncell)
        offs = np.zeros(ncell + 1, dtype=np.int64)
        ids = np.zeros(max(tot, 1), dtype=np.int64)
        areas = np.zeros(max(tot, 1))
        L.or_all_results(a, _dp(vol), offs.ctypes.data_as(C.POINTER(C.c_int64)),
                         ids.ctypes.data_as(C.POINTER(C.c_int64)), _dp(areas))
        st = CellStats()
        L.or_all_stats(a, C.byref(st))
        secs = L.or_all_seconds(a)
        L.or_all_destroy(a)
        return vol, offs, ids[:tot], areas[:tot], st, secs

    # ---- radius queries (celery.rs:682-855, interface.rs:348-365) ----------
    def check_cell_in_range(self, p, radius, i, j, k) -> bool:
        p = _v(p)
        return bool(lib().or_check_cell_in_range(self._h, _dp(p), radius, i, j, k))

    def _csr_query(self, fn, q, *args):
        q = _v(q).reshape(-1, 3)
        nq = len(q)
        offs = np.zeros(nq + 1, dtype=np.uint64)
        u64 = C.POINTER(C.c_uint64)
        total = fn(self._h, _dp(q), nq, *args, offs.ctypes.data_as(u64), None, 0)
        out = np.zeros(max(total, 1), dtype=np.uint32)
        fn(self._h, _dp(q), nq, *args, offs.ctypes.data_as(u64), _u32p(out), total)
        return offs, out[:total]

    def find_cells_in_radius(self, q, radius):
        """(offsets, bin ids) for each query position."""
        return self._csr_query(lib().or_find_cells_in_radius, q, radius)

    def find_neighbors_in_radius(self, q, radius, real_radius: bool):
        """(offsets, original indices): find_neighbors_in_{cell,real}_radius."""
        return self._csr_query(lib().or_find_neighbors_in_radius, q, radius, 1 if real_radius else 0)

    def neighbor_cloud(self, q, radius, target_group=-1):
        """(offsets, original indices): compute_neighbor_cloud from each position."""
        return self._csr_query(lib().or_neighbor_cloud, q, radius, target_group)
