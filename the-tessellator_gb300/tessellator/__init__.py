"""tessellator: GB300-native Voronoi cells behind the API of
mcomstock/the-tessellator (src/interface.rs).

The classes mirror the reference's public types:

    Polyhedron   the container box a caller hands to get_cell_at_index
                 (polyhedron.rs:226-244, Polyhedron::new)
    Diagram      point set + GPU bin grid (interface.rs:25-84; the reference
                 has no public constructor, this one takes points and a box)
    Cell         get_cell_at_index / get_cell_at_particle + compute_voronoi_cell
                 (interface.rs:186-334)
    VoronoiFace  compute_vertices / compute_area / compute_neighbor
                 (interface.rs:393-416)

plus the bulk path the GPU is built for: ``Diagram.compute_all`` with
``volumes()`` and ``neighbors_csr()`` (or ``compute_all_to_host``, which
streams every cell's faces into pinned host memory during the compute), and
``Batch`` for many diagrams in one CUDA-graph launch.  Every computation runs in libtessgpu.so on the GPU; there
is no CPU fallback.

Conventions: indices are the caller's original indices; box faces report
neighbour ids -1 (x_min), -2 (x_max), -3 (y_min), -4 (y_max), -5 (z_min),
-6 (z_max); a cell's faces come sorted by neighbour id; vertices are relative
to the cell's site (the reference leaves its polyhedron translated by
-position, interface.rs:266).
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from ._capi import (FLAG_AUTOTUNE, FLAG_COUNTERS, FLAG_NO_CAPACITY_RERUN, FLAG_SMALL_FACE_POOL, FLAG_TIMING,
                    PRECISION_FP32_GUARD, PRECISION_FP64, PRECISION_MIXED, TESS_E_CAPACITY,
                    CellGeometry, Config, Stats, TessError, Tuning, check, default_config, last_error, lib)

__all__ = ["Polyhedron", "Diagram", "Cell", "VoronoiFace", "Batch", "DeviceArray", "TessError", "Config",
           "pinned_empty", "HostResults",
           "default_config", "PRECISION_FP64", "PRECISION_FP32_GUARD", "PRECISION_MIXED", "FLAG_TIMING",
           "FLAG_COUNTERS", "FLAG_SMALL_FACE_POOL", "FLAG_NO_CAPACITY_RERUN", "FLAG_AUTOTUNE", "lib",
           "last_error"]

# "mixed": the FP32 + guard clipping with an FP64-accurate finish (FP64-grade
# results, see TESS_PRECISION_MIXED)
_PREC = {"fp64": PRECISION_FP64, "fp32": PRECISION_FP32_GUARD, "fp32_guard": PRECISION_FP32_GUARD,
         "mixed": PRECISION_MIXED, PRECISION_FP64: PRECISION_FP64, PRECISION_FP32_GUARD: PRECISION_FP32_GUARD,
         PRECISION_MIXED: PRECISION_MIXED}


def _prec(p) -> int:
    try:
        return _PREC[p]
    except KeyError:
        raise ValueError(f"unknown precision {p!r} (use 'fp64', 'fp32' or 'mixed')") from None


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _radius(r: Optional[float]) -> float:
    return -1.0 if r is None else float(r)


def _group(g: Optional[int]) -> int:
    return -1 if g is None else int(g)


class _PinnedBlock:
    """Pinned, device-mapped host memory from tess_host_alloc; freed when the
    last array over it is gone."""

    def __init__(self, nbytes: int):
        self.ptr = C.c_void_p()
        check(lib().tess_host_alloc(max(int(nbytes), 1), C.byref(self.ptr)))
        self.nbytes = max(int(nbytes), 1)

    def __del__(self):
        if getattr(self, "ptr", None) is not None and self.ptr.value:
            lib().tess_host_free(self.ptr)
            self.ptr = C.c_void_p()


def pinned_empty(n: int, dtype) -> np.ndarray:
    """An uninitialised numpy array of n elements in pinned, device-mapped host
    memory (tess_host_alloc): the face pool of compute_all_to_host."""
    dt = np.dtype(dtype)
    blk = _PinnedBlock(int(n) * dt.itemsize)
    buf = (C.c_char * blk.nbytes).from_address(blk.ptr.value)
    buf._owner = blk   # the array keeps the buffer, the buffer the block
    return np.frombuffer(buf, dtype=dt, count=int(n))


def _to_host(call, n: int, face_pool, default_cap: int) -> "HostResults":
    """Runs call(volumes, face_start, face_count, nbr, area, cap, used_ref) ->
    status into fresh per-cell arrays and the face pool (allocated when None,
    and then grown and retried once on TESS_E_CAPACITY)."""
    vol = np.empty(n, dtype=np.float64)
    fstart = np.empty(n, dtype=np.uint64)
    fcount = np.empty(n, dtype=np.uint32)
    used = C.c_size_t(0)
    retry = face_pool is None
    if face_pool is None:
        face_pool = (pinned_empty(default_cap, np.int32), pinned_empty(default_cap, np.float64))
    for _ in range(2):
        nbr, area = face_pool
        if len(nbr) != len(area) or nbr.dtype != np.int32 or area.dtype != np.float64:
            raise ValueError("face_pool: two arrays of equal length, int32 and float64")
        st = call(vol.ctypes.data, fstart.ctypes.data, fcount.ctypes.data, nbr.ctypes.data, area.ctypes.data,
                  len(nbr), C.byref(used))
        if st == TESS_E_CAPACITY and retry:   # the size needed is in used
            face_pool = (pinned_empty(used.value, np.int32), pinned_empty(used.value, np.float64))
            retry = False
            continue
        check(st)
        break
    return HostResults(vol, fstart, fcount, face_pool[0], face_pool[1], used.value)


class HostResults:
    """Every cell's results from Diagram.compute_all_to_host: cell i's faces
    are face_nbr / face_area[face_start[i] : face_start[i] + face_count[i]]
    (sorted by neighbour id, walls -1..-6)."""

    def __init__(self, volumes, face_start, face_count, face_nbr, face_area, faces_used):
        self.volumes, self.face_start, self.face_count = volumes, face_start, face_count
        self.face_nbr, self.face_area, self.faces_used = face_nbr, face_area, faces_used

    def faces(self, i: int):
        a = int(self.face_start[i])
        b = a + int(self.face_count[i])
        return self.face_nbr[a:b], self.face_area[a:b]

    def csr(self):
        """The same results as Diagram.neighbors_csr: (offsets[n+1], ids, areas)."""
        offs = np.zeros(len(self.volumes) + 1, dtype=np.uint64)
        np.cumsum(self.face_count, out=offs[1:])
        idx = (np.repeat(self.face_start.astype(np.int64) - offs[:-1].astype(np.int64), self.face_count.astype(np.int64))
               + np.arange(int(offs[-1]), dtype=np.int64))
        return offs, self.face_nbr[idx], self.face_area[idx]


class DeviceArray:
    """A device buffer of the library (results_device) exposed through the
    CUDA array interface, so torch.as_tensor(DeviceArray(...), device="cuda")
    (or any consumer of the interface) views it without a copy.  The buffer
    stays owned by the library: it is valid until the next compute, update or
    destroy of its handle."""

    _TYPES = {np.float64: "<f8", np.uint64: "<u8", np.int32: "<i4", np.uint32: "<u4"}

    def __init__(self, ptr: int, count: int, dtype):
        self.__cuda_array_interface__ = {"shape": (int(count),), "typestr": self._TYPES[np.dtype(dtype).type],
                                         "data": (int(ptr), False), "version": 3, "strides": None}


class Polyhedron:
    """The axis-aligned container box (Polyhedron::new, polyhedron.rs:226-244)."""

    def __init__(self, x_min, y_min, z_min, x_max, y_max, z_max):
        self.lo = np.array([x_min, y_min, z_min], dtype=np.float64)
        self.hi = np.array([x_max, y_max, z_max], dtype=np.float64)

    @classmethod
    def new(cls, x_min, y_min, z_min, x_max, y_max, z_max) -> "Polyhedron":
        return cls(x_min, y_min, z_min, x_max, y_max, z_max)


class Diagram:
    """Points, groups and the GPU bin grid (Diagram, interface.rs:25-84).

    ``points``: (n, 3) float64.  ``container``: a Polyhedron box, or None for
    the reference's Diagram bounding box (starts at the origin and grows to
    contain every point).  ``device_ptr``: build from n x 3 doubles already in
    device memory (an integer address) instead of ``points``.
    """

    def __init__(self, points=None, groups=None, container: Optional[Polyhedron] = None,
                 config: Optional[Config] = None, device_ptr: Optional[int] = None, n: Optional[int] = None):
        L = lib()
        self._h = C.c_void_p()
        cfg = config if config is not None else default_config()
        self.config = cfg
        g = None if groups is None else np.ascontiguousarray(groups, dtype=np.uint32)
        lo = None if container is None else np.ascontiguousarray(container.lo)
        hi = None if container is None else np.ascontiguousarray(container.hi)
        gp = None if g is None else g.ctypes.data_as(C.POINTER(C.c_uint32))
        lp = None if lo is None else _dp(lo)
        hp = None if hi is None else _dp(hi)
        if device_ptr is not None:
            if n is None:
                raise ValueError("n is required with device_ptr")
            self.n = int(n)
            check(L.tess_diagram_create_device(C.c_void_p(device_ptr), self.n, gp, lp, hp, C.byref(cfg),
                                               C.byref(self._h)))
        else:
            pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
            self.n = len(pts)
            if g is not None and len(g) != self.n:
                raise ValueError("groups must have one entry per point")
            check(L.tess_diagram_create(_dp(pts), self.n, gp, lp, hp, C.byref(cfg), C.byref(self._h)))
        self.container = container

    # ---- lifetime ----
    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().tess_diagram_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return self.n

    # ---- bulk path ----
    def rebuild(self):
        """Re-bin the points held on the device (Celery::reset, celery.rs:253-266)."""
        check(lib().tess_diagram_rebuild(self._h))

    def update_points(self, points=None, device_ptr: Optional[int] = None):
        """Replace the points (same count) and re-bin them."""
        if device_ptr is not None:
            check(lib().tess_diagram_update_points(self._h, C.c_void_p(device_ptr), 1))
        else:
            pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
            if len(pts) != self.n:
                raise ValueError("update_points keeps the point count")
            check(lib().tess_diagram_update_points(self._h, C.c_void_p(pts.ctypes.data), 0))

    def celery(self):
        """The bin grid's public fields (celery.rs:196-217):
        (cells[n], sorted_indices[n], delimiters[cpd^3 + 1])."""
        cpd, _ = self.grid()
        cells = np.empty(self.n, dtype=np.uint32)
        srt = np.empty(self.n, dtype=np.uint32)
        dl = np.empty(cpd ** 3 + 1, dtype=np.uint32)
        u = lambda a: a.ctypes.data_as(C.POINTER(C.c_uint32))
        check(lib().tess_diagram_celery(self._h, u(cells), u(srt), u(dl)))
        return cells, srt, dl

    def compute_all(self, precision="fp32", search_radius: Optional[float] = None,
                    target_group: Optional[int] = None) -> "Diagram":
        """Every cell: get_cell_at_index(i, ...) + compute_voronoi_cell().

        ``precision``: "fp32" (FP32 clipping with guard bands and FP64 re-runs;
        volumes to about 1e-7), "mixed" (the same clipping with an FP64-accurate
        finish; volumes to 1e-12) or "fp64" (plain FP64).  Neighbour lists are
        the same in all three."""
        check(lib().tess_diagram_compute_all(self._h, _prec(precision), _radius(search_radius),
                                             _group(target_group)))
        return self

    def autotune(self, precision="fp32", cache_path: Optional[str] = None) -> dict:
        """Pick the clipping launch knobs for these points by timing candidates
        on a sample of the cells (tess_diagram_autotune); later computes use
        them.  cache_path None: the default cache file; "": no cache."""
        t = Tuning()
        cp = None if cache_path is None else cache_path.encode()
        check(lib().tess_diagram_autotune(self._h, _prec(precision), cp, C.byref(t)))
        return t.as_dict()

    def compute_all_to_host(self, precision="fp32", search_radius: Optional[float] = None,
                            target_group: Optional[int] = None, face_pool=None) -> "HostResults":
        """compute_all with every cell's faces written by the GPU into a pinned
        host pool as the cells finish (tess_diagram_compute_all_to_host).

        ``face_pool``: (ids int32, areas float64) arrays from ``pinned_empty``
        of equal length to reuse; None allocates one (grown and retried once
        when the call reports a larger size).  The faces then exist only in
        that pool: neighbors_csr and the per-cell face queries need another
        compute_all."""
        def call(*a):
            return lib().tess_diagram_compute_all_to_host(self._h, _prec(precision), _radius(search_radius),
                                                          _group(target_group), *a)

        return _to_host(call, self.n, face_pool, 20 * self.n + 1024)

    def volumes(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float64)
        check(lib().tess_volumes(self._h, _dp(out)))
        return out

    def neighbors_csr(self):
        """(offsets[n+1] uint64, neighbour ids int32, face areas float64)."""
        L = lib()
        offs = np.empty(self.n + 1, dtype=np.uint64)
        total = C.c_size_t(0)
        check(L.tess_neighbors_csr(self._h, offs.ctypes.data_as(C.POINTER(C.c_uint64)), None, None, 0,
                                   C.byref(total)))
        nbr = np.empty(max(total.value, 1), dtype=np.int32)
        area = np.empty(max(total.value, 1), dtype=np.float64)
        check(L.tess_neighbors_csr(self._h, None, nbr.ctypes.data_as(C.POINTER(C.c_int32)), _dp(area),
                                   len(nbr), C.byref(total)))
        return offs, nbr[:total.value], area[:total.value]

    def results_device(self):
        """Device addresses (volumes, offsets, neighbour ids, areas, total faces)."""
        v, o, nb, a = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        total = C.c_size_t(0)
        check(lib().tess_results_device(self._h, C.byref(v), C.byref(o), C.byref(nb), C.byref(a),
                                        C.byref(total)))
        return v.value, o.value, nb.value, a.value, total.value

    def stats(self) -> dict:
        s = Stats()
        check(lib().tess_diagram_stats(self._h, C.byref(s)))
        return s.as_dict()

    # ---- fixed-radius queries (celery.rs:753-855, interface.rs:348-365) ----
    def _radius_csr(self, call, nq):
        """Runs call(out_ptr, cap, offs_ptr, total_ref) twice: sizes, then results."""
        offs = np.empty(nq + 1, dtype=np.uint64)
        total = C.c_size_t(0)
        check(call(None, 0, C.c_void_p(offs.ctypes.data), C.byref(total)))
        out = np.empty(max(total.value, 1), dtype=np.uint32)
        check(call(C.c_void_p(out.ctypes.data), len(out), None, C.byref(total)))
        return offs, out[:total.value]

    @staticmethod
    def _queries(xyz):
        q = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, 3))
        return q, C.c_void_p(q.ctypes.data if len(q) else None)

    def find_cells_in_radius_batch(self, xyz, radius: float):
        """Celery::find_cells_in_radius for each row of xyz: (offsets, bin ids)."""
        q, qp = self._queries(xyz)
        L = lib()
        return self._radius_csr(lambda o, cap, offs, tot: L.tess_find_cells_in_radius(
            self._h, qp, len(q), float(radius), 0, offs, o, cap, tot), len(q))

    def find_neighbors_in_radius_batch(self, xyz, radius: float, real_radius: bool):
        """find_neighbors_in_{cell,real}_radius for each row: (offsets, point indices)."""
        q, qp = self._queries(xyz)
        L = lib()
        return self._radius_csr(lambda o, cap, offs, tot: L.tess_find_neighbors_in_radius(
            self._h, qp, len(q), float(radius), 1 if real_radius else 0, 0, offs, o, cap, tot), len(q))

    def neighbor_cloud(self, radius: float, cells=None, target_group: Optional[int] = None):
        """Cell::compute_neighbor_cloud for the given cells (None: every cell):
        (offsets, point indices)."""
        L = lib()
        if cells is None:
            c, cp, n = None, None, self.n
        else:
            c = np.ascontiguousarray(np.asarray(cells, dtype=np.uint32).reshape(-1))
            cp, n = C.c_void_p(c.ctypes.data if len(c) else None), len(c)
        return self._radius_csr(lambda o, cap, offs, tot: L.tess_neighbor_cloud(
            self._h, cp, n, float(radius), _group(target_group), 0, offs, o, cap, tot), n)

    def neighbor_cloud_at(self, xyz, radius: float, target_group: Optional[int] = None):
        """compute_neighbor_cloud from positions (cells made by get_cell_at_particle)."""
        q, qp = self._queries(xyz)
        L = lib()
        return self._radius_csr(lambda o, cap, offs, tot: L.tess_neighbor_cloud_at(
            self._h, qp, len(q), float(radius), _group(target_group), 0, offs, o, cap, tot), len(q))

    def find_cells_in_radius(self, x: float, y: float, z: float, radius: float) -> List[int]:
        """Celery::find_cells_in_radius (celery.rs:753-796)."""
        return self.find_cells_in_radius_batch([[x, y, z]], radius)[1].tolist()

    def find_neighbors_in_cell_radius(self, x: float, y: float, z: float, radius: float) -> List[int]:
        """Celery::find_neighbors_in_cell_radius (celery.rs:802-818)."""
        return self.find_neighbors_in_radius_batch([[x, y, z]], radius, False)[1].tolist()

    def find_neighbors_in_real_radius(self, x: float, y: float, z: float, radius: float) -> List[int]:
        """Celery::find_neighbors_in_real_radius (celery.rs:825-855)."""
        return self.find_neighbors_in_radius_batch([[x, y, z]], radius, True)[1].tolist()

    def grid(self):
        """(cells_per_dimension, bounds {xmin, xmax, ymin, ymax, zmin, zmax})."""
        cpd = C.c_int64(0)
        b = np.zeros(6)
        check(lib().tess_diagram_grid(self._h, C.byref(cpd), _dp(b)))
        return cpd.value, b

    # ---- per-cell results of the last compute_all ----
    def cell_volume(self, i: int) -> float:
        v = C.c_double(0.0)
        check(lib().tess_cell_volume(self._h, i, C.byref(v)))
        return v.value

    def cell_faces(self, i: int):
        """(neighbour ids, areas) of cell i, sorted by id."""
        L = lib()
        cnt = C.c_size_t(0)
        nbr = np.empty(256, dtype=np.int32)
        area = np.empty(256, dtype=np.float64)
        check(L.tess_cell_faces(self._h, i, nbr.ctypes.data_as(C.POINTER(C.c_int32)), _dp(area), 256,
                                C.byref(cnt)))
        return nbr[:cnt.value].copy(), area[:cnt.value].copy()

    def cell_neighbors(self, i: int) -> np.ndarray:
        return self.cell_faces(i)[0]

    def cell_vertices(self, i: int) -> np.ndarray:
        cnt = C.c_size_t(0)
        buf = np.empty((256, 3), dtype=np.float64)
        check(lib().tess_cell_vertices(self._h, i, _dp(buf), 256, C.byref(cnt)))
        return buf[:cnt.value].copy()

    def cell_face_vertices(self, i: int, face: int) -> np.ndarray:
        cnt = C.c_size_t(0)
        buf = np.empty((256, 3), dtype=np.float64)
        check(lib().tess_cell_face_vertices(self._h, i, face, _dp(buf), 256, C.byref(cnt)))
        return buf[:cnt.value].copy()

    # ---- the reference's per-cell API ----
    def get_cell_at_index(self, index: int, polyhedron: Optional[Polyhedron] = None,
                          search_radius: Optional[float] = None, target_group: Optional[int] = None,
                          precision="fp64") -> "Cell":
        """Diagram::get_cell_at_index (interface.rs:186-208)."""
        if not 0 <= index < self.n:
            raise IndexError(index)
        return Cell(self, index, None, polyhedron, search_radius, target_group, precision)

    def get_cell_at_particle(self, point, polyhedron: Optional[Polyhedron] = None,
                             search_radius: Optional[float] = None, target_group: Optional[int] = None,
                             precision="fp64") -> "Cell":
        """Diagram::get_cell_at_particle (interface.rs:211-232)."""
        return Cell(self, None, np.asarray(point, dtype=np.float64), polyhedron, search_radius,
                    target_group, precision)


class Cell:
    """A Voronoi cell (Cell, interface.rs:237-390)."""

    def __init__(self, diagram: Diagram, index, point, polyhedron, search_radius, target_group, precision):
        self.diagram = diagram
        self.index = index
        self.point = point
        self.polyhedron = polyhedron
        self.search_radius = search_radius
        self.target_group = target_group
        self.precision = precision
        self._g: Optional[CellGeometry] = None

    def compute_voronoi_cell(self) -> "Cell":
        """Cell::compute_voronoi_cell (interface.rs:257-313), on the GPU."""
        L = lib()
        g = CellGeometry()
        lo = hi = None
        if self.polyhedron is not None:
            lo = np.ascontiguousarray(self.polyhedron.lo)
            hi = np.ascontiguousarray(self.polyhedron.hi)
        lp = None if lo is None else _dp(lo)
        hp = None if hi is None else _dp(hi)
        if self.index is not None:
            st = L.tess_cell_compute(self.diagram._h, self.index, _prec(self.precision),
                                     _radius(self.search_radius), _group(self.target_group), lp, hp,
                                     C.byref(g))
        else:
            p = np.ascontiguousarray(self.point)
            st = L.tess_cell_compute_at(self.diagram._h, _dp(p), _prec(self.precision),
                                        _radius(self.search_radius), _group(self.target_group), lp, hp,
                                        C.byref(g))
        check(st)
        self._g = g
        return self

    def _geom(self) -> CellGeometry:
        if self._g is None:
            self.compute_voronoi_cell()
        return self._g

    def compute_volume(self) -> float:
        """Cell::compute_volume (interface.rs:337-339)."""
        return self._geom().volume

    def compute_neighbors(self) -> List[int]:
        """Cell::compute_neighbors (interface.rs:342-344); walls are negative ids."""
        g = self._geom()
        return [g.face_neighbor[f] for f in range(g.nfaces)]

    def compute_vertices(self) -> np.ndarray:
        """Cell::compute_vertices (interface.rs:368-370), site-relative."""
        g = self._geom()
        return np.ctypeslib.as_array(g.vertices)[: 3 * g.nvertices].reshape(-1, 3).copy()

    def compute_faces(self) -> List["VoronoiFace"]:
        """Cell::compute_faces (interface.rs:373-384)."""
        g = self._geom()
        return [VoronoiFace(self, f) for f in range(g.nfaces)]

    def original_index(self) -> Optional[int]:
        """Cell::original_index (interface.rs:387-389)."""
        return self.index

    def compute_neighbor_cloud(self, radius: float, target_group: Optional[int] = None) -> List[int]:
        """Cell::compute_neighbor_cloud (interface.rs:348-365): the points of the
        bins an expanding search from the cell's position reaches within
        `radius` (self included), optionally only target_group's."""
        if self.index is not None:
            return self.diagram.neighbor_cloud(radius, [self.index], target_group)[1].tolist()
        return self.diagram.neighbor_cloud_at([self.point], radius, target_group)[1].tolist()


class VoronoiFace:
    """A face of a Voronoi cell (VoronoiFace, interface.rs:393-416)."""

    def __init__(self, cell: Cell, face_index: int):
        self.cell = cell
        self.face_index = face_index

    def compute_vertices(self) -> np.ndarray:
        g = self.cell._geom()
        b, e = g.face_offset[self.face_index], g.face_offset[self.face_index + 1]
        verts = np.ctypeslib.as_array(g.vertices)[: 3 * g.nvertices].reshape(-1, 3)
        idx = [g.face_vertex[t] for t in range(b, e)]
        return verts[idx].copy()

    def compute_area(self) -> float:
        return self.cell._geom().face_area[self.face_index]

    def compute_neighbor(self) -> int:
        return self.cell._geom().face_neighbor[self.face_index]


class Batch:
    """Many independent diagrams computed in one CUDA-graph launch.

    ``points``: (total, 3) float64 concatenated; ``offsets``: ndiag+1 point
    offsets; ``boxes``: (ndiag, 6) {xlo, ylo, zlo, xhi, yhi, zhi}.
    """

    def __init__(self, points, offsets, boxes, config: Optional[Config] = None):
        L = lib()
        pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
        offs = np.ascontiguousarray(offsets, dtype=np.uint64)
        bx = np.ascontiguousarray(np.asarray(boxes, dtype=np.float64).reshape(-1, 6))
        self.n = len(pts)
        self.ndiag = len(offs) - 1
        self._h = C.c_void_p()
        cfg = config if config is not None else default_config()
        check(L.tess_batch_create(self.ndiag, offs.ctypes.data_as(C.POINTER(C.c_uint64)), _dp(pts), _dp(bx),
                                  C.byref(cfg), C.byref(self._h)))

    def compute(self, precision="fp32") -> "Batch":
        """Every cell of every diagram ("fp32", "mixed" or "fp64", as
        Diagram.compute_all), in one CUDA-graph launch per precision."""
        check(lib().tess_batch_compute(self._h, _prec(precision)))
        return self

    def compute_to_host(self, precision="fp32", face_pool=None) -> "HostResults":
        """compute with the faces written into a pinned host pool as the cells
        finish (tess_batch_compute_to_host); see Diagram.compute_all_to_host.
        Neighbour ids are local to each diagram."""
        def call(*a):
            return lib().tess_batch_compute_to_host(self._h, _prec(precision), *a)

        return _to_host(call, self.n, face_pool, 20 * self.n + 1024)

    def autotune(self, precision="fp32", cache_path: Optional[str] = None) -> dict:
        """As Diagram.autotune, with the batch's grid density among the knobs."""
        t = Tuning()
        cp = None if cache_path is None else cache_path.encode()
        check(lib().tess_batch_autotune(self._h, _prec(precision), cp, C.byref(t)))
        return t.as_dict()

    def update_points(self, points=None, device_ptr: Optional[int] = None):
        """Replace every diagram's points (same offsets and boxes); the next
        compute() bins them again."""
        if device_ptr is not None:
            check(lib().tess_batch_update_points(self._h, C.c_void_p(device_ptr), 1))
        else:
            pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, 3))
            if len(pts) != self.n:
                raise ValueError("update_points keeps the point count")
            check(lib().tess_batch_update_points(self._h, C.c_void_p(pts.ctypes.data), 0))

    def volumes(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float64)
        check(lib().tess_batch_volumes(self._h, _dp(out)))
        return out

    def neighbors_csr(self):
        L = lib()
        offs = np.empty(self.n + 1, dtype=np.uint64)
        total = C.c_size_t(0)
        check(L.tess_batch_neighbors_csr(self._h, offs.ctypes.data_as(C.POINTER(C.c_uint64)), None, None, 0,
                                         C.byref(total)))
        nbr = np.empty(max(total.value, 1), dtype=np.int32)
        area = np.empty(max(total.value, 1), dtype=np.float64)
        check(L.tess_batch_neighbors_csr(self._h, None, nbr.ctypes.data_as(C.POINTER(C.c_int32)), _dp(area),
                                         len(nbr), C.byref(total)))
        return offs, nbr[:total.value], area[:total.value]

    def results_device(self):
        """Device addresses (volumes, offsets, neighbour ids, areas, total faces)."""
        v, o, nb, a = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_void_p()
        total = C.c_size_t(0)
        check(lib().tess_batch_results_device(self._h, C.byref(v), C.byref(o), C.byref(nb), C.byref(a),
                                              C.byref(total)))
        return v.value, o.value, nb.value, a.value, total.value

    def stats(self) -> dict:
        s = Stats()
        check(lib().tess_batch_stats(self._h, C.byref(s)))
        return s.as_dict()

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().tess_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
