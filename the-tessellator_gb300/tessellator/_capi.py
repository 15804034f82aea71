"""ctypes declarations of include/tessellator.h (libtessgpu.so).

The shared library is built in-tree by ``build_lib.py``.  Loading fails
loudly when it is missing: there is no CPU implementation behind this API.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# $TESS_LIB selects another build of the library, e.g. libtessgpu_checked.so
# (every device index bounds-checked; calls that met a bad one fail with
# TESS_E_CHECK).
LIB_PATH = os.environ.get("TESS_LIB") or os.path.join(HERE, "libtessgpu.so")

TESS_OK, TESS_E_INVALID, TESS_E_CUDA, TESS_E_CAPACITY = 0, 1, 2, 3
TESS_E_OVERFLOW, TESS_E_STATE, TESS_E_NOMEM, TESS_E_LIMIT, TESS_E_CHECK = 4, 5, 6, 7, 8
STATUS_NAMES = {0: "TESS_OK", 1: "TESS_E_INVALID", 2: "TESS_E_CUDA", 3: "TESS_E_CAPACITY",
                4: "TESS_E_OVERFLOW", 5: "TESS_E_STATE", 6: "TESS_E_NOMEM", 7: "TESS_E_LIMIT",
                8: "TESS_E_CHECK"}
PRECISION_FP64, PRECISION_FP32_GUARD, PRECISION_MIXED = 0, 1, 2
FLAG_TIMING = 1
FLAG_COUNTERS = 2
FLAG_SMALL_FACE_POOL = 4
FLAG_NO_CAPACITY_RERUN = 8
FLAG_AUTOTUNE = 16
MAX_CELL_VERTICES, MAX_CELL_FACES = 255, 254

# Every function the header declares, in header order.
EXPORTS = (
    "tess_config_default", "tess_last_error", "tess_version",
    "tess_diagram_create", "tess_diagram_create_device", "tess_diagram_rebuild",
    "tess_diagram_update_points", "tess_diagram_celery",
    "tess_diagram_destroy", "tess_diagram_compute_all", "tess_diagram_stats", "tess_diagram_grid",
    "tess_cell_volume", "tess_cell_neighbors", "tess_cell_faces", "tess_cell_vertices",
    "tess_cell_face_vertices", "tess_cell_original_index", "tess_cell_compute",
    "tess_cell_compute_at", "tess_volumes", "tess_neighbors_csr", "tess_results_device",
    "tess_diagram_compute_all_to_host", "tess_host_alloc", "tess_host_free",
    "tess_find_cells_in_radius", "tess_find_neighbors_in_radius", "tess_neighbor_cloud",
    "tess_neighbor_cloud_at",
    "tess_batch_create", "tess_batch_compute", "tess_batch_compute_to_host", "tess_batch_update_points", "tess_batch_stats", "tess_batch_volumes",
    "tess_batch_neighbors_csr", "tess_batch_results_device", "tess_batch_destroy",
    "tess_diagram_autotune", "tess_batch_autotune", "tess_csr_offsets_noalloc",
)


class Config(C.Structure):
    _fields_ = [("guard_rel", C.c_double), ("verify_rel", C.c_double), ("bin_density", C.c_double),
                ("table_gaps", C.c_int32), ("warps_per_block", C.c_int32),
                ("slots_per_lane", C.c_int32), ("device", C.c_int32), ("stream", C.c_void_p),
                ("flags", C.c_uint32), ("crowded_bin", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("cells", C.c_uint64), ("faces", C.c_uint64), ("rerun_fp64", C.c_uint64),
                ("rerun_capacity", C.c_uint64), ("failed", C.c_uint64),
                ("table_entries", C.c_uint64), ("ms_grid", C.c_double), ("ms_clip", C.c_double),
                ("ms_rerun", C.c_double), ("ms_csr", C.c_double), ("launches", C.c_uint64),
                ("rerun_guard", C.c_uint64), ("rerun_verify", C.c_uint64), ("rerun_degenerate", C.c_uint64),
                ("candidates_tested", C.c_uint64), ("cuts", C.c_uint64), ("new_vertices", C.c_uint64),
                ("windows", C.c_uint64), ("batches", C.c_uint64), ("ms_query_count", C.c_double),
                ("ms_query_fill", C.c_double), ("rerun_fp64_full", C.c_uint64),
                ("dense_cells", C.c_uint64), ("face_pool_regrows", C.c_uint64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("warps_per_block", C.c_int32), ("crowded_bin", C.c_int32), ("bin_density", C.c_double),
                ("ms_chosen", C.c_double), ("ms_default", C.c_double), ("sample_cells", C.c_uint64),
                ("trials", C.c_int32), ("from_cache", C.c_int32), ("max_bin_points", C.c_uint32),
                ("crowded_fraction", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class CellGeometry(C.Structure):
    _fields_ = [("volume", C.c_double), ("nvertices", C.c_int32), ("nfaces", C.c_int32),
                ("vertices", C.c_double * 768), ("face_neighbor", C.c_int32 * 256),
                ("face_area", C.c_double * 256), ("face_offset", C.c_int32 * 257),
                ("face_vertex", C.c_int32 * 768)]


class TessError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


_lib = None


def lib():
    """Load libtessgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with build_lib.py (nvcc, sm_103a)")
    L = C.CDLL(LIB_PATH)
    dp, u32p, u64p, i32p = C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_int32)
    vp, szp = C.c_void_p, C.POINTER(C.c_size_t)
    st = C.c_int
    sig = {
        "tess_config_default": (None, [C.POINTER(Config)]),
        "tess_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
        "tess_version": (C.c_char_p, []),
        "tess_diagram_create": (st, [dp, C.c_size_t, u32p, dp, dp, C.POINTER(Config), C.POINTER(vp)]),
        "tess_diagram_create_device": (st, [vp, C.c_size_t, u32p, dp, dp, C.POINTER(Config), C.POINTER(vp)]),
        "tess_diagram_rebuild": (st, [vp]),
        "tess_diagram_update_points": (st, [vp, vp, C.c_int]),
        "tess_diagram_celery": (st, [vp, u32p, u32p, u32p]),
        "tess_diagram_destroy": (st, [vp]),
        "tess_diagram_compute_all": (st, [vp, C.c_int, C.c_double, C.c_int64]),
        "tess_diagram_stats": (st, [vp, C.POINTER(Stats)]),
        "tess_diagram_grid": (st, [vp, C.POINTER(C.c_int64), dp]),
        "tess_cell_volume": (st, [vp, C.c_size_t, dp]),
        "tess_cell_neighbors": (st, [vp, C.c_size_t, i32p, C.c_size_t, szp]),
        "tess_cell_faces": (st, [vp, C.c_size_t, i32p, dp, C.c_size_t, szp]),
        "tess_cell_vertices": (st, [vp, C.c_size_t, dp, C.c_size_t, szp]),
        "tess_cell_face_vertices": (st, [vp, C.c_size_t, C.c_size_t, dp, C.c_size_t, szp]),
        "tess_cell_original_index": (st, [vp, C.c_size_t, szp]),
        "tess_cell_compute": (st, [vp, C.c_size_t, C.c_int, C.c_double, C.c_int64, dp, dp,
                                   C.POINTER(CellGeometry)]),
        "tess_cell_compute_at": (st, [vp, dp, C.c_int, C.c_double, C.c_int64, dp, dp,
                                      C.POINTER(CellGeometry)]),
        "tess_volumes": (st, [vp, dp]),
        "tess_neighbors_csr": (st, [vp, u64p, i32p, dp, C.c_size_t, szp]),
        "tess_results_device": (st, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), szp]),
        "tess_diagram_compute_all_to_host": (st, [vp, C.c_int, C.c_double, C.c_int64, vp, vp, vp, vp, vp,
                                                  C.c_size_t, szp]),
        "tess_host_alloc": (st, [C.c_size_t, C.POINTER(vp)]),
        "tess_host_free": (st, [vp]),
        "tess_find_cells_in_radius": (st, [vp, vp, C.c_size_t, C.c_double, C.c_int, vp, vp, C.c_size_t, szp]),
        "tess_find_neighbors_in_radius": (st, [vp, vp, C.c_size_t, C.c_double, C.c_int, C.c_int, vp, vp,
                                               C.c_size_t, szp]),
        "tess_neighbor_cloud": (st, [vp, vp, C.c_size_t, C.c_double, C.c_int64, C.c_int, vp, vp, C.c_size_t,
                                     szp]),
        "tess_neighbor_cloud_at": (st, [vp, vp, C.c_size_t, C.c_double, C.c_int64, C.c_int, vp, vp,
                                        C.c_size_t, szp]),
        "tess_batch_create": (st, [C.c_size_t, u64p, dp, dp, C.POINTER(Config), C.POINTER(vp)]),
        "tess_batch_compute": (st, [vp, C.c_int]),
        "tess_batch_compute_to_host": (st, [vp, C.c_int, vp, vp, vp, vp, vp, C.c_size_t, szp]),
        "tess_batch_update_points": (st, [vp, vp, C.c_int]),
        "tess_batch_stats": (st, [vp, C.POINTER(Stats)]),
        "tess_batch_volumes": (st, [vp, dp]),
        "tess_batch_neighbors_csr": (st, [vp, u64p, i32p, dp, C.c_size_t, szp]),
        "tess_batch_results_device": (st, [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), C.POINTER(vp), szp]),
        "tess_batch_destroy": (st, [vp]),
        "tess_diagram_autotune": (st, [vp, C.c_int, C.c_char_p, C.POINTER(Tuning)]),
        "tess_batch_autotune": (st, [vp, C.c_int, C.c_char_p, C.POINTER(Tuning)]),
        "tess_csr_offsets_noalloc": (st, [vp, C.c_size_t, vp, vp]),
    }
    for name in EXPORTS:
        fn = getattr(L, name)
        fn.restype, fn.argtypes = sig[name]
    _lib = L
    return L


def last_error() -> str:
    L = lib()
    n = L.tess_last_error(None, 0)
    buf = C.create_string_buffer(n + 1)
    L.tess_last_error(buf, n + 1)
    return buf.value.decode(errors="replace")


def check(status: int):
    if status != TESS_OK:
        raise TessError(status, last_error())


def default_config(**overrides) -> Config:
    c = Config()
    lib().tess_config_default(C.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c
