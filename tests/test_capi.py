"""The C ABI library without a GPU: it loads, exports every function that
include/tessellator.h declares, and rejects bad arguments with an error
status (no compute calls are made here)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "tessellator.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tess_[a-z_0-9]+)\s*\(", text)))


def exported_symbols(path):
    import subprocess

    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_every_declared_function_is_exported(tess):
    decl = declared_functions()
    assert len(decl) >= 25
    syms = exported_symbols(tess._capi.LIB_PATH)
    missing = [f for f in decl if f not in syms]
    assert not missing, missing
    # the Python binding declares the same set
    assert sorted(tess._capi.EXPORTS) == decl


RUST_FFI = os.path.join(ROOT, "rust", "src", "gpu_ffi.rs")
RUST_API = os.path.join(ROOT, "rust", "src", "interface.rs")


def test_rust_binding_declares_every_function():
    """The crate's extern block (rust/src/gpu_ffi.rs) names every function of
    the header, and no other."""
    text = open(RUST_FFI).read()
    rust = sorted(set(re.findall(r"\bpub fn (tess_[a-z_0-9]+)\s*\(", text)))
    assert rust == declared_functions()


def test_rust_constants_match_the_header():
    """Status codes and precisions in the crate equal the header's enums."""
    header = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "tessellator.h")).read(), flags=re.S)
    cvals = dict(re.findall(r"\b(TESS_(?:OK|E_[A-Z]+|PRECISION_[A-Z0-9_]+))\s*=\s*(\d+)", header))
    rvals = dict(re.findall(r"pub const (TESS_(?:OK|E_[A-Z]+|PRECISION_[A-Z0-9_]+)):[^=]*=\s*(\d+)",
                            open(RUST_FFI).read()))
    assert len(cvals) >= 11
    assert rvals == cvals


def test_rust_wrapper_keeps_the_reference_names():
    """The safe wrapper (rust/src/interface.rs) has the public methods of the
    reference's interface.rs and calls only functions the binding declares."""
    text = open(RUST_API).read()
    for name in ("get_cell_at_index", "get_cell_at_particle", "compute_voronoi_cell", "compute_volume",
                 "compute_neighbors", "compute_neighbor_cloud", "compute_vertices", "compute_faces",
                 "original_index", "compute_area", "compute_neighbor", "compute_all", "volumes",
                 "neighbors_csr", "find_neighbors_in_real_radius", "find_cells_in_radius"):
        assert re.search(r"pub fn " + name + r"\b", text), name
    called = set(re.findall(r"\b(tess_[a-z_0-9]+)\s*\(", text))
    assert called and called <= set(declared_functions())
    for f in ("Cargo.toml", "build.rs", os.path.join("src", "lib.rs")):
        assert os.path.exists(os.path.join(ROOT, "rust", f)), f


def test_library_needs_no_gpu_to_load(tess):
    L = tess.lib()
    assert L.tess_version().startswith(b"tessellator-gb300")


def test_default_config(tess):
    c = tess.default_config()
    assert c.bin_density == 1.25          # celery.rs:185-188
    assert c.slots_per_lane == 2 and c.table_gaps == 8
    assert c.guard_rel == 4e-7            # the FP32 test's rounding bound, 3e-7, with a third in hand
    assert c.stream is None and c.flags == 0


@pytest.mark.parametrize("field,value", [("guard_rel", 1e-7), ("guard_rel", 0.0), ("guard_rel", float("nan")),
                                         ("verify_rel", 0.0), ("bin_density", -1.0), ("slots_per_lane", 3)])
def test_config_rejected(tess, field, value):
    """Settings that would void the FP32 form's guarantees (or make no sense)
    are refused before any device work."""
    L = tess.lib()
    c = tess.default_config()
    setattr(c, field, value)
    pts = np.random.default_rng(1).random((10, 3))
    h = C.c_void_p()
    st = L.tess_diagram_create(pts.ctypes.data_as(C.POINTER(C.c_double)), 10, None, None, None, C.byref(c),
                               C.byref(h))
    assert st == tess._capi.TESS_E_INVALID
    assert field in tess.last_error()


def test_argument_errors(tess):
    L = tess.lib()
    h = C.c_void_p()
    st = L.tess_diagram_create(None, 10, None, None, None, None, C.byref(h))
    assert st == tess._capi.TESS_E_INVALID
    assert "xyz" in tess.last_error()
    pts = np.zeros((4, 3))
    lo = np.array([1.0, 0, 0])
    hi = np.array([0.0, 1, 1])
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    st = L.tess_diagram_create(dp(pts), 0, None, None, None, None, C.byref(h))
    assert st == tess._capi.TESS_E_INVALID
    st = L.tess_diagram_create(dp(pts), 4, None, dp(lo), None, None, C.byref(h))
    assert st == tess._capi.TESS_E_INVALID
    assert L.tess_cell_volume(None, 0, None) == tess._capi.TESS_E_INVALID
    assert L.tess_diagram_compute_all(None, 0, -1.0, -1) == tess._capi.TESS_E_INVALID
    offs = np.array([0, 5, 5], dtype=np.uint64)
    st = L.tess_batch_create(2, offs.ctypes.data_as(C.POINTER(C.c_uint64)), dp(np.zeros((5, 3))),
                             dp(np.zeros((2, 6))), None, C.byref(h))
    assert st == tess._capi.TESS_E_INVALID   # second diagram empty
    bad = tess.default_config(slots_per_lane=3)
    with pytest.raises(tess.TessError) as e:
        tess.Diagram(np.random.rand(10, 3), config=bad)
    assert e.value.status in (tess._capi.TESS_E_INVALID, tess._capi.TESS_E_CUDA)


def test_fails_loudly_without_a_device(tess):
    """No CPU fallback: without a CUDA device the constructor reports TESS_E_CUDA."""
    pytest.importorskip("torch")
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(tess.TessError) as e:
        tess.Diagram(np.random.rand(10, 3))
    assert e.value.status == tess._capi.TESS_E_CUDA


def test_python_api_mirrors_interface_rs(tess):
    """The reference's public method names exist on the mirror classes."""
    for name in ("get_cell_at_index", "get_cell_at_particle"):
        assert hasattr(tess.Diagram, name)
    for name in ("compute_voronoi_cell", "compute_volume", "compute_neighbors", "compute_vertices",
                 "compute_faces", "original_index"):
        assert hasattr(tess.Cell, name)
    for name in ("compute_vertices", "compute_area", "compute_neighbor"):
        assert hasattr(tess.VoronoiFace, name)
    assert hasattr(tess.Polyhedron, "new")


def c_struct_fields(name):
    """Field names, in order, of `typedef struct {...} name;` in the header."""
    text = open(os.path.join(ROOT, "include", "tessellator.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = re.search(r"typedef struct \{([^}]*)\}\s*" + name + r"\s*;", text, flags=re.S).group(1)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        if decl:
            names.append(re.sub(r"\[.*?\]", "", decl).split()[-1].lstrip("*"))
    return names


@pytest.mark.parametrize("cname,pyname", [("tess_stats", "Stats"), ("tess_config", "Config"),
                                           ("tess_tuning", "Tuning")])
def test_struct_layouts_agree(tess, cname, pyname):
    """tess_stats and tess_config: the same fields in the same order in the
    header, the Python mirror and the Rust binding."""
    fields = c_struct_fields(cname)
    assert [f for f, _ in getattr(tess._capi, pyname)._fields_] == fields
    text = open(RUST_FFI).read()
    body = re.search(r"pub struct " + cname + r" \{(.*?)\}", text, flags=re.S).group(1)
    assert re.findall(r"pub (\w+):", body) == fields



def test_checked_build_loads_and_matches_the_exports():
    """The bounds-checked build (TESS_CHECKED=1) exports the same functions as
    the library, loads without a GPU and fails loudly there like it."""
    import ctypes

    import build_lib

    lib = build_lib.build(checked=True)
    syms = exported_symbols(lib)
    missing = [f for f in declared_functions() if f not in syms]
    assert not missing, missing
    assert {x for x in syms if x.startswith("tess_")} == \
        {x for x in exported_symbols(build_lib.build()) if x.startswith("tess_")}
    chk = ctypes.CDLL(lib)
    cfg = (ctypes.c_char * 4096)()
    chk.tess_config_default(cfg)
    pytest.importorskip("torch")
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    pts = (ctypes.c_double * 30)(*([0.1] * 30))
    h = ctypes.c_void_p()
    st = chk.tess_diagram_create(pts, ctypes.c_size_t(10), None, None, None, cfg, ctypes.byref(h))
    assert st == 2   # TESS_E_CUDA
