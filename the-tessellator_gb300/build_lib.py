"""Builds libtessgpu.so (the CUDA library behind include/tessellator.h) in-tree.

nvcc compiles each translation unit for sm_103a only, in parallel, then links
a shared library with the CUDA runtime linked statically (the library loads
on machines without a GPU; every compute call then reports TESS_E_CUDA).

build(checked=True) makes libtessgpu_checked.so instead: the same sources with
TESS_CHECKED=1, whose kernels test every data-dependent device index and whose
calls fail with TESS_E_CHECK when one was out of range.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "tessellator", "libtessgpu.so")
OUT_CHECKED = os.path.join(HERE, "tessellator", "libtessgpu_checked.so")
BUILD = os.path.join(ROOT, "_build", "tessgpu")
SOURCES = ["tess_grid.cu", "tess_clip.cu", "tess_clip_f32.cu", "tess_clip_f32x.cu", "tess_clip_f64.cu", "tess_api.cu",
           "tess_noalloc.cu", "tess_radius.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _inputs():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "tessellator.h"))
    return files


def up_to_date(out: str = OUT) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> str:
    out = OUT_CHECKED if checked else OUT
    if not force and up_to_date(out):
        return out
    build_dir = BUILD + ("_checked" if checked else "")
    os.makedirs(build_dir, exist_ok=True)
    nvcc = _nvcc()
    # Host code keeps IEEE operation order (no FMA contraction on any host ISA):
    # the radius table's keys must match the FP64 key formula bit for bit.
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I", os.path.join(ROOT, "include"), "-I", CSRC] + (["-DTESS_CHECKED=1"] if checked else [])

    def compile_one(src):
        obj = os.path.join(build_dir, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = out + ".tmp"
    cmd = [nvcc, "-shared"] + ARCH + ["-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv))
