"""The C ABI from C and C++ (tests/c/abi_demo.c): the header compiles as C11 and
as C++17, the program links against the library and runs.  Without a GPU it
must see TESS_E_CUDA from create (no CPU fallback); on the GPU it computes a
jittered lattice in the three precisions and checks the volume sum, the CSR
and one cell's queries against the bulk results."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _build(tmp_path, lang):
    import build_lib

    lib = build_lib.build()
    libdir = os.path.dirname(lib)
    src = os.path.join(HERE, "c", "abi_demo.c")
    out = str(tmp_path / f"abi_demo_{lang}")
    if lang == "c":
        cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-x", "c", src]
    else:
        cmd = ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-x", "c++", src]
    cmd += ["-I", os.path.join(ROOT, "include"), "-L", libdir, "-ltessgpu", f"-Wl,-rpath,{libdir}", "-lm", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _run(exe):
    return subprocess.run([exe], capture_output=True, text=True, timeout=600)


@pytest.mark.parametrize("lang", ["c", "cxx"])
def test_c_abi_builds_and_fails_loudly_without_a_gpu(tmp_path, lang):
    if shutil.which("gcc" if lang == "c" else "g++") is None:
        pytest.skip("no host compiler")
    torch = pytest.importorskip("torch")
    exe = _build(tmp_path, lang)
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the GPU test runs the program)")
    r = _run(exe)
    assert r.returncode == 2, r.stdout + r.stderr
    assert "TESS_E_CUDA" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("lang", ["c", "cxx"])
def test_c_abi_on_the_gpu(tmp_path, lang):
    exe = _build(tmp_path, lang)
    r = _run(exe)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
