"""The C++ layer (include/schro_gpu/schro_gpu.hpp) and the reference-style
C++ test program built on it (tests/cpp/test_schro_gpu.cpp)."""
import os
import shutil
import subprocess

import pytest

from tests.util import ROOT, SMALL_MESH


def _compile(out, syntax_only=False):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    cuda_inc = "/usr/local/cuda/include"
    cmd = [gxx, "-std=c++20", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), "-I" + cuda_inc,
           os.path.join(ROOT, "tests", "cpp", "test_schro_gpu.cpp")]
    if syntax_only:
        cmd += ["-fsyntax-only"]
    else:
        import schrodingersem_gb300 as S
        lib = S.build()
        libdir = os.path.dirname(lib)
        cmd += ["-L" + libdir, "-lsemgb300", "-L/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath," + libdir,
                "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_layer_compiles():
    _compile(None, syntax_only=True)


@pytest.mark.gpu
def test_reference_test_suite_through_cpp_layer(tmp_path):
    exe = str(tmp_path / "test_schro_gpu")
    _compile(exe)
    r = subprocess.run([exe, SMALL_MESH], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all tests passed!" in r.stdout
