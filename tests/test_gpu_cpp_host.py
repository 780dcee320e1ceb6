"""The C ABI from C++: tests/cpp/capi_host_test.cpp (an imager handle on device and host
buffers, deterministic repeatability, the reference's free-function call order, the serving
runtime) compiled with g++ against include/ and the library, and run."""
import os
import shutil
import subprocess

import pytest

from imager_gb300 import capi

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def test_cpp_host_program(tmp_path):
    lib = capi.library_path()
    capi.lib(build_if_missing=True)
    cuda = _cuda_home()
    exe = str(tmp_path / "capi_host_test")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(cuda, "include"), os.path.join(HERE, "cpp", "capi_host_test.cpp"), "-o", exe,
           lib, "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.dirname(lib)}",
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "C++ host checks passed" in r.stdout
