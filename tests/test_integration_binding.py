"""The reference-side binding compiles against the reference's own headers and
include/blink_imager_gb300.h (g++ -fsyntax-only, with the host-only stand-ins of oracle/ref_shim
for the astroio types; skipped where the reference checkout or g++ is absent):
- tests/cpp/reference_binding.cpp, the C++ a maintainer puts in the reference's src/gpu/ in place
  of gridding_gpu.cpp, corrections_gpu.cpp and gpu_utils.cpp (the integration guide prints the
  same code): the signatures it defines are the reference's (src/gpu/gridding_gpu.h:12-18,
  src/gpu/corrections_gpu.h:7-9, src/gpu/gpu_utils.h:8-19) and the calls it makes are the ABI's;
- tests/cpp/reference_imager_class.cpp, the counterpart of CPacerImagerHip: a CPacerImager
  (src/pacer_imager.h) with the same constructor and virtuals, each a call of the ABI."""
import os
import re
import shutil
import subprocess

import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpp", "reference_binding.cpp")
CLASS_SRC = os.path.join(HERE, "cpp", "reference_imager_class.cpp")


def _cuda_include() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.isfile(os.path.join(inc, "cuda_runtime.h")) else ""


def test_reference_binding_compiles():
    gpu_dir = os.path.join(O.REF_SRC, "gpu") if O.REF_SRC else ""
    if not gpu_dir or not os.path.isfile(os.path.join(gpu_dir, "gridding_gpu.h")):
        pytest.skip("no reference checkout (BGI_REFERENCE_SRC)")
    if not shutil.which("g++"):
        pytest.skip("no g++")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I",
           gpu_dir, "-I", os.path.join(ROOT, "include"), SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    # every function of the reference's three src/gpu headers that carries GPU work is defined
    src = open(SRC).read()
    for name in ("apply_geometric_corrections_gpu", "apply_cable_lengths_corrections_gpu", "gridding_gpu",
                 "vector_sum_gpu", "fft_shift_and_norm_gpu", "image_averaging_gpu"):
        assert re.search(rf"\b{name}\s*\(", src), name


def test_reference_imager_class_compiles():
    gpu_dir = os.path.join(O.REF_SRC, "gpu") if O.REF_SRC else ""
    if not gpu_dir or not os.path.isfile(os.path.join(O.REF_SRC, "pacer_imager.h")):
        pytest.skip("no reference checkout (BGI_REFERENCE_SRC)")
    if not shutil.which("g++"):
        pytest.skip("no g++")
    cuda_inc = _cuda_include()
    if not cuda_inc:
        pytest.skip("no CUDA runtime header")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I",
           gpu_dir, "-I", O.REF_SRC, "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, CLASS_SRC]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    src = open(CLASS_SRC).read()
    # the virtuals CPacerImager::grid() and run() call (src/pacer_imager.h:124-141) are overridden
    for name in ("gridding", "image", "ApplyGeometricCorrections", "ApplyCableCorrections"):
        assert re.search(rf"\b{name}\([^)]*\)\s*override", src), name
