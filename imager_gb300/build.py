"""Build the CUDA library of the imaging path for sm_103a (GB300), in tree.

    python -m imager_gb300.build          # -> imager_gb300/_lib/libblink_imager_gb300.so

Each .cu file under csrc/ compiles to an object in parallel, then one shared library is
linked with the CUDA runtime statically.  No CMake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
BUILD_DIR = os.path.join(PKG, "_build")
LIB_NAME = "libblink_imager_gb300.so"
LIB_PATH = os.path.join(OUT_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def extra_flags():
    """Extra nvcc flags from BGI_EXTRA_NVCC_FLAGS (space-separated), e.g. -DC2R_THREADS=256;
    objects built with other flags are rebuilt."""
    return os.environ.get("BGI_EXTRA_NVCC_FLAGS", "").split()


def _flags_changed() -> bool:
    stamp = os.path.join(BUILD_DIR, "flags.txt")
    want = " ".join(NVCC_FLAGS + extra_flags())
    have = open(stamp).read() if os.path.exists(stamp) else None
    if have != want:
        with open(stamp, "w") as f:
            f.write(want)
        return True
    return False


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "blink_imager_gb300.h"))
    objs, jobs = [], []
    rebuild = _flags_changed()
    for src in sources():
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if rebuild or _stale(obj, [src] + headers) or ptxas_info:
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra_flags(), "-c", src, "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_info or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if jobs or _stale(LIB_PATH, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB_PATH, *objs, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
