"""C ABI library on the host: it builds, loads, exports every symbol the public header
declares, and rejects bad arguments before touching the GPU."""
import ctypes as C
import shutil

import pytest

from imager_gb300 import capi


@pytest.fixture(scope="module")
def lib():
    if shutil.which("nvcc") is None and not __import__("os").path.exists(capi.library_path()):
        pytest.skip("nvcc not available to build the library")
    return capi.lib(build_if_missing=True)


def test_exports_every_header_symbol(lib):
    names = capi.header_functions()
    assert len(names) >= 17
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(capi._SIGNATURES), "ctypes signatures out of date with the header"


def test_version(lib):
    assert lib.bgi_version() == 1


def test_host_side_argument_checks(lib):
    # odd x side is rejected as in src/gpu/gpu_utils.cpp:129-131
    assert lib.bgi_fft_shift_and_norm_gpu(C.c_void_p(16), 3, 2, 1, C.c_void_p(16), 1, None) == capi.ERR_INVALID
    assert b"even" in lib.bgi_last_error()
    # unsupported FFT sizes: every side 1..4096 is taken (powers of two and mixed radix)
    for side in (0, 4097, 5000):
        assert lib.bgi_fft_inverse_gpu(C.c_void_p(16), C.c_void_p(32), side, 1, None) == capi.ERR_UNSUPPORTED
    # uniform weighting: null and misaligned buffers
    assert lib.bgi_uniform_weighting_gpu(None, C.c_void_p(16), 32, 1, None) == capi.ERR_INVALID
    assert lib.bgi_uniform_weighting_gpu(C.c_void_p(12), C.c_void_p(16), 32, 1, None) == capi.ERR_INVALID
    # in-place FFT is refused
    assert lib.bgi_fft_inverse_gpu(C.c_void_p(16), C.c_void_p(16), 64, 1, None) == capi.ERR_INVALID
    # null buffers
    assert lib.bgi_gridding_gpu(None, 4, 1, 1, None, None, 1, None, None, None, 1.0, 1.0, 64, -1.0, 0,
                                1, None, None, None) == capi.ERR_INVALID
    assert lib.bgi_vector_sum_gpu(None, 10, 1, None, None) == capi.ERR_INVALID
    # misaligned visibilities
    assert lib.bgi_apply_cable_lengths_corrections_gpu(C.c_void_p(8), 4, 1, 1, C.c_void_p(16),
                                                      C.c_void_p(16), None) == capi.ERR_INVALID
    # bad pol
    assert lib.bgi_gridding_gpu(C.c_void_p(16), 4, 1, 1, C.c_void_p(16), C.c_void_p(16), 1, C.c_void_p(16),
                                None, C.c_void_p(16), 1.0, 1.0, 64, -1.0, 7, 1, None,
                                C.c_void_p(16), None) == capi.ERR_INVALID


def test_create_rejects_bad_config(lib):
    h = C.c_void_p()
    for cfg in (capi.Config(5000, 2.0, 0, -1.0, 0, 0), capi.Config(0, 2.0, 0, -1.0, 0, 0),
                capi.Config(512, 0.0, 0, -1.0, 0, 0),
                capi.Config(512, 2.0, 9, -1.0, 0, 0), capi.Config(512, 2.0, 0, -1.0, -3, 0)):
        st = lib.bgi_create(C.byref(cfg), C.byref(h))
        assert st in (capi.ERR_UNSUPPORTED, capi.ERR_INVALID), (cfg.n_pixels, st)
        assert not h.value
    assert lib.bgi_create(None, C.byref(h)) == capi.ERR_INVALID
    # null handle calls
    assert lib.bgi_image(None, C.c_void_p(16), 1, 0, C.c_void_p(16), None) == capi.ERR_INVALID
    assert lib.bgi_image_compressed(None, 1, C.c_void_p(16), C.c_void_p(16), 1, 0, C.c_void_p(16),
                                    None) == capi.ERR_INVALID
    assert lib.bgi_replay_ready(None) == capi.ERR_INVALID
    assert lib.bgi_set_replay(None, 1) == capi.ERR_INVALID
    assert lib.bgi_set_gridding_aggregation(None, 1) == capi.ERR_INVALID
    assert lib.bgi_get_gridding_aggregation(None, None) == capi.ERR_INVALID
    assert lib.bgi_destroy(None) == capi.OK


def test_sorted_workspace_size(lib):
    n = C.c_size_t(0)
    assert lib.bgi_gridding_sorted_workspace(256, 512, 1, C.byref(n)) == capi.OK
    one = n.value
    nb = 256 * 257 // 2
    # per image: key, value and segment entry per point (2 per baseline), 3 counts per cell
    assert one >= 2 * nb * 16 + 3 * 512 * 512 * 4
    assert lib.bgi_gridding_sorted_workspace(256, 512, 10, C.byref(n)) == capi.OK
    assert n.value == 10 * one
    assert lib.bgi_gridding_sorted_workspace(0, 512, 1, C.byref(n)) == capi.ERR_INVALID
    assert lib.bgi_gridding_sorted_workspace(256, 512, 1, None) == capi.ERR_INVALID
    # a workspace that is not 16-byte aligned is refused before any launch
    assert lib.bgi_gridding_sorted_gpu(C.c_void_p(16), 4, 1, 1, C.c_void_p(16), C.c_void_p(16), 1,
                                       C.c_void_p(16), C.c_void_p(16), 1.0, 1.0, 64, -1.0, 0, 1, None,
                                       C.c_void_p(16), C.c_void_p(24), 1 << 20, None) == capi.ERR_INVALID


def test_uvw_step_from_angles(lib):
    """The timestep helper fills the 17 numbers the pointed-UVW routines take (no GPU needed)."""
    import os
    import numpy as np
    from imager_gb300 import imager
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pointed_uvw.npz"))
    steps = imager.uvw_steps(g["rmat"], g["ha2000"], g["dec_aber"], g["lmst"], g["lmst2000"])
    np.testing.assert_allclose(steps, g["steps"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("lang,std", [("c", "c99"), ("c++", "c++11")])
def test_header_compiles_alone(lang, std):
    """The public header is plain C: it compiles on its own as C99 (pedantic) and as C++11, with
    every warning on and none raised, so C, C++ and FFI binding generators can take it as is."""
    import os
    import subprocess
    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no compiler")
    hdr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                       "blink_imager_gb300.h")
    flags = ["-Wall", "-Wextra", "-Werror"] + (["-pedantic"] if lang == "c" else [])
    r = subprocess.run([cc, f"-std={std}", *flags, "-fsyntax-only", "-x", lang, hdr], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
