"""ctypes wrapper of the CPU oracle (oracle/blink_oracle.c) -- test infrastructure only.

The oracle restates the reference imager's CPU path (PaCER-BLINK-Project/imager,
src/pacer_imager.cpp, src/corrections.cpp) in C.  Only tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this module, and only as the checker.

``ref_library()`` loads the reference's own CPU sources compiled here against the stand-ins in
``oracle/ref_shim`` (``make -C oracle ref``), when that build exists.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libblink_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libpacer_ref.so")
# The reference checkout's src/ (only for compiling the reference's CPU sources): the
# BGI_REFERENCE_SRC environment variable, else a checkout named "reference" beside this
# repository; empty when neither exists.
def _find_ref_src() -> str:
    env = os.environ.get("BGI_REFERENCE_SRC", "")
    if env:
        return env
    sibling = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference", "src")
    return sibling if os.path.isfile(os.path.join(sibling, "pacer_imager.cpp")) else ""


REF_SRC = _find_ref_src()

POL = {"XX": 0, "YY": 1, "I": 2, "V": 3}

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
VIS_FORMAT = {"c64": 0, "s16": 1, "bf16": 2, "fp16": 3}

_lib = None
_ref = None


def build(ref: bool = False) -> None:
    """Compile the oracle (and, when the reference checkout exists and ref is set, the
    reference CPU build)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref and REF_SRC and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={REF_SRC}"], check=True)


def library():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        lib = C.CDLL(LIB_PATH)
        i64, i32, dbl, flt = C.c_int64, C.c_int, C.c_double, C.c_float
        sig = {
            "bgo_update_flags": (None, [i32, _i32p, i32, _i32p]),
            "bgo_zenith_uvw": (None, [i32, _f64p, _f64p, _f64p, _f32p, _f32p, _f32p]),
            "bgo_uv_max": (None, [i32, _f32p, _f32p, _i32p, C.POINTER(dbl), C.POINTER(dbl)]),
            "bgo_delta_uv": (dbl, [flt, dbl, i32]),
            "bgo_channel_frequency_hz": (dbl, [dbl, i32, dbl, i32, i32, i32]),
            "bgo_apply_geometric": (None, [_f32p, i32, i32, i32, _f32p, i32, _f64p]),
            "bgo_apply_cable": (None, [_f32p, i32, i32, i32, _f64p, _f64p]),
            "bgo_cell_index": (i64, [flt, flt, dbl, dbl, dbl, dbl, i32, i32]),
            "bgo_gridding": (i64, [_f32p, i32, i32, i32, _f32p, _f32p, i32, _i32p, _f64p, dbl,
                                   dbl, i32, dbl, i32, i32, _f32p, _f32p]),
            "bgo_fft2_inverse_f64": (None, [_f64p, _f64p, i32, i32]),
            "bgo_fft2_inverse_f32": (None, [_f32p, _f32p, i32, i32]),
            "bgo_fft2_inverse_f32_scalar": (None, [_f32p, _f32p, i32, i32]),
            "bgo_fft_shift_f32": (None, [_f32p, i32, i32]),
            "bgo_fft_shift_f64": (None, [_f64p, i32, i32]),
            "bgo_image_f64": (None, [_f32p, _f32p, i32, i32, _f64p]),
            "bgo_run_f32": (None, [_f32p, i32, i32, i32, _f32p, _f32p, i32, _i32p, _f64p, dbl,
                                   dbl, i32, dbl, i32, _f32p, _f32p, _f32p]),
            "bgo_vector_sum": (None, [_f32p, i64, i32, _f64p]),
            "bgo_image_average": (None, [_f32p, i64, i32, _f32p]),
            "bgo_max_threads": (i32, []),
            "bgo_compressed_blocks": (i64, [i64]),
            "bgo_ingest_matrices": (None, [_f32p, _f32p, C.c_void_p, C.c_void_p, i32, i64, _f32p]),
            "bgo_kb_tables": (None, [i32, i32, _f64p]),
            "bgo_pointed_uvw": (None, [_f64p, i32, _f64p, i32, _f32p, _f32p, _f32p]),
            "bgo_gridding_kb": (i64, [_f32p, i32, i32, i32, _f32p, _f32p, i32, _i32p, _f64p, dbl, dbl, i32, dbl,
                                      i32, i32, i32, _f32p, _f32p]),
            "bgo_compress": (None, [_f32p, i64, i64, i32, _u16p, _f32p]),
            "bgo_decompress": (None, [_u16p, _f32p, i64, i64, i32, _f32p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def ref_library():
    """The reference's own CPU code (built here against ref_shim), or None when absent."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        lib = C.CDLL(REF_PATH)
        i32, dbl, flt = C.c_int, C.c_double, C.c_float
        lib.ref_apply_geometric_cpu.argtypes = [_f32p, i32, i32, i32, _f32p, _f64p]
        lib.ref_apply_cable_cpu.argtypes = [_f32p, i32, i32, i32, _f64p, _f64p]
        lib.ref_fft_shift.argtypes = [_f32p, i32, i32]
        lib.ref_fft_shift.restype = None
        lib.ref_pointed_uvw.argtypes = [_f64p, i32, _f64p, _f64p, _f64p, _f64p, _f64p, i32, _f32p, _f32p, _f32p, _f64p]
        lib.ref_pointed_uvw.restype = None
        lib.ref_set_kernel_size.argtypes = [i32]
        lib.ref_set_kernel_size.restype = None
        lib.ref_run.argtypes = [_f32p, i32, i32, i32, _f32p, _f32p, _f32p, _f64p, _i32p, i32,
                                dbl, i32, dbl, i32, dbl, i32, flt, dbl, i32, C.c_char_p, i32,
                                i32, _f32p, _f32p, _f32p, _f32p, _f64p]
        _ref = lib
    return _ref


# ---------------------------------------------------------------------------------------------
# numpy-level helpers
# ---------------------------------------------------------------------------------------------
def n_baselines(n_ant: int) -> int:
    return n_ant * (n_ant + 1) // 2


def update_flags(n_ant, flagged_ants=()):
    fl = np.zeros(n_baselines(n_ant), np.int32)
    fa = np.ascontiguousarray(np.asarray(list(flagged_ants) or [0], np.int32))
    library().bgo_update_flags(n_ant, fa, len(flagged_ants), fl)
    return fl


def zenith_uvw(x, y, z):
    x, y, z = (np.ascontiguousarray(a, np.float64) for a in (x, y, z))
    nb = n_baselines(len(x))
    u, v, w = (np.zeros(nb, np.float32) for _ in range(3))
    library().bgo_zenith_uvw(len(x), x, y, z, u, v, w)
    return u, v, w


def uv_max(u, v, flags):
    """max |u|, |v| over unflagged baselines of every UVW set in u, v ([sets][B] or [B])."""
    u = np.ascontiguousarray(u, np.float32).reshape(-1)
    v = np.ascontiguousarray(v, np.float32).reshape(-1)
    fl = np.ascontiguousarray(np.tile(np.asarray(flags, np.int32), len(u) // len(flags)))
    um, vm = C.c_double(), C.c_double()
    library().bgo_uv_max(len(u), u, v, fl, C.byref(um), C.byref(vm))
    return um.value, vm.value


def delta_uv(osf, uvmax, n_pixels):
    return library().bgo_delta_uv(osf, uvmax, n_pixels)


def apply_geometric(vis, w, freqs, n_uvw_sets=1):
    """In place on a float32 array [T][C][B][4][2]."""
    T, Cn, nb = vis.shape[:3]
    n_ant = int(round((-1 + np.sqrt(1 + 8 * nb)) / 2))
    library().bgo_apply_geometric(vis.reshape(-1), T, Cn, n_ant, np.ascontiguousarray(w, np.float32),
                                  n_uvw_sets, np.ascontiguousarray(freqs, np.float64))


def apply_cable(vis, cable, freqs):
    T, Cn, nb = vis.shape[:3]
    n_ant = len(cable)
    library().bgo_apply_cable(vis.reshape(-1), T, Cn, n_ant, np.ascontiguousarray(cable, np.float64),
                              np.ascontiguousarray(freqs, np.float64))


def cell_index(u, v, du, dv, wavelength, min_uv, n_pixels, sign):
    return library().bgo_cell_index(u, v, du, dv, wavelength, min_uv, n_pixels, sign)


def gridding(vis, u, v, flags, freqs, du, dv, n_pixels, min_uv=-1000.0, pol="XX", uniform=False,
             n_uvw_sets=1):
    T, Cn, nb = vis.shape[:3]
    n_ant = int(round((-1 + np.sqrt(1 + 8 * nb)) / 2))
    grids = np.zeros((T, Cn, n_pixels, n_pixels, 2), np.float32)
    counters = np.zeros((T, Cn, n_pixels, n_pixels), np.float32)
    n = library().bgo_gridding(np.ascontiguousarray(vis, np.float32).reshape(-1), T, Cn, n_ant,
                               np.ascontiguousarray(u, np.float32), np.ascontiguousarray(v, np.float32),
                               n_uvw_sets, np.ascontiguousarray(flags, np.int32),
                               np.ascontiguousarray(freqs, np.float64), du, dv, n_pixels, min_uv,
                               POL[pol], int(uniform), grids.reshape(-1), counters.reshape(-1))
    return grids, counters, n


def fft2_inverse_f64(x):
    """x complex128 [..., N, N] -> unnormalised inverse 2D DFT."""
    n = x.shape[-1]
    a = np.ascontiguousarray(x, np.complex128)
    out = np.empty_like(a)
    library().bgo_fft2_inverse_f64(a.view(np.float64).reshape(-1), out.view(np.float64).reshape(-1),
                                   n, a.size // (n * n))
    return out


def fft_shift(img):
    """fftshift of a complex64 [ny, nx] image by the reference's half swaps (returns a copy)."""
    a = np.ascontiguousarray(img, np.complex64).copy()
    library().bgo_fft_shift_f32(a.view(np.float32).reshape(-1), a.shape[1], a.shape[0])
    return a


def image_f64(grids, counters):
    """grids float32 [..., N, N, 2], counters [..., N, N] -> complex128 images [..., N, N]."""
    n = counters.shape[-1]
    n_images = counters.size // (n * n)
    out = np.empty(counters.shape, np.complex128)
    library().bgo_image_f64(np.ascontiguousarray(grids, np.float32).reshape(-1),
                            np.ascontiguousarray(counters, np.float32).reshape(-1), n, n_images,
                            out.view(np.float64).reshape(-1))
    return out


def run_f32(vis, u, v, flags, freqs, du, dv, n_pixels, min_uv=-1000.0, pol="XX", n_uvw_sets=1):
    T, Cn, nb = vis.shape[:3]
    n_ant = int(round((-1 + np.sqrt(1 + 8 * nb)) / 2))
    grids = np.zeros((T, Cn, n_pixels, n_pixels, 2), np.float32)
    counters = np.zeros((T, Cn, n_pixels, n_pixels), np.float32)
    images = np.zeros((T, Cn, n_pixels, n_pixels, 2), np.float32)
    library().bgo_run_f32(np.ascontiguousarray(vis, np.float32).reshape(-1), T, Cn, n_ant,
                          np.ascontiguousarray(u, np.float32), np.ascontiguousarray(v, np.float32),
                          n_uvw_sets, np.ascontiguousarray(flags, np.int32),
                          np.ascontiguousarray(freqs, np.float64), du, dv, n_pixels, min_uv, POL[pol],
                          grids.reshape(-1), counters.reshape(-1), images.reshape(-1))
    return images.view(np.complex64)[..., 0]


def vector_sum(data, image_size, n_images):
    out = np.zeros(n_images, np.float64)
    library().bgo_vector_sum(np.ascontiguousarray(data, np.float32).reshape(-1), image_size, n_images, out)
    return out


def image_average(images):
    """complex64 [n, ...] -> complex64 mean image."""
    a = np.ascontiguousarray(images, np.complex64)
    n = a.shape[0]
    size = a[0].size
    out = np.zeros(a.shape[1:], np.complex64)
    library().bgo_image_average(a.view(np.float32).reshape(-1), size, n, out.view(np.float32).reshape(-1))
    return out


def full_pipeline(vis_raw, u, v, w, cable, flags, freqs, n_pixels, osf=2.0, min_uv=-1000.0,
                  pol="XX", n_uvw_sets=1, apply_geom=True, apply_cable_corr=True):
    """Reference run(): corrections, delta_u from u_max, gridding, FP64 images.
    Returns (corrected vis, grids, counters, images complex128, (du, dv))."""
    vis = np.array(vis_raw, np.float32, copy=True)
    if apply_geom:
        apply_geometric(vis, w, freqs, n_uvw_sets)
    if apply_cable_corr:
        apply_cable(vis, cable, freqs)
    umax, vmax = uv_max(u, v, flags)
    du, dv = delta_uv(osf, umax, n_pixels), delta_uv(osf, vmax, n_pixels)
    grids, counters, _ = gridding(vis, u, v, flags, freqs, du, dv, n_pixels, min_uv, pol,
                                  n_uvw_sets=n_uvw_sets)
    images = image_f64(grids, counters)
    return vis, grids, counters, images, (du, dv)


def compress(vis, fmt="s16"):
    """Block-scaled 16-bit storage of vis float32 [T][C][B][4][2] (blink_compress.c): returns
    (data uint16 [T][C][4][B][2], scales float32 [T][C][4][ceil(B/128)])."""
    vis = np.ascontiguousarray(vis, np.float32)
    T, Cn, nb = vis.shape[:3]
    nblk = int(library().bgo_compressed_blocks(nb))
    data = np.empty((T, Cn, 4, nb, 2), np.uint16)
    scales = np.empty((T, Cn, 4, nblk), np.float32)
    library().bgo_compress(vis.reshape(-1), T * Cn, nb, VIS_FORMAT[fmt], data.reshape(-1), scales.reshape(-1))
    return data, scales


def decompress(data, scales, fmt="s16"):
    """Inverse of compress(): float32 visibilities [T][C][B][4][2]."""
    data = np.ascontiguousarray(data, np.uint16)
    scales = np.ascontiguousarray(scales, np.float32)
    T, Cn, _, nb = data.shape[:4]
    vis = np.empty((T, Cn, nb, 4, 2), np.float32)
    library().bgo_decompress(data.reshape(-1), scales.reshape(-1), T * Cn, nb, VIS_FORMAT[fmt], vis.reshape(-1))
    return vis


def ingest_matrices(re_xx, im_xx, re_yy=None, im_yy=None):
    """Correlation matrices float32 [M][n][n] -> visibility records float32 [M][B][4][2]
    (apps/pacer_imager_main.cpp:720-804)."""
    re_xx = np.ascontiguousarray(re_xx, np.float32)
    im_xx = np.ascontiguousarray(im_xx, np.float32)
    M, n = re_xx.shape[0], re_xx.shape[1]
    yy = re_yy is not None and im_yy is not None
    ry = np.ascontiguousarray(re_yy, np.float32) if yy else None
    iy = np.ascontiguousarray(im_yy, np.float32) if yy else None
    vis = np.empty((M, n * (n + 1) // 2, 4, 2), np.float32)
    library().bgo_ingest_matrices(re_xx.reshape(-1), im_xx.reshape(-1), ry.ctypes.data if yy else None,
                                  iy.ctypes.data if yy else None, n, M, vis.reshape(-1))
    return vis


def kb_tables(kernel_size, with_sinc=True):
    """The reference's Kaiser-Bessel gridding kernels, float64 [1023][kernel_size]."""
    t = np.empty((1023, kernel_size), np.float64)
    library().bgo_kb_tables(int(kernel_size), int(bool(with_sinc)), t.reshape(-1))
    return t


def gridding_kb(vis, u, v, flags, freqs, du, dv, n_pixels, kernel_size, min_uv=-1000.0, pol="XX", n_uvw_sets=1,
                with_sinc=True):
    """Kaiser-Bessel convolutional gridding (src/pacer_imager.cpp:378-403, 565-750)."""
    T, Cn, nb = vis.shape[:3]
    n_ant = int(round((-1 + np.sqrt(1 + 8 * nb)) / 2))
    grids = np.zeros((T, Cn, n_pixels, n_pixels, 2), np.float32)
    counters = np.zeros((T, Cn, n_pixels, n_pixels), np.float32)
    n = library().bgo_gridding_kb(np.ascontiguousarray(vis, np.float32).reshape(-1), T, Cn, n_ant,
                                  np.ascontiguousarray(u, np.float32), np.ascontiguousarray(v, np.float32),
                                  n_uvw_sets, np.ascontiguousarray(flags, np.int32),
                                  np.ascontiguousarray(freqs, np.float64), du, dv, n_pixels, min_uv, POL[pol],
                                  int(kernel_size), int(bool(with_sinc)), grids.reshape(-1), counters.reshape(-1))
    return grids, counters, n


def uvw_step(rmatpr, ha2000, dec_aber, lmst, lmst2000):
    """One timestep's geometry as the 17 numbers the pointed-UVW routines take."""
    r = np.asarray(rmatpr, np.float64).reshape(9)
    return np.concatenate([r, [np.sin(lmst), np.cos(lmst), np.sin(lmst2000), np.cos(lmst2000), np.sin(ha2000),
                               np.cos(ha2000), np.sin(dec_aber), np.cos(dec_aber)]])


def pointed_uvw(xyz, steps):
    """Pointed UVW float32 [T][B] x3 from antenna XYZ [n][3] and steps [T][17]."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    steps = np.ascontiguousarray(np.atleast_2d(steps), np.float64)
    n, T = xyz.shape[0], steps.shape[0]
    nb = n * (n + 1) // 2
    u, v, w = (np.empty((T, nb), np.float32) for _ in range(3))
    library().bgo_pointed_uvw(xyz.reshape(-1), n, steps.reshape(-1), T, u.reshape(-1), v.reshape(-1), w.reshape(-1))
    return u, v, w
