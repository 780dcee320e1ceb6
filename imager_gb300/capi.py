"""ctypes binding of the C ABI in include/blink_imager_gb300.h.

The library is built in tree (``python -m imager_gb300.build``) to
``imager_gb300/_lib/libblink_imager_gb300.so``.  Loading fails loudly when it is missing: there
is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

HEADER = os.path.join(_build.ROOT, "include", "blink_imager_gb300.h")

OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_UNSUPPORTED, ERR_STATE = 0, -1, -2, -3, -4, -5
ERR_BUSY, ERR_CANCELLED = -6, -7
POL = {"XX": 0, "YY": 1, "I": 2, "V": 3}
COUNTERS_FIRST_INTERVAL, COUNTERS_PER_IMAGE = 0, 1
APPLY_GEOMETRIC, APPLY_CABLE, OUTPUT_REAL, WEIGHT_UNIFORM = 0x1, 0x2, 0x4, 0x8
VIS_FORMAT = {"c64": 0, "s16": 1, "bf16": 2, "fp16": 3}
FFT_MODE = {"simt": 0, "tensor_split16": 1}


class BgiError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("n_pixels", C.c_int), ("oversampling_factor", C.c_float), ("pol", C.c_int),
                ("min_uv", C.c_double), ("max_images_per_wave", C.c_int), ("device", C.c_int),
                ("full_plane", C.c_int)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("max_slots", C.c_int), ("hbm_budget_bytes", C.c_size_t),
                ("reserve_bytes", C.c_size_t), ("deterministic", C.c_int), ("max_queued", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("images", C.c_uint64), ("admission_waits", C.c_uint64), ("queued", C.c_uint64),
                ("device_bytes_in_use", C.c_size_t), ("device_budget_bytes", C.c_size_t),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double), ("mean_ms", C.c_double),
                ("wall_s", C.c_double), ("images_per_s", C.c_double), ("rejected", C.c_uint64),
                ("cancelled", C.c_uint64)]


class BatchItem(C.Structure):
    _fields_ = [("imager", C.c_void_p), ("format", C.c_int), ("data", C.c_void_p), ("scales", C.c_void_p),
                ("n_intervals", C.c_int), ("flags", C.c_uint), ("images", C.c_void_p)]


class UvwStep(C.Structure):
    _fields_ = [("rmatpr", C.c_double * 9), ("sin_lmst", C.c_double), ("cos_lmst", C.c_double),
                ("sin_lmst2000", C.c_double), ("cos_lmst2000", C.c_double), ("sin_ha2000", C.c_double),
                ("cos_ha2000", C.c_double), ("sin_dec", C.c_double), ("cos_dec", C.c_double)]


class ImageWcs(C.Structure):
    _fields_ = [("ra_deg", C.c_double), ("dec_deg", C.c_double), ("pixscale_ra_deg", C.c_double),
                ("pixscale_dec_deg", C.c_double)]


_vp, _i, _i64, _d, _f, _u = C.c_void_p, C.c_int, C.c_int64, C.c_double, C.c_float, C.c_uint
_SIGNATURES = {
    "bgi_last_error": (C.c_char_p, []),
    "bgi_version": (_i, []),
    "bgi_apply_geometric_corrections_gpu": (_i, [_vp, _i, _i, _i, _vp, _i, _vp, _vp]),
    "bgi_apply_cable_lengths_corrections_gpu": (_i, [_vp, _i, _i, _i, _vp, _vp, _vp]),
    "bgi_gridding_gpu": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _vp, _vp, _vp, _d, _d, _i, _d, _i, _i,
                              _vp, _vp, _vp]),
    "bgi_gridding_sorted_workspace": (_i, [_i, _i, _i, C.POINTER(C.c_size_t)]),
    "bgi_gridding_sorted_gpu": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _vp, _vp, _d, _d, _i, _d, _i, _i,
                                     _vp, _vp, _vp, C.c_size_t, _vp]),
    "bgi_fft_inverse_gpu": (_i, [_vp, _vp, _i, _i, _vp]),
    "bgi_compressed_size": (_i, [_i, _i, _i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "bgi_compress_visibilities": (_i, [_vp, _i, _i, _i, _i, _vp, _vp, _vp]),
    "bgi_ingest_correlation_matrices": (_i, [_vp, _vp, _vp, _vp, _i, _i, _i, _i, _vp, _vp, _vp]),
    "bgi_image_compressed": (_i, [_vp, _i, _vp, _vp, _i, C.c_uint, _vp, _vp]),
    "bgi_image_compressed_host": (_i, [_vp, _i, _vp, _vp, _i, C.c_uint, _vp, _vp]),
    "bgi_fft_shift_and_norm_gpu": (_i, [_vp, _i, _i, _i, _vp, _i, _vp]),
    "bgi_vector_sum_gpu": (_i, [_vp, _i64, _i, _vp, _vp]),
    "bgi_uniform_weighting_gpu": (_i, [_vp, _vp, _i, _i, _vp]),
    "bgi_set_fft_mode": (_i, [_vp, _i]),
    "bgi_set_gridding_images_per_thread": (_i, [_vp, _i]),
    "bgi_set_column_radix": (_i, [_vp, _i]),
    "bgi_image_correlation_matrices_host": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _i, _u, _vp, _vp]),
    "bgi_get_column_radix": (_i, [_vp, _vp]),
    "bgi_get_gridding_images_per_thread": (_i, [_vp, _vp]),
    "bgi_set_gridding_aggregation": (_i, [_vp, _i]),
    "bgi_replay_ready": (_i, [_vp]),
    "bgi_set_replay": (_i, [_vp, _i]),
    "bgi_get_gridding_aggregation": (_i, [_vp, _vp]),
    "bgi_get_fft_mode": (_i, [_vp, _vp]),
    "bgi_image_averaging_gpu": (_i, [_vp, _i64, _i, _vp, _vp]),
    "bgi_create": (_i, [C.POINTER(Config), C.POINTER(_vp)]),
    "bgi_destroy": (_i, [_vp]),
    "bgi_set_array": (_i, [_vp, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "bgi_set_frequencies": (_i, [_vp, _i, _vp]),
    "bgi_half_plane": (_i, [_vp]),
    "bgi_set_uv_cell": (_i, [_vp, _d, _d]),
    "bgi_get_uv_cell": (_i, [_vp, C.POINTER(_d), C.POINTER(_d), C.POINTER(_d), C.POINTER(_d)]),
    "bgi_get_uv_extent": (_i, [_vp, C.POINTER(_i), C.POINTER(_i)]),
    "bgi_uv_extent": (_i, [_d, _d, _d, _d, _d, _i, C.POINTER(_i), C.POINTER(_i)]),
    "bgi_image": (_i, [_vp, _vp, _i, _u, _vp, _vp]),
    "bgi_image_host": (_i, [_vp, _vp, _i, _u, _vp, _vp]),
    "bgi_last_weight_sums": (_i, [_vp, _vp, _i, _vp]),
    "bgi_image_noalloc": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _vp, _vp, _d, _d, _i, _d, _i, _vp, _vp]),
    "bgi_set_deterministic": (_i, [_vp, _i]),
    "bgi_uvw_step_from_angles": (_i, [_vp, _d, _d, _d, _d, C.POINTER(UvwStep)]),
    "bgi_pointed_uvw_gpu": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp, _vp]),
    "bgi_set_array_pointed": (_i, [_vp, _i, _vp, _i, _vp, _vp, _vp]),
    "bgi_set_gridding_kernel": (_i, [_vp, _i, _i]),
    "bgi_gridding_kb_gpu": (_i, [_vp, _i, _i, _i, _vp, _vp, _i, _vp, _vp, _d, _d, _i, _d, _i, _i, _vp, _vp, _i, _i,
                                 _vp]),
    "bgi_batch_create": (_i, [C.POINTER(BatchItem), _i, _vp, C.POINTER(_vp)]),
    "bgi_batch_launch": (_i, [_vp, _vp]),
    "bgi_batch_destroy": (_i, [_vp]),
    "bgi_server_create": (_i, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "bgi_server_destroy": (_i, [_vp]),
    "bgi_server_add_array": (_i, [_vp, C.POINTER(Config), _i, _i, _vp, _vp, _vp, _vp, _vp, _i, _vp, C.POINTER(_i)]),
    "bgi_server_submit": (_i, [_vp, _i, _i, _vp, _vp, _i, C.c_uint, _vp, C.POINTER(C.c_uint64)]),
    "bgi_server_wait": (_i, [_vp, C.c_uint64, _i, C.POINTER(_i)]),
    "bgi_server_poll": (_i, [_vp, C.c_uint64, C.POINTER(_i), C.POINTER(_i)]),
    "bgi_server_cancel": (_i, [_vp, C.c_uint64]),
    "bgi_server_get_stats": (_i, [_vp, C.POINTER(ServerStats)]),
    "bgi_server_reset_stats": (_i, [_vp]),
    "bgi_set_schedule": (_i, [_vp, _i, _i]),
    "bgi_get_schedule": (_i, [_vp, C.POINTER(_i), C.POINTER(_i)]),
    "bgi_autotune": (_i, [_vp, _i, _vp, _vp, _i, C.c_uint, _vp, _vp, C.POINTER(C.c_double)]),
    "bgi_device_fault": (_i, [_i, C.POINTER(C.c_uint), _i]),
    "bgi_selftest_wait_timeout": (_i, [_i, _vp]),
    "bgi_get_image_wcs": (_i, [_vp, _d, _d, C.POINTER(ImageWcs)]),
    "bgi_write_fits": (_i, [C.c_char_p, _vp, _i, _i, _i, C.POINTER(ImageWcs), _d]),
    "bgi_write_fits_block": (_i, [C.c_char_p, C.c_char_p, _vp, _i, _i, _i, _i, _i, C.POINTER(ImageWcs), _vp]),
    "bgi_set_stage_timing": (_i, [_vp, _i]),
    "bgi_get_stage_times": (_i, [_vp, C.POINTER(_d), C.POINTER(_i64)]),
}

_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def lib(build_if_missing: bool = False):
    """The loaded C library.  Raises when it has not been built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"{path} is missing: run `python -m imager_gb300.build` "
                                   "(the imaging path has no CPU fallback)")
            _build.build()
        L = C.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def header_functions():
    """Names of every function the public header declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bgi_\w+)\s*\(", text)))


def check(status: int) -> None:
    if status != OK:
        msg = lib().bgi_last_error()
        raise BgiError(status, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
