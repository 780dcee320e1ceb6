"""Python host API over the C ABI, with torch tensors as device memory.

Mirrors the reference imager's GPU entry points (PaCER-BLINK-Project/imager, src/gpu/*.h) and
its CPacerImagerHip driver (src/gpu/pacer_imager_hip.cpp) for scripting, tests and the
benchmark.  Every call goes to the CUDA library; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import capi
from .capi import APPLY_CABLE, APPLY_GEOMETRIC, OUTPUT_REAL, POL, VIS_FORMAT, WEIGHT_UNIFORM, call

__all__ = ["Imager", "apply_geometric_corrections", "apply_cable_corrections", "gridding",
           "fft_inverse", "fft_shift_and_norm", "uniform_weighting", "vector_sum", "image_averaging",
           "APPLY_GEOMETRIC", "APPLY_CABLE", "OUTPUT_REAL", "WEIGHT_UNIFORM", "POL"]


def _ptr(t):
    if t is None:
        return None
    if isinstance(t, torch.Tensor):
        if not t.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return C.c_void_p(t.data_ptr())
    if isinstance(t, np.ndarray):
        if not t.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return C.c_void_p(t.ctypes.data)
    raise TypeError(type(t))


def _stream(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def _n_ant(n_baselines: int) -> int:
    n = int(round((-1 + math.sqrt(1 + 8 * n_baselines)) / 2))
    if n * (n + 1) // 2 != n_baselines:
        raise ValueError(f"{n_baselines} is not a triangular baseline count")
    return n


def _out_dtype(flags):
    return torch.float32 if flags & OUTPUT_REAL else torch.complex64


def _vis_dims(vis: torch.Tensor):
    """(T, C, B) of a visibility tensor: complex64 [T][C][B][4] or float32 [T][C][B][4][2]."""
    if vis.dtype == torch.complex64:
        if vis.dim() != 4 or vis.shape[3] != 4:
            raise ValueError("complex visibilities must be [T][C][B][4]")
    elif vis.dtype == torch.float32:
        if vis.dim() != 5 or vis.shape[3:] != (4, 2):
            raise ValueError("float visibilities must be [T][C][B][4][2]")
    else:
        raise TypeError(vis.dtype)
    return int(vis.shape[0]), int(vis.shape[1]), int(vis.shape[2])


# ----------------------------------------------------------------------------------------------
# reference GPU entry points
# ----------------------------------------------------------------------------------------------
def apply_geometric_corrections(vis, w, freqs, n_uvw_sets=1, stream=None):
    """apply_geometric_corrections_gpu (src/gpu/corrections_gpu.cpp:90): in place."""
    T, Cn, B = _vis_dims(vis)
    call("bgi_apply_geometric_corrections_gpu", _ptr(vis), _n_ant(B), Cn, T, _ptr(w), n_uvw_sets,
         _ptr(freqs), _stream(stream))


def apply_cable_corrections(vis, cable, freqs, stream=None):
    """apply_cable_lengths_corrections_gpu (src/gpu/corrections_gpu.cpp:75): in place."""
    T, Cn, B = _vis_dims(vis)
    call("bgi_apply_cable_lengths_corrections_gpu", _ptr(vis), _n_ant(B), Cn, T, _ptr(cable),
         _ptr(freqs), _stream(stream))


def gridding(vis, u, v, flags, freqs, delta_u, delta_v, n_pixels, min_uv, pol, grids, counters=None,
             counter_mode=capi.COUNTERS_PER_IMAGE, n_uvw_sets=1, stream=None):
    """gridding_gpu (src/gpu/gridding_gpu.cpp:130): accumulates into grids (complex64
    [T][C][N][N]) and counters."""
    T, Cn, B = _vis_dims(vis)
    call("bgi_gridding_gpu", _ptr(vis), _n_ant(B), Cn, T, _ptr(u), _ptr(v), n_uvw_sets, _ptr(flags),
         None, _ptr(freqs), float(delta_u), float(delta_v), int(n_pixels), float(min_uv),
         POL[pol] if isinstance(pol, str) else int(pol), int(counter_mode), _ptr(counters),
         _ptr(grids), _stream(stream))


def gridding_kb(vis, u, v, flags, freqs, delta_u, delta_v, n_pixels, min_uv, pol, grids, counters=None,
                kernel_size=7, with_sinc=True, counter_mode=capi.COUNTERS_PER_IMAGE, n_uvw_sets=1, stream=None):
    """Kaiser-Bessel convolutional gridding (src/pacer_imager.cpp:378-403, 565-750) into grids."""
    T, Cn, B = _vis_dims(vis)
    call("bgi_gridding_kb_gpu", _ptr(vis), _n_ant(B), Cn, T, _ptr(u), _ptr(v), n_uvw_sets, _ptr(flags),
         _ptr(freqs), float(delta_u), float(delta_v), int(n_pixels), float(min_uv),
         POL[pol] if isinstance(pol, str) else int(pol), int(counter_mode), _ptr(counters), _ptr(grids),
         int(kernel_size), int(bool(with_sinc)), _stream(stream))


def pointed_uvw(xyz, steps, stream=None):
    """Pointed-observation UVW on the device: xyz (device float64 [n_ant][3]) and steps (device
    float64 [T][17], see uvw_steps) -> u, v, w float32 [T][B] on the device."""
    n_ant, T = int(xyz.shape[0]), int(steps.shape[0])
    B = n_ant * (n_ant + 1) // 2
    u, v, w = (torch.empty((T, B), dtype=torch.float32, device=xyz.device) for _ in range(3))
    call("bgi_pointed_uvw_gpu", _ptr(xyz), n_ant, _ptr(steps), T, _ptr(u), _ptr(v), _ptr(w), _stream(stream))
    return u, v, w


def uvw_steps(rmatpr, ha2000, dec_aber, lmst, lmst2000):
    """Timestep geometry float64 [T][17] from per-timestep matrices and angles (host libm)."""
    rm = np.asarray(rmatpr, np.float64).reshape(-1, 9)
    ha, dec, lm, lm2 = (np.atleast_1d(np.asarray(a, np.float64)) for a in (ha2000, dec_aber, lmst, lmst2000))
    out = np.empty((len(ha), 17), np.float64)
    for t in range(len(ha)):
        st = capi.UvwStep()
        r = (C.c_double * 9)(*rm[t])
        call("bgi_uvw_step_from_angles", C.cast(r, C.c_void_p), float(ha[t]), float(dec[t]), float(lm[t]),
             float(lm2[t]), C.byref(st))
        out[t, :9] = list(st.rmatpr)
        out[t, 9:] = [st.sin_lmst, st.cos_lmst, st.sin_lmst2000, st.cos_lmst2000, st.sin_ha2000, st.cos_ha2000,
                      st.sin_dec, st.cos_dec]
    return out


def gridding_sorted_workspace_bytes(n_ant, n_pixels, n_images):
    """Device bytes bgi_gridding_sorted_gpu needs to grid n_images images in one chunk."""
    out = C.c_size_t(0)
    call("bgi_gridding_sorted_workspace", int(n_ant), int(n_pixels), int(n_images), C.byref(out))
    return int(out.value)


def gridding_sorted(vis, u, v, flags, freqs, delta_u, delta_v, n_pixels, min_uv, pol, grids, counters=None,
                    counter_mode=capi.COUNTERS_PER_IMAGE, n_uvw_sets=1, workspace=None, stream=None):
    """Deterministic gridding: gridding()'s result with every cell summed in the CPU loop's order
    (src/pacer_imager.cpp:297-408), bit-identical run to run.  workspace: a uint8 CUDA tensor;
    by default one sized for all images is allocated."""
    T, Cn, B = _vis_dims(vis)
    n_ant = _n_ant(B)
    if workspace is None:
        workspace = torch.empty(gridding_sorted_workspace_bytes(n_ant, n_pixels, max(1, T * Cn)),
                                dtype=torch.uint8, device=vis.device)
    call("bgi_gridding_sorted_gpu", _ptr(vis), n_ant, Cn, T, _ptr(u), _ptr(v), n_uvw_sets, _ptr(flags),
         _ptr(freqs), float(delta_u), float(delta_v), int(n_pixels), float(min_uv),
         POL[pol] if isinstance(pol, str) else int(pol), int(counter_mode), _ptr(counters),
         _ptr(grids), _ptr(workspace), workspace.numel(), _stream(stream))


def compress_visibilities(vis, fmt="s16", stream=None):
    """Block-scaled 16-bit storage of device visibilities complex64 [T][C][B][4] (or float32
    [T][C][B][4][2]): returns (data uint16 [T][C][4][B][2], scales float32 [T][C][4][ceil(B/128)])
    on the same device."""
    T, Cn, B = _vis_dims(vis)
    nblk = (B + 127) // 128
    data = torch.empty((T, Cn, 4, B, 2), dtype=torch.int16, device=vis.device)
    scales = torch.empty((T, Cn, 4, nblk), dtype=torch.float32, device=vis.device)
    call("bgi_compress_visibilities", _ptr(vis), _n_ant(B), Cn, T, VIS_FORMAT[fmt], _ptr(data), _ptr(scales),
         _stream(stream))
    return data, scales


def ingest_correlation_matrices(re_xx, im_xx, re_yy=None, im_yy=None, fmt="c64", stream=None):
    """Correlation matrices (device float32 [T][C][n][n]) to visibilities: complex64 records
    [T][C][B][4] for fmt "c64", else 16-bit stored (data, scales) as compress_visibilities."""
    T, Cn, n = int(re_xx.shape[0]), int(re_xx.shape[1]), int(re_xx.shape[2])
    B = n * (n + 1) // 2
    if fmt == "c64":
        vis = torch.empty((T, Cn, B, 4), dtype=torch.complex64, device=re_xx.device)
        call("bgi_ingest_correlation_matrices", _ptr(re_xx), _ptr(im_xx), _ptr(re_yy), _ptr(im_yy), n, Cn, T,
             VIS_FORMAT[fmt], _ptr(vis), None, _stream(stream))
        return vis
    data = torch.empty((T, Cn, 4, B, 2), dtype=torch.int16, device=re_xx.device)
    scales = torch.empty((T, Cn, 4, (B + 127) // 128), dtype=torch.float32, device=re_xx.device)
    call("bgi_ingest_correlation_matrices", _ptr(re_xx), _ptr(im_xx), _ptr(re_yy), _ptr(im_yy), n, Cn, T,
         VIS_FORMAT[fmt], _ptr(data), _ptr(scales), _stream(stream))
    return data, scales


def fft_inverse(grids, images, stream=None):
    """gpufftExecC2C(..., BACKWARD) replacement: unnormalised inverse 2D FFT, out of place."""
    n = int(grids.shape[-1])
    call("bgi_fft_inverse_gpu", _ptr(grids), _ptr(images), n, grids.numel() // (n * n), _stream(stream))


def fft_shift_and_norm(images, fnorm, stream=None):
    """fft_shift_and_norm_gpu (src/gpu/gpu_utils.cpp:128), images complex64 [..., Y, X]."""
    ys, xs = int(images.shape[-2]), int(images.shape[-1])
    call("bgi_fft_shift_and_norm_gpu", _ptr(images), xs, ys, images.numel() // (xs * ys), _ptr(fnorm),
         int(fnorm.numel()), _stream(stream))


def uniform_weighting(grids, counters, stream=None):
    """Weighting "U" of the CPU gridder (src/pacer_imager.cpp:419-428): grids (complex64
    [..., N, N]) divided cell by cell by counters (float32, same shape), in place."""
    n = int(grids.shape[-1])
    n_images = grids.numel() // (n * n)
    call("bgi_uniform_weighting_gpu", _ptr(grids), _ptr(counters), n, n_images, _stream(stream))


def vector_sum(data, image_size, n_images, sums, stream=None):
    call("bgi_vector_sum_gpu", _ptr(data), int(image_size), int(n_images), _ptr(sums), _stream(stream))


def image_averaging(images, out, stream=None):
    n = int(images.shape[0])
    call("bgi_image_averaging_gpu", _ptr(images), images[0].numel(), n, _ptr(out), _stream(stream))


# ----------------------------------------------------------------------------------------------
# imager handle
# ----------------------------------------------------------------------------------------------
class Imager:
    """Resident-state imager (CPacerImagerHip's members, src/gpu/pacer_imager_hip.h:14-27)."""

    def __init__(self, n_pixels: int, oversampling_factor: float = 2.0, pol="XX",
                 min_uv: float = -math.inf, max_images_per_wave: int = 0, device: int = 0,
                 full_plane: bool = False):
        cfg = capi.Config(int(n_pixels), float(oversampling_factor),
                          POL[pol] if isinstance(pol, str) else int(pol), float(min_uv),
                          int(max_images_per_wave), int(device), int(bool(full_plane)))
        h = C.c_void_p()
        call("bgi_create", C.byref(cfg), C.byref(h))
        self._h = h
        self.n_pixels = int(n_pixels)
        self.device = int(device)
        self.n_channels = 0

    def close(self):
        if self._h:
            capi.lib().bgi_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_array(self, u, v, w, flags, cable):
        u = np.ascontiguousarray(np.atleast_2d(u), np.float32)
        v = np.ascontiguousarray(np.atleast_2d(v), np.float32)
        w = None if w is None else np.ascontiguousarray(np.atleast_2d(w), np.float32)
        flags = np.ascontiguousarray(flags, np.int32)
        cable = None if cable is None else np.ascontiguousarray(cable, np.float64)
        n_ant = _n_ant(u.shape[1])
        call("bgi_set_array", self._h, n_ant, u.shape[0], _ptr(u), _ptr(v), _ptr(w), _ptr(flags),
             _ptr(cable))

    def set_array_pointed(self, xyz, steps, flags, cable):
        """Resident state with pointed UVW computed on the device: xyz float64 [n_ant][3] (local
        XYZ, metres), steps float64 [T][17] (uvw_steps), one UVW set per interval."""
        xyz = np.ascontiguousarray(xyz, np.float64)
        steps = np.ascontiguousarray(np.atleast_2d(steps), np.float64)
        flags = np.ascontiguousarray(flags, np.int32)
        cable = None if cable is None else np.ascontiguousarray(cable, np.float64)
        call("bgi_set_array_pointed", self._h, xyz.shape[0], _ptr(xyz), steps.shape[0], _ptr(steps), _ptr(flags),
             _ptr(cable))

    def set_frequencies(self, freqs):
        f = np.ascontiguousarray(freqs, np.float64)
        call("bgi_set_frequencies", self._h, len(f), _ptr(f))
        self.n_channels = len(f)

    @property
    def half_plane(self) -> bool:
        """Whether image() takes the half-plane (complex-to-real) path for the current state."""
        st = capi.lib().bgi_half_plane(self._h)
        capi.check(min(st, 0))
        return bool(st)

    def set_uv_cell(self, delta_u: float, delta_v: float):
        """Use the uv cell of a whole observation (when this handle images one shard of it)."""
        call("bgi_set_uv_cell", self._h, float(delta_u), float(delta_v))

    @property
    def uv_cell(self):
        du, dv, um, vm = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        call("bgi_get_uv_cell", self._h, C.byref(du), C.byref(dv), C.byref(um), C.byref(vm))
        return du.value, dv.value, um.value, vm.value

    @property
    def uv_extent(self):
        """(ext_u, ext_v): bound on the |u|, |v| pixel coordinates of every gridded point; the
        half-plane FFT passes skip the grid beyond it (n_pixels/2 each on the full plane)."""
        eu, ev = C.c_int(), C.c_int()
        call("bgi_get_uv_extent", self._h, C.byref(eu), C.byref(ev))
        return eu.value, ev.value

    def image(self, vis: torch.Tensor, flags: int = APPLY_GEOMETRIC | APPLY_CABLE, out=None,
              stream=None) -> torch.Tensor:
        """Dirty images complex64 [T][C][N][N] of device visibilities."""
        T, Cn, _ = _vis_dims(vis)
        n = self.n_pixels
        if out is None:
            out = torch.empty((T, Cn, n, n), dtype=_out_dtype(flags), device=vis.device)
        call("bgi_image", self._h, _ptr(vis), T, int(flags), _ptr(out), _stream(stream))
        return out

    def image_host(self, vis, flags: int = APPLY_GEOMETRIC | APPLY_CABLE, out=None, stream=None):
        """Host buffers in and out (pinned torch tensors or numpy arrays); synchronous."""
        T = int(vis.shape[0])
        Cn = int(vis.shape[1])
        n = self.n_pixels
        if out is None:
            out = np.empty((T, Cn, n, n), np.float32 if flags & OUTPUT_REAL else np.complex64)
        call("bgi_image_host", self._h, _ptr(vis), T, int(flags), _ptr(out), _stream(stream))
        return out

    def image_compressed(self, data, scales, fmt="s16", flags: int = APPLY_GEOMETRIC | APPLY_CABLE, out=None,
                         stream=None) -> torch.Tensor:
        """Dirty images of block-scaled 16-bit device visibilities (compress_visibilities)."""
        T, Cn = int(data.shape[0]), int(data.shape[1])
        n = self.n_pixels
        if out is None:
            out = torch.empty((T, Cn, n, n), dtype=_out_dtype(flags), device=data.device)
        call("bgi_image_compressed", self._h, VIS_FORMAT[fmt], _ptr(data), _ptr(scales), T, int(flags), _ptr(out),
             _stream(stream))
        return out

    def image_compressed_host(self, data, scales, fmt="s16", flags: int = APPLY_GEOMETRIC | APPLY_CABLE,
                              out=None, stream=None):
        """Host buffers in and out; uploads only the pol planes the handle's pol needs."""
        T, Cn = int(data.shape[0]), int(data.shape[1])
        n = self.n_pixels
        if out is None:
            out = np.empty((T, Cn, n, n), np.float32 if flags & OUTPUT_REAL else np.complex64)
        call("bgi_image_compressed_host", self._h, VIS_FORMAT[fmt], _ptr(data), _ptr(scales), T, int(flags),
             _ptr(out), _stream(stream))
        return out

    def image_matrices_host(self, re_xx, im_xx, re_yy=None, im_yy=None, fmt="s16",
                            flags: int = APPLY_GEOMETRIC | APPLY_CABLE, out=None, stream=None):
        """Host correlation matrices float32 [T][C][A][A] (XX; YY optional) to host images: uploaded,
        converted to stored visibilities of `fmt` and imaged on the device, chunk by chunk."""
        T, Cn = int(re_xx.shape[0]), int(re_xx.shape[1])
        n = self.n_pixels
        if out is None:
            out = np.empty((T, Cn, n, n), np.float32 if flags & OUTPUT_REAL else np.complex64)
        call("bgi_image_correlation_matrices_host", self._h, VIS_FORMAT[fmt], _ptr(re_xx), _ptr(im_xx),
             _ptr(re_yy), _ptr(im_yy), T, int(flags), _ptr(out), _stream(stream))
        return out

    @property
    def schedule(self):
        """(images per wave, lanes) of the bgi_image* calls; 0 images per wave = auto."""
        w, l = C.c_int(0), C.c_int(0)
        call("bgi_get_schedule", self._h, C.byref(w), C.byref(l))
        return w.value, l.value

    def set_schedule(self, images_per_wave: int = 0, lanes: int = 2):
        call("bgi_set_schedule", self._h, int(images_per_wave), int(lanes))

    def autotune(self, data, scales=None, fmt="c64", flags: int = APPLY_GEOMETRIC | APPLY_CABLE, out=None,
                 stream=None):
        """Times wave sizes and lane counts on this block (device buffers) and keeps the fastest;
        returns (images per wave, lanes, ms per call)."""
        T, Cn = int(data.shape[0]), int(data.shape[1])
        n = self.n_pixels
        if out is None:
            out = torch.empty((T, Cn, n, n), dtype=_out_dtype(flags), device=data.device)
        best = C.c_double(0.0)
        call("bgi_autotune", self._h, VIS_FORMAT[fmt], _ptr(data), _ptr(scales), T, int(flags), _ptr(out),
             _stream(stream), C.byref(best))
        return (*self.schedule, best.value)

    def set_gridding_kernel(self, kernel_size: int = 0, with_sinc: bool = True):
        """0: nearest neighbour; 1..16: the reference's Kaiser-Bessel convolution kernel."""
        call("bgi_set_gridding_kernel", self._h, int(kernel_size), int(bool(with_sinc)))

    def set_gridding_images_per_thread(self, k: int = 0):
        """Images per gridding thread: 2, 4 or 8 (0: by array size)."""
        call("bgi_set_gridding_images_per_thread", self._h, int(k))

    @property
    def gridding_images_per_thread(self) -> int:
        k = C.c_int()
        call("bgi_get_gridding_images_per_thread", self._h, C.byref(k))
        return k.value

    def set_replay(self, enable: bool = True):
        """Record repeated calls as a CUDA graph and launch it for later repeats (default on)."""
        call("bgi_set_replay", self._h, int(bool(enable)))

    @property
    def replay_ready(self) -> bool:
        """Whether the next call identical to the last one launches its recorded CUDA graph."""
        st = capi.lib().bgi_replay_ready(self._h)
        if st < 0:
            capi.check(st)
        return st == 1

    def set_gridding_aggregation(self, on: bool = False):
        """Warp-aggregated gridding atomics (half plane, 4 or 8 images per thread): points of a
        warp on the same cell summed before one atomic per cell."""
        call("bgi_set_gridding_aggregation", self._h, int(on))

    @property
    def gridding_aggregation(self) -> bool:
        k = C.c_int()
        call("bgi_get_gridding_aggregation", self._h, C.byref(k))
        return bool(k.value)

    def set_column_radix(self, radix: int = 0):
        """Radix of the half-plane column pass (0: the side's default; sides 256..4096 have a
        second compiled radix)."""
        call("bgi_set_column_radix", self._h, int(radix))

    @property
    def column_radix(self) -> int:
        r = C.c_int()
        call("bgi_get_column_radix", self._h, C.byref(r))
        return r.value

    def set_fft_mode(self, mode: str = "simt"):
        """"simt" (FP32 passes) or "tensor_split16" (the complex-to-real pass's transforms as
        split-FP16 DFT products on the tensor cores; image side 512)."""
        call("bgi_set_fft_mode", self._h, capi.FFT_MODE[mode])

    @property
    def fft_mode(self) -> str:
        m = C.c_int()
        call("bgi_get_fft_mode", self._h, C.byref(m))
        return {v: k for k, v in capi.FFT_MODE.items()}[m.value]

    def set_deterministic(self, enable: bool = True):
        """Grid by sort and ordered per-cell sums (the half plane when the handle takes it): the
        same image bits on every run."""
        call("bgi_set_deterministic", self._h, int(bool(enable)))

    def image_wcs(self, ra_deg: float = 0.0, dec_deg: float = -26.703319) -> dict:
        """Phase centre and pixel scales (degrees) of this handle's images, as the reference
        attaches them to its Images (bgi_get_image_wcs)."""
        w = capi.ImageWcs()
        call("bgi_get_image_wcs", self._h, float(ra_deg), float(dec_deg), C.byref(w))
        return {"ra_deg": w.ra_deg, "dec_deg": w.dec_deg, "pixscale_ra_deg": w.pixscale_ra_deg,
                "pixscale_dec_deg": w.pixscale_dec_deg}

    def set_stage_timing(self, enable: bool = True):
        call("bgi_set_stage_timing", self._h, int(bool(enable)))

    def stage_times(self):
        """{stage: (total ms, launches)} since the last read: gridding, the first FFT pass (rows,
        or the half-plane column pass) and the second (columns with the epilogue, or the
        complex-to-real row pass)."""
        ms = (C.c_double * 3)()
        n = (C.c_int64 * 3)()
        call("bgi_get_stage_times", self._h, ms, n)
        return {k: (ms[i], int(n[i])) for i, k in enumerate(("gridding", "fft_pass1", "fft_pass2"))}

    def weight_sums(self, n_images: int, stream=None) -> np.ndarray:
        out = np.zeros(n_images, np.uint32)
        call("bgi_last_weight_sums", self._h, _ptr(out), int(n_images), _stream(stream))
        return out


class Batch:
    """Uneven items (imager, device data, images) replayed as one CUDA graph.

    items: list of dicts with keys imager, data, and optionally scales, fmt ("c64"), flags,
    out (allocated when missing).  Creating the batch runs the items once."""

    def __init__(self, items, stream=None):
        self._items = []
        arr = (capi.BatchItem * len(items))()
        for k, it in enumerate(items):
            h = it["imager"]
            data = it["data"]
            fmt = it.get("fmt", "c64")
            flags = int(it.get("flags", APPLY_GEOMETRIC | APPLY_CABLE))
            T, Cn = int(data.shape[0]), int(data.shape[1])
            out = it.get("out")
            if out is None:
                out = torch.empty((T, Cn, h.n_pixels, h.n_pixels), dtype=_out_dtype(flags), device=data.device)
            scales = it.get("scales")
            arr[k] = capi.BatchItem(h._h.value, VIS_FORMAT[fmt], data.data_ptr(),
                                    scales.data_ptr() if scales is not None else None, T, flags, out.data_ptr())
            self._items.append((h, data, scales, out))
        b = C.c_void_p()
        call("bgi_batch_create", arr, len(items), _stream(stream), C.byref(b))
        self._b = b

    @property
    def outputs(self):
        return [it[3] for it in self._items]

    def launch(self, stream=None):
        call("bgi_batch_launch", self._b, _stream(stream))

    def close(self):
        if self._b:
            capi.lib().bgi_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------------
# FITS output (bgi_write_fits, bgi_write_fits_block)
# ------------------------------------------------------------------------------------------
def _wcs_struct(wcs):
    if wcs is None:
        return None
    return C.byref(capi.ImageWcs(wcs["ra_deg"], wcs["dec_deg"], wcs["pixscale_ra_deg"], wcs["pixscale_dec_deg"]))


def _host_image_block(images):
    """(float32 host array, pixel stride): real images as they are, complex ones by real part."""
    if isinstance(images, torch.Tensor):
        images = images.detach().cpu().numpy()
    a = np.ascontiguousarray(images)
    if a.dtype == np.complex64:
        return a.view(np.float32), 2
    if a.dtype != np.float32:
        raise TypeError("images must be float32 (real) or complex64")
    return a, 1


def write_fits(path, image, wcs=None, freq_hz: float = 0.0):
    """One image [ny][nx] (float32, or complex64: its real part) to a FITS file; wcs from
    Imager.image_wcs."""
    if len(image.shape) != 2:
        raise ValueError("one image [ny][nx]")
    ny, nx = int(image.shape[0]), int(image.shape[1])
    a, stride = _host_image_block(image)
    call("bgi_write_fits", str(path).encode(), _ptr(a), int(nx), int(ny), stride, _wcs_struct(wcs), float(freq_hz))


def write_fits_block(directory, prefix, images, wcs=None, freqs_hz=None):
    """Every image of a block [T][C][ny][nx] to <directory>/<prefix>_t<TTTT>_c<CCCC>.fits."""
    a, stride = _host_image_block(images)
    T, Cn, ny, nx = (int(x) for x in images.shape)
    f = None if freqs_hz is None else np.ascontiguousarray(freqs_hz, np.float64)
    call("bgi_write_fits_block", str(directory).encode(), str(prefix).encode(), _ptr(a), T, Cn, nx, ny, stride,
         _wcs_struct(wcs), _ptr(f) if f is not None else None)
