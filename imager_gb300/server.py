"""Python face of the serving runtime (bgi_server_* in the C ABI).

    sv = Server(device=0, max_slots=4)
    a = sv.add_array(512, u, v, w, flags, cable, freqs)        # resident array state
    t = sv.submit(a, vis)                                      # returns at once
    images = sv.wait(t)                                        # the block's images
    sv.stats()                                                 # p50/p99 latency, images/s

Host buffers stay referenced here until their request is collected.  Pinned buffers (torch
tensors with pin_memory) give asynchronous copies; numpy arrays work too.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import torch

from . import capi
from .capi import APPLY_CABLE, APPLY_GEOMETRIC, OUTPUT_REAL, POL, VIS_FORMAT, call
from .imager import _ptr


class Server:
    def __init__(self, device: int = 0, max_slots: int = 4, hbm_budget_bytes: int = 0,
                 reserve_bytes: int = 1 << 30, deterministic: bool = False, max_queued: int = 0):
        cfg = capi.ServerConfig(int(device), int(max_slots), int(hbm_budget_bytes), int(reserve_bytes),
                                int(bool(deterministic)), int(max_queued))
        h = C.c_void_p()
        call("bgi_server_create", C.byref(cfg), C.byref(h))
        self._h = h
        self.device = int(device)
        self._arrays = {}   # id -> (n_pixels, n_channels)
        self._live = {}     # ticket -> (buffers kept alive, output)

    def close(self):
        if self._h:
            capi.lib().bgi_server_destroy(self._h)
            self._h = C.c_void_p()
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_array(self, n_pixels, u, v, w, flags, cable, freqs, oversampling_factor=2.0, pol="XX",
                  min_uv=-math.inf, full_plane=False, max_images_per_wave=0) -> int:
        cfg = capi.Config(int(n_pixels), float(oversampling_factor), POL[pol] if isinstance(pol, str) else int(pol),
                          float(min_uv), int(max_images_per_wave), self.device, int(bool(full_plane)))
        u = np.ascontiguousarray(np.atleast_2d(u), np.float32)
        v = np.ascontiguousarray(np.atleast_2d(v), np.float32)
        w = None if w is None else np.ascontiguousarray(np.atleast_2d(w), np.float32)
        flags = np.ascontiguousarray(flags, np.int32)
        cable = None if cable is None else np.ascontiguousarray(cable, np.float64)
        freqs = np.ascontiguousarray(freqs, np.float64)
        nb = u.shape[1]
        n_ant = int(round((-1 + math.sqrt(1 + 8 * nb)) / 2))
        aid = C.c_int(-1)
        call("bgi_server_add_array", self._h, C.byref(cfg), n_ant, u.shape[0], _ptr(u), _ptr(v), _ptr(w),
             _ptr(flags), _ptr(cable), len(freqs), _ptr(freqs), C.byref(aid))
        self._arrays[aid.value] = (int(n_pixels), len(freqs))
        return aid.value

    def submit(self, array_id: int, vis=None, *, data=None, scales=None, fmt: str = "c64",
               flags: int = APPLY_GEOMETRIC | APPLY_CABLE, out=None) -> int:
        """Queues one block: complex64 visibilities `vis` [T][C][B][4] (float32 [..][4][2] too), or
        16-bit stored `data` [T][C][4][B][2] with `scales`, host memory.  Returns a ticket."""
        if array_id not in self._arrays:
            raise capi.BgiError(capi.ERR_INVALID, f"no array {array_id} on this server")
        n, n_ch = self._arrays[array_id]
        src = vis if fmt == "c64" else data
        T = int(src.shape[0])
        if out is None:
            dtype = torch.float32 if flags & OUTPUT_REAL else torch.complex64
            out = torch.empty((T, n_ch, n, n), dtype=dtype, pin_memory=True)
        ticket = C.c_uint64(0)
        call("bgi_server_submit", self._h, int(array_id), VIS_FORMAT[fmt], _ptr(src), _ptr(scales), T, int(flags),
             _ptr(out), C.byref(ticket))
        self._live[ticket.value] = ((src, scales), out)
        return ticket.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """The request's images once it has finished (raises BgiError if it failed)."""
        st = C.c_int(0)
        call("bgi_server_wait", self._h, C.c_uint64(ticket), int(timeout_ms), C.byref(st))
        _, out = self._live.pop(ticket)
        capi.check(st.value)
        return out

    def poll(self, ticket: int):
        """The images if the request has finished, else None."""
        done, st = C.c_int(0), C.c_int(0)
        call("bgi_server_poll", self._h, C.c_uint64(ticket), C.byref(done), C.byref(st))
        if not done.value:
            return None
        _, out = self._live.pop(ticket)
        capi.check(st.value)
        return out

    def cancel(self, ticket: int) -> bool:
        """Cancels a request not yet admitted (its wait then raises BgiError ERR_CANCELLED);
        False when it is already on the GPU or finished."""
        st = capi.lib().bgi_server_cancel(self._h, C.c_uint64(ticket))
        if st == capi.ERR_STATE:
            return False
        capi.check(st)
        return True

    def stats(self) -> dict:
        s = capi.ServerStats()
        call("bgi_server_get_stats", self._h, C.byref(s))
        return {name: getattr(s, name) for name, _ in s._fields_}

    def reset_stats(self):
        call("bgi_server_reset_stats", self._h)
