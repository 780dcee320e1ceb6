"""The uv-coverage bound that the half-plane FFT passes are pruned to (bgi_uv_extent, the
function the imager handle calls), checked on the host against the oracle's cell indices.

The top frequency of each case puts the largest pixel coordinate (N * nu_max / (c * osf) with
the reference's delta_u = osf * u_max / N) on a tie, just either side of an integer, or near N/2.
Every cell that the oracle's gridder touches must lie within the bound, and the bound may be at
most two pixels loose."""
import ctypes as C
import math
import os
import shutil

import numpy as np
import pytest

from imager_gb300 import capi, synth
from oracle import oracle as O

C_LIGHT = 299792458.0


@pytest.fixture(scope="module")
def lib():
    if shutil.which("nvcc") is None and not os.path.exists(capi.library_path()):
        pytest.skip("nvcc not available to build the library")
    O.build()
    return capi.lib(build_if_missing=True)


def _extent(lib, um, vm, du, dv, fmax, n):
    eu, ev = C.c_int(), C.c_int()
    assert lib.bgi_uv_extent(um, vm, du, dv, fmax, n, C.byref(eu), C.byref(ev)) == capi.OK
    return eu.value, ev.value


def _cases():
    out = []
    for n in (64, 512):
        h = n // 2
        for x in (0.3 * h + 0.5, math.floor(0.6 * h) - 1e-9, math.floor(0.6 * h) + 1e-9, h - 2.5, h - 2.0 - 1e-9,
                  h - 1.5):
            out.append((n, x))
    return out


@pytest.mark.parametrize("seed", [53, 54])
@pytest.mark.parametrize("osf", [1.0, 2.0, 3.5])
@pytest.mark.parametrize("n,x", _cases())
def test_bound_covers_every_gridded_cell(lib, n, x, osf, seed):
    f_top = x * C_LIGHT * osf / n
    obs = synth.small(seed=seed, n_ant=24, n_intervals=2, n_channels=3, n_pixels=n, f0=f_top - 2e6, df=1e6)
    um, vm = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(osf, um, n), O.delta_uv(osf, vm, n)
    eu, ev = _extent(lib, um, vm, du, dv, float(obs.freqs.max()), n)
    _, counters, _ = O.gridding(obs.vis_f32(), obs.u, obs.v, obs.flags, obs.freqs, du, dv, n, -1000.0, "XX",
                                n_uvw_sets=2)
    vi, ui = np.nonzero(counters.reshape(-1, n, n).sum(0))
    assert len(ui) > 0
    h = n // 2
    for idx, e in ((ui, eu), (vi, ev)):
        if e >= h:  # the bound reaches the half plane's edge: no pruning
            assert e == h
            continue
        top = np.abs(np.where(idx > h, idx - n, idx)).max()  # wrapped index -> signed pixel
        assert top <= e, (top, e)
        assert top >= e - 2, (top, e)


def test_bound_arguments(lib):
    eu, ev = C.c_int(), C.c_int()
    assert _extent(lib, 10.0, 20.0, 1.0, 1.0, C_LIGHT, 512) == (12, 22)
    assert _extent(lib, 10.0, 20.0, 0.1, 1.0, C_LIGHT, 64) == (32, 22)  # capped at N/2
    assert _extent(lib, 0.0, 0.0, 1.0, 1.0, C_LIGHT, 64) == (2, 2)
    for args in ((1.0, 1.0, 0.0, 1.0, 1e8, 64), (1.0, 1.0, 1.0, -1.0, 1e8, 64), (float("nan"), 1.0, 1.0, 1.0, 1e8, 64),
                 (1.0, 1.0, 1.0, 1.0, 1e8, 1)):
        assert lib.bgi_uv_extent(*args, C.byref(eu), C.byref(ev)) == capi.ERR_INVALID
    assert lib.bgi_uv_extent(1.0, 1.0, 1.0, 1.0, 1e8, 64, None, C.byref(ev)) == capi.ERR_INVALID
