"""Seeded synthetic observations for the imaging path (tests and benchmark inputs).

No public data set exists for this path, so these generators stand in for real correlator
output with the shapes and distributions of the five workloads the imager is measured on:
antenna layouts, point-source skies with a power-law flux distribution, complex Gaussian
noise, cable lengths, channel frequencies and zenith-phased UVW rotated by the Earth.

Conventions follow the reference imager (PaCER-BLINK-Project/imager):
  * baseline b = a1*(a1+1)/2 + a2 with a1 >= a2, autos included (src/pacer_imager.cpp:69-70);
  * u_b = -(x_a1 - x_a2) at zenith (src/antenna_positions.cpp:81-89), in metres, float32;
  * visibilities complex64 [interval][channel][baseline][XX, XY, YX, YY].

The returned "raw" visibilities carry the inverse of the geometric and cable phase
corrections, so that correcting them recovers the sky model.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

VEL_LIGHT = 299792458.0
SIDEREAL_RATE = 2.0 * math.pi / 86164.0905  # rad/s
MWA_LATITUDE_DEG = -26.703319  # src/pacer_imager_defs.h:15


def n_baselines(n_ant: int) -> int:
    return n_ant * (n_ant + 1) // 2


def baseline_antennas(n_ant: int):
    a1 = np.repeat(np.arange(n_ant), np.arange(1, n_ant + 1))
    a2 = np.concatenate([np.arange(i + 1) for i in range(n_ant)])
    return a1, a2


@dataclass
class Observation:
    """One block of visibilities plus the array state needed to image it."""
    vis: np.ndarray            # complex64 [T][C][B][4]
    u: np.ndarray              # float32 [n_uvw_sets][B] metres
    v: np.ndarray
    w: np.ndarray
    cable: np.ndarray          # float64 [A] metres
    flags: np.ndarray          # int32 [B], 1 = flagged
    freqs: np.ndarray          # float64 [C] Hz
    n_pixels: int
    osf: float = 2.0
    min_uv: float = -1000.0
    pol: str = "XX"
    enu: np.ndarray = field(default=None)  # float64 [A][3]

    @property
    def n_ant(self) -> int:
        return len(self.cable)

    @property
    def n_intervals(self) -> int:
        return self.vis.shape[0]

    @property
    def n_channels(self) -> int:
        return self.vis.shape[1]

    @property
    def n_uvw_sets(self) -> int:
        return self.u.shape[0]

    def vis_f32(self):
        """float32 view [T][C][B][4][2] (a numpy array, or a torch tensor when the block was
        kept on the device)."""
        if not isinstance(self.vis, np.ndarray):
            import torch
            return torch.view_as_real(self.vis)
        return self.vis.view(np.float32).reshape(self.vis.shape + (2,))


# ------------------------------------------------------------------------------------------
# antenna layouts
# ------------------------------------------------------------------------------------------
def layout_uniform_disk(rng, n_ant, radius_m, z_sigma=0.1):
    r = radius_m * np.sqrt(rng.random(n_ant))
    th = 2 * np.pi * rng.random(n_ant)
    return np.stack([r * np.cos(th), r * np.sin(th), rng.normal(0.0, z_sigma, n_ant)], 1)


def layout_log_radial(rng, n_ant, radius_m, r_min=10.0, z_sigma=0.1):
    r = r_min * np.exp(rng.random(n_ant) * math.log(radius_m / r_min))
    th = 2 * np.pi * rng.random(n_ant)
    return np.stack([r * np.cos(th), r * np.sin(th), rng.normal(0.0, z_sigma, n_ant)], 1)


def layout_substations(rng, n_ant, n_stations, station_radius_m=17.5, spread_m=3000.0):
    per = n_ant // n_stations
    centres = layout_uniform_disk(rng, n_stations, spread_m, 0.0)
    out = []
    for s in range(n_stations):
        k = per if s < n_stations - 1 else n_ant - per * (n_stations - 1)
        out.append(layout_uniform_disk(rng, k, station_radius_m) + centres[s] * [1, 1, 0])
    return np.concatenate(out, 0)


# ------------------------------------------------------------------------------------------
# UVW: zenith phase centre at interval 0, Earth rotation over the intervals
# (Thompson, Moran & Swenson, eq. 4.1, with local ENU -> equatorial XYZ)
# ------------------------------------------------------------------------------------------
def antenna_uvw(enu, hour_angle_rad, lat_rad):
    e, n, up = enu[:, 0], enu[:, 1], enu[:, 2]
    X = -math.sin(lat_rad) * n + math.cos(lat_rad) * up
    Y = e
    Z = math.cos(lat_rad) * n + math.sin(lat_rad) * up
    h, d = hour_angle_rad, lat_rad
    u = math.sin(h) * X + math.cos(h) * Y
    v = -math.sin(d) * math.cos(h) * X + math.sin(d) * math.sin(h) * Y + math.cos(d) * Z
    w = math.cos(d) * math.cos(h) * X - math.cos(d) * math.sin(h) * Y + math.sin(d) * Z
    return np.stack([u, v, w], 1)


def baseline_uvw(enu, n_sets, cadence_s=1.0, lat_deg=MWA_LATITUDE_DEG):
    """float64 [n_sets][B][3]: baseline = antenna a2 minus antenna a1 (u = -(x_a1 - x_a2))."""
    n_ant = len(enu)
    a1, a2 = baseline_antennas(n_ant)
    out = np.empty((n_sets, n_baselines(n_ant), 3))
    for t in range(n_sets):
        au = antenna_uvw(enu, SIDEREAL_RATE * cadence_s * t, math.radians(lat_deg))
        out[t] = au[a2] - au[a1]
    return out


# ------------------------------------------------------------------------------------------
# sky and visibilities
# ------------------------------------------------------------------------------------------
def point_sources(rng, n_src, s_min=0.1, s_max=100.0, alpha=-2.0):
    """Fluxes from p(S) ~ S^alpha on [s_min, s_max]; directions uniform over the hemisphere."""
    a1 = alpha + 1.0
    s = (s_min ** a1 + rng.random(n_src) * (s_max ** a1 - s_min ** a1)) ** (1.0 / a1)
    n = rng.random(n_src)  # cos(zenith angle) uniform = uniform in solid angle
    phi = 2 * np.pi * rng.random(n_src)
    sin_t = np.sqrt(1 - n * n)
    return s, sin_t * np.cos(phi), sin_t * np.sin(phi), n


def _model_vis(uvw, freqs, flux, l, m, n, device, fast=False):
    """Sum over sources of S*exp(-2*pi*i*(u*l + v*m + w*(n-1))/lambda): complex128 [T][C][B].
    fast: the phase is reduced to a fractional turn in FP64 and the exponential and the sum run
    in FP32 (for large blocks; the result is input data, not a reference)."""
    import torch
    dev = torch.device(device)
    uvw_t = torch.as_tensor(uvw, dtype=torch.float64, device=dev)          # [T][B][3]
    inv_lam = torch.as_tensor(freqs / VEL_LIGHT, dtype=torch.float64, device=dev)  # [C]
    T, B = uvw_t.shape[:2]
    out = torch.zeros((T, len(freqs), B), dtype=torch.complex128, device=dev)
    lmn = torch.as_tensor(np.stack([l, m, n - 1.0], 1), dtype=torch.float64, device=dev)
    s = torch.as_tensor(flux, dtype=torch.float64, device=dev)
    delay = uvw_t @ lmn.T                                                   # [T][B][S] metres
    if fast:
        s32 = s.to(torch.float32)
        for c in range(len(freqs)):
            turns = inv_lam[c] * delay
            frac = (turns - torch.round(turns)).to(torch.float32)           # [T][B][S]
            ph = (-2 * math.pi) * frac
            out[:, c, :] = torch.complex(torch.cos(ph) @ s32, torch.sin(ph) @ s32).to(torch.complex128)
        return out
    for c in range(len(freqs)):
        ph = (-2 * math.pi) * inv_lam[c] * delay                            # [T][B][S]
        out[:, c, :] = torch.sum(s * torch.exp(1j * ph), dim=-1)
    return out


def make_observation(seed, n_ant, enu, n_intervals, freqs, n_pixels, n_src=50, noise_sigma=1.0,
                     per_interval_uvw=True, flagged_ants=(), cadence_s=1.0, device="cpu",
                     cable_max_m=200.0, pol="XX", fast=False, diffuse=None, keep_device=False) -> Observation:
    """diffuse = (amp_jy, beta): a diffuse background whose visibilities are complex Gaussian with
    rms amp * (1 + |uv|/10 wavelengths)^(-beta/2) (a power-law sky), the same in XX and YY.
    keep_device: the visibilities stay a complex64 torch tensor on `device`."""
    import torch
    rng = np.random.Generator(np.random.PCG64(seed))
    freqs = np.asarray(freqs, np.float64)
    n_sets = n_intervals if per_interval_uvw else 1
    uvw = baseline_uvw(enu, n_sets, cadence_s)
    uvw32 = uvw.astype(np.float32)
    flux, l, m, n = point_sources(rng, n_src)
    cable = rng.uniform(0.0, cable_max_m, n_ant)
    B = n_baselines(n_ant)
    T, Cn = n_intervals, len(freqs)
    uvw_full = uvw32.astype(np.float64)
    if n_sets == 1 and T > 1:
        uvw_full = np.ascontiguousarray(np.broadcast_to(uvw_full, (T,) + uvw_full.shape[1:]))
    model = _model_vis(uvw_full, freqs, flux, l, m, n, device, fast=fast)  # [T][C][B]
    dev = model.device
    g = torch.Generator(device="cpu").manual_seed(seed)
    sig = noise_sigma / math.sqrt(2.0)

    gd = torch.Generator(device=dev).manual_seed(seed) if fast else None  # large blocks: draw on the device

    def noise():
        if gd is not None:
            re = torch.randn((T, Cn, B), generator=gd, dtype=torch.float32, device=dev)
            im = torch.randn((T, Cn, B), generator=gd, dtype=torch.float32, device=dev)
        else:
            re = torch.randn((T, Cn, B), generator=g, dtype=torch.float32).to(dev)
            im = torch.randn((T, Cn, B), generator=g, dtype=torch.float32).to(dev)
        return torch.complex(re, im).to(torch.complex128) * sig

    if diffuse is not None:
        amp, beta = diffuse
        uv = torch.as_tensor(np.hypot(uvw_full[..., 0], uvw_full[..., 1]), dtype=torch.float64, device=dev)  # [T][B]
        uv_lam = uv[:, None, :] * torch.as_tensor(freqs / VEL_LIGHT, dtype=torch.float64, device=dev)[None, :, None]
        model = model + noise() * (amp / sig if sig else amp) * (1.0 + uv_lam / 10.0) ** (-beta / 2.0)
    vis = torch.empty((T, Cn, B, 4), dtype=torch.complex128, device=dev)
    vis[..., 0] = model + noise()
    vis[..., 1] = noise()
    vis[..., 2] = noise()
    vis[..., 3] = model + noise()
    # undo the corrections: geometric +2*pi*w*nu/c, cable -2*pi*(L[a2]-L[a1])*nu/c
    a1, a2 = baseline_antennas(n_ant)
    dl = torch.as_tensor(cable[a2] - cable[a1], dtype=torch.float64, device=dev)       # [B]
    w = torch.as_tensor(uvw_full[..., 2], dtype=torch.float64, device=dev)            # [T][B]
    f = torch.as_tensor(freqs / VEL_LIGHT, dtype=torch.float64, device=dev)           # [C]
    phase = 2 * math.pi * (w[:, None, :] - dl[None, None, :]) * f[None, :, None]      # [T][C][B]
    vis = vis * torch.exp(-1j * phase)[..., None]
    del phase, model
    vis = vis.to(torch.complex64)
    if not keep_device:
        vis = vis.cpu().numpy()
    flags = np.zeros(B, np.int32)
    for b, (i, j) in enumerate(zip(a1, a2)):
        if i == j or i in flagged_ants or j in flagged_ants:
            flags[b] = 1
    return Observation(vis=vis, u=np.ascontiguousarray(uvw32[..., 0]),
                       v=np.ascontiguousarray(uvw32[..., 1]), w=np.ascontiguousarray(uvw32[..., 2]),
                       cable=cable, flags=flags, freqs=freqs, n_pixels=n_pixels, pol=pol, enu=enu)


# ------------------------------------------------------------------------------------------
# the measured workloads (seed = 1234 + workload number)
# ------------------------------------------------------------------------------------------
def config1(device="cpu") -> Observation:
    """256 antennas in a 35 m disk, 1 channel at 159.375 MHz, 1 interval, 256x256."""
    rng = np.random.Generator(np.random.PCG64(1235))
    enu = layout_uniform_disk(rng, 256, 35.0)
    return make_observation(1235, 256, enu, 1, [159.375e6], 256, device=device)


def config2_freqs():
    return 150e6 + np.arange(64) * (30e6 / 64)


def config2(device="cpu", n_intervals=10, n_channels=64) -> Observation:
    """Same 256-antenna array, 64 channels over 150-180 MHz x 10 intervals of 1 s, 512x512."""
    rng = np.random.Generator(np.random.PCG64(1236))
    enu = layout_uniform_disk(rng, 256, 35.0)
    freqs = config2_freqs()[:n_channels]
    return make_observation(1236, 256, enu, n_intervals, freqs, 512, device=device)


def precision_form(device="cuda", n_intervals=20, n_channels=768, keep_device=True) -> Observation:
    """128 antennas in a 3 km disk with log-radial density, 768 channels of 10 kHz from 150 MHz x
    20 intervals of 1 s, 1024x1024 images (15,360 per block; seed 1237).  The visibilities
    (4 GB) stay on the device unless keep_device is False."""
    rng = np.random.Generator(np.random.PCG64(1237))
    enu = layout_log_radial(rng, 128, 1500.0)
    freqs = 150e6 + 10e3 * np.arange(n_channels)
    return make_observation(1237, 128, enu, n_intervals, freqs, 1024, device=device, fast=True,
                            keep_device=keep_device)


def small(seed=7, n_ant=24, n_intervals=2, n_channels=3, n_pixels=64, radius=35.0,
          per_interval_uvw=True, flagged_ants=(3,), n_src=10, pol="XX", f0=150e6,
          df=1.28e6, device="cpu") -> Observation:
    """A small block for parity tests."""
    rng = np.random.Generator(np.random.PCG64(seed))
    enu = layout_uniform_disk(rng, n_ant, radius)
    freqs = f0 + df * np.arange(n_channels)
    return make_observation(seed, n_ant, enu, n_intervals, freqs, n_pixels, n_src=n_src,
                            per_interval_uvw=per_interval_uvw, flagged_ants=flagged_ants,
                            pol=pol, device=device)


def serving_arrays(device="cpu", n_channels=32):
    """The serving workload's arrays, one 1-interval block of `n_channels` channels each:
    128 antennas in a 35 m disk imaged at 256x256, 256 antennas in a 35 m disk at 512x512 and
    512 antennas in 16 clustered sub-stations over 3 km at 1024x1024 (seed 1239)."""
    freqs = 150e6 + np.arange(n_channels) * 0.9375e6
    out = []
    for k, (n_ant, n_pix) in enumerate(((128, 256), (256, 512), (512, 1024))):
        rng = np.random.Generator(np.random.PCG64(1239 + k))
        enu = layout_substations(rng, n_ant, 16) if n_ant == 512 else layout_uniform_disk(rng, n_ant, 35.0)
        out.append(make_observation(1239 + k, n_ant, enu, 1, freqs, n_pix, device=device))
    return out



def batched_bands(device="cpu", n_intervals=5, n_channels=64):
    """The uneven batch workload: 512 antennas in 16 clustered sub-stations over 3 km, 256 channels
    over 100-200 MHz in four bands of 64 imaged at 256, 512, 1024 and 2048 pixels, 5 intervals,
    400 point sources and a diffuse power-law background (seed 1238).  One Observation per band
    (the same array).  n_channels < 64 keeps the first channels of each band (a slice of the
    workload with its array, image sides and sky)."""
    rng = np.random.Generator(np.random.PCG64(1238))
    enu = layout_substations(rng, 512, 16)
    freqs = 100e6 + np.arange(256) * (100e6 / 256)
    return [make_observation(1238 + k, 512, enu, n_intervals, freqs[64 * k:64 * k + n_channels], 256 << k,
                             n_src=400, device=device, fast=True, diffuse=(10.0, 2.0)) for k in range(4)]
