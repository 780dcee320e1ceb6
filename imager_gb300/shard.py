"""Splitting one observation block over several GPUs (one process per GPU).

Every (interval, channel) image is independent once the array state is resident, so a block
shards with no collective on the data path: a rank images a contiguous range of intervals (its
UVW sets and all channels) or, when there are fewer intervals than ranks, a contiguous range of
channels for all intervals.  Only gathering the images, if the caller wants them in one place,
needs communication.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Shard:
    t0: int
    t1: int
    c0: int
    c1: int

    @property
    def n_images(self) -> int:
        return max(0, self.t1 - self.t0) * max(0, self.c1 - self.c0)


def _split(n: int, world: int, rank: int):
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def plan_shard(n_intervals: int, n_channels: int, world: int, rank: int) -> Shard:
    """Contiguous share of rank `rank` among `world` ranks: by intervals when there are at least
    as many intervals as ranks, otherwise by channels."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    if n_intervals >= world:
        t0, t1 = _split(n_intervals, world, rank)
        return Shard(t0, t1, 0, n_channels)
    c0, c1 = _split(n_channels, world, rank)
    return Shard(0, n_intervals, c0, c1)


def shard_inputs(obs, shard: Shard):
    """The visibilities, UVW sets and frequencies of one shard of an observation
    (imager_gb300.synth.Observation-like: vis [T][C][B][4], u/v/w [sets][B], freqs [C])."""
    vis = np.ascontiguousarray(obs.vis[shard.t0:shard.t1, shard.c0:shard.c1])
    if obs.u.shape[0] > 1:
        u, v, w = (np.ascontiguousarray(a[shard.t0:shard.t1]) for a in (obs.u, obs.v, obs.w))
    else:
        u, v, w = obs.u, obs.v, obs.w
    return vis, u, v, w, np.ascontiguousarray(obs.freqs[shard.c0:shard.c1])


def assemble(parts, shards, n_intervals: int, n_channels: int, n_pixels: int):
    """Images of all shards (each [t1-t0][c1-c0][N][N]) into one [T][C][N][N] array."""
    out = np.zeros((n_intervals, n_channels, n_pixels, n_pixels), parts[0].dtype)
    for img, s in zip(parts, shards):
        out[s.t0:s.t1, s.c0:s.c1] = img
    return out


def shard_observation(obs, world: int, rank: int):
    """(shard, the observation restricted to it): rank `rank`'s share of `obs` as an Observation
    of its own (visibilities, UVW sets and frequencies of the shard; array, flags and cable
    lengths unchanged).  The rank images it with the whole observation's uv cell
    (Imager.set_uv_cell), so its images are the whole observation's images of that share."""
    sh = plan_shard(obs.n_intervals, obs.n_channels, world, rank)
    vis, u, v, w, freqs = shard_inputs(obs, sh)
    return sh, dataclasses.replace(obs, vis=vis, u=u, v=v, w=w, freqs=freqs)
