"""Sharding one observation over ranks (imager_gb300/shard.py): world_size-2 gloo processes
on the CPU each image their shard with the oracle, using the whole observation's uv cell, and
the gathered images equal the unsharded ones exactly."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from imager_gb300 import shard as S
from imager_gb300 import synth


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _oracle_images(O, vis_c, u, v, w, cable, flags, freqs, n, du, dv, n_sets):
    vis = np.ascontiguousarray(vis_c.view(np.float32).reshape(vis_c.shape + (2,))).copy()
    O.apply_geometric(vis, w, freqs, n_uvw_sets=n_sets)
    O.apply_cable(vis, cable, freqs)
    g, c, _ = O.gridding(vis, u, v, flags, freqs, du, dv, n, n_uvw_sets=n_sets)
    return O.image_f64(g, c)


def _case(n_intervals, n_channels):
    return synth.small(seed=55, n_ant=16, n_intervals=n_intervals, n_channels=n_channels, n_pixels=32)


def _worker(rank, world, port, n_intervals, n_channels, out_q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O
        obs = _case(n_intervals, n_channels)
        umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
        du, dv = O.delta_uv(2.0, umax, 32), O.delta_uv(2.0, vmax, 32)
        sh = S.plan_shard(n_intervals, n_channels, world, rank)
        vis, u, v, w, freqs = S.shard_inputs(obs, sh)
        img = _oracle_images(O, vis, u, v, w, obs.cable, obs.flags, freqs, 32, du, dv, u.shape[0])
        parts = [None] * world
        dist.all_gather_object(parts, (sh, img))
        if rank == 0:
            full = S.assemble([p[1] for p in parts], [p[0] for p in parts], n_intervals, n_channels, 32)
            ref = _oracle_images(O, obs.vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 32,
                                 du, dv, obs.u.shape[0])
            out_q.put(bool(np.array_equal(full, ref)) and all(p[0].n_images > 0 for p in parts))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("n_intervals,n_channels", [(4, 3), (1, 5)])
def test_two_rank_shards_equal_unsharded(n_intervals, n_channels):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_intervals, n_channels, q)) for r in range(2)]
    for p in procs:
        p.start()
    result = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert result


def test_plan_covers_every_image_once():
    for T, C in ((10, 64), (3, 8), (1, 7), (5, 1)):
        for world in (1, 2, 3, 4, 8):
            seen = np.zeros((T, C), int)
            for r in range(world):
                s = S.plan_shard(T, C, world, r)
                seen[s.t0:s.t1, s.c0:s.c1] += 1
            assert np.all(seen == 1), (T, C, world)
    with pytest.raises(ValueError):
        S.plan_shard(4, 4, 2, 2)
