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


def _library_worker(rank, world, port, out_q):
    """One rank of a sharded observation on the library's host side: its shard (as bench.py's
    sharded run takes it), the whole observation's uv cell, the half-plane extent the library
    computes from that cell (host only, bgi_uv_extent), and the library's argument checks on the
    shard's block, which run before any device work."""
    import ctypes as C
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from imager_gb300 import capi
        from oracle import oracle as O
        lib = capi.lib(build_if_missing=True)
        obs = synth.small(seed=56, n_ant=16, n_intervals=4, n_channels=3, n_pixels=64)
        umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
        du, dv = O.delta_uv(2.0, umax, 64), O.delta_uv(2.0, vmax, 64)
        sh, part = S.shard_observation(obs, world, rank)
        eu, ev = C.c_int(), C.c_int()
        assert lib.bgi_uv_extent(umax, vmax, du, dv, float(obs.freqs.max()), 64, C.byref(eu), C.byref(ev)) == capi.OK
        # the shard's block with a UVW-set count that does not match its intervals is refused
        # before any launch (n_uvw_sets must be 1 or the interval count)
        buf = C.c_void_p(16)
        bad_sets = part.n_intervals + 1
        st = lib.bgi_gridding_gpu(buf, obs.n_ant, part.n_channels, part.n_intervals, buf, buf, bad_sets, buf, None,
                                  buf, du, dv, 64, -1.0, 0, 1, None, buf, None)
        parts = [None] * world
        dist.all_gather_object(parts, (sh, part.vis, part.u, part.freqs, (eu.value, ev.value), st))
        if rank == 0:
            vis = np.zeros_like(obs.vis)
            for s, v, u, f, _, _ in parts:
                vis[s.t0:s.t1, s.c0:s.c1] = v
                assert np.array_equal(u, obs.u[s.t0:s.t1]) and np.array_equal(f, obs.freqs[s.c0:s.c1])
            ok = (np.array_equal(vis, obs.vis) and len({p[4] for p in parts}) == 1
                  and all(p[5] == capi.ERR_INVALID for p in parts) and all(p[0].n_images > 0 for p in parts))
            out_q.put(bool(ok))
    finally:
        dist.destroy_process_group()


def test_two_rank_library_host_side():
    import shutil
    from imager_gb300 import capi
    if shutil.which("nvcc") is None and not os.path.exists(capi.library_path()):
        pytest.skip("nvcc not available to build the library")
    capi.lib(build_if_missing=True)  # build once, before the ranks load it
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_library_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    result = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert result
