"""bgi_image_noalloc: imaging with scratch the library holds statically, for callers that
cannot allocate device memory while they run (a pipeline that budgets all GPU memory up front,
a framework that owns the allocator, or code that must not let cudaMalloc synchronise a live
device).  Its images must match the allocating entry point (bgi_image with no corrections) to
the tolerance the other image tests use, on two calls in a row: the second call finds the
scratch as the first left it and must still start from a clean grid.

This file is collected last so that a run stopping at its first failure has run every other
test first."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu
IMAGE_TOL = 1e-4  # relative L2 per image, as the other image tests


def _rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_no_alloc_matches_image_on_two_calls():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from imager_gb300 import capi, synth
    from imager_gb300.imager import Imager

    lib = capi.lib(build_if_missing=True)
    n = 512
    # 3 intervals x 8 channels = 24 images of 512^2: more than the 16 one scratch wave holds
    obs = synth.small(seed=77, n_ant=48, n_intervals=3, n_channels=8, n_pixels=n)
    vis = torch.from_numpy(np.ascontiguousarray(obs.vis_f32())).cuda()
    u = torch.from_numpy(obs.u).cuda()
    v = torch.from_numpy(obs.v).cuda()
    flags = torch.from_numpy(obs.flags).cuda()
    freqs = torch.from_numpy(obs.freqs).cuda()
    T, Cn = 3, 8

    h = Imager(n, 2.0, "XX", -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    ref = h.image(vis, flags=0).cpu().numpy()
    du, dv = h.uv_cell[:2]
    h.close()

    # the oracle of the same block (no corrections), for a check that does not go through the
    # allocating entry point
    from oracle import oracle as O
    vis_np = np.ascontiguousarray(obs.vis_f32())
    grids, counters, _ = O.gridding(vis_np, obs.u, obs.v, obs.flags, obs.freqs, du, dv, n, n_uvw_sets=T)
    oracle_images = O.image_f64(grids, counters)

    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = [torch.full((T, Cn, n, n), float("nan"), dtype=torch.complex64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    free_after_first = None
    for call in range(2):
        out = outs[call]
        st = lib.bgi_image_noalloc(C.c_void_p(vis.data_ptr()), obs.n_ant, Cn, T, C.c_void_p(u.data_ptr()),
                                   C.c_void_p(v.data_ptr()), T, C.c_void_p(flags.data_ptr()),
                                   C.c_void_p(freqs.data_ptr()), du, dv, n, -1000.0, capi.POL["XX"],
                                   C.c_void_p(out.data_ptr()), stream)
        assert st == capi.OK, lib.bgi_last_error()
        torch.cuda.synchronize()
        # driver-level free memory: the first call may load the library's modules (and so commit
        # the static scratch); the second call must take no device memory at all
        free_now = torch.cuda.mem_get_info()[0]
        if call == 0:
            free_after_first = free_now
        else:
            assert free_now == free_after_first, (free_after_first, free_now)
        got = out.cpu().numpy()
        assert np.isfinite(got).all(), call
        for i in range(T):
            for j in range(Cn):
                assert _rel_l2(got[i, j], ref[i, j]) < IMAGE_TOL, (call, i, j)
                assert _rel_l2(got[i, j], oracle_images[i, j]) < IMAGE_TOL, (call, i, j)


def test_no_alloc_rejects_grid_beyond_scratch():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from imager_gb300 import capi

    lib = capi.lib(build_if_missing=True)
    buf = torch.zeros(64, dtype=torch.float32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    st = lib.bgi_image_noalloc(p, 4, 1, 1, p, p, 1, p, p, 1.0, 1.0, 4096, -1.0, 0, p, None)
    assert st == capi.ERR_UNSUPPORTED
    assert b"MiB" in lib.bgi_last_error()
