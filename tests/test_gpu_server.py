"""Serving runtime (bgi_server_*): requests of several arrays, sizes and storage formats
submitted together overlap on the GPU, and each request's images are the same as when it runs
alone (bit for bit with the ordered gridder, to summation order otherwise) and as the imager
handle's; admission waits for memory under a small budget; faults injected on the host -- a
request larger than the budget, malformed blocks, a full queue, a cancelled request -- fail
cleanly while the server keeps serving; latency statistics are reported."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    from imager_gb300 import imager, server
    return imager, server


def _arrays():
    a = synth.small(seed=71, n_ant=40, n_intervals=2, n_channels=3, n_pixels=128)
    b = synth.small(seed=72, n_ant=64, n_intervals=1, n_channels=2, n_pixels=256)
    c = synth.small(seed=73, n_ant=24, n_intervals=3, n_channels=4, n_pixels=64)
    return [(a, "XX"), (b, "I"), (c, "V")]


def _register(sv, arrays):
    return [sv.add_array(o.n_pixels, o.u, o.v, o.w, o.flags, o.cable, o.freqs, pol=pol) for o, pol in arrays]


def _handle_images(imager, obs, pol, deterministic):
    h = imager.Imager(obs.n_pixels, 2.0, pol)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    h.set_deterministic(deterministic)
    out = h.image(torch.from_numpy(obs.vis_f32()).cuda()).cpu().numpy()
    h.close()
    return out


def _rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("deterministic", [True, False])
def test_alone_and_in_the_mix(mods, deterministic):
    imager, server = mods
    arrays = _arrays()
    with server.Server(max_slots=3, deterministic=deterministic) as sv:
        ids = _register(sv, arrays)
        vis = [o.vis_f32() for o, _ in arrays]
        alone = [sv.wait(sv.submit(i, v)).numpy().copy() for i, v in zip(ids, vis)]
        # the mix: every array several times, 16-bit stored blocks among them, all queued at once
        stored = [imager.compress_visibilities(torch.from_numpy(v).cuda(), "s16") for v in vis]
        stored = [(d.cpu().numpy(), s.cpu().numpy()) for d, s in stored]
        tickets = []
        for rep in range(3):
            for k, i in enumerate(ids):
                tickets.append((k, "c64", sv.submit(i, vis[k])))
                tickets.append((k, "s16", sv.submit(i, data=stored[k][0], scales=stored[k][1], fmt="s16")))
        s16_first = {}
        for k, fmt, t in tickets:
            out = sv.wait(t).numpy()
            if fmt == "c64":
                if deterministic:
                    assert np.array_equal(out.view(np.uint32), alone[k].view(np.uint32)), k
                else:
                    assert _rel(out, alone[k]) < 1e-6, k
            else:
                assert _rel(out, alone[k]) < 1e-4, k  # 16-bit storage against complex64
                if k in s16_first and deterministic:
                    assert np.array_equal(out.view(np.uint32), s16_first[k].view(np.uint32)), k
                s16_first.setdefault(k, out.copy())
        st = sv.stats()
        assert st["completed"] == st["submitted"] == 3 + len(tickets) and st["failed"] == 0
        assert st["images"] == sum(v.shape[0] * v.shape[1] for v in vis) * 7
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"] and st["images_per_s"] > 0
    for k, (o, pol) in enumerate(arrays):  # the server's images are the handle's
        ref = _handle_images(imager, o, pol, deterministic)
        assert _rel(alone[k], ref) < (1e-7 if deterministic else 1e-6), k


def test_admission_waits_for_memory(mods):
    imager, server = mods
    obs = synth.small(seed=74, n_ant=48, n_intervals=2, n_channels=4, n_pixels=256)
    vis = obs.vis_f32()
    req_bytes = vis.nbytes + 2 * 4 * 256 * 256 * 8
    with server.Server(max_slots=4, hbm_budget_bytes=int(req_bytes * 1.5), deterministic=True) as sv:
        aid = sv.add_array(256, obs.u, obs.v, obs.w, obs.flags, obs.cable, obs.freqs)
        outs = [sv.wait(t).numpy() for t in [sv.submit(aid, vis) for _ in range(6)]]
        st = sv.stats()
        assert st["admission_waits"] >= 1 and st["completed"] == 6 and st["failed"] == 0
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint32), outs[0].view(np.uint32))


def test_request_larger_than_budget_fails(mods):
    imager, server = mods
    obs = synth.small(seed=75, n_ant=16, n_intervals=1, n_channels=2, n_pixels=64)
    with server.Server(max_slots=2, hbm_budget_bytes=1024) as sv:
        aid = sv.add_array(64, obs.u, obs.v, obs.w, obs.flags, obs.cable, obs.freqs)
        t = sv.submit(aid, obs.vis_f32())
        with pytest.raises(capi.BgiError) as e:
            sv.wait(t)
        assert e.value.status == capi.ERR_ALLOC
        assert sv.stats()["failed"] == 1
        with pytest.raises(capi.BgiError):
            sv.submit(aid + 5, obs.vis_f32())  # unknown array
        import ctypes as C
        buf = np.zeros(16, np.float32)
        ticket = C.c_uint64(0)
        st = capi.lib().bgi_server_submit(sv._h, aid + 5, 0, buf.ctypes.data, None, 1, 3, buf.ctypes.data,
                                          C.byref(ticket))
        assert st == capi.ERR_INVALID


def test_malformed_blocks_are_refused_at_submission(mods):
    """Faults injected on the host: every malformed submission fails at once with
    BGI_ERR_INVALID and leaves the server serving."""
    import ctypes as C
    imager, server = mods
    obs = synth.small(seed=76, n_ant=16, n_intervals=2, n_channels=2, n_pixels=64)
    with server.Server(max_slots=2) as sv:
        aid = sv.add_array(64, obs.u, obs.v, obs.w, obs.flags, obs.cable, obs.freqs)
        lib, buf, t = capi.lib(), np.zeros(64, np.float32), C.c_uint64(0)
        p = buf.ctypes.data
        bad = [
            (aid, 0, None, None, 2, 3, p),      # no visibilities
            (aid, 0, p, None, 2, 3, None),      # no image buffer
            (aid, 9, p, None, 2, 3, p),         # unknown storage format
            (aid, 1, p, None, 2, 3, p),         # 16-bit storage without scales
            (aid, 0, p, None, 3, 3, p),         # 3 intervals for an array with 2 UVW sets
            (aid, 0, p, None, 0, 3, p),         # no interval
            (aid, 0, p, None, 2, 1 << 9, p),    # unknown flag
        ]
        for a, fmt, vis, sc, T, fl, img in bad:
            assert lib.bgi_server_submit(sv._h, a, fmt, vis, sc, T, fl, img, C.byref(t)) == capi.ERR_INVALID
        out = sv.wait(sv.submit(aid, obs.vis_f32())).numpy()   # still serving
        assert np.isfinite(out).all() and sv.stats()["failed"] == 0


def test_queue_limit_and_cancellation(mods):
    """A full queue refuses submissions with BGI_ERR_BUSY; a request still waiting for
    admission can be cancelled (its wait reports BGI_ERR_CANCELLED) and the others complete with
    the images of the handle."""
    imager, server = mods
    obs = synth.small(seed=77, n_ant=64, n_intervals=1, n_channels=16, n_pixels=1024)
    vis = obs.vis_f32()
    req_bytes = vis.nbytes + 16 * 1024 * 1024 * 8
    # one slot and memory for one request at a time: the others wait in the queue
    with server.Server(max_slots=1, hbm_budget_bytes=int(req_bytes * 1.5), deterministic=True,
                       max_queued=2) as sv:
        aid = sv.add_array(1024, obs.u, obs.v, obs.w, obs.flags, obs.cable, obs.freqs)
        tickets, busy = [], 0
        for _ in range(8):
            try:
                tickets.append(sv.submit(aid, vis))
            except capi.BgiError as e:
                assert e.status == capi.ERR_BUSY
                busy += 1
        assert busy >= 1 and len(tickets) + busy == 8
        assert len(tickets) >= 2                          # the second submission always fits
        assert sv.cancel(tickets[-1])                     # behind at least one request: still queued
        with pytest.raises(capi.BgiError) as e:
            sv.wait(tickets[-1])
        assert e.value.status == capi.ERR_CANCELLED
        outs = [sv.wait(t).numpy() for t in tickets[:-1]]
        st = sv.stats()
        assert st["rejected"] == busy and st["cancelled"] == 1 and st["failed"] == 0
        with pytest.raises(capi.BgiError):
            sv.cancel(tickets[0])                         # already collected
    ref = _handle_images(imager, obs, "XX", True)
    for o in outs:
        assert np.array_equal(o.view(np.uint32), ref.view(np.uint32))
