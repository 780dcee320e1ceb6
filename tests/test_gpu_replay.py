"""Replay of repeated calls (a repeated bgi_image* call launches the CUDA graph recorded from
it): the replayed calls give the images of the calls they repeat -- bit for bit with the
ordered gridder, within FP32 summation order with the atomic one -- follow new contents of
the same buffers, and stop replaying when the handle's state or the call changes."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    from imager_gb300 import imager
    return imager


def _imager(im, obs, n, pol="XX", wave=0):
    h = im.Imager(n, 2.0, pol, -1000.0, max_images_per_wave=wave)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    return h


def _bits(t):
    return np.ascontiguousarray(t.cpu().numpy()).view(np.uint32)


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_replay_same_bits_and_new_contents(im):
    """Ordered gridder (exact sums): the recorded graph gives the eager call's bits, reads the
    buffers' current contents, and writes the weight sums."""
    obs = synth.small(seed=101, n_ant=48, n_intervals=2, n_channels=3, n_pixels=128)
    vis = torch.from_numpy(obs.vis_f32()).cuda()
    h = _imager(im, obs, 128, wave=2)
    h.set_deterministic(True)
    out = torch.empty((2, 3, 128, 128), dtype=torch.complex64, device="cuda")
    h.image(vis, out=out)
    first = _bits(out)
    assert not h.replay_ready
    h.image(vis, out=out)          # the repeat: run, then recorded
    assert h.replay_ready
    assert np.array_equal(_bits(out), first)
    sums = h.weight_sums(6)
    out.zero_()
    h.image(vis, out=out)          # launched from the graph
    assert h.replay_ready
    assert np.array_equal(_bits(out), first)
    assert np.array_equal(h.weight_sums(6), sums)
    # new contents in the same buffer: the graph reads them
    vis2 = torch.from_numpy(synth.small(seed=102, n_ant=48, n_intervals=2, n_channels=3,
                                        n_pixels=128).vis_f32()).cuda()
    vis.copy_(vis2)
    h.image(vis, out=out)
    assert h.replay_ready
    fresh = _imager(im, obs, 128, wave=2)
    fresh.set_deterministic(True)
    ref = torch.empty_like(out)
    fresh.image(vis2, out=ref)
    assert np.array_equal(_bits(out), _bits(ref))
    fresh.close()
    h.close()


@pytest.mark.parametrize("change", ["frequencies", "schedule", "aggregation", "images_per_thread", "fft_mode",
                                    "column_radix", "deterministic"])
def test_replay_dropped_by_setters(im, change):
    """A setter between two identical calls drops the graph: the next call runs with the new
    state (compared with a fresh handle in that state)."""
    n = 512
    obs = synth.small(seed=103, n_ant=40, n_intervals=1, n_channels=4, n_pixels=n)
    vis = torch.from_numpy(obs.vis_f32()).cuda()
    h = _imager(im, obs, n, wave=2)
    out = torch.empty((1, 4, n, n), dtype=torch.complex64, device="cuda")
    for _ in range(3):
        h.image(vis, out=out)
    assert h.replay_ready
    freqs = obs.freqs
    fresh = _imager(im, obs, n, wave=2)

    def apply(x):
        if change == "frequencies":
            x.set_frequencies(freqs * 1.05)
        elif change == "schedule":
            x.set_schedule(1, 3)
        elif change == "aggregation":
            x.set_gridding_images_per_thread(4)
            x.set_gridding_aggregation(True)
        elif change == "images_per_thread":
            x.set_gridding_images_per_thread(8)
        elif change == "fft_mode":
            x.set_fft_mode("tensor_split16")
        elif change == "column_radix":
            x.set_column_radix(16)
        else:
            x.set_deterministic(True)

    apply(h)
    assert not h.replay_ready
    apply(fresh)
    ref = torch.empty_like(out)
    fresh.image(vis, out=ref)
    for _ in range(3):  # eager, eager + recorded, replayed
        out.zero_()
        h.image(vis, out=out)
        got = out.cpu().numpy()
        for j in range(4):
            assert rel_l2(got[0, j], ref[0, j].cpu().numpy()) < 2e-6, (change, j)
    assert h.replay_ready
    fresh.close()
    h.close()


def test_replay_alternating_calls_and_batches(im):
    """Calls that alternate between two outputs never replay a stale graph; a batch built on
    the handle afterwards, and calls after it, image correctly."""
    n = 256
    obs = synth.small(seed=104, n_ant=40, n_intervals=1, n_channels=3, n_pixels=n)
    vis = torch.from_numpy(obs.vis_f32()).cuda()
    h = _imager(im, obs, n)
    a = torch.empty((1, 3, n, n), dtype=torch.complex64, device="cuda")
    b = torch.empty_like(a)
    h.image(vis, out=a)
    ref = a.cpu().numpy()
    for _ in range(3):
        a.zero_()
        b.zero_()
        h.image(vis, out=a)
        h.image(vis, out=b)
        assert not h.replay_ready
        for j in range(3):
            assert rel_l2(a.cpu().numpy()[0, j], ref[0, j]) < 2e-6
            assert rel_l2(b.cpu().numpy()[0, j], ref[0, j]) < 2e-6
    for _ in range(3):
        h.image(vis, out=a)
    assert h.replay_ready
    c = torch.empty((1, 3, n, n), dtype=torch.complex64, device="cuda")
    batch = im.Batch([dict(imager=h, data=vis, fmt="c64", out=c)])
    assert not h.replay_ready
    batch.launch()
    torch.cuda.synchronize()
    for j in range(3):
        assert rel_l2(c.cpu().numpy()[0, j], ref[0, j]) < 2e-6
    batch.close()
    for _ in range(3):
        a.zero_()
        h.image(vis, out=a)
        for j in range(3):
            assert rel_l2(a.cpu().numpy()[0, j], ref[0, j]) < 2e-6
    h.close()


def test_replay_host_buffers(im):
    """The host-buffer call: page-locked buffers replay (the graph reads the host buffer's
    current contents); pageable ones run eagerly every time; both give the device call's
    images."""
    n = 256
    obs = synth.small(seed=105, n_ant=40, n_intervals=2, n_channels=3, n_pixels=n)
    vis_np = np.ascontiguousarray(obs.vis_f32())
    h = _imager(im, obs, n, wave=2)
    ref = torch.empty((2, 3, n, n), dtype=torch.complex64, device="cuda")
    h.image(torch.from_numpy(vis_np).cuda(), out=ref)
    ref = ref.cpu().numpy()
    pinned_in = torch.from_numpy(vis_np.copy()).pin_memory()
    pinned_out = torch.empty((2, 3, n, n), dtype=torch.complex64).pin_memory()
    for k in range(4):
        pinned_out.zero_()
        h.image_host(pinned_in, out=pinned_out)
        got = pinned_out.numpy()
        for i in range(2):
            for j in range(3):
                assert rel_l2(got[i, j], ref[i, j]) < 2e-6, (k, i, j)
    assert h.replay_ready
    # new contents of the page-locked input, replayed
    obs2 = synth.small(seed=106, n_ant=40, n_intervals=2, n_channels=3, n_pixels=n)
    vis2 = np.ascontiguousarray(obs2.vis_f32())
    pinned_in.copy_(torch.from_numpy(vis2))
    h.image_host(pinned_in, out=pinned_out)
    assert h.replay_ready
    ref2 = torch.empty((2, 3, n, n), dtype=torch.complex64, device="cuda")
    h.image(torch.from_numpy(vis2).cuda(), out=ref2)
    ref2 = ref2.cpu().numpy()
    for i in range(2):
        for j in range(3):
            assert rel_l2(pinned_out.numpy()[i, j], ref2[i, j]) < 2e-6
    # pageable buffers: never recorded, same images
    for _ in range(3):
        got = h.image_host(vis2)
        assert not h.replay_ready
        for i in range(2):
            for j in range(3):
                assert rel_l2(got[i, j], ref2[i, j]) < 2e-6
    h.close()


def test_replay_off(im):
    """bgi_set_replay(0): repeated calls issue their work every time, with the same images."""
    n = 128
    obs = synth.small(seed=107, n_ant=32, n_intervals=1, n_channels=3, n_pixels=n)
    vis = torch.from_numpy(obs.vis_f32()).cuda()
    h = _imager(im, obs, n)
    h.set_deterministic(True)
    out = torch.empty((1, 3, n, n), dtype=torch.complex64, device="cuda")
    h.image(vis, out=out)
    ref = _bits(out)
    h.set_replay(False)
    for _ in range(3):
        out.zero_()
        h.image(vis, out=out)
        assert not h.replay_ready
        assert np.array_equal(_bits(out), ref)
    h.set_replay(True)
    for _ in range(3):
        h.image(vis, out=out)
    assert h.replay_ready and np.array_equal(_bits(out), ref)
    h.close()


@pytest.mark.parametrize("path", ["compressed_host", "matrices_host"])
def test_replay_stored_and_matrix_host_calls(im, path):
    """The 16-bit host call and the correlation-matrix host call with page-locked buffers:
    recorded on the second call and replayed after it (ingest, uploads and downloads in the
    graph), the same bits as the first, direct call (ordered gridder)."""
    n = 128
    obs = synth.small(seed=108, n_ant=32, n_intervals=2, n_channels=3, n_pixels=n)
    h = _imager(im, obs, n, pol="I", wave=2)
    h.set_deterministic(True)
    out = torch.empty((2, 3, n, n), dtype=torch.complex64).pin_memory()
    if path == "compressed_host":
        d, sc = im.compress_visibilities(torch.from_numpy(obs.vis_f32()).cuda(), "s16")
        args = (d.cpu().pin_memory(), sc.cpu().pin_memory())

        def call():
            return h.image_compressed_host(*args, "s16", out=out)
    else:
        na, B = 32, obs.vis.shape[2]
        i, j = np.tril_indices(na)
        mats = []
        for p in (0, 3):
            full = np.zeros((2, 3, na, na), np.complex64)
            full[:, :, i, j] = obs.vis[:, :, np.arange(B), p]
            mats += [torch.from_numpy(np.ascontiguousarray(full.real)).pin_memory(),
                     torch.from_numpy(np.ascontiguousarray(full.imag)).pin_memory()]

        def call():
            return h.image_matrices_host(*mats, fmt="s16", out=out)
    call()
    first = np.ascontiguousarray(out.numpy()).view(np.uint32).copy()
    assert not h.replay_ready
    for k in range(3):
        out.zero_()
        call()
        assert h.replay_ready  # recorded by the first repeat, launched by the others
        assert np.array_equal(np.ascontiguousarray(out.numpy()).view(np.uint32), first), k
    h.close()
