"""The workloads the path is measured on, imaged at their full shapes through the C ABI and
checked against the oracle (the FP64 restatement of the reference's CPU path,
src/pacer_imager.cpp:440-526 with src/corrections.cpp):

* the CPU-runnable plain case: 256 antennas in a 35 m disk, one channel at 159.375 MHz, one
  interval, 256 x 256, through bgi_image and bgi_image_host;
* a slice of the precision form (128 antennas in a 3 km log-radial disk, 10 kHz channels,
  1024 x 1024) in every storage format;
* one image per band of the uneven batch (512 antennas in 16 sub-stations, 256^2 to 2048^2).

Tolerances: weight sums (gridded point counts) exact; images within 1e-4 relative L2 of the FP64
oracle for complex64 and 16-bit block floating point storage.  binary16 and bfloat16 storage carry
11 and 8 significant bits per component, so their images are held to the error their rounding
gives (below 5e-4 and 4e-3), not to 1e-4."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
IMAGE_TOL = 1e-4
FORMAT_TOL = {"c64": 1e-5, "s16": IMAGE_TOL, "fp16": 5e-4, "bf16": 4e-3}


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from imager_gb300 import capi, imager
    capi.lib(build_if_missing=True)
    O.build()
    return imager


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _oracle(obs, vis):
    return O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, obs.n_pixels,
                           n_uvw_sets=obs.n_uvw_sets)


def _imager(im, obs):
    h = im.Imager(obs.n_pixels, 2.0, "XX", -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    return h


def test_cpu_runnable_plain_case(im):
    """256 antennas, 159.375 MHz, 256 x 256: the device entry point and the host-buffer entry
    point both match the oracle, and the gridded point count is the oracle's."""
    obs = synth.config1()
    assert obs.n_ant == 256 and obs.vis.shape[:3] == (1, 1, 32896) and obs.n_pixels == 256
    assert np.array_equal(obs.freqs, [159.375e6])
    vis = np.ascontiguousarray(obs.vis_f32())
    _, _, counters, ref, (du, dv) = _oracle(obs, vis)
    h = _imager(im, obs)
    assert h.uv_cell[:2] == (du, dv)
    out = h.image(torch.from_numpy(vis).cuda()).cpu().numpy()
    assert rel_l2(out[0, 0], ref[0, 0]) < IMAGE_TOL
    assert np.array_equal(h.weight_sums(1), counters.reshape(1, -1).sum(1).astype(np.uint32))
    host = h.image_host(vis)
    assert rel_l2(host[0, 0], ref[0, 0]) < IMAGE_TOL
    # the reference's free gridding call on the same (corrected) visibilities: counters exact
    corr, grids_ref, counters_ref, _, _ = _oracle(obs, vis)
    corr = corr.reshape(vis.shape)
    n = obs.n_pixels
    grids = torch.zeros((1, 1, n, n), dtype=torch.complex64, device="cuda")
    cnt = torch.zeros((1, 1, n, n), dtype=torch.float32, device="cuda")
    im.gridding(torch.from_numpy(np.ascontiguousarray(corr)).cuda(), torch.from_numpy(obs.u).cuda(),
                torch.from_numpy(obs.v).cuda(), torch.from_numpy(obs.flags).cuda(),
                torch.from_numpy(obs.freqs).cuda(), du, dv, n, -1000.0, "XX", grids, cnt)
    assert np.array_equal(cnt.cpu().numpy(), counters_ref)
    g = grids.cpu().numpy()
    gr = grids_ref.view(np.complex64)[..., 0]
    assert np.abs(g - gr).max() <= 1e-5 * np.abs(gr).max()
    h.close()


def test_precision_form_slice_every_storage(im):
    """128 antennas in a 3 km log-radial disk, 4 channels of 10 kHz x 2 intervals of 1024 x 1024:
    complex64 records and the three 16-bit formats, each against the FP64 oracle of the
    complex64 visibilities."""
    obs = synth.precision_form(device="cuda", n_intervals=2, n_channels=4, keep_device=False)
    assert obs.n_ant == 128 and obs.n_pixels == 1024
    vis = np.ascontiguousarray(obs.vis_f32())
    _, _, counters, ref, _ = _oracle(obs, vis)
    h = _imager(im, obs)
    assert h.half_plane
    tv = torch.from_numpy(vis).cuda()
    for fmt, tol in FORMAT_TOL.items():
        if fmt == "c64":
            out = h.image(tv)
        else:
            data, scales = im.compress_visibilities(tv, fmt)
            out = h.image_compressed(data, scales, fmt)
        out = out.cpu().numpy()
        errs = [rel_l2(out[i, j], ref[i, j]) for i in range(2) for j in range(4)]
        assert max(errs) < tol, (fmt, max(errs))
        assert np.array_equal(h.weight_sums(8), counters.reshape(8, -1).sum(1).astype(np.uint32)), fmt
    h.close()


@pytest.mark.parametrize("band", [0, 1, 2, 3])
def test_uneven_batch_band_image(im, band):
    """One channel of each band of the uneven batch (512 antennas, sides 256 << band), from
    complex64 and from 16-bit block floating point storage."""
    obs = synth.batched_bands(device="cuda", n_intervals=1, n_channels=1)[band]
    assert obs.n_ant == 512 and obs.n_pixels == 256 << band
    vis = np.ascontiguousarray(obs.vis_f32())
    _, _, counters, ref, _ = _oracle(obs, vis)
    h = _imager(im, obs)
    tv = torch.from_numpy(vis).cuda()
    out = h.image(tv).cpu().numpy()
    assert rel_l2(out[0, 0], ref[0, 0]) < FORMAT_TOL["c64"]
    data, scales = im.compress_visibilities(tv, "s16")
    out = h.image_compressed(data, scales, "s16").cpu().numpy()
    assert rel_l2(out[0, 0], ref[0, 0]) < IMAGE_TOL
    assert int(h.weight_sums(1)[0]) == int(counters.sum())
    h.close()
