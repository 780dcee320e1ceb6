"""Block-scaled 16-bit visibility storage through the C ABI: the CUDA encoder against the
storage oracle bit for bit; imaging from stored blocks against the oracle's pipeline on the
decoded values (the imaging tolerance, 1e-4 relative L2), and the precision each format keeps
against the FP64 oracle of the original complex64 visibilities."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
IMAGE_TOL = 1e-4
# relative L2 of an image against the FP64 oracle of the unquantised visibilities: S16 meets
# the imaging tolerance; BF16 and FP16 carry their element precision (2^-9, 2^-12 relative)
PRECISION = {"s16": 1e-4, "fp16": 5e-4, "bf16": 4e-3}


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    O.build()
    from imager_gb300 import imager
    return imager


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _awkward_vis(seed, T, Cn, nb):
    rng = np.random.default_rng(seed)
    vis = (rng.standard_normal((T, Cn, nb, 4, 2)) * 10.0 ** rng.integers(-3, 3, (T, Cn, nb, 1, 1))).astype(np.float32)
    vis[0, 0, 3, 0, 0] = np.nan
    vis[0, 0, 4, 1, 1] = np.float32(999999995904.0)    # valid: just below 1e12
    vis[0, 0, 5, 2, 0] = np.float32(1000000061440.0)   # invalid: just above
    vis[0, 0, 6, 3, 1] = -np.inf
    vis[-1, -1, 128:256] = 0.0                          # an all-zero block in every plane
    vis[0, -1, 256:300, 0] *= 1e-7                      # tiny values beside large ones
    vis[0, -1, 260, 0, 0] = 7.0
    return vis


@pytest.mark.parametrize("fmt", ["s16", "bf16", "fp16"])
def test_encoder_bit_exact(im, fmt):
    nb = 40 * 41 // 2  # 820 baselines: the last block of each plane is partial
    vis = _awkward_vis(3, 2, 3, nb)
    d_ref, s_ref = O.compress(vis, fmt)
    d, s = im.compress_visibilities(dev(vis), fmt)
    d = d.cpu().numpy().view(np.uint16)
    s = s.cpu().numpy()
    assert np.array_equal(s.view(np.uint32), s_ref.view(np.uint32))
    assert np.array_equal(d, d_ref)


def _imager(im, obs, n, pol, full_plane=False):
    h = im.Imager(n, 2.0, pol, -1000.0, full_plane=full_plane)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    return h


@pytest.mark.parametrize("fmt", ["s16", "bf16", "fp16"])
@pytest.mark.parametrize("pol", ["XX", "YY", "I", "V"])
@pytest.mark.parametrize("full_plane", [False, True])
def test_image_compressed_against_oracle(im, fmt, pol, full_plane):
    n = 128
    obs = synth.small(seed=47, n_ant=40, n_intervals=2, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    data, scales = im.compress_visibilities(dev(vis), fmt)
    decoded = O.decompress(data.cpu().numpy().view(np.uint16), scales.cpu().numpy(), fmt)
    _, _, counters, ref_dec, _ = O.full_pipeline(decoded, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n,
                                                 pol=pol, n_uvw_sets=2)
    _, _, _, ref_raw, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n, pol=pol,
                                          n_uvw_sets=2)
    h = _imager(im, obs, n, pol, full_plane)
    out = h.image_compressed(data, scales, fmt).cpu().numpy()
    worst = 0.0
    for i in range(out.shape[0]):
        for j in range(out.shape[1]):
            assert rel_l2(out[i, j], ref_dec[i, j]) < IMAGE_TOL, (i, j)
            worst = max(worst, rel_l2(out[i, j], ref_raw[i, j]))
    assert worst < PRECISION[fmt], worst
    assert np.array_equal(h.weight_sums(6), counters.reshape(6, -1).sum(1).astype(np.uint32))
    host = h.image_compressed_host(data.cpu().numpy(), scales.cpu().numpy(), fmt)
    assert rel_l2(host, out) < 1e-6
    h.close()


def test_compressed_deterministic_and_corrections_off(im):
    """Deterministic mode on stored blocks gives the same bits twice; flags 0 images the stored
    values as they are."""
    n = 64
    obs = synth.small(seed=5, n_ant=24, n_intervals=1, n_channels=2, n_pixels=n)
    vis = obs.vis_f32()
    data, scales = im.compress_visibilities(dev(vis), "s16")
    decoded = O.decompress(data.cpu().numpy().view(np.uint16), scales.cpu().numpy(), "s16")
    _, _, _, ref, _ = O.full_pipeline(decoded, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n, pol="I",
                                      apply_geom=False, apply_cable_corr=False)
    h = _imager(im, obs, n, "I")
    h.set_deterministic(True)
    a = h.image_compressed(data, scales, "s16", flags=0).cpu().numpy()
    b = h.image_compressed(data, scales, "s16", flags=0).cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for j in range(2):
        assert rel_l2(a[0, j], ref[0, j]) < IMAGE_TOL
    h.close()


def test_compressed_argument_checks(im):
    obs = synth.small(seed=5, n_ant=8, n_intervals=1, n_channels=1, n_pixels=32)
    h = _imager(im, obs, 32, "XX")
    data, scales = im.compress_visibilities(dev(obs.vis_f32()), "s16")
    with pytest.raises(capi.BgiError):
        h.image_compressed(data, scales, "c64")
    with pytest.raises(capi.BgiError):
        h.image_compressed(data, None, "s16")
    h.close()


def test_precision_form_array_at_1024(im):
    """The precision form's array and image side on a reduced block: 128 antennas in a 3 km disk
    with log-radial density, 10 kHz channels, 1024^2 images.  16-bit integer storage stays
    within the 1e-4 image tolerance of the FP64 oracle; bfloat16 (8 significant bits per
    component) does not, by the margin its rounding predicts."""
    obs = synth.precision_form(device="cpu", n_intervals=2, n_channels=3, keep_device=False)
    vis = obs.vis_f32()
    n = obs.n_pixels
    assert n == 1024 and obs.n_ant == 128
    _, _, counters, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n,
                                             n_uvw_sets=2)
    h = im.Imager(n, 2.0, "XX", -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    errs = {}
    for fmt in ("s16", "bf16"):
        data, scales = im.compress_visibilities(dev(vis), fmt)
        out = h.image_compressed(data, scales, fmt).cpu().numpy()
        errs[fmt] = max(rel_l2(out[i, j], ref[i, j]) for i in range(2) for j in range(3))
        assert np.array_equal(h.weight_sums(6), counters.reshape(6, -1).sum(1).astype(np.uint32))
    assert errs["s16"] < IMAGE_TOL
    assert IMAGE_TOL < errs["bf16"] < 1e-2
    h.close()
