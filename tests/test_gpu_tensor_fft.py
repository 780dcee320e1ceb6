"""The complex-to-real row pass on the tensor cores (BGI_FFT_TENSOR_SPLIT16: split-FP16 hi + lo DFT
products, FP32 accumulation) against the oracle's FP64 images and against the FP32 passes.

Tolerances: images within 1e-4 relative L2 of the FP64 oracle (the path's bound), and within 5e-6
relative L2 (max error within 1e-5 of the image peak) of the FP32 Stockham passes -- the split
operands carry about 22 significant bits."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
IMAGE_TOL = 1e-4
VS_FP32_TOL = 5e-6


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


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _pair(im, obs, pol="XX", wave=0):
    hs = []
    for mode in ("simt", "tensor_split16"):
        h = im.Imager(512, 2.0, pol, -1000.0, max_images_per_wave=wave)
        h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
        h.set_frequencies(obs.freqs)
        h.set_fft_mode(mode)
        assert h.fft_mode == mode and h.half_plane
        hs.append(h)
    return hs


@pytest.mark.parametrize("pol", ["XX", "I", "V"])
def test_tensor_rows_against_oracle_and_fp32(im, pol):
    obs = synth.small(seed=512, n_ant=64, n_intervals=2, n_channels=3, n_pixels=512)
    vis = obs.vis_f32()
    _, _, counters, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 512,
                                             pol=pol, n_uvw_sets=2)
    simt, tc = _pair(im, obs, pol, wave=4)  # two waves: the scratch is cleared between them
    a = simt.image(dev(vis)).cpu().numpy()
    b = tc.image(dev(vis)).cpu().numpy()
    for i in range(2):
        for j in range(3):
            assert rel_l2(b[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
            assert rel_l2(b[i, j], a[i, j]) < VS_FP32_TOL, (i, j)
            assert np.abs(b[i, j] - a[i, j]).max() < 1e-5 * np.abs(a[i, j]).max(), (i, j)
            assert np.all(b[i, j].imag == 0)
    assert np.array_equal(tc.weight_sums(6), counters.reshape(6, -1).sum(1).astype(np.uint32))
    for h in (simt, tc):
        h.close()


def test_tensor_rows_real_output_and_storage(im):
    """Real images and 16-bit block floating point storage through the tensor-core pass."""
    obs = synth.small(seed=513, n_ant=48, n_intervals=1, n_channels=4, n_pixels=512)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 512)
    _, tc = _pair(im, obs)
    fl = im.APPLY_GEOMETRIC | im.APPLY_CABLE
    real = tc.image(dev(vis), flags=fl | im.OUTPUT_REAL).cpu().numpy()
    data, scales = im.compress_visibilities(dev(vis), "s16")
    s16 = tc.image_compressed(data, scales, "s16").cpu().numpy()
    for j in range(4):
        assert rel_l2(real[0, j], ref[0, j]) < IMAGE_TOL, j
        assert rel_l2(s16[0, j], ref[0, j]) < IMAGE_TOL, j


def test_tensor_rows_dynamic_range(im):
    """A bright source 1e6 times the others and an all-zero block: the per-row power-of-two scale
    keeps every value inside FP16's range and the weak structure within tolerance."""
    obs = synth.small(seed=514, n_ant=48, n_intervals=1, n_channels=2, n_pixels=512)
    vis = obs.vis_f32().copy()
    vis[0, 0, :, 0, 0] *= 1e6  # channel 0: XX real parts scaled up (a bright, real component)
    vis[0, 1] = 0.0            # channel 1: nothing but zeros (weights still count)
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 512)
    simt, tc = _pair(im, obs)
    a = simt.image(dev(vis)).cpu().numpy()
    b = tc.image(dev(vis)).cpu().numpy()
    assert rel_l2(b[0, 0], ref[0, 0]) < IMAGE_TOL
    assert rel_l2(b[0, 0], a[0, 0]) < VS_FP32_TOL
    assert np.all(np.isfinite(b)) and np.all(b[0, 1] == 0)
    for h in (simt, tc):
        h.close()


def test_autotune_chooses_among_fft_modes(im):
    """bgi_autotune at 512 also times the tensor-core row pass; whatever it keeps images the
    block within tolerance."""
    obs = synth.small(seed=515, n_ant=48, n_intervals=2, n_channels=4, n_pixels=512)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 512, n_uvw_sets=2)
    h, _ = _pair(im, obs)
    wave, lanes, ms = h.autotune(dev(vis))
    assert ms > 0 and h.fft_mode in ("simt", "tensor_split16") and h.gridding_images_per_thread in (0, 2, 4, 8)
    out = h.image(dev(vis)).cpu().numpy()
    for i in range(2):
        for j in range(4):
            assert rel_l2(out[i, j], ref[i, j]) < IMAGE_TOL, (i, j)


def test_tensor_mode_rejected_off_512(im):
    from imager_gb300 import capi
    h = im.Imager(256)
    with pytest.raises(capi.BgiError) as e:
        h.set_fft_mode("tensor_split16")
    assert e.value.status == capi.ERR_UNSUPPORTED
    assert h.fft_mode == "simt"
    h.close()
