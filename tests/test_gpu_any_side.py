"""Image sides that are not powers of two, and the CPU gridder's uniform weighting, through the
C ABI against the oracle.

The reference images any side N through cuFFT / FFTW (src/gpu/pacer_imager_hip.cpp:83-95,
src/pacer_imager.cpp:145-156), with the CPU fftshift's half swaps for odd sides
(src/pacer_imager.cpp:110-128); its in-repo EDA2 template is imaged at N = 180.  Weighting "U"
divides every grid cell by its counter after gridding (src/pacer_imager.cpp:419-428), empty cells
included (0/0).

Tolerances: images within 1e-4 relative L2 of the FP64 oracle; weight sums exact; uniform grids
NaN for NaN and within FP32 summation-order error elsewhere."""
import ast
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
IMAGE_TOL = 1e-4


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from imager_gb300 import capi, imager
    capi.lib(build_if_missing=True)
    O.build()
    return imager


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _imager(im, obs, n, osf=2.0, pol="XX"):
    h = im.Imager(n, osf, pol, -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    return h


@pytest.mark.parametrize("n", [24, 48, 100, 180, 243, 375])
@pytest.mark.parametrize("pol", ["XX", "I"])
def test_image_any_side_against_oracle(im, n, pol):
    """bgi_image and bgi_image_host at even and odd sides that are not powers of two (full plane,
    mixed-radix passes, the CPU path's fftshift for odd sides)."""
    obs = synth.small(seed=60 + n, n_ant=40, n_intervals=2, n_channels=2, n_pixels=n)
    vis = obs.vis_f32()
    _, _, counters, ref, (du, dv) = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n,
                                                    pol=pol, n_uvw_sets=2)
    h = _imager(im, obs, n, pol=pol)
    assert not h.half_plane
    assert h.uv_cell[:2] == (du, dv)
    out = h.image(dev(vis)).cpu().numpy()
    for i in range(2):
        for j in range(2):
            assert rel_l2(out[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
    assert np.array_equal(h.weight_sums(4), counters.reshape(4, -1).sum(1).astype(np.uint32))
    real = h.image(dev(vis), flags=im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.OUTPUT_REAL).cpu().numpy()
    assert rel_l2(real, out.real) < 1e-6  # separate calls: atomic sums may round differently
    host = h.image_host(np.ascontiguousarray(vis))
    assert rel_l2(host, out) < 1e-6
    h.close()


def test_image_any_side_s16_storage(im):
    """16-bit block floating point storage imaged at 180 x 180 (the reference's EDA2 side)."""
    obs = synth.small(seed=180, n_ant=64, n_intervals=1, n_channels=3, n_pixels=180)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 180)
    h = _imager(im, obs, 180)
    data, scales = im.compress_visibilities(dev(vis), "s16")
    out = h.image_compressed(data, scales, "s16").cpu().numpy()
    for j in range(3):
        assert rel_l2(out[0, j], ref[0, j]) < IMAGE_TOL, j
    h.close()


def _uniform_oracle(obs, vis, n, osf, pol="XX"):
    """Corrections, gridding with weighting "U", FP64 images (the CPU path with weighting "U")."""
    corr = np.array(vis, np.float32, copy=True)
    O.apply_geometric(corr, obs.w, obs.freqs, obs.n_uvw_sets)
    O.apply_cable(corr, obs.cable, obs.freqs)
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(osf, umax, n), O.delta_uv(osf, vmax, n)
    g, c, _ = O.gridding(corr, obs.u, obs.v, obs.flags, obs.freqs, du, dv, n, -1000.0, pol, uniform=True,
                         n_uvw_sets=obs.n_uvw_sets)
    return corr, g, c, O.image_f64(g, c), (du, dv)


@pytest.mark.parametrize("n", [16, 24])
def test_uniform_weighting_full_coverage(im, n):
    """64 antennas at oversampling 0.5: every cell is gridded, so the uniformly weighted images are
    finite and match the oracle; the same block on 16-bit storage too."""
    obs = synth.small(seed=21, n_ant=64, n_intervals=1, n_channels=2, n_pixels=n)
    vis = obs.vis_f32()
    _, g, c, ref, _ = _uniform_oracle(obs, vis, n, 0.5)
    assert (c > 0).all() and np.isfinite(ref).all()
    h = _imager(im, obs, n, osf=0.5)
    fl = im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.WEIGHT_UNIFORM
    out = h.image(dev(vis), flags=fl).cpu().numpy()
    for j in range(2):
        assert rel_l2(out[0, j], ref[0, j]) < IMAGE_TOL, j
    assert np.array_equal(h.weight_sums(2), c.reshape(2, -1).sum(1).astype(np.uint32))
    # twice in a row: the counter scratch is clean for the second call
    again = h.image(dev(vis), flags=fl).cpu().numpy()
    assert rel_l2(again, out) < 1e-6
    data, scales = im.compress_visibilities(dev(vis), "s16")
    s16 = h.image_compressed(data, scales, "s16", flags=fl).cpu().numpy()
    for j in range(2):
        assert rel_l2(s16[0, j], ref[0, j]) < IMAGE_TOL, j
    # natural weighting on the same handle afterwards is unaffected
    _, _, _, nat, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n, osf=0.5)
    natural = h.image(dev(vis)).cpu().numpy()
    assert rel_l2(natural[0, 0], nat[0, 0]) < IMAGE_TOL
    h.close()


def test_uniform_weighting_empty_cells_and_golden(im):
    """The reference's own uniformly weighted grids (golden case run_XX_32_uniform): the free
    function on the oracle's natural grids gives NaN exactly where the reference has empty cells
    and its values elsewhere; the handle's images are NaN wherever the reference's are."""
    g = np.load(os.path.join(GOLD, "imager_run.npz"))
    meta = ast.literal_eval(str(g["meta"]))
    name = "run_XX_32_uniform"
    m = meta[name]
    n = m["n_pixels"]
    vis_c = g[f"{name}__vis_out"]
    Cn = vis_c.shape[1]
    freqs = g["freqs_cotter"]
    flags = O.update_flags(len(g["cable"]), m.get("flagged", (3,)))
    du, dv = g[f"{name}__scalars"][:2]
    grids, counters, _ = O.gridding(vis_c, g["u"][None], g["v"][None], flags, freqs, du, dv, n)
    t_grids = dev(grids.view(np.complex64)[..., 0])
    im.uniform_weighting(t_grids, dev(counters))
    got = t_grids.cpu().numpy()
    ref = g[f"{name}__grids"].view(np.complex64)[..., 0]
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.array_equal(got[ok], ref[ok])  # the same FP32 sums, divided with IEEE rounding
    h = im.Imager(n, 2.0, "XX", -1000.0)
    h.set_array(g["u"], g["v"], g["w"], flags, g["cable"])
    h.set_frequencies(freqs[:Cn])
    out = h.image(dev(g["vis"]), flags=im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.WEIGHT_UNIFORM).cpu().numpy()
    ref_img = g[f"{name}__images"].view(np.complex64)[..., 0]
    assert np.array_equal(np.isnan(out), np.isnan(ref_img))
    h.close()


def test_deterministic_gridder_any_side_and_uniform(im):
    """The ordered gridder at 180 x 180 (full plane, mixed-radix passes): the same image bits on
    two calls and within tolerance of the oracle; with weighting "U" as well (counters from the
    ordered reduce, then the division)."""
    n = 180
    obs = synth.small(seed=181, n_ant=48, n_intervals=1, n_channels=2, n_pixels=n)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n)
    h = _imager(im, obs, n)
    h.set_deterministic(True)
    a = h.image(dev(vis)).cpu().numpy()
    b = h.image(dev(vis)).cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for j in range(2):
        assert rel_l2(a[0, j], ref[0, j]) < IMAGE_TOL, j
    h.close()
    # uniform weighting at full coverage (oversampling 0.5, 64 antennas, a 24-pixel side)
    obs = synth.small(seed=21, n_ant=64, n_intervals=1, n_channels=2, n_pixels=24)
    vis = obs.vis_f32()
    _, _, c, ref, _ = _uniform_oracle(obs, vis, 24, 0.5)
    assert (c > 0).all()
    h = _imager(im, obs, 24, osf=0.5)
    h.set_deterministic(True)
    fl = im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.WEIGHT_UNIFORM
    a = h.image(dev(vis), flags=fl).cpu().numpy()
    b = h.image(dev(vis), flags=fl).cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    for j in range(2):
        assert rel_l2(a[0, j], ref[0, j]) < IMAGE_TOL, j
    h.close()


@pytest.mark.parametrize("n", [1, 2, 3, 8, 15])
def test_image_tiny_sides(im, n):
    """The smallest sides through the handle (full plane, mixed-radix passes below 16): the
    oracle's images, and the weight sums exact."""
    obs = synth.small(seed=90 + n, n_ant=12, n_intervals=1, n_channels=2, n_pixels=n)
    vis = obs.vis_f32()
    _, _, counters, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n)
    h = _imager(im, obs, n)
    out = h.image(dev(vis)).cpu().numpy()
    for j in range(2):
        assert rel_l2(out[0, j], ref[0, j]) < IMAGE_TOL, j
    assert np.array_equal(h.weight_sums(2), counters.reshape(2, -1).sum(1).astype(np.uint32))
    h.close()
