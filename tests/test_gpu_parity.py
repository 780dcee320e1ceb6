"""CUDA path against the oracle and the reference's own outputs (golden vectors), through the
C ABI.  Tolerances: cell indices and counters bit-exact; grids within FP32 summation-order
error; images within 1e-4 relative L2 of the FP64 oracle (the path's stated bound)."""
import ast
import math
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
IMAGE_TOL = 1e-4      # relative L2 per image vs the FP64 oracle
C_LIGHT = 299792458.0


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    O.build()
    from imager_gb300 import imager
    return imager


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ------------------------------------------------------------------------------------------
# corrections
# ------------------------------------------------------------------------------------------
def test_corrections_against_reference_golden(im):
    g = np.load(os.path.join(GOLD, "corrections.npz"))
    vis = g["vis"]
    for name, fn, after in (("geometric", lambda t: im.apply_geometric_corrections(t, dev(g["w"]), dev(g["freqs"])),
                             g["after_geometric"]),
                            ("cable", lambda t: im.apply_cable_corrections(t, dev(g["cable"]), dev(g["freqs"])),
                             g["after_cable"])):
        t = dev(vis)
        fn(t)
        out = t.cpu().numpy()
        err = np.abs(out - after).max() / np.abs(after).max()
        assert err < 2e-6, (name, err)
        assert rel_l2(out.view(np.complex64), after.view(np.complex64)) < 1e-6, name


def test_corrections_per_interval_uvw(im):
    obs = synth.small(seed=21, n_ant=30, n_intervals=3, n_channels=2)
    vis = obs.vis_f32().copy()
    ref = vis.copy()
    O.apply_geometric(ref, obs.w, obs.freqs, n_uvw_sets=3)
    t = dev(vis)
    im.apply_geometric_corrections(t, dev(obs.w), dev(obs.freqs), n_uvw_sets=3)
    assert rel_l2(t.cpu().numpy().view(np.complex64), ref.view(np.complex64)) < 1e-6


# ------------------------------------------------------------------------------------------
# gridding: counters exact (proves every cell index), grids within summation-order error
# ------------------------------------------------------------------------------------------
def _grid_gpu(im, vis, u, v, flags, freqs, du, dv, n, min_uv, pol, n_uvw_sets, mode=capi.COUNTERS_PER_IMAGE):
    T, Cn = vis.shape[:2]
    grids = torch.zeros((T, Cn, n, n), dtype=torch.complex64, device="cuda")
    cshape = (T, Cn, n, n) if mode == capi.COUNTERS_PER_IMAGE else (Cn, n, n)
    counters = torch.zeros(cshape, dtype=torch.float32, device="cuda")
    im.gridding(dev(vis), dev(u), dev(v), dev(flags), dev(freqs), du, dv, n, min_uv, pol, grids,
                counters, counter_mode=mode, n_uvw_sets=n_uvw_sets)
    return grids.cpu().numpy(), counters.cpu().numpy()


def _check_grids(g_gpu, g_ref_f32):
    ref = g_ref_f32.view(np.complex64)[..., 0]
    scale = max(np.abs(ref).max(), 1e-30)
    assert np.abs(g_gpu - ref).max() <= 1e-5 * scale
    # cells the oracle never touched stay exactly zero
    assert np.all(g_gpu[ref == 0] == 0)


@pytest.mark.parametrize("pol", ["XX", "YY", "I", "V"])
@pytest.mark.parametrize("min_uv", [-1000.0, 3.0])
def test_gridding_against_oracle(im, pol, min_uv):
    obs = synth.small(seed=31, n_ant=40, n_intervals=3, n_channels=4, n_pixels=128)
    vis = obs.vis_f32().copy()
    vis[0, 1, 17, 0, 0] = np.nan
    vis[1, 0, 23, 3, 1] = np.inf
    vis[2, 3, 40, 0, 1] = 3e12
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, 128), O.delta_uv(2.0, vmax, 128)
    g_ref, c_ref, _ = O.gridding(vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 128, min_uv, pol, n_uvw_sets=3)
    g, c = _grid_gpu(im, vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 128, min_uv, pol, 3)
    assert np.array_equal(c, c_ref)
    _check_grids(g, g_ref)
    # counters of interval 0 only, laid out per channel (src/gpu/gridding_gpu.cpp:107,117)
    _, c0 = _grid_gpu(im, vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 128, min_uv, pol, 3,
                      mode=capi.COUNTERS_FIRST_INTERVAL)
    assert np.array_equal(c0, c_ref[0])


def test_gridding_rounding_ties_and_wraps(im):
    """Pixel coordinates at and one ulp either side of half-integers, min_uv equal to the uv
    distance, and coordinates beyond the grid (wrapped or dropped as in calculate_pos)."""
    n_ant, n = 32, 64
    nb = n_ant * (n_ant + 1) // 2
    rng = np.random.default_rng(3)
    base = rng.integers(-40, 40, nb).astype(np.float32) + np.float32(0.5)
    u = base.copy()
    u[::3] = np.nextafter(base[::3], np.float32(np.inf))
    u[1::3] = np.nextafter(base[1::3], np.float32(-np.inf))
    v = (rng.integers(-40, 40, nb) + 0.5).astype(np.float32)
    v[5] = 4.0
    u[5] = 3.0                       # distance exactly 5 wavelengths
    u[7], v[7] = 100.5, 2.0          # beyond N/2: wraps
    u[8], v[8] = -70.5, 3.5          # below -N: negative index, dropped or wrapped as the reference
    u[9], v[9] = 2.5, -80.0
    flags = np.zeros(nb, np.int32)
    freqs = np.array([C_LIGHT, C_LIGHT * 0.75])  # wavelength exactly 1 m, then 4/3 m
    vis = (rng.standard_normal((1, 2, nb, 4, 2))).astype(np.float32)
    for min_uv in (-1.0, 5.0):
        g_ref, c_ref, _ = O.gridding(vis, u, v, flags, freqs, 1.0, 1.0, n, min_uv, "XX")
        g, c = _grid_gpu(im, vis, u, v, flags, freqs, 1.0, 1.0, n, min_uv, "XX", 1)
        assert np.array_equal(c, c_ref), min_uv
        _check_grids(g, g_ref)


def test_gridding_max_vis_edge(im):
    """|x| < 1e12 is decided in double by the reference (src/pacer_imager.cpp:329): the float
    just below 1e12 is gridded, the float just above is skipped."""
    obs = synth.small(seed=9, n_ant=16, n_intervals=1, n_channels=2, n_pixels=64)
    vis = obs.vis_f32().copy()
    below, above = np.float32(999999995904.0), np.float32(1000000061440.0)
    vis[0, 0, 22, 0, 0] = below      # baselines 22-25: antenna 6 with antennas 1-4
    vis[0, 0, 23, 0, 1] = -below
    vis[0, 1, 24, 0, 0] = above
    vis[0, 1, 25, 0, 1] = -above
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, 64), O.delta_uv(2.0, vmax, 64)
    g_ref, c_ref, n_ref = O.gridding(vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 64)
    g, c = _grid_gpu(im, vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 64, -1000.0, "XX", 1)
    assert np.array_equal(c, c_ref)
    assert (np.abs(g) >= 9e11).sum() >= 2  # the two components just below 1e12 were gridded


def test_gridding_against_reference_golden(im):
    """bgi_gridding_gpu on the reference's corrected visibilities reproduces the reference's
    counters exactly and its grids to summation order, including the 48-pixel case."""
    g = np.load(os.path.join(GOLD, "imager_run.npz"))
    meta = ast.literal_eval(str(g["meta"]))
    pols = ["XX", "YY", "I", "V"]
    for name, m in meta.items():
        if m.get("weighting") == "U" or m.get("kernel"):
            continue
        vis_c = g[f"{name}__vis_out"]
        Cn = vis_c.shape[1]
        freqs = (np.full(Cn, m["freq_override_mhz"] * 1e6) if "freq_override_mhz" in m else g["freqs_cotter"])
        flags = O.update_flags(len(g["cable"]), m.get("flagged", (3,)))
        du, dv = g[f"{name}__scalars"][:2]
        gr, c = _grid_gpu(im, vis_c, g["u"], g["v"], flags, freqs, du, dv, m["n_pixels"],
                          m.get("min_uv", -1000.0), pols[m["pol"]], 1)
        assert np.array_equal(c, g[f"{name}__counters"]), name
        _check_grids(gr, g[f"{name}__grids"])


# ------------------------------------------------------------------------------------------
# FFT and epilogues
# ------------------------------------------------------------------------------------------
@pytest.mark.parametrize("n,batch", [(16, 3), (32, 2), (64, 3), (128, 2), (256, 2), (512, 2),
                                     (1024, 1), (2048, 1), (4096, 1),
                                     # sides that are not powers of two (mixed-radix passes)
                                     (1, 3), (2, 2), (6, 2), (12, 2), (48, 2), (97, 1), (180, 2), (200, 2),
                                     (243, 1), (1000, 1), (4095, 1)])
def test_fft_inverse_against_numpy(im, n, batch):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))).astype(np.complex64)
    out = torch.empty((batch, n, n), dtype=torch.complex64, device="cuda")
    im.fft_inverse(dev(x), out)
    ref = np.fft.ifft2(x.astype(np.complex128)) * n * n
    assert rel_l2(out.cpu().numpy(), ref) < 2e-6 * max(math.log2(n), 1.0)


def _shift_norm_reference_gpu_semantics(data, fnorm):
    """numpy restatement of fft_shift_and_norm_x/_y (src/gpu/gpu_utils.cpp:80-123)."""
    out = data.copy()
    n_img, ys, xs = out.shape
    sh = lambda p, s: (p + s // 2 + s % 2) % s  # noqa: E731
    for i in range(n_img):
        for y in range(ys):
            for x in range(xs // 2):
                d = sh(x, xs)
                out[i, y, x], out[i, y, d] = out[i, y, d], out[i, y, x]
        f = np.float32(fnorm[i % len(fnorm)])
        for y in range(ys // 2):
            d = sh(y, ys)
            a, b = out[i, y].copy(), out[i, d].copy()
            out[i, d] = (a.real / f) + 1j * (a.imag / f)
            out[i, y] = (b.real / f) + 1j * (b.imag / f)
    return out.astype(np.complex64)


def test_fft_shift_and_norm_known_answer(im):
    """tests/gpu_utils_test.cpp:60-88 of the reference."""
    x = np.tile(np.array([0, 1, 2, 3], np.complex64), 3).reshape(3, 2, 2)
    t = dev(x)
    im.fft_shift_and_norm(t, dev(np.ones(3, np.float32)))
    assert np.array_equal(t.cpu().numpy().ravel(), np.tile(np.array([3, 2, 1, 0], np.complex64), 3))


@pytest.mark.parametrize("ys,xs,nf", [(8, 6, 3), (5, 8, 2), (16, 16, 1)])
def test_fft_shift_and_norm_against_reference_semantics(im, ys, xs, nf):
    rng = np.random.default_rng(ys * xs)
    x = (rng.standard_normal((4, ys, xs)) + 1j * rng.standard_normal((4, ys, xs))).astype(np.complex64)
    fn = rng.uniform(1, 50, nf).astype(np.float32)
    t = dev(x)
    im.fft_shift_and_norm(t, dev(fn))
    assert np.array_equal(t.cpu().numpy(), _shift_norm_reference_gpu_semantics(x, fn))


def test_vector_sum_known_answer(im):
    """tests/gpu_utils_test.cpp:20-58 of the reference: 5 images x 3000 ints in [0, 50)."""
    rng = np.random.default_rng(1)
    data = rng.integers(0, 50, (5, 3000)).astype(np.float32)
    sums = torch.zeros(5, dtype=torch.float32, device="cuda")
    im.vector_sum(dev(data), 3000, 5, sums)
    assert np.array_equal(sums.cpu().numpy(), data.sum(1).astype(np.float32))


def test_image_averaging_known_answer(im):
    """tests/gpu_utils_test.cpp:91-125 of the reference: 4 images 512^2 of (i % 100)."""
    n_pix = 512 * 512
    x = np.tile((np.arange(n_pix) % 100).astype(np.complex64), (4, 1)).reshape(4, 512, 512)
    out = torch.empty((512, 512), dtype=torch.complex64, device="cuda")
    im.image_averaging(dev(x), out)
    assert np.array_equal(out.cpu().numpy(), x[0])


# ------------------------------------------------------------------------------------------
# whole path (bgi_image)
# ------------------------------------------------------------------------------------------
def _imager_for(im, obs, n, pol="XX", min_uv=-1000.0, wave=0, full_plane=False):
    h = im.Imager(n, 2.0, pol, min_uv, max_images_per_wave=wave, full_plane=full_plane)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    return h


@pytest.mark.parametrize("full_plane", [False, True])
@pytest.mark.parametrize("pol", ["XX", "YY", "I", "V"])
@pytest.mark.parametrize("n,wave", [(64, 0), (128, 2)])
def test_image_against_oracle(im, pol, n, wave, full_plane):
    obs = synth.small(seed=41, n_ant=40, n_intervals=2, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    _, _, counters, ref, (du, dv) = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags,
                                                    obs.freqs, n, pol=pol, n_uvw_sets=2)
    h = _imager_for(im, obs, n, pol, wave=wave, full_plane=full_plane)
    assert h.half_plane == (not full_plane)
    assert h.uv_cell[:2] == (du, dv)
    out = h.image(dev(vis)).cpu().numpy()
    for i in range(out.shape[0]):
        for j in range(out.shape[1]):
            assert rel_l2(out[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
    sums = h.weight_sums(6)
    assert np.array_equal(sums, counters.reshape(6, -1).sum(1).astype(np.uint32))
    # the host-buffer entry point gives the same images
    host = h.image_host(np.ascontiguousarray(vis))
    assert rel_l2(host, out) < 1e-6
    h.close()


def test_image_against_reference_golden(im):
    """bgi_image on the reference's inputs against the reference's own dirty images."""
    g = np.load(os.path.join(GOLD, "imager_run.npz"))
    meta = ast.literal_eval(str(g["meta"]))
    pols = ["XX", "YY", "I", "V"]
    checked = 0
    for name, m in meta.items():
        n = m["n_pixels"]
        if m.get("weighting") == "U" or m.get("kernel"):
            continue
        vis = g["vis_bad"] if name.endswith("_bad") else g["vis"]
        Cn = vis.shape[1]
        freqs = (np.full(Cn, m["freq_override_mhz"] * 1e6) if "freq_override_mhz" in m else g["freqs_cotter"])
        flags = O.update_flags(len(g["cable"]), m.get("flagged", (3,)))
        h = im.Imager(n, 2.0, pols[m["pol"]], m.get("min_uv", -1000.0))
        h.set_array(g["u"], g["v"], g["w"], flags, g["cable"])
        h.set_frequencies(freqs)
        assert h.uv_cell[:2] == tuple(g[f"{name}__scalars"][:2]), name
        fl = (im.APPLY_GEOMETRIC if m.get("geom", 1) else 0) | (im.APPLY_CABLE if m.get("cable", 1) else 0)
        out = h.image(dev(vis), flags=fl).cpu().numpy()
        ref = g[f"{name}__images"].view(np.complex64)[..., 0]
        for i in range(out.shape[0]):
            for j in range(out.shape[1]):
                assert rel_l2(out[i, j], ref[i, j]) < IMAGE_TOL, (name, i, j)
        h.close()
        checked += 1
    assert checked >= 9  # the 48-pixel case included


def test_image_state_errors(im):
    h = im.Imager(64)
    with pytest.raises(capi.BgiError) as e:
        h.image(torch.zeros((1, 1, 3, 4, 2), device="cuda"))
    assert e.value.status == capi.ERR_STATE
    obs = synth.small(seed=5, n_ant=2, n_intervals=2, n_channels=1, n_pixels=64)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    with pytest.raises(capi.BgiError) as e:  # 2 UVW sets for 3 intervals
        h.image(torch.zeros((3, 1, 3, 4, 2), device="cuda"))
    assert e.value.status == capi.ERR_INVALID
    h.close()


# ------------------------------------------------------------------------------------------
# the measured workload at full size: 256 antennas, 64 channels x 10 intervals, 512^2
# ------------------------------------------------------------------------------------------
def test_full_size_workload_properties(im):
    obs = synth.config2(device="cuda")
    vis = obs.vis_f32()
    n = obs.n_pixels
    h = _imager_for(im, obs, n)
    out = h.image(dev(vis))
    torch.cuda.synchronize()
    T, Cn = vis.shape[:2]
    sums = h.weight_sums(T * Cn)
    # every unflagged baseline lands twice (min_uv = -1000, all cells in range)
    assert np.all(sums == 2 * int((obs.flags == 0).sum()))
    # centre pixel = sum of all grid cells / weight sum = 2 * sum(Re z) / sum(w)
    corr = vis.copy()
    O.apply_geometric(corr, obs.w, obs.freqs, n_uvw_sets=T)
    O.apply_cable(corr, obs.cable, obs.freqs)
    re = corr[..., 0, 0].astype(np.float64)                     # XX real parts [T][C][B]
    expect = 2 * (re * (obs.flags == 0)).sum(-1) / sums.reshape(T, Cn)
    centre = out[:, :, n // 2, n // 2].real.cpu().numpy()
    peak = out.abs().amax(dim=(2, 3)).cpu().numpy()
    # FP32 summation over N^2 cells: bound the error by the image peak, not the (small) sum
    assert np.all(np.abs(centre - expect) <= 1e-5 * peak)
    # a few whole images against the FP64 oracle
    du, dv, _, _ = h.uv_cell
    for t, c in ((0, 0), (4, 31), (9, 63)):
        g, cnt, _ = O.gridding(corr[t:t + 1, c:c + 1], obs.u[t:t + 1], obs.v[t:t + 1], obs.flags,
                               obs.freqs[c:c + 1], du, dv, n)
        ref = O.image_f64(g, cnt)[0, 0]
        assert rel_l2(out[t, c].cpu().numpy(), ref) < IMAGE_TOL, (t, c)
    h.close()


def test_sharded_images_equal_unsharded(im):
    """Two shards of one block (by intervals), each on its own handle with the whole block's uv
    cell, reproduce the unsharded images (the multi-GPU split, run here one after the other)."""
    from imager_gb300 import shard as S
    obs = synth.small(seed=61, n_ant=40, n_intervals=4, n_channels=3, n_pixels=64)
    full = _imager_for(im, obs, 64)
    ref = full.image(dev(obs.vis_f32())).cpu().numpy()
    du, dv, _, _ = full.uv_cell
    full.close()
    parts, shards = [], []
    for rank in range(2):
        sh = S.plan_shard(4, 3, 2, rank)
        vis, u, v, w, freqs = S.shard_inputs(obs, sh)
        h = im.Imager(64, 2.0, "XX", -1000.0)
        h.set_array(u, v, w, obs.flags, obs.cable)
        h.set_frequencies(freqs)
        h.set_uv_cell(du, dv)
        parts.append(h.image(dev(vis.view(np.float32).reshape(vis.shape + (2,)))).cpu().numpy())
        shards.append(sh)
        h.close()
    got = S.assemble(parts, shards, 4, 3, 64)
    for i in range(4):
        for j in range(3):
            assert rel_l2(got[i, j], ref[i, j]) < 1e-6, (i, j)


def test_image_host_many_chunks_equals_device(im):
    """bgi_image_host cuts the block into chunks whose uploads, waves and downloads overlap;
    with a 2-image wave, 24 images make 12 waves in 6 chunks over both lanes."""
    obs = synth.small(seed=63, n_ant=40, n_intervals=3, n_channels=8, n_pixels=128)
    h = _imager_for(im, obs, 128, wave=2)
    vis = np.ascontiguousarray(obs.vis_f32())
    dev_out = h.image(dev(vis)).cpu().numpy()
    host_out = h.image_host(vis)
    sums = h.weight_sums(24)
    assert rel_l2(host_out, dev_out) < 1e-6
    assert np.all(sums == 2 * int((obs.flags == 0).sum()))
    h.close()


def test_half_plane_falls_back_when_pixels_reach_the_side(im):
    """At 1.5 GHz with oversampling 1 the largest pixel coordinate exceeds N, where the
    reference's wrap no longer pairs mirror cells; the handle then images the full plane and
    still matches the oracle."""
    obs = synth.small(seed=47, n_ant=24, n_intervals=1, n_channels=2, n_pixels=64, f0=1.5e9, df=1e6)
    h = im.Imager(64, 1.0, "XX", -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    assert not h.half_plane
    assert h.uv_extent == (32, 32)
    out = h.image(dev(obs.vis_f32())).cpu().numpy()
    _, _, _, ref, _ = O.full_pipeline(obs.vis_f32(), obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 64,
                                      osf=1.0)
    for j in range(2):
        assert rel_l2(out[0, j], ref[0, j]) < IMAGE_TOL, j
    h.close()


@pytest.mark.parametrize("n,extent", [(64, 10.5), (64, 11.0 - 1e-9), (64, 11.0 + 1e-9), (64, 27.5), (64, 29.5),
                                      (64, 30.0), (64, 31.5), (512, 109.5), (512, 110.5), (512, 126.0 - 1e-9),
                                      (512, 253.5)])
def test_half_plane_pruning_at_the_coverage_edge(im, n, extent):
    """The half-plane column pass transforms only the columns and loads only the rows that the
    uv coverage can reach: |pixel| <= floor(u_max * nu_max / (c * delta_u)) + 2, N/2 when that
    reaches the half plane's edge.  With delta_u = osf * u_max / N the longest baselines at the
    top frequency land on pixel round(N * nu_max / (c * osf)); the top frequency is chosen so
    that this coordinate is a tie, just below or just above an integer, or near N/2, and the
    images must still match the oracle (one baseline lost would move them by about 1e-1)."""
    osf = 2.0
    f_top = extent * C_LIGHT * osf / n
    obs = synth.small(seed=53, n_ant=24, n_intervals=2, n_channels=3, n_pixels=n, f0=f_top - 2e6, df=1e6)
    assert abs(obs.freqs.max() - f_top) < 1e-3
    vis = obs.vis_f32()
    _, _, counters, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n,
                                             osf=osf, n_uvw_sets=2)
    h = _imager_for(im, obs, n)
    assert h.half_plane
    du, dv, um, vm = h.uv_cell
    fmax = float(obs.freqs.max())

    def bound(m, d):  # the handle's bound, in the same FP64 operations
        x = m * fmax / (C_LIGHT * d)
        return math.floor(x) + 2 if x + 2.0 < n // 2 else n // 2

    assert h.uv_extent == (bound(um, du), bound(vm, dv))
    # every gridded point's pixel coordinate (the reference's rounding) lies within the bound,
    # which is at most two pixels loose
    lam = C_LIGHT / obs.freqs
    for coord, d, b in ((obs.u, du, h.uv_extent[0]), (obs.v, dv, h.uv_extent[1])):
        x = (coord[:, obs.flags <= 0][:, None, :].astype(np.float64) / lam[None, :, None]) / d
        top = np.floor(np.abs(x) + 0.5).max()
        assert top <= b and (b == n // 2 or top >= b - 2), (top, b)
    out = h.image(dev(vis)).cpu().numpy()
    for i in range(2):
        for j in range(3):
            assert rel_l2(out[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
    assert np.array_equal(h.weight_sums(6), counters.reshape(6, -1).sum(1).astype(np.uint32))
    h.close()


def test_negative_flag_keeps_blocks_off_the_half_plane(im):
    """A baseline flag below zero is gridded (the GPU gridder's flags <= 0, as
    src/gpu/gridding_gpu.cpp:101) but u_max / v_max cover flag 0 only
    (src/pacer_imager.cpp:213-221), so its pixel may reach the side: the handle images such an
    array on the full plane, whose cell indices are checked, and counts the baseline."""
    obs = synth.small(seed=49, n_ant=24, n_intervals=1, n_channels=2, n_pixels=64)
    h = _imager_for(im, obs, 64)
    assert h.half_plane
    h.image(dev(obs.vis_f32()))
    base = h.weight_sums(2)
    flags = obs.flags.copy()
    b = 5 * 6 // 2 + 3  # baseline (5, 3): antenna 3 is flagged
    assert flags[b] == 1
    flags[b] = -1
    h.set_array(obs.u, obs.v, obs.w, flags, obs.cable)
    assert not h.half_plane
    h.image(dev(obs.vis_f32()))
    assert np.array_equal(h.weight_sums(2), base + 2)
    h.close()


@pytest.mark.parametrize("full_plane", [False, True])
@pytest.mark.parametrize("pol", ["XX", "I"])
def test_image_real_output(im, full_plane, pol):
    """BGI_OUTPUT_REAL: float images equal to the real part of the complex images (bit for bit
    in deterministic mode), within the image tolerance of the oracle's real part, on device and
    host buffers."""
    n = 128
    obs = synth.small(seed=53, n_ant=40, n_intervals=2, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n, pol=pol,
                                      n_uvw_sets=2)
    h = _imager_for(im, obs, n, pol, full_plane=full_plane)
    h.set_deterministic(True)
    fl = im.APPLY_GEOMETRIC | im.APPLY_CABLE
    cplx = h.image(dev(vis), flags=fl).cpu().numpy()
    real = h.image(dev(vis), flags=fl | im.OUTPUT_REAL)
    assert real.dtype == torch.float32 and tuple(real.shape) == (2, 3, n, n)
    real = real.cpu().numpy()
    assert np.array_equal(real.view(np.uint32), np.ascontiguousarray(cplx.real).view(np.uint32))
    for i in range(2):
        for j in range(3):
            assert rel_l2(real[i, j], ref[i, j].real) < IMAGE_TOL, (i, j)
    host = h.image_host(np.ascontiguousarray(vis), flags=fl | im.OUTPUT_REAL)
    assert host.dtype == np.float32 and np.array_equal(host.view(np.uint32), real.view(np.uint32))
    h.set_deterministic(False)
    fast = h.image(dev(vis), flags=fl | im.OUTPUT_REAL).cpu().numpy()  # atomic gridder
    assert rel_l2(fast, real) < 1e-6
    h.close()


def test_schedule_and_autotune(im):
    """Any schedule (wave size, lanes) gives the same images; the autotuner keeps a valid one."""
    n = 128
    obs = synth.small(seed=61, n_ant=40, n_intervals=3, n_channels=4, n_pixels=n)
    vis = dev(obs.vis_f32())
    h = _imager_for(im, obs, n, "XX")
    h.set_deterministic(True)
    ref = h.image(vis).cpu().numpy()
    for wave, lanes in ((1, 1), (5, 3), (12, 4), (1, 8), (0, 2)):
        h.set_schedule(wave, lanes)
        assert h.schedule == (wave, lanes)
        out = h.image(vis).cpu().numpy()
        assert np.array_equal(out.view(np.uint32), ref.view(np.uint32)), (wave, lanes)
    with pytest.raises(capi.BgiError):
        h.set_schedule(8, 9)
    h.set_deterministic(False)
    for cpt in (2, 4, 8, 0):  # images per gridding thread (0: by array size)
        h.set_gridding_images_per_thread(cpt)
        assert h.gridding_images_per_thread == cpt
        assert rel_l2(h.image(vis).cpu().numpy(), ref) < 1e-6, cpt
    with pytest.raises(capi.BgiError):
        h.set_gridding_images_per_thread(3)
    wave, lanes, ms = h.autotune(vis)
    assert wave in (0, 4, 8, 12) and 1 <= lanes <= 8 and ms > 0
    assert h.gridding_images_per_thread in (0, 2, 4, 8) and h.fft_mode == "simt"  # no tensor pass at 128
    assert rel_l2(h.image(vis).cpu().numpy(), ref) < 1e-6
    h.close()


@pytest.mark.parametrize("full_plane", [False, True])
def test_image_largest_side(im, full_plane):
    """The largest image side (4096), half and full plane, against the FP64 oracle."""
    n = 4096
    obs = synth.small(seed=121, n_ant=40, n_intervals=1, n_channels=2, n_pixels=n)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n, n_uvw_sets=1)
    h = _imager_for(im, obs, n, "XX", full_plane=full_plane)
    assert h.half_plane == (not full_plane)
    out = h.image(dev(vis)).cpu().numpy()
    for j in range(2):
        assert rel_l2(out[0, j], ref[0, j]) < IMAGE_TOL, j
    h.close()


def test_single_image_block(im):
    """One interval of one channel: a one-image wave on one lane."""
    obs = synth.small(seed=122, n_ant=24, n_intervals=1, n_channels=1, n_pixels=64)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, 64, n_uvw_sets=1)
    h = _imager_for(im, obs, 64, "XX")
    out = h.image(dev(vis)).cpu().numpy()
    assert out.shape == (1, 1, 64, 64) and rel_l2(out[0, 0], ref[0, 0]) < IMAGE_TOL
    host = h.image_host(np.ascontiguousarray(vis))
    assert rel_l2(host, out) < 1e-6
    h.close()


def test_image_wcs_and_fits_output(im, tmp_path):
    """bgi_get_image_wcs gives the reference's pixel scales (src/gpu/pacer_imager_hip.cpp:113-115)
    and a block of images goes to FITS files whose pixels are the images' real parts."""
    obs = synth.small(seed=55, n_ant=32, n_intervals=2, n_channels=2, n_pixels=64)
    h = _imager_for(im, obs, 64)
    out = h.image(dev(obs.vis_f32())).cpu().numpy()
    wcs = h.image_wcs(10.0, -26.7)
    _, _, umax, vmax = h.uv_cell
    assert wcs["pixscale_ra_deg"] == (1.0 / (2.0 * umax)) * (180.0 / math.pi)
    assert wcs["pixscale_dec_deg"] == (1.0 / (2.0 * vmax)) * (180.0 / math.pi)
    im.write_fits_block(tmp_path, "img", out, wcs, obs.freqs)
    raw = open(tmp_path / "img_t0001_c0001.fits", "rb").read()
    header = raw[:2880].decode("ascii")
    assert header.startswith("SIMPLE  =                    T") and "RA---SIN" in header
    data = np.frombuffer(raw[2880:2880 + 4 * 64 * 64], ">f4").reshape(64, 64)
    assert np.array_equal(data, out[1, 1].real)
    h.close()


def test_image_buffers_off_16_byte_boundaries(im):
    """The complex-to-real pass stores pixel pairs (16 bytes of complex, 8 of real pixels): a
    complex image buffer aligned to 8 bytes but not 16 routes the block to the full plane, with
    the same images; real images 8-byte aligned stay on the half plane; buffers not 8-byte
    aligned are refused before any launch."""
    obs = synth.small(seed=57, n_ant=32, n_intervals=1, n_channels=2, n_pixels=64)
    h = _imager_for(im, obs, 64)
    vis = dev(obs.vis_f32())
    ref = h.image(vis).cpu().numpy()
    npix = 2 * 64 * 64
    raw = torch.empty(npix + 1, dtype=torch.complex64, device="cuda")
    shifted = raw[1:].view(1, 2, 64, 64)            # 8 bytes past a 16-byte boundary
    assert shifted.data_ptr() % 16 == 8
    h.image(vis, out=shifted)
    assert rel_l2(shifted.cpu().numpy(), ref) < 1e-6
    raw_r = torch.empty(npix + 4, dtype=torch.float32, device="cuda")
    real8 = raw_r[2:2 + npix].view(1, 2, 64, 64)      # real images, 8 bytes past 16
    assert real8.data_ptr() % 16 == 8
    h.image(vis, flags=im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.OUTPUT_REAL, out=real8)
    assert rel_l2(real8.cpu().numpy(), ref.real) < 1e-6
    real4 = raw_r[1:1 + npix].view(1, 2, 64, 64)      # 4-byte aligned
    with pytest.raises(capi.BgiError) as e:
        h.image(vis, flags=im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.OUTPUT_REAL, out=real4)
    assert e.value.status == capi.ERR_INVALID
    h.close()


@pytest.mark.parametrize("pol", ["XX", "YY", "I", "V"])
@pytest.mark.parametrize("cpt", [4, 8])
def test_gridding_images_per_thread_against_oracle(im, pol, cpt):
    """Four and eight images per gridding thread (all of a thread's visibility loads issued
    first): every pol, complex64 and s16 storage, per-interval UVW sets, so a block's images
    cross an interval boundary (3 channels per interval) and reload u/v/w mid-block."""
    n = 128
    obs = synth.small(seed=70 + cpt, n_ant=40, n_intervals=4, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    _, _, counters, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n,
                                             pol=pol, n_uvw_sets=4)
    h = _imager_for(im, obs, n, pol)
    h.set_gridding_images_per_thread(cpt)
    out = h.image(dev(vis)).cpu().numpy()
    data, scales = im.compress_visibilities(dev(vis), "s16")
    s16 = h.image_compressed(data, scales, "s16").cpu().numpy()
    for i in range(4):
        for j in range(3):
            assert rel_l2(out[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
            assert rel_l2(s16[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
    assert np.array_equal(h.weight_sums(12), counters.reshape(12, -1).sum(1).astype(np.uint32))
    h.close()


@pytest.mark.parametrize("pol", ["XX", "I"])
@pytest.mark.parametrize("cpt", [4, 8])
def test_gridding_aggregation_against_oracle(im, pol, cpt):
    """Warp-aggregated gridding atomics on a crowded grid (100 antennas in a 35 m disk imaged at
    64^2: about 15,000 points per image on at most 2,080 half-plane cells, so most warps hold
    repeated cells): the oracle within 1e-4, the plain atomics within FP32 rounding, weight sums
    exact; complex64 and s16 storage, per-interval UVW sets."""
    n = 64
    obs = synth.small(seed=90 + cpt, n_ant=100, n_intervals=3, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    _, _, counters, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n,
                                             pol=pol, n_uvw_sets=3)
    h = _imager_for(im, obs, n, pol)
    assert h.half_plane and not h.gridding_aggregation
    h.set_gridding_images_per_thread(cpt)
    plain = h.image(dev(vis)).cpu().numpy()
    h.set_gridding_aggregation(True)
    assert h.gridding_aggregation
    agg = h.image(dev(vis)).cpu().numpy()
    data, scales = im.compress_visibilities(dev(vis), "s16")
    s16 = h.image_compressed(data, scales, "s16").cpu().numpy()
    for i in range(3):
        for j in range(3):
            assert rel_l2(agg[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
            assert rel_l2(s16[i, j], ref[i, j]) < IMAGE_TOL, (i, j)
            assert rel_l2(agg[i, j], plain[i, j]) < 2e-6, (i, j)
    assert np.array_equal(h.weight_sums(9), counters.reshape(9, -1).sum(1).astype(np.uint32))
    with pytest.raises(capi.BgiError):
        h.set_gridding_aggregation(2)
    h.close()


@pytest.mark.parametrize("n", [256, 512, 1024])
def test_column_radix_alternatives(im, n):
    """The column pass's second compiled radix images the same block as the default one (the
    oracle within 1e-4, the default radix within FP32 rounding); other radices are refused."""
    obs = synth.small(seed=80 + n // 256, n_ant=40, n_intervals=1, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    _, _, _, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n, n_uvw_sets=1)
    h = _imager_for(im, obs, n, "XX")
    default = h.column_radix
    a = h.image(dev(vis)).cpu().numpy()
    alt = {256: 8, 512: 16, 1024: 16}[n]
    h.set_column_radix(alt)
    assert h.column_radix == alt
    b = h.image(dev(vis)).cpu().numpy()
    for j in range(3):
        assert rel_l2(b[0, j], ref[0, j]) < IMAGE_TOL, j
        assert rel_l2(b[0, j], a[0, j]) < 2e-6, j
    with pytest.raises(capi.BgiError) as e:
        h.set_column_radix(4)
    assert e.value.status == capi.ERR_UNSUPPORTED
    h.set_column_radix(0)
    assert h.column_radix == default
    h.close()
