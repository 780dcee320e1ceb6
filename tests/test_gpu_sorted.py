"""Deterministic gridding (bgi_gridding_sorted_gpu) through the C ABI.  Its grids are summed
in the CPU gridding loop's order, so the bar is bit-identity: with the oracle's FP32 gridding
(a restatement of src/pacer_imager.cpp:297-408) and with the reference's own CPU grids in the
golden vectors; counters exact; the same bits on every run."""
import ast
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    O.build()
    from imager_gb300 import imager
    return imager


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _grid_sorted(im, vis, u, v, flags, freqs, du, dv, n, min_uv, pol, n_uvw_sets,
                 mode=capi.COUNTERS_PER_IMAGE, ws_images=None):
    T, Cn = vis.shape[:2]
    grids = torch.zeros((T, Cn, n, n), dtype=torch.complex64, device="cuda")
    cshape = (T, Cn, n, n) if mode == capi.COUNTERS_PER_IMAGE else (Cn, n, n)
    counters = torch.zeros(cshape, dtype=torch.float32, device="cuda")
    ws = None
    if ws_images is not None:
        nb = vis.shape[2]
        n_ant = int(round((-1 + np.sqrt(1 + 8 * nb)) / 2))
        ws = torch.empty(im.gridding_sorted_workspace_bytes(n_ant, n, ws_images), dtype=torch.uint8,
                         device="cuda")
    im.gridding_sorted(dev(vis), dev(u), dev(v), dev(flags), dev(freqs), du, dv, n, min_uv, pol, grids,
                       counters, counter_mode=mode, n_uvw_sets=n_uvw_sets, workspace=ws)
    return grids.cpu().numpy(), counters.cpu().numpy()


def _bits(g_gpu_c64):
    return np.ascontiguousarray(g_gpu_c64).view(np.uint32)


def _assert_bit_identical(g_gpu, g_ref_f32):
    a = _bits(g_gpu).reshape(-1)
    b = np.ascontiguousarray(g_ref_f32, np.float32).view(np.uint32).reshape(-1)
    diff = np.flatnonzero(a != b)
    assert diff.size == 0, f"{diff.size} words differ, first at {diff[:5]}"


@pytest.mark.parametrize("pol", ["XX", "YY", "I", "V"])
@pytest.mark.parametrize("min_uv", [-1000.0, 3.0])
def test_sorted_bit_identical_to_oracle(im, pol, min_uv):
    obs = synth.small(seed=31, n_ant=40, n_intervals=3, n_channels=4, n_pixels=128)
    vis = obs.vis_f32().copy()
    vis[0, 1, 17, 0, 0] = np.nan
    vis[1, 0, 23, 3, 1] = np.inf
    vis[2, 3, 40, 0, 1] = 3e12
    vis[2, 2, 41, 1, 0] = -np.inf   # XY: reaches V only
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, 128), O.delta_uv(2.0, vmax, 128)
    g_ref, c_ref, _ = O.gridding(vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 128, min_uv, pol,
                                 n_uvw_sets=3)
    g, c = _grid_sorted(im, vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 128, min_uv, pol, 3)
    assert np.array_equal(c, c_ref)
    _assert_bit_identical(g, g_ref)
    _, c0 = _grid_sorted(im, vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 128, min_uv, pol, 3,
                         mode=capi.COUNTERS_FIRST_INTERVAL)
    assert np.array_equal(c0, c_ref[0])


def test_sorted_crowded_cells(im):
    """Short baselines piled into a few cells: segments of hundreds of points take the
    block-per-cell path, which must give the same bits as the loop."""
    n_ant, n = 64, 64
    nb = n_ant * (n_ant + 1) // 2
    rng = np.random.default_rng(5)
    u = rng.uniform(-1.4, 1.4, nb).astype(np.float32)   # |u|,|v| < 1.5 cells: 9 cells
    v = rng.uniform(-1.4, 1.4, nb).astype(np.float32)
    u[:50] = 0.0
    v[:50] = 0.0                                        # direct and conjugate share cell 0
    u[60], v[60] = 30.0, 20.0
    flags = np.zeros(nb, np.int32)
    flags[::97] = 1
    freqs = np.array([299792458.0, 150e6])
    vis = (rng.standard_normal((2, 2, nb, 4, 2)) * 10).astype(np.float32)
    g_ref, c_ref, _ = O.gridding(vis, u, v, flags, freqs, 1.0, 1.0, n, -1000.0, "I")
    assert c_ref.max() > 200
    g, c = _grid_sorted(im, vis, u, v, flags, freqs, 1.0, 1.0, n, -1000.0, "I", 1)
    assert np.array_equal(c, c_ref)
    _assert_bit_identical(g, g_ref)


def test_sorted_long_segments_both_paths(im):
    """Segments longer than the shared-memory sort holds (8,192 points: about 19,500 points on
    the centre cell, ordered by counting ranks) beside segments of about 1,400 points (sorted in
    shared memory) and short ones: the same bits as the loop, counters exact."""
    n_ant, n = 180, 64
    nb = n_ant * (n_ant + 1) // 2
    rng = np.random.default_rng(11)
    u = rng.uniform(-1.4, 1.4, nb).astype(np.float32)
    v = rng.uniform(-1.4, 1.4, nb).astype(np.float32)
    centre = rng.random(nb) < 0.6
    u[centre] = 0.0
    v[centre] = 0.0
    far = rng.choice(nb, 40, replace=False)
    u[far] = rng.uniform(-25, 25, 40).astype(np.float32)
    v[far] = rng.uniform(-25, 25, 40).astype(np.float32)
    flags = np.zeros(nb, np.int32)
    flags[::131] = 1
    freqs = np.array([299792458.0, 150e6])
    vis = (rng.standard_normal((1, 2, nb, 4, 2)) * 10).astype(np.float32)
    g_ref, c_ref, _ = O.gridding(vis, u, v, flags, freqs, 1.0, 1.0, n, -1000.0, "XX")
    assert c_ref.max() > 8192 and np.sort(c_ref.reshape(-1))[-2] > 1000
    g, c = _grid_sorted(im, vis, u, v, flags, freqs, 1.0, 1.0, n, -1000.0, "XX", 1)
    assert np.array_equal(c, c_ref)
    _assert_bit_identical(g, g_ref)


def test_sorted_reference_golden_bits(im):
    """The reference's own CPU grids (golden vectors from its gridding loop) come out bit for
    bit from the reference's corrected visibilities."""
    g = np.load(os.path.join(GOLD, "imager_run.npz"))
    meta = ast.literal_eval(str(g["meta"]))
    pols = ["XX", "YY", "I", "V"]
    checked = 0
    for name, m in meta.items():
        if m.get("weighting") == "U" or m.get("kernel"):
            continue
        vis_c = g[f"{name}__vis_out"]
        Cn = vis_c.shape[1]
        freqs = (np.full(Cn, m["freq_override_mhz"] * 1e6) if "freq_override_mhz" in m else g["freqs_cotter"])
        flags = O.update_flags(len(g["cable"]), m.get("flagged", (3,)))
        du, dv = g[f"{name}__scalars"][:2]
        gr, c = _grid_sorted(im, vis_c, g["u"], g["v"], flags, freqs, du, dv, m["n_pixels"],
                             m.get("min_uv", -1000.0), pols[m["pol"]], 1)
        assert np.array_equal(c, g[f"{name}__counters"]), name
        _assert_bit_identical(gr, g[f"{name}__grids"])
        checked += 1
    assert checked > 0


def test_sorted_repeatable_and_chunked(im):
    """Same bits on every run, whatever the workspace (one image per chunk or all at once),
    and within summation-order error of the atomic gridder."""
    obs = synth.small(seed=7, n_ant=96, n_intervals=2, n_channels=5, n_pixels=256)
    vis = obs.vis_f32()
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, 256), O.delta_uv(2.0, vmax, 256)
    args = (vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 256, -1000.0, "XX", 2)
    g1, c1 = _grid_sorted(im, *args)
    g2, c2 = _grid_sorted(im, *args, ws_images=1)
    g3, _ = _grid_sorted(im, *args, ws_images=3)
    assert np.array_equal(_bits(g1), _bits(g2)) and np.array_equal(_bits(g1), _bits(g3))
    assert np.array_equal(c1, c2)
    ga = torch.zeros_like(torch.from_numpy(g1)).cuda()
    im.gridding(dev(vis), dev(obs.u), dev(obs.v), dev(obs.flags), dev(obs.freqs), du, dv, 256, -1000.0,
                "XX", ga, None, n_uvw_sets=2)
    ga = ga.cpu().numpy()
    assert np.abs(ga - g1).max() <= 1e-5 * np.abs(g1).max()


def test_sorted_workspace_errors(im):
    obs = synth.small(seed=1, n_ant=8, n_intervals=1, n_channels=2, n_pixels=32)
    vis = dev(obs.vis_f32())
    grids = torch.zeros((1, 2, 32, 32), dtype=torch.complex64, device="cuda")
    args = (vis, dev(obs.u), dev(obs.v), dev(obs.flags), dev(obs.freqs), 1.0, 1.0, 32, -1.0, "XX", grids)
    per = im.gridding_sorted_workspace_bytes(8, 32, 1)
    small = torch.empty(per - 1, dtype=torch.uint8, device="cuda")
    with pytest.raises(capi.BgiError):
        im.gridding_sorted(*args, workspace=small)
    odd = torch.empty(per + 64, dtype=torch.uint8, device="cuda")[8:]
    with pytest.raises(capi.BgiError):
        im.gridding_sorted(*args, workspace=odd)


def test_deterministic_imager(im):
    """bgi_image in deterministic mode: the images match the oracle within the image
    tolerance, and are the same bits across runs, wave sizes and the host entry point."""
    n = 128
    obs = synth.small(seed=43, n_ant=40, n_intervals=2, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    _, _, counters, ref, _ = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, obs.flags, obs.freqs, n,
                                             pol="I", n_uvw_sets=2)
    outs = []
    for wave in (0, 1, 4):
        h = im.Imager(n, 2.0, "I", -1000.0, max_images_per_wave=wave)
        h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
        h.set_frequencies(obs.freqs)
        assert h.half_plane
        extent = h.uv_extent
        h.set_deterministic(True)
        # the ordered gridder sums the half plane's cells, and the passes stay pruned
        assert h.half_plane and h.uv_extent == extent
        a = h.image(dev(vis)).cpu().numpy()
        b = h.image(dev(vis)).cpu().numpy()
        assert np.array_equal(_bits(a), _bits(b))
        c = h.image_host(np.ascontiguousarray(vis))
        assert np.array_equal(_bits(a), _bits(c))
        assert np.array_equal(h.weight_sums(6), counters.reshape(6, -1).sum(1).astype(np.uint32))
        h.close()
        outs.append(a)
    for a in outs[1:]:
        assert np.array_equal(_bits(a), _bits(outs[0]))
    a = outs[0]
    for i in range(a.shape[0]):
        for j in range(a.shape[1]):
            d = np.asarray(a[i, j], np.complex128) - ref[i, j]
            assert np.linalg.norm(d) / np.linalg.norm(ref[i, j]) < 1e-4, (i, j)
