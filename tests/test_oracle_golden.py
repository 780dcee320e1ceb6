"""The oracle against golden vectors made by the reference imager's own CPU code
(tests/golden/make_golden.py) and against the reference tests' known answers."""
import ast
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
POLS = ["XX", "YY", "I", "V"]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_corrections_bit_exact(oracle_lib):
    O = oracle_lib
    g = np.load(os.path.join(GOLD, "corrections.npz"))
    a = g["vis"].copy()
    O.apply_geometric(a, g["w"], g["freqs"])
    assert np.array_equal(_bits(a), _bits(g["after_geometric"]))
    b = g["vis"].copy()
    O.apply_cable(b, g["cable"], g["freqs"])
    assert np.array_equal(_bits(b), _bits(g["after_cable"]))


@pytest.fixture(scope="module")
def run_gold():
    g = np.load(os.path.join(GOLD, "imager_run.npz"))
    meta = ast.literal_eval(str(g["meta"]))
    return g, meta


def test_imager_run_golden(oracle_lib, run_gold):
    """CPacerImager::run(): corrected visibilities, grids and counters bit-exact, delta_u/v
    exact, FP64 images within 1e-6 relative L2 of the reference's (FP32-rounded) images."""
    O = oracle_lib
    g, meta = run_gold
    flags_default = O.update_flags(len(g["cable"]), [3])
    for name, m in meta.items():
        vis = g["vis_bad"] if name.endswith("_bad") else g["vis"]
        T, Cn = vis.shape[:2]
        if "freq_override_mhz" in m:
            freqs = np.full(Cn, m["freq_override_mhz"] * 1e6)
        else:
            freqs = g["freqs_cotter"]
        flags = O.update_flags(len(g["cable"]), m.get("flagged", (3,))) if "flagged" in m else flags_default
        geom = m.get("geom", 1)
        cab = m.get("cable", 1)
        pol = POLS[m["pol"]]
        n = m["n_pixels"]
        vis_c, grids, counters, images, (du, dv) = O.full_pipeline(
            vis, g["u"][None], g["v"][None], g["w"][None], g["cable"], flags, freqs, n,
            min_uv=m.get("min_uv", -1000.0), pol=pol, apply_geom=geom, apply_cable_corr=cab)
        sc = g[f"{name}__scalars"]
        assert du == sc[0] and dv == sc[1], name
        assert np.array_equal(_bits(vis_c), _bits(g[f"{name}__vis_out"])), name
        if m.get("kernel"):  # Kaiser-Bessel convolutional gridding (src/pacer_imager.cpp:378-403, 565-750)
            grids, counters, _ = O.gridding_kb(vis_c, g["u"][None], g["v"][None], flags, freqs, du, dv, n,
                                               m["kernel"], m.get("min_uv", -1000.0), pol)
            images = O.image_f64(grids, counters)
        if m.get("weighting") == "U":
            grids, counters, _ = O.gridding(vis_c, g["u"][None], g["v"][None], flags, freqs, du, dv, n,
                                            m.get("min_uv", -1000.0), pol, uniform=True)
            ref = g[f"{name}__grids"]
            assert np.array_equal(np.isnan(grids), np.isnan(ref)), name
            ok = ~np.isnan(ref)
            assert np.array_equal(_bits(grids[ok]), _bits(ref[ok])), name
            continue
        assert np.array_equal(_bits(grids), _bits(g[f"{name}__grids"])), name
        assert np.array_equal(counters, g[f"{name}__counters"]), name
        ref_img = g[f"{name}__images"].view(np.complex64)[..., 0]
        err = np.linalg.norm(images - ref_img) / np.linalg.norm(images)
        assert err < 1e-6, (name, err)


def test_fft_shift_known_answers(oracle_lib):
    """tests/imager_test.cpp:21-40 of the reference, plus the reference's outputs on more shapes."""
    O = oracle_lib
    x = np.array([[0, 1], [2, 3]], np.complex64)
    assert np.array_equal(O.fft_shift(x).ravel(), np.array([3, 2, 1, 0], np.complex64))
    x = np.arange(6, dtype=np.complex64).reshape(2, 3)
    assert np.array_equal(O.fft_shift(x).ravel(), np.arange(6)[::-1].astype(np.complex64))
    g = np.load(os.path.join(GOLD, "fft_shift.npz"))
    for k in g.files:
        if k.startswith("in_"):
            assert np.array_equal(O.fft_shift(g[k]), g["out_" + k[3:]]), k


def test_fft_against_numpy(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(5)
    for n in (8, 12, 64):
        z = rng.standard_normal((2, n, n)) + 1j * rng.standard_normal((2, n, n))
        ref = np.fft.ifft2(z) * n * n
        assert np.abs(O.fft2_inverse_f64(z) - ref).max() < 1e-10 * n * n


def test_vector_sum_and_average(oracle_lib):
    """tests/gpu_utils_test.cpp:20-58 and :91-125 of the reference, on the oracle."""
    O = oracle_lib
    rng = np.random.default_rng(0)
    data = rng.integers(0, 50, (5, 3000)).astype(np.float32)
    assert np.array_equal(O.vector_sum(data, 3000, 5), data.sum(1).astype(np.float64))
    n_pix = 512 * 512
    img = np.tile((np.arange(n_pix) % 100).astype(np.complex64), (4, 1))
    assert np.array_equal(O.image_average(img), (np.arange(n_pix) % 100).astype(np.complex64))


def test_cell_index_edges(oracle_lib):
    """calculate_pos (src/gpu/gridding_gpu.cpp:24-54): wrap of negative pixels, min_uv cut."""
    O = oracle_lib
    c = 299792458.0
    lam = 2.0
    # u_lambda = 10, du = 1 -> u_pix 10; conjugate -> N - 10
    assert O.cell_index(20.0, 0.0, 1.0, 1.0, lam, -1000.0, 64, +1) == 10
    assert O.cell_index(20.0, 0.0, 1.0, 1.0, lam, -1000.0, 64, -1) == 64 - 10
    assert O.cell_index(0.0, 20.0, 1.0, 1.0, lam, -1000.0, 64, -1) == 64 * 54
    # uv distance exactly min_uv is cut (strict >)
    assert O.cell_index(20.0, 0.0, 1.0, 1.0, lam, 10.0, 64, +1) == -1
    # half-way rounds away from zero: 2.5 -> 3, -2.5 -> -3
    assert O.cell_index(5.0, 0.0, 1.0, 1.0, lam, -1.0, 64, +1) == 3
    assert O.cell_index(-5.0, 0.0, 1.0, 1.0, lam, -1.0, 64, +1) == 64 - 3
    del c


def test_compress_encoders_round_to_nearest_even(oracle_lib):
    """The storage oracle's 16-bit encoders (oracle/blink_compress.c) agree with numpy's
    binary16 and torch's bfloat16 conversions (both round to nearest even): a block whose
    largest component is 1.0 stores x / 1.0 = x."""
    O = oracle_lib
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    n = 128 * 64
    x = (rng.standard_normal(n * 8) * 10.0 ** rng.integers(-9, 1, n * 8)).astype(np.float32)
    x = np.clip(x, -0.999, 0.999)
    x[:16] = np.float32([6.1035156e-05, 6.097555e-05, 5.9604645e-08, 2.9802322e-08, 2.9802326e-08,
                         8.9406967e-08, 0.5, -0.5, 1e-30, -1e-30, 0.0, -0.0, 0.33333334, 2.0 ** -14,
                         2.0 ** -24 * 1.5, 2.0 ** -24 * 2.5])
    vis = x.reshape(1, 1, n, 4, 2).copy()
    vis[0, 0, ::128, :, 0] = 1.0  # every block's max is exactly 1
    for fmt in ("fp16", "bf16"):
        data, scales = O.compress(vis, fmt)
        assert np.all(scales == 1.0)
        planar = np.ascontiguousarray(vis[0, 0].transpose(1, 0, 2))  # [4][B][2]
        if fmt == "fp16":
            want = planar.astype(np.float16).view(np.uint16)
        else:
            want = torch.from_numpy(planar).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
        assert np.array_equal(data[0, 0], want), fmt
        back = O.decompress(data, scales, fmt)
        ref = want.view(np.float16).astype(np.float32) if fmt == "fp16" else \
            torch.from_numpy(want.view(np.int16)).view(torch.bfloat16).float().numpy()
        assert np.array_equal(back[0, 0].transpose(1, 0, 2), ref), fmt


def test_compress_s16_known_answers(oracle_lib):
    """S16: scale = max/32767, elements rint(x/scale) clamped, invalid components -32768
    and decoded as NaN, an all-zero block has scale 0."""
    O = oracle_lib
    vis = np.zeros((1, 1, 130, 4, 2), np.float32)
    vis[0, 0, 0, 0] = (3.0, -1.5)
    vis[0, 0, 1, 0] = (np.nan, 0.75)
    vis[0, 0, 2, 0] = (2e12, 1.0)
    vis[0, 0, 129, 0] = (-4.0, 0.0)   # second block of the XX plane
    data, scales = O.compress(vis, "s16")
    assert scales.shape == (1, 1, 4, 2)
    assert scales[0, 0, 0, 0] == np.float32(3.0) / np.float32(32767.0)
    assert scales[0, 0, 1, 0] == 0.0 and scales[0, 0, 0, 1] == np.float32(4.0) / np.float32(32767.0)
    e = data[0, 0, 0].view(np.int16)
    assert e[0, 0] == 32767 and e[0, 1] in (-16384, -16383)
    assert e[1, 0] == -32768 and e[2, 0] == -32768
    assert e[129, 0] == -32767
    back = O.decompress(data, scales, "s16")
    assert np.isnan(back[0, 0, 1, 0, 0]) and np.isnan(back[0, 0, 2, 0, 0])
    assert back[0, 0, 0, 0, 0] == np.float32(32767) * scales[0, 0, 0, 0]


def test_ingest_matrices_known_answer(oracle_lib):
    """ConvertFits2XCorr's mapping (apps/pacer_imager_main.cpp:720-804): element (i, j), j <= i,
    of the XX matrix is baseline i(i+1)/2 + j, pol 0; YY goes to pol 3, zero without YY."""
    O = oracle_lib
    n = 3
    re = np.arange(9, dtype=np.float32).reshape(1, n, n)
    im = -re - 0.5
    vis = O.ingest_matrices(re, im)
    assert vis.shape == (1, 6, 4, 2)
    # baselines (0,0) (1,0) (1,1) (2,0) (2,1) (2,2) -> matrix elements 0, 3, 4, 6, 7, 8
    assert np.array_equal(vis[0, :, 0, 0], np.float32([0, 3, 4, 6, 7, 8]))
    assert np.array_equal(vis[0, :, 0, 1], np.float32([0, 3, 4, 6, 7, 8]) * -1 - 0.5)
    assert not vis[0, :, 1:, :].any()
    vis_yy = O.ingest_matrices(re, im, re * 2, im * 2)
    assert np.array_equal(vis_yy[0, :, 3, 0], 2 * vis[0, :, 0, 0])
    assert not vis_yy[0, :, 1:3, :].any()


def test_pointed_uvw_golden(oracle_lib):
    """Pointed UVW of the oracle against the reference's own geometry routines
    (src/pacer_geometry.h, src/antenna_positions.cpp:57-89), bit for bit."""
    O = oracle_lib
    g = np.load(os.path.join(GOLD, "pointed_uvw.npz"))
    steps = np.stack([O.uvw_step(g["rmat"][t], g["ha2000"][t], g["dec_aber"][t], g["lmst"][t], g["lmst2000"][t])
                      for t in range(len(g["ha2000"]))])
    # the sines and cosines come from this host's libm; the pin is on the reference's libm values
    np.testing.assert_allclose(steps, g["steps"], rtol=0, atol=1e-15)
    u, v, w = O.pointed_uvw(g["xyz"], g["steps"])
    for a, b in ((u, g["u"]), (v, g["v"]), (w, g["w"])):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_cpu_runnable_plain_case_against_reference_build(oracle_lib):
    """The oracle against the reference's own CPU imager (CPacerImager::run,
    src/pacer_imager.cpp:440-526, compiled from its sources with the stand-ins in oracle/ref_shim)
    on the CPU-runnable plain case: 256 antennas in a 35 m disk, one channel at 159.375 MHz, one
    interval, 256 x 256, both corrections.  Corrected visibilities, grids and counters are the
    same bits; images agree to FP32-vs-FP64 transform rounding.  Needs the reference build
    (oracle/_ref, made only where the reference checkout is found); skipped elsewhere."""
    O = oracle_lib
    ref = O.ref_library()
    if ref is None:
        pytest.skip("reference CPU build (oracle/_ref) not present")
    from imager_gb300 import synth
    obs = synth.config1()
    vis = np.ascontiguousarray(obs.vis_f32())
    T, Cn, nb = vis.shape[:3]
    n = obs.n_pixels
    npix = n * n * T * Cn
    vout = np.zeros(vis.size, np.float32)
    g = np.zeros(npix * 2, np.float32)
    c = np.zeros(npix, np.float32)
    im = np.zeros(npix * 2, np.float32)
    sc = np.zeros(4)
    no_flagged = np.zeros(1, np.int32)  # the case flags only the autocorrelations
    ref.ref_set_kernel_size(0)
    # obsInfo fields are unused with the frequency override (159.375 MHz)
    ref.ref_run(vis.reshape(-1), T, Cn, obs.n_ant, np.ascontiguousarray(obs.u[0]),
                np.ascontiguousarray(obs.v[0]), np.ascontiguousarray(obs.w[0]), obs.cable, no_flagged, 0,
                0.04, 4, 1.28, 118, 159.375, n, 2.0, -1000.0, 0, b"N", 1, 1, vout, g, c, im, sc)
    flags = O.update_flags(obs.n_ant, [])
    assert np.array_equal(flags, obs.flags)
    vis_c, grids, counters, images, (du, dv) = O.full_pipeline(vis, obs.u, obs.v, obs.w, obs.cable, flags,
                                                               obs.freqs, n)
    assert du == sc[0] and dv == sc[1]
    assert np.array_equal(_bits(vis_c.reshape(-1)), _bits(vout))
    assert np.array_equal(_bits(grids.reshape(-1)), _bits(g))
    assert np.array_equal(counters.reshape(-1), c)
    ref_img = im.view(np.complex64).reshape(n, n)
    err = np.linalg.norm(images[0, 0] - ref_img) / np.linalg.norm(images[0, 0])
    assert err < 1e-6, err


def test_fp32_fft_blocked_equals_scalar(oracle_lib):
    """The CPU baseline's FP32 2D transform, blocked over 16 lines with a vectorisable inner loop
    and its radix-2 stages taken two at a time, gives the same bits as the one-line-at-a-time form
    (same butterflies, order and twiddles), for even and odd stage counts, for batches below and
    above the thread count, and matches numpy to FP32 rounding."""
    O = oracle_lib
    lib = O.library()
    rng = np.random.default_rng(5)
    for n, batch in ((2, 1), (8, 2), (16, 1), (32, 5), (64, 3), (512, 1), (256, 40)):
        x = rng.standard_normal((batch, n, n, 2)).astype(np.float32)
        a = np.empty_like(x)
        b = np.empty_like(x)
        lib.bgo_fft2_inverse_f32(x.reshape(-1), a.reshape(-1), n, batch)
        lib.bgo_fft2_inverse_f32_scalar(x.reshape(-1), b.reshape(-1), n, batch)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (n, batch)
        ref = np.fft.ifft2(x[..., 0].astype(np.float64) + 1j * x[..., 1]) * n * n
        got = a[..., 0] + 1j * a[..., 1]
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-6 * np.log2(n), (n, batch)
