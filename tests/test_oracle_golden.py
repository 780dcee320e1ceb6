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
