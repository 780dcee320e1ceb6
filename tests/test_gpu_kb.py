"""Kaiser-Bessel convolutional gridding on the GPU (bgi_gridding_kb_gpu and the handle's
kernel mode) against the oracle's restatement of the reference's CPU gridder and against the
reference's own KB grids and images.  Counters exactly; grids to float summation order (the
reference sums double products into float cells, the GPU float products with atomics); images
within the 1e-4 image tolerance."""
import ast
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GRID_TOL = 2e-5   # of the grid's largest cell


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
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _grid_kb(im, vis, u, v, flags, freqs, du, dv, n, k, min_uv, pol, n_uvw_sets, with_sinc=True):
    T, Cn = vis.shape[:2]
    grids = torch.zeros((T, Cn, n, n), dtype=torch.complex64, device="cuda")
    counters = torch.zeros((T, Cn, n, n), dtype=torch.float32, device="cuda")
    im.gridding_kb(dev(vis), dev(u), dev(v), dev(flags), dev(freqs), du, dv, n, min_uv, pol, grids, counters,
                   kernel_size=k, with_sinc=with_sinc, n_uvw_sets=n_uvw_sets)
    return grids.cpu().numpy(), counters.cpu().numpy()


def _check(g, c, g_ref, c_ref):
    ref = np.ascontiguousarray(g_ref).view(np.complex64)[..., 0]
    assert np.array_equal(c, c_ref)
    assert np.abs(g - ref).max() <= GRID_TOL * np.abs(ref).max()


@pytest.mark.parametrize("k,pol,min_uv,sinc", [(7, "XX", -1000.0, True), (10, "I", -1000.0, True),
                                               (11, "V", 3.0, True), (5, "YY", -1000.0, False)])
def test_kb_grids_against_oracle(im, k, pol, min_uv, sinc):
    obs = synth.small(seed=101, n_ant=40, n_intervals=2, n_channels=3, n_pixels=64)
    vis = obs.vis_f32()
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, 64), O.delta_uv(2.0, vmax, 64)
    g_ref, c_ref, _ = O.gridding_kb(vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 64, k, min_uv, pol,
                                    n_uvw_sets=2, with_sinc=sinc)
    g, c = _grid_kb(im, vis, obs.u, obs.v, obs.flags, obs.freqs, du, dv, 64, k, min_uv, pol, 2, sinc)
    _check(g, c, g_ref, c_ref)


def test_kb_against_reference_golden(im):
    """The reference's own KB grids (its CPU code with m_nConvolvingKernelSize set) from its
    corrected visibilities; and its images through the handle (48 pixels included)."""
    g = np.load(os.path.join(GOLD, "imager_run.npz"))
    meta = ast.literal_eval(str(g["meta"]))
    pols = ["XX", "YY", "I", "V"]
    checked = images = 0
    for name, m in meta.items():
        if not m.get("kernel"):
            continue
        Cn = g[f"{name}__vis_out"].shape[1]
        freqs = g["freqs_cotter"]
        flags = O.update_flags(len(g["cable"]), m.get("flagged", (3,)))
        du, dv = g[f"{name}__scalars"][:2]
        n, k, pol = m["n_pixels"], m["kernel"], pols[m["pol"]]
        gr, c = _grid_kb(im, g[f"{name}__vis_out"], g["u"], g["v"], flags, freqs, du, dv, n, k,
                         m.get("min_uv", -1000.0), pol, 1)
        _check(gr, c, g[f"{name}__grids"], g[f"{name}__counters"])
        checked += 1
        h = im.Imager(n, 2.0, pol, m.get("min_uv", -1000.0))
        h.set_array(g["u"], g["v"], g["w"], flags, g["cable"])
        h.set_frequencies(freqs[:Cn])
        h.set_gridding_kernel(k)
        out = h.image(dev(g["vis"])).cpu().numpy()
        ref = g[f"{name}__images"].view(np.complex64)[..., 0]
        for i in range(out.shape[0]):
            for j in range(out.shape[1]):
                assert rel_l2(out[i, j], ref[i, j]) < 1e-4, (name, i, j)
        h.close()
        images += 1
    assert checked == 3 and images == 3  # the 48-pixel case on the mixed-radix passes


def test_kb_imager_against_oracle(im):
    n, k = 128, 7
    obs = synth.small(seed=102, n_ant=48, n_intervals=2, n_channels=3, n_pixels=n)
    vis = obs.vis_f32()
    corr = vis.copy()
    O.apply_geometric(corr, obs.w, obs.freqs, n_uvw_sets=2)
    O.apply_cable(corr, obs.cable, obs.freqs)
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, n), O.delta_uv(2.0, vmax, n)
    g_ref, c_ref, _ = O.gridding_kb(corr, obs.u, obs.v, obs.flags, obs.freqs, du, dv, n, k, -1000.0, "XX", n_uvw_sets=2)
    ref = O.image_f64(g_ref, c_ref)
    h = im.Imager(n, 2.0, "XX", -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    h.set_gridding_kernel(k)
    out = h.image(dev(vis)).cpu().numpy()
    for i in range(2):
        for j in range(3):
            assert rel_l2(out[i, j], ref[i, j]) < 1e-4, (i, j)
    assert np.array_equal(h.weight_sums(6), c_ref.reshape(6, -1).sum(1).astype(np.uint32))
    h.set_deterministic(True)
    with pytest.raises(capi.BgiError) as e:
        h.image(dev(vis))
    assert e.value.status == capi.ERR_UNSUPPORTED
    h.set_deterministic(False)
    h.set_gridding_kernel(0)  # back to nearest neighbour
    nn = h.image(dev(vis)).cpu().numpy()
    assert rel_l2(nn, out) > 1e-3
    with pytest.raises(capi.BgiError):
        h.set_gridding_kernel(17)
    h.close()


def test_kb_free_function_on_concurrent_streams(im):
    """Calls with different kernel sizes issued on two streams at once each use their own
    kernel table (stream-ordered memory of the call): the same counters and grids as alone."""
    obs = synth.small(seed=103, n_ant=40, n_intervals=1, n_channels=2, n_pixels=64)
    vis = dev(obs.vis_f32())
    umax, vmax = O.uv_max(obs.u, obs.v, obs.flags)
    du, dv = O.delta_uv(2.0, umax, 64), O.delta_uv(2.0, vmax, 64)
    args = [dev(a) for a in (obs.u, obs.v, obs.flags, obs.freqs)]
    alone = {k: _grid_kb(im, obs.vis_f32(), obs.u, obs.v, obs.flags, obs.freqs, du, dv, 64, k, -1000.0, "XX", 1)
             for k in (5, 11)}
    streams = {k: torch.cuda.Stream() for k in (5, 11)}
    outs = {}
    for rep in range(3):
        for k in (5, 11):
            g = torch.zeros((1, 2, 64, 64), dtype=torch.complex64, device="cuda")
            c = torch.zeros((1, 2, 64, 64), dtype=torch.float32, device="cuda")
            streams[k].wait_stream(torch.cuda.current_stream())  # inputs and zeroed outputs ready
            im.gridding_kb(vis, *args, du, dv, 64, -1000.0, "XX", g, c, kernel_size=k, stream=streams[k])
            outs[(rep, k)] = (g, c)
    torch.cuda.synchronize()
    for (rep, k), (g, c) in outs.items():
        assert np.array_equal(c.cpu().numpy(), alone[k][1]), (rep, k)
        ref = alone[k][0]
        assert np.abs(g.cpu().numpy() - ref).max() <= GRID_TOL * np.abs(ref).max(), (rep, k)
