"""Pointed-observation UVW on the device (bgi_pointed_uvw_gpu, bgi_set_array_pointed) against the
reference's own geometry routines (golden vectors), bit for bit, and imaging with it."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    from imager_gb300 import imager
    return imager


def test_pointed_uvw_bit_exact(im):
    g = np.load(os.path.join(GOLD, "pointed_uvw.npz"))
    u, v, w = im.pointed_uvw(torch.from_numpy(g["xyz"]).cuda(), torch.from_numpy(g["steps"]).cuda())
    for a, b in ((u, g["u"]), (v, g["v"]), (w, g["w"])):
        assert np.array_equal(a.cpu().numpy().view(np.uint32), b.view(np.uint32))


def test_imager_with_pointed_uvw(im):
    """A handle whose UVW is computed on the device images exactly as one given the same UVW."""
    g = np.load(os.path.join(GOLD, "pointed_uvw.npz"))
    n_ant, T = g["xyz"].shape[0], len(g["ha2000"])
    obs = synth.small(seed=111, n_ant=n_ant, n_intervals=T, n_channels=2, n_pixels=128)
    vis = torch.from_numpy(obs.vis_f32()).cuda()
    a = im.Imager(128, 2.0, "XX")
    a.set_array_pointed(g["xyz"], g["steps"], obs.flags, obs.cable)
    a.set_frequencies(obs.freqs)
    b = im.Imager(128, 2.0, "XX")
    b.set_array(g["u"], g["v"], g["w"], obs.flags, obs.cable)
    b.set_frequencies(obs.freqs)
    assert a.uv_cell == b.uv_cell
    for h in (a, b):
        h.set_deterministic(True)
    ia, ib = a.image(vis).cpu().numpy(), b.image(vis).cpu().numpy()
    assert np.array_equal(ia.view(np.uint32), ib.view(np.uint32))
    a.close()
    b.close()
