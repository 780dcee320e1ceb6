"""Uneven batches replayed as one CUDA graph (bgi_batch_*): items of different image sizes,
pols, storage formats and arrays, one imager used twice; every replay writes the images that
the same calls made one by one write (bit for bit with the ordered gridder)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    from imager_gb300 import imager
    return imager


def _imager(im, obs, pol, wave=0):
    h = im.Imager(obs.n_pixels, 2.0, pol, max_images_per_wave=wave)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    h.set_deterministic(True)
    return h


def test_batch_replays_match_direct_calls(im):
    obs = [synth.small(seed=81, n_ant=40, n_intervals=2, n_channels=3, n_pixels=128),
           synth.small(seed=82, n_ant=64, n_intervals=1, n_channels=2, n_pixels=256),
           synth.small(seed=83, n_ant=24, n_intervals=3, n_channels=4, n_pixels=64)]
    pols = ["XX", "I", "V"]
    hs = [_imager(im, o, p, wave=2) for o, p in zip(obs, pols)]
    vis = [torch.from_numpy(o.vis_f32()).cuda() for o in obs]
    d1, s1 = im.compress_visibilities(vis[1], "s16")
    vis0b = torch.from_numpy(synth.small(seed=84, n_ant=40, n_intervals=2, n_channels=3,
                                         n_pixels=128).vis_f32()).cuda()
    items = [dict(imager=hs[0], data=vis[0]),
             dict(imager=hs[1], data=d1, scales=s1, fmt="s16"),
             dict(imager=hs[2], data=vis[2], flags=im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.OUTPUT_REAL),
             dict(imager=hs[0], data=vis0b)]  # the same imager again: chained after the first item
    direct = [hs[0].image(vis[0]).cpu().numpy(),
              hs[1].image_compressed(d1, s1, "s16").cpu().numpy(),
              hs[2].image(vis[2], flags=im.APPLY_GEOMETRIC | im.APPLY_CABLE | im.OUTPUT_REAL).cpu().numpy(),
              hs[0].image(vis0b).cpu().numpy()]
    b = im.Batch(items)
    for rep in range(2):
        for out in b.outputs:
            out.zero_()
        b.launch()
        torch.cuda.synchronize()
        for k, out in enumerate(b.outputs):
            got = out.cpu().numpy()
            assert np.array_equal(got.view(np.uint32), direct[k].view(np.uint32)), (rep, k)
    b.close()
    for h in hs:
        h.close()


def test_batch_argument_checks(im):
    obs = synth.small(seed=85, n_ant=16, n_intervals=1, n_channels=2, n_pixels=64)
    h = _imager(im, obs, "XX")
    h.set_stage_timing(True)
    with pytest.raises(capi.BgiError):
        im.Batch([dict(imager=h, data=torch.from_numpy(obs.vis_f32()).cuda())])
    h.close()
