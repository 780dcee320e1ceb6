"""The device fault word: bounded waits on bulk asynchronous copies record a fault instead of
hanging.  The wait limit is exercised with a barrier nothing arrives on; the imaging kernels,
run normally, leave the word clear."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return capi.lib(build_if_missing=True)


def _fault(lib, clear=False):
    bits = C.c_uint(0xFFFF)
    assert lib.bgi_device_fault(0, C.byref(bits), int(clear)) == capi.OK
    return bits.value


def test_imaging_leaves_fault_word_clear(lib):
    from imager_gb300 import imager
    _fault(lib, clear=True)
    obs = synth.small(seed=2, n_ant=32, n_intervals=2, n_channels=4, n_pixels=256)
    h = imager.Imager(256, 2.0, "XX", -1000.0)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    assert h.half_plane
    out = h.image_host(np.ascontiguousarray(obs.vis_f32()))
    assert np.isfinite(out).all()
    assert _fault(lib) == 0
    h.close()


def test_bounded_wait_records_fault(lib):
    _fault(lib, clear=True)
    assert lib.bgi_selftest_wait_timeout(0, None) == capi.OK
    torch.cuda.synchronize()
    assert _fault(lib, clear=True) & 1
    assert _fault(lib) == 0
    # the context is still usable
    x = torch.ones(1024, device="cuda")
    assert float(x.sum()) == 1024.0
