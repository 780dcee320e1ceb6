"""Correlation-matrix ingest (bgi_ingest_correlation_matrices) against the oracle's restatement
of ConvertFits2XCorr, bit for bit: complex64 records, and the 16-bit stored formats written in the
same pass (equal to encoding the oracle's records); with and without YY matrices."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from imager_gb300 import capi, synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def im():
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    capi.lib(build_if_missing=True)
    O.build()
    from imager_gb300 import imager
    return imager


def _matrices(seed, T, Cn, n):
    rng = np.random.default_rng(seed)
    m = [(rng.standard_normal((T, Cn, n, n)) * 10.0 ** rng.integers(-2, 3, (T, Cn, 1, 1))).astype(np.float32)
         for _ in range(4)]
    m[0][0, 0, 5, 2] = np.nan
    m[1][1, 2, 30, 7] = np.float32(2e12)
    return m


@pytest.mark.parametrize("with_yy", [True, False])
@pytest.mark.parametrize("fmt", ["c64", "s16", "bf16", "fp16"])
def test_ingest_bit_exact(im, fmt, with_yy):
    T, Cn, n = 2, 3, 37  # 703 baselines: the last scale block of each plane is partial
    rxx, ixx, ryy, iyy = _matrices(11, T, Cn, n)
    ref = O.ingest_matrices(rxx.reshape(-1, n, n), ixx.reshape(-1, n, n),
                            ryy.reshape(-1, n, n) if with_yy else None, iyy.reshape(-1, n, n) if with_yy else None)
    ref = ref.reshape(T, Cn, -1, 4, 2)
    dev = [torch.from_numpy(a).cuda() for a in (rxx, ixx, ryy, iyy)]
    out = im.ingest_correlation_matrices(dev[0], dev[1], dev[2] if with_yy else None, dev[3] if with_yy else None,
                                         fmt=fmt)
    if fmt == "c64":
        got = out.cpu().numpy().view(np.float32).reshape(ref.shape)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    else:
        d_ref, s_ref = O.compress(ref, fmt)
        d, s = out
        assert np.array_equal(s.cpu().numpy().view(np.uint32), s_ref.view(np.uint32))
        assert np.array_equal(d.cpu().numpy().view(np.uint16), d_ref)


def test_ingest_then_image(im):
    """Matrices -> s16 in one pass -> images equal (bit for bit, ordered gridder) to encoding the
    ingested records and imaging those."""
    obs = synth.small(seed=91, n_ant=32, n_intervals=1, n_channels=2, n_pixels=64)
    n, B = 32, obs.vis.shape[2]
    # the observation's XX and YY as full Hermitian correlation matrices
    i, j = np.tril_indices(n)
    mats = []
    for p in (0, 3):
        full = np.zeros((1, 2, n, n), np.complex64)
        full[:, :, i, j] = obs.vis[:, :, np.arange(B), p]
        mats += [np.ascontiguousarray(full.real), np.ascontiguousarray(full.imag)]
    dev = [torch.from_numpy(a).cuda() for a in mats]
    h = im.Imager(64, 2.0, "I")
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    h.set_deterministic(True)
    d1, s1 = im.ingest_correlation_matrices(*dev, fmt="s16")
    recs = im.ingest_correlation_matrices(*dev, fmt="c64")
    d2, s2 = im.compress_visibilities(recs, "s16")
    a = h.image_compressed(d1, s1, "s16").cpu().numpy()
    b = h.image_compressed(d2, s2, "s16").cpu().numpy()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    h.close()


@pytest.mark.parametrize("pol,fmt", [("XX", "s16"), ("I", "s16"), ("YY", "c64"), ("XX", "bf16")])
def test_image_correlation_matrices_host(im, pol, fmt):
    """bgi_image_correlation_matrices_host (host matrices uploaded and ingested chunk by chunk,
    then imaged) gives the same image bits as ingesting the same matrices on the device and
    imaging them (ordered gridder), over several chunks (waves of two images)."""
    obs = synth.small(seed=92, n_ant=32, n_intervals=3, n_channels=4, n_pixels=64)
    n, B = 32, obs.vis.shape[2]
    i, j = np.tril_indices(n)
    mats = []
    for p in (0, 3):
        full = np.zeros((3, 4, n, n), np.complex64)
        full[:, :, i, j] = obs.vis[:, :, np.arange(B), p]
        mats += [np.ascontiguousarray(full.real), np.ascontiguousarray(full.imag)]
    h = im.Imager(64, 2.0, pol)
    h.set_array(obs.u, obs.v, obs.w, obs.flags, obs.cable)
    h.set_frequencies(obs.freqs)
    h.set_deterministic(True)
    h.set_schedule(2, 2)
    host = h.image_matrices_host(*mats, fmt=fmt)
    dev = [torch.from_numpy(a).cuda() for a in mats]
    if fmt == "c64":
        ref = h.image(im.ingest_correlation_matrices(*dev, fmt="c64")).cpu().numpy()
    else:
        d, s = im.ingest_correlation_matrices(*dev, fmt=fmt)
        ref = h.image_compressed(d, s, fmt).cpu().numpy()
    assert np.array_equal(host.view(np.uint32), ref.view(np.uint32))
    # XX alone: the YY matrices are not needed (and not uploaded) for pol XX
    if pol == "XX":
        alone = h.image_matrices_host(mats[0], mats[1], fmt=fmt)
        assert np.array_equal(alone.view(np.uint32), ref.view(np.uint32))
    h.close()
