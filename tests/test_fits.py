"""FITS output (bgi_write_fits, bgi_write_fits_block) on the host: files parsed back with a
small reader of the FITS standard (80-character cards in 2880-byte blocks, big-endian float32
pixels, NAXIS1 fastest), pixels compared bit for bit, header cards and error cases checked."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

from imager_gb300 import capi


@pytest.fixture(scope="module")
def im():
    if shutil.which("nvcc") is None and not os.path.exists(capi.library_path()):
        pytest.skip("nvcc not available to build the library")
    capi.lib(build_if_missing=True)
    from imager_gb300 import imager
    return imager


def read_fits(path):
    raw = open(path, "rb").read()
    assert len(raw) % 2880 == 0
    cards, pos = {}, 0
    order = []
    while True:
        card = raw[pos:pos + 80].decode("ascii")
        pos += 80
        assert len(card) == 80
        key = card[:8].strip()
        order.append(key)
        if key == "END":
            break
        assert card[8:10] == "= ", card
        value = card[10:].split(" / ")[0].strip()
        if value.startswith("'"):
            value = value.strip("'").rstrip()
        elif value in ("T", "F"):
            value = value == "T"
        elif any(ch in value for ch in ".E"):
            value = float(value)
        else:
            value = int(value)
        cards[key] = value
    data_start = (pos + 2879) // 2880 * 2880
    assert raw[pos:data_start] == b" " * (data_start - pos)
    nx, ny = cards["NAXIS1"], cards["NAXIS2"]
    data = np.frombuffer(raw[data_start:data_start + 4 * nx * ny], ">f4").reshape(ny, nx)
    assert raw[data_start + 4 * nx * ny:] == b"\0" * (len(raw) - data_start - 4 * nx * ny)
    return cards, order, data.astype(np.float32)


WCS = {"ra_deg": 123.25, "dec_deg": -26.703319, "pixscale_ra_deg": 0.0123456789, "pixscale_dec_deg": 0.0234567891}


def test_write_fits_real_image(im, tmp_path):
    rng = np.random.default_rng(5)
    img = rng.standard_normal((6, 10)).astype(np.float32)
    img[2, 3] = np.nan
    img[0, 0] = -0.0
    path = tmp_path / "one.fits"
    im.write_fits(path, img, WCS, freq_hz=159.375e6)
    cards, order, data = read_fits(path)
    assert order[:5] == ["SIMPLE", "BITPIX", "NAXIS", "NAXIS1", "NAXIS2"] and order[-1] == "END"
    assert cards["SIMPLE"] is True and cards["BITPIX"] == -32 and cards["NAXIS"] == 2
    assert (cards["NAXIS1"], cards["NAXIS2"]) == (10, 6)
    assert cards["CTYPE1"] == "RA---SIN" and cards["CTYPE2"] == "DEC--SIN"
    assert cards["CRVAL1"] == WCS["ra_deg"] and cards["CRVAL2"] == WCS["dec_deg"]
    assert cards["CDELT1"] == -WCS["pixscale_ra_deg"] and cards["CDELT2"] == WCS["pixscale_dec_deg"]
    assert (cards["CRPIX1"], cards["CRPIX2"]) == (6.0, 4.0)
    assert cards["FREQ"] == 159.375e6
    assert np.array_equal(data.view(np.uint32), img.view(np.uint32))


def test_write_fits_complex_block(im, tmp_path):
    rng = np.random.default_rng(6)
    block = (rng.standard_normal((2, 3, 4, 8)) + 1j * rng.standard_normal((2, 3, 4, 8))).astype(np.complex64)
    freqs = 150e6 + 1.28e6 * np.arange(3)
    im.write_fits_block(tmp_path, "dirty", block, WCS, freqs)
    names = sorted(os.listdir(tmp_path))
    assert names == [f"dirty_t{t:04d}_c{c:04d}.fits" for t in range(2) for c in range(3)]
    for t in range(2):
        for c in range(3):
            cards, _, data = read_fits(tmp_path / f"dirty_t{t:04d}_c{c:04d}.fits")
            assert (cards["INTERVAL"], cards["CHANNEL"]) == (t, c)
            assert cards["FREQ"] == freqs[c]
            assert np.array_equal(data, block[t, c].real)
    # no coordinates, no frequencies
    im.write_fits_block(tmp_path, "plain", block.real.copy(), None, None)
    cards, _, data = read_fits(tmp_path / "plain_t0001_c0002.fits")
    assert "CTYPE1" not in cards and "FREQ" not in cards
    assert np.array_equal(data, block[1, 2].real)


def test_write_fits_errors(im, tmp_path):
    lib = capi.lib()
    img = np.zeros((4, 4), np.float32)
    p = C.c_void_p(img.ctypes.data)
    assert lib.bgi_write_fits(None, p, 4, 4, 1, None, 0.0) == capi.ERR_INVALID
    assert lib.bgi_write_fits(str(tmp_path / "x.fits").encode(), p, 0, 4, 1, None, 0.0) == capi.ERR_INVALID
    assert lib.bgi_write_fits(str(tmp_path / "x.fits").encode(), p, 4, 4, 3, None, 0.0) == capi.ERR_INVALID
    bad = capi.ImageWcs(float("nan"), 0.0, 1.0, 1.0)
    assert lib.bgi_write_fits(str(tmp_path / "x.fits").encode(), p, 4, 4, 1, C.byref(bad), 0.0) == capi.ERR_INVALID
    assert lib.bgi_write_fits(str(tmp_path / "no_such_dir" / "x.fits").encode(), p, 4, 4, 1, None, 0.0) \
        == capi.ERR_INVALID
    assert b"cannot open" in lib.bgi_last_error()
    assert lib.bgi_write_fits_block(str(tmp_path).encode(), b"a/b", p, 1, 1, 4, 4, 1, None, None) == capi.ERR_INVALID
    assert lib.bgi_write_fits_block(str(tmp_path).encode(), b"a", p, 0, 1, 4, 4, 1, None, None) == capi.ERR_INVALID
    assert lib.bgi_get_image_wcs(None, 0.0, 0.0, None) == capi.ERR_INVALID
