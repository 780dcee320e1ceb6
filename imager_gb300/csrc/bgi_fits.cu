// FITS output of dirty images (host code only).
//
// The reference hands its Images (pixels plus ra_deg, dec_deg and the pixel scales set at
// src/gpu/pacer_imager_hip.cpp:110-119 and src/pacer_imager.cpp:192-201) to astroio's
// Images::to_fits_files (apps/pacer_imager_main.cpp:578, tests/imager_test.cpp:57); astroio is
// an external library that is not part of the reference.  This writer follows the FITS
// standard (version 4.0): a primary HDU whose header is 80-character ASCII cards in
// 2880-byte blocks, then the pixels as big-endian IEEE float32 (BITPIX = -32), NAXIS1 (x)
// varying fastest, padded with zeros to a whole block.  The pixel scales go to CDELT1/2 as the
// reference's comments say, in a SIN projection about the fftshifted centre.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "bgi_internal.h"

namespace bgi {
namespace {

constexpr size_t kBlock = 2880;
constexpr size_t kCard = 80;

std::string pad_card(std::string s) {
    s.resize(kCard, ' ');
    return s;
}

// KEYWORD = value / comment, the value right-aligned to column 30 (fixed format)
std::string card_value(const char *key, const char *value, const char *comment) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "%-8.8s= %20s", key, value);
    std::string s(buf);
    if (comment && *comment) s += std::string(" / ") + comment;
    return pad_card(s);
}

std::string card_int(const char *key, long long v, const char *comment) {
    char val[32];
    std::snprintf(val, sizeof val, "%lld", v);
    return card_value(key, val, comment);
}

std::string card_real(const char *key, double v, const char *comment) {
    char val[32];
    std::snprintf(val, sizeof val, "%.13E", v);  // 20 characters at most
    return card_value(key, val, comment);
}

std::string card_logical(const char *key, bool v, const char *comment) { return card_value(key, v ? "T" : "F", comment); }

// KEYWORD = 'string  ' / comment: the quoted string starts in column 11, at least 8 characters
std::string card_string(const char *key, const char *v, const char *comment) {
    char buf[128];
    std::snprintf(buf, sizeof buf, "%-8.8s= '%-8s'", key, v);
    std::string s(buf);
    if (comment && *comment) s += std::string(" / ") + comment;
    return pad_card(s);
}

// interval, channel: written as INTERVAL and CHANNEL cards when >= 0
int write_one(const char *path, const float *image, int nx, int ny, int stride, const bgi_image_wcs *wcs,
              double freq_hz, int interval, int channel) {
    std::vector<std::string> cards;
    cards.push_back(card_logical("SIMPLE", true, "conforms to FITS standard"));
    cards.push_back(card_int("BITPIX", -32, "IEEE single precision"));
    cards.push_back(card_int("NAXIS", 2, nullptr));
    cards.push_back(card_int("NAXIS1", nx, "columns (x)"));
    cards.push_back(card_int("NAXIS2", ny, "rows (y)"));
    cards.push_back(card_string("BUNIT", "Jy/beam", nullptr));
    if (wcs) {
        cards.push_back(card_string("CTYPE1", "RA---SIN", nullptr));
        cards.push_back(card_real("CRVAL1", wcs->ra_deg, "phase centre RA (deg)"));
        cards.push_back(card_real("CRPIX1", nx / 2 + 1.0, "fftshifted centre"));
        cards.push_back(card_real("CDELT1", -wcs->pixscale_ra_deg, "deg per pixel"));
        cards.push_back(card_string("CUNIT1", "deg", nullptr));
        cards.push_back(card_string("CTYPE2", "DEC--SIN", nullptr));
        cards.push_back(card_real("CRVAL2", wcs->dec_deg, "phase centre Dec (deg)"));
        cards.push_back(card_real("CRPIX2", ny / 2 + 1.0, "fftshifted centre"));
        cards.push_back(card_real("CDELT2", wcs->pixscale_dec_deg, "deg per pixel"));
        cards.push_back(card_string("CUNIT2", "deg", nullptr));
        cards.push_back(card_real("EQUINOX", 2000.0, nullptr));
    }
    if (freq_hz > 0) cards.push_back(card_real("FREQ", freq_hz, "channel frequency (Hz)"));
    if (interval >= 0) cards.push_back(card_int("INTERVAL", interval, "timestep index in the block"));
    if (channel >= 0) cards.push_back(card_int("CHANNEL", channel, "channel index in the block"));
    cards.push_back(pad_card("END"));
    std::string header;
    for (const std::string &c : cards) header += c;
    header.resize((header.size() + kBlock - 1) / kBlock * kBlock, ' ');

    const size_t n = (size_t)nx * ny;
    std::vector<unsigned char> data((n * 4 + kBlock - 1) / kBlock * kBlock, 0);
    for (size_t i = 0; i < n; ++i) {
        uint32_t u;
        std::memcpy(&u, image + i * (size_t)stride, 4);
        data[4 * i] = (unsigned char)(u >> 24);
        data[4 * i + 1] = (unsigned char)(u >> 16);
        data[4 * i + 2] = (unsigned char)(u >> 8);
        data[4 * i + 3] = (unsigned char)u;
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) return set_error(BGI_ERR_INVALID, "write_fits: cannot open %s: %s", path, std::strerror(errno));
    const bool ok = std::fwrite(header.data(), 1, header.size(), f) == header.size() &&
                    std::fwrite(data.data(), 1, data.size(), f) == data.size();
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) return set_error(BGI_ERR_INVALID, "write_fits: cannot write %s", path);
    return BGI_OK;
}

int check_args(const float *image, int nx, int ny, int stride, const bgi_image_wcs *wcs) {
    if (!image || nx < 1 || ny < 1 || (stride != 1 && stride != 2))
        return set_error(BGI_ERR_INVALID, "write_fits: null image, sides < 1 or pixel stride not 1 or 2");
    if (wcs && !(std::isfinite(wcs->ra_deg) && std::isfinite(wcs->dec_deg) && std::isfinite(wcs->pixscale_ra_deg) &&
                 std::isfinite(wcs->pixscale_dec_deg)))
        return set_error(BGI_ERR_INVALID, "write_fits: non-finite coordinates");
    return BGI_OK;
}

}  // namespace
}  // namespace bgi

using namespace bgi;

extern "C" {

int bgi_write_fits(const char *path, const float *image_host, int nx, int ny, int pixel_stride,
                   const bgi_image_wcs *wcs, double freq_hz) {
    if (!path || !*path) return set_error(BGI_ERR_INVALID, "write_fits: null path");
    const int st = check_args(image_host, nx, ny, pixel_stride, wcs);
    if (st) return st;
    return write_one(path, image_host, nx, ny, pixel_stride, wcs, freq_hz, -1, -1);
}

int bgi_write_fits_block(const char *dir, const char *prefix, const float *images_host, int n_intervals,
                         int n_channels, int nx, int ny, int pixel_stride, const bgi_image_wcs *wcs,
                         const double *freqs_hz) {
    if (!dir || !prefix || n_intervals < 1 || n_channels < 1)
        return set_error(BGI_ERR_INVALID, "write_fits_block: null directory or prefix, or an empty block");
    if (std::strchr(prefix, '/')) return set_error(BGI_ERR_INVALID, "write_fits_block: prefix holds a '/'");
    const int st = check_args(images_host, nx, ny, pixel_stride, wcs);
    if (st) return st;
    const size_t per = (size_t)nx * ny * pixel_stride;
    for (int t = 0; t < n_intervals; ++t)
        for (int c = 0; c < n_channels; ++c) {
            char name[64];
            std::snprintf(name, sizeof name, "_t%04d_c%04d.fits", t, c);
            const std::string path = std::string(dir) + "/" + prefix + name;
            const size_t img = (size_t)t * n_channels + c;
            const int w = write_one(path.c_str(), images_host + img * per, nx, ny, pixel_stride, wcs,
                                    freqs_hz ? freqs_hz[c] : 0.0, t, c);
            if (w) return w;
        }
    return BGI_OK;
}

}  // extern "C"
