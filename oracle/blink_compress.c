/*
 * CPU statement of the block-scaled 16-bit visibility storage -- test infrastructure only.
 *
 * This format is the GB300 imager's own (the reference stores complex64 records only); the
 * tests compare the CUDA encoder with these functions bit for bit, and image the decoded
 * values with the oracle's restatement of the reference path to check the imaging kernels.
 *
 * Layout: data uint16[T][C][4 pol planes XX,XY,YX,YY][B][re,im]; scales float[T][C][4][NB],
 * NB = ceil(B / 128): block k of a plane holds baselines 128k .. 128k+127 (256 components).
 * A component is invalid when it is NaN or |x| >= 1e12 (the values the reference's gridding
 * skips, src/pacer_imager.cpp:327-329); m = the largest |x| of the block's valid components
 * (0 when none).
 *   S16:  scale = m / 32767 (0 when m == 0); elem = rint(x / scale) clamped to +-32767; an
 *         invalid component is -32768; decode: -32768 -> NaN, else (float)elem * scale.
 *   BF16: scale = m (1 when m == 0); elem = bfloat16(x / scale), round to nearest even;
 *         invalid -> 0x7FC0; decode: float(elem) * scale.
 *   FP16: as BF16 with IEEE binary16 elements; invalid -> 0x7E00.
 * All divisions and products are single FP32 operations, correctly rounded.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "blink_oracle.h"

static inline uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static inline float u2f(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/* bfloat16, round to nearest even (finite inputs) */
static uint16_t to_bf16(float f) {
    uint32_t u = f2u(f);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

/* IEEE binary16, round to nearest even, from the definition: normal numbers keep the top 10
 * mantissa bits and round on the 13 dropped ones; below 2^-14 the value is a multiple of
 * 2^-24, rounded as an integer count of that step. */
static uint16_t to_fp16(float f) {
    const uint32_t u = f2u(f);
    const uint16_t sign = (uint16_t)((u >> 16) & 0x8000u);
    const uint32_t a = u & 0x7FFFFFFFu;
    if (a >= 0x7F800000u) return sign | (a > 0x7F800000u ? 0x7E00u : 0x7C00u);
    if (a >= 0x477FF000u) return sign | 0x7C00u; /* >= 65520 rounds to infinity */
    if (a < 0x38800000u) {                        /* below 2^-14 */
        const float q = rintf(u2f(a) * 16777216.0f);  /* exact scaling by 2^24 */
        return sign | (uint16_t)q;
    }
    uint32_t h = ((((a >> 23) - 112u)) << 10) | ((a & 0x7FFFFFu) >> 13);
    const uint32_t rem = a & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

static float from_fp16(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu;
    if (e == 0) {
        const float v = (float)m * (1.0f / 16777216.0f);
        return (h & 0x8000u) ? -v : v;
    }
    if (e == 31) return u2f(sign | 0x7F800000u | (m << 13));
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

static inline int valid(float x) { return !isnan(x) && (double)fabsf(x) < BGO_MAX_VIS; }

int64_t bgo_compressed_blocks(int64_t n_baselines) { return (n_baselines + 127) / 128; }

void bgo_compress(const float *vis, int64_t n_images, int64_t nb, int format, uint16_t *data,
                  float *scales) {
    const int64_t n_blk = bgo_compressed_blocks(nb);
    for (int64_t img = 0; img < n_images; ++img) {
        for (int p = 0; p < 4; ++p) {
            uint16_t *plane = data + ((img * 4 + p) * nb) * 2;
            for (int64_t k = 0; k < n_blk; ++k) {
                const int64_t b0 = k * 128, b1 = b0 + 128 < nb ? b0 + 128 : nb;
                float m = 0.0f;
                for (int64_t b = b0; b < b1; ++b)
                    for (int c = 0; c < 2; ++c) {
                        const float x = vis[((img * nb + b) * 4 + p) * 2 + c];
                        if (valid(x) && fabsf(x) > m) m = fabsf(x);
                    }
                float scale;
                if (format == BGO_VIS_S16) scale = m / 32767.0f;
                else scale = m > 0.0f ? m : 1.0f;
                scales[(img * 4 + p) * n_blk + k] = scale;
                for (int64_t b = b0; b < b1; ++b)
                    for (int c = 0; c < 2; ++c) {
                        const float x = vis[((img * nb + b) * 4 + p) * 2 + c];
                        uint16_t e;
                        if (format == BGO_VIS_S16) {
                            if (!valid(x)) e = 0x8000u;
                            else if (scale == 0.0f) e = 0;
                            else {
                                float q = rintf(x / scale);
                                if (q > 32767.0f) q = 32767.0f;
                                if (q < -32767.0f) q = -32767.0f;
                                e = (uint16_t)(int16_t)q;
                            }
                        } else if (format == BGO_VIS_BF16) {
                            e = valid(x) ? to_bf16(x / scale) : 0x7FC0u;
                        } else {
                            e = valid(x) ? to_fp16(x / scale) : 0x7E00u;
                        }
                        plane[b * 2 + c] = e;
                    }
            }
        }
    }
}

void bgo_decompress(const uint16_t *data, const float *scales, int64_t n_images, int64_t nb,
                    int format, float *vis) {
    const int64_t n_blk = bgo_compressed_blocks(nb);
    for (int64_t img = 0; img < n_images; ++img)
        for (int p = 0; p < 4; ++p)
            for (int64_t b = 0; b < nb; ++b) {
                const float scale = scales[(img * 4 + p) * n_blk + b / 128];
                for (int c = 0; c < 2; ++c) {
                    const uint16_t e = data[((img * 4 + p) * nb + b) * 2 + c];
                    float x;
                    if (format == BGO_VIS_S16)
                        x = e == 0x8000u ? NAN : (float)(int16_t)e * scale;
                    else if (format == BGO_VIS_BF16)
                        x = u2f((uint32_t)e << 16) * scale;
                    else
                        x = from_fp16(e) * scale;
                    vis[((img * nb + b) * 4 + p) * 2 + c] = x;
                }
            }
}
