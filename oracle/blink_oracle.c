/*
 * CPU oracle for the BLINK dirty-imaging path: test infrastructure only (see blink_oracle.h).
 * Reference citations are paths inside PaCER-BLINK-Project/imager.
 *
 * Built with -ffp-contract=off so that no multiply-add is fused: the reference's CPU build on
 * x86-64 has no FMA, and the results must not depend on the host architecture.
 */
#include "blink_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

int bgo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* src/pacer_imager.cpp:69-70 (also src/gpu/corrections_gpu.cpp:24-25). */
void bgo_baseline_antennas(uint32_t baseline, uint32_t *a1, uint32_t *a2) {
    uint32_t i = (uint32_t)(-0.5 + sqrt(0.25 + 2.0 * (double)baseline));
    *a1 = i;
    *a2 = baseline - ((i + 1) * i) / 2u;
}

/* src/pacer_imager.cpp:60-86 */
void bgo_update_flags(int n_ant, const int *flagged_ants, int n_flagged, int *baseline_flags) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2;
    for (int64_t b = 0; b < nb; ++b) {
        uint32_t a1, a2;
        bgo_baseline_antennas((uint32_t)b, &a1, &a2);
        int listed = 0;
        for (int k = 0; k < n_flagged; ++k) {
            if (flagged_ants[k] == (int)a1 || flagged_ants[k] == (int)a2) { listed = 1; break; }
        }
        baseline_flags[b] = (listed || a1 == a2) ? 1 : 0;
    }
}

/* src/antenna_positions.cpp:54-56 (pair from the triangular index), :81-89 (zenith branch). */
void bgo_zenith_uvw(int n_ant, const double *x, const double *y, const double *z,
                    float *u, float *v, float *w) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2;
    for (int64_t b = 0; b < nb; ++b) {
        uint32_t i, j;
        bgo_baseline_antennas((uint32_t)b, &i, &j);
        double uu = x[i] - x[j], vv = y[i] - y[j], ww = z[i] - z[j];
        u[b] = (float)(-uu);
        v[b] = (float)(-vv);
        w[b] = (float)(-ww);
    }
}

/* src/pacer_imager.cpp:213-221 */
void bgo_uv_max(int n_baselines, const float *u, const float *v, const int *baseline_flags,
                double *u_max, double *v_max) {
    double um = -INFINITY, vm = -INFINITY;
    for (int b = 0; b < n_baselines; ++b) {
        if (baseline_flags[b] == 0) {
            if (um < fabsf(u[b])) um = fabsf(u[b]);
            if (vm < fabsf(v[b])) vm = fabsf(v[b]);
        }
    }
    *u_max = um;
    *v_max = vm;
}

/* src/pacer_imager.cpp:497-499: float oversampling factor promoted to double. */
double bgo_delta_uv(float oversampling_factor, double uv_max, int n_pixels) {
    return (double)oversampling_factor * uv_max / n_pixels;
}

/* src/pacer_imager.cpp:528-555 */
double bgo_channel_frequency_hz(double frequency_resolution_mhz, int n_averaged_channels,
                                double coarse_channel_bw_mhz, int coarse_channel,
                                int fine_channel, int cotter_compatible) {
    double fine_ch_bw = frequency_resolution_mhz * n_averaged_channels;
    double coarse_ch_bw = coarse_channel_bw_mhz;
    double centre = coarse_channel * coarse_ch_bw;
    double f;
    if (cotter_compatible)
        f = centre - coarse_ch_bw / 2.00 + fine_ch_bw * fine_channel;
    else
        f = centre - coarse_ch_bw / 2.00 + fine_ch_bw * fine_channel + fine_ch_bw / 2.00;
    return f * 1e6;
}

/* Rotation of one complex value by (cos, sin) in double, stored as float
 * (src/corrections.cpp:26-33, src/gpu/corrections_gpu.cpp:62-69). */
static inline void rotate_store(float *p, double c, double s) {
    double re = p[0], im = p[1];
    double re_prim = re * c - im * s;
    double im_prim = im * c + re * s;
    p[0] = (float)re_prim;
    p[1] = (float)im_prim;
}

/* src/corrections.cpp:7-39 with w[baseline] as src/gpu/corrections_gpu.cpp:61. */
void bgo_apply_geometric(float *vis, int n_intervals, int n_channels, int n_ant,
                         const float *w, int n_uvw_sets, const double *freqs_hz) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2;
#pragma omp parallel for collapse(2) schedule(static)
    for (int t = 0; t < n_intervals; ++t) {
        for (int ch = 0; ch < n_channels; ++ch) {
            const float *wt = w + (n_uvw_sets > 1 ? (int64_t)t * nb : 0);
            float *rec = vis + (((int64_t)t * n_channels + ch) * nb) * 8;
            for (int64_t b = 0; b < nb; ++b) {
                double ww = wt[b];
                double angle = 2.0 * M_PI * ww * freqs_hz[ch] / BGO_VEL_LIGHT;
                double s = sin(angle), c = cos(angle);
                for (int p = 0; p < 4; ++p) rotate_store(rec + b * 8 + 2 * p, c, s);
            }
        }
    }
}

/* src/corrections.cpp:41-73 */
void bgo_apply_cable(float *vis, int n_intervals, int n_channels, int n_ant,
                     const double *cable_lengths, const double *freqs_hz) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2;
#pragma omp parallel for collapse(2) schedule(static)
    for (int t = 0; t < n_intervals; ++t) {
        for (int ch = 0; ch < n_channels; ++ch) {
            float *rec = vis + (((int64_t)t * n_channels + ch) * nb) * 8;
            for (int a1 = 0; a1 < n_ant; ++a1) {
                for (int a2 = 0; a2 <= a1; ++a2) {
                    int64_t b = (int64_t)a1 * (a1 + 1) / 2 + a2;
                    double d = cable_lengths[a2] - cable_lengths[a1];
                    double angle = -2.0 * M_PI * d * freqs_hz[ch] / BGO_VEL_LIGHT;
                    double s = sin(angle), c = cos(angle);
                    for (int p = 0; p < 4; ++p) rotate_store(rec + b * 8 + 2 * p, c, s);
                }
            }
        }
    }
}

/* src/gpu/gridding_gpu.cpp:18-21 */
static inline int64_t wrap_index(int64_t i, int side) { return i >= 0 ? i % side : side + i; }

/* src/gpu/gridding_gpu.cpp:24-54.  A rounded pixel coordinate of magnitude 2^30 or more
 * (far outside any grid) is reported as -1 instead of overflowing the int conversion. */
int64_t bgo_cell_index(float u, float v, double delta_u, double delta_v, double wavelength,
                       double min_uv, int n_pixels, int uv_sign) {
    double ul = (double)u / wavelength;
    double vl = (double)v / wavelength;
    double dist = sqrt(ul * ul + vl * vl);
    if (!(dist > min_uv)) return -1;
    double up = round(ul / delta_u);
    double vp = round(vl / delta_v);
    if (!(fabs(up) < 1073741824.0) || !(fabs(vp) < 1073741824.0)) return -1;
    int64_t ui = wrap_index((int64_t)(uv_sign * up), n_pixels);
    int64_t vi = wrap_index((int64_t)(uv_sign * vp), n_pixels);
    return (int64_t)n_pixels * vi + ui;
}

/* Polarisation selection, src/pacer_imager.cpp:301-325. */
static inline void select_pol(const float *rec, int pol, float *re, float *im) {
    if (pol == BGO_POL_XX) {
        *re = rec[0]; *im = rec[1];
    } else if (pol == BGO_POL_YY) {
        *re = rec[6]; *im = rec[7];
    } else if (pol == BGO_POL_V) {
        /* (0 + 0.5i) * (xy - yx) */
        float dr = rec[2] - rec[4], di = rec[3] - rec[5];
        *re = 0.0f * dr - 0.5f * di;
        *im = 0.0f * di + 0.5f * dr;
    } else {
        *re = (rec[0] + rec[6]) / 2.0f;
        *im = (rec[1] + rec[7]) / 2.0f;
    }
}

static int64_t grid_one_image(const float *rec0, int64_t nb, const float *u, const float *v,
                              const int *flags, double wavelength, double du, double dv, int n,
                              double min_uv, int pol, int uniform, float *grid, float *counter) {
    const int64_t npix = (int64_t)n * n;
    int64_t gridded = 0;
    memset(grid, 0, sizeof(float) * 2 * npix);
    memset(counter, 0, sizeof(float) * npix);
    for (int64_t b = 0; b < nb; ++b) {
        if (flags[b]) continue; /* :299 */
        float re, im;
        select_pol(rec0 + b * 8, pol, &re, &im);
        if (isnan(re) || isnan(im)) continue;                          /* :327 */
        if (!(fabsf(re) < BGO_MAX_VIS && fabsf(im) < BGO_MAX_VIS)) continue; /* :329 */
        int64_t pos = bgo_cell_index(u[b], v[b], du, dv, wavelength, min_uv, n, +1);
        if (pos >= 0 && pos < npix) {
            grid[2 * pos] = grid[2 * pos] + re;
            grid[2 * pos + 1] = grid[2 * pos + 1] + im;
            counter[pos] += 1.0f;
            ++gridded;
        }
        int64_t pos2 = bgo_cell_index(u[b], v[b], du, dv, wavelength, min_uv, n, -1);
        if (pos2 >= 0 && pos2 < npix) {
            grid[2 * pos2] = grid[2 * pos2] + re;
            grid[2 * pos2 + 1] = grid[2 * pos2 + 1] - im;
            counter[pos2] += 1.0f;
            ++gridded;
        }
    }
    if (uniform) { /* :421-428, empty cells become 0/0 as in the reference */
        for (int64_t i = 0; i < npix; ++i) {
            grid[2 * i] = grid[2 * i] / counter[i];
            grid[2 * i + 1] = grid[2 * i + 1] / counter[i];
        }
    }
    return gridded;
}

/* src/pacer_imager.cpp:250-432 */
int64_t bgo_gridding(const float *vis, int n_intervals, int n_channels, int n_ant,
                     const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                     const double *freqs_hz, double delta_u, double delta_v, int n_pixels,
                     double min_uv, int pol, int uniform, float *grids, float *counters) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2;
    const int64_t npix = (int64_t)n_pixels * n_pixels;
    int64_t total = 0;
#pragma omp parallel for collapse(2) schedule(static) reduction(+ : total)
    for (int t = 0; t < n_intervals; ++t) {
        for (int ch = 0; ch < n_channels; ++ch) {
            int64_t img = (int64_t)t * n_channels + ch;
            int64_t set = n_uvw_sets > 1 ? t : 0;
            double wavelength = BGO_VEL_LIGHT / freqs_hz[ch]; /* :289 */
            total += grid_one_image(vis + img * nb * 8, nb, u + set * nb, v + set * nb,
                                    baseline_flags, wavelength, delta_u, delta_v, n_pixels,
                                    min_uv, pol, uniform, grids + img * npix * 2,
                                    counters + img * npix);
        }
    }
    return total;
}

/* ------------------------------------------------------------------------------------------
 * Inverse DFT of our own: iterative radix-2 (Cooley-Tukey, decimation in time with bit
 * reversal) for powers of two, direct O(n^2) summation otherwise.  Twiddles exp(+2*pi*i*k/n)
 * are computed in double from cos/sin.  Generated for double and float arithmetic.
 * ------------------------------------------------------------------------------------------ */
static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

#define DEFINE_FFT(T, SUF)                                                                       \
    static void twiddles_##SUF(T *tw, int n) {                                                 \
        for (int k = 0; k < n; ++k) {                                                          \
            double a = 2.0 * M_PI * (double)k / (double)n;                                     \
            tw[2 * k] = (T)cos(a);                                                             \
            tw[2 * k + 1] = (T)sin(a);                                                         \
        }                                                                                      \
    }                                                                                          \
    /* in-place inverse transform of n complex values at x[j*stride] */                        \
    static void fft1_##SUF(T *x, int n, int64_t stride, T *buf, const T *tw) {                 \
        for (int j = 0; j < n; ++j) {                                                          \
            buf[2 * j] = x[2 * j * stride];                                                    \
            buf[2 * j + 1] = x[2 * j * stride + 1];                                            \
        }                                                                                      \
        if (is_pow2(n)) {                                                                      \
            for (int i = 1, j = 0; i < n; ++i) {                                               \
                int bit = n >> 1;                                                              \
                for (; j & bit; bit >>= 1) j ^= bit;                                           \
                j ^= bit;                                                                      \
                if (i < j) {                                                                   \
                    T r = buf[2 * i], m = buf[2 * i + 1];                                      \
                    buf[2 * i] = buf[2 * j]; buf[2 * i + 1] = buf[2 * j + 1];                  \
                    buf[2 * j] = r; buf[2 * j + 1] = m;                                        \
                }                                                                              \
            }                                                                                  \
            for (int len = 2; len <= n; len <<= 1) {                                           \
                int half = len >> 1, step = n / len;                                           \
                for (int s = 0; s < n; s += len) {                                             \
                    for (int k = 0; k < half; ++k) {                                           \
                        T wr = tw[2 * k * step], wi = tw[2 * k * step + 1];                    \
                        T *a = buf + 2 * (s + k), *b = buf + 2 * (s + k + half);               \
                        T br = b[0] * wr - b[1] * wi, bi = b[0] * wi + b[1] * wr;              \
                        b[0] = a[0] - br; b[1] = a[1] - bi;                                    \
                        a[0] = a[0] + br; a[1] = a[1] + bi;                                    \
                    }                                                                          \
                }                                                                              \
            }                                                                                  \
            for (int j = 0; j < n; ++j) {                                                      \
                x[2 * j * stride] = buf[2 * j];                                                \
                x[2 * j * stride + 1] = buf[2 * j + 1];                                        \
            }                                                                                  \
        } else {                                                                               \
            for (int k = 0; k < n; ++k) {                                                      \
                T sr = 0, si = 0;                                                              \
                for (int j = 0; j < n; ++j) {                                                  \
                    int64_t m = ((int64_t)j * k) % n;                                          \
                    T wr = tw[2 * m], wi = tw[2 * m + 1];                                      \
                    sr += buf[2 * j] * wr - buf[2 * j + 1] * wi;                               \
                    si += buf[2 * j] * wi + buf[2 * j + 1] * wr;                               \
                }                                                                              \
                x[2 * k * stride] = sr;                                                        \
                x[2 * k * stride + 1] = si;                                                    \
            }                                                                                  \
        }                                                                                      \
    }                                                                                          \
    /* in-place 2D inverse transform of one n x n image (rows, then columns) */                \
    static void fft2_inplace_##SUF(T *img, int n, const T *tw, T *buf) {                       \
        for (int r = 0; r < n; ++r) fft1_##SUF(img + (int64_t)2 * r * n, n, 1, buf, tw);       \
        for (int c = 0; c < n; ++c) fft1_##SUF(img + 2 * c, n, n, buf, tw);                   \
    }

DEFINE_FFT(double, f64)
DEFINE_FFT(float, f32)

void bgo_fft2_inverse_f64(const double *in, double *out, int n, int n_images) {
    const int64_t npix = (int64_t)n * n;
    double *tw = (double *)malloc(sizeof(double) * 2 * n);
    twiddles_f64(tw, n);
    memcpy(out, in, sizeof(double) * 2 * npix * n_images);
#pragma omp parallel
    {
        double *buf = (double *)malloc(sizeof(double) * 2 * n);
#pragma omp for schedule(static)
        for (int i = 0; i < n_images; ++i) fft2_inplace_f64(out + 2 * npix * i, n, tw, buf);
        free(buf);
    }
    free(tw);
}

/* One image's 2D transform split over threads (rows, then columns), for batches smaller than
 * the thread count. */
static void fft2_parallel_f32(float *img, int n, const float *tw) {
#pragma omp parallel
    {
        float *buf = (float *)malloc(sizeof(float) * 2 * n);
#pragma omp for schedule(static)
        for (int r = 0; r < n; ++r) fft1_f32(img + (int64_t)2 * r * n, n, 1, buf, tw);
#pragma omp for schedule(static)
        for (int c = 0; c < n; ++c) fft1_f32(img + 2 * c, n, n, buf, tw);
        free(buf);
    }
}

/* Powers of two in FP32 for the CPU baseline, blocked: BGO_LINES independent lines (rows, or
 * adjacent columns) at a time as re[n][BGO_LINES], im[n][BGO_LINES], so every butterfly runs
 * over the lines in a unit-stride inner loop the compiler vectorises, and columns are read in
 * 64-byte row segments instead of one value per cache line.  Each line sees exactly the
 * arithmetic of fft1_f32 (same bit reversal, butterfly order and twiddles), so the results are
 * the same bits as the scalar path. */
#define BGO_LINES 16
static void fft_lines_f32(float *re, float *im, int n, const float *tw) {
    for (int i = 1, j = 0; i < n; ++i) {
        int bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            for (int v = 0; v < BGO_LINES; ++v) {
                float t = re[i * BGO_LINES + v];
                re[i * BGO_LINES + v] = re[j * BGO_LINES + v];
                re[j * BGO_LINES + v] = t;
                t = im[i * BGO_LINES + v];
                im[i * BGO_LINES + v] = im[j * BGO_LINES + v];
                im[j * BGO_LINES + v] = t;
            }
        }
    }
    /* Two radix-2 stages (lengths 2m and 4m) per pass: each group of four elements s+k, s+k+m,
     * s+k+2m, s+k+3m goes through both stages' butterflies in registers, with the radix-2 stages'
     * own twiddle entries and operation order, so the results are the same bits in half the
     * passes over the block.  (ivdep: the four rows of a group are at least 16 floats apart, so
     * the lanes of the inner loop carry no dependence.) */
    int len = 2;
    for (; 2 * len <= n; len *= 4) {
        const int m = len >> 1, step2 = n / len, step4 = n / (2 * len);
        const int o1 = m * BGO_LINES, o2 = 2 * m * BGO_LINES, o3 = 3 * m * BGO_LINES;
        for (int s = 0; s < n; s += 2 * len) {
            for (int k = 0; k < m; ++k) {
                const float w2r = tw[2 * k * step2], w2i = tw[2 * k * step2 + 1];
                const float wAr = tw[2 * k * step4], wAi = tw[2 * k * step4 + 1];
                const float wBr = tw[2 * (k + m) * step4], wBi = tw[2 * (k + m) * step4 + 1];
                float *restrict R = re + (s + k) * BGO_LINES;
                float *restrict I = im + (s + k) * BGO_LINES;
#pragma GCC ivdep
                for (int v = 0; v < BGO_LINES; ++v) {
                    const float x0r = R[v], x0i = I[v], x1r = R[o1 + v], x1i = I[o1 + v];
                    const float x2r = R[o2 + v], x2i = I[o2 + v], x3r = R[o3 + v], x3i = I[o3 + v];
                    const float t1r = x1r * w2r - x1i * w2i, t1i = x1r * w2i + x1i * w2r;
                    const float a1r = x0r - t1r, a1i = x0i - t1i, a0r = x0r + t1r, a0i = x0i + t1i;
                    const float t3r = x3r * w2r - x3i * w2i, t3i = x3r * w2i + x3i * w2r;
                    const float a3r = x2r - t3r, a3i = x2i - t3i, a2r = x2r + t3r, a2i = x2i + t3i;
                    const float u2r = a2r * wAr - a2i * wAi, u2i = a2r * wAi + a2i * wAr;
                    const float u3r = a3r * wBr - a3i * wBi, u3i = a3r * wBi + a3i * wBr;
                    R[v] = a0r + u2r;
                    I[v] = a0i + u2i;
                    R[o2 + v] = a0r - u2r;
                    I[o2 + v] = a0i - u2i;
                    R[o1 + v] = a1r + u3r;
                    I[o1 + v] = a1i + u3i;
                    R[o3 + v] = a1r - u3r;
                    I[o3 + v] = a1i - u3i;
                }
            }
        }
    }
    if (len <= n) { /* an odd number of stages: the last, of length n, alone */
        const int half = len >> 1, step = n / len;
        for (int s = 0; s < n; s += len) {
            for (int k = 0; k < half; ++k) {
                const float wr = tw[2 * k * step], wi = tw[2 * k * step + 1];
                float *restrict ar = re + (s + k) * BGO_LINES, *restrict ai = im + (s + k) * BGO_LINES;
                float *restrict br = re + (s + k + half) * BGO_LINES, *restrict bi = im + (s + k + half) * BGO_LINES;
                for (int v = 0; v < BGO_LINES; ++v) {
                    const float xr = br[v] * wr - bi[v] * wi, xi = br[v] * wi + bi[v] * wr;
                    br[v] = ar[v] - xr;
                    bi[v] = ai[v] - xi;
                    ar[v] = ar[v] + xr;
                    ai[v] = ai[v] + xi;
                }
            }
        }
    }
}

/* lines l0 .. l0+BGO_LINES-1 of an n x n image: rows (cols == 0) or columns (cols == 1) */
static void fft_line_block_f32(float *img, int n, int l0, int cols, const float *tw, float *re, float *im) {
    const int nv = n - l0 < BGO_LINES ? n - l0 : BGO_LINES;
    for (int i = 0; i < n; ++i)
        for (int v = 0; v < BGO_LINES; ++v) {
            const int64_t e = cols ? (int64_t)i * n + l0 + v : (int64_t)(l0 + v) * n + i;
            re[i * BGO_LINES + v] = v < nv ? img[2 * e] : 0.0f;
            im[i * BGO_LINES + v] = v < nv ? img[2 * e + 1] : 0.0f;
        }
    fft_lines_f32(re, im, n, tw);
    for (int i = 0; i < n; ++i)
        for (int v = 0; v < nv; ++v) {
            const int64_t e = cols ? (int64_t)i * n + l0 + v : (int64_t)(l0 + v) * n + i;
            img[2 * e] = re[i * BGO_LINES + v];
            img[2 * e + 1] = im[i * BGO_LINES + v];
        }
}

static void fft2_blocked_f32(float *img, int n, const float *tw, float *re, float *im) {
    for (int l0 = 0; l0 < n; l0 += BGO_LINES) fft_line_block_f32(img, n, l0, 0, tw, re, im);
    for (int l0 = 0; l0 < n; l0 += BGO_LINES) fft_line_block_f32(img, n, l0, 1, tw, re, im);
}

/* the scalar path (one line at a time), kept as the blocked path's check */
void bgo_fft2_inverse_f32_scalar(const float *in, float *out, int n, int n_images) {
    const int64_t npix = (int64_t)n * n;
    float *tw = (float *)malloc(sizeof(float) * 2 * n);
    float *buf = (float *)malloc(sizeof(float) * 2 * n);
    twiddles_f32(tw, n);
    memcpy(out, in, sizeof(float) * 2 * npix * n_images);
    for (int i = 0; i < n_images; ++i) fft2_inplace_f32(out + 2 * npix * i, n, tw, buf);
    free(buf);
    free(tw);
}

void bgo_fft2_inverse_f32(const float *in, float *out, int n, int n_images) {
    const int64_t npix = (int64_t)n * n;
    float *tw = (float *)malloc(sizeof(float) * 2 * n);
    twiddles_f32(tw, n);
    memcpy(out, in, sizeof(float) * 2 * npix * n_images);
    if (is_pow2(n) && n_images >= bgo_max_threads()) {
#pragma omp parallel
        {
            float *re = (float *)malloc(sizeof(float) * (size_t)n * BGO_LINES);
            float *im = (float *)malloc(sizeof(float) * (size_t)n * BGO_LINES);
#pragma omp for schedule(static)
            for (int i = 0; i < n_images; ++i) fft2_blocked_f32(out + 2 * npix * i, n, tw, re, im);
            free(re);
            free(im);
        }
    } else if (is_pow2(n)) {  /* fewer images than threads: the blocks of each image over threads */
        for (int i = 0; i < n_images; ++i) {
            float *img = out + 2 * npix * i;
#pragma omp parallel
            {
                float *re = (float *)malloc(sizeof(float) * (size_t)n * BGO_LINES);
                float *im = (float *)malloc(sizeof(float) * (size_t)n * BGO_LINES);
#pragma omp for schedule(static)
                for (int l0 = 0; l0 < n; l0 += BGO_LINES) fft_line_block_f32(img, n, l0, 0, tw, re, im);
#pragma omp for schedule(static)
                for (int l0 = 0; l0 < n; l0 += BGO_LINES) fft_line_block_f32(img, n, l0, 1, tw, re, im);
                free(re);
                free(im);
            }
        }
    } else if (n_images < bgo_max_threads()) {
        for (int i = 0; i < n_images; ++i) fft2_parallel_f32(out + 2 * npix * i, n, tw);
    } else {
#pragma omp parallel
        {
            float *buf = (float *)malloc(sizeof(float) * 2 * n);
#pragma omp for schedule(static)
            for (int i = 0; i < n_images; ++i) fft2_inplace_f32(out + 2 * npix * i, n, tw, buf);
            free(buf);
        }
    }
    free(tw);
}

/* src/pacer_imager.cpp:30-35 */
static inline int calc_fft_shift(int pos, int side) {
    int is_odd = side % 2;
    return (pos + side / 2 + is_odd) % side;
}

#define DEFINE_SHIFT(T, SUF)                                                                     \
    void bgo_fft_shift_##SUF(T *image, int xs, int ys) {                                         \
        for (int y = 0; y < ys; ++y) {                                                           \
            for (int x = 0; x < xs / 2; ++x) {                                                   \
                int64_t src = (int64_t)y * xs + x;                                               \
                int64_t dst = (int64_t)y * xs + calc_fft_shift(x, xs);                           \
                T r = image[2 * src], i = image[2 * src + 1];                                    \
                image[2 * src] = image[2 * dst]; image[2 * src + 1] = image[2 * dst + 1];        \
                image[2 * dst] = r; image[2 * dst + 1] = i;                                      \
            }                                                                                    \
        }                                                                                        \
        for (int y = 0; y < ys / 2; ++y) {                                                       \
            for (int x = 0; x < xs; ++x) {                                                       \
                int64_t src = (int64_t)y * xs + x;                                               \
                int64_t dst = (int64_t)calc_fft_shift(y, ys) * xs + x;                           \
                T r = image[2 * src], i = image[2 * src + 1];                                    \
                image[2 * src] = image[2 * dst]; image[2 * src + 1] = image[2 * dst + 1];        \
                image[2 * dst] = r; image[2 * dst + 1] = i;                                      \
            }                                                                                    \
        }                                                                                        \
    }

DEFINE_SHIFT(double, f64)
DEFINE_SHIFT(float, f32)

/* src/pacer_imager.cpp:134-208 in FP64: FFT, multiply by 1/sum(counter), shift. */
void bgo_image_f64(const float *grids, const float *counters, int n, int n_images,
                   double *images) {
    const int64_t npix = (int64_t)n * n;
    double *tw = (double *)malloc(sizeof(double) * 2 * n);
    twiddles_f64(tw, n);
#pragma omp parallel
    {
        double *buf = (double *)malloc(sizeof(double) * 2 * n);
#pragma omp for schedule(static)
        for (int i = 0; i < n_images; ++i) {
            double *img = images + 2 * npix * i;
            const float *g = grids + 2 * npix * i;
            for (int64_t k = 0; k < 2 * npix; ++k) img[k] = g[k];
            fft2_inplace_f64(img, n, tw, buf);
            double sum = 0.0;
            const float *c = counters + npix * i;
            for (int64_t k = 0; k < npix; ++k) sum += c[k];
            double fnorm = 1.00 / sum;
            for (int64_t k = 0; k < 2 * npix; ++k) img[k] *= fnorm;
            bgo_fft_shift_f64(img, n, n);
        }
        free(buf);
    }
    free(tw);
}

/* Reference CPU run() in FP32: gridding (:250-432), FFT (:150-152), normalise by
 * (float)(1/sum) (:171-178) and shift (:179). */
void bgo_run_f32(const float *vis, int n_intervals, int n_channels, int n_ant,
                 const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                 const double *freqs_hz, double delta_u, double delta_v, int n_pixels,
                 double min_uv, int pol, float *grids, float *counters, float *images) {
    const int n_images = n_intervals * n_channels;
    const int64_t npix = (int64_t)n_pixels * n_pixels;
    bgo_gridding(vis, n_intervals, n_channels, n_ant, u, v, n_uvw_sets, baseline_flags, freqs_hz,
                 delta_u, delta_v, n_pixels, min_uv, pol, 0, grids, counters);
    bgo_fft2_inverse_f32(grids, images, n_pixels, n_images);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n_images; ++i) {
        double sum = 0.0;
        const float *c = counters + npix * i;
        for (int64_t k = 0; k < npix; ++k) sum += c[k];
        float fnorm = (float)(1.00 / sum);
        float *img = images + 2 * npix * i;
        for (int64_t k = 0; k < 2 * npix; ++k) img[k] *= fnorm;
        bgo_fft_shift_f32(img, n_pixels, n_pixels);
    }
}

/* src/gpu/gpu_utils.cpp:19-71 (per-image sum); double accumulation makes it exact for the
 * integer-valued counters it is used on. */
void bgo_vector_sum(const float *data, int64_t image_size, int n_images, double *sums) {
    for (int i = 0; i < n_images; ++i) {
        double s = 0.0;
        for (int64_t k = 0; k < image_size; ++k) s += data[(int64_t)i * image_size + k];
        sums[i] = s;
    }
}

/* src/gpu/gpu_utils.cpp:143-150: running complex sum over images, then divide by count. */
void bgo_image_average(const float *images, int64_t image_size, int n_images, float *out) {
    for (int64_t k = 0; k < image_size; ++k) {
        float r = images[2 * k], m = images[2 * k + 1];
        for (int i = 1; i < n_images; ++i) {
            r += images[2 * (k + (int64_t)i * image_size)];
            m += images[2 * (k + (int64_t)i * image_size) + 1];
        }
        out[2 * k] = r / (float)n_images;
        out[2 * k + 1] = m / (float)n_images;
    }
}

/* apps/pacer_imager_main.cpp:720-804 (ConvertFits2XCorr): the lower triangle of the XX (and YY)
 * correlation matrices into visibility records.  Element (row i, column j) of a matrix, j <= i,
 * is baseline i*(i+1)/2 + j (the reference reads getXY(j, i) of its row-major FITS image); XX
 * goes to record slot 0 and YY to slot 3 (zero when no YY matrices are given, :777); the
 * reference leaves XY and YX unset, here they are zero.  Matrices float[n_matrices][n][n]. */
void bgo_ingest_matrices(const float *re_xx, const float *im_xx, const float *re_yy,
                         const float *im_yy, int n_ant, int64_t n_matrices, float *vis) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2, nn = (int64_t)n_ant * n_ant;
    for (int64_t m = 0; m < n_matrices; ++m)
        for (int i = 0; i < n_ant; ++i)
            for (int j = 0; j <= i; ++j) {
                const int64_t b = (int64_t)i * (i + 1) / 2 + j, e = m * nn + (int64_t)i * n_ant + j;
                float *rec = vis + (m * nb + b) * 8;
                rec[0] = (float)(double)re_xx[e];
                rec[1] = (float)(double)im_xx[e];
                rec[2] = rec[3] = rec[4] = rec[5] = 0.0f;
                rec[6] = re_yy && im_yy ? (float)(double)re_yy[e] : 0.0f;
                rec[7] = re_yy && im_yy ? (float)(double)im_yy[e] : 0.0f;
            }
}

/* ------------------------------------------------------------------------------------------
 * Kaiser-Bessel convolutional gridding, CPU only in the reference (m_nConvolvingKernelSize > 0,
 * src/pacer_imager.cpp:378-403 and 565-750).
 * ------------------------------------------------------------------------------------------ */

/* src/pacer_imager.cpp:565-577: unnormalised modified Bessel function I0 by its series */
static double kb_bessel0(double x, double precision) {
    double d = 0.0, ds = 1.0, sum = 1.0;
    do {
        d += 2.0;
        ds *= x * x / (d * d);
        sum += ds;
    } while (ds > sum * precision);
    return sum;
}

/* src/pacer_imager.cpp:579-596.  For an even length the reference also writes kernel[n], one
 * element past its vector; nothing reads it, and it is not written here. */
static void kb_kernel_1d(double *kernel, size_t n, double alpha, size_t osf, int with_sinc) {
    const size_t mid = n / 2;
    double *sinc = (double *)malloc(sizeof(double) * (mid + 1));
    const double filter_ratio = 1.0 / (double)osf;
    sinc[0] = filter_ratio;
    for (size_t i = 1; i != mid + 1; i++) {
        const double x = (double)i;
        sinc[i] = with_sinc ? (sin(M_PI * filter_ratio * x) / (M_PI * x)) : filter_ratio;
    }
    const double norm = (double)osf / kb_bessel0(alpha, 1e-8);
    for (size_t i = 0; i != mid + 1; i++) {
        const double term = (double)i / (double)mid;
        if (mid + i < n) kernel[mid + i] = sinc[i] * kb_bessel0(alpha * sqrt(1.0 - (term * term)), 1e-8) * norm;
    }
    for (size_t i = 0; i != mid; i++) kernel[i] = kernel[n - 1 - i];
    free(sinc);
}

/* src/pacer_imager.cpp:599-651 (makeKernels, alpha 8.6, oversampling 1023): tables[o][x] for
 * o < 1023, x < kernel_size, with the reference's reversed order of the oversampled rows. */
void bgo_kb_tables(int kernel_size, int with_sinc, double *tables) {
    const size_t osf = BGO_KB_OVERSAMPLING, n = (size_t)kernel_size * osf;
    double *k1 = (double *)malloc(sizeof(double) * n);
    kb_kernel_1d(k1, n, 8.6, osf, with_sinc);
    for (size_t i = 0; i != osf; ++i)
        for (size_t x = 0; x != (size_t)kernel_size; ++x) tables[(osf - i - 1) * kernel_size + x] = k1[x * osf + i];
    free(k1);
}

/* src/pacer_imager.cpp:753-778 (calc_xy_grid2 with is_odd = 0) */
static void kb_xy_grid(double u_pix, double v_pix, int n, int *x_grid, int *y_grid, int im_sign) {
    const int cx = n / 2, cy = n / 2;
    const int ui = (int)(im_sign * u_pix + n / 2), vi = (int)(im_sign * v_pix + n / 2);
    *x_grid = ui < cx ? cx + ui : ui - cx;
    *y_grid = vi < cy ? cy + vi : vi - cy;
}

/* src/pacer_imager.cpp:655-750 (convolve_with_kernel): u, v in wavelengths; im_sign +1 for the
 * visibility, -1 for its conjugate (the same u, v: the taps are mirrored by calc_xy_grid2). */
static void kb_convolve(float *grid, double re, double im, double u, double v, double du, double dv, int n,
                        double im_sign, int ksize, const double *tables) {
    const int osf = BGO_KB_OVERSAMPLING;
    const double u_exact = u / du, v_exact = v / dv;
    const double u_pix = round(u / du), v_pix = round(v / dv);
    int xk = (int)round((u_exact - u_pix) * osf);
    int yk = (int)round((v_exact - v_pix) * osf);
    xk = (xk + (osf * 3) / 2) % osf;
    yk = (yk + (osf * 3) / 2) % osf;
    const double *xkern = tables + (size_t)xk * ksize, *ykern = tables + (size_t)yk * ksize;
    const int mid = ksize / 2;
    int vv = (int)(v_pix - mid);
    for (int j = 0; j != ksize; ++j) {
        const double ykv = ykern[j];
        int uu = (int)(u_pix - mid);
        for (int i = 0; i != ksize; ++i) {
            const double kv = ykv * xkern[i];
            const double re_conv = re * kv;
            const double im_conv = im_sign * im * kv;
            int xg, yg;
            kb_xy_grid(uu, vv, n, &xg, &yg, (int)im_sign);
            if (xg >= 0 && yg >= 0 && xg < n && yg < n) {
                float *c = grid + 2 * ((int64_t)yg * n + xg);
                c[0] = (float)((double)c[0] + re_conv);
                c[1] = (float)((double)c[1] + im_conv);
            }
            uu++;
        }
        vv++;
    }
}

/* The gridding loop of src/pacer_imager.cpp:297-408 with the convolution kernel: the checks and
 * counters as the nearest-neighbour loop (counter +1 at the visibility's own cell). */
int64_t bgo_gridding_kb(const float *vis, int n_intervals, int n_channels, int n_ant, const float *u,
                        const float *v, int n_uvw_sets, const int *baseline_flags, const double *freqs_hz,
                        double delta_u, double delta_v, int n_pixels, double min_uv, int pol, int kernel_size,
                        int with_sinc, float *grids, float *counters) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2, npix = (int64_t)n_pixels * n_pixels;
    double *tables = (double *)malloc(sizeof(double) * BGO_KB_OVERSAMPLING * kernel_size);
    bgo_kb_tables(kernel_size, with_sinc, tables);
    int64_t total = 0;
    for (int t = 0; t < n_intervals; ++t)
        for (int ch = 0; ch < n_channels; ++ch) {
            const int64_t img = (int64_t)t * n_channels + ch, set = n_uvw_sets > 1 ? t : 0;
            const double wavelength = BGO_VEL_LIGHT / freqs_hz[ch];
            float *grid = grids + img * npix * 2, *counter = counters + img * npix;
            memset(grid, 0, sizeof(float) * 2 * npix);
            memset(counter, 0, sizeof(float) * npix);
            const float *rec0 = vis + img * nb * 8;
            for (int64_t b = 0; b < nb; ++b) {
                if (baseline_flags[b]) continue;
                float re, im;
                select_pol(rec0 + b * 8, pol, &re, &im);
                if (isnan(re) || isnan(im)) continue;
                if (!(fabsf(re) < BGO_MAX_VIS && fabsf(im) < BGO_MAX_VIS)) continue;
                const double uu = (double)u[set * nb + b] / wavelength, vv = (double)v[set * nb + b] / wavelength;
                const int64_t pos = bgo_cell_index(u[set * nb + b], v[set * nb + b], delta_u, delta_v, wavelength,
                                                   min_uv, n_pixels, +1);
                const int64_t pos2 = bgo_cell_index(u[set * nb + b], v[set * nb + b], delta_u, delta_v, wavelength,
                                                    min_uv, n_pixels, -1);
                if (pos < 0 && pos2 < 0) continue; /* cut by min_uv */
                kb_convolve(grid, re, im, uu, vv, delta_u, delta_v, n_pixels, 1.0, kernel_size, tables);
                if (pos >= 0 && pos < npix) { counter[pos] += 1.0f; ++total; }
                kb_convolve(grid, re, im, uu, vv, delta_u, delta_v, n_pixels, -1.0, kernel_size, tables);
                if (pos2 >= 0 && pos2 < npix) { counter[pos2] += 1.0f; ++total; }
            }
        }
    free(tables);
    return total;
}

/* Pointed-observation UVW (CAntennaPositions::CalculateUVW with metadata,
 * src/antenna_positions.cpp:23-92, and PacerGeometry::CalcUVW_NEW / precXYZ / CalcUVW,
 * src/pacer_geometry.h:101-134, 208-215, 312-334): per timestep, each antenna's XYZ rotated to the
 * frame at lmst, precessed by rmatpr, rotated back at lmst2000, projected with the hour angle and
 * declination (TMS eq. 4.1); baseline (i >= j) = -(uvw_i - uvw_j) as float.  step[17]:
 * rmatpr[9] row-major, sin/cos of lmst, lmst2000, ha2000 and dec_aber (computed by the caller, as
 * the reference computes them once per timestep with PAL). */
static void bgo_antenna_uvw(const double *st, double x, double y, double z, double *u, double *v, double *w) {
    const double *r = st;
    const double sep = st[9], cep = st[10], s2000 = st[11], c2000 = st[12];
    const double sh = st[13], ch = st[14], sd = st[15], cd = st[16];
    const double xpr = cep * x - sep * y;
    const double ypr = sep * x + cep * y;
    const double zpr = z;
    const double xpr2 = (r[0]) * xpr + (r[1]) * ypr + (r[2]) * zpr;
    const double ypr2 = (r[3]) * xpr + (r[4]) * ypr + (r[5]) * zpr;
    const double zpr2 = (r[6]) * xpr + (r[7]) * ypr + (r[8]) * zpr;
    const double xp = c2000 * xpr2 + s2000 * ypr2;
    const double yp = -s2000 * xpr2 + c2000 * ypr2;
    const double zp = zpr2;
    *u = sh * xp + ch * yp;
    *v = -sd * ch * xp + sd * sh * yp + cd * zp;
    *w = cd * ch * xp - cd * sh * yp + sd * zp;
}

void bgo_pointed_uvw(const double *xyz, int n_ant, const double *steps, int n_steps, float *u, float *v, float *w) {
    const int64_t nb = (int64_t)n_ant * (n_ant + 1) / 2;
    for (int t = 0; t < n_steps; ++t)
        for (int i = 0; i < n_ant; ++i)
            for (int j = 0; j <= i; ++j) {
                double u1, v1, w1, u2, v2, w2;
                bgo_antenna_uvw(steps + 17 * t, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], &u1, &v1, &w1);
                bgo_antenna_uvw(steps + 17 * t, xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], &u2, &v2, &w2);
                const int64_t b = t * nb + (int64_t)i * (i + 1) / 2 + j;
                u[b] = (float)(-(u1 - u2));
                v[b] = (float)(-(v1 - v2));
                w[b] = (float)(-(w1 - w2));
            }
}
