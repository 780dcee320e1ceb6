/*
 * CPU oracle for the BLINK dirty-imaging path: test infrastructure only.
 *
 * A plain-C restatement of the reference imager's CPU path (PaCER-BLINK-Project/imager):
 * baseline flags, zenith UVW, u_max / delta_u, cable and geometric phase corrections,
 * nearest-neighbour uv gridding with conjugate points, batched inverse 2D FFT (sign +,
 * unnormalised), normalisation by the weight sum and fftshift.  Every function names the
 * reference file:line it follows.  The FFT is our own (FP64, or FP32 for the timed CPU
 * baseline); the reference calls FFTW there.
 *
 * Only the tests, the smoke check and the CPU-baseline leg of the benchmark may call this
 * library, and only as the checker.  The product path never links it.
 *
 * Conventions (reference layout, src/gpu/gridding_gpu.cpp:72-76):
 *   visibilities  float[T][C][B][4 pols][re,im], pols ordered XX, XY, YX, YY
 *   baseline b    = a1*(a1+1)/2 + a2 with a1 >= a2 (lower triangle incl. autos)
 *   grids         float[T][C][N][N][re,im]; counters float[T][C][N][N]
 */
#ifndef BLINK_ORACLE_H
#define BLINK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BGO_VEL_LIGHT 299792458.0 /* src/pacer_imager_defs.h:12-13 */
#define BGO_MAX_VIS 1e12          /* src/pacer_imager_defs.h:21 */

enum { BGO_POL_XX = 0, BGO_POL_YY = 1, BGO_POL_I = 2, BGO_POL_V = 3 }; /* src/gridding.hpp:4 */

/* Antenna pair of a lower-triangular baseline index (src/pacer_imager.cpp:69-70). */
void bgo_baseline_antennas(uint32_t baseline, uint32_t *a1, uint32_t *a2);

/* Baseline flags: 1 when either antenna is in the flagged list or the baseline is an
 * auto-correlation (src/pacer_imager.cpp:60-86). */
void bgo_update_flags(int n_ant, const int *flagged_ants, int n_flagged, int *baseline_flags);

/* Zenith-phased UVW of the lower-triangular baselines: u = -(x_a1 - x_a2) stored as float
 * (src/antenna_positions.cpp:54-56,81-89). */
void bgo_zenith_uvw(int n_ant, const double *x, const double *y, const double *z,
                    float *u, float *v, float *w);

/* max |u|, max |v| over unflagged baselines (src/pacer_imager.cpp:213-221). */
void bgo_uv_max(int n_baselines, const float *u, const float *v, const int *baseline_flags,
                double *u_max, double *v_max);

/* delta_u = oversampling_factor * u_max / n_pixels, in metres (src/pacer_imager.cpp:497-499). */
double bgo_delta_uv(float oversampling_factor, double uv_max, int n_pixels);

/* Cotter-compatible channel frequency (src/pacer_imager.cpp:528-555). */
double bgo_channel_frequency_hz(double frequency_resolution_mhz, int n_averaged_channels,
                                double coarse_channel_bw_mhz, int coarse_channel,
                                int fine_channel, int cotter_compatible);

/* In-place geometric correction, phase +2*pi*w*nu/c, with w indexed per triangular baseline as
 * on the GPU (src/gpu/corrections_gpu.cpp:41-72); arithmetic as src/corrections.cpp:19-33.
 * w holds n_uvw_sets * B entries (one set for all intervals, or one per interval). */
void bgo_apply_geometric(float *vis, int n_intervals, int n_channels, int n_ant,
                         const float *w, int n_uvw_sets, const double *freqs_hz);

/* In-place cable correction, phase -2*pi*(L[a2]-L[a1])*nu/c (src/corrections.cpp:41-73). */
void bgo_apply_cable(float *vis, int n_intervals, int n_channels, int n_ant,
                     const double *cable_lengths, const double *freqs_hz);

/* uv cell of one baseline (src/gpu/gridding_gpu.cpp:24-54; CPU src/pacer_imager.cpp:332-369).
 * Returns N*v_index + u_index, or -1 when uv distance <= min_uv.  uv_sign is +1 or -1. */
int64_t bgo_cell_index(float u, float v, double delta_u, double delta_v, double wavelength,
                       double min_uv, int n_pixels, int uv_sign);

/*
 * Nearest-neighbour gridding, CPU semantics (src/pacer_imager.cpp:250-432):
 *  - one grid and one counter image per (interval, channel);
 *  - flagged baselines, NaN values and |re|,|im| >= 1e12 are skipped;
 *  - the visibility goes to (u,v) and its conjugate to (-u,-v), each adding 1 to the counter;
 *  - accumulation in float, baselines in ascending order;
 *  - uniform != 0 divides every cell by its counter afterwards (weighting "U", :421-428).
 * u, v hold n_uvw_sets * B entries; set t is used by interval t (n_uvw_sets == T) or set 0
 * for all intervals (n_uvw_sets == 1, the reference's case).  A cell index outside [0, N*N)
 * is skipped, as on the GPU (src/gpu/gridding_gpu.cpp:103,115).
 * Grids and counters are overwritten.  Returns the number of gridded points.
 */
int64_t bgo_gridding(const float *vis, int n_intervals, int n_channels, int n_ant,
                     const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                     const double *freqs_hz, double delta_u, double delta_v, int n_pixels,
                     double min_uv, int pol, int uniform, float *grids, float *counters);

/* Batched unnormalised 2D inverse DFT (sign +), out of place, FP64 (the checker's FFT). */
void bgo_fft2_inverse_f64(const double *in, double *out, int n_pixels, int n_images);
/* The same transform in FP32 arithmetic (used for the timed CPU baseline). */
void bgo_fft2_inverse_f32(const float *in, float *out, int n_pixels, int n_images);
/* the same transform one line at a time (the check of bgo_fft2_inverse_f32's blocked form) */
void bgo_fft2_inverse_f32_scalar(const float *in, float *out, int n_pixels, int n_images);

/* fftshift by swapping halves along x then y (src/pacer_imager.cpp:110-128), complex data. */
void bgo_fft_shift_f32(float *image, int x_side, int y_side);
void bgo_fft_shift_f64(double *image, int x_side, int y_side);

/*
 * Dirty images from grids (src/pacer_imager.cpp:134-208): inverse FFT, multiply every pixel
 * by 1/sum(counter) of its own image, fftshift.  FP64 output.
 */
void bgo_image_f64(const float *grids, const float *counters, int n_pixels, int n_images,
                   double *images);

/* Whole CPU path in FP32 arithmetic (reference CPU run(): gridding, FFT, normalise, shift),
 * OpenMP over images; used as the timed CPU baseline. */
void bgo_run_f32(const float *vis, int n_intervals, int n_channels, int n_ant,
                 const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                 const double *freqs_hz, double delta_u, double delta_v, int n_pixels,
                 double min_uv, int pol, float *grids, float *counters, float *images);

/* Per-image sum of a float buffer (src/gpu/gpu_utils.cpp:19-71), accumulated in double. */
void bgo_vector_sum(const float *data, int64_t image_size, int n_images, double *sums);

/* Mean of complex images, pixel by pixel (src/gpu/gpu_utils.cpp:143-161). */
void bgo_image_average(const float *images, int64_t image_size, int n_images, float *out);

int bgo_max_threads(void);

/* Kaiser-Bessel convolutional gridding (src/pacer_imager.cpp:378-403, 565-750): oversampling
 * 1023, alpha 8.6, with or without the sinc factor.  bgo_kb_tables writes the reference's
 * _griddingKernels as double[1023][kernel_size]; bgo_gridding_kb is bgo_gridding with each point
 * and its conjugate spread over kernel_size^2 cells (sums in double, rounded to float per add). */
#define BGO_KB_OVERSAMPLING 1023
void bgo_kb_tables(int kernel_size, int with_sinc, double *tables);
int64_t bgo_gridding_kb(const float *vis, int n_intervals, int n_channels, int n_ant, const float *u,
                        const float *v, int n_uvw_sets, const int *baseline_flags, const double *freqs_hz,
                        double delta_u, double delta_v, int n_pixels, double min_uv, int pol,
                        int kernel_size, int with_sinc, float *grids, float *counters);

/* Pointed-observation UVW of every baseline for n_steps timesteps (src/antenna_positions.cpp:23-92,
 * src/pacer_geometry.h:101-134, 208-215, 312-334): xyz double[n_ant][3]; steps double[n_steps][17]
 * = rmatpr row-major, then sin, cos of lmst, lmst2000, ha2000 and dec_aber; u, v, w float[n_steps][B]. */
void bgo_pointed_uvw(const double *xyz, int n_ant, const double *steps, int n_steps, float *u, float *v,
                     float *w);

/* Correlation matrices float[n_matrices][n_ant][n_ant] (XX, and YY or NULL) to visibility
 * records float[n_matrices][B][4][2] (apps/pacer_imager_main.cpp:720-804). */
void bgo_ingest_matrices(const float *re_xx, const float *im_xx, const float *re_yy,
                         const float *im_yy, int n_ant, int64_t n_matrices, float *vis);

/* Block-scaled 16-bit visibility storage of the GB300 imager (no reference counterpart; the
 * format is stated in blink_compress.c).  format: BGO_VIS_S16, BGO_VIS_BF16 or BGO_VIS_FP16. */
enum { BGO_VIS_C64 = 0, BGO_VIS_S16 = 1, BGO_VIS_BF16 = 2, BGO_VIS_FP16 = 3 };
int64_t bgo_compressed_blocks(int64_t n_baselines);
void bgo_compress(const float *vis, int64_t n_images, int64_t n_baselines, int format,
                  uint16_t *data, float *scales);
void bgo_decompress(const uint16_t *data, const float *scales, int64_t n_images,
                    int64_t n_baselines, int format, float *vis);

#ifdef __cplusplus
}
#endif
#endif
