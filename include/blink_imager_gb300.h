/*
 * blink_imager_gb300 -- C ABI of the GB300-native BLINK dirty-imaging path.
 *
 * Replaces the GPU half of PaCER-BLINK-Project/imager: the phase corrections, nearest-
 * neighbour uv gridding, inverse 2D FFT, fftshift and normalisation that CPacerImagerHip runs
 * (src/gpu/pacer_imager_hip.cpp:36-146).  Two layers:
 *
 *  1. Free functions with the reference's argument meaning, on device pointers, one per
 *     reference GPU entry point (the headers in src/gpu).  A caller that already holds device buffers
 *     (the CPacerImagerHip shape) swaps the call and nothing else.
 *  2. An imager handle that keeps the array state (UVW, flags, cable lengths, frequencies)
 *     resident on the device and images whole blocks in one call, with the corrections fused
 *     into gridding and the fftshift / normalisation fused into the FFT (bgi_image).
 *
 * Data layout (as the reference, src/gpu/gridding_gpu.cpp:72-76):
 *   visibilities  float[T][C][B][4 pols][re,im]; pols XX, XY, YX, YY; B = A(A+1)/2;
 *                 baseline b = a1*(a1+1)/2 + a2 with a1 >= a2
 *   grids/images  float[T][C][N][N][re,im]      counters float[...][N][N]
 *   u, v, w       float[n_uvw_sets][B] metres; set t serves interval t when n_uvw_sets == T,
 *                 set 0 serves every interval when n_uvw_sets == 1 (the reference's case)
 *
 * Every function returns BGI_OK (0) or a negative status; bgi_last_error() gives the message
 * of the calling thread's last failure.  Nothing throws across this interface.
 *
 * Device memory the library keeps (a handle's buffers, the twiddle table of each image side
 * that is not a power of two, the address of bgi_image_noalloc's static scratch) belongs to the
 * device's primary context: after a cudaDeviceReset the library must not be used again in that
 * process.  Streams are
 * cudaStream_t passed as void* (NULL = legacy default stream).  Launches are asynchronous
 * unless stated otherwise.
 */
#ifndef BLINK_IMAGER_GB300_H
#define BLINK_IMAGER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Exported symbols: the library is built with hidden visibility and exports only these. */
#if defined(__GNUC__)
#define BGI_API __attribute__((visibility("default")))
#else
#define BGI_API
#endif

#define BGI_VERSION_MAJOR 0
#define BGI_VERSION_MINOR 1

enum bgi_status {
    BGI_OK = 0,
    BGI_ERR_INVALID = -1,     /* bad argument (size, pointer, enum) */
    BGI_ERR_CUDA = -2,        /* a CUDA call or launch failed */
    BGI_ERR_ALLOC = -3,       /* device or pinned allocation failed */
    BGI_ERR_UNSUPPORTED = -4, /* valid input this build does not handle (e.g. image side) */
    BGI_ERR_STATE = -5,       /* handle not ready (array or frequencies not set) */
    BGI_ERR_BUSY = -6,        /* serving: the request queue is full (bgi_server_config.max_queued) */
    BGI_ERR_CANCELLED = -7    /* serving: the request was cancelled before it was admitted */
};

/* Polarisation to image; same order as the reference's enum class Polarization
 * (src/gridding.hpp:4). */
enum bgi_pol { BGI_POL_XX = 0, BGI_POL_YY = 1, BGI_POL_I = 2, BGI_POL_V = 3 };

/* Visibility storage.  BGI_VIS_C64 is the reference's layout, float[T][C][B][4 pols][re,im]
 * (pols XX, XY, YX, YY).  The block-scaled 16-bit formats (no reference counterpart) store
 * pol planes, data uint16[T][C][4][B][re,im], with one float scale per block of 128 baselines
 * of a plane (256 components): scales float[T][C][4][ceil(B/128)], value = element * scale.
 * A component that is NaN or has |x| >= 1e12 (skipped by the gridding) is stored as invalid
 * and read back as NaN; m is the largest |x| of a block's valid components (0 if none).
 *   BGI_VIS_S16:  scale = m / 32767, element = rint(x / scale) as int16 (+-32767), invalid
 *                 -32768.  Error <= scale / 2 per component (relative L2 about 3e-5).
 *   BGI_VIS_BF16: scale = m (1 if m == 0), element = bfloat16(x / scale), nearest even;
 *                 relative error up to 2^-9 per component (about 2e-3 relative L2).
 *   BGI_VIS_FP16: as BF16 with IEEE binary16 elements; up to 2^-12 relative (about 2e-4). */
enum bgi_vis_format { BGI_VIS_C64 = 0, BGI_VIS_S16 = 1, BGI_VIS_BF16 = 2, BGI_VIS_FP16 = 3 };

/* Counter layout for bgi_gridding_gpu. */
enum bgi_counter_mode {
    /* counters float[C][N][N], counted for interval 0 only (src/gpu/gridding_gpu.cpp:107,117) */
    BGI_COUNTERS_FIRST_INTERVAL = 0,
    /* counters float[T][C][N][N], one per image (the CPU path, src/pacer_imager.cpp:269,387) */
    BGI_COUNTERS_PER_IMAGE = 1
};

/* Flags of bgi_image / bgi_image_host. */
#define BGI_APPLY_GEOMETRIC 0x1u /* ApplyGeometricCorrections (src/pacer_imager.cpp:463-464) */
#define BGI_APPLY_CABLE 0x2u     /* ApplyCableCorrections (src/pacer_imager.cpp:466-473) */
/* Real images float[T][C][N][N] instead of complex64 images: the real part, the part the
 * reference's image averaging reads (src/utils.cpp:4-22), written by the last FFT pass with
 * half the output bytes.  (On the half-plane path the images are real by construction; on the
 * full plane the imaginary parts, rounding noise of a Hermitian grid, are dropped.) */
#define BGI_OUTPUT_REAL 0x4u
/* Weighting "U" of the CPU path (src/pacer_imager.cpp:419-428): after gridding, every cell of an
 * image's grid is divided by its counter (the number of points gridded into it), before the
 * transform; the normalisation stays 1/sum(counters).  As there, every cell is divided, so an
 * empty cell becomes 0/0 = NaN and so does every pixel of that image's transform.  Grids the full
 * plane, with per-image counter grids in the handle's scratch. */
#define BGI_WEIGHT_UNIFORM 0x8u

BGI_API const char *bgi_last_error(void);
BGI_API int bgi_version(void); /* 100 * major + minor */

/* ------------------------------------------------------------------------------------------
 * 1. Reference GPU entry points on device pointers
 * ------------------------------------------------------------------------------------------ */

/* apply_geometric_corrections_gpu (src/gpu/corrections_gpu.cpp:90-101): in place,
 * V <- V * exp(+2*pi*i*w[b]*nu/c) on all four pols; w indexed per triangular baseline. */
BGI_API int bgi_apply_geometric_corrections_gpu(float *vis, int n_ant, int n_channels, int n_intervals,
                                        const float *w, int n_uvw_sets, const double *freqs_hz,
                                        void *stream);

/* apply_cable_lengths_corrections_gpu (src/gpu/corrections_gpu.cpp:75-87): in place,
 * V <- V * exp(-2*pi*i*(L[a2]-L[a1])*nu/c). */
BGI_API int bgi_apply_cable_lengths_corrections_gpu(float *vis, int n_ant, int n_channels,
                                            int n_intervals, const double *cable_lengths,
                                            const double *freqs_hz, void *stream);

/* gridding_gpu (src/gpu/gridding_gpu.cpp:130-155): adds every unflagged, finite visibility
 * (|re|,|im| < 1e12) with uv distance > min_uv at its uv cell and its conjugate at the mirrored
 * cell of grids[T][C][N][N], and 1 to the matching counters cells.  Cell indices are bit-exact
 * with the reference (FP64 round-half-away of u/lambda/delta_u).  Grids and counters are
 * accumulated into, not cleared (the caller zeroes them, as the reference's caller does).
 * antenna_weights is accepted for signature parity and unused, as in the reference. */
BGI_API int bgi_gridding_gpu(const float *vis, int n_ant, int n_channels, int n_intervals,
                     const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                     const float *antenna_weights, const double *freqs_hz, double delta_u,
                     double delta_v, int n_pixels, double min_uv, int pol, int counter_mode,
                     float *counters, float *grids, void *stream);

/* Deterministic gridding: the same inputs, checks and cell indices as bgi_gridding_gpu, but
 * every cell sums its points in the CPU gridding loop's order (baseline by baseline, each
 * visibility before its conjugate: src/pacer_imager.cpp:297-408), so grids are reproducible
 * run to run and bit-identical to that loop's FP32 sums.  No reference GPU counterpart (the
 * reference's gridding_kernel adds with float atomics in scheduling order).  The caller
 * provides a 16-byte aligned device workspace; bgi_gridding_sorted_workspace gives the bytes
 * needed to grid n_images images in one chunk (a smaller workspace of at least one image's
 * share is used chunk by chunk).  At most 46,340 antennas. */
BGI_API int bgi_gridding_sorted_workspace(int n_ant, int n_pixels, int n_images, size_t *bytes);
BGI_API int bgi_gridding_sorted_gpu(const float *vis, int n_ant, int n_channels, int n_intervals,
                            const float *u, const float *v, int n_uvw_sets,
                            const int *baseline_flags, const double *freqs_hz, double delta_u,
                            double delta_v, int n_pixels, double min_uv, int pol,
                            int counter_mode, float *counters, float *grids, void *workspace,
                            size_t workspace_bytes, void *stream);

/* Kaiser-Bessel convolutional gridding (the reference's CPU gridding with
 * m_nConvolvingKernelSize > 0, src/pacer_imager.cpp:378-403 and 565-750; CPU only there): as
 * bgi_gridding_gpu, but each visibility and its conjugate are spread over kernel_size^2 cells
 * (1..16) with the reference's kernel (1023 oversampled rows, Kaiser-Bessel alpha 8.6, times a
 * sinc unless with_sinc == 0); counters count the nearest cells, as the reference's.  Each call
 * uploads its kernel table into stream-ordered memory on `stream` (cudaMallocAsync, freed after
 * the launch), so calls on different streams do not share it. */
BGI_API int bgi_gridding_kb_gpu(const float *vis, int n_ant, int n_channels, int n_intervals,
                                const float *u, const float *v, int n_uvw_sets,
                                const int *baseline_flags, const double *freqs_hz, double delta_u,
                                double delta_v, int n_pixels, double min_uv, int pol, int counter_mode,
                                float *counters, float *grids, int kernel_size, int with_sinc,
                                void *stream);

/* gpufftPlanMany + gpufftExecC2C(..., BACKWARD) (src/gpu/pacer_imager_hip.cpp:83-99): batched
 * unnormalised inverse 2D FFT, out of place, our own kernels.  n_pixels: any side 1..4096
 * (powers of two 16..4096 with compile-time radix-8/16/32 passes; every other side with
 * mixed-radix passes -- radices 2, 3, 4, 5, 8 in registers, other primes as direct sums -- whose
 * twiddle table is allocated once per device and side, at its first use, and kept until exit). */
BGI_API int bgi_fft_inverse_gpu(const float *grids, float *images, int n_pixels, int n_images,
                        void *stream);

/* fft_shift_and_norm_gpu (src/gpu/gpu_utils.cpp:128-140): swap halves along x then y and
 * divide every pixel of image i by fnorm[i % fnorm_size].  x_side must be even. */
BGI_API int bgi_fft_shift_and_norm_gpu(float *images, int x_side, int y_side, int n_images,
                               const float *fnorm, int fnorm_size, void *stream);

/* The CPU gridder's weighting "U" step (src/pacer_imager.cpp:419-428; no GPU counterpart in the
 * reference): grids[i] /= counters[i] for every cell of n_images complex grids of n_pixels^2
 * cells (IEEE division, so empty cells become 0/0 = NaN as in the reference).  In place. */
BGI_API int bgi_uniform_weighting_gpu(float *grids, const float *counters, int n_pixels, int n_images,
                                      void *stream);

/* vector_sum_gpu (src/gpu/gpu_utils.cpp:62-71): sums[i] = sum of data[i*image_size ...]. */
BGI_API int bgi_vector_sum_gpu(const float *data, int64_t image_size, int n_images, float *sums,
                       void *stream);

/* image_averaging_gpu (src/gpu/gpu_utils.cpp:153-161): out = mean of n_images complex
 * images of image_size pixels. */
BGI_API int bgi_image_averaging_gpu(const float *images, int64_t image_size, int n_images, float *out,
                            void *stream);

/* ------------------------------------------------------------------------------------------
 * 2. Imager handle: resident array state, fused whole-path imaging
 *    (CPacerImagerHip with its members, src/gpu/pacer_imager_hip.h:12-58)
 * ------------------------------------------------------------------------------------------ */
/* A handle holds device state and per-call scratch: calls on one handle must not overlap (one
 * host thread at a time, and a later call may reuse the scratch of an earlier one on its
 * streams); different handles are independent.  The serving runtime (section 3) gives each of
 * its slots its own handles. */
typedef struct bgi_imager bgi_imager;

typedef struct bgi_config {
    int n_pixels;              /* image side N, 1..4096 (sides that are not powers of two from 16
                                  up are imaged on the full plane with mixed-radix FFT passes) */
    float oversampling_factor; /* delta_u = osf * u_max / N (src/pacer_imager.cpp:497) */
    int pol;                   /* enum bgi_pol */
    double min_uv;             /* uv distance cut in wavelengths (strictly greater passes) */
    int max_images_per_wave;   /* images gridded and transformed per launch wave; 0 = auto */
    int device;                /* CUDA device ordinal */
    int full_plane;            /* 1: always transform the full N x N grid; 0: when every pixel
                                  coordinate is below N, grid only the half plane u <= N/2 and
                                  finish with a complex-to-real transform (the grid is
                                  Hermitian, so the image is real: same images, half the work) */
} bgi_config;

BGI_API int bgi_create(const bgi_config *cfg, bgi_imager **out);
BGI_API int bgi_destroy(bgi_imager *im);

/* Resident array state from host arrays (copied).  u, v, w: float[n_uvw_sets][B];
 * baseline_flags: int[B], flag > 0 = flagged as in the reference's GPU gridder
 * (src/gpu/gridding_gpu.cpp:101; for the 0/1 flags of CPacerImager::UpdateFlags,
 * src/pacer_imager.cpp:60-86, the CPU path's nonzero test agrees; autos are flagged by the
 * caller); cable_lengths: double[n_ant].  Computes u_max/v_max over baselines with flag 0 in
 * every set and delta_u/delta_v (src/pacer_imager.cpp:213-221, 497-499).  A negative flag
 * (gridded, but outside u_max) keeps the handle's blocks on the full plane. */
BGI_API int bgi_set_array(bgi_imager *im, int n_ant, int n_uvw_sets, const float *u, const float *v,
                  const float *w, const int *baseline_flags, const double *cable_lengths);

/* Channel frequencies in Hz (host array, copied). */
BGI_API int bgi_set_frequencies(bgi_imager *im, int n_channels, const double *freqs_hz);

/* 1 when bgi_image would take the half-plane path for the current array, frequencies and
 * configuration (16-byte aligned complex images; not with a convolution kernel or
 * BGI_WEIGHT_UNIFORM, which grid the full plane), 0 when it would transform the full plane;
 * negative status on error. */
BGI_API int bgi_half_plane(const bgi_imager *im);

/* Overrides delta_u and delta_v (metres) of the current array state, e.g. with the values of
 * a whole observation when this handle images one shard of it (gridding_gpu takes them as
 * arguments, src/gpu/gridding_gpu.cpp:134).  bgi_set_array recomputes them. */
BGI_API int bgi_set_uv_cell(bgi_imager *im, double delta_u, double delta_v);

/* delta_u, delta_v (metres) and u_max, v_max of the current array state. */
BGI_API int bgi_get_uv_cell(const bgi_imager *im, double *delta_u, double *delta_v, double *u_max,
                    double *v_max);

/* Bound on the pixel coordinates |u| and |v| of every point the half-plane path grids for the
 * current array, frequencies and uv cell: floor(u_max * nu_max / (c * delta_u)) + 2, and the
 * same in v, capped at N/2 (no addition of the reference; with delta_u = osf * u_max / N it is
 * about N * nu_max / (c * osf)).  The half-plane FFT passes transform and stage only columns
 * 0..ext_u and load only rows 0..ext_v and N-ext_v..N-1: the rest of the grid is zero.  N/2 in
 * both when bgi_half_plane is 0. */
BGI_API int bgi_get_uv_extent(const bgi_imager *im, int *ext_u, int *ext_v);

/* The same bound for given values (host only, no handle): u_max, v_max and delta_u, delta_v in
 * metres, the highest channel frequency in Hz, the image side. */
BGI_API int bgi_uv_extent(double u_max, double v_max, double delta_u, double delta_v,
                          double freq_max_hz, int n_pixels, int *ext_u, int *ext_v);

/* Pointed-observation UVW on the device (CAntennaPositions::CalculateUVW with metadata,
 * src/antenna_positions.cpp:23-92; PacerGeometry::CalcUVW_NEW, precXYZ and CalcUVW,
 * src/pacer_geometry.h).  A timestep is what the reference derives once per timestep with PAL
 * (PrepareTimestepUVW): the precession-nutation matrix rmatpr and the sines and cosines of the
 * local mean sidereal time, its J2000 value, the J2000 hour angle and the aberrated
 * declination; bgi_uvw_step_from_angles fills one from the angles (host libm).  Antenna
 * positions xyz are local XYZ in metres, double[n_ant][3].  bgi_pointed_uvw_gpu writes
 * u, v, w float[n_steps][B] on the device (xyz and steps in device memory); the result is the
 * reference's, bit for bit, for the same timestep numbers.  bgi_set_array_pointed does the same
 * into a handle's resident state (one UVW set per interval) and derives u_max, v_max and
 * delta_u/v there, as bgi_set_array. */
typedef struct bgi_uvw_step {
    double rmatpr[9]; /* row-major */
    double sin_lmst, cos_lmst, sin_lmst2000, cos_lmst2000, sin_ha2000, cos_ha2000, sin_dec, cos_dec;
} bgi_uvw_step;
BGI_API int bgi_uvw_step_from_angles(const double *rmatpr, double ha2000, double dec_aber, double lmst,
                                     double lmst2000, bgi_uvw_step *out);
BGI_API int bgi_pointed_uvw_gpu(const double *xyz, int n_ant, const bgi_uvw_step *steps, int n_steps,
                                float *u, float *v, float *w, void *stream);
BGI_API int bgi_set_array_pointed(bgi_imager *im, int n_ant, const double *xyz_host, int n_steps,
                                  const bgi_uvw_step *steps_host, const int *baseline_flags,
                                  const double *cable_lengths);

/* Whole path on device buffers: vis float[T][C][B][4][2] (read only: corrections are applied
 * in registers and not written back), images float[T][C][N][N][2] out.  Each image is
 * normalised by its own weight sum (the CPU path, src/pacer_imager.cpp:171-178) and
 * fftshifted.  Stream-ordered; no host synchronisation.
 * Repeated calls: when a call repeats the previous call on the handle exactly (same buffers,
 * interval count, flags and format, no setter in between), the second such call is also
 * recorded into a CUDA graph, and the calls after it launch that graph on `stream` instead of
 * issuing each wave's kernels: the same work and results, one host launch per call.  Not under
 * stage timing or inside a stream capture of the caller's; the same holds for the host-buffer
 * calls below when their host buffers are page-locked.  A replayed call is ordered after the
 * earlier work of `stream` only (not after the handle's own streams), so a caller who moves a
 * handle's calls to another stream orders the two streams first, as the handle's rule that
 * calls do not overlap already asks. */
/* 1 when the handle holds the recorded graph of its last call (the next identical call
 * launches it), 0 otherwise; negative status on error.  bgi_set_replay(im, 0) turns the
 * recording off for the handle (every call issues its stream work; for one-off calls, whose
 * recording would not be used), 1 (the default) on. */
BGI_API int bgi_replay_ready(const bgi_imager *im);
BGI_API int bgi_set_replay(bgi_imager *im, int enable);
BGI_API int bgi_image(bgi_imager *im, const float *vis, int n_intervals, unsigned flags, float *images,
              void *stream);

/* The same on host buffers: copies vis to the device, images it, copies images back and
 * synchronises the stream before returning. */
BGI_API int bgi_image_host(bgi_imager *im, const float *vis_host, int n_intervals, unsigned flags,
                   float *images_host, void *stream);

/* Block-scaled 16-bit visibilities (enum bgi_vis_format; no reference counterpart).
 * bgi_compressed_size gives the bytes of a block's data and scales; bgi_compress_visibilities
 * encodes complex64 visibilities float[T][C][B][4][2] (device) into them, bit for bit as the
 * format states.  bgi_image_compressed / bgi_image_compressed_host image such a block as
 * bgi_image / bgi_image_host do (corrections, if flagged, applied to the decoded values); the
 * gridding reads only the pol planes the handle's pol needs, and the host variant uploads only
 * those planes and their scales.  Device data must be 4-byte aligned. */
BGI_API int bgi_compressed_size(int n_ant, int n_channels, int n_intervals, size_t *data_bytes,
                                size_t *scale_bytes);
BGI_API int bgi_compress_visibilities(const float *vis, int n_ant, int n_channels, int n_intervals,
                                      int format, void *data, float *scales, void *stream);
/* ConvertFits2XCorr (apps/pacer_imager_main.cpp:720-804), on the GPU for whole blocks:
 * correlation matrices float[T][C][n_ant][n_ant] (row = first antenna; XX, and YY or both NULL)
 * to visibilities.  Element (i, j), j <= i, is baseline i(i+1)/2 + j; XX goes to pol 0, YY to
 * pol 3 (zero without YY matrices, as the reference), XY and YX are zero (the reference leaves
 * them unset).  format BGI_VIS_C64 writes records float[T][C][B][4][2] to data; the 16-bit
 * formats write the pol planes and scales directly, encoded as bgi_compress_visibilities would
 * encode the records (one pass from correlator output to stored visibilities). */
BGI_API int bgi_ingest_correlation_matrices(const float *re_xx, const float *im_xx,
                                            const float *re_yy, const float *im_yy, int n_ant,
                                            int n_channels, int n_intervals, int format, void *data,
                                            float *scales, void *stream);
BGI_API int bgi_image_compressed(bgi_imager *im, int format, const void *data, const float *scales,
                                 int n_intervals, unsigned flags, float *images, void *stream);
BGI_API int bgi_image_compressed_host(bgi_imager *im, int format, const void *data_host,
                                      const float *scales_host, int n_intervals, unsigned flags,
                                      float *images_host, void *stream);

/* From correlator output to images, on host buffers: the block's correlation matrices
 * float[T][C][n_ant][n_ant] (XX; YY or both NULL, as bgi_ingest_correlation_matrices) are
 * uploaded chunk by chunk, converted on the device into stored visibilities of `format` (complex64
 * records or a 16-bit format, encoded as bgi_compress_visibilities encodes), imaged as
 * bgi_image_compressed / bgi_image do with `flags`, and the images copied back; uploads, ingest,
 * imaging and downloads of different chunks overlap.  Replaces the reference's host-side
 * ConvertFits2XCorr (apps/pacer_imager_main.cpp:720-804) followed by run(); the YY matrices are
 * uploaded only for pols YY and I.  Synchronises the stream before returning. */
BGI_API int bgi_image_correlation_matrices_host(bgi_imager *im, int format, const float *re_xx, const float *im_xx,
                                                const float *re_yy, const float *im_yy, int n_intervals,
                                                unsigned flags, float *images_host, void *stream);

/* Per-image weight sums (number of gridded points) of the last bgi_image call on this
 * handle, as uint32[n_images]; copies to host and synchronises the stream. */
BGI_API int bgi_last_weight_sums(bgi_imager *im, uint32_t *sums_host, int n_images, void *stream);

/* Image coordinates as the reference attaches them to its Images
 * (src/gpu/pacer_imager_hip.cpp:110-119, src/pacer_imager.cpp:192-201): the phase centre in
 * degrees (the caller's; the reference takes it from its metadata) and the pixel scales
 * (1 / (osf * u_max)) * 180/pi and (1 / (osf * v_max)) * 180/pi in degrees, u_max and v_max
 * in metres as the handle holds them.  Needs the array state. */
typedef struct bgi_image_wcs {
    double ra_deg, dec_deg;
    double pixscale_ra_deg, pixscale_dec_deg;
} bgi_image_wcs;
BGI_API int bgi_get_image_wcs(const bgi_imager *im, double ra_deg, double dec_deg, bgi_image_wcs *out);

/* FITS files of host images (the reference writes its Images through astroio's
 * Images::to_fits_files, apps/pacer_imager_main.cpp:578; astroio is not part of the
 * reference, so the layout here is the FITS standard's).  One image per file: a primary HDU with
 * BITPIX -32 (big-endian float32), NAXIS1 = nx columns varying fastest, NAXIS2 = ny rows in
 * memory order, BUNIT, and with wcs the SIN-projection keywords CTYPE/CRVAL/CRPIX/CDELT/CUNIT
 * (centre pixel nx/2+1, ny/2+1, the fftshifted phase centre; CDELT1 = -pixscale_ra,
 * CDELT2 = pixscale_dec) and EQUINOX; FREQ (Hz) when freq_hz > 0.  pixel_stride: floats from
 * one pixel to the next, 1 for real images, 2 to write the real parts of complex images.
 * bgi_write_fits_block writes every image of a block [T][C][ny][nx] to
 * <dir>/<prefix>_t<TTTT>_c<CCCC>.fits with INTERVAL and CHANNEL cards (and FREQ from
 * freqs_hz[c] when given).  Host code only; no reference counterpart in the imaging path. */
BGI_API int bgi_write_fits(const char *path, const float *image_host, int nx, int ny, int pixel_stride,
                           const bgi_image_wcs *wcs, double freq_hz);
BGI_API int bgi_write_fits_block(const char *dir, const char *prefix, const float *images_host,
                                 int n_intervals, int n_channels, int nx, int ny, int pixel_stride,
                                 const bgi_image_wcs *wcs, const double *freqs_hz);

/* Dirty images with no device allocation.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory while they run -- a real-time pipeline that
 * budgets all GPU memory when an observation starts, a host framework that owns the device
 * allocator, or code that must not call cudaMalloc/cudaFree on a live stream because they can
 * synchronise the device.  Same work and arguments as bgi_gridding_gpu on already-corrected
 * visibilities followed by bgi_fft_inverse_gpu, the fftshift and 1/sum(weights) of each image
 * (the CPU path's normalisation): vis float[T][C][B][4][2] in, images float[T][C][N][N][2] out.
 * Scratch is a static 32 MiB grid plus weight counters that every GPU loading the library
 * holds until exit; the image side is limited to 2048 (larger sides return
 * BGI_ERR_UNSUPPORTED).  CUDA loads device code lazily by default, so the scratch is committed
 * on a device by the first call there (which looks up its address and loads the modules it
 * uses): make one warm-up call per device when setting a memory budget and before any stream
 * capture, or run with CUDA_MODULE_LOADING=EAGER to commit it when the context is created.
 * The address is cached per device: do not use the library after a cudaDeviceReset.  All calls share the scratch: each clears what it uses, but
 * calls that overlap on the GPU race -- serialise them.  Makes no allocating call. */
BGI_API int bgi_image_noalloc(const float *vis, int n_ant, int n_channels, int n_intervals,
                              const float *u, const float *v, int n_uvw_sets,
                              const int *baseline_flags, const double *freqs_hz, double delta_u,
                              double delta_v, int n_pixels, double min_uv, int pol, float *images,
                              void *stream);

/* Device fault word of a device: bit 0 set when a kernel's bounded wait on its own bulk
 * asynchronous copies gave up (after about 50 ms) and the kernel skipped its work instead of
 * hanging.  clear != 0 resets it after reading.  Synchronous.  bgi_image_host checks it and
 * returns BGI_ERR_CUDA when it is set.  bgi_selftest_wait_timeout launches one kernel that
 * waits on a barrier nothing arrives on, so that the limit runs out and sets the bit (a test of
 * that path; it takes about 50 ms of one SM).  No reference counterpart. */
BGI_API int bgi_device_fault(int device, unsigned int *fault_bits, int clear);
BGI_API int bgi_selftest_wait_timeout(int device, void *stream);

/* Arithmetic of the inverse FFT's last pass on the half-plane path (no reference counterpart).
 * BGI_FFT_SIMT (default): FP32 radix-16/32 Stockham passes on the CUDA cores.
 * BGI_FFT_TENSOR_SPLIT16: the complex-to-real row pass's length-N/2 transforms as two dense
 *   16-point DFT products on the tensor cores (warp-level mma.sync, FP16 operands, FP32
 *   accumulation), every operand split into FP16 hi + lo parts (three products: lo*hi, hi*lo,
 *   hi*hi), each row scaled by a power of two into FP16's range; about 22 significant bits per
 *   operand, so images stay within ~1e-6 relative L2 of the FP32 passes.  Image side 512 only
 *   (BGI_ERR_UNSUPPORTED otherwise); full-plane calls keep the FP32 passes. */
enum bgi_fft_mode { BGI_FFT_SIMT = 0, BGI_FFT_TENSOR_SPLIT16 = 1 };
BGI_API int bgi_set_fft_mode(bgi_imager *im, int mode);
BGI_API int bgi_get_fft_mode(const bgi_imager *im, int *mode);

/* Launch schedule of the bgi_image* calls: images per wave (0 = auto: about 26 MiB of grid
 * per lane, 24 half-plane images at 512^2), lanes (1..8 streams that image alternate waves,
 * each with its own grid scratch; 2 by default), images per gridding thread (2, 4 or 8; 0 =
 * default: 4 on the half-plane path, else 2 below 65,536 baselines and 4 above; on the half
 * plane 4 and 8 issue all of a thread's visibility loads before gridding any), warp-aggregated
 * gridding atomics (bgi_set_gridding_aggregation) and the FFT arithmetic (bgi_set_fft_mode).
 * bgi_autotune times every wave size in {auto, 1, 2, 3, 4, 8, 12, 16, 20, 24, 28, 32, 40, 48,
 * 64} (up to the block's image count) with 1-8 lanes on the caller's own block (one call to size
 * the scratch, then three timed with CUDA events on the stream as launches of the call's
 * recorded graph, the form repeated calls take), times the three fastest again over ten calls each, then, at the best of those, 2, 4 and 8 images per gridding thread, 4 and 8
 * with aggregated atomics (half plane), the column pass's second radix (bgi_set_column_radix)
 * and (image side 512, half plane) the tensor-core row pass (ten timed calls each);
 * it keeps the fastest on the handle, frees the candidates' scratch and writes the best
 * milliseconds per call to *best_ms (may be NULL).  Synchronous; `images` receives the block's
 * images.  No reference counterpart. */
BGI_API int bgi_set_gridding_images_per_thread(bgi_imager *im, int images_per_thread);
/* Radix of the half-plane column pass: every power-of-two side has its default radix (8 up to
 * 128, 16 at 256, 32 at 512 and 1024, 16 above), and sides 256..4096 a second compiled one (8,
 * 16, 16, 32, 32); 0 = the default, another value BGI_ERR_UNSUPPORTED.  bgi_autotune times the
 * second one too.  bgi_get_column_radix reports the radix in use. */
BGI_API int bgi_set_column_radix(bgi_imager *im, int radix);
BGI_API int bgi_get_column_radix(const bgi_imager *im, int *radix);
BGI_API int bgi_get_gridding_images_per_thread(const bgi_imager *im, int *images_per_thread);
/* Warp-aggregated gridding atomics (0 = off, the default; 1 = on): the visibilities of a warp
 * that land on the same cell are summed across its lanes before one atomic per distinct cell.
 * Applies on the half-plane path with 4 or 8 images per gridding thread (the default 4 there);
 * elsewhere the setting is kept and has no effect.  It pays where many points share few cells
 * (short baselines on a small grid) and costs a few percent where they are spread.  Sums are
 * regrouped, so cells agree with the plain atomics to FP32 rounding. */
BGI_API int bgi_set_gridding_aggregation(bgi_imager *im, int on);
BGI_API int bgi_get_gridding_aggregation(const bgi_imager *im, int *on);
BGI_API int bgi_set_schedule(bgi_imager *im, int images_per_wave, int lanes);
BGI_API int bgi_get_schedule(const bgi_imager *im, int *images_per_wave, int *lanes);
BGI_API int bgi_autotune(bgi_imager *im, int format, const void *data, const float *scales,
                         int n_intervals, unsigned flags, float *images, void *stream,
                         double *best_ms);

/* Batches of uneven items replayed as one CUDA graph (no reference counterpart).  An item is
 * one bgi_image / bgi_image_compressed call on device buffers: its imager (array, image side,
 * pol and schedule), storage format, data (+ scales), interval count, flags and images.
 * bgi_batch_create runs the items once on `stream` (sizing every scratch buffer; synchronous),
 * then captures them, in order, into a graph and instantiates it (each item overlaps its own
 * waves on its imager's lanes; items are not run at once, which would hold several imagers'
 * L2-sized grid scratch together and push it out of L2).  bgi_batch_launch
 * replays the whole batch with one graph launch on `stream`: the same buffers, read and written
 * again.  The imagers and buffers must outlive the batch and keep their state (no set_array,
 * set_frequencies, set_uv_cell, set_schedule or set_deterministic on them while it exists;
 * stage timing off). */
typedef struct bgi_batch bgi_batch;
typedef struct bgi_batch_item {
    bgi_imager *imager;
    int format;          /* enum bgi_vis_format */
    const void *data;    /* device visibilities in that format */
    const float *scales; /* device block scales (16-bit formats), else NULL */
    int n_intervals;
    unsigned flags;      /* BGI_APPLY_*, BGI_OUTPUT_REAL */
    float *images;       /* device images */
} bgi_batch_item;
BGI_API int bgi_batch_create(const bgi_batch_item *items, int n_items, void *stream, bgi_batch **out);
BGI_API int bgi_batch_launch(bgi_batch *batch, void *stream);
BGI_API int bgi_batch_destroy(bgi_batch *batch);

/* Gridding kernel of the handle: 0 (default) nearest neighbour; 1..16 the Kaiser-Bessel kernel
 * of bgi_gridding_kb_gpu (the full-plane path; not with deterministic mode). */
BGI_API int bgi_set_gridding_kernel(bgi_imager *im, int kernel_size, int with_sinc);

/* Deterministic mode (default off): bgi_image and bgi_image_host grid with the ordered
 * per-cell sums of bgi_gridding_sorted_gpu (on the half plane when the handle takes it: its
 * cells hold the same sums as those cells of the full plane), so every image is the same bits
 * on every run and whatever else shares the call.  No reference counterpart. */
BGI_API int bgi_set_deterministic(bgi_imager *im, int enable);

/* Stage timing of bgi_image: when enabled, CUDA events are recorded on the stream of each
 * launch around it: gridding, the first FFT pass (rows in place, or the half-plane column
 * pass) and the second (columns with fftshift and normalisation, or the complex-to-real row
 * pass).  Recording adds no host
 * synchronisation.  bgi_get_stage_times synchronises on the recorded events, writes the summed
 * milliseconds and launch counts of the three stages since the last read, and resets them. */
BGI_API int bgi_set_stage_timing(bgi_imager *im, int enable);
BGI_API int bgi_get_stage_times(bgi_imager *im, double ms[3], int64_t launches[3]);

/* ------------------------------------------------------------------------------------------
 * 3. Serving runtime (no reference counterpart)
 *
 * A request loop over imager handles.  Arrays are registered once: each slot makes its own
 * handle from the registered state, so UVW, flags, cable lengths and frequencies stay resident on
 * the device.  bgi_server_submit queues a block of visibilities in host memory (pinned memory
 * gives asynchronous copies) and returns at once with a ticket.  A scheduler thread admits queued
 * requests in arrival order as soon as a slot (a CUDA stream) is free and the request's device
 * buffers (visibilities -- for the 16-bit formats only the pol planes the array's pol needs --
 * and images) fit both the byte budget and the device's free memory less reserve_bytes; it then
 * uploads, images and downloads on the slot's stream, so requests that arrive while others run
 * overlap with them on the GPU.  A request that cannot fit even on an idle device fails with
 * BGI_ERR_ALLOC.  Latency is measured from submission to the completion of the download.
 * With deterministic = 1 every request grids with the ordered gridder, so a request's images
 * are the same bits whatever else runs beside it; otherwise they agree to float summation
 * order (~1e-7 relative).  All calls are thread-safe.
 * ------------------------------------------------------------------------------------------ */
typedef struct bgi_server bgi_server;

typedef struct bgi_server_config {
    int device;               /* CUDA device of the server and of every array's config */
    int max_slots;            /* requests on the GPU at once (1..64) */
    size_t hbm_budget_bytes;  /* request buffers at once; 0 = free memory at creation less the reserve */
    size_t reserve_bytes;     /* device memory left free at admission (handles' scratch, other users) */
    int deterministic;        /* 1: ordered gridding (results independent of the mix) */
    int max_queued;           /* requests waiting for admission at most (0 = no limit); beyond it
                                 bgi_server_submit fails with BGI_ERR_BUSY */
} bgi_server_config;

typedef struct bgi_server_stats {
    uint64_t submitted, completed, failed, images, admission_waits, queued;
    size_t device_bytes_in_use, device_budget_bytes;
    double p50_ms, p99_ms, max_ms, mean_ms; /* submit-to-done latency of completed requests */
    double wall_s, images_per_s;            /* first submission to last completion */
    uint64_t rejected, cancelled;           /* submissions refused by a full queue; cancellations */
} bgi_server_stats;

BGI_API int bgi_server_create(const bgi_server_config *cfg, bgi_server **out);
/* Finishes every queued request, then frees the server. */
BGI_API int bgi_server_destroy(bgi_server *sv);
/* Registers an array (arguments as bgi_create + bgi_set_array + bgi_set_frequencies, copied). */
BGI_API int bgi_server_add_array(bgi_server *sv, const bgi_config *cfg, int n_ant, int n_uvw_sets,
                                 const float *u, const float *v, const float *w,
                                 const int *baseline_flags, const double *cable_lengths,
                                 int n_channels, const double *freqs_hz, int *array_id);
/* Queues a block: vis_host in `format` (scales_host for the 16-bit formats) for n_intervals
 * intervals of the array's channels; images_host receives T*C images (flags as bgi_image,
 * BGI_OUTPUT_REAL included).  Host buffers must stay valid until the request is collected. */
BGI_API int bgi_server_submit(bgi_server *sv, int array_id, int format, const void *vis_host,
                              const float *scales_host, int n_intervals, unsigned flags,
                              float *images_host, uint64_t *ticket);
/* Wait for (timeout_ms < 0: without limit) or poll a request; a finished request reports its
 * status once (BGI_OK or the failure, message in bgi_last_error) and its ticket is released. */
BGI_API int bgi_server_wait(bgi_server *sv, uint64_t ticket, int timeout_ms, int *status);
/* Cancels a request that has not been admitted yet: it leaves the queue and reports
 * BGI_ERR_CANCELLED to its wait or poll.  A request already on the GPU (or finished) is not
 * cancelled: BGI_ERR_STATE. */
BGI_API int bgi_server_cancel(bgi_server *sv, uint64_t ticket);
BGI_API int bgi_server_poll(bgi_server *sv, uint64_t ticket, int *done, int *status);
BGI_API int bgi_server_get_stats(bgi_server *sv, bgi_server_stats *out);
BGI_API int bgi_server_reset_stats(bgi_server *sv);

#ifdef __cplusplus
}
#endif
#endif
