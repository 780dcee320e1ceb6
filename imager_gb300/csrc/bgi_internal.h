// Host-side launchers shared between the kernel files and the C ABI (bgi_capi.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "bgi_common.cuh"

namespace bgi {

// Per-image weight counts live 128 bytes apart: blocks of many images add to them at once, and
// counters sharing a cache line would serialise those atomics in one L2 slice.
constexpr int kWsumStride = 32;

// ---- corrections (bgi_corrections.cu) ------------------------------------------------------
// In place on all four pols.  geometric: delay = w[set][b]; cable: delay = -(L[a2]-L[a1]).
int launch_geometric(float *vis, int n_ant, int n_channels, int n_intervals, const float *w,
                     int n_uvw_sets, const double *freqs, cudaStream_t s);
int launch_cable(float *vis, int n_ant, int n_channels, int n_intervals, const double *cable,
                 const double *freqs, cudaStream_t s);

// ---- gridding (bgi_gridding.cu) ------------------------------------------------------------
struct GridParams {
    const float *vis;        // [T][C][B][4][2] (BGI_VIS_C64), or uint32 pol planes [T][C][4][B]
    const float *vis_scales; // block-scaled formats: [T][C][4][vis_blocks]
    long long vis_blocks;    // scale blocks per pol plane, ceil(B / 128)
    int vis_format;          // enum bgi_vis_format
    const float *u, *v, *w;  // [n_uvw_sets][B]
    const float2 *dl;        // [B] L[a2]-L[a1] (cable delay) as a float pair (hi, lo), or null
    const int *flags;        // [B]
    const double *freqs;     // [C] Hz
    const ChannelConst *chan_consts;  // [C] make_channel_const(freqs[c], du, dv), or null (then
                                      // the gridding kernels compute them)
    float2 *grids;           // images [img - img_base][N*N]
    float *counters;         // optional counter grids, image img at counters[(img - counter_base) * N*N]
    unsigned int *wsum;      // optional per-image weight counts at wsum[(img - img_base) * kWsumStride]
    double du, dv, min_uv;
    long long n_baselines;
    int n_channels, n_intervals, n_uvw_sets, n_pixels, pol;
    int img_begin, img_count;  // images [img_begin, img_begin + img_count) of the block
    int img_base;              // grids/wsum index = img - img_base
    int counter_mode;          // -1 none, 0 first interval, 1 per image
    int counter_base;          // counter grid index = img - counter_base (0: the block's layout)
    int half_width;            // 0: full N x N grids; W > 0: half-plane grids [N][W], u <= N/2
    int apply_geom, apply_cable;
    int grids_zero;            // 1: grids hold zeros on entry (the ordered gridder then writes
                               // cells instead of reading them first)
    const float *kb_table;     // Kaiser-Bessel kernel rows [1023][kb_size] (kb_size > 0), else null
    int kb_size;               // 0: nearest neighbour; K: K x K convolution kernel (full plane)
    int cpt;                   // images per gridding thread: 2, 4 or 8, 0 = by array size
    int aggregate;             // 1: warp-aggregated atomics (half plane, 4 or 8 images per thread)
};
int launch_gridding(const GridParams &p, cudaStream_t s);
// table[c] = make_channel_const(freqs[c], du, dv) for c < n_channels
int launch_channel_consts(const double *freqs, int n_channels, double du, double dv, ChannelConst *table,
                          cudaStream_t s);
// Weighting "U" of the CPU path (src/pacer_imager.cpp:419-428): every cell divided by its
// counter (empty cells become 0/0, as there); clear_counters zeroes the counters after reading.
int launch_uniform_weighting(float2 *grids, float *counters, long long n_cells, bool clear_counters, cudaStream_t s);

// ---- pointed-observation UVW (bgi_geometry.cu) -------------------------------------------------
// steps: double[n_steps][17] (bgi_uvw_step); u, v, w: float[n_steps][B]
int launch_pointed_uvw(const double *xyz, int n_ant, const double *steps, int n_steps, float *u, float *v, float *w,
                       cudaStream_t s);
// out2[0], out2[1] = bit patterns of max |u|, max |v| over unflagged baselines of every set
int launch_uv_absmax(const float *u, const float *v, const int *flags, long long nb, int n_sets, unsigned *out2,
                     cudaStream_t s);

// ---- Kaiser-Bessel convolutional gridding (bgi_kb.cu) ----------------------------------------
constexpr int kMaxKernel = 16;
// the reference's kernel rows [1023][ksize] as float
void kb_tables(int ksize, bool with_sinc, std::vector<float> &out);
int launch_gridding_kb(const GridParams &p, const float *table, int ksize, cudaStream_t s);
// the free function's gridding: `table` uploaded into stream-ordered memory of this call, used
// by the launch and freed after it on `s`
int launch_gridding_kb_free(GridParams p, const std::vector<float> &table, int ksize, cudaStream_t s);

// ---- block-scaled 16-bit visibilities (bgi_compress.cu) -------------------------------------
long long vis_blocks(long long n_baselines);
int launch_compress(const float *vis, long long n_baselines, long long n_images, int format, void *data,
                    float *scales, cudaStream_t s);
// correlation matrices [img][n_ant][n_ant] (XX, YY or null) -> records (BGI_VIS_C64) or planes
int launch_ingest(const float *re_xx, const float *im_xx, const float *re_yy, const float *im_yy, int n_ant,
                  long long n_images, int format, void *data, float *scales, cudaStream_t s);

// ---- deterministic gridding (bgi_sorted.cu) ------------------------------------------------
// Point indices 2*b(+1) are 32-bit: at most 46,340 antennas (about 1.07e9 baselines).
constexpr int kSortedMaxAnt = 46340;
size_t sorted_workspace_bytes(long long n_baselines, int n_pixels, int n_images);
// Same parameters as launch_gridding (full-plane grids only, half_width 0); the workspace is
// reused chunk by chunk, so any size of at least one image's share works.
int launch_gridding_sorted(const GridParams &p, void *ws, size_t ws_bytes, cudaStream_t s);

// ---- FFT and image epilogues (bgi_fft.cu) --------------------------------------------------
// Image sides of the FFT: any side 1..4096 (powers of two 16..4096 with the compile-time passes of
// bgi_fft.cu, every other side with the mixed-radix passes of bgi_fft_any.cu, which keep one
// twiddle table per device and side, allocated at its first use).
bool fft_size_supported(int n);
bool fft_pow2_size(int n);
// Mixed-radix passes (bgi_fft_any.cu), the same contracts as launch_fft_rows and
// launch_fft_cols_to; an fftshift (wsum given) needs src != dst.
int launch_fft_any_rows(const float2 *src, float2 *dst, int n, int n_images, bool zero_src, cudaStream_t s);
int launch_fft_any_cols(float2 *src, float2 *dst, int n, int n_images, const unsigned int *wsum, bool zero_src,
                        bool real, cudaStream_t s);
// Row pass: src rows -> dst rows (inverse DFT along x); zero_src clears src after reading.
int launch_fft_rows(const float2 *src, float2 *dst, int n, int n_images, bool zero_src,
                    cudaStream_t s);
// Column pass in place on images; with wsum != null, also fftshift and multiply image i by
// (float)(1/wsum[i * kWsumStride]).
int launch_fft_cols(float2 *images, int n, int n_images, const unsigned int *wsum,
                    cudaStream_t s);
// Column pass from src into dst (src == dst: in place); zero_src clears src behind the loads
// (needs src != dst).  Final stores stream past L2.
// real: dst holds real images float[N][N] (needs wsum and zero_src).
int launch_fft_cols_to(float2 *src, float2 *dst, int n, int n_images, const unsigned int *wsum,
                       bool zero_src, cudaStream_t s, bool real = false);
// Half-plane imaging (real images of Hermitian grids): grids [img][N][W] hold columns
// u = 0..N/2 (W = half_plane_width(N), padding columns stay zero).
int half_plane_width(int n);
// Column pass in place on half-plane grids, storing row y at (y + N/2) mod N.  Only columns
// 0..ext_u and rows 0..ext_v, N-ext_v..N-1 may hold gridded values (the caller's bound on the
// pixel coordinates; N/2 for no bound): the columns beyond are left as they are (zero, so their
// transforms are zero) and the rows between read as zero.
// radix: the column transforms' radix, col_default_radix(n) or col_alt_radix(n) (0 = default).
int launch_fft_cols_half(float2 *grids, int n, int n_images, int ext_u, int ext_v, cudaStream_t s, int radix = 0);
int col_default_radix(int n);
int col_alt_radix(int n);  // 0 when the side has one compiled radix
// Complex-to-real row pass: half-plane rows -> image rows (fftshift of columns and
// (float)(1/wsum) applied), clearing the grid rows it read.  Images are complex with zero
// imaginary parts and must be 16-byte aligned.  Columns beyond ext_u are zero in the grid (the
// bound of launch_fft_cols_half; N/2 for none): they are neither read nor cleared.
// real: images are float[N][N] (8-byte aligned) instead of complex.
// tensor: the length-N/2 transforms as split-FP16 DFT products on the tensor cores (sides with
// c2r_tensor_supported only; others ignore it).
int launch_c2r_rows(float2 *grids, float2 *images, int n, int n_images, const unsigned int *wsum, int ext_u,
                    cudaStream_t s, bool real = false, bool tensor = false);
bool c2r_tensor_supported(int n);
int launch_shift_and_norm(float2 *images, int x_side, int y_side, int n_images,
                          const float *fnorm, int fnorm_size, cudaStream_t s);
int launch_vector_sum(const float *data, int64_t image_size, int n_images, float *sums,
                      cudaStream_t s);
int launch_image_average(const float2 *images, int64_t image_size, int n_images, float2 *out,
                         cudaStream_t s);

// Device fault word of the current device (bit 0: a bounded wait on a bulk copy gave up);
// cleared after reading when `clear` is set.  Synchronous.
int read_device_fault(unsigned int *bits, bool clear);
int launch_wait_timeout_selftest(cudaStream_t s);

// number of SMs of the current device (cached)
int sm_count();

}  // namespace bgi
