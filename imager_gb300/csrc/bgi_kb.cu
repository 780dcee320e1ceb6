// Kaiser-Bessel convolutional gridding (the reference's CPU-only anti-aliasing gridder,
// src/pacer_imager.cpp:378-403 and 565-750; no GPU counterpart there).
//
// Each visibility and its conjugate are spread over K x K cells around their nearest cells with
// the separable kernel k(y) k(x), taken from a table of 1023 oversampled rows (Kaiser-Bessel,
// alpha 8.6, times a sinc) by the rounded fractional pixel offset.  Taps land at
// calc_xy_grid2's cells (a tap whose coordinate leaves [-N, N) is dropped), the conjugate's at
// the mirrored coordinates with the same kernel rows (src/pacer_imager.cpp:655-750).  Counters
// and weight counts count the nearest cells, as the reference does.
//
// Work split: a warp takes 32 baselines of one image.  Each lane first derives its own
// visibility (pol selection, fused corrections, value checks, uv in wavelengths in FP64 as the
// reference, kernel rows); then the warp walks its 32 points and the lanes share each point's
// K^2 taps, so the float2 atomics of adjacent taps go to adjacent cells.
#include <cmath>
#include <vector>

#include "bgi_internal.h"

namespace bgi {
namespace {

constexpr int kOversampling = 1023;
constexpr int kWarps = 8;

struct KbPoint {
    float2 z;           // the visibility (the conjugate is placed with -im)
    int u_pix, v_pix;   // rounded pixel coordinates (FP64 recipe)
    int xk, yk;         // kernel rows
    int valid;
};

template <int POL, int FMT>
__device__ __forceinline__ KbPoint kb_point(const GridParams &p, size_t img, long long b, const ChannelConst &cc,
                                            double wavelength, unsigned *counted) {
    KbPoint q{};
    q.valid = 0;
    const long long nb = p.n_baselines;
    const int t = (int)(img / p.n_channels);
    const size_t set = p.n_uvw_sets > 1 ? (size_t)t * nb : 0;
    if (p.flags[b] > 0) return q;
    float2 a = make_float2(0.f, 0.f), bb = a;
    if (FMT == BGI_VIS_C64) load_pols<POL>(reinterpret_cast<const float2 *>(p.vis) + (img * nb + b) * 4, a, bb);
    else load_pols_planar<POL, FMT>(reinterpret_cast<const uint32_t *>(p.vis), p.vis_scales, img, nb, p.vis_blocks,
                                    b, a, bb);
    float2 z = combine_pols<POL>(a, bb);
    if (p.apply_geom || p.apply_cable) {
        float d_hi, d_lo;
        const float wv = p.apply_geom ? p.w[set + b] : 0.f;
        const float2 dl = p.apply_cable ? p.dl[b] : make_float2(0.f, 0.f);
        delay_df(wv, dl.x, dl.y, d_hi, d_lo);
        z = rotate(z, phasor_df(d_hi, d_lo, cc.f_hi, cc.f_lo));
    }
    if (isnan(z.x) || isnan(z.y) || !(fabsf(z.x) < kMaxVis) || !(fabsf(z.y) < kMaxVis)) return q;
    const float uf = p.u[set + b], vf = p.v[set + b];
    // the reference's u and v in wavelengths, distance cut, pixel coordinates (FP64)
    const double ul = __ddiv_rn((double)uf, wavelength), vl = __ddiv_rn((double)vf, wavelength);
    const double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(ul, ul), __dmul_rn(vl, vl)));
    if (!(dist > p.min_uv)) return q;
    const double ue = __ddiv_rn(ul, p.du), ve = __ddiv_rn(vl, p.dv);
    const double up = round(ue), vp = round(ve);
    if (!(fabs(up) < 1073741824.0) || !(fabs(vp) < 1073741824.0)) return q;
    int xk = (int)round(__dmul_rn(__dsub_rn(ue, up), (double)kOversampling));
    int yk = (int)round(__dmul_rn(__dsub_rn(ve, vp), (double)kOversampling));
    q.xk = (xk + (kOversampling * 3) / 2) % kOversampling;
    q.yk = (yk + (kOversampling * 3) / 2) % kOversampling;
    q.u_pix = (int)up;
    q.v_pix = (int)vp;
    q.z = z;
    q.valid = 1;
    // the nearest cells count, as the nearest-neighbour gridding
    const int n = p.n_pixels;
    const long long pos = cell_pos(q.u_pix, q.v_pix, +1, n), pos2 = cell_pos(q.u_pix, q.v_pix, -1, n);
    const long long npix = (long long)n * n;
    const int img_i = (int)img;
    float *cnt = nullptr;
    if (p.counters && (p.counter_mode == BGI_COUNTERS_PER_IMAGE || img_i < p.n_channels))
        cnt = p.counters + (size_t)(img - p.counter_base) * npix;
    if (pos >= 0) {
        if (cnt) atomicAdd(cnt + pos, 1.0f);
        ++*counted;
    }
    if (pos2 >= 0) {
        if (cnt) atomicAdd(cnt + pos2, 1.0f);
        ++*counted;
    }
    return q;
}

// calc_xy_grid2 (src/pacer_imager.cpp:753-778) for one coordinate x (already signed): -1 when
// the cell is off the grid
__device__ __forceinline__ int kb_cell(int x, int n) {
    const int h = n / 2, ui = x + h;
    const int g = ui < h ? h + ui : ui - h;
    return (g >= 0 && g < n) ? g : -1;
}

template <int POL, int FMT>
__global__ void __launch_bounds__(kWarps * 32) grid_kb_kernel(const GridParams p, const float *__restrict__ table,
                                                              int ksize) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t img = (size_t)p.img_begin + blockIdx.y;
    const long long b = ((long long)blockIdx.x * kWarps + warp) * 32 + lane;
    const int ch = (int)(img % p.n_channels);
    const ChannelConst cc = p.chan_consts ? p.chan_consts[ch] : make_channel_const(p.freqs[ch], p.du, p.dv);
    const double wavelength = cc.wavelength;
    unsigned counted = 0;
    KbPoint mine{};
    if (b < p.n_baselines) mine = kb_point<POL, FMT>(p, img, b, cc, wavelength, &counted);
    if (p.wsum) {
        const unsigned total = __reduce_add_sync(0xffffffffu, counted);
        if (lane == 0 && total) atomicAdd(p.wsum + (size_t)(img - p.img_base) * kWsumStride, total);
    }
    const int n = p.n_pixels, mid = ksize / 2, taps = ksize * ksize;
    float2 *grid = p.grids + (size_t)(img - p.img_base) * n * n;
    unsigned pending = __ballot_sync(0xffffffffu, mine.valid);
    while (pending) {
        const int src = __ffs(pending) - 1;
        pending &= pending - 1;
        const float zr = __shfl_sync(0xffffffffu, mine.z.x, src), zi = __shfl_sync(0xffffffffu, mine.z.y, src);
        const int up = __shfl_sync(0xffffffffu, mine.u_pix, src), vp = __shfl_sync(0xffffffffu, mine.v_pix, src);
        const int xk = __shfl_sync(0xffffffffu, mine.xk, src), yk = __shfl_sync(0xffffffffu, mine.yk, src);
        const float *kx = table + (size_t)xk * ksize, *ky = table + (size_t)yk * ksize;
        for (int t = lane; t < taps; t += 32) {
            const int j = t / ksize, i = t - j * ksize;
            const float kv = __ldg(ky + j) * __ldg(kx + i);
            const int x = up - mid + i, y = vp - mid + j;
            const float re = zr * kv, im = zi * kv;
            const int gx = kb_cell(x, n), gy = kb_cell(y, n);
            if (gx >= 0 && gy >= 0) atomicAdd(grid + (size_t)gy * n + gx, make_float2(re, im));
            const int cx = kb_cell(-x, n), cy = kb_cell(-y, n);
            if (cx >= 0 && cy >= 0) atomicAdd(grid + (size_t)cy * n + cx, make_float2(re, -im));
        }
    }
}

template <int POL>
void launch_pol(const dim3 &grid, const GridParams &p, const float *table, int ksize, cudaStream_t s) {
    switch (p.vis_format) {
        case BGI_VIS_S16: grid_kb_kernel<POL, BGI_VIS_S16><<<grid, kWarps * 32, 0, s>>>(p, table, ksize); break;
        case BGI_VIS_BF16: grid_kb_kernel<POL, BGI_VIS_BF16><<<grid, kWarps * 32, 0, s>>>(p, table, ksize); break;
        case BGI_VIS_FP16: grid_kb_kernel<POL, BGI_VIS_FP16><<<grid, kWarps * 32, 0, s>>>(p, table, ksize); break;
        default: grid_kb_kernel<POL, BGI_VIS_C64><<<grid, kWarps * 32, 0, s>>>(p, table, ksize);
    }
}

// unnormalised modified Bessel function I0 by its power series, to relative precision `eps`
double bessel_i0(double x, double eps) {
    double d = 0.0, term = 1.0, sum = 1.0;
    do {
        d += 2.0;
        term *= x * x / (d * d);
        sum += term;
    } while (term > sum * eps);
    return sum;
}

}  // namespace

int launch_gridding_kb_free(GridParams p, const std::vector<float> &table, int ksize, cudaStream_t s) {
    // the table in stream-ordered memory of this call: calls on other streams have their own
    float *d_table = nullptr;
    const size_t bytes = sizeof(float) * table.size();
    int st = check_cuda(cudaMallocAsync(reinterpret_cast<void **>(&d_table), bytes, s), "kb table");
    if (st) return st;
    // pageable source: the copy has taken the host data when the call returns
    st = check_cuda(cudaMemcpyAsync(d_table, table.data(), bytes, cudaMemcpyHostToDevice, s), "kb table upload");
    p.kb_table = d_table;
    p.kb_size = ksize;
    if (!st) st = launch_gridding(p, s);
    const int freed = check_cuda(cudaFreeAsync(d_table, s), "kb table free");
    return st ? st : freed;
}

void kb_tables(int ksize, bool with_sinc, std::vector<float> &out) {
    // The 1D kernel over ksize * 1023 oversampled points: Kaiser-Bessel window (alpha 8.6) times
    // sin(pi x / 1023) / (pi x), scaled by 1023 / I0(alpha), symmetric about the middle; row o of
    // the table holds every 1023rd point from offset 1022 - o (src/pacer_imager.cpp:579-651).
    const size_t osf = kOversampling, n = (size_t)ksize * osf, mid = n / 2;
    const double alpha = 8.6, ratio = 1.0 / (double)osf, norm = (double)osf / bessel_i0(alpha, 1e-8);
    std::vector<double> k1(n);
    for (size_t i = 0; i <= mid && mid + i < n; ++i) {
        const double x = (double)i, r = x / (double)mid;
        const double sinc = i == 0 ? ratio : (with_sinc ? std::sin(M_PI * ratio * x) / (M_PI * x) : ratio);
        k1[mid + i] = sinc * bessel_i0(alpha * std::sqrt(1.0 - r * r), 1e-8) * norm;
    }
    for (size_t i = 0; i < mid; ++i) k1[i] = k1[n - 1 - i];
    out.assign(osf * ksize, 0.f);
    for (size_t o = 0; o < osf; ++o)
        for (size_t x = 0; x < (size_t)ksize; ++x) out[(osf - o - 1) * ksize + x] = (float)k1[x * osf + o];
}

int launch_gridding_kb(const GridParams &p, const float *table, int ksize, cudaStream_t s) {
    if (p.img_count <= 0 || p.n_baselines <= 0) return BGI_OK;
    if (ksize < 1 || ksize > kMaxKernel || !table) return set_error(BGI_ERR_INVALID, "kb gridding: kernel size 1..%d", kMaxKernel);
    const unsigned bx = (unsigned)((p.n_baselines + kWarps * 32 - 1) / (kWarps * 32));
    for (int done = 0; done < p.img_count; done += 65535) {
        GridParams q = p;
        q.img_begin = p.img_begin + done;
        q.img_count = std::min(65535, p.img_count - done);
        const dim3 grid(bx, (unsigned)q.img_count);
        switch (p.pol) {
            case BGI_POL_XX: launch_pol<BGI_POL_XX>(grid, q, table, ksize, s); break;
            case BGI_POL_YY: launch_pol<BGI_POL_YY>(grid, q, table, ksize, s); break;
            case BGI_POL_I: launch_pol<BGI_POL_I>(grid, q, table, ksize, s); break;
            default: launch_pol<BGI_POL_V>(grid, q, table, ksize, s); break;
        }
        const int st = check_launch("kb gridding");
        if (st) return st;
    }
    return BGI_OK;
}

}  // namespace bgi
