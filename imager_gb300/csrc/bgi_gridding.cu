// Nearest-neighbour uv gridding (the reference's gridding_kernel,
// src/gpu/gridding_gpu.cpp:58-124, with the CPU path's value checks,
// src/pacer_imager.cpp:297-418).
//
// Grid: x = blocks over baselines, y = images.  Each block serves one image, so the channel
// constants (wavelength, fast cell scales) are computed once per block in FP64 by one thread.
// Per thread: one baseline record (16-byte streaming loads of the needed pols), flags, optional
// fused corrections (one delay phasor and one complex rotation of the selected pol -- the
// selection is linear, so rotating after selecting equals rotating the four pols first), value
// checks, exact cell indices, and two 8-byte vector atomics (float2 atomicAdd) for the point
// and its conjugate.  Weight counts are reduced per warp before one atomic per warp.
#include "bgi_internal.h"

namespace bgi {
namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) grid_kernel(const GridParams p) {
    __shared__ ChannelConst s_cc;
    const int img = p.img_begin + blockIdx.y;
    const int ch = img % p.n_channels;
    const int t = img / p.n_channels;
    if (threadIdx.x == 0) {
        const double nu = p.freqs[ch];
        ChannelConst cc;
        cc.wavelength = kVelLight / nu;
        cc.turns_per_m = nu * (1.0 / kVelLight);
        cc.su = (float)(nu / (kVelLight * p.du));
        cc.sv = (float)(nu / (kVelLight * p.dv));
        cc.inv_wl = (float)(nu / kVelLight);
        cc.pad = 0.f;
        s_cc = cc;
    }
    __syncthreads();
    const ChannelConst cc = s_cc;

    const long long b = (long long)blockIdx.x * kThreads + threadIdx.x;
    const int set = p.n_uvw_sets > 1 ? t : 0;
    const int n = p.n_pixels;
    const long long npix = (long long)n * n;
    const int local = img - p.img_base;
    unsigned int counted = 0;

    if (b < p.n_baselines && p.flags[b] <= 0) {
        const float4 *rec = reinterpret_cast<const float4 *>(p.vis) + ((size_t)img * p.n_baselines + b) * 2;
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
        if (p.pol != BGI_POL_YY) lo = ld_stream_f4(rec);
        if (p.pol != BGI_POL_XX) hi = ld_stream_f4(rec + 1);
        float2 z = select_pol(lo, hi, p.pol);
        if (p.apply_geom || p.apply_cable) {
            double delay = 0.0;
            if (p.apply_geom) delay = (double)p.w[(size_t)set * p.n_baselines + b];
            if (p.apply_cable) delay -= p.dl[b];
            z = rotate(z, phasor(delay, cc.turns_per_m));
        }
        const bool finite_ok = !isnan(z.x) && !isnan(z.y) && fabsf(z.x) < kMaxVis && fabsf(z.y) < kMaxVis;
        int ui, vi;
        if (finite_ok &&
            uv_pixels(p.u[(size_t)set * p.n_baselines + b], p.v[(size_t)set * p.n_baselines + b], cc,
                      p.du, p.dv, p.min_uv, p.min_uv >= 0.0, &ui, &vi)) {
            const long long pos = cell_pos(ui, vi, +1, n);
            const long long pos2 = cell_pos(ui, vi, -1, n);
            float2 *grid = p.grids + (size_t)local * npix;
            float *cnt = nullptr;
            if (p.counter_mode == BGI_COUNTERS_PER_IMAGE) cnt = p.counters + (size_t)img * npix;
            else if (p.counter_mode == BGI_COUNTERS_FIRST_INTERVAL && t == 0) cnt = p.counters + (size_t)ch * npix;
            if (pos >= 0) {
                atomicAdd(grid + pos, z);
                if (cnt) atomicAdd(cnt + pos, 1.0f);
                ++counted;
            }
            if (pos2 >= 0) {
                atomicAdd(grid + pos2, make_float2(z.x, -z.y));
                if (cnt) atomicAdd(cnt + pos2, 1.0f);
                ++counted;
            }
        }
    }
    if (p.wsum) {
        unsigned int warp_total = __reduce_add_sync(0xffffffffu, counted);
        if ((threadIdx.x & 31) == 0 && warp_total) atomicAdd(p.wsum + local, warp_total);
    }
}

}  // namespace

int launch_gridding(const GridParams &p, cudaStream_t s) {
    if (p.img_count <= 0 || p.n_baselines <= 0) return BGI_OK;
    const long long bx = (p.n_baselines + kThreads - 1) / kThreads;
    for (int done = 0; done < p.img_count; done += 65535) {
        GridParams q = p;
        q.img_begin = p.img_begin + done;
        const int cnt = p.img_count - done < 65535 ? p.img_count - done : 65535;
        grid_kernel<<<dim3((unsigned)bx, (unsigned)cnt), kThreads, 0, s>>>(q);
        int st = check_launch("gridding");
        if (st) return st;
    }
    return BGI_OK;
}

}  // namespace bgi
