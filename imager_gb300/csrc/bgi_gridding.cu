// Nearest-neighbour uv gridding (the reference's gridding_kernel,
// src/gpu/gridding_gpu.cpp:58-124, with the CPU path's value checks,
// src/pacer_imager.cpp:297-418).
//
// Grid: x = blocks of GRID_THREADS baselines, y = groups of CPT consecutive images.  A thread
// owns one baseline for CPT images (consecutive channels of an interval in the common case), so
// the flags and cable delay it loads -- and u/v/w and the delay when the images share a UVW set
// -- serve several visibilities, and all of its loads are issued before any is used.  The
// channel constants (wavelength, fast cell scales, nu/c as a float pair) come from a table the
// handle computes once per frequency or uv-cell change (else CPT threads compute them).
//
// Per visibility: optional fused corrections (one delay phasor in double-float arithmetic and
// one rotation of the selected pol -- selection is linear, so rotating after selecting equals
// rotating the four pols first), value checks, exact cell indices, and 8-byte vector atomics
// (float2 atomicAdd): one for the half-plane point (two on columns 0 and N/2), or the point and
// its conjugate on the full plane.  Weight counts are reduced per warp, then per block, before
// one atomic per block and image.
#include "bgi_internal.h"

namespace bgi {
namespace {

#ifndef GRID_THREADS
#define GRID_THREADS 128
#endif
constexpr int kThreads = GRID_THREADS;
constexpr int kMinBlocks = 768 / GRID_THREADS;  // resident blocks per SM the registers must allow

// Images per thread, by array size (measured, u/v/w loaded once per thread): 2 for arrays below
// 65,536 baselines (256 antennas, 640 images of 512^2: 0.657 ms per step against 0.662 with 4),
// 4 above (512 antennas, the uneven batch: 9.26 ms against 9.77 with 2) -- small arrays need the
// extra blocks, large ones the loads shared by more visibilities.
constexpr long long kCpt4Baselines = 65536;
#ifndef GRID_CPT_SMALL
#define GRID_CPT_SMALL 2
#endif
int images_per_thread(long long n_baselines) { return n_baselines >= kCpt4Baselines ? 4 : GRID_CPT_SMALL; }

// CPT: images per thread.  ONE_SET: the CPT images of every block share one UVW set (one set, or
// blocks that start at multiples of CPT with CPT dividing the channel count), so a thread loads
// u, v, w and forms the delay once for all of them.
template <int POL, bool COUNTERS, bool HALF, int FMT, bool ONE_SET, int CPT>
__global__ void __launch_bounds__(kThreads, kMinBlocks) grid_kernel(const GridParams p) {
    constexpr int kCPT = CPT;
    constexpr int NUV = ONE_SET ? 1 : kCPT;  // u, v, w registers
    __shared__ ChannelConst s_cc[kCPT];
    __shared__ unsigned int s_count[kCPT][kThreads / 32];  // per-warp weight counts
    const int img_first = p.img_begin + blockIdx.y * kCPT;
    const int img_end = p.img_begin + p.img_count;
    const int n_here = min(kCPT, img_end - img_first);
    const long long nb = p.n_baselines;
    const long long b = (long long)blockIdx.x * kThreads + threadIdx.x;
    const bool in_range = b < nb;
    const int ch_first = img_first % p.n_channels;
    const int t_first = img_first / p.n_channels;

    // ---- issue every load of this thread ----------------------------------------------------
    int flag = 1;
    float2 pa[kCPT], pb[kCPT];
    float uu[NUV], vv[NUV], ww[NUV];
    float2 dl = make_float2(0.f, 0.f);
    if (in_range) {
        flag = p.flags[b];
        if (p.apply_cable) dl = p.dl[b];
        int ch = ch_first, t = t_first;
#pragma unroll
        for (int j = 0; j < kCPT; ++j) {
            pa[j] = pb[j] = make_float2(0.f, 0.f);
            if (j < NUV) uu[j] = vv[j] = ww[j] = 0.f;
            if (j < n_here) {
                const size_t img = (size_t)img_first + j;
                const size_t off = (p.n_uvw_sets > 1 ? (size_t)t * nb : 0) + b;
                if (FMT == BGI_VIS_C64)
                    load_pols<POL>(reinterpret_cast<const float2 *>(p.vis) + (img * nb + b) * 4, pa[j], pb[j]);
                else
                    load_pols_planar<POL, FMT>(reinterpret_cast<const uint32_t *>(p.vis), p.vis_scales, img, nb,
                                               p.vis_blocks, b, pa[j], pb[j]);
                if (j < NUV) {
                    uu[j] = p.u[off];
                    vv[j] = p.v[off];
                    if (p.apply_geom) ww[j] = p.w[off];
                }
            }
            if (++ch == p.n_channels) {
                ch = 0;
                ++t;
            }
        }
    }
    // channel constants: from the caller's table when there is one (no FP64 work and no block
    // barrier here), else computed by kCPT threads while the loads are in flight
    if (!p.chan_consts) {  // uniform across the block
        if (threadIdx.x < n_here) {
            int ch = ch_first + threadIdx.x;
            while (ch >= p.n_channels) ch -= p.n_channels;
            s_cc[threadIdx.x] = make_channel_const(p.freqs[ch], p.du, p.dv);
        }
        __syncthreads();
    }

    const int n = p.n_pixels;
    const long long npix = (long long)n * n;
    const bool corr = p.apply_geom || p.apply_cable;
    const bool min_uv_active = p.min_uv >= 0.0;
    float d1_hi = 0.f, d1_lo = 0.f;  // the delay, once per thread when the images share a set
    if (ONE_SET && corr) delay_df(ww[0], dl.x, dl.y, d1_hi, d1_lo);
#pragma unroll
    for (int j = 0; j < kCPT; ++j) {
        if (j >= n_here) break;  // uniform across the block
        const int img = img_first + j;
        const int local = img - p.img_base;
        unsigned int counted = 0;
        if (in_range && flag <= 0) {
            int chj = ch_first + j;
            if (chj >= p.n_channels) chj %= p.n_channels;
            const ChannelConst *ccp = p.chan_consts ? p.chan_consts + chj : &s_cc[j];
            const float4 hot = p.chan_consts ? __ldg(reinterpret_cast<const float4 *>(ccp))
                                             : make_float4(s_cc[j].su, s_cc[j].sv, s_cc[j].f_hi, s_cc[j].f_lo);
            float2 z = combine_pols<POL>(pa[j], pb[j]);
            constexpr int J = ONE_SET ? 0 : 1;  // u, v, w index: 0 or j
            if (corr) {
                float d_hi = d1_hi, d_lo = d1_lo;
                if (!ONE_SET) delay_df(ww[J * j], dl.x, dl.y, d_hi, d_lo);
                z = rotate(z, phasor_df(d_hi, d_lo, hot.z, hot.w));
            }
            int ui, vi;
            const bool gridded = !isnan(z.x) && !isnan(z.y) && fabsf(z.x) < kMaxVis && fabsf(z.y) < kMaxVis &&
                                 uv_pixels(uu[J * j], vv[J * j], hot.x, hot.y, ccp, p.du, p.dv, p.min_uv,
                                           min_uv_active, &ui, &vi);
            if (HALF && gridded) {
                // half-plane grid: keep each of the two points whose u index is <= N/2 (the
                // caller guarantees |u|,|v| pixels < N, so both cells exist, are each other's
                // mirror, and wrap_index is i + N for negative i)
                const int w = p.half_width;
                float2 *grid = p.grids + (size_t)local * n * w;
                const int u1 = ui + (n & (ui >> 31)), v1 = vi + (n & (vi >> 31));
                const int u2 = -ui + (n & (-ui >> 31)), v2 = -vi + (n & (-vi >> 31));
                if (u1 <= n / 2) atomicAdd(grid + (size_t)v1 * w + u1, z);
                if (u2 <= n / 2) atomicAdd(grid + (size_t)v2 * w + u2, make_float2(z.x, -z.y));
                counted += 2;
            } else if (gridded) {
                const long long pos = cell_pos(ui, vi, +1, n);
                const long long pos2 = cell_pos(ui, vi, -1, n);
                float2 *grid = p.grids + (size_t)local * npix;
                float *cnt = nullptr;
                if (COUNTERS) {
                    if (p.counter_mode == BGI_COUNTERS_PER_IMAGE || img < p.n_channels)
                        cnt = p.counters + (size_t)(img - p.counter_base) * npix;
                }
                if (pos >= 0) {
                    atomicAdd(grid + pos, z);
                    if (COUNTERS && cnt) atomicAdd(cnt + pos, 1.0f);
                    ++counted;
                }
                if (pos2 >= 0) {
                    atomicAdd(grid + pos2, make_float2(z.x, -z.y));
                    if (COUNTERS && cnt) atomicAdd(cnt + pos2, 1.0f);
                    ++counted;
                }
            }
        }
        if (p.wsum) {
            const unsigned int warp_total = __reduce_add_sync(0xffffffffu, counted);
            if ((threadIdx.x & 31) == 0) s_count[j][threadIdx.x >> 5] = warp_total;
        }
    }
    // one global atomic per block and image
    if (p.wsum) {
        __syncthreads();
        if (threadIdx.x < n_here) {
            unsigned int total = 0;
#pragma unroll
            for (int w = 0; w < kThreads / 32; ++w) total += s_count[threadIdx.x][w];
            if (total) atomicAdd(p.wsum + (size_t)(img_first + threadIdx.x - p.img_base) * kWsumStride, total);
        }
    }
}

// whether every block's cpt images share one UVW set (grid_kernel's ONE_SET)
bool one_set(const GridParams &q, int cpt) {
    return q.n_uvw_sets == 1 || (q.n_channels % cpt == 0 && q.img_begin % cpt == 0);
}

// ---- the half-plane gridding of the imaging handle, lean form ---------------------------------
// The same work as grid_kernel<HALF, ONE_SET> for the handle's common case -- half-plane grids,
// the CPT images of a block sharing one UVW set, the channel-constant table, no min_uv cut, no
// counter grids -- with fewer instructions per visibility:
//  * 64-bit addresses are formed once per block (the block's first image); a thread adds 32-bit
//    offsets (j * 4 * B + b < 2^31 and (j * N + v) * W + u < 2^31, checked on the host);
//  * rounding to the nearest integer (ties to even, as rintf) and the conversion to int use the
//    exact FP32 addition of 1.5 * 2^23 (valid for |x| < 2^22; larger values take the exact FP64
//    path), so no rounding or float-to-int conversion instruction is issued;
//  * the weight count of a thread is the number of its gridded visibilities times two.
// The cell indices are the same integers (the same filter, the same exact fallback).
#ifndef GRID_LEAN
#define GRID_LEAN 1
#endif
constexpr float kRoundMagic = 12582912.0f;  // 1.5 * 2^23

// rint(x) as a float and as an int, and whether it is certainly the reference's rounding of the
// exact value (x within |x| * 2^-21 of it; see round_certain)
__device__ __forceinline__ bool round_certain_lean(float x, int *i) {
    const float t = __fadd_rn(x, kRoundMagic);
    const float r = __fsub_rn(t, kRoundMagic);  // rint(x) for |x| < 2^22
    *i = __float_as_int(t) - 0x4B400000;
    const float d = 0.5f - fabsf(x - r);
    return d > fabsf(x) * 4.76837158e-7f + 1e-30f && fabsf(x) < 4194304.0f;  // 2^-21, |x| < 2^22
}

template <int POL, int FMT, int CPT>
__global__ void __launch_bounds__(kThreads, kMinBlocks) grid_half_lean_kernel(const GridParams p) {
    __shared__ unsigned int s_count[CPT][kThreads / 32];
    constexpr int P0 = POL == BGI_POL_XX ? 0 : POL == BGI_POL_YY ? 3 : POL == BGI_POL_I ? 0 : 1;  // planes
    constexpr int P1 = POL == BGI_POL_I ? 3 : 2;
    constexpr bool TWO = POL == BGI_POL_I || POL == BGI_POL_V;
    const int img_first = p.img_begin + blockIdx.y * CPT;
    const int n_here = min(CPT, p.img_begin + p.img_count - img_first);
    const int nb = (int)p.n_baselines;
    const int b = blockIdx.x * kThreads + threadIdx.x;
    const bool in_range = b < nb;
    const int ch_first = img_first % p.n_channels;
    const int t_first = img_first / p.n_channels;
    const int n = p.n_pixels, w = p.half_width;
    // ---- loads -------------------------------------------------------------------------------
    int flag = 1;
    float2 pa[CPT], pb[CPT];
    float4 hot[CPT];
    float u = 0.f, v = 0.f, wv = 0.f;
    float2 dl = make_float2(0.f, 0.f);
    if (in_range) {
        flag = p.flags[b];
        if (p.apply_cable) dl = p.dl[b];
        const size_t set_off = p.n_uvw_sets > 1 ? (size_t)t_first * nb : 0;
        u = p.u[set_off + b];
        v = p.v[set_off + b];
        if (p.apply_geom) wv = p.w[set_off + b];
        if (FMT == BGI_VIS_C64) {
            const float2 *rec = reinterpret_cast<const float2 *>(p.vis) + (size_t)img_first * nb * 4;
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                pa[j] = pb[j] = make_float2(0.f, 0.f);
                if (j < n_here) load_pols<POL>(rec + (unsigned)(j * nb + b) * 4u, pa[j], pb[j]);
            }
        } else {
            const uint32_t *d = reinterpret_cast<const uint32_t *>(p.vis) + (size_t)img_first * 4 * nb;
            const int nblk = (int)p.vis_blocks;
            const float *sc = p.vis_scales + (size_t)img_first * 4 * nblk;
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                pa[j] = pb[j] = make_float2(0.f, 0.f);
                if (j < n_here) {
                    const unsigned o = (unsigned)(j * 4 * nb + b), os = (unsigned)(j * 4 * nblk + (b >> 7));
                    pa[j] = decode_vis<FMT>(__ldcs(d + o + P0 * nb), __ldg(sc + os + P0 * nblk));
                    if (TWO) pb[j] = decode_vis<FMT>(__ldcs(d + o + P1 * nb), __ldg(sc + os + P1 * nblk));
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
        int ch = ch_first + j;
        if (ch >= p.n_channels) ch %= p.n_channels;
        hot[j] = __ldg(reinterpret_cast<const float4 *>(p.chan_consts + ch));
    }
    const bool corr = p.apply_geom || p.apply_cable;
    float d_hi = 0.f, d_lo = 0.f;
    if (corr) delay_df(wv, dl.x, dl.y, d_hi, d_lo);
    float2 *gbase = p.grids + (size_t)(img_first - p.img_base) * n * w;
    unsigned int counted[CPT];
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
        counted[j] = 0;
        if (j >= n_here) break;  // uniform across the block
        if (in_range && flag <= 0) {
            float2 z = combine_pols<POL>(pa[j], pb[j]);
            if (corr) z = rotate(z, phasor_df(d_hi, d_lo, hot[j].z, hot[j].w));
            const float xu = u * hot[j].x, xv = v * hot[j].y;
            int ui, vi;
            const bool cu = round_certain_lean(xu, &ui), cv = round_certain_lean(xv, &vi);
            bool ok = !isnan(z.x) && !isnan(z.y) && fabsf(z.x) < kMaxVis && fabsf(z.y) < kMaxVis;
            if (ok && !(cu && cv)) {  // within the FP32 bound of a half-integer: the exact recipe
                int ch = ch_first + j;
                if (ch >= p.n_channels) ch %= p.n_channels;
                double up, vp;
                const ChannelConst *ccp = p.chan_consts + ch;
                ok = uv_pixels_exact(u, v, ccp->wavelength, p.du, p.dv, p.min_uv, &up, &vp) &&
                     fabs(up) < 1073741824.0 && fabs(vp) < 1073741824.0;
                ui = (int)up;
                vi = (int)vp;
            }
            if (ok) {
                // both mirror cells exist (every pixel coordinate is below N on this path)
                const int u1 = ui + (n & (ui >> 31)), v1 = vi + (n & (vi >> 31));
                const int u2 = -ui + (n & (-ui >> 31)), v2 = -vi + (n & (-vi >> 31));
                float2 *g = gbase + (unsigned)(j * n * w);
                if (u1 <= n / 2) atomicAdd(g + (unsigned)(v1 * w + u1), z);
                if (u2 <= n / 2) atomicAdd(g + (unsigned)(v2 * w + u2), make_float2(z.x, -z.y));
                counted[j] = 2;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < CPT; ++j) {
        if (j >= n_here) break;
        const unsigned int warp_total = __reduce_add_sync(0xffffffffu, counted[j]);
        if ((threadIdx.x & 31) == 0) s_count[j][threadIdx.x >> 5] = warp_total;
    }
    __syncthreads();
    if (threadIdx.x < n_here) {
        unsigned int total = 0;
#pragma unroll
        for (int k = 0; k < kThreads / 32; ++k) total += s_count[threadIdx.x][k];
        if (total) atomicAdd(p.wsum + (size_t)(img_first + threadIdx.x - p.img_base) * kWsumStride, total);
    }
}

// whether the lean kernel applies to a launch (its preconditions; else grid_kernel runs)
bool lean_applies(const GridParams &q, int cpt) {
    if (!GRID_LEAN || q.half_width <= 0 || !q.chan_consts || q.min_uv >= 0.0 || q.counter_mode >= 0 || !q.wsum ||
        q.kb_size > 0)
        return false;
    const long long nb = q.n_baselines;
    const long long per_image_grid = (long long)q.n_pixels * q.half_width;
    const bool one = q.n_uvw_sets == 1 || (q.n_channels % cpt == 0 && q.img_begin % cpt == 0);
    return one && nb < (1LL << 27) && (long long)cpt * 4 * nb < (1LL << 31) && cpt * per_image_grid < (1LL << 31);
}

// ---- the half-plane gridding with several images per thread, raw loads first ----------------
// grid_half_lean_kernel holds its images' decoded values and channel constants in registers, which
// limits it to a few images per thread.  This form keeps only the raw stored words of its IMG
// images (one or two 4-byte words and block scales per image for the 16-bit formats), issues every
// one of those loads before the first use, and per image decodes, reads the channel constants
// (cached) and grids: the per-baseline work -- flags, cable delay, u/v/w and the delay phase --
// is done once for all IMG images, and all of a thread's global loads are in flight together.
// The images of a block may span two intervals with their own UVW sets (the block's images are
// consecutive); u/v/w and the delay are then reloaded where the set changes.
// Warp aggregation (AGG): the points of a warp that fall on the same cell are summed at one lane
// before a single atomic per distinct cell.  It pays where many points share few cells (an array
// whose short baselines crowd the centre of a small grid: the uneven batch's 256^2 band puts its
// 130,816 points of an image on about 300 cells, 9.5 % of a warp's points on distinct cells) and
// costs where they are spread (99.8 % distinct at the 512^2 workload); bgi_autotune times it.
__device__ __forceinline__ void warp_aggregated_add(float2 *base, int key, float2 v) {
    const int lane = (int)(threadIdx.x & 31);
    const unsigned grp = __match_any_sync(0xffffffffu, key >= 0 ? key : -1 - lane);  // idle lanes alone
    if (__any_sync(0xffffffffu, __popc(grp) > 1)) {
        float2 sum = make_float2(0.f, 0.f);
        for (int src = 0; src < 32; ++src) {
            const float vx = __shfl_sync(0xffffffffu, v.x, src), vy = __shfl_sync(0xffffffffu, v.y, src);
            if ((grp >> src) & 1u) {
                sum.x += vx;
                sum.y += vy;
            }
        }
        v = sum;
    }
    if (key >= 0 && lane == __ffs(grp) - 1) atomicAdd(base + (unsigned)key, v);
}

template <int POL, int FMT, int IMG, bool AGG = false>
__global__ void __launch_bounds__(kThreads, kMinBlocks) grid_half_loop_kernel(const GridParams p) {
    __shared__ unsigned int s_count[IMG][kThreads / 32];
    constexpr int P0 = POL == BGI_POL_XX ? 0 : POL == BGI_POL_YY ? 3 : POL == BGI_POL_I ? 0 : 1;  // planes
    constexpr int P1 = POL == BGI_POL_I ? 3 : 2;
    constexpr bool TWO = POL == BGI_POL_I || POL == BGI_POL_V;
    constexpr bool C64 = FMT == BGI_VIS_C64;
    const int img_first = p.img_begin + blockIdx.y * IMG;
    const int n_here = min(IMG, p.img_begin + p.img_count - img_first);
    const int nb = (int)p.n_baselines;
    const int b = blockIdx.x * kThreads + threadIdx.x;
    const bool in_range = b < nb;
    const int n = p.n_pixels, w = p.half_width;
    const int nblk = (int)p.vis_blocks;
    // ---- every global load of the thread's images first ----------------------------------------
    int flag = 1;
    float2 dl = make_float2(0.f, 0.f);
    float2 ra[IMG], rb[IMG];  // complex64: the pol values; 16-bit: (word bits, scale) pairs
    if (in_range) {
        flag = p.flags[b];
        if (p.apply_cable) dl = p.dl[b];
    }
#pragma unroll
    for (int j = 0; j < IMG; ++j) {
        ra[j] = rb[j] = make_float2(0.f, 0.f);
        if (in_range && j < n_here) {
            const size_t img = (size_t)img_first + j;
            if (C64) {
                load_pols<POL>(reinterpret_cast<const float2 *>(p.vis) + (img * nb + b) * 4, ra[j], rb[j]);
            } else {
                const uint32_t *d = reinterpret_cast<const uint32_t *>(p.vis) + img * 4 * nb + b;
                const float *sc = p.vis_scales + img * 4 * nblk + (b >> 7);
                ra[j] = make_float2(__uint_as_float(__ldcs(d + P0 * nb)), __ldg(sc + P0 * nblk));
                if (TWO) rb[j] = make_float2(__uint_as_float(__ldcs(d + P1 * nb)), __ldg(sc + P1 * nblk));
            }
        }
    }
    const bool corr = p.apply_geom || p.apply_cable;
    float u = 0.f, v = 0.f, wv = 0.f, d_hi = 0.f, d_lo = 0.f;
    int cur_set = -1;
    int ch = img_first % p.n_channels;
    float2 *gbase = p.grids + (size_t)(img_first - p.img_base) * n * w;
#pragma unroll
    for (int j = 0; j < IMG; ++j) {
        if (j >= n_here) break;  // uniform across the block
        const int set = p.n_uvw_sets > 1 ? (img_first + j) / p.n_channels : 0;
        if (set != cur_set) {  // uniform across the block
            cur_set = set;
            if (in_range) {
                const size_t off = (size_t)set * nb + b;
                u = p.u[off];
                v = p.v[off];
                if (p.apply_geom) wv = p.w[off];
            }
            if (corr) delay_df(wv, dl.x, dl.y, d_hi, d_lo);
        }
        const float4 hot = __ldg(reinterpret_cast<const float4 *>(p.chan_consts + ch));
        unsigned int counted = 0;
        int key1 = -1, key2 = -1;  // AGG: the point's cell offsets from gbase (-1: none)
        float2 z1 = make_float2(0.f, 0.f), z2 = z1;
        if (in_range && flag <= 0) {
            float2 a = ra[j], bb = rb[j];
            if (!C64) {
                a = decode_vis<FMT>(__float_as_uint(ra[j].x), ra[j].y);
                if (TWO) bb = decode_vis<FMT>(__float_as_uint(rb[j].x), rb[j].y);
            }
            float2 z = combine_pols<POL>(a, bb);
            if (corr) z = rotate(z, phasor_df(d_hi, d_lo, hot.z, hot.w));
            int ui, vi;
            const bool cu = round_certain_lean(u * hot.x, &ui), cv = round_certain_lean(v * hot.y, &vi);
            bool ok = !isnan(z.x) && !isnan(z.y) && fabsf(z.x) < kMaxVis && fabsf(z.y) < kMaxVis;
            if (ok && !(cu && cv)) {  // within the FP32 bound of a half-integer: the exact recipe
                double up, vp;
                const ChannelConst *ccp = p.chan_consts + ch;
                ok = uv_pixels_exact(u, v, ccp->wavelength, p.du, p.dv, p.min_uv, &up, &vp) &&
                     fabs(up) < 1073741824.0 && fabs(vp) < 1073741824.0;
                ui = (int)up;
                vi = (int)vp;
            }
            if (ok) {
                const int u1 = ui + (n & (ui >> 31)), v1 = vi + (n & (vi >> 31));
                const int u2 = -ui + (n & (-ui >> 31)), v2 = -vi + (n & (-vi >> 31));
                if constexpr (AGG) {
                    if (u1 <= n / 2) {
                        key1 = j * n * w + v1 * w + u1;
                        z1 = z;
                    }
                    if (u2 <= n / 2) {
                        key2 = j * n * w + v2 * w + u2;
                        z2 = make_float2(z.x, -z.y);
                    }
                } else {
                    float2 *g = gbase + (unsigned)(j * n * w);
                    if (u1 <= n / 2) atomicAdd(g + (unsigned)(v1 * w + u1), z);
                    if (u2 <= n / 2) atomicAdd(g + (unsigned)(v2 * w + u2), make_float2(z.x, -z.y));
                }
                counted = 2;
            }
        }
        if constexpr (AGG) {  // every lane of the warp takes part
            warp_aggregated_add(gbase, key1, z1);
            warp_aggregated_add(gbase, key2, z2);
        }
        const unsigned int warp_total = __reduce_add_sync(0xffffffffu, counted);
        if ((threadIdx.x & 31) == 0) s_count[j][threadIdx.x >> 5] = warp_total;
        if (++ch == p.n_channels) ch = 0;
    }
    __syncthreads();
    if (threadIdx.x < n_here) {
        unsigned int total = 0;
#pragma unroll
        for (int k = 0; k < kThreads / 32; ++k) total += s_count[threadIdx.x][k];
        if (total) atomicAdd(p.wsum + (size_t)(img_first + threadIdx.x - p.img_base) * kWsumStride, total);
    }
}

// whether the looping kernel applies (the lean kernel's preconditions; the block's images may
// span UVW sets)
bool loop_applies(const GridParams &q, int img) {
    if (q.half_width <= 0 || !q.chan_consts || q.min_uv >= 0.0 || q.counter_mode >= 0 || !q.wsum || q.kb_size > 0)
        return false;
    const long long per_image_grid = (long long)q.n_pixels * q.half_width;
    return q.n_baselines < (1LL << 27) && img * per_image_grid < (1LL << 31);
}

template <int POL, int FMT, int CPT>
void launch_fmt(const dim3 &grid, const GridParams &q, cudaStream_t s) {
    const bool one = one_set(q, CPT);
    if constexpr (CPT >= 4) {
        if (loop_applies(q, CPT)) {
            if (q.aggregate) grid_half_loop_kernel<POL, FMT, CPT, true><<<grid, kThreads, 0, s>>>(q);
            else grid_half_loop_kernel<POL, FMT, CPT><<<grid, kThreads, 0, s>>>(q);
            return;
        }
    }
    if (lean_applies(q, CPT)) {
        grid_half_lean_kernel<POL, FMT, CPT><<<grid, kThreads, 0, s>>>(q);
        return;
    }
    if (q.half_width > 0) {
        if (one) grid_kernel<POL, false, true, FMT, true, CPT><<<grid, kThreads, 0, s>>>(q);
        else grid_kernel<POL, false, true, FMT, false, CPT><<<grid, kThreads, 0, s>>>(q);
    } else {
        if (one) grid_kernel<POL, false, false, FMT, true, CPT><<<grid, kThreads, 0, s>>>(q);
        else grid_kernel<POL, false, false, FMT, false, CPT><<<grid, kThreads, 0, s>>>(q);
    }
}

template <int POL, int CPT>
void launch_pol(const dim3 &grid, const GridParams &q, cudaStream_t s) {
    if (q.counter_mode >= 0) {  // counter grids: full plane
        switch (q.vis_format) {
            case BGI_VIS_S16: grid_kernel<POL, true, false, BGI_VIS_S16, false, CPT><<<grid, kThreads, 0, s>>>(q); break;
            case BGI_VIS_BF16: grid_kernel<POL, true, false, BGI_VIS_BF16, false, CPT><<<grid, kThreads, 0, s>>>(q); break;
            case BGI_VIS_FP16: grid_kernel<POL, true, false, BGI_VIS_FP16, false, CPT><<<grid, kThreads, 0, s>>>(q); break;
            default: grid_kernel<POL, true, false, BGI_VIS_C64, false, CPT><<<grid, kThreads, 0, s>>>(q);
        }
        return;
    }
    switch (q.vis_format) {
        case BGI_VIS_S16: launch_fmt<POL, BGI_VIS_S16, CPT>(grid, q, s); break;
        case BGI_VIS_BF16: launch_fmt<POL, BGI_VIS_BF16, CPT>(grid, q, s); break;
        case BGI_VIS_FP16: launch_fmt<POL, BGI_VIS_FP16, CPT>(grid, q, s); break;
        default: launch_fmt<POL, BGI_VIS_C64, CPT>(grid, q, s);
    }
}

template <int POL>
void launch_loop8_pol(const dim3 &grid, const GridParams &q, cudaStream_t s) {
    switch (q.vis_format) {
        case BGI_VIS_S16:
            if (q.aggregate) grid_half_loop_kernel<POL, BGI_VIS_S16, 8, true><<<grid, kThreads, 0, s>>>(q);
            else grid_half_loop_kernel<POL, BGI_VIS_S16, 8><<<grid, kThreads, 0, s>>>(q);
            break;
        case BGI_VIS_BF16:
            if (q.aggregate) grid_half_loop_kernel<POL, BGI_VIS_BF16, 8, true><<<grid, kThreads, 0, s>>>(q);
            else grid_half_loop_kernel<POL, BGI_VIS_BF16, 8><<<grid, kThreads, 0, s>>>(q);
            break;
        case BGI_VIS_FP16:
            if (q.aggregate) grid_half_loop_kernel<POL, BGI_VIS_FP16, 8, true><<<grid, kThreads, 0, s>>>(q);
            else grid_half_loop_kernel<POL, BGI_VIS_FP16, 8><<<grid, kThreads, 0, s>>>(q);
            break;
        default:
            if (q.aggregate) grid_half_loop_kernel<POL, BGI_VIS_C64, 8, true><<<grid, kThreads, 0, s>>>(q);
            else grid_half_loop_kernel<POL, BGI_VIS_C64, 8><<<grid, kThreads, 0, s>>>(q);
    }
}

void launch_loop8(const dim3 &grid, const GridParams &q, cudaStream_t s) {
    switch (q.pol) {
        case BGI_POL_XX: launch_loop8_pol<BGI_POL_XX>(grid, q, s); break;
        case BGI_POL_YY: launch_loop8_pol<BGI_POL_YY>(grid, q, s); break;
        case BGI_POL_I: launch_loop8_pol<BGI_POL_I>(grid, q, s); break;
        default: launch_loop8_pol<BGI_POL_V>(grid, q, s); break;
    }
}

template <int CPT>
void launch_cpt(const dim3 &grid, const GridParams &q, cudaStream_t s) {
    switch (q.pol) {
        case BGI_POL_XX: launch_pol<BGI_POL_XX, CPT>(grid, q, s); break;
        case BGI_POL_YY: launch_pol<BGI_POL_YY, CPT>(grid, q, s); break;
        case BGI_POL_I: launch_pol<BGI_POL_I, CPT>(grid, q, s); break;
        default: launch_pol<BGI_POL_V, CPT>(grid, q, s); break;
    }
}

__global__ void uniform_weighting_kernel(float2 *grids, float *counters, long long n_cells, bool clear) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n_cells;
         i += (long long)gridDim.x * blockDim.x) {
        const float c = counters[i];
        const float2 g = grids[i];
        grids[i] = make_float2(__fdiv_rn(g.x, c), __fdiv_rn(g.y, c));
        if (clear) counters[i] = 0.f;
    }
}

__global__ void channel_consts_kernel(const double *freqs, int n_channels, double du, double dv, ChannelConst *table) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n_channels) table[c] = make_channel_const(freqs[c], du, dv);
}

}  // namespace

int launch_channel_consts(const double *freqs, int n_channels, double du, double dv, ChannelConst *table,
                          cudaStream_t s) {
    if (n_channels <= 0) return BGI_OK;
    channel_consts_kernel<<<(n_channels + 127) / 128, 128, 0, s>>>(freqs, n_channels, du, dv, table);
    return check_launch("channel constants");
}

int launch_uniform_weighting(float2 *grids, float *counters, long long n_cells, bool clear_counters, cudaStream_t s) {
    if (n_cells <= 0) return BGI_OK;
    const long long blocks = std::min<long long>((n_cells + 255) / 256, (long long)sm_count() * 16);
    uniform_weighting_kernel<<<(unsigned)blocks, 256, 0, s>>>(grids, counters, n_cells, clear_counters);
    return check_launch("uniform weighting");
}

int launch_gridding(const GridParams &p, cudaStream_t s) {
    if (p.img_count <= 0 || p.n_baselines <= 0) return BGI_OK;
    if (p.kb_size > 0) {
        if (p.half_width > 0) return set_error(BGI_ERR_INVALID, "kb gridding: full-plane grids only");
        return launch_gridding_kb(p, p.kb_table, p.kb_size, s);
    }
    const long long bx = (p.n_baselines + kThreads - 1) / kThreads;
    const int max_groups = 65535;
    // by default 4 on the half-plane path (the looping kernel: 0.518-0.521 against 0.530 ms per
    // step with 2 at 256 antennas, and the uneven 512-antenna batch 7.41 against 7.87 ms), else by
    // array size
    int cpt = p.cpt == 2 || p.cpt == 4 || p.cpt == 8 ? p.cpt
              : loop_applies(p, 4)                  ? 4
                                                    : images_per_thread(p.n_baselines);
    if (cpt == 8 && !loop_applies(p, 8)) cpt = 4;  // eight images per thread: the looping kernel only
    for (int done = 0; done < p.img_count; done += max_groups * cpt) {
        GridParams q = p;
        q.img_begin = p.img_begin + done;
        q.img_count = std::min(p.img_count - done, max_groups * cpt);
        const dim3 grid((unsigned)bx, (unsigned)((q.img_count + cpt - 1) / cpt));
        if (cpt == 8) launch_loop8(grid, q, s);
        else if (cpt == 4) launch_cpt<4>(grid, q, s);
        else launch_cpt<2>(grid, q, s);
        int st = check_launch("gridding");
        if (st) return st;
    }
    return BGI_OK;
}

}  // namespace bgi
