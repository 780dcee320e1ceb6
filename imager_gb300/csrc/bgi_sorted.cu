// Deterministic gridding by sort and segmented reduction.
//
// The atomic gridder adds the points of a cell in whatever order the GPU schedules them, so its
// float sums differ in the last bits from run to run.  This variant sums every cell in a fixed
// order -- the reference CPU loop's order, baseline by baseline, each visibility before its
// conjugate (src/pacer_imager.cpp:297-408) -- so its grids are reproducible and bit-identical
// to the CPU gridding given the same visibilities.  Per chunk of images:
//
//   keys:    one thread per (image, baseline): the two points' cells (or "none") and values,
//            and a per-cell point count (integer atomics: order-free);
//   scan:    exclusive prefix sum of the counts of each image, giving each cell's segment;
//   place:   each point writes its index into its cell's segment (slot order arbitrary);
//   reduce:  one thread per cell orders its segment by point index and adds the values to the
//            cell in that order, starting from the grid's current value (as the CPU's +=).
//
// Workspace (caller provided, bgi_gridding_sorted_workspace gives the size): per image
// 2B point keys, values and segment entries, and three N*N integer arrays.
#include <algorithm>

#include "bgi_internal.h"

namespace bgi {
namespace {

constexpr unsigned kNoCell = 0xffffffffu;
constexpr int kThreads = 256;

struct SortedWs {
    unsigned *key;      // [chunk][2B] cell of each point, kNoCell when not gridded
    float2 *val;        // [chunk][2B]
    unsigned *seg;      // [chunk][2B] point indices grouped by cell
    unsigned *cnt;      // [chunk][N*N] points per cell
    unsigned *start;    // [chunk][N*N] first segment slot of each cell within its tile
    unsigned *tile_off; // [chunk][tiles(N)] first segment slot of each tile of kScanTile cells
    unsigned *cursor;   // [chunk][N*N] slots used so far
    unsigned *n_long;   // [chunk] cells whose segment is longer than kShortSeg, up to kLongSort
    unsigned *n_huge;   // [chunk] cells whose segment is longer than kLongSort
    unsigned *longs;    // [chunk][long_cap(B)] the first from the front, the second from the back
};

// Segments up to this length are ordered by the thread of their cell; longer ones (many short
// baselines in one cell) are handed to one block each.
constexpr unsigned kShortSeg = 32;
constexpr int kLongThreads = 512;
constexpr int kLongBlocks = 32;  // blocks per image sharing its long cells, at least (four per SM
                                 // across the chunk's images when that is more)
constexpr int kHugeBlocks = 8;   // blocks per image sharing its huge cells
constexpr int kTile = 1024;
// Long segments up to kLongSort points are ordered by a bitonic sort in shared memory (32 KB,
// several blocks per SM), huge ones up to kHugeSort in a block of 128 KB of shared memory, and
// longer ones still (over 32,768 points in one cell) by counting ranks against tiles.
constexpr unsigned kLongSort = 8192;
constexpr unsigned kHugeSort = 32768;
// The per-image prefix sum runs over tiles of 4096 cells (256 threads x 16 cells), then over
// the tiles' totals.
constexpr int kScanTile = 4096;
constexpr int kScanPer = kScanTile / kThreads;

// Cells of one image's grid: N x N, or N x W on the half plane (half_width W > 0).
__host__ __device__ inline size_t grid_cells(const GridParams &p) {
    return (size_t)p.n_pixels * (p.half_width > 0 ? (size_t)p.half_width : (size_t)p.n_pixels);
}
__host__ __device__ inline size_t scan_tiles(size_t cells) { return (cells + kScanTile - 1) / kScanTile; }
__device__ __forceinline__ unsigned seg_start(const SortedWs &w, int local, size_t cells, size_t c) {
    return w.tile_off[(size_t)local * scan_tiles(cells) + c / kScanTile] + w.start[(size_t)local * cells + c];
}

__host__ __device__ inline size_t long_cap(long long nb) { return (size_t)(2 * nb) / (kShortSeg + 1) + 1; }

// Workspace per image for grids of `cells` cells (the full plane's N * N bounds either plane).
size_t per_image_bytes(long long nb, size_t cells) {
    const size_t pts = 2 * (size_t)nb;
    return pts * (sizeof(unsigned) + sizeof(float2) + sizeof(unsigned)) + 3 * cells * sizeof(unsigned) +
           (2 + long_cap(nb) + scan_tiles(cells)) * sizeof(unsigned) + 10 * 256;  // 10 arrays, each start rounded up to 256 B
}

SortedWs carve(void *ws, int chunk, long long nb, size_t image_cells) {
    const size_t pts = 2 * (size_t)nb * chunk, cells = image_cells * chunk;
    char *p = static_cast<char *>(ws);
    auto take = [&](size_t bytes) {
        char *q = p;
        p += (bytes + 255) & ~(size_t)255;
        return q;
    };
    SortedWs w;
    w.val = reinterpret_cast<float2 *>(take(pts * sizeof(float2)));
    w.key = reinterpret_cast<unsigned *>(take(pts * sizeof(unsigned)));
    w.seg = reinterpret_cast<unsigned *>(take(pts * sizeof(unsigned)));
    w.cnt = reinterpret_cast<unsigned *>(take(cells * sizeof(unsigned)));
    w.start = reinterpret_cast<unsigned *>(take(cells * sizeof(unsigned)));
    w.cursor = reinterpret_cast<unsigned *>(take(cells * sizeof(unsigned)));
    w.tile_off = reinterpret_cast<unsigned *>(take(chunk * scan_tiles(image_cells) * sizeof(unsigned)));
    w.n_long = reinterpret_cast<unsigned *>(take(chunk * sizeof(unsigned)));
    w.n_huge = reinterpret_cast<unsigned *>(take(chunk * sizeof(unsigned)));
    w.longs = reinterpret_cast<unsigned *>(take(chunk * long_cap(nb) * sizeof(unsigned)));
    return w;
}

// the selected pol of one visibility, in any storage format
template <int POL>
__device__ __forceinline__ float2 load_selected(const GridParams &p, size_t img, long long nb, long long b) {
    float2 a = make_float2(0.f, 0.f), bb = a;
    const uint32_t *planes = reinterpret_cast<const uint32_t *>(p.vis);
    switch (p.vis_format) {
        case BGI_VIS_S16: load_pols_planar<POL, BGI_VIS_S16>(planes, p.vis_scales, img, nb, p.vis_blocks, b, a, bb); break;
        case BGI_VIS_BF16: load_pols_planar<POL, BGI_VIS_BF16>(planes, p.vis_scales, img, nb, p.vis_blocks, b, a, bb); break;
        case BGI_VIS_FP16: load_pols_planar<POL, BGI_VIS_FP16>(planes, p.vis_scales, img, nb, p.vis_blocks, b, a, bb); break;
        default: load_pols<POL>(reinterpret_cast<const float2 *>(p.vis) + (img * nb + b) * 4, a, bb);
    }
    return combine_pols<POL>(a, bb);
}

// keys: grid x = baselines, y = images of the chunk.  On the half plane (half_width > 0; every
// point's mirror cell exists, |u|, |v| pixels < N) a visibility's two points keep the cells whose
// u index is at most N/2, numbered v * W + u: the same points, in the same order, as those
// cells of the full plane, so their ordered sums are the same bits.
__global__ void __launch_bounds__(kThreads) keys_kernel(const GridParams p, int chunk_first, SortedWs w) {
    __shared__ ChannelConst s_cc;
    const int img = chunk_first + blockIdx.y;
    const int local = blockIdx.y;
    const int ch = img % p.n_channels, t = img / p.n_channels;
    if (threadIdx.x == 0) s_cc = make_channel_const(p.freqs[ch], p.du, p.dv);
    __syncthreads();
    const long long nb = p.n_baselines;
    const long long b = (long long)blockIdx.x * kThreads + threadIdx.x;
    const bool in_range = b < nb;
    const size_t set = p.n_uvw_sets > 1 ? (size_t)t * nb : 0;
    const int n = p.n_pixels;
    unsigned k1 = kNoCell, k2 = kNoCell, counted = 0;
    float2 z = make_float2(0.f, 0.f);
    if (in_range && p.flags[b] <= 0) {
        switch (p.pol) {
            case BGI_POL_XX: z = load_selected<BGI_POL_XX>(p, img, nb, b); break;
            case BGI_POL_YY: z = load_selected<BGI_POL_YY>(p, img, nb, b); break;
            case BGI_POL_I: z = load_selected<BGI_POL_I>(p, img, nb, b); break;
            default: z = load_selected<BGI_POL_V>(p, img, nb, b); break;
        }
        if (p.apply_geom || p.apply_cable) {
            float d_hi, d_lo;
            const float wv = p.apply_geom ? p.w[set + b] : 0.f;
            const float2 dl = p.apply_cable ? p.dl[b] : make_float2(0.f, 0.f);
            delay_df(wv, dl.x, dl.y, d_hi, d_lo);
            z = rotate(z, phasor_df(d_hi, d_lo, s_cc.f_hi, s_cc.f_lo));
        }
        int ui, vi;
        if (!isnan(z.x) && !isnan(z.y) && fabsf(z.x) < kMaxVis && fabsf(z.y) < kMaxVis &&
            uv_pixels(p.u[set + b], p.v[set + b], s_cc.su, s_cc.sv, &s_cc, p.du, p.dv, p.min_uv, p.min_uv >= 0.0, &ui,
                      &vi)) {
            long long pos, pos2;
            if (p.half_width > 0) {
                const int u1 = ui + (n & (ui >> 31)), v1 = vi + (n & (vi >> 31));
                const int u2 = -ui + (n & (-ui >> 31)), v2 = -vi + (n & (-vi >> 31));
                pos = u1 <= n / 2 ? (long long)v1 * p.half_width + u1 : -1;
                pos2 = u2 <= n / 2 ? (long long)v2 * p.half_width + u2 : -1;
                counted = 2;  // both points of the full plane
            } else {
                pos = cell_pos(ui, vi, +1, n);
                pos2 = cell_pos(ui, vi, -1, n);
                counted = (pos >= 0) + (pos2 >= 0);
            }
            unsigned *cnt = w.cnt + (size_t)local * grid_cells(p);
            if (pos >= 0) {
                k1 = (unsigned)pos;
                atomicAdd(cnt + pos, 1u);
            }
            if (pos2 >= 0) {
                k2 = (unsigned)pos2;
                atomicAdd(cnt + pos2, 1u);
            }
        }
    }
    if (p.wsum) {
        const unsigned total = __reduce_add_sync(0xffffffffu, counted);
        if ((threadIdx.x & 31) == 0 && total)
            atomicAdd(p.wsum + (size_t)(img - p.img_base) * kWsumStride, total);
    }
    if (!in_range) return;
    const size_t q = (size_t)local * 2 * nb + 2 * b;
    w.key[q] = k1;
    w.key[q + 1] = k2;
    w.val[q] = z;
    w.val[q + 1] = make_float2(z.x, -z.y);
}

// scan, first level: grid (tiles, images); each thread owns 16 consecutive cells (read and
// written as 16-byte vectors when the image's cell count is a multiple of 4).  Writes each
// cell's exclusive prefix within its tile and the tile's total.
template <bool VEC>
__global__ void __launch_bounds__(kThreads) scan_tiles_kernel(SortedWs w, size_t cells) {
    __shared__ unsigned s_warp[kThreads / 32];
    const int local = blockIdx.y;
    const size_t c0 = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPer;
    const unsigned *cnt = w.cnt + (size_t)local * cells;
    unsigned *start = w.start + (size_t)local * cells;
    unsigned v[kScanPer];
    if (VEC) {
#pragma unroll
        for (int j = 0; j < kScanPer; j += 4) {
            uint4 q = make_uint4(0u, 0u, 0u, 0u);
            if (c0 + j < cells) q = *reinterpret_cast<const uint4 *>(cnt + c0 + j);
            v[j] = q.x;
            v[j + 1] = q.y;
            v[j + 2] = q.z;
            v[j + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < kScanPer; ++j) v[j] = c0 + j < cells ? cnt[c0 + j] : 0u;
    }
    unsigned sum = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) sum += v[j];
    // block-wide exclusive scan of the thread sums
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned incl = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        unsigned x = lane < kThreads / 32 ? s_warp[lane] : 0u;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += t;
        }
        if (lane < kThreads / 32) s_warp[lane] = x;  // inclusive warp totals
    }
    __syncthreads();
    unsigned run = incl - sum + (wid > 0 ? s_warp[wid - 1] : 0u);
    unsigned out[kScanPer];
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        out[j] = run;
        run += v[j];
    }
    if (VEC) {
#pragma unroll
        for (int j = 0; j < kScanPer; j += 4)
            if (c0 + j < cells) *reinterpret_cast<uint4 *>(start + c0 + j) = make_uint4(out[j], out[j + 1], out[j + 2], out[j + 3]);
    } else {
#pragma unroll
        for (int j = 0; j < kScanPer; ++j)
            if (c0 + j < cells) start[c0 + j] = out[j];
    }
    if (threadIdx.x == kThreads - 1) w.tile_off[(size_t)local * scan_tiles(cells) + blockIdx.x] = run;
}

// scan, second level: one block per image turns its tile totals into exclusive offsets (each
// thread owns a contiguous run of tiles).
__global__ void __launch_bounds__(1024) scan_offsets_kernel(SortedWs w, size_t cells) {
    __shared__ unsigned s_part[1024];
    const size_t tiles = scan_tiles(cells);
    unsigned *off = w.tile_off + (size_t)blockIdx.x * tiles;
    const size_t per = (tiles + blockDim.x - 1) / blockDim.x;
    const size_t t0 = threadIdx.x * per, t1 = t0 + per < tiles ? t0 + per : tiles;
    unsigned sum = 0;
    for (size_t t = t0; t < t1; ++t) sum += off[t];
    s_part[threadIdx.x] = sum;
    __syncthreads();
    for (int d = 1; d < (int)blockDim.x; d <<= 1) {  // inclusive Hillis-Steele scan
        const unsigned x = threadIdx.x >= (unsigned)d ? s_part[threadIdx.x - d] : 0u;
        __syncthreads();
        s_part[threadIdx.x] += x;
        __syncthreads();
    }
    unsigned run = s_part[threadIdx.x] - sum;
    for (size_t t = t0; t < t1; ++t) {
        const unsigned x = off[t];
        off[t] = run;
        run += x;
    }
}

// place: one thread per point
__global__ void __launch_bounds__(kThreads) place_kernel(SortedWs w, long long n_points, size_t cells) {
    const long long q = (long long)blockIdx.x * kThreads + threadIdx.x;
    const int local = blockIdx.y;
    if (q >= n_points) return;
    const size_t base = (size_t)local * n_points;
    const unsigned key = w.key[base + q];
    if (key == kNoCell) return;
    const size_t cbase = (size_t)local * cells;
    const unsigned slot = atomicAdd(w.cursor + cbase + key, 1u);
    w.seg[base + seg_start(w, local, cells, key) + slot] = (unsigned)q;
}

// Orders a segment of at most K point indices in registers (adjacent compare-exchanges of an
// unrolled insertion sort; the padding sorts last), gathers the values, and adds them to acc in
// index order.
template <int K>
__device__ __forceinline__ void sum_segment_in_registers(const unsigned *seg, unsigned len, const float2 *val,
                                                         float2 &acc) {
    unsigned idx[K];
#pragma unroll
    for (int j = 0; j < K; ++j) idx[j] = (unsigned)j < len ? seg[j] : 0xffffffffu;
#pragma unroll
    for (int i = 1; i < K; ++i) {
#pragma unroll
        for (int j = i; j > 0; --j) {
            const unsigned lo = min(idx[j - 1], idx[j]), hi = max(idx[j - 1], idx[j]);
            idx[j - 1] = lo;
            idx[j] = hi;
        }
    }
    float2 v[K];
#pragma unroll
    for (int j = 0; j < K; ++j) v[j] = (unsigned)j < len ? val[idx[j]] : make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < K; ++j) {
        if ((unsigned)j < len) {
            acc.x = __fadd_rn(acc.x, v[j].x);
            acc.y = __fadd_rn(acc.y, v[j].y);
        }
    }
}

// reduce: one thread per cell; orders the cell's point indices (in registers up to 16 points,
// by insertion in the segment up to kShortSeg) and adds the values in that order to the cell's
// current value.
__global__ void __launch_bounds__(kThreads) reduce_kernel(const GridParams p, int chunk_first, SortedWs w,
                                                          long long n_points) {
    const long long cells = (long long)grid_cells(p);
    const long long c = (long long)blockIdx.x * kThreads + threadIdx.x;
    const int local = blockIdx.y;
    if (c >= cells) return;
    const size_t cbase = (size_t)local * cells;
    const unsigned len = w.cnt[cbase + c];
    if (len == 0) return;
    if (len > kShortSeg) {  // every listed cell holds more than kShortSeg points: both lists fit
        const size_t cap = long_cap(n_points / 2);
        if (len <= kLongSort)
            w.longs[(size_t)local * cap + atomicAdd(w.n_long + local, 1u)] = (unsigned)c;
        else
            w.longs[(size_t)local * cap + cap - 1 - atomicAdd(w.n_huge + local, 1u)] = (unsigned)c;
        return;
    }
    const int img = chunk_first + local;
    float2 *cell = p.grids + (size_t)(img - p.img_base) * cells + c;
    float2 acc = p.grids_zero ? make_float2(0.f, 0.f) : *cell;
    unsigned *seg = w.seg + (size_t)local * n_points + seg_start(w, local, (size_t)cells, c);
    const float2 *val = w.val + (size_t)local * n_points;
    if (len == 1) {
        const float2 v = val[seg[0]];
        acc.x = __fadd_rn(acc.x, v.x);
        acc.y = __fadd_rn(acc.y, v.y);
    } else if (len <= 4) {
        sum_segment_in_registers<4>(seg, len, val, acc);
    } else if (len <= 16) {
        sum_segment_in_registers<16>(seg, len, val, acc);
    } else {
        for (unsigned i = 1; i < len; ++i) {
            const unsigned v = seg[i];
            unsigned j = i;
            while (j > 0 && seg[j - 1] > v) {
                seg[j] = seg[j - 1];
                --j;
            }
            seg[j] = v;
        }
        for (unsigned i = 0; i < len; ++i) {
            const float2 v = val[seg[i]];
            acc.x = __fadd_rn(acc.x, v.x);
            acc.y = __fadd_rn(acc.y, v.y);
        }
    }
    *cell = acc;
    if (p.counter_mode == BGI_COUNTERS_PER_IMAGE || (p.counter_mode == BGI_COUNTERS_FIRST_INTERVAL && img < p.n_channels)) {
        float *cnt = p.counters + (size_t)(img - p.counter_base) * cells + c;
        float f = *cnt;
        for (unsigned i = 0; i < len; ++i) f = __fadd_rn(f, 1.0f);
        *cnt = f;
    }
}

// Ascending bitonic sort of s[0..len) in shared memory, padded with 0xffffffff to the next power
// of two P (the padding sorts last; s holds P entries).  Every thread of the block takes part.
__device__ void bitonic_sort_shared(unsigned *s, unsigned len) {
    unsigned P = 2;
    while (P < len) P <<= 1;
    for (unsigned i = len + threadIdx.x; i < P; i += blockDim.x) s[i] = 0xffffffffu;
    __syncthreads();
    for (unsigned k = 2; k <= P; k <<= 1) {
        for (unsigned j = k >> 1; j > 0; j >>= 1) {
            for (unsigned i = threadIdx.x; i < P; i += blockDim.x) {
                const unsigned ixj = i ^ j;  // < P: j < P and P is a power of two
                if (ixj > i) {
                    const unsigned a = s[i], b = s[ixj];
                    if ((a > b) == ((i & k) == 0)) {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// long segments: one block per cell.  A segment of up to kLongSort points is loaded into shared
// memory and sorted there; a longer one has each point index placed at its rank (the number of
// smaller indices in the segment, counted against shared-memory tiles) in the cell's range of
// the key array, which is free after placement.  Then the values are staged in tiles in index
// order and thread 0 adds them in that order.
// HUGE: the cells listed from the back (more than kLongSort points), sorted in shared memory up
// to kHugeSort.  Shared memory (dynamic): CAP point indices, then kTile staged values.
template <bool HUGE>
__global__ void __launch_bounds__(kLongThreads) long_kernel(const GridParams p, int chunk_first, SortedWs w,
                                                            long long n_points) {
    constexpr unsigned CAP = HUGE ? kHugeSort : kLongSort;
    extern __shared__ __align__(16) unsigned s_dyn[];
    unsigned *s_idx = s_dyn;
    float2 *s_val = reinterpret_cast<float2 *>(s_dyn + CAP);
    const size_t cells = grid_cells(p);
    const int local = blockIdx.y;
    const int img = chunk_first + local;
    const size_t cap = long_cap(n_points / 2);
    const unsigned n_list = HUGE ? w.n_huge[local] : w.n_long[local];
    for (unsigned li = blockIdx.x; li < n_list; li += gridDim.x) {
        const unsigned c = w.longs[(size_t)local * cap + (HUGE ? cap - 1 - li : li)];
        const size_t cbase = (size_t)local * cells;
        const unsigned len = w.cnt[cbase + c];
        const unsigned st = seg_start(w, local, cells, c);
        const unsigned *seg = w.seg + (size_t)local * n_points + st;
        unsigned *ordered = w.key + (size_t)local * n_points + st;
        const bool in_shared = len <= CAP;
        if (in_shared) {
            for (unsigned i = threadIdx.x; i < len; i += kLongThreads) s_idx[i] = seg[i];
            bitonic_sort_shared(s_idx, len);  // ends with a block barrier
            ordered = s_idx;
        }
        for (unsigned i0 = 0; !in_shared && i0 < len; i0 += kLongThreads) {
            const bool mine_valid = i0 + threadIdx.x < len;
            const unsigned mine = mine_valid ? seg[i0 + threadIdx.x] : 0u;
            unsigned rank = 0;
            for (unsigned j0 = 0; j0 < len; j0 += kTile) {
                const unsigned m = min((unsigned)kTile, len - j0);
                __syncthreads();
                for (unsigned t = threadIdx.x; t < m; t += kLongThreads) s_idx[t] = seg[j0 + t];
                __syncthreads();
                for (unsigned t = 0; t < m; ++t) rank += s_idx[t] < mine;
            }
            if (mine_valid) ordered[rank] = mine;
        }
        __syncthreads();
        float2 *cell = p.grids + (size_t)(img - p.img_base) * cells + c;
        float2 acc = make_float2(0.f, 0.f);
        if (threadIdx.x == 0 && !p.grids_zero) acc = *cell;
        const float2 *val = w.val + (size_t)local * n_points;
        for (unsigned j0 = 0; j0 < len; j0 += kTile) {
            const unsigned m = min((unsigned)kTile, len - j0);
            __syncthreads();
            for (unsigned t = threadIdx.x; t < m; t += kLongThreads) s_val[t] = val[ordered[j0 + t]];
            __syncthreads();
            if (threadIdx.x == 0) {
                for (unsigned t = 0; t < m; ++t) {
                    acc.x = __fadd_rn(acc.x, s_val[t].x);
                    acc.y = __fadd_rn(acc.y, s_val[t].y);
                }
            }
        }
        if (threadIdx.x == 0) {
            *cell = acc;
            if (p.counter_mode == BGI_COUNTERS_PER_IMAGE ||
                (p.counter_mode == BGI_COUNTERS_FIRST_INTERVAL && img < p.n_channels)) {
                float *cnt = p.counters + (size_t)(img - p.counter_base) * cells + c;
                float f = *cnt;
                for (unsigned i = 0; i < len; ++i) f = __fadd_rn(f, 1.0f);
                *cnt = f;
            }
        }
        __syncthreads();
    }
}

constexpr size_t long_smem_bytes(unsigned cap) { return cap * sizeof(unsigned) + kTile * sizeof(float2); }

}  // namespace

size_t sorted_workspace_bytes(long long n_baselines, int n_pixels, int n_images) {
    return per_image_bytes(n_baselines, (size_t)n_pixels * n_pixels) * (size_t)std::max(1, n_images);
}

int launch_gridding_sorted(const GridParams &p, void *ws, size_t ws_bytes, cudaStream_t s) {
    if (p.img_count <= 0 || p.n_baselines <= 0) return BGI_OK;
    {  // the huge-segment kernel's shared memory is above the default 48 KB
        const int st = check_cuda(cudaFuncSetAttribute(long_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)long_smem_bytes(kHugeSort)),
                                  "gridding_sorted: shared memory of the huge-segment kernel");
        if (st) return st;
    }
    int dev = 0, n_sm = 0;
    {
        int st = check_cuda(cudaGetDevice(&dev), "gridding_sorted: device");
        if (!st) st = check_cuda(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev), "gridding_sorted: SMs");
        if (st) return st;
    }
    const size_t cells = grid_cells(p);
    const size_t per = per_image_bytes(p.n_baselines, cells);
    const int chunk = (int)std::min<size_t>((size_t)p.img_count, ws_bytes / per);
    if (chunk < 1 || !ws) return set_error(BGI_ERR_INVALID, "gridding_sorted: workspace of %zu bytes is below %zu", ws_bytes, per);
    const long long n_points = 2 * p.n_baselines;
    const unsigned bx_b = (unsigned)((p.n_baselines + kThreads - 1) / kThreads);
    const unsigned bx_p = (unsigned)((n_points + kThreads - 1) / kThreads);
    const unsigned bx_c = (unsigned)((cells + kThreads - 1) / kThreads);
    for (int img0 = p.img_begin; img0 < p.img_begin + p.img_count; img0 += chunk) {
        const int cnt = std::min(chunk, p.img_begin + p.img_count - img0);
        SortedWs w = carve(ws, cnt, p.n_baselines, cells);
        const size_t cell_bytes = sizeof(unsigned) * cells * cnt;
        int st = check_cuda(cudaMemsetAsync(w.cnt, 0, cell_bytes, s), "gridding_sorted: clear counts");
        if (st) return st;
        st = check_cuda(cudaMemsetAsync(w.cursor, 0, cell_bytes, s), "gridding_sorted: clear cursors");
        if (st) return st;
        st = check_cuda(cudaMemsetAsync(w.n_long, 0, sizeof(unsigned) * cnt, s), "gridding_sorted: clear long list");
        if (st) return st;
        st = check_cuda(cudaMemsetAsync(w.n_huge, 0, sizeof(unsigned) * cnt, s), "gridding_sorted: clear huge list");
        if (st) return st;
        for (int done = 0; done < cnt; done += 65535) {
            const int k = std::min(65535, cnt - done);
            SortedWs wd = w;
            wd.key += (size_t)done * n_points;
            wd.val += (size_t)done * n_points;
            wd.cnt += (size_t)done * cells;
            keys_kernel<<<dim3(bx_b, k), kThreads, 0, s>>>(p, img0 + done, wd);
            if ((st = check_launch("gridding_sorted keys"))) return st;
        }
        for (int done = 0; done < cnt; done += 65535) {
            const int k = std::min(65535, cnt - done);
            SortedWs wd = w;
            wd.cnt += (size_t)done * cells;
            wd.start += (size_t)done * cells;
            wd.tile_off += (size_t)done * scan_tiles(cells);
            if (cells % 4 == 0)
                scan_tiles_kernel<true><<<dim3((unsigned)scan_tiles(cells), k), kThreads, 0, s>>>(wd, cells);
            else
                scan_tiles_kernel<false><<<dim3((unsigned)scan_tiles(cells), k), kThreads, 0, s>>>(wd, cells);
            if ((st = check_launch("gridding_sorted scan tiles"))) return st;
        }
        scan_offsets_kernel<<<cnt, 1024, 0, s>>>(w, cells);
        if ((st = check_launch("gridding_sorted scan offsets"))) return st;
        for (int done = 0; done < cnt; done += 65535) {
            const int k = std::min(65535, cnt - done);
            SortedWs wd = w;
            wd.key += (size_t)done * n_points;
            wd.val += (size_t)done * n_points;
            wd.seg += (size_t)done * n_points;
            wd.cnt += (size_t)done * cells;
            wd.start += (size_t)done * cells;
            wd.cursor += (size_t)done * cells;
            wd.tile_off += (size_t)done * scan_tiles(cells);
            place_kernel<<<dim3(bx_p, k), kThreads, 0, s>>>(wd, n_points, cells);
            if ((st = check_launch("gridding_sorted place"))) return st;
            wd.n_long += done;
            wd.n_huge += done;
            wd.longs += (size_t)done * long_cap(p.n_baselines);
            reduce_kernel<<<dim3(bx_c, k), kThreads, 0, s>>>(p, img0 + done, wd, n_points);
            if ((st = check_launch("gridding_sorted reduce"))) return st;
            const unsigned long_blocks = (unsigned)std::max(kLongBlocks, (4 * n_sm + k - 1) / k);
            long_kernel<false><<<dim3(long_blocks, k), kLongThreads, long_smem_bytes(kLongSort), s>>>(p, img0 + done, wd,
                                                                                                   n_points);
            if ((st = check_launch("gridding_sorted long segments"))) return st;
            long_kernel<true><<<dim3(kHugeBlocks, k), kLongThreads, long_smem_bytes(kHugeSort), s>>>(p, img0 + done, wd,
                                                                                                  n_points);
            if ((st = check_launch("gridding_sorted huge segments"))) return st;
        }
    }
    return BGI_OK;
}

}  // namespace bgi
