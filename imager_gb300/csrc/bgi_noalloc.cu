// Dirty imaging without any device allocation: bgi_image_noalloc.
//
// Some callers cannot allocate device memory while they run.  A real-time correlator/imager
// chain that budgets all of the GPU's memory when an observation starts and forbids allocation
// on the data path is one; another is a host framework that owns the device allocator and
// hands out only the buffers it manages; a third is code that must not call cudaMalloc or
// cudaFree on a live pipeline because those calls can synchronise the device and stall the
// other streams.  For them, this entry point grids and transforms with scratch memory that the
// library holds statically in this file: a 32 MiB grid and per-image weight counters for up
// to 1024 images per wave.  The caller still passes its inputs and its output images.
//
// The cost of that convenience: every GPU on which the library's code is loaded holds these
// 32.1 MiB until the process exits.  CUDA loads a library's device code lazily by default (at
// the first use of each of its modules), so the scratch is committed on a device by the first
// call of this function there -- its address look-up loads this file's module -- and the
// gridding and FFT modules load at their first launches.  A caller that budgets device memory
// up front makes one warm-up call per device when it sets its budget (or runs with
// CUDA_MODULE_LOADING=EAGER, which loads every module, and so commits the scratch, when the
// library's first CUDA call creates the context).
//
// Limits and behaviour:
//  * one N x N complex grid must fit the scratch: N <= 2048 (an image side of 4096 is
//    rejected); larger blocks are processed in waves of as many images as fit;
//  * the first call on each device looks up the scratch's device address
//    (cudaGetSymbolAddress), which loads the module and commits the scratch; make it before
//    any stream capture on that device and before the device's memory is budgeted;
//  * the address is cached per device for the life of the process: after cudaDeviceReset (or
//    any other teardown of the device's primary context) the library must not be used again
//    in that process, as every device pointer it holds is then stale;
//  * every call shares the one scratch and leaves its last contents there; each call clears the
//    part it uses before gridding, so no state carries over from an earlier call, but calls
//    whose work overlaps on the GPU (different streams, or different host threads) race on
//    the scratch and give wrong images -- serialise them;
//  * no cudaMalloc, cudaFree or other allocating call is made.
#include <algorithm>
#include <mutex>

#include "bgi_internal.h"

namespace bgi {
namespace {
constexpr size_t kNoAllocGridBytes = (size_t)32 << 20;
constexpr size_t kNoAllocGridElems = kNoAllocGridBytes / sizeof(float2);
constexpr int kNoAllocMaxWave = 1024;
constexpr int kMaxDevices = 64;
}  // namespace
}  // namespace bgi

// The static scratch (one copy per device that loads the library).
static __device__ __align__(256) float2 g_noalloc_grid[bgi::kNoAllocGridElems];
static __device__ __align__(256) unsigned int g_noalloc_wsum[bgi::kNoAllocMaxWave * bgi::kWsumStride];

namespace bgi {
namespace {

struct Scratch {
    float2 *grid = nullptr;
    unsigned int *wsum = nullptr;
};

std::mutex g_scratch_mutex;
Scratch g_scratch[kMaxDevices];

// Device addresses of the static scratch on the current device, looked up once per device.
int scratch_for_current_device(Scratch *out) {
    int dev = -1;
    int st = check_cuda(cudaGetDevice(&dev), "image_noalloc: cudaGetDevice");
    if (st) return st;
    if (dev < 0 || dev >= kMaxDevices) return set_error(BGI_ERR_UNSUPPORTED, "image_noalloc: device %d", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    Scratch &s = g_scratch[dev];
    if (!s.grid) {
        void *grid = nullptr, *wsum = nullptr;
        st = check_cuda(cudaGetSymbolAddress(&grid, g_noalloc_grid), "image_noalloc: scratch grid address");
        if (st) return st;
        st = check_cuda(cudaGetSymbolAddress(&wsum, g_noalloc_wsum), "image_noalloc: scratch counter address");
        if (st) return st;
        s.grid = static_cast<float2 *>(grid);
        s.wsum = static_cast<unsigned int *>(wsum);
    }
    *out = s;
    return BGI_OK;
}

}  // namespace
}  // namespace bgi

using namespace bgi;

extern "C" BGI_API int bgi_image_noalloc(const float *vis, int n_ant, int n_channels, int n_intervals,
                                         const float *u, const float *v, int n_uvw_sets,
                                         const int *baseline_flags, const double *freqs_hz,
                                         double delta_u, double delta_v, int n_pixels, double min_uv,
                                         int pol, float *images, void *stream) {
    if (!vis || !u || !v || !baseline_flags || !freqs_hz || !images || n_ant < 1 || n_channels < 1 ||
        n_intervals < 1)
        return set_error(BGI_ERR_INVALID, "image_noalloc: bad arguments");
    if (pol < BGI_POL_XX || pol > BGI_POL_V) return set_error(BGI_ERR_INVALID, "image_noalloc: bad pol %d", pol);
    if (n_uvw_sets != 1 && n_uvw_sets != n_intervals)
        return set_error(BGI_ERR_INVALID, "image_noalloc: n_uvw_sets must be 1 or n_intervals");
    if (!(delta_u > 0) || !(delta_v > 0)) return set_error(BGI_ERR_INVALID, "image_noalloc: delta_u/v must be > 0");
    if ((reinterpret_cast<uintptr_t>(vis) & 15u) || (reinterpret_cast<uintptr_t>(images) & 7u))
        return set_error(BGI_ERR_INVALID, "image_noalloc: vis must be 16-byte and images 8-byte aligned");
    if ((long long)n_intervals * n_channels > 2147483647LL)
        return set_error(BGI_ERR_INVALID, "image_noalloc: n_intervals * n_channels exceeds 2^31 - 1");
    // powers of two only: the mixed-radix passes of other sides allocate a twiddle table
    if (!fft_pow2_size(n_pixels))
        return set_error(BGI_ERR_UNSUPPORTED, "image_noalloc: image side %d (powers of two 16..2048)", n_pixels);
    const size_t npix = (size_t)n_pixels * n_pixels;
    if (npix > kNoAllocGridElems)
        return set_error(BGI_ERR_UNSUPPORTED,
                         "image_noalloc: a %dx%d grid needs %zu MiB; the static scratch holds %zu MiB "
                         "(image side <= 2048)", n_pixels, n_pixels, (npix * sizeof(float2)) >> 20,
                         kNoAllocGridBytes >> 20);
    Scratch sc;
    int st = scratch_for_current_device(&sc);
    if (st) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const int n_images = n_intervals * n_channels;
    const int wave = (int)std::min(std::min((size_t)n_images, kNoAllocGridElems / npix), (size_t)kNoAllocMaxWave);

    // The grid must start at zero; the row pass re-zeroes what it reads, so one clear per call
    // covers every wave of the call.
    st = check_cuda(cudaMemsetAsync(sc.grid, 0, sizeof(float2) * npix * wave, s), "image_noalloc: clear grid");
    if (st) return st;

    GridParams p{};
    p.vis = vis;
    p.u = u;
    p.v = v;
    p.flags = baseline_flags;
    p.freqs = freqs_hz;
    p.grids = sc.grid;
    p.wsum = sc.wsum;
    p.du = delta_u;
    p.dv = delta_v;
    p.min_uv = min_uv;
    p.n_baselines = (long long)n_ant * (n_ant + 1) / 2;
    p.n_channels = n_channels;
    p.n_intervals = n_intervals;
    p.n_uvw_sets = n_uvw_sets;
    p.n_pixels = n_pixels;
    p.pol = pol;
    p.counter_mode = -1;
    float2 *out = reinterpret_cast<float2 *>(images);
    for (int img0 = 0; img0 < n_images; img0 += wave) {
        const int cnt = std::min(wave, n_images - img0);
        st = check_cuda(cudaMemsetAsync(sc.wsum, 0, sizeof(unsigned int) * kWsumStride * cnt, s),
                        "image_noalloc: clear weight counters");
        if (st) return st;
        p.img_begin = img0;
        p.img_count = cnt;
        p.img_base = img0;
        st = launch_gridding(p, s);
        if (st) return st;
        st = launch_fft_rows(sc.grid, out + (size_t)img0 * npix, n_pixels, cnt, true, s);
        if (st) return st;
        st = launch_fft_cols(out + (size_t)img0 * npix, n_pixels, cnt, sc.wsum, s);
        if (st) return st;
    }
    return BGI_OK;
}
