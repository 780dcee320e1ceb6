// C ABI of the BLINK GB300 imaging path (include/blink_imager_gb300.h).
//
// Free functions mirror the reference's GPU entry points (src/gpu/*.h) on device pointers.
// The imager handle mirrors CPacerImagerHip's resident members (src/gpu/pacer_imager_hip.h:14-27)
// and runs the fused path: per wave of images, one gridding launch (corrections fused), one
// row-FFT launch (which also re-zeroes the grid scratch) and one column-FFT launch (fftshift
// and 1/sum(weights) fused into its stores).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <memory>
#include <vector>

#include <nvtx3/nvToolsExt.h>  // header-only; ranges cost nothing without a profiler attached

#include "bgi_internal.h"

namespace bgi {

static thread_local std::string g_last_error;

int set_error(int status, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return BGI_OK;
    return set_error(e == cudaErrorMemoryAllocation ? BGI_ERR_ALLOC : BGI_ERR_CUDA, "%s: %s (%s)",
                     what, cudaGetErrorString(e), cudaGetErrorName(e));
}

int check_launch(const char *what) { return check_cuda(cudaGetLastError(), what); }

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace bgi

using namespace bgi;

#define BGI_TRY(expr)              \
    do {                           \
        int _st = (expr);          \
        if (_st != BGI_OK) return _st; \
    } while (0)

namespace {
// An NVTX range over a scope, named for the C-ABI call it covers: it shows the call on timelines
// of Nsight Systems and similar tools, and `ncu --nvtx --nvtx-include "<name>/"` profiles only
// the kernels that call launched.
struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};
}  // namespace

namespace {

cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Visibility records are read and written as 16-byte vectors.
bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

long long baselines_of(int n_ant) { return (long long)n_ant * (n_ant + 1) / 2; }

template <class T>
int dev_alloc(T **p, size_t count, const char *what) {
    *p = nullptr;
    if (count == 0) return BGI_OK;
    return check_cuda(cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * count), what);
}

template <class T>
void dev_free(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// grow-only device buffer
template <class T>
struct DevBuf {
    T *ptr = nullptr;
    size_t cap = 0;
    int ensure(size_t count, const char *what, bool *fresh = nullptr) {
        if (fresh) *fresh = false;
        if (count <= cap) return BGI_OK;
        dev_free(ptr);
        cap = 0;
        BGI_TRY(dev_alloc(&ptr, count, what));
        cap = count;
        if (fresh) *fresh = true;
        return BGI_OK;
    }
    void release() {
        dev_free(ptr);
        cap = 0;
    }
};

}  // namespace

struct bgi_imager {
    bgi_config cfg{};
    int n_ant = 0, n_uvw_sets = 0, n_channels = 0;
    long long n_baselines = 0;
    double u_max = 0, v_max = 0, delta_u = 0, delta_v = 0;
    double freq_max = 0;  // highest channel frequency (Hz)
    // a baseline flag below zero: gridded (flags <= 0 are) but outside u_max / v_max (flag 0
    // only), so the largest pixel coordinate is unknown and the half plane is not used
    bool negative_flags = false;

    // The half-plane path needs every gridded point's mirror cell: |u|,|v| pixels < N.  The
    // largest pixel coordinate is u_max * nu_max / (c * delta_u); one pixel of margin covers
    // the rounding of the FP64 recipe.
    bool half_plane() const {
        if (cfg.full_plane || half_plane_width(cfg.n_pixels) == 0 || freq_max <= 0 || negative_flags) return false;
        const double up = u_max * freq_max / (kVelLight * delta_u);
        const double vp = v_max * freq_max / (kVelLight * delta_v);
        return up < cfg.n_pixels - 1 && vp < cfg.n_pixels - 1;
    }
    // Whether bgi_image grids the half plane (images 16-byte aligned): the exactness condition
    // above, and no convolution kernel (full plane).  The ordered gridder sums the half plane's
    // cells as it sums the full plane's.
    bool half_plane_path() const { return half_plane() && kb_size == 0; }
    // Bound on the pixel coordinates |u|, |v| of every gridded point (bgi_uv_extent), for
    // pruning the half-plane FFT passes.
    void half_plane_extent(int *eu, int *ev) const {
        int u = cfg.n_pixels / 2, v = cfg.n_pixels / 2;  // no pruning unless the bound is known
        if (bgi_uv_extent(u_max, v_max, delta_u, delta_v, freq_max, cfg.n_pixels, &u, &v) != BGI_OK)
            u = v = cfg.n_pixels / 2;
        *eu = u;
        *ev = v;
    }
    float *d_u = nullptr, *d_v = nullptr, *d_w = nullptr;
    float2 *d_dl = nullptr;  // cable delay L[a2]-L[a1] per baseline as (hi, lo) floats
    DevBuf<ChannelConst> d_cc; // per-channel gridding constants for the current delta_u/v
    int kb_size = 0;           // Kaiser-Bessel kernel size (0: nearest neighbour)
    int fft_mode = BGI_FFT_SIMT;  // enum bgi_fft_mode
    int grid_cpt = 0;             // gridding images per thread (0: by array size)
    int col_radix = 0;            // column-pass radix of the half plane (0: the side's default)
    int grid_agg = 0;             // 1: warp-aggregated gridding atomics (4 or 8 images per thread)
    DevBuf<float> kb_table;    // its rows [1023][kb_size]
    bool cc_valid = false;     // d_cc matches the frequencies and delta_u/v
    int *d_flags = nullptr;
    double *d_freqs = nullptr;
    // Lanes (streams; two unless bgi_set_schedule or bgi_autotune chose otherwise) image
    // alternate waves, each with its own grid scratch, so one wave's
    // FFT passes overlap the next wave's gridding; the scratch of a lane is reused wave after
    // wave and sized to stay in L2.
    static constexpr int kLanes = 8;  // at most; `lanes` are in use (bgi_set_schedule, bgi_autotune)
    int lanes = 2;
    DevBuf<float2> grid[kLanes];  // wave scratch: images x N*N, zero between waves
    bool grid_dirty[kLanes] = {};
    // counter grids of a wave (uniform weighting only): images x N*N, zero between waves
    DevBuf<float> cnt[kLanes];
    bool cnt_dirty[kLanes] = {};
    cudaStream_t lane[kLanes] = {};
    cudaEvent_t ev_fork = nullptr, ev_join[kLanes] = {};
    // Deterministic mode: gridding by sort and ordered per-cell sums (the half plane when the
    // handle takes it), with a workspace per lane for one wave.
    bool deterministic = false;
    DevBuf<unsigned char> sorted_ws[kLanes];
    DevBuf<unsigned int> wsum;    // per-image weight counts of the last call
    DevBuf<float> io_vis, io_img; // device staging of bgi_image_host
    DevBuf<float> io_scales;      // block scales staged by bgi_image_compressed_host
    DevBuf<float> io_mat;         // correlation matrices staged by bgi_image_correlation_matrices_host
    int last_images = 0;

    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    std::vector<cudaEvent_t> ev_in, ev_done;  // per chunk of bgi_image_host

    // Replay of repeated calls.  The second of two consecutive calls with the same arguments
    // on an unchanged handle is also captured into a CUDA graph (on cap_stream: recorded, not
    // run); while the calls keep repeating, each one is that graph launched on the caller's
    // stream, one launch in place of the ~100-200 stream operations of the waves and copies.
    // Any other call, and every call that changes the handle's state, drops the graph.
    struct CallKey {
        int kind = -1, format = 0, n_intervals = 0;
        unsigned flags = 0;
        const void *in[5] = {};
        const void *out = nullptr;
        bool operator==(const CallKey &o) const {
            if (kind != o.kind || format != o.format || n_intervals != o.n_intervals || flags != o.flags || out != o.out)
                return false;
            for (int i = 0; i < 5; ++i)
                if (in[i] != o.in[i]) return false;
            return true;
        }
    };
    CallKey last_key, graph_key;
    bool replay_enabled = true;  // bgi_set_replay
    bool have_last = false, replay_refused = false;
    cudaGraphExec_t graph_exec = nullptr;
    cudaStream_t cap_stream = nullptr;
    void drop_graph() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
        have_last = false;
        replay_refused = false;
    }

    int ensure_copy_streams() {
        if (copy_in) return BGI_OK;
        BGI_TRY(check_cuda(cudaStreamCreateWithFlags(&copy_in, cudaStreamNonBlocking), "copy stream"));
        return check_cuda(cudaStreamCreateWithFlags(&copy_out, cudaStreamNonBlocking), "copy stream");
    }
    int ensure_chunk_events(int n_chunks) {
        while ((int)ev_in.size() < n_chunks) {
            cudaEvent_t e;
            BGI_TRY(check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "chunk event"));
            ev_in.push_back(e);
        }
        while ((int)ev_done.size() < n_chunks * kLanes) {
            cudaEvent_t e;
            BGI_TRY(check_cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "chunk event"));
            ev_done.push_back(e);
        }
        return BGI_OK;
    }

    int ensure_lanes() {
        if (lane[0]) return BGI_OK;
        for (int l = 0; l < kLanes; ++l) {
            BGI_TRY(check_cuda(cudaStreamCreateWithFlags(&lane[l], cudaStreamNonBlocking), "lane stream"));
            BGI_TRY(check_cuda(cudaEventCreateWithFlags(&ev_join[l], cudaEventDisableTiming), "lane event"));
        }
        return check_cuda(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming), "fork event");
    }
    // stage timing: event quads (before gridding, after gridding, after rows, after cols)
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;

    int next_event(cudaEvent_t *e) {
        if (ev_used == ev_pool.size()) {
            cudaEvent_t ne;
            BGI_TRY(check_cuda(cudaEventCreate(&ne), "stage timing event"));
            ev_pool.push_back(ne);
        }
        *e = ev_pool[ev_used++];
        return BGI_OK;
    }
    int mark(cudaStream_t s) {
        if (!timing) return BGI_OK;
        cudaEvent_t e;
        BGI_TRY(next_event(&e));
        return check_cuda(cudaEventRecord(e, s), "stage timing record");
    }

    int activate() const {
        int cur = -1;
        cudaGetDevice(&cur);
        if (cur != cfg.device) return check_cuda(cudaSetDevice(cfg.device), "cudaSetDevice");
        return BGI_OK;
    }
    void release_array() {
        dev_free(d_u);
        dev_free(d_v);
        dev_free(d_w);
        dev_free(d_dl);
        dev_free(d_flags);
    }
};

extern "C" {

const char *bgi_last_error(void) { return g_last_error.c_str(); }

int bgi_version(void) { return 100 * BGI_VERSION_MAJOR + BGI_VERSION_MINOR; }

// ------------------------------------------------------------------------------------------
// Free functions
// ------------------------------------------------------------------------------------------
int bgi_apply_geometric_corrections_gpu(float *vis, int n_ant, int n_channels, int n_intervals,
                                        const float *w, int n_uvw_sets, const double *freqs_hz,
                                        void *stream) {
    TraceRange trace("bgi_apply_geometric_corrections_gpu");
    if (!vis || !w || !freqs_hz || n_ant < 1 || n_channels < 1 || n_intervals < 0)
        return set_error(BGI_ERR_INVALID, "apply_geometric_corrections: bad arguments");
    if (n_uvw_sets != 1 && n_uvw_sets != n_intervals)
        return set_error(BGI_ERR_INVALID, "apply_geometric_corrections: n_uvw_sets must be 1 or n_intervals");
    if (!aligned16(vis)) return set_error(BGI_ERR_INVALID, "apply_geometric_corrections: vis must be 16-byte aligned");
    return launch_geometric(vis, n_ant, n_channels, n_intervals, w, n_uvw_sets, freqs_hz,
                            as_stream(stream));
}

int bgi_apply_cable_lengths_corrections_gpu(float *vis, int n_ant, int n_channels,
                                            int n_intervals, const double *cable_lengths,
                                            const double *freqs_hz, void *stream) {
    TraceRange trace("bgi_apply_cable_lengths_corrections_gpu");
    if (!vis || !cable_lengths || !freqs_hz || n_ant < 1 || n_channels < 1 || n_intervals < 0)
        return set_error(BGI_ERR_INVALID, "apply_cable_lengths_corrections: bad arguments");
    if (!aligned16(vis)) return set_error(BGI_ERR_INVALID, "apply_cable_lengths_corrections: vis must be 16-byte aligned");
    return launch_cable(vis, n_ant, n_channels, n_intervals, cable_lengths, freqs_hz,
                        as_stream(stream));
}

namespace {

// Checks the arguments shared by both gridders and fills the launch parameters.
int gridding_params(const char *who, const float *vis, int n_ant, int n_channels, int n_intervals,
                    const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                    const double *freqs_hz, double delta_u, double delta_v, int n_pixels, double min_uv,
                    int pol, int counter_mode, float *counters, float *grids, GridParams *out) {
    if (!vis || !u || !v || !baseline_flags || !freqs_hz || !grids || n_ant < 1 ||
        n_channels < 1 || n_intervals < 0 || n_pixels < 1 || n_pixels > 46340)
        return set_error(BGI_ERR_INVALID, "%s: bad arguments", who);
    if (pol < BGI_POL_XX || pol > BGI_POL_V) return set_error(BGI_ERR_INVALID, "%s: bad pol %d", who, pol);
    if (n_uvw_sets != 1 && n_uvw_sets != n_intervals)
        return set_error(BGI_ERR_INVALID, "%s: n_uvw_sets must be 1 or n_intervals", who);
    if (counters && counter_mode != BGI_COUNTERS_FIRST_INTERVAL && counter_mode != BGI_COUNTERS_PER_IMAGE)
        return set_error(BGI_ERR_INVALID, "%s: bad counter_mode %d", who, counter_mode);
    if (!(delta_u > 0) || !(delta_v > 0)) return set_error(BGI_ERR_INVALID, "%s: delta_u/v must be > 0", who);
    if (!aligned16(vis)) return set_error(BGI_ERR_INVALID, "%s: vis must be 16-byte aligned", who);
    if ((reinterpret_cast<uintptr_t>(grids) & 7u) != 0) return set_error(BGI_ERR_INVALID, "%s: grids must be 8-byte aligned", who);
    GridParams p{};
    p.vis = vis;
    p.u = u;
    p.v = v;
    p.flags = baseline_flags;
    p.freqs = freqs_hz;
    p.grids = reinterpret_cast<float2 *>(grids);
    p.counters = counters;
    p.du = delta_u;
    p.dv = delta_v;
    p.min_uv = min_uv;
    p.n_baselines = baselines_of(n_ant);
    p.n_channels = n_channels;
    p.n_intervals = n_intervals;
    p.n_uvw_sets = n_uvw_sets;
    p.n_pixels = n_pixels;
    p.pol = pol;
    p.img_begin = 0;
    p.img_count = n_channels * n_intervals;
    p.img_base = 0;
    p.counter_mode = counters ? counter_mode : -1;
    *out = p;
    return BGI_OK;
}

}  // namespace

int bgi_gridding_gpu(const float *vis, int n_ant, int n_channels, int n_intervals,
                     const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                     const float *antenna_weights, const double *freqs_hz, double delta_u,
                     double delta_v, int n_pixels, double min_uv, int pol, int counter_mode,
                     float *counters, float *grids, void *stream) {
    (void)antenna_weights;
    TraceRange trace("bgi_gridding_gpu");
    GridParams p;
    BGI_TRY(gridding_params("gridding", vis, n_ant, n_channels, n_intervals, u, v, n_uvw_sets, baseline_flags,
                            freqs_hz, delta_u, delta_v, n_pixels, min_uv, pol, counter_mode, counters, grids, &p));
    return launch_gridding(p, as_stream(stream));
}

int bgi_gridding_sorted_workspace(int n_ant, int n_pixels, int n_images, size_t *bytes) {
    if (!bytes || n_ant < 1 || n_ant > kSortedMaxAnt || n_pixels < 1 || n_pixels > 46340 || n_images < 1)
        return set_error(BGI_ERR_INVALID, "gridding_sorted_workspace: bad arguments");
    *bytes = sorted_workspace_bytes(baselines_of(n_ant), n_pixels, n_images);
    return BGI_OK;
}

int bgi_gridding_sorted_gpu(const float *vis, int n_ant, int n_channels, int n_intervals,
                            const float *u, const float *v, int n_uvw_sets, const int *baseline_flags,
                            const double *freqs_hz, double delta_u, double delta_v, int n_pixels,
                            double min_uv, int pol, int counter_mode, float *counters, float *grids,
                            void *workspace, size_t workspace_bytes, void *stream) {
    TraceRange trace("bgi_gridding_sorted_gpu");
    if (n_ant > kSortedMaxAnt)
        return set_error(BGI_ERR_INVALID, "gridding_sorted: at most %d antennas", kSortedMaxAnt);
    if (!workspace || !aligned16(workspace))
        return set_error(BGI_ERR_INVALID, "gridding_sorted: workspace must be a 16-byte aligned device buffer");
    GridParams p;
    BGI_TRY(gridding_params("gridding_sorted", vis, n_ant, n_channels, n_intervals, u, v, n_uvw_sets,
                            baseline_flags, freqs_hz, delta_u, delta_v, n_pixels, min_uv, pol, counter_mode,
                            counters, grids, &p));
    return launch_gridding_sorted(p, workspace, workspace_bytes, as_stream(stream));
}

int bgi_fft_inverse_gpu(const float *grids, float *images, int n_pixels, int n_images,
                        void *stream) {
    TraceRange trace("bgi_fft_inverse_gpu");
    if (!grids || !images || n_images < 0) return set_error(BGI_ERR_INVALID, "fft_inverse: bad arguments");
    if (!fft_size_supported(n_pixels))
        return set_error(BGI_ERR_UNSUPPORTED, "fft_inverse: image side %d (1..4096)", n_pixels);
    if ((const void *)grids == (const void *)images)
        return set_error(BGI_ERR_INVALID, "fft_inverse: out of place only (grids != images)");
    cudaStream_t s = as_stream(stream);
    BGI_TRY(launch_fft_rows(reinterpret_cast<const float2 *>(grids), reinterpret_cast<float2 *>(images),
                            n_pixels, n_images, false, s));
    return launch_fft_cols(reinterpret_cast<float2 *>(images), n_pixels, n_images, nullptr, s);
}

int bgi_fft_shift_and_norm_gpu(float *images, int x_side, int y_side, int n_images,
                               const float *fnorm, int fnorm_size, void *stream) {
    TraceRange trace("bgi_fft_shift_and_norm_gpu");
    if (x_side % 2 != 0)  // src/gpu/gpu_utils.cpp:129-131
        return set_error(BGI_ERR_INVALID, "fft_shift_and_norm: only even image size is handled");
    if (!images || !fnorm || fnorm_size < 1 || x_side < 0 || y_side < 0 || n_images < 0)
        return set_error(BGI_ERR_INVALID, "fft_shift_and_norm: bad arguments");
    return launch_shift_and_norm(reinterpret_cast<float2 *>(images), x_side, y_side, n_images, fnorm,
                                 fnorm_size, as_stream(stream));
}

int bgi_uniform_weighting_gpu(float *grids, const float *counters, int n_pixels, int n_images, void *stream) {
    TraceRange trace("bgi_uniform_weighting_gpu");
    if (!grids || !counters || n_pixels < 1 || n_pixels > 46340 || n_images < 0)
        return set_error(BGI_ERR_INVALID, "uniform_weighting: bad arguments");
    if ((reinterpret_cast<uintptr_t>(grids) & 7u) != 0 || (reinterpret_cast<uintptr_t>(counters) & 3u) != 0)
        return set_error(BGI_ERR_INVALID, "uniform_weighting: grids must be 8-byte and counters 4-byte aligned");
    return launch_uniform_weighting(reinterpret_cast<float2 *>(grids), const_cast<float *>(counters),
                                    (long long)n_pixels * n_pixels * n_images, false, as_stream(stream));
}

int bgi_vector_sum_gpu(const float *data, int64_t image_size, int n_images, float *sums,
                       void *stream) {
    if (!data || !sums || image_size < 0 || n_images < 0)
        return set_error(BGI_ERR_INVALID, "vector_sum: bad arguments");
    return launch_vector_sum(data, image_size, n_images, sums, as_stream(stream));
}

int bgi_image_averaging_gpu(const float *images, int64_t image_size, int n_images, float *out,
                            void *stream) {
    if (!images || !out || image_size < 0 || n_images < 1)
        return set_error(BGI_ERR_INVALID, "image_averaging: bad arguments");
    return launch_image_average(reinterpret_cast<const float2 *>(images), image_size, n_images,
                                reinterpret_cast<float2 *>(out), as_stream(stream));
}

// ------------------------------------------------------------------------------------------
// Imager handle
// ------------------------------------------------------------------------------------------
int bgi_create(const bgi_config *cfg, bgi_imager **out) {
    if (!cfg || !out) return set_error(BGI_ERR_INVALID, "create: null argument");
    *out = nullptr;
    if (!fft_size_supported(cfg->n_pixels))
        return set_error(BGI_ERR_UNSUPPORTED, "create: image side %d (1..4096)", cfg->n_pixels);
    if (!(cfg->oversampling_factor > 0.0f)) return set_error(BGI_ERR_INVALID, "create: oversampling_factor must be > 0");
    if (cfg->pol < BGI_POL_XX || cfg->pol > BGI_POL_V) return set_error(BGI_ERR_INVALID, "create: bad pol %d", cfg->pol);
    if (cfg->max_images_per_wave < 0) return set_error(BGI_ERR_INVALID, "create: max_images_per_wave < 0");
    int n_dev = 0;
    BGI_TRY(check_cuda(cudaGetDeviceCount(&n_dev), "cudaGetDeviceCount"));
    if (cfg->device < 0 || cfg->device >= n_dev) return set_error(BGI_ERR_INVALID, "create: no device %d", cfg->device);
    bgi_imager *im = new (std::nothrow) bgi_imager();
    if (!im) return set_error(BGI_ERR_ALLOC, "create: out of host memory");
    im->cfg = *cfg;
    *out = im;
    return BGI_OK;
}

int bgi_destroy(bgi_imager *im) {
    if (!im) return BGI_OK;
    im->activate();
    im->drop_graph();
    if (im->cap_stream) cudaStreamDestroy(im->cap_stream);
    im->release_array();
    dev_free(im->d_freqs);
    for (cudaEvent_t e : im->ev_pool) cudaEventDestroy(e);
    for (int l = 0; l < bgi_imager::kLanes; ++l) {
        if (im->lane[l]) cudaStreamDestroy(im->lane[l]);
        if (im->ev_join[l]) cudaEventDestroy(im->ev_join[l]);
        im->grid[l].release();
        im->cnt[l].release();
        im->sorted_ws[l].release();
    }
    im->d_cc.release();
    im->kb_table.release();
    if (im->ev_fork) cudaEventDestroy(im->ev_fork);
    for (cudaEvent_t e : im->ev_in) cudaEventDestroy(e);
    for (cudaEvent_t e : im->ev_done) cudaEventDestroy(e);
    if (im->copy_in) cudaStreamDestroy(im->copy_in);
    if (im->copy_out) cudaStreamDestroy(im->copy_out);
    im->wsum.release();
    im->io_vis.release();
    im->io_scales.release();
    im->io_mat.release();
    im->io_img.release();
    delete im;
    return BGI_OK;
}

int bgi_set_array(bgi_imager *im, int n_ant, int n_uvw_sets, const float *u, const float *v,
                  const float *w, const int *baseline_flags, const double *cable_lengths) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im || !u || !v || !baseline_flags || n_ant < 1 || n_uvw_sets < 1)
        return set_error(BGI_ERR_INVALID, "set_array: bad arguments");
    BGI_TRY(im->activate());
    const long long nb = baselines_of(n_ant);
    const size_t nuv = (size_t)nb * n_uvw_sets;
    // u_max, v_max over unflagged baselines (src/pacer_imager.cpp:213-221), every set
    double um = -std::numeric_limits<double>::infinity(), vm = um;
    for (int s = 0; s < n_uvw_sets; ++s)
        for (long long b = 0; b < nb; ++b)
            if (baseline_flags[b] == 0) {
                um = std::max(um, (double)std::fabs(u[s * nb + b]));
                vm = std::max(vm, (double)std::fabs(v[s * nb + b]));
            }
    bool negative = false;
    for (long long b = 0; b < nb; ++b) negative = negative || baseline_flags[b] < 0;
    std::vector<float2> dl(nb, make_float2(0.f, 0.f));
    if (cable_lengths) {
        for (int a1 = 0; a1 < n_ant; ++a1)
            for (int a2 = 0; a2 <= a1; ++a2) {
                const double d = cable_lengths[a2] - cable_lengths[a1];
                const float hi = (float)d;
                dl[(size_t)a1 * (a1 + 1) / 2 + a2] = make_float2(hi, (float)(d - (double)hi));
            }
    }
    im->release_array();
    BGI_TRY(dev_alloc(&im->d_u, nuv, "set_array u"));
    BGI_TRY(dev_alloc(&im->d_v, nuv, "set_array v"));
    BGI_TRY(dev_alloc(&im->d_w, nuv, "set_array w"));
    BGI_TRY(dev_alloc(&im->d_dl, (size_t)nb, "set_array dl"));
    BGI_TRY(dev_alloc(&im->d_flags, (size_t)nb, "set_array flags"));
    BGI_TRY(check_cuda(cudaMemcpy(im->d_u, u, sizeof(float) * nuv, cudaMemcpyHostToDevice), "set_array copy"));
    BGI_TRY(check_cuda(cudaMemcpy(im->d_v, v, sizeof(float) * nuv, cudaMemcpyHostToDevice), "set_array copy"));
    if (w) BGI_TRY(check_cuda(cudaMemcpy(im->d_w, w, sizeof(float) * nuv, cudaMemcpyHostToDevice), "set_array copy"));
    else BGI_TRY(check_cuda(cudaMemset(im->d_w, 0, sizeof(float) * nuv), "set_array memset"));
    BGI_TRY(check_cuda(cudaMemcpy(im->d_dl, dl.data(), sizeof(float2) * nb, cudaMemcpyHostToDevice), "set_array copy"));
    BGI_TRY(check_cuda(cudaMemcpy(im->d_flags, baseline_flags, sizeof(int) * nb, cudaMemcpyHostToDevice), "set_array copy"));
    im->n_ant = n_ant;
    im->n_baselines = nb;
    im->n_uvw_sets = n_uvw_sets;
    im->negative_flags = negative;
    im->u_max = um;
    im->v_max = vm;
    // src/pacer_imager.cpp:497-499: float oversampling factor promoted to double
    im->cc_valid = false;
    im->delta_u = (double)im->cfg.oversampling_factor * um / im->cfg.n_pixels;
    im->delta_v = (double)im->cfg.oversampling_factor * vm / im->cfg.n_pixels;
    return BGI_OK;
}

int bgi_uvw_step_from_angles(const double *rmatpr, double ha2000, double dec_aber, double lmst, double lmst2000,
                             bgi_uvw_step *out) {
    if (!rmatpr || !out) return set_error(BGI_ERR_INVALID, "uvw_step_from_angles: null argument");
    for (int k = 0; k < 9; ++k) out->rmatpr[k] = rmatpr[k];
    out->sin_lmst = std::sin(lmst);
    out->cos_lmst = std::cos(lmst);
    out->sin_lmst2000 = std::sin(lmst2000);
    out->cos_lmst2000 = std::cos(lmst2000);
    out->sin_ha2000 = std::sin(ha2000);
    out->cos_ha2000 = std::cos(ha2000);
    out->sin_dec = std::sin(dec_aber);
    out->cos_dec = std::cos(dec_aber);
    return BGI_OK;
}

int bgi_pointed_uvw_gpu(const double *xyz, int n_ant, const bgi_uvw_step *steps, int n_steps, float *u, float *v,
                        float *w, void *stream) {
    if (!xyz || !steps || !u || !v || !w || n_ant < 1 || n_ant > 46340 || n_steps < 0)
        return set_error(BGI_ERR_INVALID, "pointed_uvw: bad arguments");
    static_assert(sizeof(bgi_uvw_step) == 17 * sizeof(double), "bgi_uvw_step is 17 doubles");
    return launch_pointed_uvw(xyz, n_ant, reinterpret_cast<const double *>(steps), n_steps, u, v, w,
                              as_stream(stream));
}

int bgi_set_array_pointed(bgi_imager *im, int n_ant, const double *xyz_host, int n_steps,
                          const bgi_uvw_step *steps_host, const int *baseline_flags, const double *cable_lengths) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im || !xyz_host || !steps_host || !baseline_flags || n_ant < 1 || n_ant > 46340 || n_steps < 1)
        return set_error(BGI_ERR_INVALID, "set_array_pointed: bad arguments");
    BGI_TRY(im->activate());
    const long long nb = baselines_of(n_ant);
    const size_t nuv = (size_t)nb * n_steps;
    // flags and cable delays as bgi_set_array installs them (with zero placeholder UVW), then the
    // UVW computed on the device in place of the placeholder
    double *d_xyz = nullptr, *d_steps = nullptr;
    unsigned *d_max = nullptr;
    int st = BGI_OK;
    {
        std::vector<float> zero((size_t)nb, 0.f);
        BGI_TRY(bgi_set_array(im, n_ant, 1, zero.data(), zero.data(), nullptr, baseline_flags, cable_lengths));
    }
    // grow the resident UVW to one set per step and compute it
    dev_free(im->d_u);
    dev_free(im->d_v);
    dev_free(im->d_w);
    im->d_u = im->d_v = im->d_w = nullptr;
    BGI_TRY(dev_alloc(&im->d_u, nuv, "set_array_pointed u"));
    BGI_TRY(dev_alloc(&im->d_v, nuv, "set_array_pointed v"));
    BGI_TRY(dev_alloc(&im->d_w, nuv, "set_array_pointed w"));
    if (!st) st = dev_alloc(&d_xyz, (size_t)n_ant * 3, "set_array_pointed xyz");
    if (!st) st = dev_alloc(&d_steps, (size_t)n_steps * 17, "set_array_pointed steps");
    if (!st) st = dev_alloc(&d_max, (size_t)2, "set_array_pointed max");
    if (!st) st = check_cuda(cudaMemcpy(d_xyz, xyz_host, sizeof(double) * 3 * n_ant, cudaMemcpyHostToDevice), "copy");
    if (!st)
        st = check_cuda(cudaMemcpy(d_steps, steps_host, sizeof(double) * 17 * n_steps, cudaMemcpyHostToDevice), "copy");
    if (!st) st = launch_pointed_uvw(d_xyz, n_ant, d_steps, n_steps, im->d_u, im->d_v, im->d_w, nullptr);
    if (!st) st = launch_uv_absmax(im->d_u, im->d_v, im->d_flags, nb, n_steps, d_max, nullptr);
    unsigned mx[2] = {0, 0};
    if (!st) st = check_cuda(cudaMemcpy(mx, d_max, sizeof(mx), cudaMemcpyDeviceToHost), "uv max");
    dev_free(d_xyz);
    dev_free(d_steps);
    dev_free(d_max);
    if (st) return st;
    float fu, fv;
    std::memcpy(&fu, &mx[0], 4);
    std::memcpy(&fv, &mx[1], 4);
    im->n_uvw_sets = n_steps;
    im->u_max = fu;
    im->v_max = fv;
    im->cc_valid = false;
    im->delta_u = (double)im->cfg.oversampling_factor * im->u_max / im->cfg.n_pixels;
    im->delta_v = (double)im->cfg.oversampling_factor * im->v_max / im->cfg.n_pixels;
    return BGI_OK;
}

int bgi_set_frequencies(bgi_imager *im, int n_channels, const double *freqs_hz) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im || !freqs_hz || n_channels < 1) return set_error(BGI_ERR_INVALID, "set_frequencies: bad arguments");
    for (int c = 0; c < n_channels; ++c)
        if (!(freqs_hz[c] > 0.0) || !std::isfinite(freqs_hz[c]))
            return set_error(BGI_ERR_INVALID, "set_frequencies: frequency %d is not a positive number", c);
    BGI_TRY(im->activate());
    dev_free(im->d_freqs);
    BGI_TRY(dev_alloc(&im->d_freqs, (size_t)n_channels, "set_frequencies"));
    BGI_TRY(check_cuda(cudaMemcpy(im->d_freqs, freqs_hz, sizeof(double) * n_channels, cudaMemcpyHostToDevice),
                       "set_frequencies copy"));
    im->n_channels = n_channels;
    im->freq_max = *std::max_element(freqs_hz, freqs_hz + n_channels);
    im->cc_valid = false;
    return BGI_OK;
}

int bgi_half_plane(const bgi_imager *im) {
    if (!im) return set_error(BGI_ERR_INVALID, "half_plane: null handle");
    if (im->n_ant == 0 || im->n_channels == 0)
        return set_error(BGI_ERR_STATE, "half_plane: set_array and set_frequencies first");
    return im->half_plane_path() ? 1 : 0;
}

int bgi_set_uv_cell(bgi_imager *im, double delta_u, double delta_v) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im) return set_error(BGI_ERR_INVALID, "set_uv_cell: null handle");
    if (im->n_ant == 0) return set_error(BGI_ERR_STATE, "set_uv_cell: array not set");
    if (!(delta_u > 0) || !(delta_v > 0) || !std::isfinite(delta_u) || !std::isfinite(delta_v))
        return set_error(BGI_ERR_INVALID, "set_uv_cell: delta_u/v must be finite and > 0");
    im->cc_valid = false;
    im->delta_u = delta_u;
    im->delta_v = delta_v;
    return BGI_OK;
}

int bgi_get_image_wcs(const bgi_imager *im, double ra_deg, double dec_deg, bgi_image_wcs *out) {
    if (!im || !out) return set_error(BGI_ERR_INVALID, "get_image_wcs: bad arguments");
    if (im->n_ant == 0 || !(im->u_max > 0) || !(im->v_max > 0))
        return set_error(BGI_ERR_STATE, "get_image_wcs: no array state with u_max, v_max > 0");
    // src/gpu/pacer_imager_hip.cpp:113-115: (1/(osf*u_max))*(180/pi), u_max in metres
    const double osf = (double)im->cfg.oversampling_factor;
    const double rad2deg = 180.00 / 3.14159265358979323846;
    out->ra_deg = ra_deg;
    out->dec_deg = dec_deg;
    out->pixscale_ra_deg = (1.00 / (osf * im->u_max)) * rad2deg;
    out->pixscale_dec_deg = (1.00 / (osf * im->v_max)) * rad2deg;
    return BGI_OK;
}

int bgi_get_uv_cell(const bgi_imager *im, double *delta_u, double *delta_v, double *u_max,
                    double *v_max) {
    if (!im) return set_error(BGI_ERR_INVALID, "get_uv_cell: null handle");
    if (im->n_ant == 0) return set_error(BGI_ERR_STATE, "get_uv_cell: array not set");
    if (delta_u) *delta_u = im->delta_u;
    if (delta_v) *delta_v = im->delta_v;
    if (u_max) *u_max = im->u_max;
    if (v_max) *v_max = im->v_max;
    return BGI_OK;
}

// Rounding u_max * nu_max / (c * delta_u) (half away from zero) reaches at most its floor + 1;
// one more pixel of margin covers the FP64 error of the quotient.  N/2 (no pruning) when the
// bound reaches the half plane's edge, where the cell indices wrap.
int bgi_uv_extent(double u_max, double v_max, double delta_u, double delta_v, double freq_max_hz,
                  int n_pixels, int *ext_u, int *ext_v) {
    if (!ext_u || !ext_v || n_pixels < 2 || !(delta_u > 0) || !(delta_v > 0) || !(u_max >= 0) ||
        !(v_max >= 0) || !(freq_max_hz >= 0))
        return set_error(BGI_ERR_INVALID, "uv_extent: bad arguments");
    const int h = n_pixels / 2;
    const double up = u_max * freq_max_hz / (kVelLight * delta_u);
    const double vp = v_max * freq_max_hz / (kVelLight * delta_v);
    *ext_u = up + 2.0 < h ? (int)up + 2 : h;
    *ext_v = vp + 2.0 < h ? (int)vp + 2 : h;
    return BGI_OK;
}

int bgi_get_uv_extent(const bgi_imager *im, int *ext_u, int *ext_v) {
    if (!im || !ext_u || !ext_v) return set_error(BGI_ERR_INVALID, "get_uv_extent: bad arguments");
    if (im->n_ant == 0 || im->n_channels == 0)
        return set_error(BGI_ERR_STATE, "get_uv_extent: set_array and set_frequencies first");
    if (im->half_plane_path()) im->half_plane_extent(ext_u, ext_v);
    else *ext_u = *ext_v = im->cfg.n_pixels / 2;
    return BGI_OK;
}

static int image_checks(bgi_imager *im, int n_intervals, unsigned flags) {
    if (!im) return set_error(BGI_ERR_INVALID, "image: null handle");
    if (im->n_ant == 0 || im->n_channels == 0)
        return set_error(BGI_ERR_STATE, "image: set_array and set_frequencies first");
    if (n_intervals < 1) return set_error(BGI_ERR_INVALID, "image: n_intervals must be >= 1");
    if (im->n_uvw_sets != 1 && im->n_uvw_sets != n_intervals)
        return set_error(BGI_ERR_INVALID, "image: array has %d UVW sets for %d intervals", im->n_uvw_sets, n_intervals);
    if (flags & ~(BGI_APPLY_GEOMETRIC | BGI_APPLY_CABLE | BGI_OUTPUT_REAL | BGI_WEIGHT_UNIFORM))
        return set_error(BGI_ERR_INVALID, "image: unknown flags");
    if (!(im->delta_u > 0) || !(im->delta_v > 0))
        return set_error(BGI_ERR_STATE, "image: u_max/v_max is zero (no unflagged baseline?)");
    return BGI_OK;
}

}  // extern "C"

namespace {

// Per-call set-up on stream s: wave size, grid scratch of the lanes in use (cleared when new or
// left dirty by a failed call), weight counters of every image cleared.
int prepare_call(bgi_imager *im, int n_images, bool half, bool uniform, cudaStream_t s, int *wave_out,
                 int *lanes_out) {
    const int n = im->cfg.n_pixels;
    const size_t npix = (size_t)n * n;
    int wave = im->cfg.max_images_per_wave;
    if (wave == 0) {
        // about 26-32 MiB of grid per lane, so that two lanes' scratch stays resident in the
        // 129 MB L2 (measured best: 16 full-plane or 24 half-plane images at 512^2)
        const size_t per_image = half ? (size_t)n * half_plane_width(n) * sizeof(float2) : npix * sizeof(float2);
        const size_t budget = (size_t)(half ? 26 : 32) << 20;
        wave = (int)std::max<size_t>(1, budget / per_image);
    }
    wave = std::min(wave, n_images);
    const int n_waves = (n_images + wave - 1) / wave;
    const int n_lanes = std::min(n_waves, im->lanes);
    for (int l = 0; l < n_lanes; ++l) {
        bool fresh = false;
        BGI_TRY(im->grid[l].ensure((size_t)wave * npix, "grid scratch", &fresh));
        if (fresh || im->grid_dirty[l]) {
            BGI_TRY(check_cuda(cudaMemsetAsync(im->grid[l].ptr, 0, sizeof(float2) * im->grid[l].cap, s),
                               "grid scratch clear"));
            im->grid_dirty[l] = false;
        }
        if (uniform) {
            BGI_TRY(im->cnt[l].ensure((size_t)wave * npix, "counter scratch", &fresh));
            if (fresh || im->cnt_dirty[l]) {
                BGI_TRY(check_cuda(cudaMemsetAsync(im->cnt[l].ptr, 0, sizeof(float) * im->cnt[l].cap, s),
                                   "counter scratch clear"));
                im->cnt_dirty[l] = false;
            }
        }
        if (im->deterministic)
            BGI_TRY(im->sorted_ws[l].ensure(sorted_workspace_bytes(im->n_baselines, n, wave), "gridding workspace"));
    }
    if (!im->cc_valid) {
        BGI_TRY(im->d_cc.ensure((size_t)im->n_channels, "channel constants"));
        BGI_TRY(launch_channel_consts(im->d_freqs, im->n_channels, im->delta_u, im->delta_v, im->d_cc.ptr, s));
        im->cc_valid = true;
    }
    BGI_TRY(im->wsum.ensure((size_t)n_images * kWsumStride, "weight sums"));
    BGI_TRY(check_cuda(cudaMemsetAsync(im->wsum.ptr, 0, sizeof(unsigned int) * kWsumStride * n_images, s),
                       "weight sums clear"));
    *wave_out = wave;
    *lanes_out = n_lanes;
    return BGI_OK;
}

GridParams block_params(const bgi_imager *im, const float *vis, int n_intervals, unsigned flags,
                        const void *images, int format = BGI_VIS_C64, const float *scales = nullptr) {
    GridParams p{};
    p.vis = vis;
    p.vis_format = format;
    p.vis_scales = scales;
    p.vis_blocks = vis_blocks(im->n_baselines);
    p.u = im->d_u;
    p.v = im->d_v;
    p.w = im->d_w;
    p.dl = im->d_dl;
    p.flags = im->d_flags;
    p.freqs = im->d_freqs;
    p.chan_consts = nullptr;  // set after prepare_call builds the table
    p.du = im->delta_u;
    p.dv = im->delta_v;
    p.min_uv = im->cfg.min_uv;
    p.n_baselines = im->n_baselines;
    p.n_channels = im->n_channels;
    p.n_intervals = n_intervals;
    p.n_uvw_sets = im->n_uvw_sets;
    p.n_pixels = im->cfg.n_pixels;
    p.pol = im->cfg.pol;
    p.counter_mode = -1;
    p.half_width = im->half_plane_path() ? half_plane_width(im->cfg.n_pixels) : 0;
    p.kb_size = im->kb_size;
    p.kb_table = im->kb_table.ptr;
    p.cpt = im->grid_cpt;
    p.aggregate = im->grid_agg;
    // the complex-to-real pass stores pixel pairs: 16 bytes of complex or 8 bytes of real pixels
    if ((reinterpret_cast<uintptr_t>(images) & ((flags & BGI_OUTPUT_REAL) ? 7u : 15u)) != 0) p.half_width = 0;
    // uniform weighting divides cells by their counters: full-plane grids with counter grids
    if (flags & BGI_WEIGHT_UNIFORM) p.half_width = 0;
    p.apply_geom = (flags & BGI_APPLY_GEOMETRIC) ? 1 : 0;
    p.apply_cable = (flags & BGI_APPLY_CABLE) ? 1 : 0;
    return p;
}

// First pixel of image img: complex images are npix float2 apart, real images npix floats.
float2 *image_ptr(float2 *out, int img, size_t npix, bool real) {
    return real ? reinterpret_cast<float2 *>(reinterpret_cast<float *>(out) + (size_t)img * npix) : out + (size_t)img * npix;
}

// Images [img_first, img_first + count) of a block, in waves of `wave` images that alternate on
// streams[0..n_streams) starting at stream *next.  Per wave: gridding into the stream's grid
// scratch, the row pass in place, the column pass into the images (clearing the scratch).
int run_waves(bgi_imager *im, GridParams p, float2 *out, int img_first, int count, int wave,
              cudaStream_t *streams, int n_streams, int *next, bool real, bool uniform) {
    const int n = im->cfg.n_pixels;
    const size_t npix = (size_t)n * n;
    for (int img0 = img_first; img0 < img_first + count; img0 += wave) {
        const int l = *next;
        *next = (*next + 1) % n_streams;
        cudaStream_t ls = streams[l];
        const int cnt = std::min(wave, img_first + count - img0);
        TraceRange trace("wave");
        float2 *grid = im->grid[l].ptr;
        const size_t need = (size_t)cnt * (p.half_width > 0 ? (size_t)n * p.half_width : npix);
        if (need > im->grid[l].cap) return set_error(BGI_ERR_STATE, "grid scratch too small for a wave");
        unsigned int *ws = im->wsum.ptr + (size_t)img0 * kWsumStride;
        p.grids = grid;
        p.img_begin = img0;
        p.img_count = cnt;
        p.img_base = img0;
        p.wsum = ws;  // indexed img - img_base
        im->grid_dirty[l] = true;
        if (uniform) {
            if ((size_t)cnt * npix > im->cnt[l].cap) return set_error(BGI_ERR_STATE, "counter scratch too small for a wave");
            p.counters = im->cnt[l].ptr;
            p.counter_mode = BGI_COUNTERS_PER_IMAGE;
            p.counter_base = img0;
            im->cnt_dirty[l] = true;
        }
        BGI_TRY(im->mark(ls));
        if (im->deterministic) {
            p.grids_zero = 1;  // the wave scratch is zero between waves
            BGI_TRY(launch_gridding_sorted(p, im->sorted_ws[l].ptr, im->sorted_ws[l].cap, ls));
        }
        else
            BGI_TRY(launch_gridding(p, ls));
        if (uniform)  // weighting "U": cells divided by their counters, counters cleared
            BGI_TRY(launch_uniform_weighting(grid, im->cnt[l].ptr, (long long)cnt * (long long)npix, true, ls));
        BGI_TRY(im->mark(ls));
        if (p.half_width > 0) {
            int eu, ev;
            im->half_plane_extent(&eu, &ev);
            BGI_TRY(launch_fft_cols_half(grid, n, cnt, eu, ev, ls, im->col_radix));  // in place, rows shifted
            BGI_TRY(im->mark(ls));
            BGI_TRY(launch_c2r_rows(grid, image_ptr(out, img0, npix, real), n, cnt, ws, eu, ls, real,
                                    im->fft_mode == BGI_FFT_TENSOR_SPLIT16));  // clears the scratch
        } else {
            BGI_TRY(launch_fft_rows(grid, grid, n, cnt, false, ls));  // in place in the scratch
            BGI_TRY(im->mark(ls));
            BGI_TRY(launch_fft_cols_to(grid, image_ptr(out, img0, npix, real), n, cnt, ws, true, ls, real));  // clears the scratch
        }
        BGI_TRY(im->mark(ls));
        im->grid_dirty[l] = false;
        if (uniform) im->cnt_dirty[l] = false;
    }
    return BGI_OK;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

int image_impl(bgi_imager *im, int format, const void *data, const float *scales, int n_intervals, unsigned flags,
               float *images, void *stream) {
    TraceRange trace("bgi_image");
    BGI_TRY(image_checks(im, n_intervals, flags));
    const float *vis = static_cast<const float *>(data);
    if (!vis || !images || (format != BGI_VIS_C64 && !scales)) return set_error(BGI_ERR_INVALID, "image: null buffer");
    if (im->deterministic && im->kb_size > 0)
        return set_error(BGI_ERR_UNSUPPORTED, "image: the ordered gridder has no convolution kernel");
    const uintptr_t need = format == BGI_VIS_C64 ? 15u : 3u;
    if ((reinterpret_cast<uintptr_t>(vis) & need) != 0 || (reinterpret_cast<uintptr_t>(scales) & 3u) != 0 ||
        (reinterpret_cast<uintptr_t>(images) & 7u) != 0)
        return set_error(BGI_ERR_INVALID, "image: visibilities must be 16-byte (complex64) or 4-byte (16-bit) "
                                          "aligned, scales 4-byte and images 8-byte aligned");
    BGI_TRY(im->activate());
    cudaStream_t s = as_stream(stream);
    const int n_images = n_intervals * im->n_channels;
    int wave = 0, n_lanes = 0;
    GridParams p = block_params(im, vis, n_intervals, flags, images, format, scales);
    const bool uniform = (flags & BGI_WEIGHT_UNIFORM) != 0;
    BGI_TRY(prepare_call(im, n_images, p.half_width > 0, uniform, s, &wave, &n_lanes));
    p.chan_consts = im->d_cc.ptr;
    cudaStream_t streams[bgi_imager::kLanes];
    std::fill(streams, streams + bgi_imager::kLanes, s);
    if (n_lanes > 1) {
        BGI_TRY(im->ensure_lanes());
        BGI_TRY(check_cuda(cudaEventRecord(im->ev_fork, s), "fork record"));
        for (int l = 0; l < n_lanes; ++l) {
            streams[l] = im->lane[l];
            BGI_TRY(check_cuda(cudaStreamWaitEvent(im->lane[l], im->ev_fork, 0), "fork wait"));
        }
    }
    int next = 0;
    BGI_TRY(run_waves(im, p, reinterpret_cast<float2 *>(images), 0,
                      n_images, wave, streams, n_lanes, &next, (flags & BGI_OUTPUT_REAL) != 0, uniform));
    if (n_lanes > 1) {
        for (int l = 0; l < n_lanes; ++l) {
            BGI_TRY(check_cuda(cudaEventRecord(im->ev_join[l], im->lane[l]), "join record"));
            BGI_TRY(check_cuda(cudaStreamWaitEvent(s, im->ev_join[l], 0), "join wait"));
        }
    }
    im->last_images = n_images;
    return BGI_OK;
}

}  // namespace

namespace {
int image_replayed(bgi_imager *im, int format, const void *data, const float *scales, int n_intervals, unsigned flags,
                   float *images, void *stream);

// Records enqueue(stream) -- the stream work of one call, whose scratch an earlier run of the
// same call has sized -- into an executable graph on the handle's capture stream (nothing
// runs).  On failure *exec is null, the handle's scratch is marked for clearing and the CUDA
// error state is reset.
template <class F>
int record_call(bgi_imager *im, F &&enqueue, cudaGraphExec_t *exec) {
    *exec = nullptr;
    int st = BGI_OK;
    if (!im->cap_stream) st = check_cuda(cudaStreamCreateWithFlags(&im->cap_stream, cudaStreamNonBlocking), "capture stream");
    cudaGraph_t g = nullptr;
    if (!st) st = check_cuda(cudaStreamBeginCapture(im->cap_stream, cudaStreamCaptureModeThreadLocal), "image capture");
    if (!st) {
        const int issued = enqueue(im->cap_stream);
        const int ended = check_cuda(cudaStreamEndCapture(im->cap_stream, &g), "image end capture");
        st = issued ? issued : ended;
    }
    if (!st) st = check_cuda(cudaGraphInstantiate(exec, g, 0), "image graph instantiate");
    if (g) cudaGraphDestroy(g);
    if (st) {
        if (*exec) cudaGraphExecDestroy(*exec);
        *exec = nullptr;
        cudaGetLastError();
        for (int l = 0; l < bgi_imager::kLanes; ++l) im->grid_dirty[l] = im->cnt_dirty[l] = true;
    }
    return st;
}
}  // namespace

extern "C" {

int bgi_set_replay(bgi_imager *im, int enable) {
    if (!im) return set_error(BGI_ERR_INVALID, "set_replay: null handle");
    im->drop_graph();
    im->replay_enabled = enable != 0;
    return BGI_OK;
}

int bgi_replay_ready(const bgi_imager *im) {
    if (!im) return set_error(BGI_ERR_INVALID, "replay_ready: null handle");
    return im->graph_exec != nullptr ? 1 : 0;
}

int bgi_image(bgi_imager *im, const float *vis, int n_intervals, unsigned flags, float *images, void *stream) {
    return image_replayed(im, BGI_VIS_C64, vis, nullptr, n_intervals, flags, images, stream);
}

int bgi_image_compressed(bgi_imager *im, int format, const void *data, const float *scales, int n_intervals,
                         unsigned flags, float *images, void *stream) {
    if (format != BGI_VIS_S16 && format != BGI_VIS_BF16 && format != BGI_VIS_FP16)
        return set_error(BGI_ERR_INVALID, "image_compressed: bad format %d", format);
    return image_replayed(im, format, data, scales, n_intervals, flags, images, stream);
}

}  // extern "C"

struct bgi_batch {
    int device = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int n_items = 0;
};

namespace {

// Issues every item on stream s, in order.  Each item overlaps its own waves on its imager's
// lanes; running different items at once as well would hold several imagers' L2-sized grid
// scratch at the same time and push it out of L2 (measured slower).
int issue_batch(const bgi_batch_item *items, int n_items, cudaStream_t s) {
    for (int i = 0; i < n_items; ++i) {
        const bgi_batch_item &it = items[i];
        BGI_TRY(image_impl(it.imager, it.format, it.data, it.scales, it.n_intervals, it.flags, it.images, s));
    }
    return BGI_OK;
}

}  // namespace

extern "C" {

int bgi_batch_create(const bgi_batch_item *items, int n_items, void *stream, bgi_batch **out) {
    if (!items || n_items < 1 || !out) return set_error(BGI_ERR_INVALID, "batch_create: bad arguments");
    *out = nullptr;
    const int device = items[0].imager ? items[0].imager->cfg.device : -1;
    for (int i = 0; i < n_items; ++i) {
        if (!items[i].imager) return set_error(BGI_ERR_INVALID, "batch_create: item %d has no imager", i);
        if (items[i].imager->cfg.device != device)
            return set_error(BGI_ERR_INVALID, "batch_create: items on different devices");
        if (items[i].imager->timing) return set_error(BGI_ERR_STATE, "batch_create: stage timing is on (item %d)", i);
    }
    // the items' warm-up run may grow an imager's scratch: no replay of its earlier calls
    for (int i = 0; i < n_items; ++i) items[i].imager->drop_graph();
    BGI_TRY(items[0].imager->activate());
    // the items run and are captured on a stream of our own (the legacy default stream cannot
    // be captured), ordered after the caller's stream
    cudaStream_t user = as_stream(stream), s = nullptr;
    BGI_TRY(check_cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "batch stream"));
    cudaEvent_t fork = nullptr;
    int st = check_cuda(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "batch event");
    if (!st) st = check_cuda(cudaEventRecord(fork, user), "batch order");
    if (!st) st = check_cuda(cudaStreamWaitEvent(s, fork, 0), "batch order");
    // one run outside the capture sizes every scratch buffer and builds the channel tables, so
    // that the captured calls allocate nothing
    if (!st) st = issue_batch(items, n_items, s);
    if (!st) st = check_cuda(cudaStreamSynchronize(s), "batch warm-up");
    if (!st) st = check_cuda(cudaGetLastError(), "batch warm-up");
    auto b = std::make_unique<bgi_batch>();
    b->device = device;
    b->n_items = n_items;
    if (!st) st = check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "batch capture");
    if (!st) {
        const int issued = issue_batch(items, n_items, s);
        const int ended = check_cuda(cudaStreamEndCapture(s, &b->graph), "batch end capture");
        st = issued ? issued : ended;
    }
    if (!st) st = check_cuda(cudaGraphInstantiate(&b->exec, b->graph, 0), "batch instantiate");
    if (fork) cudaEventDestroy(fork);
    cudaStreamDestroy(s);
    if (st) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        return st;
    }
    *out = b.release();
    return BGI_OK;
}

int bgi_batch_launch(bgi_batch *b, void *stream) {
    if (!b || !b->exec) return set_error(BGI_ERR_INVALID, "batch_launch: no batch");
    TraceRange trace("bgi_batch_launch");
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != b->device) BGI_TRY(check_cuda(cudaSetDevice(b->device), "cudaSetDevice"));
    return check_cuda(cudaGraphLaunch(b->exec, as_stream(stream)), "batch launch");
}

int bgi_batch_destroy(bgi_batch *b) {
    if (!b) return BGI_OK;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    delete b;
    return BGI_OK;
}

int bgi_set_fft_mode(bgi_imager *im, int mode) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im) return set_error(BGI_ERR_INVALID, "set_fft_mode: null handle");
    if (mode != BGI_FFT_SIMT && mode != BGI_FFT_TENSOR_SPLIT16)
        return set_error(BGI_ERR_INVALID, "set_fft_mode: bad mode %d", mode);
    if (mode == BGI_FFT_TENSOR_SPLIT16 && !c2r_tensor_supported(im->cfg.n_pixels))
        return set_error(BGI_ERR_UNSUPPORTED, "set_fft_mode: no tensor-core stage for image side %d (512 only)",
                         im->cfg.n_pixels);
    im->fft_mode = mode;
    return BGI_OK;
}

int bgi_get_fft_mode(const bgi_imager *im, int *mode) {
    if (!im || !mode) return set_error(BGI_ERR_INVALID, "get_fft_mode: bad arguments");
    *mode = im->fft_mode;
    return BGI_OK;
}

int bgi_set_schedule(bgi_imager *im, int images_per_wave, int lanes) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im || images_per_wave < 0 || lanes < 1 || lanes > bgi_imager::kLanes)
        return set_error(BGI_ERR_INVALID, "set_schedule: wave >= 0 (0 = auto) and 1 <= lanes <= %d", bgi_imager::kLanes);
    im->cfg.max_images_per_wave = images_per_wave;
    im->lanes = lanes;
    return BGI_OK;
}

int bgi_get_schedule(const bgi_imager *im, int *images_per_wave, int *lanes) {
    if (!im || !images_per_wave || !lanes) return set_error(BGI_ERR_INVALID, "get_schedule: bad arguments");
    *images_per_wave = im->cfg.max_images_per_wave;
    *lanes = im->lanes;
    return BGI_OK;
}

int bgi_autotune(bgi_imager *im, int format, const void *data, const float *scales, int n_intervals, unsigned flags,
                 float *images, void *stream, double *best_ms) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    BGI_TRY(image_checks(im, n_intervals, flags));
    if (format < BGI_VIS_C64 || format > BGI_VIS_FP16) return set_error(BGI_ERR_INVALID, "autotune: bad format %d", format);
    BGI_TRY(im->activate());
    cudaStream_t s = as_stream(stream);
    const int n_images = n_intervals * im->n_channels;
    const bool timing = im->timing;
    im->timing = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    BGI_TRY(check_cuda(cudaEventCreate(&e0), "autotune event"));
    int st = check_cuda(cudaEventCreate(&e1), "autotune event");
    // milliseconds per call of the handle's current schedule: one call to size the scratch, then
    // three timed with CUDA events on the stream -- as launches of the call's recorded graph, the
    // form repeated calls take (issued directly where recording fails)
    auto time_current = [&](float *ms, int reps = 3) {
        auto enqueue = [&](cudaStream_t st) {
            return image_impl(im, format, data, scales, n_intervals, flags, images, st);
        };
        int r = enqueue(s);
        cudaGraphExec_t ex = nullptr;
        if (!r) record_call(im, enqueue, &ex);
        if (!r) r = check_cuda(cudaEventRecord(e0, s), "autotune record");
        for (int rep = 0; !r && rep < reps; ++rep)
            r = ex ? check_cuda(cudaGraphLaunch(ex, s), "autotune graph launch") : enqueue(s);
        if (!r) r = check_cuda(cudaEventRecord(e1, s), "autotune record");
        if (!r) r = check_cuda(cudaEventSynchronize(e1), "autotune sync");
        if (ex) {
            if (r) cudaStreamSynchronize(s);  // no launch of it still in flight
            cudaGraphExecDestroy(ex);
        }
        float t = 0.f;
        if (!r) r = check_cuda(cudaEventElapsedTime(&t, e0, e1), "autotune elapsed");
        *ms = t / (float)reps;
        return r;
    };
    // 0: the automatic wave; 1-3 suit the large sides, whose single images fill the GPU
    static const int kWaves[] = {0, 1, 2, 3, 4, 8, 12, 16, 20, 24, 28, 32, 40, 48, 64};
    int best_wave = im->cfg.max_images_per_wave, best_lanes = im->lanes;
    int best_cpt = im->grid_cpt, best_fft = im->fft_mode, best_radix = im->col_radix, best_agg = im->grid_agg;
    float best = 3.4e38f;
    // 1. images per wave x lanes, with the gridding and FFT defaults: every candidate timed over
    // three calls, then the three fastest again over ten calls each (a three-call time of a
    // ~0.5 ms block varies by a few percent, enough to mis-rank neighbouring candidates)
    im->grid_cpt = 0;
    im->fft_mode = BGI_FFT_SIMT;
    im->col_radix = 0;
    im->grid_agg = 0;
    struct Cand {
        float ms;
        int wave, lanes;
    };
    std::vector<Cand> cands;
    for (int wi = 0; !st && wi < (int)(sizeof(kWaves) / sizeof(kWaves[0])); ++wi) {
        if (kWaves[wi] > n_images) break;
        for (int lanes = 1; !st && lanes <= bgi_imager::kLanes; ++lanes) {
            im->cfg.max_images_per_wave = kWaves[wi];
            im->lanes = lanes;
            float ms = 0.f;
            st = time_current(&ms);
            if (!st) cands.push_back({ms, kWaves[wi], lanes});
        }
    }
    std::sort(cands.begin(), cands.end(), [](const Cand &a, const Cand &b) { return a.ms < b.ms; });
    for (size_t c = 0; !st && c < std::min<size_t>(3, cands.size()); ++c) {
        im->cfg.max_images_per_wave = cands[c].wave;
        im->lanes = cands[c].lanes;
        float ms = 0.f;
        st = time_current(&ms, 10);
        if (!st && ms < best) {
            best = ms;
            best_wave = cands[c].wave;
            best_lanes = cands[c].lanes;
            best_cpt = 0;
            best_fft = BGI_FFT_SIMT;
            best_radix = 0;
            best_agg = 0;
        }
    }
    // 2. at the best wave and lanes: gridding images per thread, then the last FFT pass's arithmetic
    im->cfg.max_images_per_wave = best_wave;
    im->lanes = best_lanes;
    for (int cpt : {2, 4, 8}) {
        if (st) break;
        im->grid_cpt = cpt;
        float ms = 0.f;
        st = time_current(&ms, 10);
        if (!st && ms < best) {
            best = ms;
            best_cpt = cpt;
        }
    }
    // warp-aggregated atomics (the looping kernel: half plane, 4 or 8 images per thread); they
    // pay where the array's points crowd few cells
    if (im->half_plane_path()) {
        im->grid_agg = 1;
        for (int cpt : {4, 8}) {
            if (st) break;
            im->grid_cpt = cpt;
            float ms = 0.f;
            st = time_current(&ms, 10);
            if (!st && ms < best) {
                best = ms;
                best_cpt = cpt;
                best_agg = 1;
            }
        }
        im->grid_agg = best_agg;
    }
    im->grid_cpt = best_cpt;
    // 3. the column pass's other compiled radix (half plane)
    const int alt = col_alt_radix(im->cfg.n_pixels);
    if (!st && alt && im->half_plane_path()) {
        im->col_radix = alt;
        float ms = 0.f;
        st = time_current(&ms, 10);
        if (!st && ms < best) {
            best = ms;
            best_radix = alt;
        }
    }
    im->col_radix = best_radix;
    if (!st && c2r_tensor_supported(im->cfg.n_pixels) && im->half_plane_path()) {
        im->fft_mode = BGI_FFT_TENSOR_SPLIT16;
        float ms = 0.f;
        st = time_current(&ms, 10);
        if (!st && ms < best) {
            best = ms;
            best_fft = BGI_FFT_TENSOR_SPLIT16;
        }
    }
    cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    im->timing = timing;
    im->cfg.max_images_per_wave = best_wave;
    im->lanes = best_lanes;
    im->grid_cpt = best_cpt;
    im->fft_mode = best_fft;
    im->col_radix = best_radix;
    im->grid_agg = best_agg;
    if (st) return st;
    // drop the candidates' scratch; the chosen schedule sizes its own on the next call
    BGI_TRY(check_cuda(cudaStreamSynchronize(s), "autotune sync"));
    for (int l = 0; l < bgi_imager::kLanes; ++l) {
        im->grid[l].release();
        im->cnt[l].release();
        im->sorted_ws[l].release();
        im->grid_dirty[l] = false;
    }
    if (best_ms) *best_ms = best;
    return BGI_OK;
}

int bgi_set_column_radix(bgi_imager *im, int radix) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im) return set_error(BGI_ERR_INVALID, "set_column_radix: null handle");
    const int n = im->cfg.n_pixels;
    if (radix != 0 && radix != col_default_radix(n) && radix != col_alt_radix(n))
        return set_error(BGI_ERR_UNSUPPORTED, "set_column_radix: radix %d not compiled for image side %d (%d%s%d)", radix,
                         n, col_default_radix(n), col_alt_radix(n) ? " or " : "", col_alt_radix(n));
    im->col_radix = radix == col_default_radix(n) ? 0 : radix;
    return BGI_OK;
}

int bgi_get_column_radix(const bgi_imager *im, int *radix) {
    if (!im || !radix) return set_error(BGI_ERR_INVALID, "get_column_radix: bad arguments");
    *radix = im->col_radix ? im->col_radix : col_default_radix(im->cfg.n_pixels);
    return BGI_OK;
}

int bgi_set_gridding_images_per_thread(bgi_imager *im, int images_per_thread) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im || (images_per_thread != 0 && images_per_thread != 2 && images_per_thread != 4 && images_per_thread != 8))
        return set_error(BGI_ERR_INVALID, "set_gridding_images_per_thread: 0 (auto), 2, 4 or 8");
    im->grid_cpt = images_per_thread;
    return BGI_OK;
}

int bgi_get_gridding_images_per_thread(const bgi_imager *im, int *images_per_thread) {
    if (!im || !images_per_thread) return set_error(BGI_ERR_INVALID, "get_gridding_images_per_thread: bad arguments");
    *images_per_thread = im->grid_cpt;
    return BGI_OK;
}

int bgi_set_gridding_aggregation(bgi_imager *im, int on) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im || (on != 0 && on != 1)) return set_error(BGI_ERR_INVALID, "set_gridding_aggregation: 0 or 1");
    im->grid_agg = on;
    return BGI_OK;
}

int bgi_get_gridding_aggregation(const bgi_imager *im, int *on) {
    if (!im || !on) return set_error(BGI_ERR_INVALID, "get_gridding_aggregation: bad arguments");
    *on = im->grid_agg;
    return BGI_OK;
}

int bgi_compressed_size(int n_ant, int n_channels, int n_intervals, size_t *data_bytes, size_t *scale_bytes) {
    if (n_ant < 1 || n_channels < 1 || n_intervals < 0 || !data_bytes || !scale_bytes)
        return set_error(BGI_ERR_INVALID, "compressed_size: bad arguments");
    const size_t imgs = (size_t)n_channels * n_intervals;
    const long long nb = baselines_of(n_ant);
    *data_bytes = imgs * 4 * (size_t)nb * sizeof(uint32_t);
    *scale_bytes = imgs * 4 * (size_t)vis_blocks(nb) * sizeof(float);
    return BGI_OK;
}

int bgi_ingest_correlation_matrices(const float *re_xx, const float *im_xx, const float *re_yy, const float *im_yy,
                                    int n_ant, int n_channels, int n_intervals, int format, void *data,
                                    float *scales, void *stream) {
    if (!re_xx || !im_xx || !data || n_ant < 1 || n_ant > 46340 || n_channels < 1 || n_intervals < 0)
        return set_error(BGI_ERR_INVALID, "ingest: bad arguments");
    if ((re_yy == nullptr) != (im_yy == nullptr)) return set_error(BGI_ERR_INVALID, "ingest: YY needs both parts");
    if (format < BGI_VIS_C64 || format > BGI_VIS_FP16) return set_error(BGI_ERR_INVALID, "ingest: bad format %d", format);
    if (format != BGI_VIS_C64 && !scales) return set_error(BGI_ERR_INVALID, "ingest: the 16-bit formats need scales");
    const uintptr_t need = format == BGI_VIS_C64 ? 15u : 3u;
    if ((reinterpret_cast<uintptr_t>(data) & need) || (reinterpret_cast<uintptr_t>(scales) & 3u) ||
        (reinterpret_cast<uintptr_t>(re_xx) & 3u) || (reinterpret_cast<uintptr_t>(im_xx) & 3u))
        return set_error(BGI_ERR_INVALID, "ingest: misaligned buffer");
    return launch_ingest(re_xx, im_xx, re_yy, im_yy, n_ant, (long long)n_channels * n_intervals, format, data, scales,
                         as_stream(stream));
}

int bgi_compress_visibilities(const float *vis, int n_ant, int n_channels, int n_intervals, int format, void *data,
                              float *scales, void *stream) {
    if (!vis || !data || !scales || n_ant < 1 || n_channels < 1 || n_intervals < 0)
        return set_error(BGI_ERR_INVALID, "compress: bad arguments");
    if (format != BGI_VIS_S16 && format != BGI_VIS_BF16 && format != BGI_VIS_FP16)
        return set_error(BGI_ERR_INVALID, "compress: bad format %d", format);
    if (!aligned16(vis) || (reinterpret_cast<uintptr_t>(data) & 3u) != 0 || (reinterpret_cast<uintptr_t>(scales) & 3u) != 0)
        return set_error(BGI_ERR_INVALID, "compress: vis must be 16-byte, data and scales 4-byte aligned");
    return launch_compress(vis, baselines_of(n_ant), (long long)n_channels * n_intervals, format, data, scales,
                           as_stream(stream));
}

}  // extern "C"

namespace {

// Pol planes of a block-scaled block that a pol needs (planes XX=0, XY=1, YX=2, YY=3).
int planes_for(int pol, int out[2]) {
    switch (pol) {
        case BGI_POL_XX: out[0] = 0; return 1;
        case BGI_POL_YY: out[0] = 3; return 1;
        case BGI_POL_I: out[0] = 0, out[1] = 3; return 2;
        default: out[0] = 1, out[1] = 2; return 2;
    }
}

// Host buffers: the block is cut into chunks of whole waves; each chunk's visibilities go up on
// a copy stream (for the block-scaled formats only the pol planes the image needs, and their
// scales), its waves run on the lanes as soon as they have landed, and its images come back on
// a second copy stream as soon as they are done, so uploads, imaging and downloads of
// different chunks overlap.
// mats (optional): host correlation matrices re_xx, im_xx, re_yy, im_yy [T][C][A][A] in place of
// stored visibilities: each chunk's matrices are uploaded and converted on the device
// (launch_ingest, on the upload stream) into the staged visibilities in `format`.
int image_host_enqueue(bgi_imager *im, int format, const void *vis_host, const float *scales_host, int n_intervals,
                       unsigned flags, float *images_host, cudaStream_t s, const float *const *mats) {
    const int n_images = n_intervals * im->n_channels;
    const long long nb = im->n_baselines, nblk = vis_blocks(nb);
    const bool planar = format != BGI_VIS_C64;
    const size_t rec_floats = (size_t)nb * (planar ? 4 : 8);  // one image's stored visibilities
    const size_t sc_floats = planar ? (size_t)4 * nblk : 0;
    const bool real = (flags & BGI_OUTPUT_REAL) != 0;
    const size_t img_floats = (size_t)im->cfg.n_pixels * im->cfg.n_pixels * (real ? 1 : 2);
    BGI_TRY(im->io_vis.ensure(rec_floats * n_images, "image_host vis staging"));
    if (planar) BGI_TRY(im->io_scales.ensure(sc_floats * n_images, "image_host scale staging"));
    BGI_TRY(im->io_img.ensure(img_floats * n_images, "image_host image staging"));
    // correlation matrices: XX always, YY when given and the pol reads it
    const size_t mat_floats = (size_t)im->n_ant * im->n_ant;  // one image's matrix
    const bool with_yy = mats && mats[2] && mats[3] && (im->cfg.pol == BGI_POL_YY || im->cfg.pol == BGI_POL_I);
    const int n_mats = mats ? (with_yy ? 4 : 2) : 0;
    if (mats) BGI_TRY(im->io_mat.ensure(mat_floats * n_images * n_mats, "image_host matrix staging"));
    int wave = 0, n_lanes = 0;
    GridParams p = block_params(im, im->io_vis.ptr, n_intervals, flags, im->io_img.ptr, format,
                                      planar ? im->io_scales.ptr : nullptr);
    const bool uniform = (flags & BGI_WEIGHT_UNIFORM) != 0;
    BGI_TRY(prepare_call(im, n_images, p.half_width > 0, uniform, s, &wave, &n_lanes));
    p.chan_consts = im->d_cc.ptr;
    BGI_TRY(im->ensure_lanes());
    BGI_TRY(im->ensure_copy_streams());
    int planes[2] = {0, 0};
    const int n_planes = planar ? planes_for(im->cfg.pol, planes) : 0;
    // about eight chunks of whole waves
    const int waves_total = (n_images + wave - 1) / wave;
    const int chunk = wave * std::max(1, (waves_total + 7) / 8);
    const int n_chunks = (n_images + chunk - 1) / chunk;
    BGI_TRY(im->ensure_chunk_events(n_chunks));
    BGI_TRY(check_cuda(cudaEventRecord(im->ev_fork, s), "fork record"));
    BGI_TRY(check_cuda(cudaStreamWaitEvent(im->copy_in, im->ev_fork, 0), "fork wait"));
    BGI_TRY(check_cuda(cudaStreamWaitEvent(im->copy_out, im->ev_fork, 0), "fork wait"));
    for (int l = 0; l < n_lanes; ++l)
        BGI_TRY(check_cuda(cudaStreamWaitEvent(im->lane[l], im->ev_fork, 0), "fork wait"));
    int next = 0;
    const float *src = static_cast<const float *>(vis_host);
    for (int c = 0; c < n_chunks; ++c) {
        const int img0 = c * chunk;
        const int cnt = std::min(chunk, n_images - img0);
        if (mats) {
            float *dm[4] = {nullptr, nullptr, nullptr, nullptr};
            for (int q = 0; q < n_mats; ++q) {
                dm[q] = im->io_mat.ptr + mat_floats * ((size_t)q * n_images + img0);
                BGI_TRY(check_cuda(cudaMemcpyAsync(dm[q], mats[q] + mat_floats * img0, sizeof(float) * mat_floats * cnt,
                                                   cudaMemcpyHostToDevice, im->copy_in),
                                   "image_host H2D matrices"));
            }
            BGI_TRY(launch_ingest(dm[0], dm[1], dm[2], dm[3], im->n_ant, cnt, format, im->io_vis.ptr + rec_floats * img0,
                                  planar ? im->io_scales.ptr + sc_floats * img0 : nullptr, im->copy_in));
        } else if (!planar) {
            BGI_TRY(check_cuda(cudaMemcpyAsync(im->io_vis.ptr + rec_floats * img0, src + rec_floats * img0,
                                               sizeof(float) * rec_floats * cnt, cudaMemcpyHostToDevice, im->copy_in),
                               "image_host H2D"));
        } else {
            for (int q = 0; q < n_planes; ++q) {
                const size_t off = rec_floats * img0 + (size_t)planes[q] * nb;
                BGI_TRY(check_cuda(cudaMemcpy2DAsync(im->io_vis.ptr + off, sizeof(float) * rec_floats, src + off,
                                                     sizeof(float) * rec_floats, sizeof(float) * nb, cnt,
                                                     cudaMemcpyHostToDevice, im->copy_in),
                                   "image_host H2D planes"));
                const size_t soff = sc_floats * img0 + (size_t)planes[q] * nblk;
                BGI_TRY(check_cuda(cudaMemcpy2DAsync(im->io_scales.ptr + soff, sizeof(float) * sc_floats,
                                                     scales_host + soff, sizeof(float) * sc_floats,
                                                     sizeof(float) * nblk, cnt, cudaMemcpyHostToDevice, im->copy_in),
                                   "image_host H2D scales"));
            }
        }
        BGI_TRY(check_cuda(cudaEventRecord(im->ev_in[c], im->copy_in), "chunk in record"));
        for (int l = 0; l < n_lanes; ++l)
            BGI_TRY(check_cuda(cudaStreamWaitEvent(im->lane[l], im->ev_in[c], 0), "chunk in wait"));
        BGI_TRY(run_waves(im, p, reinterpret_cast<float2 *>(im->io_img.ptr), img0, cnt, wave, im->lane, n_lanes,
                          &next, real, uniform));
        for (int l = 0; l < n_lanes; ++l) {
            BGI_TRY(check_cuda(cudaEventRecord(im->ev_done[c * bgi_imager::kLanes + l], im->lane[l]), "chunk done"));
            BGI_TRY(check_cuda(cudaStreamWaitEvent(im->copy_out, im->ev_done[c * bgi_imager::kLanes + l], 0),
                               "chunk done wait"));
        }
        BGI_TRY(check_cuda(cudaMemcpyAsync(images_host + img_floats * img0, im->io_img.ptr + img_floats * img0,
                                           sizeof(float) * img_floats * cnt, cudaMemcpyDeviceToHost, im->copy_out),
                           "image_host D2H"));
    }
    BGI_TRY(check_cuda(cudaEventRecord(im->ev_join[0], im->copy_out), "join record"));
    BGI_TRY(check_cuda(cudaStreamWaitEvent(s, im->ev_join[0], 0), "join wait"));
    return BGI_OK;
}

// Whether a host pointer is page-locked (registered with CUDA): copies from pageable memory
// cannot be captured into a graph.
bool pinned(const void *p) {
    if (!p) return true;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

// Runs enqueue(s) -- the stream work of one imaging call -- or, when the same call on the same
// handle state was the last one and has been captured, launches its graph on s.  The second of
// two identical calls in a row is run and then also captured (on the handle's capture stream,
// recorded and not run) for the calls that repeat it.  No replay under stage timing, inside a
// caller's stream capture, or where a capture failed for this call.
template <class F>
int run_replayed(bgi_imager *im, const bgi_imager::CallKey &key, bool capturable, cudaStream_t s, F &&enqueue) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    BGI_TRY(check_cuda(cudaStreamIsCapturing(s, &cs), "capture status"));
    const bool replay = capturable && im->replay_enabled && !im->timing && cs == cudaStreamCaptureStatusNone;
    const bool same = im->have_last && im->last_key == key;
    if (replay && same && im->graph_exec && im->graph_key == key) {
        const int st = check_cuda(cudaGraphLaunch(im->graph_exec, s), "image graph launch");
        if (st) {
            im->drop_graph();
            for (int l = 0; l < bgi_imager::kLanes; ++l) im->grid_dirty[l] = im->cnt_dirty[l] = true;
        }
        return st;
    }
    if (im->graph_exec) {
        cudaGraphExecDestroy(im->graph_exec);
        im->graph_exec = nullptr;
    }
    if (!same) im->replay_refused = false;
    im->last_key = key;
    im->have_last = false;  // set again once this call's work is issued
    BGI_TRY(enqueue(s));
    im->have_last = true;
    if (!replay || !same || im->replay_refused) return BGI_OK;
    // the same call twice in a row: record it for the calls that repeat it
    if (record_call(im, enqueue, &im->graph_exec) != BGI_OK) {
        im->replay_refused = true;  // the call itself has run: keep its result, replay nothing for it
        return BGI_OK;
    }
    im->graph_key = key;
    return BGI_OK;
}

// bgi_image / bgi_image_compressed: image_impl, replayed as a graph while the call repeats.
int image_replayed(bgi_imager *im, int format, const void *data, const float *scales, int n_intervals, unsigned flags,
                   float *images, void *stream) {
    if (!im) return set_error(BGI_ERR_INVALID, "image: null handle");
    BGI_TRY(im->activate());
    bgi_imager::CallKey key;
    key.kind = 0;
    key.format = format;
    key.n_intervals = n_intervals;
    key.flags = flags;
    key.out = images;
    key.in[0] = data;
    key.in[1] = scales;
    return run_replayed(im, key, true, as_stream(stream), [&](cudaStream_t st) {
        return image_impl(im, format, data, scales, n_intervals, flags, images, st);
    });
}

int image_host_impl(bgi_imager *im, int format, const void *vis_host, const float *scales_host, int n_intervals,
                    unsigned flags, float *images_host, void *stream, const float *const *mats = nullptr) {
    TraceRange trace("bgi_image_host");
    BGI_TRY(image_checks(im, n_intervals, flags));
    if (!images_host || (!mats && (!vis_host || (format != BGI_VIS_C64 && !scales_host))) ||
        (mats && (!mats[0] || !mats[1])))
        return set_error(BGI_ERR_INVALID, "image_host: null buffer");
    BGI_TRY(im->activate());
    cudaStream_t s = as_stream(stream);
    bgi_imager::CallKey key;
    key.kind = mats ? 2 : 1;
    key.format = format;
    key.n_intervals = n_intervals;
    key.flags = flags;
    key.out = images_host;
    key.in[0] = vis_host;
    key.in[1] = scales_host;
    bool capturable = pinned(images_host) && pinned(vis_host) && pinned(scales_host);
    for (int q = 0; mats && q < 4; ++q) {
        key.in[1 + q] = mats[q];
        capturable = capturable && pinned(mats[q]);
    }
    if (mats) key.in[0] = nullptr;
    BGI_TRY(run_replayed(im, key, capturable, s, [&](cudaStream_t st) {
        return image_host_enqueue(im, format, vis_host, scales_host, n_intervals, flags, images_host, st, mats);
    }));
    im->last_images = n_intervals * im->n_channels;
    BGI_TRY(check_cuda(cudaStreamSynchronize(s), "image_host sync"));
    unsigned int fault = 0;
    BGI_TRY(read_device_fault(&fault, false));
    if (fault) return set_error(BGI_ERR_CUDA, "image_host: device fault word 0x%x (a bounded wait gave up)", fault);
    return BGI_OK;
}

}  // namespace

extern "C" {

int bgi_image_host(bgi_imager *im, const float *vis_host, int n_intervals, unsigned flags,
                   float *images_host, void *stream) {
    return image_host_impl(im, BGI_VIS_C64, vis_host, nullptr, n_intervals, flags, images_host, stream);
}

int bgi_image_compressed_host(bgi_imager *im, int format, const void *data_host, const float *scales_host,
                              int n_intervals, unsigned flags, float *images_host, void *stream) {
    if (format != BGI_VIS_S16 && format != BGI_VIS_BF16 && format != BGI_VIS_FP16)
        return set_error(BGI_ERR_INVALID, "image_compressed_host: bad format %d", format);
    return image_host_impl(im, format, data_host, scales_host, n_intervals, flags, images_host, stream);
}

int bgi_image_correlation_matrices_host(bgi_imager *im, int format, const float *re_xx, const float *im_xx,
                                        const float *re_yy, const float *im_yy, int n_intervals, unsigned flags,
                                        float *images_host, void *stream) {
    if (format < BGI_VIS_C64 || format > BGI_VIS_FP16)
        return set_error(BGI_ERR_INVALID, "image_correlation_matrices_host: bad format %d", format);
    const float *mats[4] = {re_xx, im_xx, re_yy, im_yy};
    return image_host_impl(im, format, nullptr, nullptr, n_intervals, flags, images_host, stream, mats);
}

int bgi_last_weight_sums(bgi_imager *im, uint32_t *sums_host, int n_images, void *stream) {
    if (!im || !sums_host || n_images < 0) return set_error(BGI_ERR_INVALID, "last_weight_sums: bad arguments");
    if (n_images > im->last_images) return set_error(BGI_ERR_INVALID, "last_weight_sums: last call had %d images", im->last_images);
    BGI_TRY(im->activate());
    cudaStream_t s = as_stream(stream);
    BGI_TRY(check_cuda(cudaMemcpy2DAsync(sums_host, sizeof(uint32_t), im->wsum.ptr,
                                         sizeof(uint32_t) * kWsumStride, sizeof(uint32_t), n_images,
                                         cudaMemcpyDeviceToHost, s), "last_weight_sums copy"));
    return check_cuda(cudaStreamSynchronize(s), "last_weight_sums sync");
}

int bgi_device_fault(int device, unsigned int *fault_bits, int clear) {
    if (!fault_bits) return set_error(BGI_ERR_INVALID, "device_fault: null output");
    int prev = 0;
    BGI_TRY(check_cuda(cudaGetDevice(&prev), "get device"));
    BGI_TRY(check_cuda(cudaSetDevice(device), "set device"));
    const int st = read_device_fault(fault_bits, clear != 0);
    cudaSetDevice(prev);
    return st;
}

int bgi_selftest_wait_timeout(int device, void *stream) {
    int prev = 0;
    BGI_TRY(check_cuda(cudaGetDevice(&prev), "get device"));
    BGI_TRY(check_cuda(cudaSetDevice(device), "set device"));
    const int st = launch_wait_timeout_selftest(as_stream(stream));
    cudaSetDevice(prev);
    return st;
}

int bgi_set_gridding_kernel(bgi_imager *im, int kernel_size, int with_sinc) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im) return set_error(BGI_ERR_INVALID, "set_gridding_kernel: null handle");
    if (kernel_size < 0 || kernel_size > kMaxKernel)
        return set_error(BGI_ERR_INVALID, "set_gridding_kernel: kernel size 0..%d", kMaxKernel);
    if (kernel_size == 0) {
        im->kb_size = 0;
        return BGI_OK;
    }
    BGI_TRY(im->activate());
    std::vector<float> table;
    kb_tables(kernel_size, with_sinc != 0, table);
    BGI_TRY(im->kb_table.ensure(table.size(), "kb table"));
    BGI_TRY(check_cuda(cudaMemcpy(im->kb_table.ptr, table.data(), sizeof(float) * table.size(), cudaMemcpyHostToDevice),
                       "kb table upload"));
    im->kb_size = kernel_size;
    return BGI_OK;
}

int bgi_gridding_kb_gpu(const float *vis, int n_ant, int n_channels, int n_intervals, const float *u, const float *v,
                        int n_uvw_sets, const int *baseline_flags, const double *freqs_hz, double delta_u,
                        double delta_v, int n_pixels, double min_uv, int pol, int counter_mode, float *counters,
                        float *grids, int kernel_size, int with_sinc, void *stream) {
    if (kernel_size < 1 || kernel_size > kMaxKernel)
        return set_error(BGI_ERR_INVALID, "gridding_kb: kernel size 1..%d", kMaxKernel);
    GridParams p;
    BGI_TRY(gridding_params("gridding_kb", vis, n_ant, n_channels, n_intervals, u, v, n_uvw_sets, baseline_flags,
                            freqs_hz, delta_u, delta_v, n_pixels, min_uv, pol, counter_mode, counters, grids, &p));
    std::vector<float> table;
    kb_tables(kernel_size, with_sinc != 0, table);
    return launch_gridding_kb_free(p, table, kernel_size, as_stream(stream));
}

int bgi_set_deterministic(bgi_imager *im, int enable) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im) return set_error(BGI_ERR_INVALID, "set_deterministic: null handle");
    im->deterministic = enable != 0;
    return BGI_OK;
}

int bgi_set_stage_timing(bgi_imager *im, int enable) {
    if (im) im->drop_graph();  // the handle changes: no replay of an earlier call
    if (!im) return set_error(BGI_ERR_INVALID, "set_stage_timing: null handle");
    im->timing = enable != 0;
    im->ev_used = 0;
    return BGI_OK;
}

int bgi_get_stage_times(bgi_imager *im, double ms[3], int64_t launches[3]) {
    if (!im || !ms || !launches) return set_error(BGI_ERR_INVALID, "get_stage_times: bad arguments");
    BGI_TRY(im->activate());
    for (int k = 0; k < 3; ++k) {
        ms[k] = 0.0;
        launches[k] = 0;
    }
    for (size_t q = 0; q + 3 < im->ev_used; q += 4) {
        BGI_TRY(check_cuda(cudaEventSynchronize(im->ev_pool[q + 3]), "stage timing sync"));
        for (int k = 0; k < 3; ++k) {
            float t = 0.f;
            BGI_TRY(check_cuda(cudaEventElapsedTime(&t, im->ev_pool[q + k], im->ev_pool[q + k + 1]),
                               "stage timing elapsed"));
            ms[k] += t;
            launches[k] += 1;
        }
    }
    im->ev_used = 0;
    return BGI_OK;
}

}  // extern "C"
