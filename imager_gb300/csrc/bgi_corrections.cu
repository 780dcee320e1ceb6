// Phase corrections in place on 4-pol visibility records (the reference's
// apply_geometric_corrections / apply_cable_corrections, src/gpu/corrections_gpu.cpp:7-72).
//
// One thread per 32-byte record: two 16-byte streaming loads, one delay phasor, four complex
// rotations, two 16-byte stores.  The phase turns = delay * nu/c is reduced to [-0.5, 0.5] in
// FP64 and its sine/cosine taken in FP32; the reference evaluates sincos in FP64 four times
// per record.  HBM-bound: 64 bytes moved per record.
#include "bgi_internal.h"

namespace bgi {
namespace {

// Antenna pair of a triangular baseline index, in integers (the reference's
// (unsigned)(-0.5 + sqrt(0.25 + 2b)) gives the same pair for every b below 2^31).
__device__ __forceinline__ void baseline_antennas(unsigned b, unsigned &a1, unsigned &a2) {
    unsigned i = (unsigned)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);
    while ((unsigned long long)i * (i + 1) / 2 > b) --i;
    while ((unsigned long long)(i + 1) * (i + 2) / 2 <= b) ++i;
    a1 = i;
    a2 = b - (unsigned)((unsigned long long)i * (i + 1) / 2);
}

template <bool CABLE>
__global__ void __launch_bounds__(256) correct_kernel(float4 *vis, unsigned n_baselines,
                                                      int n_channels, int n_images,
                                                      const float *w, int n_uvw_sets,
                                                      const double *cable,
                                                      const double *freqs) {
    const unsigned b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_baselines) return;
    double delay;
    if (CABLE) {
        unsigned a1, a2;
        baseline_antennas(b, a1, a2);
        delay = -(cable[a2] - cable[a1]);
    }
    for (int img = blockIdx.y; img < n_images; img += gridDim.y) {
        const int ch = img % n_channels;
        if (!CABLE) {
            const int set = n_uvw_sets > 1 ? img / n_channels : 0;
            delay = (double)w[(size_t)set * n_baselines + b];
        }
        const float2 p = phasor(delay, freqs[ch] * (1.0 / kVelLight));
        float4 *rec = vis + ((size_t)img * n_baselines + b) * 2;
        float4 lo = ld_stream_f4(rec), hi = ld_stream_f4(rec + 1);
        float2 a = rotate(make_float2(lo.x, lo.y), p), c = rotate(make_float2(lo.z, lo.w), p);
        float2 d = rotate(make_float2(hi.x, hi.y), p), e = rotate(make_float2(hi.z, hi.w), p);
        __stcs(rec, make_float4(a.x, a.y, c.x, c.y));
        __stcs(rec + 1, make_float4(d.x, d.y, e.x, e.y));
    }
}

dim3 corr_grid(unsigned nb, int n_images) {
    unsigned bx = (nb + 255) / 256;
    unsigned by = (unsigned)(n_images < 65535 ? n_images : 65535);
    return dim3(bx, by);
}

}  // namespace

int launch_geometric(float *vis, int n_ant, int n_channels, int n_intervals, const float *w,
                     int n_uvw_sets, const double *freqs, cudaStream_t s) {
    const unsigned nb = (unsigned)((long long)n_ant * (n_ant + 1) / 2);
    const int n_images = n_channels * n_intervals;
    if (nb == 0 || n_images == 0) return BGI_OK;
    correct_kernel<false><<<corr_grid(nb, n_images), 256, 0, s>>>(
        reinterpret_cast<float4 *>(vis), nb, n_channels, n_images, w, n_uvw_sets, nullptr, freqs);
    return check_launch("apply_geometric_corrections");
}

int launch_cable(float *vis, int n_ant, int n_channels, int n_intervals, const double *cable,
                 const double *freqs, cudaStream_t s) {
    const unsigned nb = (unsigned)((long long)n_ant * (n_ant + 1) / 2);
    const int n_images = n_channels * n_intervals;
    if (nb == 0 || n_images == 0) return BGI_OK;
    correct_kernel<true><<<corr_grid(nb, n_images), 256, 0, s>>>(
        reinterpret_cast<float4 *>(vis), nb, n_channels, n_images, nullptr, 1, cable, freqs);
    return check_launch("apply_cable_lengths_corrections");
}

}  // namespace bgi
