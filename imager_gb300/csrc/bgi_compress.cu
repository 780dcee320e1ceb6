// Block-scaled 16-bit visibility storage: complex64 records -> pol planes of 16-bit complex
// values with one FP32 scale per 128 baselines of a plane (the format is stated in
// blink_imager_gb300.h, enum bgi_vis_format).
//
// One warp per (image, block of 128 baselines): lane l holds baselines b0 + l + 32j (j < 4),
// all four pols of each read as the two 16-byte halves of its 32-byte record, so one pass
// reads every record once; warp max-reductions give the four blocks' scales, and each plane
// is written as 32 consecutive 4-byte values per j.  HBM-bound: 32 B read and 16 B written
// per baseline and image.
#include <cuda_bf16.h>

#include "bgi_internal.h"

namespace bgi {
namespace {

constexpr int kWarps = 8;

__device__ __forceinline__ bool valid_component(float x) { return !isnan(x) && fabsf(x) < kMaxVis; }

template <int FMT>
__device__ __forceinline__ uint32_t encode(float x, float scale) {
    if (FMT == BGI_VIS_S16) {
        if (!valid_component(x)) return 0x8000u;
        if (scale == 0.0f) return 0u;
        int q = __float2int_rn(__fdiv_rn(x, scale));
        q = max(-32767, min(32767, q));
        return (uint32_t)(uint16_t)(int16_t)q;
    } else if (FMT == BGI_VIS_BF16) {
        if (!valid_component(x)) return 0x7FC0u;
        return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(__fdiv_rn(x, scale)));
    } else {
        if (!valid_component(x)) return 0x7E00u;
        return (uint32_t)__half_as_ushort(__float2half_rn(__fdiv_rn(x, scale)));
    }
}

// Sources of the four pols of baseline b of image img, as (XX, XY) and (YX, YY) float4s.
struct RecordSource {  // complex64 visibility records [img][B][4]
    const float4 *vis;
    long long nb;
    __device__ __forceinline__ void operator()(long long img, long long b, float4 &lo, float4 &hi) const {
        const float4 *rec = vis + (img * nb + b) * 2;
        lo = __ldcs(rec);
        hi = __ldcs(rec + 1);
    }
};

// antenna pair (i >= j) of lower-triangular baseline b = i(i+1)/2 + j
__device__ __forceinline__ void baseline_pair(long long b, int &i, int &j) {
    long long a = (long long)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);  // within 1; corrected below
    while (a * (a + 1) / 2 > b) --a;
    while ((a + 1) * (a + 2) / 2 <= b) ++a;
    i = (int)a;
    j = (int)(b - a * (a + 1) / 2);
}

struct MatrixSource {  // correlation matrices [img][n][n] (row = first antenna), XX and optional YY
    const float *re_xx, *im_xx, *re_yy, *im_yy;
    int n;
    __device__ __forceinline__ void operator()(long long img, long long b, float4 &lo, float4 &hi) const {
        int i, j;
        baseline_pair(b, i, j);
        const size_t e = (size_t)img * n * n + (size_t)i * n + j;
        lo = make_float4(__ldcs(re_xx + e), __ldcs(im_xx + e), 0.f, 0.f);
        hi = re_yy ? make_float4(0.f, 0.f, __ldcs(re_yy + e), __ldcs(im_yy + e)) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
};

template <int FMT, class Source>
__global__ void __launch_bounds__(kWarps * 32) compress_kernel(const Source src, long long nb, long long nblk,
                                                               long long n_units, uint32_t *__restrict__ data,
                                                               float *__restrict__ scales) {
    const long long unit = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
    if (unit >= n_units) return;  // whole warps
    const int lane = threadIdx.x & 31;
    const long long img = unit / nblk, k = unit - img * nblk;
    const long long b0 = k * kVisBlock;
    float4 lo[4], hi[4];  // lo = (XX, XY), hi = (YX, YY)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const long long b = b0 + lane + 32 * j;
        lo[j] = hi[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (b < nb) src(img, b, lo[j], hi[j]);
    }
    float m[4] = {0.f, 0.f, 0.f, 0.f};
    auto upd = [](float &mm, float x) {
        if (valid_component(x)) mm = fmaxf(mm, fabsf(x));
    };
#pragma unroll
    for (int j = 0; j < 4; ++j) {  // padding lanes hold zeros, which change no maximum
        upd(m[0], lo[j].x), upd(m[0], lo[j].y);
        upd(m[1], lo[j].z), upd(m[1], lo[j].w);
        upd(m[2], hi[j].x), upd(m[2], hi[j].y);
        upd(m[3], hi[j].z), upd(m[3], hi[j].w);
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) m[p] = fmaxf(m[p], __shfl_xor_sync(0xffffffffu, m[p], off));
    float sc[4];
#pragma unroll
    for (int p = 0; p < 4; ++p)
        sc[p] = FMT == BGI_VIS_S16 ? __fdiv_rn(m[p], 32767.0f) : (m[p] > 0.0f ? m[p] : 1.0f);
    if (lane < 4) {
        const float mine = lane == 0 ? sc[0] : lane == 1 ? sc[1] : lane == 2 ? sc[2] : sc[3];
        scales[(img * 4 + lane) * nblk + k] = mine;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const long long b = b0 + lane + 32 * j;
        if (b >= nb) continue;
        uint32_t *d = data + img * 4 * nb + b;
        __stcs(d, encode<FMT>(lo[j].x, sc[0]) | (encode<FMT>(lo[j].y, sc[0]) << 16));
        __stcs(d + nb, encode<FMT>(lo[j].z, sc[1]) | (encode<FMT>(lo[j].w, sc[1]) << 16));
        __stcs(d + 2 * nb, encode<FMT>(hi[j].x, sc[2]) | (encode<FMT>(hi[j].y, sc[2]) << 16));
        __stcs(d + 3 * nb, encode<FMT>(hi[j].z, sc[3]) | (encode<FMT>(hi[j].w, sc[3]) << 16));
    }
}

// correlation matrices -> complex64 records, one thread per (matrix, baseline)
__global__ void __launch_bounds__(256) ingest_records_kernel(const MatrixSource src, long long nb, long long n_rec,
                                                            float4 *__restrict__ vis) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_rec) return;
    const long long img = q / nb, b = q - img * nb;
    float4 lo, hi;
    src(img, b, lo, hi);
    __stcs(vis + q * 2, lo);
    __stcs(vis + q * 2 + 1, hi);
}

template <class Source>
int launch_encoder(const Source &src, long long n_baselines, long long n_images, int format, void *data,
                   float *scales, cudaStream_t s) {
    const long long nblk = (n_baselines + kVisBlock - 1) / kVisBlock;
    const long long units = n_images * nblk;
    const long long blocks = (units + kWarps - 1) / kWarps;
    if (blocks > 0x7fffffffLL) return set_error(BGI_ERR_UNSUPPORTED, "compress: block too large");
    uint32_t *d = static_cast<uint32_t *>(data);
    switch (format) {
        case BGI_VIS_S16: compress_kernel<BGI_VIS_S16><<<(unsigned)blocks, kWarps * 32, 0, s>>>(src, n_baselines, nblk, units, d, scales); break;
        case BGI_VIS_BF16: compress_kernel<BGI_VIS_BF16><<<(unsigned)blocks, kWarps * 32, 0, s>>>(src, n_baselines, nblk, units, d, scales); break;
        case BGI_VIS_FP16: compress_kernel<BGI_VIS_FP16><<<(unsigned)blocks, kWarps * 32, 0, s>>>(src, n_baselines, nblk, units, d, scales); break;
        default: return set_error(BGI_ERR_INVALID, "compress: bad format %d", format);
    }
    return check_launch("compress");
}

}  // namespace

long long vis_blocks(long long n_baselines) { return (n_baselines + kVisBlock - 1) / kVisBlock; }

int launch_ingest(const float *re_xx, const float *im_xx, const float *re_yy, const float *im_yy, int n_ant,
                  long long n_images, int format, void *data, float *scales, cudaStream_t s) {
    const long long nb = (long long)n_ant * (n_ant + 1) / 2;
    if (n_images <= 0) return BGI_OK;
    const MatrixSource src{re_xx, im_xx, re_yy && im_yy ? re_yy : nullptr, re_yy && im_yy ? im_yy : nullptr, n_ant};
    if (format != BGI_VIS_C64) return launch_encoder(src, nb, n_images, format, data, scales, s);
    const long long n_rec = nb * n_images;
    if ((n_rec + 255) / 256 > 0x7fffffffLL) return set_error(BGI_ERR_UNSUPPORTED, "ingest: block too large");
    ingest_records_kernel<<<(unsigned)((n_rec + 255) / 256), 256, 0, s>>>(src, nb, n_rec, static_cast<float4 *>(data));
    return check_launch("ingest");
}

int launch_compress(const float *vis, long long n_baselines, long long n_images, int format, void *data,
                    float *scales, cudaStream_t s) {
    if (n_images <= 0 || n_baselines <= 0) return BGI_OK;
    return launch_encoder(RecordSource{reinterpret_cast<const float4 *>(vis), n_baselines}, n_baselines, n_images,
                          format, data, scales, s);
}

}  // namespace bgi
