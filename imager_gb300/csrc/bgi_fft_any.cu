// Inverse 2D FFT for image sides that are not powers of two (and sides below 16).  The reference
// images any side N through cuFFT / FFTW (src/gpu/pacer_imager_hip.cpp:83-95,
// src/pacer_imager.cpp:145-156); its in-repo EDA2 template is imaged at N = 180.  The
// power-of-two kernels of bgi_fft.cu keep their compile-time shapes; this file takes every other
// side up to 4096 with a runtime plan.
//
// Each 1D transform is a mixed-radix Stockham autosort FFT (the same formulation as the
// power-of-two passes, with the radix chosen per pass): N = r_0 r_1 ... r_{k-1}, pass p with radix
// R and Ns = r_0 ... r_{p-1} reads a[m] = x[j + m N/R] (m < R), multiplies by exp(+2 pi i m k / (Ns R))
// with k = j mod Ns, applies an inverse DFT of size R and writes y[(j - k) R + k + m Ns].  Radices
// 2, 3, 4, 5 and 8 are butterflies in registers; any other prime factor p is a direct sum per
// output (p multiply-adds, with the pass twiddle folded into the DFT twiddle so each term takes one
// complex multiply).  Twiddles exp(+2 pi i q / N), q < N, are one table per device and side,
// computed in double on the host and rounded to float.
//
// A block holds `lines` transforms (rows, or adjacent columns of one image) in shared memory with
// two buffers per line, loads them coalesced, runs the passes between block barriers and stores
// them.  Lines are N | 1 elements apart (an odd stride: adjacent lines start on different banks,
// so the column loads, which step across lines, do not conflict).  The column pass can apply the
// fftshift and the 1/sum(weights) normalisation in its stores (the reference's fftshift by half
// swaps, src/pacer_imager.cpp:110-128, for odd sides too: x < N/2 swaps with x + ceil(N/2), the
// middle element of an odd side stays), clear its source behind the loads, and store real parts
// only.
#include <cmath>
#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "bgi_internal.h"

namespace bgi {
namespace {

constexpr int kAnyMaxPasses = 24;
constexpr int kAnyThreads = 256;
constexpr size_t kAnySmemBudget = 64 * 1024;  // bytes of line buffers per block

struct AnyPlan {
    int n;
    int n_pass;
    int radix[kAnyMaxPasses];
    const float2 *tw;  // exp(+2 pi i q / n), q < n
};

int line_stride(int n) { return n | 1; }

int lines_per_block(int n) {
    const size_t per_line = 2 * sizeof(float2) * (size_t)line_stride(n);
    const int l = (int)(kAnySmemBudget / per_line);
    return std::max(1, std::min(l, 32));
}

size_t any_smem_bytes(int n, int lines) { return 2 * sizeof(float2) * (size_t)lines * line_stride(n); }

// Radices for n, in pass order: eights, fours and a two for the power-of-two part, then threes,
// fives and the remaining primes in increasing order.
int factorize(int n, int *radix) {
    int np = 0;
    while (n % 8 == 0 && np < kAnyMaxPasses) { radix[np++] = 8; n /= 8; }
    while (n % 4 == 0 && np < kAnyMaxPasses) { radix[np++] = 4; n /= 4; }
    while (n % 2 == 0 && np < kAnyMaxPasses) { radix[np++] = 2; n /= 2; }
    for (int p = 3; n > 1 && np < kAnyMaxPasses; p += 2) {
        if ((long long)p * p > n) p = n;  // n is prime
        while (n % p == 0 && np < kAnyMaxPasses) { radix[np++] = p; n /= p; }
    }
    return n == 1 ? np : -1;
}

// Twiddle tables, one per (device, side), kept for the life of the process (at most 32 KB each).
std::mutex g_tw_mutex;
std::map<std::pair<int, int>, float2 *> g_tw_tables;

int twiddle_table(int n, const float2 **out) {
    int dev = -1;
    int st = check_cuda(cudaGetDevice(&dev), "fft twiddles: cudaGetDevice");
    if (st) return st;
    std::lock_guard<std::mutex> lock(g_tw_mutex);
    auto it = g_tw_tables.find({dev, n});
    if (it != g_tw_tables.end()) {
        *out = it->second;
        return BGI_OK;
    }
    std::vector<float2> h((size_t)n);
    const double two_pi = 6.283185307179586476925286766559;
    for (int q = 0; q < n; ++q) {
        // reduce to the first half turn with exact integer symmetry: exp(+2 pi i (n - q) / n) is the
        // conjugate of exp(+2 pi i q / n)
        const bool upper = 2 * (long long)q > n;
        const double a = two_pi * (double)(upper ? n - q : q) / (double)n;
        const double c = std::cos(a), s = std::sin(a);
        h[q] = make_float2((float)c, (float)(upper ? -s : s));
    }
    float2 *d = nullptr;
    st = check_cuda(cudaMalloc(reinterpret_cast<void **>(&d), sizeof(float2) * n), "fft twiddle table");
    if (st) return st;
    st = check_cuda(cudaMemcpy(d, h.data(), sizeof(float2) * n, cudaMemcpyHostToDevice), "fft twiddle table copy");
    if (st) {
        cudaFree(d);
        return st;
    }
    g_tw_tables[{dev, n}] = d;
    *out = d;
    return BGI_OK;
}

int make_plan(int n, AnyPlan *p) {
    p->n = n;
    p->n_pass = factorize(n, p->radix);
    if (p->n_pass < 0) return set_error(BGI_ERR_UNSUPPORTED, "image side %d: too many FFT passes", n);
    return twiddle_table(n, &p->tw);
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
    return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}
__device__ __forceinline__ float2 ci(float2 a) { return make_float2(-a.y, a.x); }   // i * a
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// Inverse DFTs of size R in registers: A_k = sum_m a_m exp(+2 pi i m k / R).
template <int R>
__device__ __forceinline__ void dft_small(float2 *a);

template <>
__device__ __forceinline__ void dft_small<2>(float2 *a) {
    const float2 t = a[1];
    a[1] = csub(a[0], t);
    a[0] = cadd(a[0], t);
}

template <>
__device__ __forceinline__ void dft_small<4>(float2 *a) {
    const float2 s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
    const float2 s13 = cadd(a[1], a[3]), d13 = ci(csub(a[1], a[3]));
    a[0] = cadd(s02, s13);
    a[2] = csub(s02, s13);
    a[1] = cadd(d02, d13);
    a[3] = csub(d02, d13);
}

template <>
__device__ __forceinline__ void dft_small<3>(float2 *a) {
    constexpr float kS3 = 0.866025403784438646763723170753f;  // sin(2 pi / 3)
    const float2 t1 = cadd(a[1], a[2]);
    const float2 t2 = make_float2(a[0].x - 0.5f * t1.x, a[0].y - 0.5f * t1.y);
    const float2 t3 = ci(cscale(csub(a[1], a[2]), kS3));
    a[0] = cadd(a[0], t1);
    a[1] = cadd(t2, t3);
    a[2] = csub(t2, t3);
}

template <>
__device__ __forceinline__ void dft_small<5>(float2 *a) {
    constexpr float c1 = 0.309016994374947424102293417183f;   // cos(2 pi / 5)
    constexpr float c2 = -0.809016994374947424102293417183f;  // cos(4 pi / 5)
    constexpr float s1 = 0.951056516295153572116439333379f;   // sin(2 pi / 5)
    constexpr float s2 = 0.587785252292473129168705954639f;   // sin(4 pi / 5)
    const float2 b1 = cadd(a[1], a[4]), b2 = cadd(a[2], a[3]);
    const float2 d1 = csub(a[1], a[4]), d2 = csub(a[2], a[3]);
    const float2 a0 = a[0];
    const float2 r1 = make_float2(a0.x + c1 * b1.x + c2 * b2.x, a0.y + c1 * b1.y + c2 * b2.y);
    const float2 r2 = make_float2(a0.x + c2 * b1.x + c1 * b2.x, a0.y + c2 * b1.y + c1 * b2.y);
    const float2 i1 = ci(make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y));
    const float2 i2 = ci(make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y));
    a[0] = cadd(a0, cadd(b1, b2));
    a[1] = cadd(r1, i1);
    a[4] = csub(r1, i1);
    a[2] = cadd(r2, i2);
    a[3] = csub(r2, i2);
}

template <>
__device__ __forceinline__ void dft_small<8>(float2 *a) {
    constexpr float h = 0.707106781186547524400844362105f;  // sqrt(1/2)
    float2 e[4] = {a[0], a[2], a[4], a[6]};
    float2 o[4] = {a[1], a[3], a[5], a[7]};
    dft_small<4>(e);
    dft_small<4>(o);
    // o_k * exp(+2 pi i k / 8)
    o[1] = make_float2(h * (o[1].x - o[1].y), h * (o[1].x + o[1].y));
    o[2] = ci(o[2]);
    o[3] = make_float2(-h * (o[3].x + o[3].y), h * (o[3].x - o[3].y));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        a[k] = cadd(e[k], o[k]);
        a[k + 4] = csub(e[k], o[k]);
    }
}

// One pass with a register radix over `lines` transforms: in -> out (shared memory).
template <int R>
__device__ __forceinline__ void pass_reg(const float2 *in, float2 *out, int n, int ns, int stride, int lines,
                                         const float2 *__restrict__ tw) {
    const int m = n / R, step = n / (ns * R);
    for (int it = threadIdx.x; it < lines * m; it += blockDim.x) {
        const int l = it / m, j = it - l * m;
        const float2 *src = in + l * stride;
        float2 *dst = out + l * stride;
        const int k = j % ns;
        float2 a[R];
#pragma unroll
        for (int r = 0; r < R; ++r) a[r] = src[j + r * m];
        if (ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) a[r] = cmul(a[r], __ldg(tw + r * k * step));
        }
        dft_small<R>(a);
        const int base = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[base + r * ns] = a[r];
    }
}

// One pass of any radix R as a direct sum per output: y = sum_r x_r exp(+2 pi i (r k step + r o m) / n)
// for output o of butterfly j, i.e. the pass twiddle and the DFT twiddle in one table entry.
__device__ __forceinline__ void pass_generic(const float2 *in, float2 *out, int n, int R, int ns, int stride,
                                             int lines, const float2 *__restrict__ tw) {
    const int m = n / R, step = n / (ns * R);
    for (int it = threadIdx.x; it < lines * n; it += blockDim.x) {
        const int l = it / n, q = it - l * n;
        const int j = q % m, o = q / m;
        const int k = j % ns;
        const float2 *src = in + l * stride;
        float2 acc = make_float2(0.f, 0.f);
        int ro = 0;  // (r * o) mod R
        for (int r = 0; r < R; ++r) {
            int e = r * k * step + ro * m;  // both terms below n
            if (e >= n) e -= n;
            const float2 w = __ldg(tw + e), x = src[j + r * m];
            acc.x = fmaf(x.x, w.x, fmaf(-x.y, w.y, acc.x));
            acc.y = fmaf(x.x, w.y, fmaf(x.y, w.x, acc.y));
            ro += o;
            if (ro >= R) ro -= R;
        }
        out[l * stride + (j - k) * R + k + o * ns] = acc;
    }
}

// Destination of index p under the reference's fftshift by half swaps.
__device__ __forceinline__ int shift_dest(int p, int n) {
    const int h1 = n / 2, h2 = n - h1;
    return p < h1 ? p + h2 : (p >= h2 ? p - h2 : p);
}

// COLS: lines are adjacent columns of one image (else consecutive rows of the batch).
// SHIFT_NORM (columns only): fftshift both axes and multiply image i by (float)(1/wsum[i]).
// ZERO_SRC: clear the source behind the loads (src != dst).  REAL: dst holds real images.
template <bool COLS, bool SHIFT_NORM, bool ZERO_SRC, bool REAL>
__global__ void __launch_bounds__(kAnyThreads) fft_any_kernel(float2 *src, float2 *dst, const AnyPlan plan, int lines,
                                                              long long total_lines, const unsigned int *wsum) {
    extern __shared__ float2 smem[];
    __shared__ float s_scale;
    const int n = plan.n, stride = n | 1;
    float2 *buf[2] = {smem, smem + (size_t)lines * stride};
    const size_t npix = (size_t)n * n;
    long long img = 0;
    int x0 = 0, nl;
    long long row0 = 0;
    if (COLS) {
        const int bpi = (n + lines - 1) / lines;  // blocks per image
        img = blockIdx.x / bpi;
        x0 = (int)(blockIdx.x % bpi) * lines;
        nl = min(lines, n - x0);
    } else {
        row0 = (long long)blockIdx.x * lines;
        nl = (int)min((long long)lines, total_lines - row0);
    }
    if (SHIFT_NORM && threadIdx.x == 0) s_scale = (float)(1.0 / (double)wsum[(size_t)img * kWsumStride]);
    // load (and clear the source after every load of this thread has been issued)
    const int count = nl * n;
    if (COLS) {
        const float2 *s = src + (size_t)img * npix + x0;
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            const int l = i % nl, r = i / nl;
            buf[0][l * stride + r] = s[(size_t)r * n + l];
        }
        if (ZERO_SRC) {
            float2 *sc = src + (size_t)img * npix + x0;
            for (int i = threadIdx.x; i < count; i += blockDim.x) sc[(size_t)(i / nl) * n + i % nl] = make_float2(0.f, 0.f);
        }
    } else {
        const float2 *s = src + (size_t)row0 * n;
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            const int l = i / n, c = i - l * n;
            buf[0][l * stride + c] = s[i];
        }
        if (ZERO_SRC) {
            float2 *sc = src + (size_t)row0 * n;
            for (int i = threadIdx.x; i < count; i += blockDim.x) sc[i] = make_float2(0.f, 0.f);
        }
    }
    __syncthreads();
    int cur = 0, ns = 1;
    for (int p = 0; p < plan.n_pass; ++p) {  // the radix is uniform across the block
        const int R = plan.radix[p];
        const float2 *in = buf[cur];
        float2 *out = buf[cur ^ 1];
        switch (R) {
            case 2: pass_reg<2>(in, out, n, ns, stride, nl, plan.tw); break;
            case 3: pass_reg<3>(in, out, n, ns, stride, nl, plan.tw); break;
            case 4: pass_reg<4>(in, out, n, ns, stride, nl, plan.tw); break;
            case 5: pass_reg<5>(in, out, n, ns, stride, nl, plan.tw); break;
            case 8: pass_reg<8>(in, out, n, ns, stride, nl, plan.tw); break;
            default: pass_generic(in, out, n, R, ns, stride, nl, plan.tw); break;
        }
        ns *= R;
        cur ^= 1;
        __syncthreads();
    }
    const float2 *res = buf[cur];
    if (COLS) {
        const float scale = SHIFT_NORM ? s_scale : 1.f;
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            const int l = i % nl, r = i / nl;
            float2 v = res[l * stride + r];
            int y = r, x = x0 + l;
            if (SHIFT_NORM) {
                y = shift_dest(y, n);
                x = shift_dest(x, n);
                v = cscale(v, scale);
            }
            const size_t o = (size_t)img * npix + (size_t)y * n + x;
            if (REAL) __stcs(reinterpret_cast<float *>(dst) + o, v.x);
            else if (SHIFT_NORM) __stcs(dst + o, v);
            else dst[o] = v;
        }
    } else {
        float2 *d = dst + (size_t)row0 * n;
        for (int i = threadIdx.x; i < count; i += blockDim.x) {
            const int l = i / n, c = i - l * n;
            d[i] = res[l * stride + c];
        }
    }
}

template <class K>
int prepare_any(K kernel, size_t smem) {
    if (smem > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return check_cuda(e, "fft (any side) smem attribute");
    }
    return BGI_OK;
}

}  // namespace

bool fft_pow2_size(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }

bool fft_size_supported(int n) { return n >= 1 && n <= 4096; }

int launch_fft_any_rows(const float2 *src, float2 *dst, int n, int n_images, bool zero_src, cudaStream_t s) {
    if (n_images <= 0) return BGI_OK;
    if (!fft_size_supported(n)) return set_error(BGI_ERR_UNSUPPORTED, "image side %d (1..4096)", n);
    if (zero_src && src == dst) return set_error(BGI_ERR_INVALID, "fft rows: clearing the source needs src != dst");
    AnyPlan plan;
    int st = make_plan(n, &plan);
    if (st) return st;
    const int lines = lines_per_block(n);
    const long long total = (long long)n_images * n;
    const long long blocks = (total + lines - 1) / lines;
    if (blocks > 0x7fffffffLL) return set_error(BGI_ERR_UNSUPPORTED, "fft rows: too many rows in one call");
    const size_t smem = any_smem_bytes(n, lines);
    auto k = zero_src ? fft_any_kernel<false, false, true, false> : fft_any_kernel<false, false, false, false>;
    st = prepare_any(k, smem);
    if (st) return st;
    k<<<(unsigned)blocks, kAnyThreads, smem, s>>>(const_cast<float2 *>(src), dst, plan, lines, total, nullptr);
    return check_launch("fft rows (any side)");
}

int launch_fft_any_cols(float2 *src, float2 *dst, int n, int n_images, const unsigned int *wsum, bool zero_src,
                        bool real, cudaStream_t s) {
    if (n_images <= 0) return BGI_OK;
    if (!fft_size_supported(n)) return set_error(BGI_ERR_UNSUPPORTED, "image side %d (1..4096)", n);
    if (zero_src && src == dst) return set_error(BGI_ERR_INVALID, "fft cols: clearing the source needs src != dst");
    // the fftshift moves columns between blocks, so it needs a separate destination
    if (wsum && src == dst) return set_error(BGI_ERR_UNSUPPORTED, "fft cols (any side): shift in place");
    if (real && (!wsum || !zero_src)) return set_error(BGI_ERR_INVALID, "fft cols: real output is the epilogue's");
    AnyPlan plan;
    int st = make_plan(n, &plan);
    if (st) return st;
    const int lines = lines_per_block(n);
    const long long blocks = (long long)n_images * ((n + lines - 1) / lines);
    if (blocks > 0x7fffffffLL) return set_error(BGI_ERR_UNSUPPORTED, "fft cols: too many columns in one call");
    const size_t smem = any_smem_bytes(n, lines);
    auto k = real ? fft_any_kernel<true, true, true, true>
                  : wsum ? (zero_src ? fft_any_kernel<true, true, true, false> : fft_any_kernel<true, true, false, false>)
                         : (zero_src ? fft_any_kernel<true, false, true, false> : fft_any_kernel<true, false, false, false>);
    st = prepare_any(k, smem);
    if (st) return st;
    k<<<(unsigned)blocks, kAnyThreads, smem, s>>>(src, dst, plan, lines, 0, wsum);
    return check_launch("fft cols (any side)");
}

}  // namespace bgi
