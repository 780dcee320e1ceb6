// Batched inverse 2D FFT of our own (replaces gpufftExecC2C(..., BACKWARD) of
// src/gpu/pacer_imager_hip.cpp:83-99) and the image epilogues of src/gpu/gpu_utils.cpp.
//
// The 2D transform is a row pass followed by a column pass.  Each 1D transform of length N
// (power of two) is a Stockham autosort FFT (Govindaraju et al., "High Performance Discrete
// Fourier Transforms on Graphics Processors", SC'08): P = N/R threads each hold R values in
// registers, every pass applies inter-pass twiddles and an in-register radix-R DFT, and passes
// exchange data through shared memory.  The first pass reads x[t + m*P] and the last pass
// writes x[t + m*P'] -- consecutive threads touch consecutive elements -- so both HBM-facing
// passes are coalesced and no separate transpose kernel exists.  Twiddles exp(+2*pi*i*k/N)
// are compile-time tables in device memory (below).
//
//   row pass:    grids -> images rows; in the fused path it also re-zeroes the grid scratch
//                it has read, so the next wave's gridding finds a clean grid.
//   column pass: in place on images; a block owns the column tile at x and its fftshift
//                partner at x + N/2, so shifted stores never race with another block's loads.
//                In the fused path the stores apply the fftshift and the 1/sum(weights)
//                normalisation (src/pacer_imager.cpp:171-179).
//
// The imager's default is the half-plane pair instead (real images of Hermitian grids): a
// column pass over columns 0..N/2 in place, then a complex-to-real row pass into the images.
// Both are pruned to the uv coverage: columns beyond the caller's bound are zero and skipped,
// rows beyond it read as zero without a load.
#include "bgi_async.cuh"
#include "bgi_internal.h"

namespace bgi {
namespace {

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }
__host__ __device__ constexpr int bitrev(int i, int bits) {
    return bits == 0 ? 0 : ((i & 1) << (bits - 1)) | bitrev(i >> 1, bits - 1);
}

// cos(2*pi*j/32) for j = 0..8 (cos(k*pi/16)); the other octants follow by symmetry
__host__ __device__ constexpr float cos32_base(int j) {
    return j == 0 ? 1.0f : j == 1 ? 0.980785280403230449f : j == 2 ? 0.923879532511286756f
         : j == 3 ? 0.831469612302545237f : j == 4 ? 0.707106781186547524f
         : j == 5 ? 0.555570233019602225f : j == 6 ? 0.382683432365089772f
         : j == 7 ? 0.195090322016128268f : 0.0f;
}
__host__ __device__ constexpr float cos32(int j) {
    return (j & 31) <= 8 ? cos32_base(j & 31)
         : (j & 31) <= 16 ? -cos32_base(16 - (j & 31))
         : (j & 31) <= 24 ? -cos32_base((j & 31) - 16)
                          : cos32_base(32 - (j & 31));
}
__host__ __device__ constexpr float sin32(int j) { return cos32(j - 8); }

__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
    return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
}

// a * exp(+2*pi*i*j/32) with compile-time j
template <int J>
__device__ __forceinline__ float2 twiddle32(float2 a) {
    constexpr int j = J & 31;
    if (j == 0) return a;
    if (j == 8) return make_float2(-a.y, a.x);
    if (j == 16) return make_float2(-a.x, -a.y);
    if (j == 24) return make_float2(a.y, -a.x);
    return cmul(a, make_float2(cos32(j), sin32(j)));
}

// Butterflies of one radix-2 DIT stage of length LEN on the bit-reversed register array.
template <int R, int LEN, int K, bool END = (K == LEN / 2)>
struct StageLoop {
    __device__ __forceinline__ static void run(float2 *a, int s) {
        float2 u = a[s + K], v = twiddle32<K * (32 / LEN)>(a[s + K + LEN / 2]);
        a[s + K] = make_float2(u.x + v.x, u.y + v.y);
        a[s + K + LEN / 2] = make_float2(u.x - v.x, u.y - v.y);
        StageLoop<R, LEN, K + 1>::run(a, s);
    }
};
template <int R, int LEN, int K>
struct StageLoop<R, LEN, K, true> {
    __device__ __forceinline__ static void run(float2 *, int) {}
};

template <int R, int LEN, int S, bool END = (S >= R)>
struct Blocks {
    __device__ __forceinline__ static void run(float2 *a) {
        StageLoop<R, LEN, 0>::run(a, S);
        Blocks<R, LEN, S + LEN>::run(a);
    }
};
template <int R, int LEN, int S>
struct Blocks<R, LEN, S, true> {
    __device__ __forceinline__ static void run(float2 *) {}
};

template <int R, int LEN, bool END = (LEN > R)>
struct Stages {
    __device__ __forceinline__ static void run(float2 *a) {
        Blocks<R, LEN, 0>::run(a);
        Stages<R, LEN * 2>::run(a);
    }
};
template <int R, int LEN>
struct Stages<R, LEN, true> {
    __device__ __forceinline__ static void run(float2 *) {}
};

// Bit-reversal permutation of the register array, unrolled at compile time.
template <int R, int I, bool END = (I == R)>
struct BitRevSwap {
    __device__ __forceinline__ static void run(float2 *a) {
        constexpr int J = bitrev(I, ilog2(R));
        if constexpr (I < J) {
            float2 tmp = a[I];
            a[I] = a[J];
            a[J] = tmp;
        }
        BitRevSwap<R, I + 1>::run(a);
    }
};
template <int R, int I>
struct BitRevSwap<R, I, true> {
    __device__ __forceinline__ static void run(float2 *) {}
};

// In-register inverse DFT of size R (2..32): A_k = sum_m a_m exp(+2*pi*i*m*k/R).
template <int R>
__device__ __forceinline__ void dft(float2 *a) {
    BitRevSwap<R, 0>::run(a);
    Stages<R, 2>::run(a);
}

template <int N, int R>
struct FftCfg {
    static constexpr int P = N / R;  // threads per transform
    static constexpr int LOGN = ilog2(N), LOGR = ilog2(R);
    static constexpr int NFULL = LOGN / LOGR;      // radix-R passes
    static constexpr int R2 = 1 << (LOGN % LOGR);  // radix of the final pass (1 = none)
    static constexpr int NPASS = NFULL + (R2 > 1 ? 1 : 0);
    static constexpr int LEN = N + N / R;  // shared elements of one transform, padded
    static_assert(NPASS >= 2, "at least two passes (loads and stores are separated by barriers)");
};

// Shared-memory index with one pad element after every R elements, so that the first pass's
// Stockham writes (stride R between consecutive threads) fall on distinct banks.
template <int LOGR>
__device__ __forceinline__ int pidx(int i) { return i + (i >> LOGR); }

template <bool WARP>
__device__ __forceinline__ void fft_sync() {
    if (WARP) __syncwarp();
    else __syncthreads();
}

// Twiddle tables per pass, laid out [m-1][k] so that consecutive threads (consecutive k) read
// consecutive entries: full pass p >= 1 (Ns = R^p) holds exp(+2*pi*i*m*k/(Ns*R)) for m in
// [1, R), k in [0, Ns); the final radix-R2 pass holds exp(+2*pi*i*m*j/N) for m in [1, R2),
// j in [0, N/R2).
template <int N, int R>
struct TwTables {
    using C = FftCfg<N, R>;
    static constexpr int ns(int p) { return p == 0 ? 1 : R * ns(p - 1); }
    static constexpr int off_full(int p) { return p <= 1 ? 0 : off_full(p - 1) + (R - 1) * ns(p - 1); }
    static constexpr int OFF_REM = off_full(C::NFULL);
    static constexpr int TOTAL = OFF_REM + (C::R2 > 1 ? (C::R2 - 1) * (N / C::R2) : 0);
    static constexpr int SIZE = TOTAL > 0 ? TOTAL : 1;
};

// One 1D inverse transform of length N by P = N/R threads (t = 0..P-1).  sm: this transform's
// LEN shared elements; tw: the pass twiddle tables (TwTables).  gload(i) reads input element i, gstore(i, v) writes
// output element i.  WARP: the P threads of a transform lie in one warp (P <= 32), so passes
// synchronise with __syncwarp; otherwise every thread of the block calls this in lockstep and
// passes use block barriers.  ALIASED: gstore writes into sm, so the final stores wait until
// every thread has read its last inputs.
struct NoClear {
    __device__ __forceinline__ void operator()(int) const {}
};

// gclear(i), when given, runs for every input element after all of this thread's first-pass
// loads have been issued (clearing a source behind the loads without serialising them: a store
// between two loads through possibly aliasing pointers would make each load wait for the last).
// TWS: tw points to a copy of the tables in shared memory (plain loads) instead of global
// memory (read-only cached loads).
template <bool TWS>
__device__ __forceinline__ float2 tw_load(const float2 *tw, int i) {
    if constexpr (TWS) return tw[i];
    else return __ldg(tw + i);
}

// w[m] = w1^m for m = 1..R-1, by squarings and single multiplications (at most log2(R) + 1
// products deep, so a few float roundings from the exact power).
template <int R>
__device__ __forceinline__ void twiddle_powers(float2 w1, float2 *w) {
    w[1] = w1;
#pragma unroll
    for (int m = 2; m < R; ++m) w[m] = (m & 1) ? cmul(w[m - 1], w1) : cmul(w[m / 2], w[m / 2]);
}

// TWPOW: each pass reads only its m = 1 twiddle, exp(+2*pi*i*k/(Ns*R)) (or exp(+2*pi*i*j/N) in the
// final radix-R2 pass), and forms the others as its powers in registers: one table load per pass
// instead of R - 1.
template <int N, int R, bool WARP, bool ALIASED, bool TWS = false, bool TWPOW = false, class GLoad, class GStore,
          class GClear = NoClear>
__device__ __forceinline__ void fft_transform(int t, float2 *sm, const float2 *tw, GLoad gload,
                                              GStore gstore, GClear gclear = GClear()) {
    using C = FftCfg<N, R>;
    using TT = TwTables<N, R>;
    constexpr int P = C::P;
    constexpr int R2 = C::R2;
    constexpr int LR = C::LOGR;
    float2 a[R];
#pragma unroll
    for (int m = 0; m < R; ++m) a[m] = gload(t + m * P);
#pragma unroll
    for (int m = 0; m < R; ++m) gclear(t + m * P);
    int Ns = 1;
    int toff = 0;
#pragma unroll
    for (int p = 0; p < C::NFULL; ++p) {
        const int k = t & (Ns - 1);
        if (p > 0) {
            if constexpr (TWPOW) {
                float2 w[R];
                twiddle_powers<R>(tw_load<TWS>(tw, toff + k), w);
#pragma unroll
                for (int m = 1; m < R; ++m) a[m] = cmul(a[m], w[m]);
            } else {
#pragma unroll
                for (int m = 1; m < R; ++m) a[m] = cmul(a[m], tw_load<TWS>(tw, toff + (m - 1) * Ns + k));
            }
            toff += (R - 1) * Ns;
        }
        dft<R>(a);
        const int base = (t - k) * R + k;
        if (p == C::NPASS - 1) {
            if (ALIASED) fft_sync<WARP>();
#pragma unroll
            for (int m = 0; m < R; ++m) gstore(base + m * Ns, a[m]);
        } else {
            fft_sync<WARP>();
#pragma unroll
            for (int m = 0; m < R; ++m) sm[pidx<LR>(base + m * Ns)] = a[m];
            fft_sync<WARP>();
            if (p + 1 < C::NFULL) {
#pragma unroll
                for (int m = 0; m < R; ++m) a[m] = sm[pidx<LR>(t + m * P)];
            } else {
#pragma unroll
                for (int q = 0; q < R / R2; ++q)
#pragma unroll
                    for (int m = 0; m < R2; ++m) a[q * R2 + m] = sm[pidx<LR>(t + q * P + m * (N / R2))];
            }
        }
        Ns *= R;
    }
    if constexpr (R2 > 1) {
        if (ALIASED) fft_sync<WARP>();
#pragma unroll
        for (int q = 0; q < R / R2; ++q) {
            const int j = t + q * P;
            float2 b[R2];
            if constexpr (TWPOW) {
                float2 w[R2];
                twiddle_powers<R2>(tw_load<TWS>(tw, TT::OFF_REM + j), w);
#pragma unroll
                for (int m = 0; m < R2; ++m) b[m] = m ? cmul(a[q * R2 + m], w[m]) : a[q * R2];
            } else {
#pragma unroll
                for (int m = 0; m < R2; ++m)
                    b[m] = m ? cmul(a[q * R2 + m], tw_load<TWS>(tw, TT::OFF_REM + (m - 1) * (N / R2) + j)) : a[q * R2];
            }
            dft<R2>(b);
#pragma unroll
            for (int m = 0; m < R2; ++m) gstore(j + m * (N / R2), b[m]);
        }
    }
}

// ---- twiddle tables, evaluated at compile time -------------------------------------------
// exp(+2*pi*i*idx/N) for the pass tables is computed by the compiler: the index is reduced to
// the first octant with exact integer arithmetic (symmetries of sine and cosine), and sine and
// cosine of the octant angle (<= pi/4) come from their Taylor series in double precision (the
// terms fall below 1e-20 after 12 orders), then round to float.  The tables live in the
// module's global memory, initialised when the module loads: no set-up launch and no shared
// memory; kernels read them through L1.
struct TwEntry {
    float x, y;
};
constexpr double kPi = 3.14159265358979323846;
constexpr double taylor_sin(double a) {
    double term = a, sum = a;
    for (int n = 1; n < 14; ++n) {
        term *= -a * a / (double)((2 * n) * (2 * n + 1));
        sum += term;
    }
    return sum;
}
constexpr double taylor_cos(double a) {
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 14; ++n) {
        term *= -a * a / (double)((2 * n - 1) * (2 * n));
        sum += term;
    }
    return sum;
}
struct CplxD {
    double x, y;
};
// exp(+2*pi*i*idx/n) in double
constexpr CplxD exp_i_exact(int idx, int n) {
    const int q = n / 4, quad = (idx / q) & 3, k = idx % q;
    const bool swap = k > n / 8;
    const double a = 2.0 * kPi * (double)(swap ? q - k : k) / (double)n;
    double c = taylor_cos(a), s = taylor_sin(a);
    if (swap) {
        const double t = c;
        c = s;
        s = t;
    }
    double x = c, y = s;
    if (quad == 1) { x = -s; y = c; }
    else if (quad == 2) { x = -c; y = -s; }
    else if (quad == 3) { x = s; y = -c; }
    return CplxD{x, y};
}
constexpr TwEntry twiddle_exact(int idx, int n) {
    const CplxD e = exp_i_exact(idx, n);
    return TwEntry{(float)e.x, (float)e.y};
}

// cos(2*pi*j/64) for j = 0..16 as float constants evaluated by the compiler (scalar constexpr
// variables, so device code folds them), and cos64 / sin64 of any j by symmetry: the constants
// c_m = exp(+2*pi*i*m/(2R)) of the complex-to-real pass's z twiddles for radix R <= 32.
#define BGI_COS64(J) constexpr float kCos64_##J = (float)taylor_cos(kPi * (J) / 32.0);
BGI_COS64(1) BGI_COS64(2) BGI_COS64(3) BGI_COS64(4) BGI_COS64(5) BGI_COS64(6) BGI_COS64(7) BGI_COS64(8)
BGI_COS64(9) BGI_COS64(10) BGI_COS64(11) BGI_COS64(12) BGI_COS64(13) BGI_COS64(14) BGI_COS64(15)
#undef BGI_COS64
__host__ __device__ constexpr float cos64_base(int j) {
    return j == 0 ? 1.0f : j == 1 ? kCos64_1 : j == 2 ? kCos64_2 : j == 3 ? kCos64_3 : j == 4 ? kCos64_4
         : j == 5 ? kCos64_5 : j == 6 ? kCos64_6 : j == 7 ? kCos64_7 : j == 8 ? kCos64_8 : j == 9 ? kCos64_9
         : j == 10 ? kCos64_10 : j == 11 ? kCos64_11 : j == 12 ? kCos64_12 : j == 13 ? kCos64_13
         : j == 14 ? kCos64_14 : j == 15 ? kCos64_15 : 0.0f;
}
__host__ __device__ constexpr float cos64(int j) {
    return (j & 63) <= 16 ? cos64_base(j & 63)
         : (j & 63) <= 32 ? -cos64_base(32 - (j & 63))
         : (j & 63) <= 48 ? -cos64_base((j & 63) - 32)
                          : cos64_base(64 - (j & 63));
}
__host__ __device__ constexpr float sin64(int j) { return cos64(j - 16); }

template <int N, int R>
struct alignas(16) TwData {  // 16-byte aligned: bulk copies stage it in shared memory
    TwEntry v[TwTables<N, R>::SIZE];
};

template <int N, int R>
constexpr TwData<N, R> make_twiddles() {
    using C = FftCfg<N, R>;
    using TT = TwTables<N, R>;
    TwData<N, R> d{};
    for (int p = 1; p < C::NFULL; ++p) {
        const int ns = TT::ns(p), step = N / (ns * R), base = TT::off_full(p);
        for (int e = 0; e < (R - 1) * ns; ++e) d.v[base + e] = twiddle_exact((e / ns + 1) * (e % ns) * step, N);
    }
    if (C::R2 > 1) {
        const int j_count = N / C::R2;
        for (int e = 0; e < (C::R2 - 1) * j_count; ++e)
            d.v[TT::OFF_REM + e] = twiddle_exact((e / j_count + 1) * (e % j_count), N);
    }
    return d;
}

template <int N, int R>
__device__ const TwData<N, R> g_twiddles = make_twiddles<N, R>();

template <int N, int R>
__device__ __forceinline__ const float2 *twiddles() {
    return reinterpret_cast<const float2 *>(g_twiddles<N, R>.v);
}

// Launch shapes per image side: radix R, warp-synchronous transforms (P <= 32) or block
// barriers, transforms per row-pass block, columns per column-pass block (a tile pair).
template <int N>
struct Shape {
    static constexpr int R = N <= 128 ? 8 : N <= 256 ? 16 : N <= 1024 ? 32 : 16;
    static constexpr int P = N / R;
    static constexpr bool WARP = P <= 32;
    static constexpr int ROWS = WARP ? ((256 / P) < N ? (256 / P) : N) : 256 / P;
};

// Column-pass shape: COLS columns per block (a tile pair), P threads per column, block barriers.
#ifndef COL_THREADS
#define COL_THREADS 256
#endif
template <int N, int RADIX = Shape<N>::R>
struct ColShape {
    static constexpr int R = RADIX;
    static constexpr int P = N / R;
    static constexpr int COLS = (COL_THREADS / P) < 4 ? 4 : ((COL_THREADS / P) > N ? N : (COL_THREADS / P));
    static constexpr int MOD = COLS >= 16 ? 1 : 16 / COLS;  // column stride modulo 16 (banks)
    static constexpr int LEN = FftCfg<N, R>::LEN;
    static constexpr int STRIDE = LEN + ((MOD - LEN % 16) + 16) % 16;
};

template <int N, bool ZERO_SRC>
__global__ void __launch_bounds__(Shape<N>::ROWS *Shape<N>::P) fft_rows_kernel(float2 *src, float2 *dst) {
    using S = Shape<N>;
    using C = FftCfg<N, S::R>;
    extern __shared__ float2 smem[];
    float2 *buf = smem;
    const float2 *tw = twiddles<N, S::R>();
    const int slot = threadIdx.x / S::P, t = threadIdx.x % S::P;
    const size_t row = (size_t)blockIdx.x * S::ROWS + slot;
    float2 *s_row = src + row * N;
    float2 *d_row = dst + row * N;
    fft_transform<N, S::R, S::WARP, false>(
        t, buf + slot * C::LEN, tw,
        [&](int i) { return s_row[i]; }, [&](int i, float2 v) { d_row[i] = v; },
        [&](int i) {
            if (ZERO_SRC) s_row[i] = make_float2(0.f, 0.f);
        });
}

// Column pass on a tile pair: columns [x0, x0+CT) and their fftshift partners [x0+N/2, ...).
// Thread c + COLS*t runs point t of column c, so the lanes of a warp cover adjacent columns and
// every global load and store moves whole 32-byte row segments of the tile; the transforms of
// the COLS columns step through their passes together (block barriers).  All loads of the pair
// happen in the first pass, before any store, and no other block touches these columns, so the
// pass may run in place (src == dst) even with the fftshift.  With SHIFT_NORM the stores apply
// the fftshift and multiply by (float)(1/sum(w)); with ZERO_SRC the loads clear src behind them
// (src != dst), and the final stores stream past L2.  With REAL (epilogue only) dst holds real
// images float[N][N] and only the real parts are stored.
template <int N, bool SHIFT_NORM, bool ZERO_SRC, bool REAL = false>
__global__ void __launch_bounds__(ColShape<N>::COLS *ColShape<N>::P) fft_cols_kernel(float2 *src, float2 *dst,
                                                                                    const unsigned int *wsum) {
    static_assert(!REAL || SHIFT_NORM, "real output is written by the epilogue");
    using S = ColShape<N>;
    constexpr int COLS = S::COLS, CT = COLS / 2, TILES = (N / 2) / CT;
    extern __shared__ float2 smem[];
    const float2 *tw = twiddles<N, S::R>();
    const size_t img = blockIdx.x / TILES;
    const int x0 = (blockIdx.x % TILES) * CT;
    const int c = threadIdx.x % COLS, t = threadIdx.x / COLS;
    const int col = c < CT ? x0 + c : N / 2 + x0 + (c - CT);
    float2 *in = src + img * (size_t)N * N;
    float2 *out = dst + img * (size_t)N * N;
    // one FP64 reciprocal per block (its columns are one image's), read after the transform's
    // block barriers
    __shared__ float s_scale;
    if (SHIFT_NORM && threadIdx.x == 0) s_scale = (float)(1.0 / (double)wsum[img * kWsumStride]);
    const int dcol = SHIFT_NORM ? ((col + N / 2) & (N - 1)) : col;
    fft_transform<N, S::R, false, false>(
        t, smem + c * S::STRIDE, tw,
        [&](int i) { return in[(size_t)i * N + col]; },
        [&](int i, float2 v) {
            int r = i;
            if (SHIFT_NORM) {
                r = (i + N / 2) & (N - 1);
                v = make_float2(v.x * s_scale, v.y * s_scale);
            }
            if (REAL)
                __stcs(reinterpret_cast<float *>(dst) + img * (size_t)N * N + (size_t)r * N + dcol, v.x);
            else
                __stcs(out + (size_t)r * N + dcol, v);
        },
        [&](int i) {
            if (ZERO_SRC) in[(size_t)i * N + col] = make_float2(0.f, 0.f);
        });
}

// ---- half-plane path: real images of Hermitian grids ---------------------------------------
// A grid that holds every visibility and its conjugate at the mirrored cell is Hermitian, so its
// inverse transform is real.  Only columns u = 0..N/2 are kept (width W = N/2 + one column tile,
// the padding columns stay zero); the column pass transforms those along v, and each row is
// then finished by a complex-to-real transform of length N built on a complex FFT of length N/2:
// with M = N/2 and w = exp(+2*pi*i*k/N), Z[k] = X[k](1 + i w) + conj(X[M-k])(1 - i w) for
// k < M, z = IDFT_M(Z), and the image row is x[2m] = Re z[m], x[2m+1] = Im z[m].

// P[k] = 1 + i exp(+2*pi*i*k/N) = (1 - sin, cos) for k < N/2, in double then rounded
// (compile-time, as the pass tables).  With it Z[k] = X[k](1 + i w) + conj(X[M-k])(1 - i w)
// = 2 conj(b) + P[k] (a - conj(b)) for a = X[k], b = X[M-k], since 1 - i w = 2 - P.
template <int N>
struct alignas(16) ZTwData {
    TwEntry v[N / 2];
};
constexpr TwEntry one_plus_i_twiddle(int k, int n) {
    const CplxD e = exp_i_exact(k, n);
    return TwEntry{(float)(1.0 - e.y), (float)e.x};
}
template <int N>
constexpr ZTwData<N> make_z_twiddles() {
    ZTwData<N> d{};
    for (int k = 0; k < N / 2; ++k) d.v[k] = one_plus_i_twiddle(k, N);
    return d;
}
template <int N>
__device__ const ZTwData<N> g_z_twiddles = make_z_twiddles<N>();

template <int N>
constexpr int half_width_of() {
    static_assert(N / 2 + ColShape<N>::COLS <= N, "half-plane grid wider than the full grid");
    return N / 2 + ColShape<N>::COLS;
}

// Column pass of half-plane grids [img][N][W], in place: tiles of COLS adjacent columns, lanes
// across the columns (coalesced row segments), transforms stepping together (block barriers);
// row y is stored at (y + N/2) mod N, the fftshift of rows.  Pruned by the uv coverage: the
// launch covers the first `tiles` tiles of each image (the columns beyond are zero, and so are
// their transforms), and rows ext_v < y < N - ext_v, which hold no gridded value, read as zero
// without a load.
// RADIX: the column transforms' radix (Shape<N>::R by default; the other compiled radix is
// col_alt_radix(N), picked per handle).  The grid's width W is the default shape's either way.
template <int N, int RADIX = Shape<N>::R>
__global__ void __launch_bounds__(ColShape<N, RADIX>::COLS *ColShape<N, RADIX>::P) fft_cols_half_kernel(float2 *grids,
                                                                                                      int tiles,
                                                                                                      int ext_v) {
    using S = ColShape<N, RADIX>;
    constexpr int COLS = S::COLS, W = half_width_of<N>();
    static_assert(W % COLS == 0, "column tiles cover the half-plane width");
    extern __shared__ float2 smem[];
    const float2 *tw = twiddles<N, S::R>();
    const size_t img = blockIdx.x / tiles;
    const int x0 = (blockIdx.x % tiles) * COLS;
    const int c = threadIdx.x % COLS, t = threadIdx.x / COLS;
    float2 *g = grids + img * (size_t)N * W + x0 + c;
    fft_transform<N, S::R, false, false>(
        t, smem + c * S::STRIDE, tw,
        [&](int i) { return (i <= ext_v || i >= N - ext_v) ? g[(size_t)i * W] : make_float2(0.f, 0.f); },
        [&](int i, float2 v) { g[(size_t)((i + N / 2) & (N - 1)) * W] = v; });
}

// Complex-to-real row pass shape: transforms of length M = N/2.
#ifndef C2R_THREADS
#define C2R_THREADS 128
#endif
#ifndef C2R_MIN_BLOCKS_512
#define C2R_MIN_BLOCKS_512 9
#endif
template <int N>
struct C2RShape {
    static constexpr int M = N / 2;
    static constexpr int R = Shape<M>::R;
    static constexpr int P = M / R;
    static constexpr bool WARP = P <= 32;
    // threads per block: 128 gives more independent blocks (and bulk copies) in flight per SM
    static constexpr int THREADS = P <= 32 ? C2R_THREADS : 256;
    static constexpr int ROWS = WARP ? ((THREADS / P) < N ? (THREADS / P) : N) : (THREADS / P > 0 ? THREADS / P : 1);
    static constexpr int LEN = FftCfg<M, R>::LEN;
    static constexpr int BUF = ((LEN > M + 1 ? LEN : M + 1) + 1) & ~1;
    // resident blocks per SM the registers must allow: at 512^2 nine 128-thread blocks (the
    // shared-memory limit) measured faster than the eight that 60 registers leave
    static constexpr int MIN_BLOCKS = N == 512 ? C2R_MIN_BLOCKS_512 : 1;
};

// Complex-to-real pass: half-plane row y (already at its fftshifted position) -> image row y.
// One thread stages the block's rows in shared memory with bulk asynchronous copies completing
// on an mbarrier, then clears them in the grid with bulk stores from a zero row once they have
// landed.  Only the first copy_bytes of a row (the columns the uv coverage reaches, rounded up
// to 16 bytes; at most N/2 + 1 values rounded up) are copied and cleared: the rest of the row is
// zero in the grid and is zeroed in the row buffer instead.  The first pass forms Z[k] from X[k]
// and X[M-k]; the stores apply the fftshift of columns (x -> (x + N/2) mod N keeps pairs
// 2m, 2m+1 together) and (float)(1/sum(w)), and write each pair of complex pixels (zero
// imaginary parts) as one 16-byte store streaming past L2: two 8-byte stores would each
// half-fill their sectors.  With REAL the images are float [N][N] and each pixel pair is one
// 8-byte store.
template <int N>
constexpr unsigned c2r_row_bytes() {
    return (unsigned)(((N / 2 + 1) * sizeof(float2) + 15) & ~(size_t)15);
}
// bytes of the pass twiddle table and of the z twiddles staged next to the rows
template <int N>
constexpr unsigned c2r_tw_bytes() {
    return (unsigned)(TwTables<N / 2, C2RShape<N>::R>::SIZE * sizeof(float2));
}
template <int N>
constexpr unsigned c2r_wz_bytes() {
    return (unsigned)((N / 2) * sizeof(float2));
}
// Twiddles without staged tables: the pass twiddles read from the global table through the L1
// cache (or formed as powers of one table entry per pass, fft_transform's TWPOW), and the z twiddles
// 1 + i exp(+2*pi*i*k/N) for k = t + m*P as 1 + i e_t c_m with e_t = exp(+2*pi*i*t/N) loaded once
// per thread and c_m = exp(+2*pi*i*m/(2R)) compile-time constants (P/N = 1/(2R)).  The block
// then stages only its rows.
#ifndef C2R_COMPUTED_TW_MAX_R
#define C2R_COMPUTED_TW_MAX_R 32  // the largest row radix whose twiddles are formed in registers
#endif
template <int N>
constexpr bool c2r_computed_tw() {
    return C2RShape<N>::R <= C2R_COMPUTED_TW_MAX_R;
}
// with the z twiddles computed: 0 = each pass twiddle read from the global table through the L1
// cache, 1 = the pass twiddles as powers of one load per pass (no shared-memory traffic either
// way).  The same speed at 512^2 and 1024^2; the table is exact to half an ulp and needs fewer
// registers (84 against 96 at 1024^2), so it is the default.
#ifndef C2R_TW_POWERS
#define C2R_TW_POWERS 0
#endif
template <int N>
constexpr unsigned c2r_staged_tw_bytes() {
    return c2r_computed_tw<N>() ? 0u : c2r_tw_bytes<N>();
}
template <int N>
constexpr unsigned c2r_staged_wz_bytes() {
    return c2r_computed_tw<N>() ? 0u : c2r_wz_bytes<N>();
}
// exp(+2*pi*i*t/N) for t < P, the per-thread root of the z twiddles (compile-time, as the tables)
template <int N>
struct alignas(16) C2RRootData {
    TwEntry v[C2RShape<N>::P];
};
template <int N>
constexpr C2RRootData<N> make_c2r_root() {
    C2RRootData<N> d{};
    for (int t = 0; t < C2RShape<N>::P; ++t) d.v[t] = twiddle_exact(t, N);
    return d;
}
template <int N>
__device__ const C2RRootData<N> g_c2r_root = make_c2r_root<N>();

template <int N>
constexpr size_t c2r_smem_bytes() {
    return sizeof(float2) * (size_t)C2RShape<N>::ROWS * C2RShape<N>::BUF + c2r_row_bytes<N>() +
           c2r_staged_tw_bytes<N>() + c2r_staged_wz_bytes<N>() + sizeof(uint64_t) + sizeof(float);
}

template <int N, bool REAL>
__device__ __forceinline__ void c2r_rows_body(float2 *grids, float2 *images, const unsigned int *wsum,
                                              unsigned copy_bytes) {
    using S = C2RShape<N>;
    constexpr int M = S::M, W = half_width_of<N>();
    constexpr unsigned ROW_BYTES = c2r_row_bytes<N>();
    static_assert(ROW_BYTES <= S::BUF * sizeof(float2), "staged row larger than its buffer");
    static_assert(ROW_BYTES <= W * sizeof(float2) && (W * sizeof(float2)) % 16 == 0, "rows copied whole");
    static_assert((S::BUF * sizeof(float2)) % 16 == 0, "row buffers 16-byte aligned");
    constexpr bool CMP = c2r_computed_tw<N>();
    constexpr unsigned TW_BYTES = c2r_staged_tw_bytes<N>(), WZ_BYTES = c2r_staged_wz_bytes<N>();
    static_assert(TW_BYTES % 16 == 0 && WZ_BYTES % 16 == 0, "twiddle tables copied whole");
    extern __shared__ __align__(16) float2 smem[];
    float2 *zeros = smem + S::ROWS * S::BUF;
    float2 *tw = zeros + ROW_BYTES / sizeof(float2);  // pass twiddles, then z twiddles
    float2 *wz = tw + TW_BYTES / sizeof(float2);
    uint64_t *bar = reinterpret_cast<uint64_t *>(wz + WZ_BYTES / sizeof(float2));
    float *s_scale = reinterpret_cast<float *>(bar + 1);  // (float)(1/sum(w)) of the block's image
    const int slot = threadIdx.x / S::P, t = threadIdx.x % S::P;
    const size_t row0 = (size_t)blockIdx.x * S::ROWS;
    const size_t row = row0 + slot;
    float2 *buf = smem + slot * S::BUF;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    for (int i = threadIdx.x; i < (int)(ROW_BYTES / 16); i += blockDim.x)
        reinterpret_cast<float4 *>(zeros)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    {  // the part of each row buffer that no copy fills
        constexpr int Q = (int)(ROW_BYTES / 16);
        const int q0 = (int)(copy_bytes / 16), tail = Q - q0;
        for (int i = threadIdx.x; i < S::ROWS * tail; i += blockDim.x)
            reinterpret_cast<float4 *>(smem + (i / tail) * S::BUF)[q0 + i % tail] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, S::ROWS * copy_bytes + TW_BYTES + WZ_BYTES);
        if constexpr (!CMP) {
            bulk_load(tw, twiddles<M, S::R>(), TW_BYTES, bar);
            bulk_load(wz, g_z_twiddles<N>.v, WZ_BYTES, bar);
        }
        for (int r = 0; r < S::ROWS; ++r) bulk_load(smem + r * S::BUF, grids + (row0 + r) * W, copy_bytes, bar);
        // one FP64 reciprocal per block (all its rows are one image's), while the copies fly
        *s_scale = (float)(1.0 / (double)wsum[(row0 / N) * kWsumStride]);
    }
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0))) {
        mbar_wait_bounded(bar, 0);  // let copies still in flight land before the block exits
        return;
    }
    if (threadIdx.x == 0) {  // the rows have been read: clear them for the next wave
        for (int r = 0; r < S::ROWS; ++r) bulk_store(grids + (row0 + r) * W, zeros, copy_bytes);
        bulk_commit();
    }
    const float scale = *s_scale;
    float2 *dst = images + row * N;
    float2 e_t = make_float2(1.f, 0.f);
    if constexpr (CMP) e_t = __ldg(reinterpret_cast<const float2 *>(g_c2r_root<N>.v) + t);
    fft_transform<M, S::R, S::WARP, false, !CMP, CMP && C2R_TW_POWERS != 0>(
        t, buf, CMP ? twiddles<M, S::R>() : tw,
        [&](int k) {
            const float2 a = buf[k], b = buf[M - k];
            float2 P;
            if constexpr (CMP) {
                // k = t + m*P with m fixed in the unrolled loading loop: exp(+2*pi*i*k/N) = e_t c_m
                const int m = (k - t) / S::P;
                constexpr int STEP = 64 / (2 * S::R);  // c_m = exp(+2*pi*i*(m*STEP)/64)
                const float2 e = cmul(e_t, make_float2(cos64(m * STEP), sin64(m * STEP)));
                P = make_float2(1.f - e.y, e.x);
            } else {
                P = wz[k];
            }
            // 2 conj(b) + P (a - conj(b))
            const float dx = a.x - b.x, dy = a.y + b.y;
            return make_float2(fmaf(P.x, dx, fmaf(-P.y, dy, 2.f * b.x)), fmaf(P.x, dy, fmaf(P.y, dx, -2.f * b.y)));
        },
        [&](int m, float2 z) {
            // pixels x and x+1 as one 16-byte store (images are 16-byte aligned on this path)
            const int x = (2 * m + N / 2) & (N - 1);
            if (REAL)
                __stcs(reinterpret_cast<float2 *>(reinterpret_cast<float *>(images) + row * N + x),
                       make_float2(z.x * scale, z.y * scale));
            else
                __stcs(reinterpret_cast<float4 *>(dst + x), make_float4(z.x * scale, 0.f, z.y * scale, 0.f));
        });
    if (threadIdx.x == 0) bulk_wait_all();
}

// The kernel, with the compiler's own register budget, and at 512^2 with the budget that keeps
// nine blocks resident per SM (C2RShape::MIN_BLOCKS); a second launch-bounds argument of 1
// would change the other sides' register allocation (80 -> 96 at 1024^2), so they keep none.
template <int N, bool REAL>
__global__ void __launch_bounds__(C2RShape<N>::ROWS *C2RShape<N>::P) c2r_rows_kernel(float2 *grids, float2 *images,
                                                                                    const unsigned int *wsum,
                                                                                    unsigned copy_bytes) {
    c2r_rows_body<N, REAL>(grids, images, wsum, copy_bytes);
}
template <int N, bool REAL>
__global__ void __launch_bounds__(C2RShape<N>::ROWS *C2RShape<N>::P, C2RShape<N>::MIN_BLOCKS)
    c2r_rows_kernel_occ(float2 *grids, float2 *images, const unsigned int *wsum, unsigned copy_bytes) {
    c2r_rows_body<N, REAL>(grids, images, wsum, copy_bytes);
}

// ---- complex-to-real rows on the tensor cores (N = 512) ------------------------------------
// The same pass as c2r_rows_kernel with its length-256 complex transform done as two dense 16-point
// DFT products on the tensor cores (warp-level mma.sync m16n8k16, FP16 operands, FP32
// accumulation).  With z[16 n1 + n2] = X[n1][n2] (the Z values formed from the staged row):
//   Y = F16 X             (16-point inverse DFTs down the columns n1, for each n2)
//   Y'[k1][n2] = Y[k1][n2] exp(+2 pi i k1 n2 / 256)
//   Z = Y' F16            (16-point inverse DFTs along the rows), z_out[k1 + 16 k2] = Z[k1][k2]
// with F16[j][k] = exp(+2 pi i j k / 16), symmetric.  Complex products are real products of the
// stacked parts: [Yr; Yi] = [[Fr, -Fi], [Fi, Fr]] [Xr; Xi] and [Zr | Zi] = [Y'r | Y'i] [[Fr, Fi],
// [-Fi, Fr]].  The accumulator fragments of the first product are the operand fragments of the
// second (rows k1, columns n2 in both), so the two products exchange no data through shared memory.
//
// Precision: every operand is split into FP16 hi + lo parts (hi = fp16(x), lo = fp16(x - hi)) and
// each product is Alo Bhi + Ahi Blo + Ahi Bhi, accumulated in FP32 (the lo x lo term, 2^-22 of the
// product, is dropped): about 22 significant bits per operand instead of FP16's 11.  Each row is
// scaled by a power of two so that its largest component lies in [2^9, 2^10) before the first
// product (the second product's operands then stay below 2^14, inside FP16's range), and scaled back
// exactly in the stores.
constexpr int kTcRows = 8;        // rows per block: 4 warps, 2 rows each
constexpr int kTcThreads = 128;
struct alignas(16) W256Data {  // exp(+2 pi i q / 256), q < 256
    TwEntry v[256];
};
constexpr W256Data make_w256() {
    W256Data d{};
    for (int q = 0; q < 256; ++q) d.v[q] = twiddle_exact(q, 256);
    return d;
}
__device__ const W256Data g_w256 = make_w256();

__device__ __forceinline__ uint32_t h2_bits(__half2 h) { return *reinterpret_cast<uint32_t *>(&h); }

// hi and lo FP16 pairs of (a, b); a in the low half (the lower row or column index)
__device__ __forceinline__ void split_pair(float a, float b, uint32_t &hi, uint32_t &lo) {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    hi = h2_bits(h);
    lo = h2_bits(__floats2half2_rn(a - hf.x, b - hf.y));
}

__device__ __forceinline__ void mma_f16_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// d += A B with split operands: Alo Bhi + Ahi Blo + Ahi Bhi (small terms first)
__device__ __forceinline__ void mma_split(float (&d)[4], const uint32_t (&ahi)[4], const uint32_t (&alo)[4],
                                          uint32_t bh0, uint32_t bh1, uint32_t bl0, uint32_t bl1) {
    mma_f16_16816(d, alo, bh0, bh1);
    mma_f16_16816(d, ahi, bl0, bl1);
    mma_f16_16816(d, ahi, bh0, bh1);
}

__device__ __forceinline__ void neg4(const uint32_t (&a)[4], uint32_t (&o)[4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) o[i] = a[i] ^ 0x80008000u;
}

template <int N>
constexpr size_t c2r_tc_smem_bytes() {
    return sizeof(float2) * (size_t)kTcRows * (c2r_row_bytes<N>() / sizeof(float2)) + c2r_row_bytes<N>() +
           c2r_wz_bytes<N>() + sizeof(W256Data) + sizeof(uint64_t) + sizeof(float);
}

template <int N, bool REAL>
__global__ void __launch_bounds__(kTcThreads) c2r_rows_tc_kernel(float2 *grids, float2 *images,
                                                                 const unsigned int *wsum, unsigned copy_bytes) {
    static_assert(N == 512, "the tensor-core row pass is the 16 x 16 factorisation of N/2 = 256");
    constexpr int M = N / 2, W = half_width_of<N>();
    constexpr unsigned ROW_BYTES = c2r_row_bytes<N>();
    constexpr int BUF = (int)(ROW_BYTES / sizeof(float2));  // >= M + 1 values, 16-byte multiple
    static_assert(BUF >= M + 1 && ROW_BYTES % 16 == 0, "row buffers hold X[0..M] and stay 16-byte aligned");
    static_assert(ROW_BYTES <= W * sizeof(float2), "rows copied whole");
    constexpr unsigned WZ_BYTES = c2r_wz_bytes<N>(), W256_BYTES = sizeof(W256Data);
    static_assert(WZ_BYTES % 16 == 0 && W256_BYTES % 16 == 0, "tables copied whole");
    extern __shared__ __align__(16) float2 smem[];
    float2 *zeros = smem + kTcRows * BUF;
    float2 *wz = zeros + BUF;
    float2 *w256 = wz + WZ_BYTES / sizeof(float2);
    uint64_t *bar = reinterpret_cast<uint64_t *>(w256 + 256);
    float *s_scale = reinterpret_cast<float *>(bar + 1);
    const size_t row0 = (size_t)blockIdx.x * kTcRows;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    for (int i = threadIdx.x; i < (int)(ROW_BYTES / 16); i += blockDim.x)
        reinterpret_cast<float4 *>(zeros)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    {  // the part of each row buffer that no copy fills
        constexpr int Q = (int)(ROW_BYTES / 16);
        const int q0 = (int)(copy_bytes / 16), tail = Q - q0;
        for (int i = threadIdx.x; i < kTcRows * tail; i += blockDim.x)
            reinterpret_cast<float4 *>(smem + (i / tail) * BUF)[q0 + i % tail] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(bar, kTcRows * copy_bytes + WZ_BYTES + W256_BYTES);
        bulk_load(wz, g_z_twiddles<N>.v, WZ_BYTES, bar);
        bulk_load(w256, g_w256.v, W256_BYTES, bar);
        for (int r = 0; r < kTcRows; ++r) bulk_load(smem + r * BUF, grids + (row0 + r) * W, copy_bytes, bar);
        *s_scale = (float)(1.0 / (double)wsum[(row0 / N) * kWsumStride]);
    }
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0))) {
        mbar_wait_bounded(bar, 0);  // let copies still in flight land before the block exits
        return;
    }
    if (threadIdx.x == 0) {  // the rows have been read: clear them for the next wave
        for (int r = 0; r < kTcRows; ++r) bulk_store(grids + (row0 + r) * W, zeros, copy_bytes);
        bulk_commit();
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    // F16 fragments, hi and lo: A layout (rows j = g, g+8; columns k = 2t, 2t+1, 2t+8, 2t+9) and B
    // layout per column tile nt (rows j = 2t, 2t+1, 2t+8, 2t+9; column k = 8 nt + g)
    uint32_t frA_h[4], frA_l[4], fiA_h[4], fiA_l[4];
    uint32_t frB_h[2][2], frB_l[2][2], fiB_h[2][2], fiB_l[2][2];
    {
        auto f16 = [&](int j, int k) { return w256[16 * ((j * k) & 15)]; };
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int j = g + 8 * (r & 1), k = 2 * t + 8 * (r >> 1);
            const float2 e0 = f16(j, k), e1 = f16(j, k + 1);
            split_pair(e0.x, e1.x, frA_h[r], frA_l[r]);
            split_pair(e0.y, e1.y, fiA_h[r], fiA_l[r]);
        }
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const int j = 2 * t + 8 * r, k = 8 * nt + g;
                const float2 e0 = f16(j, k), e1 = f16(j + 1, k);
                split_pair(e0.x, e1.x, frB_h[nt][r], frB_l[nt][r]);
                split_pair(e0.y, e1.y, fiB_h[nt][r], fiB_l[nt][r]);
            }
    }
    uint32_t nfiA_h[4], nfiA_l[4];
    neg4(fiA_h, nfiA_h);
    neg4(fiA_l, nfiA_l);
    const float img_scale = *s_scale;
    for (int slot = warp; slot < kTcRows; slot += kTcThreads / 32) {
        const float2 *buf = smem + slot * BUF;
        const size_t row = row0 + slot;
        // z at n1 = 2t + (j & 1) + 8 (j >> 1), n2 = 8 nt + g: Z[k] = 2 conj(b) + P[k] (a - conj(b))
        float2 z[2][4];
        float mx = 0.f;
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int k = 16 * (2 * t + (j & 1) + 8 * (j >> 1)) + 8 * nt + g;
                const float2 a = buf[k], b = buf[M - k], P = wz[k];
                const float dx = a.x - b.x, dy = a.y + b.y;
                z[nt][j] = make_float2(fmaf(P.x, dx, fmaf(-P.y, dy, 2.f * b.x)), fmaf(P.x, dy, fmaf(P.y, dx, -2.f * b.y)));
                mx = fmaxf(mx, fmaxf(fabsf(z[nt][j].x), fabsf(z[nt][j].y)));
            }
        // power-of-two row scale: largest component into [2^9, 2^10)
        const unsigned mbits = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
        const int ex = (int)((mbits >> 23) & 0xffu);  // biased exponent of the row maximum
        const int sh = ex == 0 ? 0 : min(max(136 - ex, -126), 126);  // 2^sh: 2^(9 - (ex - 127))
        const float s_in = __int_as_float((127 + sh) << 23);
        const float s_out = __int_as_float((127 - sh) << 23) * img_scale;
        // B fragments of [Xr; Xi]: k-step 0 real parts, k-step 1 imaginary parts
        uint32_t xb_h[2][2][2], xb_l[2][2][2];  // [k-step][n-tile][reg]
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const float2 lo = z[nt][2 * r], hi = z[nt][2 * r + 1];
                split_pair(lo.x * s_in, hi.x * s_in, xb_h[0][nt][r], xb_l[0][nt][r]);
                split_pair(lo.y * s_in, hi.y * s_in, xb_h[1][nt][r], xb_l[1][nt][r]);
            }
        // Y = F16 X: rows k1 (m-tile 0 real, m-tile 1 imaginary), columns n2
        float yr[2][4] = {}, yi[2][4] = {};
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
            mma_split(yr[nt], frA_h, frA_l, xb_h[0][nt][0], xb_h[0][nt][1], xb_l[0][nt][0], xb_l[0][nt][1]);
            mma_split(yr[nt], nfiA_h, nfiA_l, xb_h[1][nt][0], xb_h[1][nt][1], xb_l[1][nt][0], xb_l[1][nt][1]);
            mma_split(yi[nt], fiA_h, fiA_l, xb_h[0][nt][0], xb_h[0][nt][1], xb_l[0][nt][0], xb_l[0][nt][1]);
            mma_split(yi[nt], frA_h, frA_l, xb_h[1][nt][0], xb_h[1][nt][1], xb_l[1][nt][0], xb_l[1][nt][1]);
        }
        // twiddles exp(+2 pi i k1 n2 / 256); element e: k1 = g + 8 (e >> 1), n2 = 8 nt + 2t + (e & 1)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int k1 = g + 8 * (e >> 1), n2 = 8 * nt + 2 * t + (e & 1);
                const float2 w = w256[(k1 * n2) & 255];
                const float re = yr[nt][e], im = yi[nt][e];
                yr[nt][e] = re * w.x - im * w.y;
                yi[nt][e] = re * w.y + im * w.x;
            }
        // A fragments of [Y'r | Y'i] (k-step 0 real, 1 imaginary): the accumulators as they lie
        uint32_t ya_h[2][4], ya_l[2][4];
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
            const float(*y)[4] = ks ? yi : yr;
            split_pair(y[0][0], y[0][1], ya_h[ks][0], ya_l[ks][0]);
            split_pair(y[0][2], y[0][3], ya_h[ks][1], ya_l[ks][1]);
            split_pair(y[1][0], y[1][1], ya_h[ks][2], ya_l[ks][2]);
            split_pair(y[1][2], y[1][3], ya_h[ks][3], ya_l[ks][3]);
        }
        // Z = Y' F16: column tiles q = 0, 1 real parts (k2 = 8q + ..), q = 2, 3 imaginary parts
        float zo[4][4] = {};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            // real: Y'r Fr - Y'i Fi
            mma_split(zo[q], ya_h[0], ya_l[0], frB_h[q][0], frB_h[q][1], frB_l[q][0], frB_l[q][1]);
            mma_split(zo[q], ya_h[1], ya_l[1], fiB_h[q][0] ^ 0x80008000u, fiB_h[q][1] ^ 0x80008000u,
                      fiB_l[q][0] ^ 0x80008000u, fiB_l[q][1] ^ 0x80008000u);
            // imaginary: Y'r Fi + Y'i Fr
            mma_split(zo[q + 2], ya_h[0], ya_l[0], fiB_h[q][0], fiB_h[q][1], fiB_l[q][0], fiB_l[q][1]);
            mma_split(zo[q + 2], ya_h[1], ya_l[1], frB_h[q][0], frB_h[q][1], frB_l[q][0], frB_l[q][1]);
        }
        // z_out[m], m = k1 + 16 k2 -> pixels 2m, 2m+1 (fftshift of columns: x -> (x + N/2) mod N)
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int k1 = g + 8 * (e >> 1), k2 = 8 * q + 2 * t + (e & 1);
                const int m = k1 + 16 * k2;
                const int x = (2 * m + N / 2) & (N - 1);
                const float vr = zo[q][e] * s_out, vi = zo[q + 2][e] * s_out;
                if (REAL)
                    __stcs(reinterpret_cast<float2 *>(reinterpret_cast<float *>(images) + row * N + x),
                           make_float2(vr, vi));
                else
                    __stcs(reinterpret_cast<float4 *>(images + row * N + x), make_float4(vr, 0.f, vi, 0.f));
            }
    }
    if (threadIdx.x == 0) bulk_wait_all();
}

template <class K>
int prepare(K kernel, size_t smem) {
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return check_cuda(e, "fft smem attribute");
    }
    return BGI_OK;
}

template <int N>
int rows_n(const float2 *src, float2 *dst, int n_images, bool zero_src, cudaStream_t s) {
    using S = Shape<N>;
    const size_t smem = sizeof(float2) * ((size_t)S::ROWS * FftCfg<N, S::R>::LEN);
    const unsigned blocks = (unsigned)((size_t)n_images * N / S::ROWS);
    auto k = zero_src ? fft_rows_kernel<N, true> : fft_rows_kernel<N, false>;
    int st = prepare(k, smem);
    if (st) return st;
    k<<<blocks, S::ROWS * S::P, smem, s>>>(const_cast<float2 *>(src), dst);
    return check_launch("fft rows");
}

template <int N>
int cols_n(float2 *src, float2 *dst, int n_images, const unsigned int *wsum, bool zero_src, bool real,
           cudaStream_t s) {
    using S = ColShape<N>;
    const size_t smem = sizeof(float2) * ((size_t)S::COLS * S::STRIDE);
    const unsigned blocks = (unsigned)((size_t)n_images * (N / 2) / (S::COLS / 2));
    auto k = real ? fft_cols_kernel<N, true, true, true>
                  : wsum ? (zero_src ? fft_cols_kernel<N, true, true> : fft_cols_kernel<N, true, false>)
                         : (zero_src ? fft_cols_kernel<N, false, true> : fft_cols_kernel<N, false, false>);
    int st = prepare(k, smem);
    if (st) return st;
    k<<<blocks, S::COLS * S::P, smem, s>>>(src, dst, wsum);
    return check_launch("fft cols");
}

template <int N, int RADIX = Shape<N>::R>
int cols_half_n(float2 *grids, int n_images, int ext_u, int ext_v, cudaStream_t s) {
    using S = ColShape<N, RADIX>;
    constexpr int TILES = half_width_of<N>() / S::COLS;
    const int eu = ext_u < 0 ? 0 : (ext_u > N / 2 ? N / 2 : ext_u);
    const int ev = ext_v < 0 ? 0 : (ext_v > N / 2 ? N / 2 : ext_v);
    const int tiles = std::min(TILES, eu / S::COLS + 1);  // tiles holding columns 0..eu
    const size_t smem = sizeof(float2) * ((size_t)S::COLS * S::STRIDE);
    const unsigned blocks = (unsigned)((size_t)n_images * tiles);
    auto k = fft_cols_half_kernel<N, RADIX>;
    int st = prepare(k, smem);
    if (st) return st;
    k<<<blocks, S::COLS * S::P, smem, s>>>(grids, tiles, ev);
    return check_launch("fft cols (half plane)");
}

template <int N>
int c2r_n(float2 *grids, float2 *images, int n_images, const unsigned int *wsum, int ext_u, bool real,
          cudaStream_t s, bool tensor = false) {
    using S = C2RShape<N>;
    const size_t smem = c2r_smem_bytes<N>();
    const unsigned blocks = (unsigned)((size_t)n_images * N / S::ROWS);
    // columns 0..ext_u, rounded up to 16 bytes: a multiple of 16 no larger than the staged row
    const int eu = ext_u < 0 ? 0 : (ext_u > N / 2 ? N / 2 : ext_u);
    const unsigned copy_bytes = std::min(c2r_row_bytes<N>(), (unsigned)(((eu + 1) * sizeof(float2) + 15) & ~(size_t)15));
    if constexpr (N == 512) {
        if (tensor) {  // the length-256 transforms on the tensor cores
            auto kt = real ? c2r_rows_tc_kernel<N, true> : c2r_rows_tc_kernel<N, false>;
            kt<<<(unsigned)((size_t)n_images * N / kTcRows), kTcThreads, c2r_tc_smem_bytes<N>(), s>>>(grids, images, wsum,
                                                                                                  copy_bytes);
            return check_launch("fft rows (complex to real, tensor cores)");
        }
    }
    auto k = real ? c2r_rows_kernel<N, true> : c2r_rows_kernel<N, false>;
    if constexpr (S::MIN_BLOCKS > 1) k = real ? c2r_rows_kernel_occ<N, true> : c2r_rows_kernel_occ<N, false>;
    int st = prepare(k, smem);
    if (st) return st;
    k<<<blocks, S::ROWS * S::P, smem, s>>>(grids, images, wsum, copy_bytes);
    return check_launch("fft rows (complex to real)");
}

// ---- src/gpu/gpu_utils.cpp:73-123: fftshift by half swaps, then divide -------------------
__device__ __forceinline__ int calc_fft_shift(int pos, int side) {
    return (pos + side / 2 + side % 2) % side;
}

__global__ void shift_x_kernel(float2 *data, int xs, int ys) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int half = xs / 2;
    if (tid >= half * ys) return;
    const int row = tid / half, col = tid % half;
    float2 *im = data + (size_t)blockIdx.y * xs * ys;
    const size_t src = (size_t)row * xs + col, dst = (size_t)row * xs + calc_fft_shift(col, xs);
    float2 tmp = im[dst];
    im[dst] = im[src];
    im[src] = tmp;
}

__global__ void shift_y_norm_kernel(float2 *data, int xs, int ys, const float *fnorm,
                                    int fnorm_size) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= xs * (ys / 2)) return;
    const int row = tid / xs, col = tid % xs;
    const int img = blockIdx.y;
    float2 *im = data + (size_t)img * xs * ys;
    const float f = fnorm[img % fnorm_size];
    const size_t src = (size_t)row * xs + col, dst = (size_t)calc_fft_shift(row, ys) * xs + col;
    float2 tmp = im[dst], v = im[src];
    im[dst] = make_float2(__fdiv_rn(v.x, f), __fdiv_rn(v.y, f));
    im[src] = make_float2(__fdiv_rn(tmp.x, f), __fdiv_rn(tmp.y, f));
}

// ---- src/gpu/gpu_utils.cpp:19-71: per-image sum (one block per image, FP64 partials) ------
__global__ void __launch_bounds__(256) vector_sum_kernel(const float *data, int64_t n, float *sums) {
    __shared__ double part[8];
    const float *x = data + (size_t)blockIdx.x * n;
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += x[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += part[w];
        sums[blockIdx.x] = (float)s;
    }
}

// ---- src/gpu/gpu_utils.cpp:143-150: mean of the images ------------------------------------
__global__ void average_kernel(const float2 *images, int64_t n_pix, int n_images, float2 *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pix) return;
    float2 acc = images[i];
    for (int k = 1; k < n_images; ++k) {
        float2 v = images[(size_t)k * n_pix + i];
        acc.x += v.x;
        acc.y += v.y;
    }
    out[i] = make_float2(__fdiv_rn(acc.x, (float)n_images), __fdiv_rn(acc.y, (float)n_images));
}

}  // namespace

int launch_fft_rows(const float2 *src, float2 *dst, int n, int n_images, bool zero_src,
                    cudaStream_t s) {
    if (n_images <= 0) return BGI_OK;
    switch (n) {
        case 16: return rows_n<16>(src, dst, n_images, zero_src, s);
        case 32: return rows_n<32>(src, dst, n_images, zero_src, s);
        case 64: return rows_n<64>(src, dst, n_images, zero_src, s);
        case 128: return rows_n<128>(src, dst, n_images, zero_src, s);
        case 256: return rows_n<256>(src, dst, n_images, zero_src, s);
        case 512: return rows_n<512>(src, dst, n_images, zero_src, s);
        case 1024: return rows_n<1024>(src, dst, n_images, zero_src, s);
        case 2048: return rows_n<2048>(src, dst, n_images, zero_src, s);
        case 4096: return rows_n<4096>(src, dst, n_images, zero_src, s);
        default: return launch_fft_any_rows(src, dst, n, n_images, zero_src, s);  // bgi_fft_any.cu
    }
}

int launch_fft_cols(float2 *images, int n, int n_images, const unsigned int *wsum,
                    cudaStream_t s) {
    return launch_fft_cols_to(images, images, n, n_images, wsum, false, s);
}

int launch_fft_cols_to(float2 *src, float2 *dst, int n, int n_images, const unsigned int *wsum,
                       bool zero_src, cudaStream_t s, bool real) {
    if (n_images <= 0) return BGI_OK;
    if (zero_src && src == dst) return set_error(BGI_ERR_INVALID, "fft cols: clearing the source needs src != dst");
    if (real && (!wsum || !zero_src)) return set_error(BGI_ERR_INVALID, "fft cols: real output is the epilogue's");
    switch (n) {
        case 16: return cols_n<16>(src, dst, n_images, wsum, zero_src, real, s);
        case 32: return cols_n<32>(src, dst, n_images, wsum, zero_src, real, s);
        case 64: return cols_n<64>(src, dst, n_images, wsum, zero_src, real, s);
        case 128: return cols_n<128>(src, dst, n_images, wsum, zero_src, real, s);
        case 256: return cols_n<256>(src, dst, n_images, wsum, zero_src, real, s);
        case 512: return cols_n<512>(src, dst, n_images, wsum, zero_src, real, s);
        case 1024: return cols_n<1024>(src, dst, n_images, wsum, zero_src, real, s);
        case 2048: return cols_n<2048>(src, dst, n_images, wsum, zero_src, real, s);
        case 4096: return cols_n<4096>(src, dst, n_images, wsum, zero_src, real, s);
        default: return launch_fft_any_cols(src, dst, n, n_images, wsum, zero_src, real, s);  // bgi_fft_any.cu
    }
}

int half_plane_width(int n) {
    switch (n) {
        case 64: return half_width_of<64>();
        case 128: return half_width_of<128>();
        case 256: return half_width_of<256>();
        case 512: return half_width_of<512>();
        case 1024: return half_width_of<1024>();
        case 2048: return half_width_of<2048>();
        case 4096: return half_width_of<4096>();
        default: return 0;  // no half-plane path for this side
    }
}

int col_default_radix(int n) {
    switch (n) {
        case 64: return Shape<64>::R;
        case 128: return Shape<128>::R;
        case 256: return Shape<256>::R;
        case 512: return Shape<512>::R;
        case 1024: return Shape<1024>::R;
        case 2048: return Shape<2048>::R;
        case 4096: return Shape<4096>::R;
        default: return 0;
    }
}

int col_alt_radix(int n) {
    switch (n) {
        case 256: return 8;
        case 512: return 16;
        case 1024: return 16;
        case 2048: return 32;
        case 4096: return 32;
        default: return 0;  // one compiled radix
    }
}

int launch_fft_cols_half(float2 *grids, int n, int n_images, int ext_u, int ext_v, cudaStream_t s, int radix) {
    if (n_images <= 0) return BGI_OK;
    if (radix != 0 && radix == col_alt_radix(n)) {
        switch (n) {
            case 256: return cols_half_n<256, 8>(grids, n_images, ext_u, ext_v, s);
            case 512: return cols_half_n<512, 16>(grids, n_images, ext_u, ext_v, s);
            case 1024: return cols_half_n<1024, 16>(grids, n_images, ext_u, ext_v, s);
            case 2048: return cols_half_n<2048, 32>(grids, n_images, ext_u, ext_v, s);
            case 4096: return cols_half_n<4096, 32>(grids, n_images, ext_u, ext_v, s);
            default: break;
        }
    }
    switch (n) {
        case 64: return cols_half_n<64>(grids, n_images, ext_u, ext_v, s);
        case 128: return cols_half_n<128>(grids, n_images, ext_u, ext_v, s);
        case 256: return cols_half_n<256>(grids, n_images, ext_u, ext_v, s);
        case 512: return cols_half_n<512>(grids, n_images, ext_u, ext_v, s);
        case 1024: return cols_half_n<1024>(grids, n_images, ext_u, ext_v, s);
        case 2048: return cols_half_n<2048>(grids, n_images, ext_u, ext_v, s);
        case 4096: return cols_half_n<4096>(grids, n_images, ext_u, ext_v, s);
        default: return set_error(BGI_ERR_UNSUPPORTED, "half-plane image side %d", n);
    }
}

bool c2r_tensor_supported(int n) { return n == 512; }

int launch_c2r_rows(float2 *grids, float2 *images, int n, int n_images, const unsigned int *wsum, int ext_u,
                    cudaStream_t s, bool real, bool tensor) {
    if (n_images <= 0) return BGI_OK;
    switch (n) {
        case 64: return c2r_n<64>(grids, images, n_images, wsum, ext_u, real, s);
        case 128: return c2r_n<128>(grids, images, n_images, wsum, ext_u, real, s);
        case 256: return c2r_n<256>(grids, images, n_images, wsum, ext_u, real, s);
        case 512: return c2r_n<512>(grids, images, n_images, wsum, ext_u, real, s, tensor);
        case 1024: return c2r_n<1024>(grids, images, n_images, wsum, ext_u, real, s);
        case 2048: return c2r_n<2048>(grids, images, n_images, wsum, ext_u, real, s);
        case 4096: return c2r_n<4096>(grids, images, n_images, wsum, ext_u, real, s);
        default: return set_error(BGI_ERR_UNSUPPORTED, "half-plane image side %d", n);
    }
}

int launch_shift_and_norm(float2 *images, int xs, int ys, int n_images, const float *fnorm,
                          int fnorm_size, cudaStream_t s) {
    if (n_images <= 0 || xs <= 0 || ys <= 0) return BGI_OK;
    for (int done = 0; done < n_images; done += 65535) {
        const int cnt = n_images - done < 65535 ? n_images - done : 65535;
        float2 *base = images + (size_t)done * xs * ys;
        int nx = (xs / 2) * ys;
        if (nx > 0) {
            shift_x_kernel<<<dim3((nx + 255) / 256, cnt), 256, 0, s>>>(base, xs, ys);
            int st = check_launch("fft_shift x");
            if (st) return st;
        }
        int ny = xs * (ys / 2);
        if (ny > 0) {
            // fnorm index is img % fnorm_size with img counted from the first image
            shift_y_norm_kernel<<<dim3((ny + 255) / 256, cnt), 256, 0, s>>>(base, xs, ys, fnorm, fnorm_size);
            int st = check_launch("fft_shift y");
            if (st) return st;
        }
        if (done + cnt < n_images && fnorm_size > 1 && (65535 % fnorm_size) != 0)
            return set_error(BGI_ERR_UNSUPPORTED, "more than 65535 images need fnorm_size dividing 65535");
    }
    return BGI_OK;
}

int launch_vector_sum(const float *data, int64_t image_size, int n_images, float *sums,
                      cudaStream_t s) {
    if (n_images <= 0) return BGI_OK;
    vector_sum_kernel<<<n_images, 256, 0, s>>>(data, image_size, sums);
    return check_launch("vector_sum");
}

int launch_image_average(const float2 *images, int64_t image_size, int n_images, float2 *out,
                         cudaStream_t s) {
    if (n_images <= 0 || image_size <= 0) return BGI_OK;
    const int64_t blocks = (image_size + 255) / 256;
    average_kernel<<<(unsigned)blocks, 256, 0, s>>>(images, image_size, n_images, out);
    return check_launch("image_averaging");
}

// ---- device fault word -------------------------------------------------------------------
namespace {
// One thread waits on an mbarrier that nothing arrives on: the bounded wait gives up, records
// the fault and returns (the self-test of the wait limit).
__global__ void wait_timeout_kernel() {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        mbar_wait_bounded(&bar, 0);
    }
}
}  // namespace

int read_device_fault(unsigned int *bits, bool clear) {
    int st = check_cuda(cudaMemcpyFromSymbol(bits, g_device_fault, sizeof(unsigned int)), "read device fault");
    if (st || !clear || !*bits) return st;
    const unsigned int zero = 0;
    return check_cuda(cudaMemcpyToSymbol(g_device_fault, &zero, sizeof(unsigned int)), "clear device fault");
}

int launch_wait_timeout_selftest(cudaStream_t s) {
    wait_timeout_kernel<<<1, 32, 0, s>>>();
    return check_launch("wait timeout self-test");
}

}  // namespace bgi
