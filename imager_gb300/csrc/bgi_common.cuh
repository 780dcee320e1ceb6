// Shared device helpers of the BLINK GB300 imaging kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "blink_imager_gb300.h"

namespace bgi {

constexpr double kVelLight = 299792458.0;  // src/pacer_imager_defs.h:12-13
// src/pacer_imager_defs.h:21: a component passes when |x| < 1e12, compared in double.  1e12 is
// not a float; the float test |x| < 1000000061440 (the first float above 1e12) passes exactly
// the same values (the largest float below 1e12 is 999999995904).
constexpr float kMaxVis = 1000000061440.0f;

// ------------------------------------------------------------------------------------------
// Host-side error reporting (thread-local message, status codes of blink_imager_gb300.h)
// ------------------------------------------------------------------------------------------
int set_error(int status, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
int check_launch(const char *what);

// Per-channel constants for gridding.
struct alignas(16) ChannelConst {
    // the fields every visibility reads first (one 16-byte load)
    float su, sv;       // nu / (VEL_LIGHT * delta_u), ... rounded to float (fast cell filter)
    float f_hi, f_lo;   // nu / VEL_LIGHT as an unevaluated float sum (turns of phase per metre)
    // the fields of the rare paths
    float inv_wl;       // 1 / wavelength rounded to float (fast min_uv filter)
    float pad;
    double wavelength;  // VEL_LIGHT / nu, as src/gpu/gridding_gpu.cpp:102
};

__device__ __forceinline__ ChannelConst make_channel_const(double nu, double du, double dv) {
    ChannelConst cc;
    cc.wavelength = kVelLight / nu;
    cc.su = (float)(nu / (kVelLight * du));
    cc.sv = (float)(nu / (kVelLight * dv));
    cc.inv_wl = (float)(nu / kVelLight);
    const double f = nu / kVelLight;
    cc.f_hi = (float)f;
    cc.f_lo = (float)(f - (double)cc.f_hi);
    cc.pad = 0.f;
    return cc;
}

// ------------------------------------------------------------------------------------------
// uv cell index, bit-exact with calculate_pos (src/gpu/gridding_gpu.cpp:18-54).
//
// The reference computes in FP64: ul = u/lambda; dist = sqrt(ul^2 + vl^2) (no fused
// multiply-add, as its x86-64 CPU build); cut unless dist > min_uv; pix = round(ul/delta_u)
// (half away from zero); wrap(+-pix) = i >= 0 ? i % N : N + i; pos = N*v_idx + u_idx.
//
// FP64 is slow on this GPU, so the pixel coordinate is first computed in FP32 as
// x = u * su with su = nu/(c*delta_u) rounded to float.  Its relative error against the exact
// real value is below 2^-23 (one rounding of su, one of the product) and the FP64 value's is
// below 2^-51, so |x - x64| <= |x| * 2^-21 with a 4x margin.  round(x64) == round(x) whenever
// x is farther than that from a half-integer; otherwise (about 1e-4 of visibilities near the
// grid edge) the exact FP64 recipe runs.  This is the filtered-arithmetic scheme of
// Shewchuk's adaptive predicates: a cheap approximation with a proven error bound, and the
// exact computation only where the bound cannot decide.  The min_uv cut uses the same scheme.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int wrap_index(int i, int side) {
    if ((unsigned)i < (unsigned)side) return i;  // the common case, without a division
    return i >= 0 ? i % side : side + i;
}

// Exact FP64 path (no contraction: explicit _rn intrinsics).
__device__ __forceinline__ bool uv_pixels_exact(float u, float v, double wavelength, double du,
                                                double dv, double min_uv, double *up, double *vp) {
    double ul = __ddiv_rn((double)u, wavelength);
    double vl = __ddiv_rn((double)v, wavelength);
    double dist = __dsqrt_rn(__dadd_rn(__dmul_rn(ul, ul), __dmul_rn(vl, vl)));
    if (!(dist > min_uv)) return false;
    *up = round(__ddiv_rn(ul, du));
    *vp = round(__ddiv_rn(vl, dv));
    return true;
}

// True when x (FP32 estimate of a value whose exact counterpart lies within x*2^-21) rounds
// to the same integer as the exact value; that integer is then *r.
//
// d = 0.5 - |x - rint(x)| is x's distance to the nearest half-integer: x - rint(x) is exact,
// and so is 0.5 - |.| wherever d is small enough to matter (Sterbenz), so the decision is the
// one of the exact distance.  When the test passes, x is not a half-integer, so rint(x) (ties
// to even) equals the reference's round (ties away from zero).
__device__ __forceinline__ bool round_certain(float x, float *r) {
    const float ri = rintf(x);
    const float d = 0.5f - fabsf(x - ri);
    const float tol = fabsf(x) * 4.76837158e-7f + 1e-30f;  // 2^-21
    *r = ri;
    return d > tol && fabsf(x) < 536870912.0f;  // and |x| < 2^29
}

// Returns false when the visibility is cut by min_uv (calculate_pos would return -1);
// otherwise the rounded pixel coordinates (exact integers) in *ui, *vi.
__device__ __forceinline__ bool uv_pixels(float u, float v, float su, float sv, const ChannelConst *ccp,
                                          double du, double dv, double min_uv, bool min_uv_active, int *ui,
                                          int *vi) {
    bool need_exact = false;
    if (min_uv_active) {
        // d32 and (float)min_uv each lie within 2^-22 (relative) of their exact values
        float d32 = sqrtf(u * u + v * v) * ccp->inv_wl;
        float md = (float)min_uv;
        float tol = (fabsf(d32) + fabsf(md)) * 9.5367431640625e-7f + 1e-30f;  // 2^-20
        if (!(fabsf(d32 - md) > tol)) {
            need_exact = true;
        } else if (!(d32 > md)) {
            return false;
        }
    }
    const float xu = u * su, xv = v * sv;
    float ru, rv;
    const bool cu = round_certain(xu, &ru), cv = round_certain(xv, &rv);
    if (!need_exact && cu && cv) {
        *ui = (int)ru;
        *vi = (int)rv;
        return true;
    }
    double up, vp;
    if (!uv_pixels_exact(u, v, ccp->wavelength, du, dv, min_uv, &up, &vp)) return false;
    if (!(fabs(up) < 1073741824.0) || !(fabs(vp) < 1073741824.0)) return false;
    *ui = (int)up;
    *vi = (int)vp;
    return true;
}

// pos of calculate_pos for uv_sign = +1 / -1, or -1 when outside [0, N*N).
__device__ __forceinline__ long long cell_pos(int ui, int vi, int sign, int n) {
    long long pos = (long long)n * wrap_index(sign * vi, n) + wrap_index(sign * ui, n);
    return (pos >= 0 && pos < (long long)n * n) ? pos : -1;
}

// ------------------------------------------------------------------------------------------
// Polarisation selection (src/gpu/gridding_gpu.cpp:79-98, src/pacer_imager.cpp:301-325).
// rec points at one 4-pol record: XX(0,1) XY(2,3) YX(4,5) YY(6,7).
// ------------------------------------------------------------------------------------------
// The 8-byte pol values one visibility needs: XX -> (XX, -), YY -> (YY, -), I -> (XX, YY),
// V -> (XY, YX).  Streaming loads (read once).
template <int POL>
__device__ __forceinline__ void load_pols(const float2 *rec, float2 &a, float2 &b) {
    if (POL == BGI_POL_XX) a = __ldcs(rec);
    else if (POL == BGI_POL_YY) a = __ldcs(rec + 3);
    else if (POL == BGI_POL_I) { a = __ldcs(rec); b = __ldcs(rec + 3); }
    else { a = __ldcs(rec + 1); b = __ldcs(rec + 2); }
}

// ---- block-scaled 16-bit visibilities ------------------------------------------------------
constexpr int kVisBlock = 128;  // baselines per scale block of a pol plane

// one stored complex value (re in the low half, im in the high half) times its block scale
template <int FMT>
__device__ __forceinline__ float2 decode_vis(uint32_t e, float scale) {
    const uint16_t r = (uint16_t)(e & 0xffffu), i = (uint16_t)(e >> 16);
    float x, y;
    if (FMT == BGI_VIS_S16) {
        // int16 -> float without a conversion instruction: the float whose bits are
        // 0x4B400000 + k is 1.5 * 2^23 + k for |k| < 2^22, so subtracting 1.5 * 2^23 is exact
        const float xf = __fsub_rn(__int_as_float(0x4B400000 + (int)(int16_t)r), 12582912.0f);
        const float yf = __fsub_rn(__int_as_float(0x4B400000 + (int)(int16_t)i), 12582912.0f);
        x = r == 0x8000u ? __int_as_float(0x7fc00000) : xf;
        y = i == 0x8000u ? __int_as_float(0x7fc00000) : yf;
    } else if (FMT == BGI_VIS_BF16) {
        x = __uint_as_float((uint32_t)r << 16);
        y = __uint_as_float((uint32_t)i << 16);
    } else {
        x = __half2float(__ushort_as_half(r));
        y = __half2float(__ushort_as_half(i));
    }
    return make_float2(__fmul_rn(x, scale), __fmul_rn(y, scale));
}

// Loads the pols that POL needs (as load_pols) from pol planes: data [img][4][B] of uint32,
// scales [img][4][NB].
template <int POL, int FMT>
__device__ __forceinline__ void load_pols_planar(const uint32_t *data, const float *scales, size_t img,
                                                 long long nb, long long nblk, long long b, float2 &a,
                                                 float2 &bb) {
    const uint32_t *d = data + img * 4 * nb + b;
    const float *sc = scales + img * 4 * nblk + b / kVisBlock;
    if (POL == BGI_POL_XX) {
        a = decode_vis<FMT>(__ldcs(d), __ldg(sc));
    } else if (POL == BGI_POL_YY) {
        a = decode_vis<FMT>(__ldcs(d + 3 * nb), __ldg(sc + 3 * nblk));
    } else if (POL == BGI_POL_I) {
        a = decode_vis<FMT>(__ldcs(d), __ldg(sc));
        bb = decode_vis<FMT>(__ldcs(d + 3 * nb), __ldg(sc + 3 * nblk));
    } else {
        a = decode_vis<FMT>(__ldcs(d + nb), __ldg(sc + nblk));
        bb = decode_vis<FMT>(__ldcs(d + 2 * nb), __ldg(sc + 2 * nblk));
    }
}

template <int POL>
__device__ __forceinline__ float2 combine_pols(float2 a, float2 b) {
    if (POL == BGI_POL_XX || POL == BGI_POL_YY) return a;
    if (POL == BGI_POL_V) {
        // (0 + 0.5i) * (XY - YX)
        float dr = __fsub_rn(a.x, b.x), di = __fsub_rn(a.y, b.y);
        return make_float2(__fsub_rn(__fmul_rn(0.0f, dr), __fmul_rn(0.5f, di)),
                           __fadd_rn(__fmul_rn(0.0f, di), __fmul_rn(0.5f, dr)));
    }
    return make_float2(__fdiv_rn(__fadd_rn(a.x, b.x), 2.0f), __fdiv_rn(__fadd_rn(a.y, b.y), 2.0f));
}

__device__ __forceinline__ float2 select_pol(const float4 lo, const float4 hi, int pol) {
    // lo = (XX.re, XX.im, XY.re, XY.im), hi = (YX.re, YX.im, YY.re, YY.im)
    if (pol == BGI_POL_XX) return make_float2(lo.x, lo.y);
    if (pol == BGI_POL_YY) return make_float2(hi.z, hi.w);
    if (pol == BGI_POL_V) {
        // (0 + 0.5i) * (XY - YX)
        float dr = __fsub_rn(lo.z, hi.x), di = __fsub_rn(lo.w, hi.y);
        return make_float2(__fsub_rn(__fmul_rn(0.0f, dr), __fmul_rn(0.5f, di)),
                           __fadd_rn(__fmul_rn(0.0f, di), __fmul_rn(0.5f, dr)));
    }
    return make_float2(__fdiv_rn(__fadd_rn(lo.x, hi.z), 2.0f), __fdiv_rn(__fadd_rn(lo.y, hi.w), 2.0f));
}

// ------------------------------------------------------------------------------------------
// Delay phase: turns = delay_m * nu/c reduced to [-0.5, 0.5] in FP64 (the one step that needs
// FP64: delays of km times nu/c reach 10^4 turns), then sin/cos of 2*pi*turns in FP32.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 phasor(double delay_m, double turns_per_m) {
    double t = delay_m * turns_per_m;
    double r = t - rint(t);
    float s, c;
    sincospif(2.0f * (float)r, &s, &c);
    return make_float2(c, s);
}

// The same reduction in double-float arithmetic (an unevaluated sum of two floats, Dekker
// 1971, "A floating-point technique for extending the available precision"): the delay
// d = d_hi + d_lo times f = f_hi + f_lo by the FMA two-product, then the integer part of the
// leading product removed exactly (p - rint(p) is exact for |p| < 2^23).  About 44 bits of
// the product survive, so the fractional turn is good to ~1e-11 at 10^4 turns -- FP64-grade
// reduction at FP32 issue rate.
__device__ __forceinline__ float2 phasor_df(float d_hi, float d_lo, float f_hi, float f_lo) {
    const float p = d_hi * f_hi;
    float e = fmaf(d_hi, f_hi, -p);
    e = fmaf(d_hi, f_lo, e);
    e = fmaf(d_lo, f_hi, e);
    // p - rint(p), with rint by the exact addition of 1.5 * 2^23 (valid for |p| < 2^22 turns, a
    // delay of thousands of kilometres; beyond it rintf)
    const float ip = fabsf(p) < 4194304.0f ? __fsub_rn(__fadd_rn(p, 12582912.0f), 12582912.0f) : rintf(p);
    const float r = (p - ip) + e;
    // |2*pi*r| <= pi: the SFU sine/cosine is accurate to 2^-21.4 absolute on [-pi, pi]
    float s, c;
    __sincosf(6.28318530717958648f * r, &s, &c);
    return make_float2(c, s);
}

// w - (dl_hi + dl_lo) as a double-float (Knuth's two-sum on the leading terms).
__device__ __forceinline__ void delay_df(float w, float dl_hi, float dl_lo, float &hi, float &lo) {
    const float s = w - dl_hi;
    const float bb = s - w;
    const float err = (w - (s - bb)) + (-dl_hi - bb);
    hi = s;
    lo = err - dl_lo;
}

__device__ __forceinline__ float2 rotate(float2 z, float2 p) {
    // re' = re*cos - im*sin ; im' = im*cos + re*sin  (src/corrections.cpp:29-30)
    return make_float2(z.x * p.x - z.y * p.y, z.y * p.x + z.x * p.y);
}

// Streaming 16-byte load (cache-streaming: the data is read once).  Needs 16-byte alignment,
// which the host entry points check.
__device__ __forceinline__ float4 ld_stream_f4(const float4 *p) { return __ldcs(p); }

}  // namespace bgi
