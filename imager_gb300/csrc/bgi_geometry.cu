// Pointed-observation UVW on the device (the reference computes it on the host for each block:
// CAntennaPositions::CalculateUVW with metadata, src/antenna_positions.cpp:23-92, through
// PacerGeometry::CalcUVW_NEW / precXYZ / CalcUVW, src/pacer_geometry.h:101-134, 208-215, 312-334).
//
// Per timestep the caller supplies what the reference derives once per timestep with PAL (the
// precession-nutation matrix and the sines and cosines of lmst, lmst2000, the J2000 hour angle
// and the aberrated declination); per antenna the kernel rotates XYZ to the frame at lmst,
// precesses it, rotates back at lmst2000 and projects it (TMS eq. 4.1); a baseline (i >= j) is
// -(uvw_i - uvw_j) rounded to float.  Every product and sum is a separate FP64 operation in the
// reference's order (no fused multiply-add), so the result is the reference's bit for bit given
// the same sines and cosines.
#include "bgi_internal.h"

namespace bgi {
namespace {

struct Uvw {
    double u, v, w;
};

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

__device__ Uvw antenna_uvw(const double *st, double x, double y, double z) {
    const double sep = st[9], cep = st[10], s2000 = st[11], c2000 = st[12];
    const double sh = st[13], ch = st[14], sd = st[15], cd = st[16];
    // precXYZ: to the frame with x at zero RA, precess, back to the frame at lmst2000
    const double xpr = sub(mul(cep, x), mul(sep, y));
    const double ypr = add(mul(sep, x), mul(cep, y));
    const double zpr = z;
    const double xpr2 = add(add(mul(st[0], xpr), mul(st[1], ypr)), mul(st[2], zpr));
    const double ypr2 = add(add(mul(st[3], xpr), mul(st[4], ypr)), mul(st[5], zpr));
    const double zpr2 = add(add(mul(st[6], xpr), mul(st[7], ypr)), mul(st[8], zpr));
    const double xp = add(mul(c2000, xpr2), mul(s2000, ypr2));
    const double yp = add(mul(-s2000, xpr2), mul(c2000, ypr2));
    const double zp = zpr2;
    // CalcUVW (TMS eq. 4.1)
    Uvw r;
    r.u = add(mul(sh, xp), mul(ch, yp));
    r.v = add(add(mul(mul(-sd, ch), xp), mul(mul(sd, sh), yp)), mul(cd, zp));
    r.w = add(sub(mul(mul(cd, ch), xp), mul(mul(cd, sh), yp)), mul(sd, zp));
    return r;
}

// one thread per (timestep, baseline)
__global__ void __launch_bounds__(256) pointed_uvw_kernel(const double *__restrict__ xyz, int n_ant,
                                                         const double *__restrict__ steps, long long n_steps,
                                                         float *u, float *v, float *w) {
    const long long nb = (long long)n_ant * (n_ant + 1) / 2;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nb * n_steps) return;
    const long long t = q / nb, b = q - t * nb;
    long long i = (long long)((sqrtf(8.0f * (float)b + 1.0f) - 1.0f) * 0.5f);  // within 1; corrected
    while (i * (i + 1) / 2 > b) --i;
    while ((i + 1) * (i + 2) / 2 <= b) ++i;
    const long long j = b - i * (i + 1) / 2;
    const double *st = steps + 17 * t;
    const Uvw a = antenna_uvw(st, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    const Uvw c = antenna_uvw(st, xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2]);
    u[q] = __double2float_rn(-sub(a.u, c.u));
    v[q] = __double2float_rn(-sub(a.v, c.v));
    w[q] = __double2float_rn(-sub(a.w, c.w));
}

// max |u| and max |v| over unflagged baselines of every set (src/pacer_imager.cpp:213-221):
// non-negative floats order as their bit patterns
__global__ void __launch_bounds__(256) uv_absmax_kernel(const float *u, const float *v, const int *flags,
                                                       long long nb, long long n, unsigned *out) {
    unsigned mu = 0, mv = 0;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        if (flags[q % nb] == 0) {
            mu = max(mu, __float_as_uint(fabsf(u[q])));
            mv = max(mv, __float_as_uint(fabsf(v[q])));
        }
    mu = __reduce_max_sync(0xffffffffu, mu);
    mv = __reduce_max_sync(0xffffffffu, mv);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, mu);
        atomicMax(out + 1, mv);
    }
}

}  // namespace

int launch_pointed_uvw(const double *xyz, int n_ant, const double *steps, int n_steps, float *u, float *v, float *w,
                       cudaStream_t s) {
    const long long n = (long long)n_ant * (n_ant + 1) / 2 * n_steps;
    if (n <= 0) return BGI_OK;
    if ((n + 255) / 256 > 0x7fffffffLL) return set_error(BGI_ERR_UNSUPPORTED, "pointed uvw: too many baselines");
    pointed_uvw_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(xyz, n_ant, steps, n_steps, u, v, w);
    return check_launch("pointed uvw");
}

int launch_uv_absmax(const float *u, const float *v, const int *flags, long long nb, int n_sets, unsigned *out2,
                     cudaStream_t s) {
    int st = check_cuda(cudaMemsetAsync(out2, 0, 2 * sizeof(unsigned), s), "uv max clear");
    if (st) return st;
    const long long n = nb * n_sets;
    const unsigned blocks = (unsigned)std::min<long long>((n + 255) / 256, 4LL * sm_count());
    uv_absmax_kernel<<<std::max(1u, blocks), 256, 0, s>>>(u, v, flags, nb, n, out2);
    return check_launch("uv max");
}

}  // namespace bgi
