// C-ABI driver around the reference imager's own CPU code (compiled from its sources with the
// stand-ins in this folder).  Used here only to generate golden vectors that pin the oracle.
#include "pacer_imager.h"
#include "pacer_geometry.h"
#include "corrections.h"
#include <astroio.hpp>
#include <cstring>
#include <vector>
#include <string>

extern std::vector<float> g_shim_u, g_shim_v, g_shim_w_tri;

namespace {
int g_kernel_size = 0;  // convolution kernel of the next harness (0: nearest neighbour)

struct Harness : public CPacerImager {
    Harness(int n_pixels, const std::vector<int> &flagged, Polarization pol, float osf,
            double min_uv, const char *weighting)
        : CPacerImager("", n_pixels, flagged, false, pol, osf, min_uv,
                       std::numeric_limits<double>::infinity(), weighting) {
        m_nConvolvingKernelSize = g_kernel_size;
    }
    MemoryBuffer<std::complex<float>> &grid_buffer() { return grids; }
    MemoryBuffer<float> &counter_buffer() { return grids_counters; }
};

Visibilities make_vis(const float *vis, int T, int C, int n_ant) {
    ObservationInfo oi;
    oi.nAntennas = n_ant;
    Visibilities x(oi, T, C);
    memcpy(x.data(), vis, sizeof(float) * 2 * x.buf.size());
    return x;
}
}  // namespace

extern "C" {

// m_nConvolvingKernelSize of the imagers that ref_run builds from now on (src/pacer_imager.h:169)
void ref_set_kernel_size(int k) { g_kernel_size = k; }

int ref_apply_geometric_cpu(float *vis, int T, int C, int n_ant, const float *w_tri,
                            const double *freqs) {
    Visibilities x = make_vis(vis, T, C, n_ant);
    MemoryBuffer<float> w(size_t(n_ant) * n_ant);
    for (int a1 = 0; a1 < n_ant; ++a1)
        for (int a2 = 0; a2 <= a1; ++a2) w[size_t(a1) * n_ant + a2] = w_tri[a1 * (a1 + 1) / 2 + a2];
    MemoryBuffer<double> f(C);
    for (int c = 0; c < C; ++c) f[c] = freqs[c];
    apply_geometric_corrections_cpu(x, w, f);
    memcpy(vis, x.data(), sizeof(float) * 2 * x.buf.size());
    return 0;
}

int ref_apply_cable_cpu(float *vis, int T, int C, int n_ant, const double *cable,
                        const double *freqs) {
    Visibilities x = make_vis(vis, T, C, n_ant);
    MemoryBuffer<double> L(n_ant), f(C);
    for (int a = 0; a < n_ant; ++a) L[a] = cable[a];
    for (int c = 0; c < C; ++c) f[c] = freqs[c];
    apply_cable_lengths_corrections_cpu(x, L, f);
    memcpy(vis, x.data(), sizeof(float) * 2 * x.buf.size());
    return 0;
}

void ref_fft_shift(float *image, int x_side, int y_side) {
    fft_shift(reinterpret_cast<std::complex<float> *>(image), x_side, y_side);
}

// CPacerImager::run() on host data: grid() (frequencies, corrections, delta_u, gridding) then
// image().  Frequencies come from the cotter formula with the obsInfo fields given, or from
// freq_mhz_override when it is > 0.  Outputs: corrected visibilities, grids and counters as
// left by gridding(), images, and {delta_u, delta_v, u_max, v_max}.
int ref_run(const float *vis_in, int T, int C, int n_ant, const float *u, const float *v,
            const float *w_tri, const double *cable, const int *flagged_ants, int n_flagged,
            double freq_res_mhz, int n_avg, double coarse_bw_mhz, int coarse_channel,
            double freq_mhz_override, int n_pixels, float osf, double min_uv, int pol,
            const char *weighting, int apply_geom, int apply_cable, float *vis_out,
            float *grids_out, float *counters_out, float *images_out, double *scalars_out) {
    const size_t nb = size_t(n_ant) * (n_ant + 1) / 2;
    g_shim_u.assign(u, u + nb);
    g_shim_v.assign(v, v + nb);
    g_shim_w_tri.assign(w_tri, w_tri + nb);
    std::vector<int> flagged(flagged_ants, flagged_ants + n_flagged);
    Harness im(n_pixels, flagged, static_cast<Polarization>(pol), osf, min_uv, weighting);
    im.m_MetaData.m_AntennaPositions.resize(n_ant);
    for (int a = 0; a < n_ant; ++a) im.m_MetaData.m_AntennaPositions[a].cableLenDelta = cable[a];
    im.UpdateFlags();
    im.apply_geom_correction = apply_geom != 0;
    im.apply_cable_correction = apply_cable != 0;
    im.m_fFrequencyMHz = freq_mhz_override;

    ObservationInfo oi;
    oi.nAntennas = n_ant;
    oi.frequencyResolution = freq_res_mhz;
    oi.coarseChannelBandwidth = coarse_bw_mhz;
    oi.coarseChannel = coarse_channel;
    Visibilities x(oi, T, C);
    x.nAveragedChannels = n_avg;
    memcpy(x.data(), vis_in, sizeof(float) * 2 * x.buf.size());

    // The reference builds its convolution kernels lazily inside convolve_with_kernel, which
    // runs in its OpenMP loop over images: concurrent first calls race on the kernel vectors
    // (src/pacer_imager.cpp:599-606).  Build them once here; later calls return at once.
    if (g_kernel_size > 0) im.makeKernels(g_kernel_size);
    im.grid(x);
    const size_t npix = size_t(n_pixels) * n_pixels * T * C;
    memcpy(vis_out, x.data(), sizeof(float) * 2 * x.buf.size());
    memcpy(grids_out, im.grid_buffer().data(), sizeof(float) * 2 * npix);
    memcpy(counters_out, im.counter_buffer().data(), sizeof(float) * npix);
    Images images = im.image(x.obsInfo);
    memcpy(images_out, images.data(), sizeof(float) * 2 * npix);
    scalars_out[0] = im.delta_u;
    scalars_out[1] = im.delta_v;
    scalars_out[2] = im.u_max;
    scalars_out[3] = im.v_max;
    return 0;
}

// Pointed-observation UVW with the reference's own geometry (src/pacer_geometry.h): per
// timestep t, UVWTimestepInfo from the given angles and matrix, each antenna through
// PacerGeometry::CalcUVW_NEW, and the baseline loop of CAntennaPositions::CalculateUVW
// (src/antenna_positions.cpp:57-89).  Also writes each timestep's 17 numbers (matrix, then
// sin/cos of lmst, lmst2000, ha2000, dec_aber from this libm) for the oracle.
void ref_pointed_uvw(const double *xyz, int n_ant, const double *rmat, const double *ha2000,
                     const double *dec_aber, const double *lmst, const double *lmst2000, int n_steps,
                     float *u_out, float *v_out, float *w_out, double *steps_out) {
    const unsigned nb = (unsigned)(n_ant * (n_ant + 1)) / 2;
    for (int t = 0; t < n_steps; ++t) {
        PacerGeometry::UVWTimestepInfo info;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) info.rmatpr[i][j] = rmat[9 * t + 3 * i + j];
        info.ha2000 = ha2000[t];
        info.dec_aber = dec_aber[t];
        info.lmst = lmst[t];
        info.lmst2000 = lmst2000[t];
        double *st = steps_out + 17 * t;
        for (int k = 0; k < 9; ++k) st[k] = rmat[9 * t + k];
        st[9] = sin(lmst[t]), st[10] = cos(lmst[t]), st[11] = sin(lmst2000[t]), st[12] = cos(lmst2000[t]);
        st[13] = sin(ha2000[t]), st[14] = cos(ha2000[t]), st[15] = sin(dec_aber[t]), st[16] = cos(dec_aber[t]);
        for (unsigned baseline = 0; baseline < nb; baseline++) {
            unsigned int i{static_cast<unsigned int>(-0.5 + std::sqrt(0.25 + 2 * baseline))};
            unsigned int j{baseline - ((i + 1) * i) / 2};
            double u = 0, v = 0, w = 0, u2 = 0, v2 = 0, w2 = 0;
            PacerGeometry::CalcUVW_NEW(info, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], u, v, w);
            PacerGeometry::CalcUVW_NEW(info, xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2], u2, v2, w2);
            u = u - u2;
            v = v - v2;
            w = w - w2;
            u_out[t * nb + baseline] = -u;
            v_out[t * nb + baseline] = -v;
            w_out[t * nb + baseline] = -w;
        }
    }
}
}
