// Link-time stand-ins for the parts of the reference imager that the oracle cross-check does
// not exercise (metadata files, pointed-UVW geometry, FFTW), so that the reference's own
// src/corrections.cpp, src/pacer_imager.cpp and src/utils.cpp can be compiled and run here.
// CAntennaPositions::CalculateUVW returns the UVW that the driver sets (ref_driver.cpp).
// Not product code: test infrastructure for the oracle only.
#include "observation_metadata.h"
#include "antenna_positions.h"
#include <fftw3.h>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "../blink_oracle.h"

// ---- UVW handed over by the driver -------------------------------------------------------
std::vector<float> g_shim_u, g_shim_v, g_shim_w_tri;

CAntennaPositions::CAntennaPositions(CObsMetadata *pMetaData) : m_pMetaData(pMetaData) {}
CAntennaPositions::~CAntennaPositions() {}
double CAntennaPositions::m_ObservatoryLongitudeDeg = 0;
double CAntennaPositions::m_ObservatoryLattitudeDeg = 0;
double CAntennaPositions::m_ObservatoryHeight = 0;

int CAntennaPositions::ReadAntennaPositions(const char *, bool) { return -1; }

// The CPU geometric correction reads w[ant1*n_ant + ant2] (src/corrections.cpp:19), so w is
// handed over as a square array holding each baseline's w at that position.
int CAntennaPositions::CalculateUVW(MemoryBuffer<float> &u_cpu, MemoryBuffer<float> &v_cpu,
                                    MemoryBuffer<float> &w_cpu, bool) {
    const size_t n_ant = size();
    const size_t nb = n_ant * (n_ant + 1) / 2;
    if (g_shim_u.size() != nb) { fprintf(stderr, "shim: UVW not set\n"); abort(); }
    if (!u_cpu) u_cpu.allocate(nb);
    if (!v_cpu) v_cpu.allocate(nb);
    if (!w_cpu) w_cpu.allocate(n_ant * n_ant);
    for (size_t b = 0; b < nb; ++b) { u_cpu[b] = g_shim_u[b]; v_cpu[b] = g_shim_v[b]; }
    for (size_t a1 = 0; a1 < n_ant; ++a1)
        for (size_t a2 = 0; a2 <= a1; ++a2) w_cpu[a1 * n_ant + a2] = g_shim_w_tri[a1 * (a1 + 1) / 2 + a2];
    return (int)nb;
}

// ---- metadata: nothing is read -----------------------------------------------------------
CObsMetadata::CObsMetadata(const char *) : _fptr(nullptr), m_bHasMetaFits(false), m_AntennaPositions(this) {
    raHrs = 0; decDegs = 0; haHrs = 0;
}
bool CObsMetadata::ReadMetaData(const char *) { return false; }
bool CObsMetadata::fix_metafits(double, double) { return true; }
double CObsMetadata::ux2gps(double uxtime) { return uxtime; }

// ---- FFTW stand-in: FP64 inverse DFT of the oracle, rounded to float ----------------------
struct bgi_shim_fftwf_plan { int n; int howmany; fftwf_complex *in, *out; int idist, odist; };
int fftwf_init_threads(void) { return 1; }
void fftwf_plan_with_nthreads(int) {}
void fftwf_cleanup_threads(void) {}
fftwf_plan fftwf_plan_many_dft(int rank, const int *n, int howmany, fftwf_complex *in,
                               const int *, int istride, int idist, fftwf_complex *out,
                               const int *, int ostride, int odist, int sign, unsigned) {
    if (rank != 2 || n[0] != n[1] || istride != 1 || ostride != 1 || sign != FFTW_BACKWARD) {
        fprintf(stderr, "shim: unsupported FFTW plan\n");
        abort();
    }
    return new bgi_shim_fftwf_plan{n[0], howmany, in, out, idist, odist};
}
void fftwf_execute(const fftwf_plan p) {
    const size_t npix = size_t(p->n) * p->n;
    std::vector<double> a(2 * npix), b(2 * npix);
    for (int i = 0; i < p->howmany; ++i) {
        const float *src = &p->in[size_t(i) * p->idist][0];
        float *dst = &p->out[size_t(i) * p->odist][0];
        for (size_t k = 0; k < 2 * npix; ++k) a[k] = src[k];
        bgo_fft2_inverse_f64(a.data(), b.data(), p->n, 1);
        for (size_t k = 0; k < 2 * npix; ++k) dst[k] = (float)b[k];
    }
}
void fftwf_destroy_plan(fftwf_plan p) { delete p; }
