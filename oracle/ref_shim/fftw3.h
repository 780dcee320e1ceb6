// Stand-in for the single-precision FFTW calls the reference imager makes
// (fftwf_plan_many_dft with FFTW_BACKWARD, execute, destroy, thread set-up).  The transform
// itself is the oracle's FP64 inverse DFT, rounded to float (oracle/ref_shim/ref_stubs.cpp).
#ifndef BGI_SHIM_FFTW3_H
#define BGI_SHIM_FFTW3_H
typedef float fftwf_complex[2];
typedef struct bgi_shim_fftwf_plan *fftwf_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
int fftwf_init_threads(void);
void fftwf_plan_with_nthreads(int);
void fftwf_cleanup_threads(void);
fftwf_plan fftwf_plan_many_dft(int rank, const int *n, int howmany, fftwf_complex *in,
                               const int *inembed, int istride, int idist, fftwf_complex *out,
                               const int *onembed, int ostride, int odist, int sign,
                               unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_destroy_plan(fftwf_plan p);
#endif
