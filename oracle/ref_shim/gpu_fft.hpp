// Minimal host-only stand-in for astroio's gpu_fft.hpp: the FFT types that the reference's
// src/gpu headers name, for the compile check of the reference-side binding.  Not product code.
#ifndef BGI_SHIM_GPU_FFT_HPP
#define BGI_SHIM_GPU_FFT_HPP
#include "gpu_macros.hpp"
struct gpufftComplex {
    float x, y;
};
typedef int gpufftHandle;
#endif
