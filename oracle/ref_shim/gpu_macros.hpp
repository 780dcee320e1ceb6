// Minimal host-only stand-in for astroio's gpu_macros.hpp, enough for g++ to read the
// reference's src/gpu headers (their __global__ declarations) when checking that the
// reference-side binding compiles.  Not product code.
#ifndef BGI_SHIM_GPU_MACROS_HPP
#define BGI_SHIM_GPU_MACROS_HPP
#ifndef __global__
#define __global__
#endif
#endif
