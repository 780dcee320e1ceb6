// src/gpu/gb300_bindings.cpp -- replaces gridding_gpu.cpp, corrections_gpu.cpp, gpu_utils.cpp
#include <stdexcept>
#include <blink_imager_gb300.h>
#include "gridding_gpu.h"
#include "corrections_gpu.h"
#include "gpu_utils.h"

static void check(int status) {
    if (status != BGI_OK) throw std::runtime_error(bgi_last_error());  // reference error style
}

// src/gpu/corrections_gpu.cpp:90
void apply_geometric_corrections_gpu(Visibilities &xcorr, float *w_gpu, MemoryBuffer<double> &frequencies) {
    xcorr.to_gpu();
    frequencies.to_gpu();
    check(bgi_apply_geometric_corrections_gpu(reinterpret_cast<float *>(xcorr.data()), xcorr.obsInfo.nAntennas,
                                              xcorr.nFrequencies, xcorr.integration_intervals(), w_gpu, 1,
                                              frequencies.data(), nullptr));
}

// src/gpu/corrections_gpu.cpp:75
void apply_cable_lengths_corrections_gpu(Visibilities &xcorr, MemoryBuffer<double> &cable_lengths,
                                         MemoryBuffer<double> &frequencies) {
    if (!xcorr.on_gpu()) xcorr.to_gpu();
    cable_lengths.to_gpu();
    frequencies.to_gpu();
    check(bgi_apply_cable_lengths_corrections_gpu(reinterpret_cast<float *>(xcorr.data()), xcorr.obsInfo.nAntennas,
                                                  xcorr.nFrequencies, xcorr.integration_intervals(),
                                                  cable_lengths.data(), frequencies.data(), nullptr));
}

// src/gpu/gridding_gpu.cpp:130 -- counters for interval 0 per channel, as the reference
void gridding_gpu(const Visibilities &xcorr, const MemoryBuffer<float> &u_gpu, const MemoryBuffer<float> &v_gpu,
                  const MemoryBuffer<int> &baseline_flags, const MemoryBuffer<float> &antenna_weights,
                  const MemoryBuffer<double> &frequencies, double delta_u, double delta_v, int n_pixels,
                  double min_uv, Polarization pol, MemoryBuffer<float> &grids_counters,
                  MemoryBuffer<std::complex<float>> &grids) {
    check(bgi_gridding_gpu(reinterpret_cast<const float *>(xcorr.data()), xcorr.obsInfo.nAntennas,
                           xcorr.nFrequencies, xcorr.integration_intervals(), u_gpu.data(), v_gpu.data(), 1,
                           baseline_flags.data(), antenna_weights.data(), frequencies.data(), delta_u, delta_v,
                           n_pixels, min_uv, static_cast<int>(pol), BGI_COUNTERS_FIRST_INTERVAL,
                           grids_counters.data(), reinterpret_cast<float *>(grids.data()), nullptr));
}

// src/gpu/gpu_utils.cpp:62, :128, :153
void vector_sum_gpu(float *data_gpu, int image_size, int n_images, MemoryBuffer<float> &sum_gpu) {
    sum_gpu.to_gpu();
    check(bgi_vector_sum_gpu(data_gpu, image_size, n_images, sum_gpu.data(), nullptr));
}
void fft_shift_and_norm_gpu(gpufftComplex *data_gpu, int x, int y, int n_images, MemoryBuffer<float> &fnorm) {
    if (x % 2) throw std::invalid_argument{"function fft_shift_gpu currently only handles even image size"};
    check(bgi_fft_shift_and_norm_gpu(reinterpret_cast<float *>(data_gpu), x, y, n_images, fnorm.data(),
                                     (int)fnorm.size(), nullptr));
}
Images image_averaging_gpu(const Images &images) {
    MemoryBuffer<std::complex<float>> avg{images.image_size(), MemoryType::DEVICE};
    check(bgi_image_averaging_gpu(reinterpret_cast<const float *>(images.data()), images.image_size(),
                                  images.size(), reinterpret_cast<float *>(avg.data()), nullptr));
    return {std::move(avg), images.obsInfo, 1, 1, images.side_size, images.ra_deg, images.dec_deg,
            images.pixscale_ra, images.pixscale_dec};
}
