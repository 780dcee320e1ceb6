// src/gpu/pacer_imager_gb300.cpp -- the GB300 counterpart of CPacerImagerHip
// (src/gpu/pacer_imager_hip.h:12-58, src/gpu/pacer_imager_hip.cpp): the same constructor and the
// same virtuals of CPacerImager, so CPacerImager::run() / grid() drive it unchanged, each
// virtual a call of the imaging C ABI on the imager's resident device buffers.  The FFT is the
// library's own (bgi_fft_inverse_gpu) in place of the cuFFT plan.  Errors throw, as the
// reference does.
#include <cmath>
#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include <blink_imager_gb300.h>
#include <cuda_runtime.h>

#include "../pacer_imager.h"

namespace {
void check(int status) {
    if (status != BGI_OK) throw std::runtime_error(bgi_last_error());
}
void check_cuda(cudaError_t e) {
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}
}  // namespace

class CPacerImagerGb300 : public CPacerImager {
protected:
    MemoryBuffer<double> frequencies_gpu;
    MemoryBuffer<float> fnorm;
    MemoryBuffer<float> u_gpu, v_gpu, w_gpu;
    MemoryBuffer<int> baseline_flags_gpu;

    // src/gpu/pacer_imager_hip.cpp:21-33: the baseline flags of the current antenna flags
    void UpdateBaselineFlags(int n_ant) {
        const size_t n_baselines = (size_t)n_ant * (n_ant + 1) / 2;
        if (!baseline_flags_gpu) baseline_flags_gpu.allocate(n_baselines, MemoryType::DEVICE);
        UpdateFlags();
        check_cuda(cudaMemcpy(baseline_flags_gpu.data(), m_FlaggedBaselines.data(), sizeof(int) * n_baselines,
                              cudaMemcpyHostToDevice));
    }

    void upload_frequencies(const Visibilities &xcorr) {
        if (!frequencies_gpu) frequencies_gpu.allocate(xcorr.nFrequencies, MemoryType::DEVICE);
        check_cuda(cudaMemcpy(frequencies_gpu.data(), frequencies.data(), sizeof(double) * frequencies.size(),
                              cudaMemcpyHostToDevice));
    }

    // src/gpu/pacer_imager_hip.cpp:36-66: grids and per-channel counters of interval 0
    void gridding(Visibilities &xcorr) override {
        const int n_ant = (int)xcorr.obsInfo.nAntennas;
        const size_t n_baselines = (size_t)n_ant * (n_ant + 1) / 2;
        const size_t image_size = (size_t)n_pixels * n_pixels;
        const size_t n_images = n_gridded_channels * n_gridded_intervals;
        UpdateBaselineFlags(n_ant);
        if (!u_gpu) {
            u_gpu.allocate(n_baselines, MemoryType::DEVICE);
            v_gpu.allocate(n_baselines, MemoryType::DEVICE);
        }
        check_cuda(cudaMemcpy(u_gpu.data(), u_cpu.data(), sizeof(float) * n_baselines, cudaMemcpyHostToDevice));
        check_cuda(cudaMemcpy(v_gpu.data(), v_cpu.data(), sizeof(float) * n_baselines, cudaMemcpyHostToDevice));
        if (!grids_counters) {
            grids_counters.allocate(image_size * xcorr.nFrequencies, MemoryType::DEVICE);
            check_cuda(cudaMemset(grids_counters.data(), 0, grids_counters.size() * sizeof(float)));
        }
        if (!grids) {
            grids.allocate(image_size * n_images, MemoryType::DEVICE);
            check_cuda(cudaMemset(grids.data(), 0, grids.size() * sizeof(std::complex<float>)));
        }
        upload_frequencies(xcorr);
        xcorr.to_gpu();
        check(bgi_gridding_gpu(reinterpret_cast<const float *>(xcorr.data()), n_ant, (int)xcorr.nFrequencies,
                               (int)xcorr.integration_intervals(), u_gpu.data(), v_gpu.data(), 1,
                               baseline_flags_gpu.data(), nullptr, frequencies_gpu.data(), delta_u, delta_v,
                               n_pixels, min_uv, static_cast<int>(pol_to_image), BGI_COUNTERS_FIRST_INTERVAL,
                               grids_counters.data(), reinterpret_cast<float *>(grids.data()), nullptr));
    }

    // src/gpu/pacer_imager_hip.cpp:131-141
    void ApplyGeometricCorrections(Visibilities &xcorr, MemoryBuffer<float> &w, MemoryBuffer<double> &freqs) override {
        (void)freqs;
        const int n_ant = (int)xcorr.obsInfo.nAntennas;
        const size_t n_baselines = (size_t)n_ant * (n_ant + 1) / 2;
        upload_frequencies(xcorr);
        if (!w_gpu) w_gpu.allocate(n_baselines, MemoryType::DEVICE);
        check_cuda(cudaMemcpy(w_gpu.data(), w.data(), sizeof(float) * n_baselines, cudaMemcpyHostToDevice));
        xcorr.to_gpu();
        check(bgi_apply_geometric_corrections_gpu(reinterpret_cast<float *>(xcorr.data()), n_ant,
                                                  (int)xcorr.nFrequencies, (int)xcorr.integration_intervals(),
                                                  w_gpu.data(), 1, frequencies_gpu.data(), nullptr));
    }

    // src/gpu/pacer_imager_hip.cpp:144-148
    void ApplyCableCorrections(Visibilities &xcorr, MemoryBuffer<double> &cables, MemoryBuffer<double> &freqs) override {
        (void)freqs;
        upload_frequencies(xcorr);
        cables.to_gpu();
        xcorr.to_gpu();
        check(bgi_apply_cable_lengths_corrections_gpu(reinterpret_cast<float *>(xcorr.data()),
                                                      (int)xcorr.obsInfo.nAntennas, (int)xcorr.nFrequencies,
                                                      (int)xcorr.integration_intervals(), cables.data(),
                                                      frequencies_gpu.data(), nullptr));
    }

public:
    CPacerImagerGb300(const std::string metadata_file, int n_pixels, const std::vector<int> &flagged_antennas,
                      bool average_images = false, Polarization pol_to_image = Polarization::XX,
                      float oversampling_factor = 2.0f, double min_uv = -std::numeric_limits<double>::infinity(),
                      double max_uv = std::numeric_limits<double>::infinity(), const char *weighting = "")
        : CPacerImager(metadata_file, n_pixels, flagged_antennas, average_images, pol_to_image, oversampling_factor,
                       min_uv, max_uv, weighting) {}

    // src/gpu/pacer_imager_hip.cpp:70-127: inverse FFT, per-channel weight sums, fftshift and
    // normalisation, grids cleared for the next block
    Images image(ObservationInfo &obs_info) override {
        if (!grids_counters || !grids) throw std::runtime_error{"Grids are not initialised and cannot be imaged."};
        const size_t image_size = (size_t)n_pixels * n_pixels;
        const size_t n_images = n_gridded_channels * n_gridded_intervals;
        MemoryBuffer<std::complex<float>> images_buffer(image_size * n_images, MemoryType::DEVICE);
        check(bgi_fft_inverse_gpu(reinterpret_cast<const float *>(grids.data()),
                                  reinterpret_cast<float *>(images_buffer.data()), n_pixels, (int)n_images, nullptr));
        if (!fnorm) fnorm.allocate(n_gridded_channels, MemoryType::DEVICE);
        check(bgi_vector_sum_gpu(grids_counters.data(), (int64_t)image_size, (int)n_gridded_channels, fnorm.data(),
                                 nullptr));
        check(bgi_fft_shift_and_norm_gpu(reinterpret_cast<float *>(images_buffer.data()), n_pixels, n_pixels,
                                         (int)n_images, fnorm.data(), (int)n_gridded_channels, nullptr));
        check_cuda(cudaMemset(grids_counters.data(), 0, grids_counters.size() * sizeof(float)));
        check_cuda(cudaMemset(grids.data(), 0, grids.size() * sizeof(std::complex<float>)));
        const double ra_deg = m_MetaData.raHrs * 15.0, dec_deg = m_MetaData.decDegs;
        const double pixscale_ra = (1.0 / (oversampling_factor * u_max)) * (180.0 / M_PI);
        const double pixscale_dec = (1.0 / (oversampling_factor * v_max)) * (180.0 / M_PI);
        Images images{std::move(images_buffer), obs_info, static_cast<unsigned int>(n_gridded_intervals),
                      static_cast<unsigned int>(n_gridded_channels), static_cast<unsigned int>(n_pixels), ra_deg,
                      dec_deg, pixscale_ra, pixscale_dec};
        if (average_images) {
            MemoryBuffer<std::complex<float>> avg(image_size, MemoryType::DEVICE);
            check(bgi_image_averaging_gpu(reinterpret_cast<const float *>(images.data()), (int64_t)image_size,
                                          (int)n_images, reinterpret_cast<float *>(avg.data()), nullptr));
            return {std::move(avg), obs_info, 1, 1, static_cast<unsigned int>(n_pixels), ra_deg, dec_deg,
                    pixscale_ra, pixscale_dec};
        }
        return images;
    }
};
