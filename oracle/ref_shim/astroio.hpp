// Minimal host-only stand-ins for astroio's ObservationInfo and Visibilities (layout
// [interval][channel][baseline][pol], baseline = a1*(a1+1)/2 + a2 for a1 >= a2), enough to
// compile the reference imager's CPU sources for the oracle cross-check.  Not product code.
#ifndef BGI_SHIM_ASTROIO_HPP
#define BGI_SHIM_ASTROIO_HPP
#include "memory_buffer.hpp"
#include <complex>


struct ObservationInfo {
    unsigned int nAntennas {0};
    double frequencyResolution {0};    // MHz
    double coarseChannelBandwidth {0}; // MHz
    int coarseChannel {0};
    double startTime {0};
};

class Visibilities {
public:
    ObservationInfo obsInfo;
    unsigned int nIntervals {1};
    unsigned int nFrequencies {1};
    unsigned int nAveragedChannels {1};
    MemoryBuffer<std::complex<float>> buf;

    Visibilities() {}
    Visibilities(const ObservationInfo &oi, unsigned int n_int, unsigned int n_freq)
        : obsInfo(oi), nIntervals(n_int), nFrequencies(n_freq),
          buf(size_t(n_int) * n_freq * n_baselines() * 4) {}
    size_t n_baselines() const { return size_t(obsInfo.nAntennas) * (obsInfo.nAntennas + 1) / 2; }
    unsigned int integration_intervals() const { return nIntervals; }
    std::complex<float> *data() { return buf.data(); }
    const std::complex<float> *data() const { return buf.data(); }
    std::complex<float> *at(size_t t, size_t ch, size_t baseline) {
        return buf.data() + ((t * nFrequencies + ch) * n_baselines() + baseline) * 4;
    }
    std::complex<float> *at(size_t t, size_t ch, size_t a1, size_t a2) {
        return at(t, ch, a1 * (a1 + 1) / 2 + a2);
    }
    bool on_gpu() const { return false; }
    void to_cpu() {}
    void to_gpu() {}
};
#endif
