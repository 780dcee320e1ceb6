// Minimal host-only stand-in for astroio's Images.  Not product code.
#ifndef BGI_SHIM_IMAGES_HPP
#define BGI_SHIM_IMAGES_HPP
#include "astroio.hpp"
class Images : public MemoryBuffer<std::complex<float>> {
public:
    ObservationInfo obsInfo;
    unsigned int n_intervals, n_channels, side_size;
    double ra_deg, dec_deg, pixscale_ra, pixscale_dec;
    Images(MemoryBuffer<std::complex<float>> &&b, const ObservationInfo &oi, unsigned int ni,
           unsigned int nc, unsigned int side, double ra, double dec, double pra, double pdec)
        : MemoryBuffer<std::complex<float>>(std::move(b)), obsInfo(oi), n_intervals(ni),
          n_channels(nc), side_size(side), ra_deg(ra), dec_deg(dec), pixscale_ra(pra),
          pixscale_dec(pdec) {}
    size_t image_size() const { return size_t(side_size) * side_size; }
};
#endif
