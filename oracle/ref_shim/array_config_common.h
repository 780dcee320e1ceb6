// Stand-in for msfitslib's antenna/input record, with the fields the imager reads.
#ifndef BGI_SHIM_ARRAY_CONFIG_COMMON_H
#define BGI_SHIM_ARRAY_CONFIG_COMMON_H
#include <string>
class InputMapping {
public:
    int input {-1}, antenna {-1};
    std::string szAntName;
    char pol {'U'};
    int delta {0}, flag {0};
    double x {0}, y {0}, z {0};
    double cableLenDelta {0};
};
#endif
