// Minimal host-only stand-in for astroio's MemoryBuffer<T>, enough to compile the reference
// imager's CPU sources for the oracle cross-check.  Not product code.
#ifndef BGI_SHIM_MEMORY_BUFFER_HPP
#define BGI_SHIM_MEMORY_BUFFER_HPP
#include <cstddef>
#include <cstring>
#include <vector>
#include <complex>
#include <string>
#include <fstream>
#include <stdexcept>
#include <iostream>

enum class MemoryType { HOST, DEVICE };

template <typename T>
class MemoryBuffer {
    std::vector<T> v_;
public:
    MemoryBuffer() {}
    explicit MemoryBuffer(size_t n, MemoryType = MemoryType::HOST) : v_(n) {}
    MemoryBuffer(MemoryBuffer &&o) noexcept : v_(std::move(o.v_)) {}
    MemoryBuffer &operator=(MemoryBuffer &&o) noexcept { v_ = std::move(o.v_); return *this; }
    MemoryBuffer(const MemoryBuffer &) = delete;
    void allocate(size_t n, MemoryType = MemoryType::HOST) { v_.assign(n, T{}); }
    size_t size() const { return v_.size(); }
    T *data() { return v_.data(); }
    const T *data() const { return v_.data(); }
    T &operator[](size_t i) { return v_[i]; }
    const T &operator[](size_t i) const { return v_[i]; }
    explicit operator bool() const { return !v_.empty(); }
    void to_gpu() {}
    void to_cpu() {}
    bool on_gpu() const { return false; }
};
#endif
