// Stand-in for rtac_base signal_helpers: Waveform.h includes it and
// Directivity.cpp names signal::SincFunction (used only by
// Directivity::from_sinc_parameters, which the probe never calls).
#pragma once
#include <vector>
namespace rtac { namespace signal {
template <typename T> struct SincFunction {
    std::vector<T> f_;
    SincFunction(T, T, unsigned int = 8) : f_(1, T(1)) {}
    SincFunction(T, unsigned int = 8) : f_(1, T(1)) {}
    std::size_t size() const { return f_.size(); }
    const std::vector<T>& function() const { return f_; }
};
}}
