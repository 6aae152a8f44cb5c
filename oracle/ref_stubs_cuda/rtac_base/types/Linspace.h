// Stand-in for rtac_base Linspace<T>: `size` values from lower to upper,
// element i = lower + i * (upper - lower) / (size - 1) in T arithmetic (the
// formula the oracle and this project's receiver use for range bin centres).
#pragma once
#include <rtac_base/cuda_defines.h>
namespace rtac {
template <typename T> struct Linspace {
    T lower_, upper_;
    unsigned int size_;
    RTAC_HOSTDEVICE unsigned int size() const { return size_; }
    RTAC_HOSTDEVICE T resolution() const { return (upper_ - lower_) / (T)(size_ - 1); }
    // Separate rounded multiply and add (no contraction), as on the host.
    RTAC_HOSTDEVICE T operator[](unsigned int i) const
    {
#ifdef __CUDA_ARCH__
        return __fadd_rn(lower_, __fmul_rn((T)i, (upper_ - lower_) / (T)(size_ - 1)));
#else
        return lower_ + (T)i * ((upper_ - lower_) / (T)(size_ - 1));
#endif
    }
};
}
