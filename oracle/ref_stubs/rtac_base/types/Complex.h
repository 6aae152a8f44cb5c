// Host stand-in for rtac_base Complex: the reference only needs real/imag,
// construction from (re, im) and arithmetic, which std::complex provides.
#pragma once
#include <complex>
#include <rtac_base/cuda_defines.h>
namespace rtac { template <typename T> using Complex = std::complex<T>; }
