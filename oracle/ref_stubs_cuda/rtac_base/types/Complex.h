// Stand-in for rtac_base Complex<T>: two components, construction from
// (re, im), real()/imag() accessors and setters, +=, complex and scalar
// products, make_complex(float2).
#pragma once
#include <rtac_base/cuda_defines.h>
namespace rtac {
template <typename T> struct Complex {
    T re_, im_;
    Complex() = default;
    RTAC_HOSTDEVICE constexpr Complex(T r, T i = T(0)) : re_(r), im_(i) {}
    RTAC_HOSTDEVICE T real() const { return re_; }
    RTAC_HOSTDEVICE T imag() const { return im_; }
    RTAC_HOSTDEVICE void real(T v) { re_ = v; }
    RTAC_HOSTDEVICE void imag(T v) { im_ = v; }
    RTAC_HOSTDEVICE Complex& operator+=(const Complex& o) { re_ += o.re_; im_ += o.im_; return *this; }
};
template <typename T>
RTAC_HOSTDEVICE inline Complex<T> operator*(const Complex<T>& a, const Complex<T>& b)
{
    return Complex<T>(a.re_ * b.re_ - a.im_ * b.im_, a.re_ * b.im_ + a.im_ * b.re_);
}
template <typename T>
RTAC_HOSTDEVICE inline Complex<T> operator*(const Complex<T>& a, T s) { return Complex<T>(a.re_ * s, a.im_ * s); }
RTAC_HOSTDEVICE inline Complex<float> make_complex(float2 v) { return Complex<float>(v.x, v.y); }
}
