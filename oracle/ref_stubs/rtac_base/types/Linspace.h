// Host stand-in for rtac_base Linspace<T>: bounds [lower, upper], size and the
// uniform resolution (upper - lower) / (size - 1).
#pragma once
#include <rtac_base/types/Bounds.h>
namespace rtac {
template <typename T> struct Linspace {
    T lower_, upper_; unsigned int size_;
    Linspace() = default;
    Linspace(T l, T u, unsigned int n) : lower_(l), upper_(u), size_(n) {}
    unsigned int size() const { return size_; }
    Bounds<T> bounds() const { return Bounds<T>{lower_, upper_}; }
    T resolution() const { return (upper_ - lower_) / (size_ - 1); }
};
}
