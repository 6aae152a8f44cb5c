// Host stand-in for rtac_base Bounds<T>: lower/upper plus length().
#pragma once
#include <ostream>
namespace rtac {
template <typename T> struct Bounds {
    T lower, upper;
    T length() const { return upper - lower; }
};
}
template <typename T>
inline std::ostream& operator<<(std::ostream& os, const rtac::Bounds<T>& b) {
    return os << "[" << b.lower << ", " << b.upper << "]";
}
