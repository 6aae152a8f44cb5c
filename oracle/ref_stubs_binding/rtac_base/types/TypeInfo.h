// Stand-in for rtac_base types/TypeInfo.h (not vendored with the reference):
// the scalar traits and the TypeError exception the reference's sensor
// headers name (rtac_simulation/SensorInstance.h, SensorInstance2D.h).
#pragma once
#include <complex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
namespace rtac {
enum ScalarId { RTAC_FLOAT, RTAC_CFLOAT, RTAC_OTHER };
template <typename T> struct IsRtacComplex : std::false_type {};
template <typename T> struct IsRtacComplex<std::complex<T>> : std::true_type {};
template <typename T> struct IsRtacScalar
    : std::integral_constant<bool, std::is_arithmetic<T>::value || IsRtacComplex<T>::value> {};
template <typename T> struct GetScalarId {
    static constexpr ScalarId value = std::is_same<T, float>::value ? RTAC_FLOAT
                                    : std::is_same<T, std::complex<float>>::value ? RTAC_CFLOAT : RTAC_OTHER;
};
struct TypeError : std::runtime_error {
    TypeError() : std::runtime_error("rtac TypeError") {}
    template <typename V> TypeError& operator<<(const V&) { return *this; }
};
}
