// Stand-in for rtac_base cuda::TextureVectorView<T>: element i of the table
// (the bearings; read exactly, as the reference indexes it by bearing).
#pragma once
#include <cstddef>
#include <rtac_base/cuda_defines.h>
namespace rtac { namespace cuda {
template <typename T> struct TextureVectorView {
    std::size_t size_;
    const T* data_;
    RTAC_HOSTDEVICE std::size_t size() const { return size_; }
    RTAC_HOSTDEVICE T operator[](std::size_t i) const { return data_[i]; }
};
}}
