// Stand-ins for rtac_base VectorView<T> (size + pointer, element access on
// the device) and cuda::CudaVector<T> (a device buffer handle; the harness
// owns the memory, so resizing only records the size).
#pragma once
#include <cstddef>
#include <vector>
#include <rtac_base/cuda_defines.h>
namespace rtac {
template <typename T> struct VectorView {
    std::size_t size_;
    T* data_;
    RTAC_HOSTDEVICE std::size_t size() const { return size_; }
    RTAC_HOSTDEVICE T& operator[](std::size_t i) const { return data_[i]; }
};
namespace cuda {
template <typename T> struct CudaVector {
    T* data_ = nullptr;
    std::size_t size_ = 0;
    CudaVector() = default;
    explicit CudaVector(const std::vector<T>& host) : size_(host.size()) {}
    T* data() { return data_; }
    const T* data() const { return data_; }
    std::size_t size() const { return size_; }
    void resize(std::size_t n) { size_ = n; }
    VectorView<T> view() { return VectorView<T>{size_, data_}; }
};
}
}
