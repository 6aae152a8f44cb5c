// Host stand-in for rtac_base CudaVector<T> and VectorView<T>. Only the type
// names are needed: the probe never instantiates the device containers.
#pragma once
#include <cstddef>
#include <vector>
#include <rtac_base/cuda/vec_math.h>
namespace rtac {
template <typename T> struct VectorView {
    std::size_t size_; T* data_;
    VectorView(std::size_t s = 0, T* d = nullptr) : size_(s), data_(d) {}
};
namespace cuda {
template <typename T> struct CudaVector {
    std::vector<T> data_;
    void resize(std::size_t n) { data_.resize(n); }
    std::size_t size() const { return data_.size(); }
};
}
}
