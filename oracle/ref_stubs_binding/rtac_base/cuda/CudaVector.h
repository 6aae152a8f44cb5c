// Host stand-in for rtac_base CudaVector<T> and VectorView<T> with the
// members the reference's sensor headers call (data(), size(), resize()).
// The binding compile never runs: host storage stands for device storage.
#pragma once
#include <cstddef>
#include <vector>
#include <rtac_base/cuda/vec_math.h>
namespace rtac {
template <typename T> struct VectorView {
    std::size_t size_;
    T* data_;
    VectorView(std::size_t s = 0, T* d = nullptr) : size_(s), data_(d) {}
    std::size_t size() const { return size_; }
};
namespace cuda {
template <typename T> struct CudaVector {
    std::vector<T> data_;
    CudaVector() = default;
    explicit CudaVector(std::size_t n) : data_(n) {}
    void resize(std::size_t n) { data_.resize(n); }
    std::size_t size() const { return data_.size(); }
    T* data() { return data_.data(); }
    const T* data() const { return data_.data(); }
};
}
}
