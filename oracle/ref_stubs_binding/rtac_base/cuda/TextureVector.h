// Host stand-in for rtac_base cuda::TextureVector<T> / TextureVectorView<T>:
// a table built from a host vector and its view (size and elements).
#pragma once
#include <cstddef>
#include <vector>
namespace rtac { namespace cuda {
template <typename T> struct TextureVectorView {
    std::size_t size_ = 0;
    const T* data_ = nullptr;
    std::size_t size() const { return size_; }
    T operator[](std::size_t i) const { return data_[i]; }
};
template <typename T> struct TextureVector {
    std::vector<T> data_;
    TextureVector() = default;
    template <typename V> explicit TextureVector(const V& v) : data_(v.begin(), v.end()) {}
    TextureVectorView<T> view() const { return TextureVectorView<T>{data_.size(), data_.data()}; }
};
}}
