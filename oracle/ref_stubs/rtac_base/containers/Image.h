// Host stand-in for rtac_base Image<T, Container>: a row-major height x width
// array with (h, w) indexing, enough for the reference's Directivity table
// builders (src/Directivity.cpp) to compile and run on the host.
#pragma once
#include <cstddef>
#include <vector>
#include <rtac_base/containers/HostVector.h>
#include <rtac_base/cuda/CudaVector.h>
namespace rtac {
struct ImageShape { unsigned int width, height; };
template <typename T, template <typename> class Container = HostVector>
class Image {
    ImageShape shape_{0, 0};
    std::vector<T> data_;
public:
    using Shape = ImageShape;
    Image() = default;
    Image(unsigned int w, unsigned int h) : shape_{w, h}, data_((size_t)w * h) {}
    Image(const Shape& s, const std::vector<T>& d) : shape_(s), data_(d) { data_.resize((size_t)s.width * s.height, d.empty() ? T() : d[0]); }
    unsigned int width() const { return shape_.width; }
    unsigned int height() const { return shape_.height; }
    T& operator()(unsigned int h, unsigned int w) { return data_[(size_t)h * shape_.width + w]; }
    const T& operator()(unsigned int h, unsigned int w) const { return data_[(size_t)h * shape_.width + w]; }
    T* data() { return data_.data(); }
    const T* data() const { return data_.data(); }
    const std::vector<T>& container() const { return data_; }
};
}
