// Host stand-in for rtac_base Image<T, Container> with the members the
// reference's sensor headers call: (width, height[, container])
// construction, width / height, resize({width, height}), data().
#pragma once
#include <cstddef>
#include <vector>
#include <rtac_base/containers/HostVector.h>
#include <rtac_base/cuda/CudaVector.h>
namespace rtac {
struct ImageShape { unsigned int width, height; };
template <typename T> struct ImageView { unsigned int width_ = 0, height_ = 0; T* data_ = nullptr; };
template <typename T, template <typename> class Container = HostVector>
class Image {
    ImageShape shape_{0, 0};
    std::vector<T> data_;
public:
    using Shape = ImageShape;
    Image() = default;
    Image(unsigned int w, unsigned int h) : shape_{w, h}, data_((std::size_t)w * h) {}
    template <typename C> Image(unsigned int w, unsigned int h, const C&) : shape_{w, h}, data_((std::size_t)w * h) {}
    void resize(const Shape& s) { shape_ = s; data_.resize((std::size_t)s.width * s.height); }
    unsigned int width() const { return shape_.width; }
    unsigned int height() const { return shape_.height; }
    T& operator()(unsigned int h, unsigned int w) { return data_[(std::size_t)h * shape_.width + w]; }
    const T& operator()(unsigned int h, unsigned int w) const { return data_[(std::size_t)h * shape_.width + w]; }
    T* data() { return data_.data(); }
    const T* data() const { return data_.data(); }
};
}
