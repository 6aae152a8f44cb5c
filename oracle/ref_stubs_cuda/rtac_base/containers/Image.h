// Stand-ins for rtac_base ImageView<T> (row-major width x height view with
// (h, w) indexing on the device) and Image<T, Container>.
#pragma once
#include <cstddef>
#include <vector>
#include <rtac_base/cuda_defines.h>
#include <rtac_base/containers/HostVector.h>
#include <rtac_base/cuda/CudaVector.h>
namespace rtac {
struct ImageShape { unsigned int width, height; };
template <typename T> struct ImageView {
    unsigned int width_, height_;
    T* data_;
    RTAC_HOSTDEVICE T& operator()(unsigned int h, unsigned int w) const { return data_[(std::size_t)h * width_ + w]; }
};
template <typename T, template <typename> class Container = HostVector>
class Image {
    ImageShape shape_{0, 0};
    Container<T> data_;
public:
    Image() = default;
    Image(unsigned int w, unsigned int h) : shape_{w, h} { data_.resize((std::size_t)w * h); }
    unsigned int width() const { return shape_.width; }
    unsigned int height() const { return shape_.height; }
    void resize(const ImageShape& s) { shape_ = s; data_.resize((std::size_t)s.width * s.height); }
    T& operator()(unsigned int h, unsigned int w) { return data_.data()[(std::size_t)h * shape_.width + w]; }
    T* data() { return data_.data(); }
    const T* data() const { return data_.data(); }
    const Container<T>& container() const { return data_; }
    ImageView<T> view() { return ImageView<T>{shape_.width, shape_.height, data_.data()}; }
};
}
