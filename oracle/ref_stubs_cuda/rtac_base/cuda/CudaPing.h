// Stand-in for rtac_base cuda::CudaPing2D<T>: the ping's image view.
#pragma once
#include <rtac_base/containers/Image.h>
namespace rtac { namespace cuda {
template <typename T> struct CudaPing2D {
    ImageView<T> view_{};
    CudaPing2D() = default;
    template <class Ranges, class Bearings, class Data>
    CudaPing2D(const Ranges&, const Bearings&, const Data&) {}
    unsigned int width() const { return view_.width_; }
    unsigned int height() const { return view_.height_; }
    ImageView<T> image_view() const { return view_; }
};
}}
