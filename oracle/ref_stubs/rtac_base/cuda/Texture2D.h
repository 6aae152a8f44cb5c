// Host stand-in for rtac_base cuda::Texture2D<T>: keeps the last image and
// the filter / wrap settings so that the probe can print the table the
// reference's Directivity builders upload.
#pragma once
#include <vector>
typedef unsigned long long cudaTextureObject_t;
namespace rtac { namespace cuda {
template <typename T>
struct Texture2D {
    enum FilterMode { FilterPoint, FilterLinear };
    enum WrapMode { WrapClamp, WrapMirror, WrapBorder };
    unsigned int width = 0, height = 0;
    std::vector<T> image;
    int filter = -1, wrap = -1;
    void set_filter_mode(FilterMode m, bool) { filter = m; }
    void set_wrap_mode(WrapMode m, bool) { wrap = m; }
    void set_image(unsigned int w, unsigned int h, const T* d) { width = w; height = h; image.assign(d, d + (size_t)w * h); }
    template <typename C> void set_image(unsigned int w, unsigned int h, const C& c) { width = w; height = h; image.assign(c.begin(), c.end()); }
    cudaTextureObject_t texture() const { return 0; }
};
}}
