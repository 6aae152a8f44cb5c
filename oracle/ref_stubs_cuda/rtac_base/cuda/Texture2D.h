// Stand-in for rtac_base cuda::Texture2D<T>: a texture-object handle; the
// harness creates the texture (normalized coordinates, linear filter,
// border addressing, as src/SensorInstance2D.cu:14-15 configures it).
#pragma once
#include <rtac_base/cuda_defines.h>
namespace rtac { namespace cuda {
template <typename T> class Texture2D {
    cudaTextureObject_t tex_ = 0;
public:
    void set_filter_mode(cudaTextureFilterMode, bool) {}
    void set_wrap_mode(cudaTextureAddressMode, bool) {}
    void set_image(unsigned int, unsigned int, const T*) {}
    cudaTextureObject_t texture() const { return tex_; }
};
}}
