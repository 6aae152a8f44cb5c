// Stand-in for rtac_base cuda::CudaPing2D<T> with the members the reference
// calls on it (include/rtac_simulation/SensorInstance2D.h:86-88,116,139):
// construction from (ranges, bearings), set_bearings / set_ranges, and
// ping_data_container() (a CudaVector<T> of width x height cells).
#pragma once
#include <rtac_base/cuda/CudaVector.h>
#include <rtac_base/types/Linspace.h>
#include <rtac_base/containers/HostVector.h>
namespace rtac { namespace cuda {
template <typename T> class CudaPing2D {
    Linspace<float> ranges_{};
    HostVector<float> bearings_;
    CudaVector<T> data_;
public:
    CudaPing2D() = default;
    CudaPing2D(const Linspace<float>& ranges, const HostVector<float>& bearings) : ranges_(ranges), bearings_(bearings)
    {
        data_.resize((std::size_t)ranges.size() * bearings.size());
    }
    void set_bearings(const HostVector<float>& bearings, bool resize)
    {
        bearings_ = bearings;
        if(resize) data_.resize((std::size_t)ranges_.size() * bearings_.size());
    }
    void set_ranges(const Linspace<float>& ranges, bool resize)
    {
        ranges_ = ranges;
        if(resize) data_.resize((std::size_t)ranges_.size() * bearings_.size());
    }
    const CudaVector<T>& ping_data_container() const { return data_; }
    CudaVector<T>& ping_data_container() { return data_; }
};
}}
