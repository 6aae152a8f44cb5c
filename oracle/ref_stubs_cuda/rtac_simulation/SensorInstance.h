// Stand-in for the reference's rtac_simulation/SensorInstance.h, placed
// before the reference's include directory so that src/SensorInstance2D.cu
// compiles without the rest of the sensor class hierarchy (SensorInfo
// factories, poses, receivers, pings), which needs the non-vendored
// rtac_base. It declares only what that file's definitions use (and what
// src/SensorInstance1D.cu uses, through the SensorInstance1D stand-in); the sample
// records (rtac_simulation/Sample.h) and the PSF lookup KernelView2D
// (rtac_simulation/ReductionKernel.h) are the reference's own headers.
// Nothing here runs: the harness launches do_sparse_convolve_2d_f itself.
#pragma once
#include <memory>
#include <vector>
#include <rtac_base/cuda_defines.h>
#include <rtac_base/types/Complex.h>
#include <rtac_base/types/Linspace.h>
#include <rtac_base/containers/Image.h>
#include <rtac_base/cuda/CudaVector.h>
#include <rtac_base/cuda/Texture2D.h>
#include <rtac_base/cuda/TextureVector.h>
#include <rtac_base/cuda/CudaPing.h>
#include <rtac_simulation/Sample.h>
#include <rtac_simulation/ReductionKernel.h>

namespace rtac { namespace simulation {

struct Pose {};

struct Waveform {
    using Ptr = std::shared_ptr<Waveform>;
    std::vector<Complex<float>> taps_;
    float duration_ = 0.0f;
    unsigned int size() const { return (unsigned int)taps_.size(); }
    Complex<float> operator[](unsigned int i) const { return taps_[i]; }
    float duration() const { return duration_; }
};

struct BeamDirectivity {
    using ConstPtr = std::shared_ptr<const BeamDirectivity>;
    std::vector<float> values_;
    float span_ = 0.0f;
    unsigned int size() const { return (unsigned int)values_.size(); }
    float operator[](unsigned int i) const { return values_[i]; }
    float span() const { return span_; }
};

// The 1D sensor's info: only the type is used by src/SensorInstance1D.cu.
struct SensorInfo {
    using ConstPtr = std::shared_ptr<const SensorInfo>;
};

struct SensorInfo2D {
    using ConstPtr = std::shared_ptr<const SensorInfo2D>;
    BeamDirectivity::ConstPtr beam_;
    std::vector<float> bearings_;
    cuda::TextureVectorView<float> bearings_view_{};
    BeamDirectivity::ConstPtr beam_directivity() const { return beam_; }
    const std::vector<float>& bearings() const { return bearings_; }
    cuda::TextureVectorView<float> bearings_view() const { return bearings_view_; }
};

class SensorInstance {
protected:
    Waveform::Ptr waveform_;
    float soundCelerity_;
    Linspace<float> ranges_{};
public:
    SensorInstance(const SensorInfo2D::ConstPtr&, const Pose&, float c) : soundCelerity_(c) {}
    SensorInstance(const SensorInfo::ConstPtr&, const Pose&, float c) : soundCelerity_(c) {}
    const Linspace<float>& ranges() const { return ranges_; }
};

class SensorInstance2D : public SensorInstance {
    SensorInfo2D::ConstPtr info_;
    cuda::Texture2D<float2> psfData_;
public:
    SensorInstance2D(const SensorInfo2D::ConstPtr& info, const Pose& pose, float soundCelerity);
    void generate_psf_data();
    KernelView2D<Complex<float>> kernel() const;
    unsigned int width() const { return (unsigned int)info_->bearings().size(); }
    unsigned int height() const { return ranges_.size(); }
    const std::vector<float>& bearings() const { return info_->bearings(); }
    cuda::TextureVectorView<float> bearings_view() const { return info_->bearings_view(); }
    BeamDirectivity::ConstPtr beam_directivity() const { return info_->beam_directivity(); }
    void do_reduce(Image<Complex<float>, cuda::CudaVector>& out,
                   const cuda::CudaVector<VectorView<const SimSample2D>>& bins) const;
    void do_reduce(cuda::CudaPing2D<Complex<float>>& out,
                   const cuda::CudaVector<VectorView<const SimSample2D>>& bins) const;
};

class SensorInstance2D_Complex : public SensorInstance2D {
    Image<Complex<float>, cuda::CudaVector> sensorOutput_;
public:
    using SensorInstance2D::SensorInstance2D;
    cuda::CudaPing2D<Complex<float>> get_ping() const;
};

}}
