// Stand-in for the reference's rtac_simulation/SensorInstance1D.h, placed
// before the reference's include directory so that src/SensorInstance1D.cu
// compiles without the sensor class hierarchy (poses, receivers, binner,
// factories), which needs the non-vendored rtac_base. It declares only what
// that file's definitions use: the PSF lookup KernelView1D
// (rtac_simulation/ReductionKernel.h) and the sample records are the
// reference's own headers. Nothing here runs: the harness launches
// do_sparse_convolve_1d_f itself.
#pragma once
#include <rtac_base/cuda/TextureVector.h>
#include <rtac_base/containers/HostVector.h>
#include <rtac_simulation/SensorInstance.h>

namespace rtac { namespace simulation {

class SensorInstance1D : public SensorInstance {
protected:
    SensorInfo::ConstPtr info_;
    cuda::Texture2D<float2> waveformData_;
    SensorInstance1D(const SensorInfo::ConstPtr& info, const Pose& pose, float soundCelerity);
    void generate_psf_data();
    void do_reduce(cuda::CudaVector<Complex<float>>& out,
                   const cuda::CudaVector<VectorView<const SimSample1D>>& bins) const;
public:
    unsigned int size() const { return ranges_.size(); }
    KernelView1D<Complex<float>> kernel() const;
};

}}
