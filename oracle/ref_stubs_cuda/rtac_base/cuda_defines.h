// Device-capable stand-in for the non-vendored rtac_base header of the same
// name. Together with the other files under oracle/ref_stubs_cuda it lets the
// reference's own src/SensorInstance2D.cu (the do_sparse_convolve_2d_f kernel
// and the KernelView2D texture lookup of include/rtac_simulation/
// ReductionKernel.h) compile with nvcc into a cubin, which a harness of this
// project launches to record golden pings. Test infrastructure only.
#pragma once
#include <cuda_runtime.h>
#ifdef __CUDACC__
#define RTAC_CUDACC
#define RTAC_HOSTDEVICE __host__ __device__
#else
#define RTAC_HOSTDEVICE
#endif
// The harness checks CUDA errors itself.
#define CUDA_CHECK_LAST() do { } while(0)
