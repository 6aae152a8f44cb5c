// Stand-in for rtac_base cuda/vec_math.h: the CUDA vector types.
#pragma once
#include <cuda_runtime.h>
