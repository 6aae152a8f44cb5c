// Stand-in for rtac_base cuda/geometry.h: Receiver.h includes it for device
// code compiled only under RTAC_CUDACC, which the binding compile leaves out.
#pragma once
