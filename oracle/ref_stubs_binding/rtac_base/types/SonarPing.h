// Stand-in for rtac_base types/SonarPing.h: SensorInstance2D.h includes it
// for the ping types, declared by the cuda/CudaPing.h stand-in.
#pragma once
