// Host stand-in for the CUDA vector types used by the reference headers.
#pragma once
#include <cmath>
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct uint2  { unsigned int x, y; };
inline float length(const float3& p) { return std::sqrt(p.x*p.x + p.y*p.y + p.z*p.z); }
