// Host-side parameter arithmetic of the rtacx path. Implemented in
// rtacx_host.cpp, which is compiled without floating-point contraction so
// that every float expression rounds exactly as written -- the range key
// parameters must match the reference's Binner::Key bit for bit.
#pragma once

#include <cstdint>

namespace rtacx {

// Range key parameters, computed in float exactly as Binner::Key::Key
// (include/rtac_simulation/Binner.h:34-45).
struct KeyParams {
    uint32_t nR;
    float a, b, lower, upper;
};

// Lerp constants of one PSF axis: texel coordinate x = delta * k + c with
// k = scale * n split into k_hi + k_lo floats and c = n / 2 - 0.5.
struct AxisLerp {
    float k_hi, k_lo, c;
    int n;
};

KeyParams host_key_params(uint32_t binCount, float minBin, float maxBin, float margin);
// clamp((int)fmaf(a, travel, b), 0, nR - 1): monotone in travel, equal to the
// key of every in-range sample.
uint32_t host_range_key_clamped(const KeyParams& k, float travel);
int host_bin_overlap(float rmin, float rmax, uint32_t n, float margin);
float host_linspace_at(float rmin, float rmax, uint32_t n, uint32_t r);
uint32_t host_bearing_bin(float scale, float offset, uint32_t n, float bearing);
AxisLerp host_axis_lerp(float scale, uint32_t n);
// PSF range scaling of kernel(): 1 / (duration * c)
// (src/SensorInstance2D.cu:40), or the literal 1D expression
// 1.0f / duration * c (src/SensorInstance1D.cu:30).
float host_pulse_scale(float duration, float c, bool literal_1d);

} // namespace rtacx
