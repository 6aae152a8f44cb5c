// Host-side parameter arithmetic (see rtacx_host.h). Build with
// -ffp-contract=off: these float expressions must round as written.
#include "rtacx_host.h"

#include <cmath>
#include <limits>

namespace rtacx {

namespace {
// CUDA's float->int conversion (cvt.rzi.s32.f32): truncate, saturate, NaN -> 0.
int f2i_rz(float f)
{
    if(std::isnan(f)) return 0;
    if(f >= 2147483648.0f)  return std::numeric_limits<int>::max();
    if(f <= -2147483648.0f) return std::numeric_limits<int>::min();
    return (int)f;
}
}

KeyParams host_key_params(uint32_t binCount, float minBin, float maxBin, float margin)
{
    KeyParams k;
    k.nR = binCount;
    float resolution = (maxBin - minBin) / (float)binCount;
    float m = minBin - 0.5f * resolution;
    float M = maxBin + 0.5f * resolution;
    k.a = (float)(binCount - 1u) / (M - m);
    float ma = -m * k.a;
    k.b = ma + 0.5f;
    k.lower = m - margin;
    k.upper = M + margin;
    return k;
}

uint32_t host_range_key_clamped(const KeyParams& k, float travel)
{
    int res = f2i_rz(std::fmaf(k.a, travel, k.b));
    if(res < 0) return 0u;
    if((uint32_t)res >= k.nR) return k.nR - 1u;
    return (uint32_t)res;
}

int host_bin_overlap(float rmin, float rmax, uint32_t n, float margin)
{
    float resolution = (rmax - rmin) / (float)(n - 1u);
    return f2i_rz(margin / resolution);
}

float host_linspace_at(float rmin, float rmax, uint32_t n, uint32_t r)
{
    if(n <= 1) return rmin;
    float res = (rmax - rmin) / (float)(n - 1u);
    float prod = res * (float)r;
    return rmin + prod;
}

uint32_t host_bearing_bin(float scale, float offset, uint32_t n, float bearing)
{
    float q = std::fmaf(scale, bearing, offset);
    if(!(q >= 1.0f)) return 0u;
    if(q >= (float)n) return n - 1u;
    return (uint32_t)f2i_rz(q);
}

AxisLerp host_axis_lerp(float scale, uint32_t n)
{
    AxisLerp a;
    double k = (double)scale * (double)n;
    a.k_hi = (float)k;
    a.k_lo = (float)(k - (double)a.k_hi);
    a.c = 0.5f * (float)n - 0.5f;
    a.n = (int)n;
    return a;
}

float host_pulse_scale(float duration, float c, bool literal_1d)
{
    if(literal_1d) {
        float inv = 1.0f / duration;
        return inv * c;
    }
    float ext = duration * c;
    return 1.0f / ext;
}

} // namespace rtacx
