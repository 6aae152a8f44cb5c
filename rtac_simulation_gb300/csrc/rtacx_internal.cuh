// Internal declarations shared by the rtacx translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rtacx.h"
#include "rtacx_host.h"

namespace rtacx {

constexpr uint32_t kOutOfRange = RTACX_KEY_OUT_OF_RANGE;

// Device error word bits (OR-ed by kernels, read by rtacx_stream_status).
constexpr uint32_t kErrScatterOverflow = 1u << 0;  // sorted position beyond the counted total
constexpr uint32_t kErrBadWindow       = 1u << 1;  // window bounds outside the sorted array

// Largest (range bin x bearing bin) histogram a CTA keeps in shared memory.
constexpr uint32_t kMaxSmemBins = 49152;

// Everything the binning kernels need, passed by value.
struct BinParams {
    KeyParams key;
    uint32_t nBB;          // bearing sub-bins (1: range key only)
    float bb_scale;        // bearing bin = f(fmaf(bb_scale, bearing, bb_offset))
    float bb_offset;
    uint32_t nBins;        // nR * nBB
    uint32_t stride;       // floats per input record: 3 (SimSample1D) or 4 (SimSample2D)
    int vec4;              // 1 when records are 16-byte aligned float4s
};

// Range key of one travel value: Binner::Key::operator()
// (include/rtac_simulation/Binner.h:47-53) with CUDA float->int semantics.
// side: -1 below range, +1 above range, 0 in range.
__device__ __forceinline__ uint32_t range_key(const KeyParams& k, float travel, int& side)
{
    int res = __float2int_rz(fmaf(k.a, travel, k.b));
    side = 0;
    if(res < 0) {
        if((float)res >= k.lower) return 0u;
        side = -1;
        return kOutOfRange;
    }
    if((uint32_t)res >= k.nR) {
        if((float)res <= k.upper) return k.nR - 1u;
        side = 1;
        return kOutOfRange;
    }
    return (uint32_t)res;
}

// Bearing sub-bin (extension of the reference key, see the oracle for the
// same formula): 0 if !(q >= 1), n - 1 if q >= n, else (int)q.
__device__ __forceinline__ uint32_t bearing_bin(float scale, float offset, uint32_t n, float bearing)
{
    float q = fmaf(scale, bearing, offset);
    if(!(q >= 1.0f)) return 0u;
    if(q >= (float)n) return n - 1u;
    return (uint32_t)__float2int_rz(q);
}

// Composite (range bin, bearing bin) key; kOutOfRange for out-of-range travel.
__device__ __forceinline__ uint32_t sample_key(const BinParams& p, float travel, float bearing, int& side)
{
    uint32_t rk = range_key(p.key, travel, side);
    if(rk == kOutOfRange) return kOutOfRange;
    if(p.nBB == 1u) return rk;
    return rk * p.nBB + bearing_bin(p.bb_scale, p.bb_offset, p.nBB, bearing);
}

__device__ __forceinline__ float4 load_record(const float* base, uint64_t i, const BinParams& p)
{
    if(p.vec4) return __ldg(reinterpret_cast<const float4*>(base) + i);
    const float* s = base + i * p.stride;
    return make_float4(__ldg(s), __ldg(s + 1), __ldg(s + 2), p.stride == 4 ? __ldg(s + 3) : 0.0f);
}

// Reduction parameters of a configured sensor.
struct ReduceParams {
    int dims;
    uint32_t nR, nB;
    AxisLerp range_axis;
    AxisLerp beam_axis;
};

// Scratch and configuration owned by one context.
struct Context {
    int device = 0;
    int sm_count = 0;
    std::string error;

    bool configured = false;
    int dims = 0;
    uint32_t flags = 0;

    // Host copies of the configuration.
    float rmin = 0, rmax = 0, margin = 0, c = 0, duration = 0, span = 0;
    uint32_t nR = 0, nB = 0, H = 0, W = 0;
    std::vector<float> pulse, beam, bearings;
    KeyParams key{};
    int overlap = 0;
    BinParams bin{};
    ReduceParams red{};
    uint32_t bearing_tile = 0;          // bearings per gather tile
    uint32_t range_tile = 0;            // rows per gather tile

    // Device tables (configuration-sized).
    float2* d_pulse = nullptr;          // pulse padded with a zero tap on each side
    float* d_beam = nullptr;            // beam padded with a zero tap on each side
    float* d_bearings = nullptr;        // [nB]
    float* d_ranges = nullptr;          // [nR] Linspace values
    int2* d_support = nullptr;          // [nR] range bins that can hold PSF support of row r
    int2* d_bb_tiles = nullptr;         // [bearing tiles] bearing-bin range of each tile
    uint32_t* d_offsets = nullptr;      // [nBins + 1] exclusive scan of bin counts
    uint32_t* d_totals = nullptr;       // [nBins]
    int2* d_win = nullptr;              // [nR] effective bin range per row (lo > hi: empty)
    unsigned long long* d_oor = nullptr;// [2] low / high out-of-range counts
    uint32_t* d_err = nullptr;          // device error word

    // Sample-sized scratch.
    uint64_t capacity = 0;              // samples the sorted scratch holds
    float4* d_sorted = nullptr;
    uint32_t hist_ctas = 0;             // CTAs of the count / scatter passes
    uint32_t hist_threads = 0;
    size_t hist_cols = 0;               // allocated CTA x bin entries
    uint32_t* d_hist = nullptr;         // [hist_ctas][nBins]

    // Stage tracing: events[2 * i], events[2 * i + 1] bracket stage i.
    bool tracing = false;
    cudaEvent_t events[2 * RTACX_STAGE_COUNT] = {};
    bool traced[RTACX_STAGE_COUNT] = {};
    void mark(int stage, bool end, cudaStream_t s)
    {
        if(!tracing) return;
        cudaEventRecord(events[2 * stage + (end ? 1 : 0)], s);
        if(end) traced[stage] = true;
    }

    bool fail(const std::string& msg) { error = msg; return false; }
};

// Binning pipeline (rtacx_bin.cu): count, scan, scatter, windows.
rtacx_status run_binning(Context& ctx, const void* samples, uint64_t n, cudaStream_t stream);
rtacx_status run_bin_outputs(Context& ctx, const void* samples, uint64_t n,
                             uint32_t* keys, uint32_t* segments, uint32_t* windows,
                             uint32_t* counts, uint64_t* oor, cudaStream_t stream);
bool ensure_capacity(Context& ctx, uint64_t n);

// Sparse PSF reduction (rtacx_reduce.cu).
rtacx_status run_reduce(Context& ctx, float* out, cudaStream_t stream);

} // namespace rtacx

struct rtacx_ctx {
    rtacx::Context impl;
};
