// rtacx_reduce_noalloc: a complete ping that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs under an allocation
// ban (hard real-time sensor loops that must not take the driver's allocation
// locks, host processes whose device memory is owned by another allocator or
// budgeted in advance) still needs a ping. This entry point runs the same
// sort + bin + sparse PSF kernels as rtacx_reduce, but every scratch buffer --
// sorted records, per-CTA histograms, bin offsets, windows and the PSF
// tables -- lives in one file-scope device array of fixed size. The caller
// passes the sensor description (host tables), the device samples and the
// device ping; no context is created.
//
// Limits (the array is sized for them and every GPU that loads the library
// keeps it until the process exits, about 6.6 MB):
//   samples <= RTACX_NOALLOC_MAX_SAMPLES, range bins <= RTACX_NOALLOC_MAX_RANGES,
//   bearings <= RTACX_NOALLOC_MAX_BEARINGS, pulse taps <= RTACX_NOALLOC_MAX_PULSE,
//   beam taps <= RTACX_NOALLOC_MAX_BEAM. Larger requests return
//   RTACX_ERR_UNSUPPORTED before any work is queued.
//
// The first call on a device (the current device) looks up the array's
// device address with cudaGetSymbolAddress; make that first call before any
// stream capture. Every call shares the one array and leaves its contents
// behind; each call re-uploads its tables and rewrites every scratch region it
// reads before reading it. Calls whose GPU work overlaps (different streams,
// or different host threads) race on the array: serialise them.
#include "rtacx_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

namespace rtacx {

void configure_hist_launch(Context& ctx);
size_t gather_smem_bytes(uint32_t range_tile, uint32_t bearing_tile, uint32_t H, uint32_t W);

namespace {

constexpr uint64_t kMaxSamples = RTACX_NOALLOC_MAX_SAMPLES;
constexpr uint32_t kMaxRanges = RTACX_NOALLOC_MAX_RANGES;
constexpr uint32_t kMaxBearings = RTACX_NOALLOC_MAX_BEARINGS;
constexpr uint32_t kMaxPulse = RTACX_NOALLOC_MAX_PULSE;
constexpr uint32_t kMaxBeam = RTACX_NOALLOC_MAX_BEAM;
constexpr uint32_t kMaxBins = 16384;                       // range bins x bearing sub-bins
constexpr uint32_t kMaxHistCtas = (uint32_t)(kMaxSamples / 4096);
constexpr uint32_t kMinBearingTile = 64;
constexpr uint32_t kMaxBearingTiles = (kMaxBearings + kMinBearingTile - 1) / kMinBearingTile;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of the scratch regions.
constexpr size_t kOffSorted  = 0;
constexpr size_t kOffHist    = align256(kOffSorted + kMaxSamples * sizeof(float4));
// The scatter's per-bin write cursors: kCursorStride words per bin.
constexpr size_t kHistBytes  = (size_t)kMaxBins * kCursorStride * sizeof(uint32_t);
constexpr size_t kOffOffsets = align256(kOffHist + kHistBytes);
constexpr size_t kOffTotals  = align256(kOffOffsets + (kMaxBins + 1) * 4);
constexpr size_t kOffWin     = align256(kOffTotals + (kMaxBins + kMaxBins / 1024 + 1) * 4);   // + block sums
constexpr size_t kOffOor     = align256(kOffWin + kMaxRanges * sizeof(int2));
constexpr size_t kOffErr     = align256(kOffOor + 2 * sizeof(unsigned long long));
constexpr size_t kOffPulse   = align256(kOffErr + sizeof(uint32_t));
constexpr size_t kOffBeam    = align256(kOffPulse + (kMaxPulse + 2) * sizeof(float2));
constexpr size_t kOffBear    = align256(kOffBeam + (kMaxBeam + 2) * sizeof(float));
constexpr size_t kOffRanges  = align256(kOffBear + kMaxBearings * sizeof(float));
constexpr size_t kOffSupport = align256(kOffRanges + kMaxRanges * sizeof(float));
constexpr size_t kOffTiles   = align256(kOffSupport + kMaxRanges * sizeof(int2));
constexpr size_t kScratchBytes = align256(kOffTiles + kMaxBearingTiles * sizeof(int2));

// The scratch itself. Host code must not use this name as an address: it is
// a host-side stand-in for the device symbol. Its device address comes from
// cudaGetSymbolAddress (scratch_base below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;                      // guards the tables below and the host staging
unsigned char* g_base[kMaxDevices] = {}; // device address of the scratch, per device

// Host staging of the per-call tables (copied to the scratch each call).
float2 h_pulse[kMaxPulse + 2];
float h_beam[kMaxBeam + 2];
float h_ranges[kMaxRanges];
int2 h_support[kMaxRanges];
int2 h_tiles[kMaxBearingTiles];

// Device address of the scratch on the current device; looked up once per
// device with that device current.
rtacx_status scratch_base(int device, unsigned char** base)
{
    if(device < 0 || device >= kMaxDevices) return RTACX_ERR_UNSUPPORTED;
    if(!g_base[device]) {
        void* p = nullptr;
        if(cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return RTACX_ERR_CUDA;
        }
        g_base[device] = static_cast<unsigned char*>(p);
    }
    *base = g_base[device];
    return RTACX_OK;
}

bool finite_all(const float* p, size_t n)
{
    for(size_t i = 0; i < n; i++) if(!std::isfinite(p[i])) return false;
    return true;
}

} // namespace
} // namespace rtacx

using namespace rtacx;

extern "C" rtacx_status rtacx_reduce_noalloc(int sample_kind, const void* sensor, const void* samples,
                                             uint64_t n, float* out, void* stream)
{
    if(!sensor || !out || (n && !samples)) return RTACX_ERR_INVALID_ARGUMENT;
    if(sample_kind != RTACX_SAMPLE_1D && sample_kind != RTACX_SAMPLE_2D) return RTACX_ERR_INVALID_ARGUMENT;
    if(reinterpret_cast<uintptr_t>(samples) % 4 != 0) return RTACX_ERR_INVALID_ARGUMENT;
    if(reinterpret_cast<uintptr_t>(out) % 8 != 0) return RTACX_ERR_INVALID_ARGUMENT;   // complex64 vector stores
    if(n > kMaxSamples) return RTACX_ERR_UNSUPPORTED;

    // Sensor fields of either layout.
    const rtacx_sensor_1d* s1 = static_cast<const rtacx_sensor_1d*>(sensor);
    const rtacx_sensor_2d* s2 = static_cast<const rtacx_sensor_2d*>(sensor);
    const bool two_d = sample_kind == RTACX_SAMPLE_2D;
    const float rmin = two_d ? s2->range_min : s1->range_min, rmax = two_d ? s2->range_max : s1->range_max;
    const uint32_t nR = two_d ? s2->range_count : s1->range_count;
    const float c = two_d ? s2->sound_celerity : s1->sound_celerity;
    const float duration = two_d ? s2->pulse_duration : s1->pulse_duration;
    const float margin = two_d ? s2->margin : s1->margin;
    const float* pulse = two_d ? s2->pulse : s1->pulse;
    const uint32_t H = two_d ? s2->pulse_len : s1->pulse_len;
    const uint32_t flags = two_d ? s2->flags : s1->flags;
    const uint32_t nB = two_d ? s2->bearing_count : 1u;
    const uint32_t W = two_d ? s2->beam_len : 0u;

    if(nR == 0 || !pulse || H == 0) return RTACX_ERR_INVALID_ARGUMENT;
    if(nR > kMaxRanges || H > kMaxPulse || nB > kMaxBearings || W > kMaxBeam) return RTACX_ERR_UNSUPPORTED;
    if(!(std::isfinite(rmin) && std::isfinite(rmax) && std::isfinite(margin))) return RTACX_ERR_INVALID_ARGUMENT;
    if(!(duration > 0.0f) || !(c > 0.0f) || !std::isfinite(duration * c)) return RTACX_ERR_INVALID_ARGUMENT;
    if(!finite_all(pulse, 2 * (size_t)H)) return RTACX_ERR_INVALID_ARGUMENT;
    if(flags & (RTACX_FLAG_TEXTURE_PSF | RTACX_FLAG_TEXTURE_CLAMP)) return RTACX_ERR_UNSUPPORTED;
    if(two_d) {
        if(!s2->beam || W == 0 || !s2->bearings || nB == 0) return RTACX_ERR_INVALID_ARGUMENT;
        if(!(s2->beam_span > 0.0f) || !std::isfinite(s2->beam_span)) return RTACX_ERR_INVALID_ARGUMENT;
        if(!finite_all(s2->beam, W) || !finite_all(s2->bearings, nB)) return RTACX_ERR_INVALID_ARGUMENT;
    }
    const bool literal = !two_d && (flags & RTACX_FLAG_1D_LITERAL_SCALING);
    const float pscale = host_pulse_scale(duration, c, literal);
    if(!(pscale > 0.0f) || !std::isfinite(pscale)) return RTACX_ERR_INVALID_ARGUMENT;

    int device = 0;
    if(cudaGetDevice(&device) != cudaSuccess) { cudaGetLastError(); return RTACX_ERR_CUDA; }
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    std::lock_guard<std::mutex> lock(g_mutex);
    unsigned char* base = nullptr;
    rtacx_status status = scratch_base(device, &base);
    if(status != RTACX_OK) return status;

    // A context on the stack whose device pointers all point into the scratch.
    Context ctx;
    ctx.device = device;
    if(cudaDeviceGetAttribute(&ctx.sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return RTACX_ERR_CUDA;
    }
    ctx.dims = two_d ? 2 : 1;
    ctx.flags = flags;
    ctx.rmin = rmin; ctx.rmax = rmax; ctx.nR = nR; ctx.margin = margin; ctx.c = c; ctx.duration = duration;
    ctx.H = H; ctx.nB = nB; ctx.W = W;
    ctx.key = host_key_params(nR, rmin, rmax, margin);
    ctx.overlap = (nR > 1) ? host_bin_overlap(rmin, rmax, nR, margin) : 0;
    ctx.red.dims = ctx.dims;
    ctx.red.nR = nR;
    ctx.red.nB = nB;
    ctx.red.range_axis = host_axis_lerp(pscale, H);

    // Output ranges, per-row support and the padded pulse table.
    for(uint32_t r = 0; r < nR; r++) h_ranges[r] = host_linspace_at(rmin, rmax, nR, r);
    const double half = 0.5 / (double)pscale * (1.0 + 1.0 / H) * (1.0 + 1e-4);
    for(uint32_t r = 0; r < nR; r++) {
        const double R = h_ranges[r];
        const double slack = 1e-6 * (std::fabs(R) + half) + 1e-30;
        h_support[r] = make_int2((int)host_range_key_clamped(ctx.key, (float)(R - half - slack)),
                                 (int)host_range_key_clamped(ctx.key, (float)(R + half + slack)));
    }
    h_pulse[0] = h_pulse[H + 1] = make_float2(0.f, 0.f);
    std::memcpy(h_pulse + 1, pulse, sizeof(float2) * H);

    uint32_t nBB = 1, tiles = 1;
    float bb_scale = 0.0f, bb_offset = 0.0f;
    if(two_d) {
        ctx.span = s2->beam_span;
        ctx.red.beam_axis = host_axis_lerp(1.0f / s2->beam_span, W);
        h_beam[0] = h_beam[W + 1] = 0.0f;
        std::memcpy(h_beam + 1, s2->beam, sizeof(float) * W);
        const uint64_t big = (uint64_t)((nR + 31) / 32) * ((nB + 127) / 128);
        if(big >= 2u * (uint64_t)ctx.sm_count) { ctx.range_tile = 32; ctx.bearing_tile = 128; }
        else {
            const uint64_t mid = (uint64_t)((nR + 15) / 16) * ((nB + 127) / 128);
            ctx.range_tile = 16; ctx.bearing_tile = (mid >= 2u * (uint64_t)ctx.sm_count) ? 128 : 64;
        }
        if(gather_smem_bytes(ctx.range_tile, ctx.bearing_tile, H, W) > 227 * 1024) return RTACX_ERR_UNSUPPORTED;
        float tmin = s2->bearings[0], tmax = s2->bearings[0];
        for(uint32_t b = 0; b < nB; b++) { tmin = std::min(tmin, s2->bearings[b]); tmax = std::max(tmax, s2->bearings[b]); }
        const double sb = 0.5 * (double)s2->beam_span * (1.0 + 1.0 / W) * (1.0 + 1e-4) + 1e-6;
        const double lo = (double)tmin - sb, hi = (double)tmax + sb;
        if(8.0 * sb < hi - lo) {
            while(nBB < 32 && (hi - lo) / (2.0 * nBB) > sb && (uint64_t)nR * nBB * 2 <= kMaxBins) nBB *= 2;
        }
        if(nBB > 1) {
            const float flo = (float)lo, fhi = (float)hi;
            bb_scale = (float)nBB / (fhi - flo);
            bb_offset = -flo * bb_scale;
        }
        tiles = (nB + ctx.bearing_tile - 1) / ctx.bearing_tile;
        for(uint32_t t = 0; t < tiles; t++) {
            if(nBB == 1) { h_tiles[t] = make_int2(0, 0); continue; }
            const uint32_t b0 = t * ctx.bearing_tile, b1 = std::min(nB, b0 + ctx.bearing_tile);
            float a = s2->bearings[b0], z = s2->bearings[b0];
            for(uint32_t b = b0; b < b1; b++) { a = std::min(a, s2->bearings[b]); z = std::max(z, s2->bearings[b]); }
            h_tiles[t] = make_int2((int)host_bearing_bin(bb_scale, bb_offset, nBB, (float)((double)a - sb)),
                                   (int)host_bearing_bin(bb_scale, bb_offset, nBB, (float)((double)z + sb)));
        }
    }
    else {
        ctx.red.beam_axis = AxisLerp{0.f, 0.f, 0.f, 0};
        h_beam[0] = 0.0f;
    }
    if((uint64_t)nR * nBB > kMaxBins) return RTACX_ERR_UNSUPPORTED;
    ctx.bin = BinParams{ctx.key, nBB, bb_scale, bb_offset, nR * nBB, two_d ? 4u : 3u,
                        (two_d && reinterpret_cast<uintptr_t>(samples) % 16 == 0) ? 1 : 0};

    // Point the context at the scratch regions.
    ctx.d_sorted = reinterpret_cast<float4*>(base + kOffSorted);
    ctx.capacity = kMaxSamples;
    ctx.d_hist = reinterpret_cast<uint32_t*>(base + kOffHist);
    ctx.d_offsets = reinterpret_cast<uint32_t*>(base + kOffOffsets);
    ctx.d_totals = reinterpret_cast<uint32_t*>(base + kOffTotals);
    ctx.d_win = reinterpret_cast<int2*>(base + kOffWin);
    ctx.d_oor = reinterpret_cast<unsigned long long*>(base + kOffOor);
    ctx.d_err = reinterpret_cast<uint32_t*>(base + kOffErr);
    ctx.d_pulse = reinterpret_cast<float2*>(base + kOffPulse);
    ctx.d_beam = reinterpret_cast<float*>(base + kOffBeam);
    ctx.d_bearings = reinterpret_cast<float*>(base + kOffBear);
    ctx.d_ranges = reinterpret_cast<float*>(base + kOffRanges);
    ctx.d_support = reinterpret_cast<int2*>(base + kOffSupport);
    ctx.d_bb_tiles = reinterpret_cast<int2*>(base + kOffTiles);
    configure_hist_launch(ctx);
    ctx.hist_ctas = std::min(ctx.hist_ctas, kMaxHistCtas);
    ctx.hist_cols = (size_t)ctx.bin.nBins * kCursorStride;
    if(ctx.hist_cols * sizeof(uint32_t) > kHistBytes) return RTACX_ERR_UNSUPPORTED;

    // Upload this call's tables (pageable copies: the staging above may be
    // reused as soon as these return) and clear the error word.
    const cudaError_t e =
        [&]() {
            cudaError_t r;
            if((r = cudaMemcpyAsync(ctx.d_pulse, h_pulse, sizeof(float2) * (H + 2), cudaMemcpyHostToDevice, st))) return r;
            if((r = cudaMemcpyAsync(ctx.d_ranges, h_ranges, sizeof(float) * nR, cudaMemcpyHostToDevice, st))) return r;
            if((r = cudaMemcpyAsync(ctx.d_support, h_support, sizeof(int2) * nR, cudaMemcpyHostToDevice, st))) return r;
            if((r = cudaMemsetAsync(ctx.d_err, 0, sizeof(uint32_t), st))) return r;
            if(two_d) {
                if((r = cudaMemcpyAsync(ctx.d_beam, h_beam, sizeof(float) * (W + 2), cudaMemcpyHostToDevice, st))) return r;
                if((r = cudaMemcpyAsync(ctx.d_bearings, s2->bearings, sizeof(float) * nB, cudaMemcpyHostToDevice, st))) return r;
                if((r = cudaMemcpyAsync(ctx.d_bb_tiles, h_tiles, sizeof(int2) * tiles, cudaMemcpyHostToDevice, st))) return r;
            }
            return cudaSuccess;
        }();
    if(e != cudaSuccess) { cudaGetLastError(); return RTACX_ERR_CUDA; }

    status = run_binning(ctx, samples, n, st);
    if(status != RTACX_OK) return status;
    return run_reduce(ctx, out, st);
}
