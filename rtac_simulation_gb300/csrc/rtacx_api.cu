// C ABI entry points (include/rtacx.h).
#include "rtacx_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace rtacx {

void configure_hist_launch(Context& ctx);
size_t gather_smem_bytes(uint32_t range_tile, uint32_t bearing_tile, uint32_t H, uint32_t W);
rtacx_status configure_precision(Context& ctx, const rtacx_precision_desc* d);

namespace {

constexpr size_t kMaxGatherSmem = 227 * 1024;

template <typename T>
void free_dev(T*& p)
{
    if(p) cudaFree(p);
    p = nullptr;
}

// Copy the context's echo model into the binning parameters.
void sync_echo(Context& c)
{
    c.bin.echo_flags = c.echo_flags;
    c.bin.echo_cycles = (c.c > 0.0f) ? 2.0 * c.echo_hz / (double)c.c : 0.0;
    c.bin.echo_k_hi = (float)c.bin.echo_cycles;
    c.bin.echo_k_lo = (float)(c.bin.echo_cycles - (double)c.bin.echo_k_hi);
}

// PSF image of the reference sensor (generate_psf_data,
// src/SensorInstance2D.cu:20-33): PSF[h][w] = waveform[h] * beam[w] in
// float, W = beam taps wide, H = pulse taps high, sampled by a texture with
// linear filtering, border addressing and normalized coordinates
// (src/SensorInstance2D.cu:14-15); KernelView2D scalings {1 / span, 0.5} and
// {1 / (duration c), 0.5} (src/SensorInstance2D.cu:35-42).
rtacx_status make_psf_texture(Context& c, const rtacx_sensor_2d* s)
{
    const uint32_t W = s->beam_len, H = s->pulse_len;
    std::vector<float2> img((size_t)W * H);
    for(uint32_t h = 0; h < H; h++)
        for(uint32_t w = 0; w < W; w++)
            img[(size_t)h * W + w] = make_float2(s->pulse[2 * h] * s->beam[w], s->pulse[2 * h + 1] * s->beam[w]);
    const cudaChannelFormatDesc ch = cudaCreateChannelDesc<float2>();
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    if(cudaMallocArray(&c.psf_array, &ch, W, H) != cudaSuccess ||
       cudaMemcpy2DToArray(c.psf_array, 0, 0, img.data(), W * sizeof(float2), W * sizeof(float2), H,
                           cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        c.error = "cannot upload the PSF texture (texture limits: width and height)";
        return RTACX_ERR_CUDA;
    }
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = c.psf_array;
    if(cudaCreateTextureObject(&c.psf_tex, &rd, &td, nullptr) != cudaSuccess) {
        cudaGetLastError();
        c.psf_tex = 0;
        c.error = "cannot create the PSF texture";
        return RTACX_ERR_CUDA;
    }
    c.tex_xscale = 1.0f / s->beam_span;
    c.tex_yscale = host_pulse_scale(s->pulse_duration, s->sound_celerity, false);
    return RTACX_OK;
}

// The reference's 1D pulse texture (SensorInstance1D::generate_psf_data,
// src/SensorInstance1D.cu:15-25): the waveform's taps as a one-row float2
// texture with linear filtering and normalized coordinates; the address mode
// is an rtac_base default (border, or clamp with RTACX_FLAG_TEXTURE_CLAMP).
// KernelView1D scaling {scale, 0.5} (src/SensorInstance1D.cu:27-33).
rtacx_status make_pulse_texture_1d(Context& c, const rtacx_sensor_1d* s, float scale)
{
    const cudaChannelFormatDesc ch = cudaCreateChannelDesc<float2>();
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] =
        (s->flags & RTACX_FLAG_TEXTURE_CLAMP) ? cudaAddressModeClamp : cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    if(cudaMallocArray(&c.psf_array, &ch, s->pulse_len, 0) != cudaSuccess ||
       cudaMemcpy2DToArray(c.psf_array, 0, 0, s->pulse, s->pulse_len * sizeof(float2), s->pulse_len * sizeof(float2),
                           1, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        c.error = "cannot upload the pulse texture (texture width limit)";
        return RTACX_ERR_CUDA;
    }
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = c.psf_array;
    if(cudaCreateTextureObject(&c.psf_tex, &rd, &td, nullptr) != cudaSuccess) {
        cudaGetLastError();
        c.psf_tex = 0;
        c.error = "cannot create the pulse texture";
        return RTACX_ERR_CUDA;
    }
    c.tex_xscale = 0.0f;
    c.tex_yscale = scale;
    return RTACX_OK;
}

void free_config(Context& c)
{
    free_precision(c);
    if(c.psf_tex) cudaDestroyTextureObject(c.psf_tex);
    c.psf_tex = 0;
    if(c.psf_array) cudaFreeArray(c.psf_array);
    c.psf_array = nullptr;
    free_dev(c.d_pulse); free_dev(c.d_beam); free_dev(c.d_bearings); free_dev(c.d_ranges);
    free_dev(c.d_support); free_dev(c.d_bb_tiles64); free_dev(c.d_bb_tiles128); c.d_bb_tiles = nullptr;
    free_dev(c.d_offsets); free_dev(c.d_totals);
    free_dev(c.d_win); free_dev(c.d_hist);
    free_dev(c.d_tile_parts); free_dev(c.d_tile_first); free_dev(c.d_items); free_dev(c.d_item_counter);
    c.hist_cols = 0;
    c.configured = false;
}

template <typename T>
bool upload(Context& c, T*& dst, const T* src, size_t count)
{
    free_dev(dst);
    if(count == 0) count = 1;
    if(cudaMalloc(&dst, count * sizeof(T)) != cudaSuccess) { cudaGetLastError(); return c.fail("cudaMalloc failed"); }
    if(src && cudaMemcpy(dst, src, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        return c.fail("cudaMemcpy failed");
    }
    return true;
}

bool all_finite(const float* p, size_t n)
{
    for(size_t i = 0; i < n; i++) if(!std::isfinite(p[i])) return false;
    return true;
}

struct Common {
    float rmin, rmax, c, duration, margin;
    uint32_t nR, H;
    const float* pulse;
};

// Validation and the parts shared by the 1D and 2D configurations: Binner
// reconfiguration (src/SensorInstance.cu:32, src/Binner.cu:15-22), Key
// parameters, overlap, output range table, pulse table and per-row support.
bool configure_common(Context& c, const Common& s, float pulse_scale)
{
    if(!(std::isfinite(s.rmin) && std::isfinite(s.rmax) && std::isfinite(s.margin)))
        return c.fail("range_min, range_max and margin must be finite");
    if(s.nR == 0) return c.fail("range_count must be >= 1");
    if(s.nR > (1u << 20)) return c.fail("range_count above 2^20 is not supported");
    if(!s.pulse || s.H == 0) return c.fail("pulse table is empty");
    if(!(s.duration > 0.0f) || !(s.c > 0.0f) || !std::isfinite(s.duration * s.c))
        return c.fail("pulse_duration and sound_celerity must be positive and finite");
    if(!(pulse_scale > 0.0f) || !std::isfinite(pulse_scale)) return c.fail("degenerate pulse scaling");
    if(!all_finite(s.pulse, 2 * (size_t)s.H)) return c.fail("pulse table holds non-finite values");

    c.rmin = s.rmin; c.rmax = s.rmax; c.nR = s.nR; c.margin = s.margin;
    c.c = s.c; c.duration = s.duration; c.H = s.H;
    c.pulse.assign(s.pulse, s.pulse + 2 * (size_t)s.H);
    c.key = host_key_params(s.nR, s.rmin, s.rmax, s.margin);
    c.overlap = (s.nR > 1) ? host_bin_overlap(s.rmin, s.rmax, s.nR, s.margin) : 0;

    std::vector<float> ranges(s.nR);
    for(uint32_t r = 0; r < s.nR; r++) ranges[r] = host_linspace_at(s.rmin, s.rmax, s.nR, r);

    // Range bins that can hold a sample with non-zero pulse weight for row r:
    // |travel - R_r| < extent / 2 * (1 + 1 / H), widened by a relative slack.
    const double ext = 1.0 / (double)pulse_scale;
    const double half = 0.5 * ext * (1.0 + 1.0 / s.H) * (1.0 + 1e-4);
    std::vector<int2> support(s.nR);
    for(uint32_t r = 0; r < s.nR; r++) {
        const double R = ranges[r];
        const double slack = 1e-6 * (std::fabs(R) + half) + 1e-30;
        const float lo = (float)(R - half - slack), hi = (float)(R + half + slack);
        support[r] = make_int2((int)host_range_key_clamped(c.key, lo), (int)host_range_key_clamped(c.key, hi));
    }
    std::vector<float2> pad(s.H + 2, make_float2(0.f, 0.f));
    std::memcpy(pad.data() + 1, s.pulse, 2 * sizeof(float) * s.H);
    c.red.nR = s.nR;
    c.red.range_axis = host_axis_lerp(pulse_scale, s.H);
    return upload(c, c.d_ranges, ranges.data(), ranges.size()) &&
           upload(c, c.d_support, support.data(), support.size()) &&
           upload(c, c.d_pulse, pad.data(), pad.size());
}

bool allocate_bins(Context& c)
{
    configure_hist_launch(c);
    const size_t cols = (size_t)c.bin.nBins * kCursorStride;
    return upload<uint32_t>(c, c.d_offsets, nullptr, c.bin.nBins + 1) &&
           upload<uint32_t>(c, c.d_totals, nullptr, c.bin.nBins + c.bin.nBins / 1024 + 1) &&   // + block sums
           upload<int2>(c, c.d_win, nullptr, c.nR) &&
           upload<uint32_t>(c, c.d_hist, nullptr, cols) &&
           ((c.hist_cols = cols), true);
}

rtacx_status set_device(Context& c)
{
    if(cudaSetDevice(c.device) != cudaSuccess) {
        cudaGetLastError();
        c.error = "cudaSetDevice failed";
        return RTACX_ERR_CUDA;
    }
    return RTACX_OK;
}

} // namespace
} // namespace rtacx

using namespace rtacx;

extern "C" {

const char* rtacx_version(void) { return "rtacx 0.1 (sm_103a)"; }

rtacx_status rtacx_create(rtacx_ctx** out, int device)
{
    if(!out) return RTACX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if(cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return RTACX_ERR_CUDA;
    }
    rtacx_ctx* ctx = new rtacx_ctx();
    Context& c = ctx->impl;
    c.device = device;
    if(set_device(c) != RTACX_OK ||
       cudaDeviceGetAttribute(&c.sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
       cudaMalloc(&c.d_err, sizeof(uint32_t)) != cudaSuccess ||
       cudaMemset(c.d_err, 0, sizeof(uint32_t)) != cudaSuccess ||
       cudaMalloc(&c.d_oor, 2 * sizeof(unsigned long long)) != cudaSuccess ||
       cudaMemset(c.d_oor, 0, 2 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        rtacx_destroy(ctx);
        return RTACX_ERR_CUDA;
    }
    *out = ctx;
    return RTACX_OK;
}

void rtacx_destroy(rtacx_ctx* ctx)
{
    if(!ctx) return;
    Context& c = ctx->impl;
    cudaSetDevice(c.device);
    free_config(c);
    free_dev(c.d_sorted);
    free_dev(c.d_dir);
    free_dev(c.d_rast_v); free_dev(c.d_rast_vis); free_dev(c.d_rast_large);
    free_streaming(c);
    free_dev(c.d_err);
    free_dev(c.d_oor);
    for(cudaEvent_t& e : c.events) if(e) cudaEventDestroy(e);
    delete ctx;
}

const char* rtacx_last_error(const rtacx_ctx* ctx)
{
    return ctx ? ctx->impl.error.c_str() : "null context";
}

rtacx_status rtacx_configure_1d(rtacx_ctx* ctx, const rtacx_sensor_1d* s)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(!s) { c.error = "null sensor"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    free_config(c);
    if(s->flags & ~(RTACX_FLAG_1D_LITERAL_SCALING | RTACX_FLAG_TEXTURE_PSF | RTACX_FLAG_TEXTURE_CLAMP) ||
       ((s->flags & RTACX_FLAG_TEXTURE_CLAMP) && !(s->flags & RTACX_FLAG_TEXTURE_PSF))) {
        c.error = "unknown 1D sensor flags (RTACX_FLAG_TEXTURE_CLAMP needs RTACX_FLAG_TEXTURE_PSF)";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    const bool literal = (s->flags & RTACX_FLAG_1D_LITERAL_SCALING) != 0;
    const float scale = host_pulse_scale(s->pulse_duration, s->sound_celerity, literal);
    Common cm{s->range_min, s->range_max, s->sound_celerity, s->pulse_duration, s->margin,
              s->range_count, s->pulse_len, s->pulse};
    if(!configure_common(c, cm, scale)) return RTACX_ERR_INVALID_ARGUMENT;
    if((s->pulse_len + 2) * sizeof(float2) > kMaxGatherSmem) {
        c.error = "pulse table too long for shared memory";
        return RTACX_ERR_UNSUPPORTED;
    }
    c.dims = 1; c.flags = s->flags; c.nB = 1; c.W = 0;
    c.red.dims = 1; c.red.nB = 1;
    c.red.beam_axis = AxisLerp{0.f, 0.f, 0.f, 0};
    c.bin = BinParams{c.key, 1u, 0.0f, 0.0f, c.nR, 3u, 0};
    sync_echo(c);
    if(c.nR > kMaxSmemBins) { c.error = "range_count above the shared-memory histogram limit"; return RTACX_ERR_UNSUPPORTED; }
    std::vector<float> one(1, 0.0f);
    if(!upload(c, c.d_beam, one.data(), 1) || !upload(c, c.d_bearings, one.data(), 1) || !allocate_bins(c))
        return RTACX_ERR_OUT_OF_MEMORY;
    if((s->flags & RTACX_FLAG_TEXTURE_PSF) && make_pulse_texture_1d(c, s, scale) != RTACX_OK) return RTACX_ERR_CUDA;
    if(s->flags & RTACX_FLAG_TEXTURE_CLAMP) {
        // Clamp addressing gives every sample of the window the pulse's edge
        // taps, so each row reads its whole reference window, not only the
        // bins that hold the pulse's support.
        std::vector<int2> whole(c.nR, make_int2(0, (int)c.nR - 1));
        if(!upload(c, c.d_support, whole.data(), whole.size())) return RTACX_ERR_OUT_OF_MEMORY;
    }
    c.configured = true;
    return RTACX_OK;
}

rtacx_status rtacx_configure_2d(rtacx_ctx* ctx, const rtacx_sensor_2d* s)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(!s) { c.error = "null sensor"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    free_config(c);
    if(!s->beam || s->beam_len == 0) { c.error = "beam table is empty"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(!s->bearings || s->bearing_count == 0) { c.error = "bearing table is empty"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(!(s->beam_span > 0.0f) || !std::isfinite(s->beam_span)) { c.error = "beam_span must be positive"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(s->flags & ~(RTACX_FLAG_TEXTURE_PSF | RTACX_FLAG_SIMT_GATHER)) { c.error = "unknown 2D sensor flags"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(!all_finite(s->beam, s->beam_len) || !all_finite(s->bearings, s->bearing_count)) {
        c.error = "beam or bearing table holds non-finite values";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    const float scale = host_pulse_scale(s->pulse_duration, s->sound_celerity, false);
    Common cm{s->range_min, s->range_max, s->sound_celerity, s->pulse_duration, s->margin,
              s->range_count, s->pulse_len, s->pulse};
    if(!configure_common(c, cm, scale)) return RTACX_ERR_INVALID_ARGUMENT;

    c.dims = 2; c.flags = s->flags;
    c.nB = s->bearing_count; c.W = s->beam_len; c.span = s->beam_span;
    c.beam.assign(s->beam, s->beam + s->beam_len);
    c.bearings.assign(s->bearings, s->bearings + s->bearing_count);
    const float xscale = 1.0f / s->beam_span;       // src/SensorInstance2D.cu:39
    c.red.dims = 2; c.red.nB = c.nB;
    c.red.beam_axis = host_axis_lerp(xscale, c.W);

    // Gather tile shape: prefer 32 x 128; smaller tiles when the ping is too
    // small to give every SM two CTAs.
    const uint64_t big = (uint64_t)((c.nR + 31) / 32) * ((c.nB + 127) / 128);
    if(big >= 2u * (uint64_t)c.sm_count) { c.range_tile = 32; c.bearing_tile = 128; }
    else {
        const uint64_t mid = (uint64_t)((c.nR + 15) / 16) * ((c.nB + 127) / 128);
        c.range_tile = 16; c.bearing_tile = (mid >= 2u * (uint64_t)c.sm_count) ? 128 : 64;
    }
    if(gather_smem_bytes(c.range_tile, c.bearing_tile, c.H, c.W) > kMaxGatherSmem) {
        c.error = "PSF tables too large for shared memory";
        return RTACX_ERR_UNSUPPORTED;
    }

    // Bearing sub-bins: worthwhile when the beam support is narrow compared
    // with the fan. Support of the border-addressed lerp: |dtheta| < span/2 (1 + 1/W).
    const auto mm = std::minmax_element(c.bearings.begin(), c.bearings.end());
    const double sb = 0.5 * (double)s->beam_span * (1.0 + 1.0 / c.W) * (1.0 + 1e-4) + 1e-6;
    const double lo = (double)*mm.first - sb, hi = (double)*mm.second + sb;
    uint32_t nBB = 1;
    const bool texture_psf = (s->flags & RTACX_FLAG_TEXTURE_PSF) != 0;
    if(!texture_psf && 4.0 * 2.0 * sb < hi - lo) {   // support below a quarter of the fan
        while(nBB < 32 && (hi - lo) / (2.0 * nBB) > sb && (uint64_t)c.nR * nBB * 2 <= kMaxSmemBins) nBB *= 2;
    }
    float bb_scale = 0.0f, bb_offset = 0.0f;
    if(nBB > 1) {
        const float flo = (float)lo, fhi = (float)hi;
        bb_scale = (float)nBB / (fhi - flo);
        bb_offset = -flo * bb_scale;
    }
    if((uint64_t)c.nR * nBB > kMaxSmemBins) {
        c.error = "range_count above the shared-memory histogram limit";
        return RTACX_ERR_UNSUPPORTED;
    }
    c.bin = BinParams{c.key, nBB, bb_scale, bb_offset, c.nR * nBB, 4u, 0};
    sync_echo(c);

    // Bearing-bin range of every bearing tile, for 64- and 128-bearing tiles.
    auto tile_ranges = [&](uint32_t width) {
        const uint32_t tiles = (c.nB + width - 1) / width;
        std::vector<int2> bbt(tiles);
        for(uint32_t t = 0; t < tiles; t++) {
            if(nBB == 1) { bbt[t] = make_int2(0, 0); continue; }
            const uint32_t b0 = t * width, b1 = std::min(c.nB, b0 + width);
            float tmin = c.bearings[b0], tmax = c.bearings[b0];
            for(uint32_t b = b0; b < b1; b++) { tmin = std::min(tmin, c.bearings[b]); tmax = std::max(tmax, c.bearings[b]); }
            const float qlo = (float)((double)tmin - sb), qhi = (float)((double)tmax + sb);
            bbt[t] = make_int2((int)host_bearing_bin(bb_scale, bb_offset, nBB, qlo),
                               (int)host_bearing_bin(bb_scale, bb_offset, nBB, qhi));
        }
        return bbt;
    };
    const std::vector<int2> bbt64 = tile_ranges(64), bbt128 = tile_ranges(128);
    std::vector<float> bpad(c.W + 2, 0.0f);
    std::memcpy(bpad.data() + 1, s->beam, sizeof(float) * c.W);
    if(!upload(c, c.d_beam, bpad.data(), bpad.size()) ||
       !upload(c, c.d_bearings, c.bearings.data(), c.bearings.size()) ||
       !upload(c, c.d_bb_tiles64, bbt64.data(), bbt64.size()) ||
       !upload(c, c.d_bb_tiles128, bbt128.data(), bbt128.size()) || !allocate_bins(c))
        return RTACX_ERR_OUT_OF_MEMORY;
    c.d_bb_tiles = (c.bearing_tile == 64) ? c.d_bb_tiles64 : c.d_bb_tiles128;
    if(texture_psf && make_psf_texture(c, s) != RTACX_OK) return RTACX_ERR_CUDA;
    {
        const uint64_t tiles = (uint64_t)((c.nB + c.bearing_tile - 1) / c.bearing_tile) * ((c.nR + c.range_tile - 1) / c.range_tile);
        if(!upload<uint32_t>(c, c.d_tile_parts, nullptr, tiles) || !upload<uint32_t>(c, c.d_tile_first, nullptr, tiles + 1) ||
           !upload<uint4>(c, c.d_items, nullptr, tiles * 256) || !upload<uint32_t>(c, c.d_item_counter, nullptr, 1))
            return RTACX_ERR_OUT_OF_MEMORY;
    }
    c.configured = true;
    return RTACX_OK;
}

rtacx_status rtacx_reserve(rtacx_ctx* ctx, uint64_t max_samples)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(max_samples >= (1ull << 32)) { c.error = "at most 2^32 - 1 samples per ping"; return RTACX_ERR_UNSUPPORTED; }
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    return ensure_capacity(c, max_samples) ? RTACX_OK : RTACX_ERR_OUT_OF_MEMORY;
}

static rtacx_status prepare(rtacx_ctx* ctx, const void* samples, uint64_t n, int kind)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(!c.configured) { c.error = "context is not configured"; return RTACX_ERR_NOT_CONFIGURED; }
    if(kind != c.dims) { c.error = "sample kind does not match the configured sensor"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(n && !samples) { c.error = "null sample buffer"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(n >= (1ull << 32)) { c.error = "at most 2^32 - 1 samples per ping"; return RTACX_ERR_UNSUPPORTED; }
    if(reinterpret_cast<uintptr_t>(samples) % 4 != 0) { c.error = "sample buffer must be 4-byte aligned"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    if(!ensure_capacity(c, n)) return RTACX_ERR_OUT_OF_MEMORY;
    c.bin.vec4 = (c.dims == 2 && reinterpret_cast<uintptr_t>(samples) % 16 == 0) ? 1 : 0;
    return RTACX_OK;
}

rtacx_status rtacx_bin(rtacx_ctx* ctx, const void* samples, uint64_t n, int sample_kind,
                       uint32_t* keys, uint32_t* segments, uint32_t* windows,
                       uint32_t* counts, uint64_t* oor, void* stream)
{
    rtacx_status st = prepare(ctx, samples, n, sample_kind);
    if(st != RTACX_OK) return st;
    Context& c = ctx->impl;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    st = run_binning(c, samples, n, s);
    if(st != RTACX_OK) return st;
    return run_bin_outputs(c, samples, n, keys, segments, windows, counts, oor, s);
}

rtacx_status rtacx_reduce(rtacx_ctx* ctx, const void* samples, uint64_t n, float* out, void* stream)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    if(!out) { ctx->impl.error = "null output buffer"; return RTACX_ERR_INVALID_ARGUMENT; }
    // The gathers store whole complex64 cells (8-byte vector stores and
    // vector reductions): a ping that is not 8-byte aligned is refused here
    // rather than faulting on the device.
    if(reinterpret_cast<uintptr_t>(out) % 8 != 0) { ctx->impl.error = "the ping must be 8-byte aligned"; return RTACX_ERR_INVALID_ARGUMENT; }
    rtacx_status st = prepare(ctx, samples, n, ctx->impl.dims);
    if(st != RTACX_OK) return st;
    Context& c = ctx->impl;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    for(bool& t : c.traced) t = false;
    st = run_binning(c, samples, n, s);
    if(st != RTACX_OK) return st;
    c.mark(5, false, s);
    st = run_reduce(c, out, s);
    c.mark(5, true, s);
    return st;
}

rtacx_status rtacx_set_echo_model(rtacx_ctx* ctx, const rtacx_echo_model* m)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(!m || m->flags == 0) { c.echo_flags = 0; c.echo_hz = 0.0; sync_echo(c); return RTACX_OK; }
    if(m->flags & ~(RTACX_ECHO_PHASE | RTACX_ECHO_SPREADING | RTACX_ECHO_PHASE_COMPENSATED)) {
        c.error = "unknown echo flags";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    if((m->flags & RTACX_ECHO_PHASE) && !(std::isfinite(m->carrier_hz) && m->carrier_hz > 0.0)) {
        c.error = "carrier_hz must be positive and finite";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    c.echo_flags = m->flags;
    c.echo_hz = (m->flags & RTACX_ECHO_PHASE) ? m->carrier_hz : 0.0;
    sync_echo(c);
    return RTACX_OK;
}

rtacx_status rtacx_configure_precision(rtacx_ctx* ctx, const rtacx_precision_desc* desc)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    return configure_precision(c, desc);
}

rtacx_status rtacx_reduce_precision(rtacx_ctx* ctx, const void* samples, uint64_t n, float* out, void* stream)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(!c.prec_configured) { c.error = "call rtacx_configure_precision first"; return RTACX_ERR_NOT_CONFIGURED; }
    if(!out) { c.error = "null output buffer"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(n && !samples) { c.error = "null sample buffer"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(n >= (1ull << 32)) { c.error = "at most 2^32 - 1 samples per ping"; return RTACX_ERR_UNSUPPORTED; }
    if(reinterpret_cast<uintptr_t>(samples) % 4 != 0 || reinterpret_cast<uintptr_t>(out) % 16 != 0) {
        c.error = "samples must be 4-byte and the ping 16-byte aligned";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    c.bin.vec4 = reinterpret_cast<uintptr_t>(samples) % 16 == 0 ? 1 : 0;
    for(bool& t : c.traced) t = false;
    return run_precision(c, samples, n, out, static_cast<cudaStream_t>(stream));
}

rtacx_status rtacx_diag_drop_accumulation_stage(rtacx_ctx* ctx, uint32_t stage)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    ctx->impl.diag_drop_stage = stage;
    return RTACX_OK;
}

rtacx_status rtacx_diag_sorted(rtacx_ctx* ctx, float* records, uint64_t max_records, void* stream)
{
    if(!ctx || (!records && max_records)) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    const uint64_t k = std::min(max_records, c.d_sorted ? c.capacity : 0);
    if(k && cudaMemcpyAsync(records, c.d_sorted, k * sizeof(float4), cudaMemcpyDefault,
                            static_cast<cudaStream_t>(stream)) != cudaSuccess) {
        cudaGetLastError();
        c.error = "copying the sorted scratch failed";
        return RTACX_ERR_CUDA;
    }
    return RTACX_OK;
}

rtacx_status rtacx_set_tracing(rtacx_ctx* ctx, int enable)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    if(enable && !c.events[0]) {
        for(cudaEvent_t& e : c.events) {
            if(cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); c.error = "cudaEventCreate failed"; return RTACX_ERR_CUDA; }
        }
    }
    c.tracing = enable != 0;
    return RTACX_OK;
}

int rtacx_stage_times(rtacx_ctx* ctx, float* ms, int max)
{
    if(!ctx || !ms || max < 0) return -RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(!c.events[0]) return 0;
    int written = 0;
    for(int i = 0; i < RTACX_STAGE_COUNT && written < max; i++, written++) {
        ms[i] = 0.0f;
        if(!c.traced[i]) continue;
        if(cudaEventSynchronize(c.events[2 * i + 1]) != cudaSuccess ||
           cudaEventElapsedTime(&ms[i], c.events[2 * i], c.events[2 * i + 1]) != cudaSuccess) {
            cudaGetLastError();
            return -RTACX_ERR_CUDA;
        }
    }
    return written;
}

rtacx_status rtacx_stream_status(rtacx_ctx* ctx, void* stream)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(set_device(c) != RTACX_OK) return RTACX_ERR_CUDA;
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if(e != cudaSuccess) { c.error = std::string("stream: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    uint32_t word = 0;
    if(cudaMemcpy(&word, c.d_err, sizeof(word), cudaMemcpyDeviceToHost) != cudaSuccess ||
       cudaMemset(c.d_err, 0, sizeof(word)) != cudaSuccess) {
        cudaGetLastError();
        c.error = "reading the device error word failed";
        return RTACX_ERR_CUDA;
    }
    if(word) { c.error = "device error word " + std::to_string(word); return RTACX_ERR_DEVICE; }
    return RTACX_OK;
}

} // extern "C"
