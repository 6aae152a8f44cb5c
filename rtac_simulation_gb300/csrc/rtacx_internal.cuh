// Internal declarations shared by the rtacx translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/rtacx.h"
#include "rtacx_host.h"

namespace rtacx {

// Words between two pairs of bins' write cursors: the cursors of bins 2i and
// 2i + 1 share one 8-byte word (low and high half) at the start of a 128-byte
// L2 line, so one 64-bit atomicAdd reserves runs in both bins (positions stay
// below 2^32, so the low half never carries into the high half) and the
// reservations spread over all L2 slices.
constexpr uint32_t kCursorStride = 32;
constexpr uint32_t kScanBlock = 1024;     // bins per block of the parallel bin scan

// Word index of bin b's write cursor (see kCursorStride).
__host__ __device__ __forceinline__ size_t cursor_word(uint32_t b) { return (size_t)(b >> 1) * kCursorStride + (b & 1u); }
constexpr uint32_t kOutOfRange = RTACX_KEY_OUT_OF_RANGE;

// Device error word bits (OR-ed by kernels, read by rtacx_stream_status).
constexpr uint32_t kErrScatterOverflow = 1u << 0;  // sorted position beyond the counted total
constexpr uint32_t kErrBadWindow       = 1u << 1;  // window bounds outside the sorted array
constexpr uint32_t kErrGemmTimeout     = 1u << 2;  // a bounded mbarrier wait of the tensor-core GEMM expired
constexpr uint32_t kErrAccumulateTimeout = 1u << 3; // a bounded wait for a staged copy of samples expired
constexpr uint32_t kErrBatchWaitTimeout  = 1u << 4; // a bounded grid-barrier wait of the fused batched kernel expired
constexpr uint32_t kErrGatherTimeout     = 1u << 5; // a bounded mbarrier wait of the tensor-core gather expired

// Largest (range bin x bearing bin) histogram a CTA keeps in shared memory.
constexpr uint32_t kMaxSmemBins = 49152;

// A kernel's dynamic shared-memory limit is one value per kernel and device,
// shared by every context and host thread. Raise it to `bytes` if it is
// lower, never lower it: a smaller limit set for one context would make the
// larger launches of another context fail with an invalid-argument error.
// The error of a failed call is consumed (cudaGetLastError) and returned.
inline cudaError_t raise_smem_limit(const void* fn, size_t bytes)
{
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, fn);
    if(e == cudaSuccess && (size_t)a.maxDynamicSharedSizeBytes < bytes)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if(e != cudaSuccess) cudaGetLastError();
    return e;
}

// mbarrier helpers of the TMA pipelines (tensor-core GEMM, staged
// accumulation). Shared-memory addresses are 32-bit shared-window offsets.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Wait for the phase of the given parity, for at most `limit` SM clock
// cycles. Returns false (and sets *abort_flag) when the time runs out, or
// when another thread of the CTA has already set *abort_flag.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                                  long long limit)
{
    const long long t0 = clock64();
    while(!mbar_try_wait(bar, parity)) {
        if(*abort_flag) return false;
        if(clock64() - t0 > limit) { *abort_flag = 1; return false; }
    }
    return true;
}

// Everything the binning kernels need, passed by value.
struct BinParams {
    KeyParams key;
    uint32_t nBB;          // bearing sub-bins (1: range key only)
    float bb_scale;        // bearing bin = f(fmaf(bb_scale, bearing, bb_offset))
    float bb_offset;
    uint32_t nBins;        // nR * nBB
    uint32_t stride;       // floats per input record: 3 (SimSample1D) or 4 (SimSample2D)
    int vec4;              // 1 when records are 16-byte aligned float4s
    uint32_t echo_flags;   // RTACX_ECHO_* pre-step applied to each sample value (0: none)
    double echo_cycles;    // carrier cycles per metre of travel, 2 f / c
    float echo_k_hi;       // echo_cycles split into two floats (compensated phase)
    float echo_k_lo;
};

// Echo-sample epilogue of the reference's ray generator
// (src/RayCaster.cu:37-39, 69-71): value *= exp(i 4 pi f d / c) / d^2. The
// carrier phase is reduced modulo one cycle (d * 2f/c minus its nearest
// integer) before the float sincos, in one of two ways:
//   FP64         one fused multiply-add on the FP64 pipe (the only FP64
//                instruction per sample; GB300's FP64 rate is a small
//                fraction of its FP32 rate, so conversions go through the
//                bit fields below instead);
//   compensated  RTACX_ECHO_PHASE_COMPENSATED, float arithmetic that is as
//                exact for this range: t * k_hi split into its rounded
//                product and the exact rounding error (fmaf), the integer
//                part removed from the rounded product (exact below 2^23
//                cycles), the small terms added last.
// float -> double from the IEEE-754 bit fields (exact; the FP64 pipe is not
// used). Zero and subnormal inputs give a signed zero; infinities and NaNs
// do not reach the callers (their keys are out of range).
__device__ __forceinline__ double f64_from_f32_fields(float x)
{
    const uint32_t u = __float_as_uint(x);
    const uint32_t e = (u >> 23) & 0xffu;
    const uint32_t hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    return e == 0u ? __hiloint2double((int)(u & 0x80000000u), 0) : __hiloint2double((int)hi, (int)((u & 7u) << 29));
}

// double -> float from the bit fields, mantissa truncated toward zero
// (relative error below 2^-23); magnitudes under 2^-126 give a signed zero.
// Valid for |x| < 2^128.
__device__ __forceinline__ float f32_from_f64_fields(double x)
{
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
    const uint32_t e = (hi >> 20) & 0x7ffu;
    const uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    return __uint_as_float(e <= 896u ? (hi & 0x80000000u) : f);
}

// Carrier phase in cycles, reduced to about [-0.5, 0.5]: travel * 2 f / c
// minus the nearest whole number of cycles.
//   default      one FP64 fused multiply-add, travel * k - n, with n the
//                float-rounded cycle count: the reduction itself is exact to
//                2^-53 and it is the only FP64-pipe instruction per sample
//                (the conversions are integer bit operations).
//   compensated  no FP64: the float product's exact residual (fmaf) plus the
//                low part of k.
// FP64 form: k = 2 f / c, k_hi = (float)k.
__device__ __forceinline__ float carrier_fraction_f64(float travel, double k, float k_hi)
{
    const double r = fma(f64_from_f32_fields(travel), k, -f64_from_f32_fields(rintf(travel * k_hi)));
    return f32_from_f64_fields(r);
}

// `flags` is p.echo_flags, or a compile-time constant in kernels specialised
// for one echo model (the tests on it then fold away).
__device__ __forceinline__ float carrier_fraction(const BinParams& p, float travel, uint32_t flags)
{
    if(flags & RTACX_ECHO_PHASE_COMPENSATED) {
        const float prod = travel * p.echo_k_hi;
        const float err = fmaf(travel, p.echo_k_hi, -prod);
        const float whole = prod - rintf(prod);
        return whole + fmaf(travel, p.echo_k_lo, err);
    }
    return carrier_fraction_f64(travel, p.echo_cycles, p.echo_k_hi);
}

__device__ __forceinline__ float2 apply_echo(const BinParams& p, float2 v, float travel, uint32_t flags)
{
    if(flags & RTACX_ECHO_PHASE) {
        // |phase| <= pi: the hardware sine / cosine are accurate to ~4e-7 here.
        float sn, cs;
        __sincosf(carrier_fraction(p, travel, flags) * 6.28318530717958647692f, &sn, &cs);
        v = make_float2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
    }
    if(flags & RTACX_ECHO_SPREADING) {
        const float inv = __fdividef(1.0f, travel * travel);
        v = make_float2(v.x * inv, v.y * inv);
    }
    return v;
}

__device__ __forceinline__ float2 apply_echo(const BinParams& p, float2 v, float travel)
{
    return apply_echo(p, v, travel, p.echo_flags);
}

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

// range_key without branches (selects only), for kernels that interleave
// several samples per thread; the same key, without the side.
__device__ __forceinline__ uint32_t range_key_select(const KeyParams& k, float travel)
{
    const int res = __float2int_rz(fmaf(k.a, travel, k.b));
    const float fr = (float)res;
    const uint32_t below = fr >= k.lower ? 0u : kOutOfRange;
    const uint32_t above = fr <= k.upper ? k.nR - 1u : kOutOfRange;
    return res < 0 ? below : ((uint32_t)res >= k.nR ? above : (uint32_t)res);
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

// Grid of the binned precision model (see rtacx_reduce_precision in
// include/rtacx.h): range rows at the output-range resolution, a uniform
// bearing grid of `cells` bearings. Absolute range row j (row 0 at
// range_min) is stored at grid row j + row_shift; rows outside [row_lo,
// row_hi] reach no output row.
struct GridParams {
    float rmin, res, inv_res;
    float first, step, inv_step;
    uint32_t cells;
    uint32_t pitch;                  // entries per stored grid row (cells + padding)
    int row_lo, row_hi, row_shift;
};

// Grid coordinates of one sample with the model's float arithmetic, each
// operation rounded on its own (no contraction), as the oracle computes
// them: j = floor((t - rmin) / res), alpha = (t - (rmin + j res)) / res;
// q = clamp(floor((theta - first) / step), 0, cells - 2), w = clamp((theta -
// (first + q step)) / step, 0, 1) (divisions as products with the float
// reciprocals). Returns false for samples that reach no output row or carry
// a non-finite travel or bearing.
__device__ __forceinline__ bool grid_coords(const GridParams& g, float t, float th, int& jg, float& alpha, int& q,
                                            float& w)
{
    const float jf = floorf(__fmul_rn(__fsub_rn(t, g.rmin), g.inv_res));
    const bool ok = fabsf(t) < INFINITY && fabsf(th) < INFINITY && jf >= (float)g.row_lo && jf <= (float)g.row_hi;
    const int j = ok ? (int)jf : 0;
    alpha = __fmul_rn(__fsub_rn(t, __fadd_rn(g.rmin, __fmul_rn((float)j, g.res))), g.inv_res);
    jg = j + g.row_shift;
    const float qf = fminf(fmaxf(floorf(__fmul_rn(__fsub_rn(th, g.first), g.inv_step)), 0.0f), (float)(g.cells - 2u));
    q = (int)qf;
    w = fminf(fmaxf(__fmul_rn(__fsub_rn(th, __fadd_rn(g.first, __fmul_rn(qf, g.step))), g.inv_step), 0.0f), 1.0f);
    return ok;
}

// Reduction parameters of a configured sensor.
struct ReduceParams {
    int dims;
    uint32_t nR, nB;
    AxisLerp range_axis;
    AxisLerp beam_axis;
};

// Everything one ping of a batch needs on the device (rtacx_batch_*).
struct PingDev {
    const float* samples;
    uint64_t n;
    BinParams bin;
    uint32_t chunks;                 // CTAs of its count / scatter passes
    uint32_t* hist;
    uint32_t* totals;
    uint32_t* offsets;
    unsigned long long* oor;
    uint32_t* err;
    float4* sorted;
    uint32_t nR;
    int overlap;
    const int2* support;
    int2* win;
    ReduceParams red;
    const int2* bb_tiles;
    const float* ranges;
    const float* bearings;
    const float2* pulse;
    const float* beam;
    float2* out;
};

// Grid-barrier and work-queue state of the fused batched kernel (zeroed
// before every launch): barrier arrivals and generation, then one work
// counter per dynamically scheduled phase (count, scan, scatter, gather).
struct BatchSync {
    uint32_t arrived;
    uint32_t generation;
    uint32_t next[4];
};

// Parameters of the fused batched kernel. Maps are (ping, index) pairs.
struct FusedBatch {
    const PingDev* pings;
    const uint2* col_map;   uint32_t n_col;      // 256-bin groups of the totals to zero
    const uint2* chunk_map; uint32_t n_chunks;   // chunks of the count and scatter passes
    const uint2* scan_map;  uint32_t n_scan;     // kScanBlock-bin blocks of the bin scan
    const uint2* win_map;   uint32_t n_win;      // 256-row groups of the windows
    const uint4* items;     uint32_t n_items;    // gather items (2D tiles, 1D row groups)
    BatchSync* sync;
    uint32_t* status;                            // batch error word
    uint32_t arrivals;                           // CTAs each grid barrier waits for
    unsigned long long wait_ns;                  // bound of one barrier wait
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
    cudaArray_t psf_array = nullptr;    // RTACX_FLAG_TEXTURE_PSF: W x H float2 PSF image
    cudaTextureObject_t psf_tex = 0;    // ... linear filter, border, normalized coordinates
    float tex_xscale = 0.0f, tex_yscale = 0.0f;   // KernelView2D scalings .x (.y = 0.5)
    float* d_ranges = nullptr;          // [nR] Linspace values
    int2* d_support = nullptr;          // [nR] range bins that can hold PSF support of row r
    int2* d_bb_tiles = nullptr;         // bearing-bin range of each tile of width bearing_tile
    int2* d_bb_tiles64 = nullptr;       // ... of each 64-bearing tile
    int2* d_bb_tiles128 = nullptr;      // ... of each 128-bearing tile
    uint32_t* d_offsets = nullptr;      // [nBins + 1] exclusive scan of bin counts
    uint32_t* d_totals = nullptr;       // [nBins]
    int2* d_win = nullptr;              // [nR] effective bin range per row (lo > hi: empty)
    unsigned long long* d_oor = nullptr;// [2] low / high out-of-range counts
    uint32_t* d_err = nullptr;          // device error word

    // Sample-sized scratch.
    uint64_t capacity = 0;              // samples the sorted scratch holds
    float4* d_sorted = nullptr;
    uint32_t hist_ctas = 0;             // CTAs of the count pass (and of the batched passes)
    uint32_t scatter_ctas = 0;          // CTAs of the scatter pass
    int scatter_shape = 0;              // 1 + index of the staged scatter's shape (0: per-tile scatter)
    size_t acc_smem = 0;                // dynamic shared memory of the precision accumulation
    uint32_t acc_blocks_per_sm = 1;
    uint32_t hist_threads = 0;
    size_t hist_cols = 0;               // allocated words of d_hist (the write cursors)
    uint32_t* d_hist = nullptr;         // the scatter's per-bin write cursors (cursor_word), nBins x kCursorStride words

    // Split persistent gather of 2D pings (see rtacx_reduce.cu).
    uint32_t* d_tile_parts = nullptr;   // [tiles] sample-stream length of each output tile
    uint32_t* d_tile_first = nullptr;   // [tiles + 1] first item of each tile; [tiles] = item count
    uint4* d_items = nullptr;           // [tiles * 256] work items
    uint32_t* d_item_counter = nullptr; // work-queue counter

    // Receiver model of rtacx_make_samples (rtacx_configure_receiver).
    bool rx_configured = false;
    float rx_rotation[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    uint32_t rx_flags = 0;
    double rx_hz = 0.0;
    float* d_dir = nullptr;             // [dir_h][dir_w] receiver directivity
    uint32_t dir_w = 0, dir_h = 0;

    // Rasteriser scratch (rtacx_rasterize), grown on demand.
    unsigned char* d_rast_v = nullptr;  size_t rast_v_cap = 0;
    unsigned long long* d_rast_vis = nullptr; size_t rast_vis_cap = 0;
    uint32_t* d_rast_large = nullptr;   size_t rast_large_cap = 0;

    // Echo model (rtacx_set_echo_model).
    uint32_t echo_flags = 0;
    double echo_hz = 0.0;

    // Precision form (rtacx_configure_precision).
    bool prec_configured = false;
    uint32_t taps = 0, tap_center = 0;   // taps per output-row parity, index of node offset 0
    uint32_t Mpad = 0, Npad = 0, Kp = 0;
    uint32_t ksplit = 1;                // K parts of the contraction (partial products summed by the filter)
    GridParams grid{};                  // range nodes (two output bins apart) and uniform bearing grid
    uint32_t grid_rows = 0;             // (nR - 1) / 2 + 1 + taps + 1 node rows of the binned grid
    float4* d_G = nullptr;              // [grid_rows][grid.cells] bearing intervals: {left, right} shares (complex)
    uint32_t* d_flags = nullptr;        // [(nR + 31) / 32] bitmap of non-empty range bins (reference keys)
    uint32_t acc_staged_blocks[6] = {}; // resident CTAs per SM of each staged accumulation (0: not used)
    size_t acc_staged_smem = 0;
    uint32_t diag_drop_stage = 0xFFFFFFFFu; // failure-path test: stage whose copy the staged accumulation skips
    uint16_t* d_A = nullptr;            // [Mpad][Kp] bf16 [hi | hi | lo] split of the binned grid
    uint16_t* d_B = nullptr;            // [Npad][Kp] bf16 [hi | lo | hi] split of the directivity
    float* d_C = nullptr;               // [ksplit][Mpad][Npad] GEMM partial outputs: the grid contracted over bearings
    float2* d_taps = nullptr;           // [2][taps] range taps per output-row parity at node offsets t - tap_center
    // FP16 per-row-scaled contraction (RTACX_PRECISION_FP16_ROWSCALE): A and B
    // hold fp16 splits instead of bf16 ones.
    bool prec_f16 = false;
    float* d_row_scale = nullptr;       // [Mpad] 2^-e per grid row: undoes the row's scaling in the GEMM epilogue
    float* d_col_scale = nullptr;       // [Npad] 2^-e per directivity column
    // Hot range interval (RTACX_PRECISION_HOT_RANGE), in grid rows.
    bool prec_hot = false;
    int2* d_hot = nullptr;              // {first grid row, length} of the hot interval (length 0: none)
    uint32_t* d_hotcnt = nullptr;       // [grid_rows] subsample counts (zero between pings)
    float4* d_rep = nullptr;            // [hot rows][replicas][grid.cells] grid replicas

    // Host-buffer streaming (rtacx_reduce_precision_host): two device staging
    // buffers of RTACX_STREAM_CHUNK records, a copy stream fork-joined to the
    // caller's stream, and a device ping copied back to the host.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t stream_ev[5] = {};      // fork, copied[2], used[2]
    unsigned char* d_stage[2] = {};
    size_t stage_bytes = 0;
    float* d_ping = nullptr;
    size_t ping_floats = 0;

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

// Batched plain form. Maps are (ping, index) pairs: count / scatter chunks,
// column-scan bin blocks of 256, window row blocks of 256; gather items are
// {ping, tile_b, tile_r, 0} for 2D pings and {ping, row_group, 0, 1} for 1D.
rtacx_status launch_bin_batch(std::string& error, const PingDev* pings, uint32_t n_pings,
                              const uint2* chunk_map, uint32_t n_chunks, const uint2* col_map, uint32_t n_col,
                              const uint2* win_map, uint32_t n_win, uint32_t max_bins, cudaStream_t stream);
rtacx_status prepare_bin_batch(std::string& error, uint32_t max_bins);
rtacx_status prepare_gather_batch(std::string& error, int shape, size_t smem);
size_t gather_batch_smem(int shape, uint32_t H, uint32_t W);
rtacx_status launch_gather_batch(std::string& error, int shape, const PingDev* pings, const uint4* items,
                                 uint32_t n_items, uint32_t* counter, size_t smem, uint32_t grid,
                                 cudaStream_t stream);
// Fused batched form: the whole batch (zeroing, count, scan, windows,
// scatter, gather) in one cooperative persistent launch.
rtacx_status prepare_fused_batch(std::string& error, int shape, size_t smem, int sm_count, uint32_t& grid);
rtacx_status launch_fused_batch(std::string& error, int shape, const FusedBatch& fb, size_t smem, uint32_t grid,
                                cudaStream_t stream);
int gather_shape_rows(int shape);
int gather_shape_bearings(int shape);

// Precision form (rtacx_precision.cu).
rtacx_status run_precision(Context& ctx, const void* samples, uint64_t n, float* out, cudaStream_t stream);
rtacx_status precision_begin(Context& ctx, cudaStream_t stream);
rtacx_status precision_hot_scan(Context& ctx, const void* samples, uint64_t n, cudaStream_t stream);
rtacx_status precision_accumulate(Context& ctx, const void* samples, uint64_t n, cudaStream_t stream);
rtacx_status precision_finish(Context& ctx, float* out, cudaStream_t stream);
void free_streaming(Context& ctx);
void free_precision(Context& ctx);

// Tensor-core GEMM (rtacx_umma.cu): C = row_scale * col_scale * (A * B^T),
// K-major operands, both bf16 or both fp16 (f16); scales optional; ksplit
// partial products at C + z M ldc.
rtacx_status gemm_tn(std::string& error, const void* A, const void* B, float* C, int M, int N, int K, int ldc,
                     cudaStream_t stream, uint32_t* err, bool f16, const float* row_scale, const float* col_scale,
                     int ksplit);
size_t gemm_smem_bytes();

} // namespace rtacx

struct rtacx_ctx {
    rtacx::Context impl;
};
