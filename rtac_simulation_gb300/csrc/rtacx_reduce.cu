// Plain sparse PSF reduction (FP32 SIMT).
//
// Replaces do_sparse_convolve_2d_f (src/SensorInstance2D.cu:44-119) and
// do_sparse_convolve_1d_f (src/SensorInstance1D.cu:35-89):
//   out(r, b) = sum_{s in window(r)} v_s * pulse(t_s - R_r) * beam(theta_s - theta_b)
// where pulse / beam are the texture lookups of KernelView2D
// (include/rtac_simulation/ReductionKernel.h:44-73): normalized coordinate
// u = scale * delta + 0.5, linear filter, border addressing. The bilinear
// fetch of the separable table PSF[h][w] = pulse[h] * beam[w]
// (src/SensorInstance2D.cu:20-33) is the product of the two 1D lerps, which
// this file evaluates in software from shared-memory copies of the 1D tables
// with exact (not 9-bit fixed point) weights.
//
// 2D layout: one CTA per (TR range rows x TB bearings) tile. Samples of the
// tile's range-bin span and bearing-bin span are streamed through shared
// memory in chunks of K; for each chunk the CTA evaluates
//   U[k][r] = v_k * pulse(t_k - R_r)   (zero unless bin_k is in row r's window)
//   B[k][b] = beam(theta_k - theta_b)
// once, then every thread accumulates its (rows x bearings) register block:
// acc[r][b] += U[k][r] * B[k][b]. A warp skips a chunk whose range bins lie
// outside its rows' windows.
#include "rtacx_bin_device.cuh"
#include "rtacx_internal.cuh"
#include "rtacx_tcgen05.cuh"

#include <algorithm>

namespace rtacx {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kChunk = 64;

// Lerp of a zero-padded table (tab[0] = tab[n + 1] = 0, tab[i + 1] = T[i]).
// Returns 0 outside the support of the border-addressed linear filter.
__device__ __forceinline__ float lerp_real(const float* tab, const AxisLerp& ax, float delta)
{
    const float x1 = fmaf(delta, ax.k_hi, ax.c);
    const float fi = floorf(x1);
    if(!(fi >= -1.0f && fi <= (float)(ax.n - 1))) return 0.0f;
    const float alpha = fmaf(delta, ax.k_lo, fmaf(delta, ax.k_hi, ax.c - fi));
    const int i = (int)fi + 1;
    const float lo = tab[i], hi = tab[i + 1];
    return fmaf(alpha, hi - lo, lo);
}

__device__ __forceinline__ float2 lerp_cplx(const float2* tab, const AxisLerp& ax, float delta)
{
    const float x1 = fmaf(delta, ax.k_hi, ax.c);
    const float fi = floorf(x1);
    if(!(fi >= -1.0f && fi <= (float)(ax.n - 1))) return make_float2(0.f, 0.f);
    const float alpha = fmaf(delta, ax.k_lo, fmaf(delta, ax.k_hi, ax.c - fi));
    const int i = (int)fi + 1;
    const float2 lo = tab[i], hi = tab[i + 1];
    return make_float2(fmaf(alpha, hi.x - lo.x, lo.x), fmaf(alpha, hi.y - lo.y, lo.y));
}

__device__ __forceinline__ void red_add_v2(float2* addr, float2 v)
{
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(addr), "f"(v.x), "f"(v.y) : "memory");
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

template <int TR, int TB>
struct GatherSmem {
    float2 U[kChunk][TR];
    float B[kChunk][TB];
    float4 smp[kChunk];
    int bin[kChunk];
    uint32_t seg_start[kThreads];
    uint32_t seg_pre[kThreads + 1];
    float R[TR];
    float theta[TB];
    int elo[TR], ehi[TR];
    uint32_t warp_sums[kWarps];
    int jmin, jmax;
};

// One (TR rows x TB bearings) output tile (tile_b, tile_r) of a 2D ping;
// smem_raw holds GatherSmem<TR, TB> followed by the padded pulse and beam.
template <int TR, int TB>
__device__ __forceinline__ void gather_tile_2d(const float4* __restrict__ sorted, const uint32_t* __restrict__ off,
                                               const int2* __restrict__ win, const int2* __restrict__ bb_tiles,
                                               const float* __restrict__ ranges, const float* __restrict__ bearings,
                                               const float2* __restrict__ pulse_pad, const float* __restrict__ beam_pad,
                                               const ReduceParams& rp, uint32_t nBB, float2* __restrict__ out,
                                               int tile_b, int tile_r, unsigned char* smem_raw,
                                               uint32_t g_begin = 0u, uint32_t g_end = 0xFFFFFFFFu,
                                               bool atomic_out = false)
{
    constexpr int RPW = TR / kWarps;   // rows per warp
    constexpr int BPL = TB / 32;       // bearings per lane
    static_assert(TR % kWarps == 0 && TB % 32 == 0, "tile shape");
    using Smem = GatherSmem<TR, TB>;

    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    float2* s_pulse = reinterpret_cast<float2*>(smem_raw + sizeof(Smem));
    float* s_beam = reinterpret_cast<float*>(s_pulse + (rp.range_axis.n + 2));

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = tile_r * TR, b0 = tile_b * TB;
    const int nR = (int)rp.nR, nB = (int)rp.nB;

    for(int i = tid; i < rp.range_axis.n + 2; i += kThreads) s_pulse[i] = pulse_pad[i];
    for(int i = tid; i < rp.beam_axis.n + 2; i += kThreads) s_beam[i] = beam_pad[i];
    if(tid == 0) { S.jmin = INT_MAX; S.jmax = INT_MIN; }
    __syncthreads();
    if(tid < TR) {
        const int r = r0 + tid;
        int2 w = make_int2(1, 0);
        float R = 0.0f;
        if(r < nR) { w = win[r]; R = ranges[r]; }
        S.elo[tid] = w.x; S.ehi[tid] = w.y; S.R[tid] = R;
        if(w.x <= w.y) { atomicMin(&S.jmin, w.x); atomicMax(&S.jmax, w.y); }
    }
    for(int i = tid; i < TB; i += kThreads) {
        const int b = b0 + i;
        S.theta[i] = b < nB ? bearings[b] : 0.0f;
    }
    __syncthreads();

    // Range-bin span of this warp's rows.
    int wlo = INT_MAX, whi = INT_MIN;
#pragma unroll
    for(int q = 0; q < RPW; q++) {
        const int rr = warp * RPW + q;
        if(S.elo[rr] <= S.ehi[rr]) { wlo = min(wlo, S.elo[rr]); whi = max(whi, S.ehi[rr]); }
    }

    float2 acc[RPW][BPL];
#pragma unroll
    for(int q = 0; q < RPW; q++)
#pragma unroll
        for(int c = 0; c < BPL; c++) acc[q][c] = make_float2(0.f, 0.f);

    const int jmin = S.jmin, jmax = S.jmax;
    const int2 kb = bb_tiles[tile_b];
    // The tile's samples form one stream: the bearing-bin segments of range
    // bins jmin..jmax in order. This call reduces stream positions
    // [g_begin, g_end); `base` is the stream position of the current group.
    uint32_t base = 0;
    for(int jg = jmin; jg <= jmax && base < g_end; jg += kThreads) {
        // Segment of bin (jg + tid) restricted to this tile's bearing bins.
        const int j = jg + tid;
        uint32_t start = 0, len = 0;
        if(j <= jmax) {
            start = off[(size_t)j * nBB + kb.x];
            len = off[(size_t)j * nBB + kb.y + 1] - start;
        }
        // Exclusive scan of the segment lengths.
        uint32_t x = len;
        for(int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if(lane >= o) x += y;
        }
        if(lane == 31) S.warp_sums[warp] = x;
        __syncthreads();
        uint32_t before = 0, total = 0;
        for(int w = 0; w < kWarps; w++) {
            const uint32_t v = S.warp_sums[w];
            if(w < warp) before += v;
            total += v;
        }
        S.seg_start[tid] = start;
        S.seg_pre[tid] = before + x - len;
        if(tid == 0) S.seg_pre[kThreads] = total;
        __syncthreads();

        const uint32_t lo = g_begin > base ? min(g_begin - base, total) : 0u;
        const uint32_t hi = (g_end - base < total) ? g_end - base : total;
        base += total;
        for(uint32_t c0 = lo; c0 < hi; c0 += kChunk) {
            const int valid = (int)((hi - c0) < (uint32_t)kChunk ? (hi - c0) : (uint32_t)kChunk);
            if(tid < kChunk) {
                if(tid < valid) {
                    const uint32_t g = c0 + tid;
                    int lo = 0, hi = kThreads - 1;     // largest t with seg_pre[t] <= g
                    while(lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if(S.seg_pre[mid] <= g) lo = mid; else hi = mid - 1;
                    }
                    S.smp[tid] = sorted[S.seg_start[lo] + (g - S.seg_pre[lo])];
                    S.bin[tid] = jg + lo;
                }
                else {
                    S.smp[tid] = make_float4(0.f, 0.f, 0.f, 0.f);
                    S.bin[tid] = INT_MIN;
                }
            }
            __syncthreads();
            for(int e = tid; e < kChunk * TR; e += kThreads) {
                const int k = e / TR, rr = e % TR;
                const int bin = S.bin[k];
                float2 u = make_float2(0.f, 0.f);
                if(bin >= S.elo[rr] && bin <= S.ehi[rr]) {
                    const float4 s = S.smp[k];
                    const float2 w = lerp_cplx(s_pulse, rp.range_axis, s.z - S.R[rr]);
                    u = cmul(make_float2(s.x, s.y), w);
                }
                S.U[k][rr] = u;
            }
            for(int e = tid; e < kChunk * TB; e += kThreads) {
                const int k = e / TB, bb = e % TB;
                float v = 0.0f;
                if(k < valid && b0 + bb < nB) v = lerp_real(s_beam, rp.beam_axis, S.smp[k].w - S.theta[bb]);
                S.B[k][bb] = v;
            }
            __syncthreads();
            const int cb0 = S.bin[0], cb1 = S.bin[valid - 1];
            if(cb1 >= wlo && cb0 <= whi) {
                for(int k = 0; k < valid; k++) {
                    float2 u[RPW];
                    float bv[BPL];
#pragma unroll
                    for(int q = 0; q < RPW; q++) u[q] = S.U[k][warp * RPW + q];
#pragma unroll
                    for(int c = 0; c < BPL; c++) bv[c] = S.B[k][lane * BPL + c];
#pragma unroll
                    for(int q = 0; q < RPW; q++)
#pragma unroll
                        for(int c = 0; c < BPL; c++) {
                            acc[q][c].x = fmaf(u[q].x, bv[c], acc[q][c].x);
                            acc[q][c].y = fmaf(u[q].y, bv[c], acc[q][c].y);
                        }
                }
            }
            __syncthreads();
        }
    }
#pragma unroll
    for(int q = 0; q < RPW; q++) {
        const int r = r0 + warp * RPW + q;
        if(r >= nR) continue;
#pragma unroll
        for(int c = 0; c < BPL; c++) {
            const int b = b0 + lane * BPL + c;
            if(b >= nB) continue;
            if(atomic_out) red_add_v2(out + (size_t)r * nB + b, acc[q][c]);
            else out[(size_t)r * nB + b] = acc[q][c];
        }
    }
}

template <int TR, int TB>
__global__ void __launch_bounds__(kThreads)
k_gather_2d(const float4* __restrict__ sorted, const uint32_t* __restrict__ off,
            const int2* __restrict__ win, const int2* __restrict__ bb_tiles,
            const float* __restrict__ ranges, const float* __restrict__ bearings,
            const float2* __restrict__ pulse_pad, const float* __restrict__ beam_pad,
            ReduceParams rp, uint32_t nBB, float2* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    gather_tile_2d<TR, TB>(sorted, off, win, bb_tiles, ranges, bearings, pulse_pad, beam_pad, rp, nBB, out,
                           blockIdx.x, blockIdx.y, smem_raw);
}

// 1D: one warp per output range bin; rows [row0, row0 + kWarps). The pulse
// table must already be in s_pulse.
__device__ __forceinline__ void gather_rows_1d(const float4* __restrict__ sorted, const uint32_t* __restrict__ off,
                                               const int2* __restrict__ win, const float* __restrict__ ranges,
                                               const float2* s_pulse, const ReduceParams& rp,
                                               float2* __restrict__ out, int row0)
{
    const int lane = threadIdx.x & 31;
    const int r = row0 + (threadIdx.x >> 5);
    if(r >= (int)rp.nR) return;
    const int2 w = win[r];
    float2 acc = make_float2(0.f, 0.f);
    if(w.x <= w.y) {
        const float R = ranges[r];
        const uint32_t p0 = off[w.x], p1 = off[w.y + 1];
        auto add = [&](const float4& s) {
            const float2 wv = lerp_cplx(s_pulse, rp.range_axis, s.z - R);
            const float2 u = cmul(make_float2(s.x, s.y), wv);
            acc.x += u.x; acc.y += u.y;
        };
        uint32_t i = p0 + lane;
        // Four records per lane in flight, then the remainder.
        for(; i + 96 < p1; i += 128) {
            const float4 s0 = sorted[i], s1 = sorted[i + 32], s2 = sorted[i + 64], s3 = sorted[i + 96];
            add(s0); add(s1); add(s2); add(s3);
        }
        for(; i < p1; i += 32) add(sorted[i]);
    }
    for(int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if(lane == 0) out[r] = acc;
}

__global__ void __launch_bounds__(kThreads)
k_gather_1d(const float4* __restrict__ sorted, const uint32_t* __restrict__ off,
            const int2* __restrict__ win, const float* __restrict__ ranges,
            const float2* __restrict__ pulse_pad, ReduceParams rp, float2* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s_pulse = reinterpret_cast<float2*>(smem_raw);
    for(int i = threadIdx.x; i < rp.range_axis.n + 2; i += kThreads) s_pulse[i] = pulse_pad[i];
    __syncthreads();
    gather_rows_1d(sorted, off, win, ranges, s_pulse, rp, out, blockIdx.x * kWarps);
}

// ---- RTACX_FLAG_TEXTURE_PSF: the reference's texture evaluation ------------
// One warp per output cell (r, b): the lanes stride over the samples of row
// r's window (range-only bins, so one contiguous run of the sorted samples,
// as the reference's bin view), fetch the PSF from the texture at the
// reference kernel's coordinates (fmaf(1 / span, theta_s - theta_b, 0.5),
// fmaf(1 / (duration c), t_s - R_r, 0.5); src/SensorInstance2D.cu:59-64,
// include/rtac_simulation/ReductionKernel.h:63-69) and accumulate
// value * psf in complex float; a warp reduction writes the cell.
__global__ void __launch_bounds__(kThreads)
k_gather_tex(const float4* __restrict__ sorted, const uint32_t* __restrict__ off, const int2* __restrict__ win,
             const float* __restrict__ ranges, const float* __restrict__ bearings, cudaTextureObject_t psf,
             float xscale, float yscale, uint32_t nR, uint32_t nB, float2* __restrict__ out)
{
    const uint64_t cell = ((uint64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if(cell >= (uint64_t)nR * nB) return;
    const uint32_t r = (uint32_t)(cell / nB), b = (uint32_t)(cell % nB);
    const int2 w = win[r];
    float2 acc = make_float2(0.f, 0.f);
    if(w.x <= w.y) {
        const float R = ranges[r], th = bearings[b];
        const uint32_t p0 = off[w.x], p1 = off[w.y + 1];
        for(uint32_t i = p0 + lane; i < p1; i += 32) {
            const float4 s = sorted[i];
            const float2 f = tex2D<float2>(psf, fmaf(xscale, s.w - th, 0.5f), fmaf(yscale, s.z - R, 0.5f));
            acc.x += s.x * f.x - s.y * f.y;
            acc.y += s.x * f.y + s.y * f.x;
        }
    }
    for(int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if(lane == 0) out[cell] = acc;
}

// RTACX_FLAG_TEXTURE_PSF on a 1D sensor: one warp per output range r, the
// lanes stride over row r's window and fetch the pulse as the reference's 1D
// kernel does, tex1D at fmaf(scale, t_s - R_r, 0.5)
// (src/SensorInstance1D.cu:52-55, include/rtac_simulation/ReductionKernel.h:
// 44-55); value * pulse in complex float, a warp reduction writes the row.
__global__ void __launch_bounds__(kThreads)
k_gather_tex_1d(const float4* __restrict__ sorted, const uint32_t* __restrict__ off, const int2* __restrict__ win,
                const float* __restrict__ ranges, cudaTextureObject_t pulse, float scale, uint32_t nR,
                float2* __restrict__ out)
{
    const uint32_t r = (blockIdx.x * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if(r >= nR) return;
    const int2 w = win[r];
    float2 acc = make_float2(0.f, 0.f);
    if(w.x <= w.y) {
        const float R = ranges[r];
        const uint32_t p0 = off[w.x], p1 = off[w.y + 1];
        for(uint32_t i = p0 + lane; i < p1; i += 32) {
            const float4 s = sorted[i];
            const float2 f = tex1D<float2>(pulse, fmaf(scale, s.z - R, 0.5f));
            acc.x += s.x * f.x - s.y * f.y;
            acc.y += s.x * f.y + s.y * f.x;
        }
    }
    for(int o = 16; o > 0; o >>= 1) {
        acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
        acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if(lane == 0) out[r] = acc;
}

// ---- split persistent gather of one 2D ping -------------------------------
// k_tile_plan (one CTA) counts each output tile's sample stream (same
// definition as gather_tile_2d), picks the part size so that the ping yields
// about kItemsPerWorker work items per persistent CTA (between
// kMinPartSamples and kPartSamples samples per part, at most kMaxParts parts
// per tile), scans the part counts and writes one work item per part; the
// persistent kernel reduces the parts, accumulating into the zeroed ping with
// vector atomics. Tiles whose windows hold hot bins are spread over many
// CTAs, and a small ping still spreads over the whole GPU.
constexpr uint32_t kPartSamples = 16384, kMinPartSamples = 512, kItemsPerWorker = 4;
constexpr uint32_t kMaxParts = 256;
constexpr int kPlanThreads = 1024;

// counts[t]: stream length of tile t (read by the gathers for their part
// bounds); first[t]: first item of tile t, first[tiles] = the item count.
template <int TR>
__global__ void __launch_bounds__(kPlanThreads)
k_tile_plan(const uint32_t* __restrict__ off, const int2* __restrict__ win, const int2* __restrict__ bb_tiles,
            uint32_t nR, uint32_t nBB, uint32_t tiles_b, uint32_t tiles, uint32_t workers,
            uint32_t* __restrict__ counts, uint32_t* __restrict__ first, uint4* __restrict__ items)
{
    __shared__ uint32_t s_warp[32];
    __shared__ unsigned long long s_sum[kPlanThreads / 32];
    __shared__ uint32_t s_part;
    unsigned long long mine = 0;
    for(uint32_t t = threadIdx.x; t < tiles; t += kPlanThreads) {
        const uint32_t tb = t % tiles_b, tr = t / tiles_b;
        int jmin = INT_MAX, jmax = INT_MIN;
        for(int q = 0; q < TR; q++) {
            const int r = (int)tr * TR + q;
            if(r >= (int)nR) break;
            const int2 w = win[r];
            if(w.x <= w.y) { jmin = min(jmin, w.x); jmax = max(jmax, w.y); }
        }
        uint64_t count = 0;
        const int2 kb = bb_tiles[tb];
        for(int j = jmin; j <= jmax; j++)
            count += off[(size_t)j * nBB + kb.y + 1] - off[(size_t)j * nBB + kb.x];
        const uint32_t c = (uint32_t)min(count, (uint64_t)0xFFFFFFFFu);
        counts[t] = c;
        mine += c;
    }
    for(int o = 16; o > 0; o >>= 1) mine += __shfl_down_sync(0xffffffffu, mine, o);
    if((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = mine;
    __syncthreads();
    if(threadIdx.x == 0) {
        unsigned long long total = 0;
        for(int w = 0; w < kPlanThreads / 32; w++) total += s_sum[w];
        const unsigned long long want = (unsigned long long)max(workers, 1u) * kItemsPerWorker;
        const unsigned long long part = (total + want - 1) / want;
        s_part = (uint32_t)min(max(part, (unsigned long long)kMinPartSamples), (unsigned long long)kPartSamples);
    }
    __syncthreads();
    const uint64_t part = s_part;
    uint32_t carry = 0;
    for(uint32_t t0 = 0; t0 < tiles; t0 += kPlanThreads) {
        const uint32_t t = t0 + threadIdx.x;
        uint32_t np = 0;
        if(t < tiles) np = (uint32_t)min(((uint64_t)counts[t] + part - 1) / part, (uint64_t)kMaxParts);
        uint32_t seg_total;
        const uint32_t f = carry + block_exclusive_scan(np, s_warp, seg_total);
        if(t < tiles) {
            first[t] = f;
            for(uint32_t q = 0; q < np; q++) items[f + q] = make_uint4(t % tiles_b, t / tiles_b, q, np);
        }
        carry += seg_total;
    }
    if(threadIdx.x == 0) first[tiles] = carry;
}

template <int TR, int TB>
__global__ void __launch_bounds__(kThreads)
k_gather_split(const float4* __restrict__ sorted, const uint32_t* __restrict__ off,
               const int2* __restrict__ win, const int2* __restrict__ bb_tiles,
               const float* __restrict__ ranges, const float* __restrict__ bearings,
               const float2* __restrict__ pulse_pad, const float* __restrict__ beam_pad,
               ReduceParams rp, uint32_t nBB, float2* __restrict__ out,
               const uint4* __restrict__ items, const uint32_t* __restrict__ n_items_ptr,
               const uint32_t* __restrict__ tile_counts, uint32_t tiles_b, uint32_t* __restrict__ counter)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_item;
    const uint32_t n_items = *n_items_ptr;
    for(;;) {
        if(threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if(it >= n_items) break;
        const uint4 item = items[it];
        uint32_t g0 = 0, g1 = 0xFFFFFFFFu;
        if(item.w > 1) {
            // This part's share of the tile's stream.
            const uint64_t count = tile_counts[item.y * tiles_b + item.x];
            g0 = (uint32_t)(count * item.z / item.w);
            g1 = (uint32_t)(count * (item.z + 1) / item.w);
        }
        gather_tile_2d<TR, TB>(sorted, off, win, bb_tiles, ranges, bearings, pulse_pad, beam_pad, rp, nBB, out,
                               (int)item.x, (int)item.y, smem_raw, g0, g1, true);
        __syncthreads();
    }
}

// ---- tensor-core gather of one 2D ping (tcgen05, TF32 x3) -----------------
// The gather of a tile is a sum of outer products: for every sample k of the
// tile's stream, out(r, b) += U[k][r] B[k][b] with U[k][r] = v_k pulse(t_k -
// R_r) (complex, zero outside row r's window) and B[k][b] = beam(theta_k -
// theta_b) (real). k_gather_tc evaluates U and B for chunks of 32 samples
// into shared memory and lets the tensor cores form the products: D (128 x
// 128 fp32 in TMEM, rows 0..63 the real and 64..127 the imaginary parts of
// 64 output ranges, columns 128 output bearings) += A B^T with A = [Re U; Im
// U], both operands K-major in the 128-byte swizzle layout. FP32 accuracy
// from TF32 operands: each operand is split into tf32 hi + lo (21 significant
// bits together) and three MMAs form hi*hi + hi*lo + lo*hi, products exact
// in the FP32 accumulator. Per chunk the 512 threads write the operands of
// one of two stages while the MMAs of the other run; one thread issues the
// MMAs and commits them to the stage's mbarrier. The persistent CTA takes
// (tile, part) items like k_gather_split and adds each finished tile into
// the zeroed ping with vector reductions.
constexpr int kTcRows = 64, kTcBearings = 128, kTcChunk = 32;
constexpr int kTcThreads = 512, kTcWarps = kTcThreads / 32;
constexpr uint32_t kTcOpBytes = 128u * 128u;                 // 128 rows x 32 tf32
constexpr uint32_t kTcStageBytes = 4u * kTcOpBytes;          // A hi, A lo, B hi, B lo
constexpr uint32_t kTcTmemCols = 128;
constexpr int kTcPitch = 129;                                // epilogue rows (floats), bank-conflict free
constexpr long long kTcWaitCycles = 2000000000ll;            // about one second
// The tensor cores' FP32 accumulation over a whole tile stream (up to 12
// MMAs per chunk, hundreds of chunks) drifts to ~1e-5 relative; every
// kTcFlush chunks the accumulator is added into FP32 registers (round to
// nearest) and restarted, which keeps the tensor-core chains short.
constexpr uint32_t kTcFlush = 8;
// tcgen05.mma.kind::tf32 instruction descriptor: D f32 (bits 4-5 = 1), A and
// B tf32 (format 2 at bits 7-9 and 10-12), both K-major, N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdescTf32 = (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

struct TcSmem {
    float4 smp[kTcChunk];
    int bin[kTcChunk];
    uint32_t seg_start[kTcThreads];
    uint32_t seg_pre[kTcThreads + 1];
    float R[kTcRows];
    float theta[kTcBearings];
    int elo[kTcRows], ehi[kTcRows];
    uint32_t warp_sums[kTcWarps];
    int jmin, jmax;
    uint32_t item;
    unsigned long long bar[2];
    uint32_t tmem;
    int abort;
};

__device__ __forceinline__ uint32_t tf32_bits(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// x as tf32 hi + lo: hi = tf32(x), lo = tf32(x - hi).
__device__ __forceinline__ void tf32_split(float x, uint32_t& hi, uint32_t& lo)
{
    hi = tf32_bits(x);
    lo = tf32_bits(x - __uint_as_float(hi));
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdescTf32), "r"(accumulate)
                 : "memory");
}

size_t gather_tc_smem_bytes(uint32_t H, uint32_t W)
{
    return 1024 + 2 * (size_t)kTcStageBytes + (H + 2) * sizeof(float2) + (W + 2) * sizeof(float);
}

__global__ void __launch_bounds__(kTcThreads, 1)
k_gather_tc(const float4* __restrict__ sorted, const uint32_t* __restrict__ off,
            const int2* __restrict__ win, const int2* __restrict__ bb_tiles,
            const float* __restrict__ ranges, const float* __restrict__ bearings,
            const float2* __restrict__ pulse_pad, const float* __restrict__ beam_pad,
            ReduceParams rp, uint32_t nBB, float2* __restrict__ out,
            const uint4* __restrict__ items, const uint32_t* __restrict__ n_items_ptr,
            const uint32_t* __restrict__ tile_counts, uint32_t tiles_b,
            uint32_t* __restrict__ counter, uint32_t* __restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ TcSmem S;
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* stages = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
    float2* s_pulse = reinterpret_cast<float2*>(stages + 2 * kTcStageBytes);
    float* s_beam = reinterpret_cast<float*>(s_pulse + (rp.range_axis.n + 2));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nR = (int)rp.nR, nB = (int)rp.nB;
    const uint32_t n_items = *n_items_ptr;

    for(int i = tid; i < rp.range_axis.n + 2; i += kTcThreads) s_pulse[i] = pulse_pad[i];
    for(int i = tid; i < rp.beam_axis.n + 2; i += kTcThreads) s_beam[i] = beam_pad[i];
    if(tid == 0) {
        mbar_init(smem_u32(&S.bar[0]), 1);
        mbar_init(smem_u32(&S.bar[1]), 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if(warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    uint32_t gchunk = 0;          // chunks committed by this CTA (stage = gchunk & 1)
    // This thread's share of the accumulator: TMEM lane quad * 32 + lane,
    // columns 32 cg .. 32 cg + 31.
    const int quad = warp & 3, cg = warp >> 2;
    float acc[32];
    // Waits for the last committed chunk, then adds the TMEM accumulator into
    // acc (the next MMA starts a new chain). False if the wait expired.
    auto flush = [&]() -> bool {
        if(tid == 0 &&
           !mbar_wait_bounded(smem_u32(&S.bar[(gchunk - 1) & 1u]), ((gchunk - 1) >> 1) & 1u, &S.abort, kTcWaitCycles))
            atomicOr(err, kErrGatherTimeout);
        __syncthreads();
        if(S.abort) return false;
        tc_fence_after();
        {
            uint32_t v[32];
            tmem_ld32(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(cg * 32), v);
#pragma unroll
            for(int q = 0; q < 32; q++) acc[q] += __uint_as_float(v[q]);
        }
        tc_fence_before();
        __syncthreads();
        return true;
    };

    for(;;) {
        if(tid == 0) S.item = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t it = S.item;
        if(it >= n_items || S.abort) break;
        const uint4 item = items[it];
        const int r0 = (int)item.y * kTcRows, b0 = (int)item.x * kTcBearings;
        if(tid == 0) { S.jmin = INT_MAX; S.jmax = INT_MIN; }
        __syncthreads();
        if(tid < kTcRows) {
            const int r = r0 + tid;
            int2 w = make_int2(1, 0);
            float R = 0.0f;
            if(r < nR) { w = win[r]; R = ranges[r]; }
            S.elo[tid] = w.x; S.ehi[tid] = w.y; S.R[tid] = R;
            if(w.x <= w.y) { atomicMin(&S.jmin, w.x); atomicMax(&S.jmax, w.y); }
        }
        if(tid < kTcBearings) S.theta[tid] = b0 + tid < nB ? bearings[b0 + tid] : 0.0f;
        __syncthreads();
        const int jmin = S.jmin, jmax = S.jmax;
        const int2 kb = bb_tiles[item.x];
        // This part's share [g_begin, g_end) of the tile's sample stream.
        uint32_t g_begin = 0, g_end = 0xFFFFFFFFu;
        if(item.w > 1) {
            const uint64_t count = tile_counts[item.y * tiles_b + item.x];
            g_begin = (uint32_t)(count * item.z / item.w);
            g_end = (uint32_t)(count * (item.z + 1) / item.w);
        }
        uint32_t nchunk = 0, chain = 0, base = 0;
        bool stop = false;
#pragma unroll
        for(int q = 0; q < 32; q++) acc[q] = 0.0f;
        for(int jg = jmin; jg <= jmax && base < g_end && !stop; jg += kTcThreads) {
            const int j = jg + tid;
            uint32_t start = 0, len = 0;
            if(j <= jmax) {
                start = off[(size_t)j * nBB + kb.x];
                len = off[(size_t)j * nBB + kb.y + 1] - start;
            }
            uint32_t x = len;
            for(int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if(lane >= o) x += y;
            }
            if(lane == 31) S.warp_sums[warp] = x;
            __syncthreads();
            uint32_t before = 0, total = 0;
            for(int w = 0; w < kTcWarps; w++) {
                const uint32_t v = S.warp_sums[w];
                if(w < warp) before += v;
                total += v;
            }
            S.seg_start[tid] = start;
            S.seg_pre[tid] = before + x - len;
            if(tid == 0) S.seg_pre[kTcThreads] = total;
            __syncthreads();
            const uint32_t lo = g_begin > base ? min(g_begin - base, total) : 0u;
            const uint32_t hi = (g_end - base < total) ? g_end - base : total;
            base += total;
            // Stream position g of this group -> (sample, bin), for the 32
            // loader threads.
            auto fetch = [&](uint32_t c0, float4& smp, int& bin) {
                const uint32_t g = c0 + (uint32_t)tid;
                if(g < hi) {
                    int a = 0, z = kTcThreads - 1;        // largest t with seg_pre[t] <= g
                    while(a < z) {
                        const int mid = (a + z + 1) >> 1;
                        if(S.seg_pre[mid] <= g) a = mid; else z = mid - 1;
                    }
                    smp = sorted[S.seg_start[a] + (g - S.seg_pre[a])];
                    bin = jg + a;
                }
                else {
                    smp = make_float4(0.f, 0.f, 0.f, 0.f);
                    bin = INT_MIN;
                }
            };
            float4 nsmp = make_float4(0.f, 0.f, 0.f, 0.f);
            int nbin = INT_MIN;
            if(tid < kTcChunk && lo < hi) fetch(lo, nsmp, nbin);
            for(uint32_t c0 = lo; c0 < hi; c0 += kTcChunk) {
                const int valid = (int)min((uint32_t)kTcChunk, hi - c0);
                const uint32_t st = gchunk & 1u;
                if(tid < kTcChunk) { S.smp[tid] = nsmp; S.bin[tid] = nbin; }
                // Stage st was last read by the MMAs of chunk gchunk - 2.
                if(tid == 0 && gchunk >= 2 &&
                   !mbar_wait_bounded(smem_u32(&S.bar[st]), ((gchunk >> 1) - 1) & 1u, &S.abort, kTcWaitCycles))
                    atomicOr(err, kErrGatherTimeout);
                __syncthreads();
                if(S.abort) { stop = true; break; }
                if(tid < kTcChunk && c0 + kTcChunk < hi) fetch(c0 + kTcChunk, nsmp, nbin);   // next chunk in flight
                unsigned char* sa = stages + st * kTcStageBytes;
                // A: warp w computes rows 4w .. 4w + 3 for sample k = lane.
                {
                    const int k = lane;
                    const float4 sm = S.smp[k];
                    const int bin = S.bin[k];
#pragma unroll
                    for(int q = 0; q < 4; q++) {
                        const int rr = warp * 4 + q;
                        float2 u = make_float2(0.f, 0.f);
                        if(bin >= S.elo[rr] && bin <= S.ehi[rr]) {
                            const float2 w = lerp_cplx(s_pulse, rp.range_axis, sm.z - S.R[rr]);
                            u = cmul(make_float2(sm.x, sm.y), w);
                        }
                        uint32_t h, l;
                        tf32_split(u.x, h, l);
                        *reinterpret_cast<uint32_t*>(sa + sw128_offset_b32(rr, k)) = h;
                        *reinterpret_cast<uint32_t*>(sa + kTcOpBytes + sw128_offset_b32(rr, k)) = l;
                        tf32_split(u.y, h, l);
                        *reinterpret_cast<uint32_t*>(sa + sw128_offset_b32(kTcRows + rr, k)) = h;
                        *reinterpret_cast<uint32_t*>(sa + kTcOpBytes + sw128_offset_b32(kTcRows + rr, k)) = l;
                    }
                    // B: warp w computes bearings 8w .. 8w + 7 for sample k = lane.
                    const bool live = k < valid;
#pragma unroll
                    for(int q = 0; q < 8; q++) {
                        const int n = warp * 8 + q;
                        float v = 0.0f;
                        if(live && b0 + n < nB) v = lerp_real(s_beam, rp.beam_axis, sm.w - S.theta[n]);
                        uint32_t h, l;
                        tf32_split(v, h, l);
                        *reinterpret_cast<uint32_t*>(sa + 2 * kTcOpBytes + sw128_offset_b32(n, k)) = h;
                        *reinterpret_cast<uint32_t*>(sa + 3 * kTcOpBytes + sw128_offset_b32(n, k)) = l;
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncthreads();
                if(tid == 0) {
                    tc_fence_after();
                    const uint32_t a = smem_u32(sa);
                    const uint64_t ahi = smem_desc(a), alo = smem_desc(a + kTcOpBytes);
                    const uint64_t bhi = smem_desc(a + 2 * kTcOpBytes), blo = smem_desc(a + 3 * kTcOpBytes);
#pragma unroll
                    for(int kk = 0; kk < kTcChunk / 8; kk++) {      // 32 bytes of K per MMA: +2 in descriptor units
                        umma_tf32(tmem, ahi + 2 * kk, bhi + 2 * kk, (chain > 0 || kk > 0) ? 1u : 0u);
                        umma_tf32(tmem, ahi + 2 * kk, blo + 2 * kk, 1u);
                        umma_tf32(tmem, alo + 2 * kk, bhi + 2 * kk, 1u);
                    }
                    umma_commit(smem_u32(&S.bar[st]));
                }
                nchunk++;
                gchunk++;
                if(++chain == kTcFlush) {
                    if(!flush()) { stop = true; break; }
                    chain = 0;
                }
            }
        }
        if(stop) break;
        if(nchunk == 0) continue;
        if(chain > 0 && !flush()) break;
        chain = 0;
        // Epilogue: registers -> shared (rows of kTcPitch floats) -> the ping.
        float* dsm = reinterpret_cast<float*>(stages);
        {
            const int m = quad * 32 + lane;
#pragma unroll
            for(int q = 0; q < 32; q++) dsm[m * kTcPitch + cg * 32 + q] = acc[q];
        }
        __syncthreads();
        for(int e = tid; e < kTcRows * kTcBearings; e += kTcThreads) {
            const int rr = e / kTcBearings, n = e % kTcBearings;
            const int r = r0 + rr, b = b0 + n;
            if(r < nR && b < nB)
                red_add_v2(out + (size_t)r * nB + b, make_float2(dsm[rr * kTcPitch + n], dsm[(kTcRows + rr) * kTcPitch + n]));
        }
        __syncthreads();
    }
    // Let issued MMAs finish (bounded) before the TMEM is released.
    if(tid == 0 && gchunk > 0 && S.abort) {
        volatile int keep_waiting = 0;
        mbar_wait_bounded(smem_u32(&S.bar[(gchunk - 1) & 1u]), ((gchunk - 1) >> 1) & 1u, &keep_waiting, kTcWaitCycles);
    }
    tc_fence_before();
    __syncthreads();
    if(warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
    }
}

rtacx_status launch_2d_tc(Context& ctx, float2* out, cudaStream_t stream)
{
    const size_t smem = gather_tc_smem_bytes(ctx.H, ctx.W);
    if(raise_smem_limit((const void*)k_gather_tc, smem) != cudaSuccess) {
        cudaGetLastError();
        ctx.error = "PSF tables too large for the tensor-core gather";
        return RTACX_ERR_UNSUPPORTED;
    }
    const uint32_t tiles_b = (ctx.nB + kTcBearings - 1) / kTcBearings;
    const uint32_t tiles = tiles_b * ((ctx.nR + kTcRows - 1) / kTcRows);
    k_tile_plan<kTcRows><<<1, kPlanThreads, 0, stream>>>(ctx.d_offsets, ctx.d_win, ctx.d_bb_tiles128, ctx.nR,
                                                         ctx.bin.nBB, tiles_b, tiles, (uint32_t)ctx.sm_count,
                                                         ctx.d_tile_parts, ctx.d_tile_first, ctx.d_items);
    cudaError_t me = cudaMemsetAsync(ctx.d_item_counter, 0, sizeof(uint32_t), stream);
    if(me == cudaSuccess) me = cudaMemsetAsync(out, 0, (size_t)ctx.nR * ctx.nB * sizeof(float2), stream);
    if(me != cudaSuccess) {
        cudaGetLastError();
        ctx.error = std::string("clearing the tensor-core gather's ping: ") + cudaGetErrorString(me);
        return RTACX_ERR_CUDA;
    }
    k_gather_tc<<<ctx.sm_count, kTcThreads, smem, stream>>>(
        ctx.d_sorted, ctx.d_offsets, ctx.d_win, ctx.d_bb_tiles128, ctx.d_ranges, ctx.d_bearings, ctx.d_pulse,
        ctx.d_beam, ctx.red, ctx.bin.nBB, out, ctx.d_items, ctx.d_tile_first + tiles, ctx.d_tile_parts, tiles_b,
        ctx.d_item_counter, ctx.d_err);
    const cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) { ctx.error = std::string("k_gather_tc: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    return RTACX_OK;
}

// Persistent batched gather: each CTA takes work items from a global counter
// (one atomicAdd per item, no waiting) until the list is exhausted. Items are
// 2D tiles {ping, tile_b, tile_r, 0} or 1D row groups {ping, group, 0, 1}.
template <int TR, int TB>
__global__ void __launch_bounds__(kThreads)
k_gather_batch(const PingDev* __restrict__ pings, const uint4* __restrict__ items, uint32_t n_items,
               uint32_t* __restrict__ counter)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_item;
    for(;;) {
        if(threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if(it >= n_items) break;
        const uint4 item = items[it];
        const PingDev& P = pings[item.x];
        if(item.w == 0) {
            gather_tile_2d<TR, TB>(P.sorted, P.offsets, P.win, P.bb_tiles, P.ranges, P.bearings, P.pulse, P.beam,
                                   P.red, P.bin.nBB, P.out, (int)item.y, (int)item.z, smem_raw);
        }
        else {
            float2* s_pulse = reinterpret_cast<float2*>(smem_raw);
            for(int i = threadIdx.x; i < P.red.range_axis.n + 2; i += kThreads) s_pulse[i] = P.pulse[i];
            __syncthreads();
            gather_rows_1d(P.sorted, P.offsets, P.win, P.ranges, s_pulse, P.red, P.out, (int)item.y * kWarps);
        }
        __syncthreads();
    }
}

template <int TR, int TB>
rtacx_status launch_2d(Context& ctx, float2* out, cudaStream_t stream)
{
    const size_t smem = sizeof(GatherSmem<TR, TB>) + (ctx.H + 2) * sizeof(float2) + (ctx.W + 2) * sizeof(float);
    if(raise_smem_limit((const void*)k_gather_2d<TR, TB>, smem) != cudaSuccess) {
        ctx.error = "PSF tables too large for shared memory (pulse " + std::to_string(ctx.H) +
                    " taps, beam " + std::to_string(ctx.W) + " taps)";
        return RTACX_ERR_UNSUPPORTED;
    }
    dim3 grid((ctx.nB + TB - 1) / TB, (ctx.nR + TR - 1) / TR);
    if(!ctx.d_tile_parts) {
        // One CTA per tile (contexts without split scratch).
        k_gather_2d<TR, TB><<<grid, kThreads, smem, stream>>>(ctx.d_sorted, ctx.d_offsets, ctx.d_win, ctx.d_bb_tiles,
                                                              ctx.d_ranges, ctx.d_bearings, ctx.d_pulse, ctx.d_beam,
                                                              ctx.red, ctx.bin.nBB, out);
        const cudaError_t e = cudaGetLastError();
        if(e != cudaSuccess) { ctx.error = std::string("k_gather_2d: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
        return RTACX_OK;
    }
    if(raise_smem_limit((const void*)k_gather_split<TR, TB>, smem) != cudaSuccess) {
        ctx.error = "PSF tables too large for shared memory";
        return RTACX_ERR_UNSUPPORTED;
    }
    const uint32_t tiles = grid.x * grid.y;
    int per_sm = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather_split<TR, TB>, kThreads, smem);
    per_sm = std::max(1, per_sm);
    const uint32_t workers = (uint32_t)(ctx.sm_count * per_sm);
    k_tile_plan<TR><<<1, kPlanThreads, 0, stream>>>(ctx.d_offsets, ctx.d_win, ctx.d_bb_tiles, ctx.nR, ctx.bin.nBB,
                                                    grid.x, tiles, workers, ctx.d_tile_parts, ctx.d_tile_first,
                                                    ctx.d_items);
    cudaError_t me = cudaMemsetAsync(ctx.d_item_counter, 0, sizeof(uint32_t), stream);
    if(me == cudaSuccess) me = cudaMemsetAsync(out, 0, (size_t)ctx.nR * ctx.nB * sizeof(float2), stream);
    if(me != cudaSuccess) {
        cudaGetLastError();
        ctx.error = std::string("clearing the split gather's ping: ") + cudaGetErrorString(me);
        return RTACX_ERR_CUDA;
    }
    k_gather_split<TR, TB><<<workers, kThreads, smem, stream>>>(
        ctx.d_sorted, ctx.d_offsets, ctx.d_win, ctx.d_bb_tiles, ctx.d_ranges, ctx.d_bearings, ctx.d_pulse,
        ctx.d_beam, ctx.red, ctx.bin.nBB, out, ctx.d_items, ctx.d_tile_first + tiles, ctx.d_tile_parts, grid.x,
        ctx.d_item_counter);
    const cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) { ctx.error = std::string("k_gather_split: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    return RTACX_OK;
}

// ---- fused batched form -----------------------------------------------------

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier of the cooperative launch (every CTA is resident). Thread 0
// of each CTA publishes the CTA's writes (fence), arrives, and waits for the
// generation to move; the last arrival resets the count and advances the
// generation. The wait is bounded by fb.wait_ns of the global timer: a CTA
// that gives up sets kErrBatchWaitTimeout in the batch status word and the
// whole CTA returns false. A barrier passed by any CTA had every arrival, so
// the data of the phase before it is complete; a CTA that gave up does no
// further work, so no later barrier completes and every CTA stops at it.
__device__ __forceinline__ bool grid_barrier(const FusedBatch& fb, int* s_ok)
{
    __syncthreads();
    if(threadIdx.x == 0) {
        int ok = 1;
        const uint32_t gen = ld_acquire_gpu(&fb.sync->generation);
        __threadfence();
        if(atomicAdd(&fb.sync->arrived, 1u) + 1u == fb.arrivals) {
            atomicExch(&fb.sync->arrived, 0u);
            __threadfence();
            atomicAdd(&fb.sync->generation, 1u);
        }
        else {
            const unsigned long long t0 = global_ns();
            while(ld_acquire_gpu(&fb.sync->generation) == gen) {
                if(global_ns() - t0 > fb.wait_ns) {
                    atomicOr(fb.status, kErrBatchWaitTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(200);
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// Next item of a dynamically scheduled phase (one atomicAdd per item, no
// waiting); the leading barrier frees the shared memory of the last item.
__device__ __forceinline__ uint32_t claim(uint32_t* counter, uint32_t* s_item)
{
    __syncthreads();
    if(threadIdx.x == 0) *s_item = atomicAdd(counter, 1u);
    __syncthreads();
    return *s_item;
}

// The whole batched plain form in one cooperative persistent launch:
//   phase 0  zero every ping's bin totals and out-of-range counts
//   phase 1  count chunks (a global atomic per sample)       dynamic queue
//   phase 2  bin-scan blocks of kScanBlock bins              dynamic queue
//   phase 3  reference windows (static), scatter chunks      dynamic queue
//            (a global cursor atomic per sample)
//   phase 4  gather items, heaviest first                    dynamic queue
// separated by bounded grid barriers. The binning phases use no shared
// histogram, so the dynamic shared memory is the gather's and as many CTAs
// per SM stay resident as for a gather alone.
template <int TR, int TB>
__global__ void __launch_bounds__(kThreads) k_batch_fused(const FusedBatch fb)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned long long s_oor[2];
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_prefix, s_item;
    __shared__ int s_ok;

    for(uint32_t k = blockIdx.x; k < fb.n_col; k += gridDim.x) {
        const uint2 m = fb.col_map[k];
        const PingDev& P = fb.pings[m.x];
        const uint32_t b = m.y * kThreads + threadIdx.x;
        if(b < P.bin.nBins) P.totals[b] = 0u;
        if(b < (P.bin.nBins + kScanBlock - 1) / kScanBlock) P.totals[P.bin.nBins + b] = 0u;
        if(m.y == 0 && threadIdx.x < 2) P.oor[threadIdx.x] = 0ull;
    }
    if(!grid_barrier(fb, &s_ok)) return;

    for(;;) {
        const uint32_t k = claim(&fb.sync->next[0], &s_item);
        if(k >= fb.n_chunks) break;
        const uint2 m = fb.chunk_map[k];
        const PingDev& P = fb.pings[m.x];
        count_chunk_global(P.samples, P.n, P.bin, m.y, P.chunks, P.totals, P.oor, s_oor);
    }
    if(!grid_barrier(fb, &s_ok)) return;

    for(;;) {
        const uint32_t k = claim(&fb.sync->next[1], &s_item);
        if(k >= fb.n_scan) break;
        const uint2 m = fb.scan_map[k];
        const PingDev& P = fb.pings[m.x];
        scan_bin_block(P.totals, P.bin.nBins, m.y, P.offsets, P.hist, s_warp, &s_prefix, false);   // hist = cursors
    }
    if(!grid_barrier(fb, &s_ok)) return;

    for(uint32_t k = blockIdx.x; k < fb.n_win; k += gridDim.x) {
        const uint2 m = fb.win_map[k];
        const PingDev& P = fb.pings[m.x];
        window_row(P.offsets, P.bin.nBB, P.nR, P.overlap, P.support, P.win, (int)(m.y * kThreads + threadIdx.x));
    }
    for(;;) {
        const uint32_t k = claim(&fb.sync->next[2], &s_item);
        if(k >= fb.n_chunks) break;
        const uint2 m = fb.chunk_map[k];
        const PingDev& P = fb.pings[m.x];
        scatter_chunk_global(P.samples, P.n, P.bin, m.y, P.chunks, P.hist, P.offsets, P.sorted, P.err);
    }
    if(!grid_barrier(fb, &s_ok)) return;

    for(;;) {
        const uint32_t it = claim(&fb.sync->next[3], &s_item);
        if(it >= fb.n_items) break;
        const uint4 item = fb.items[it];
        const PingDev& P = fb.pings[item.x];
        if(item.w == 0) {
            gather_tile_2d<TR, TB>(P.sorted, P.offsets, P.win, P.bb_tiles, P.ranges, P.bearings, P.pulse, P.beam,
                                   P.red, P.bin.nBB, P.out, (int)item.y, (int)item.z, smem_raw);
        }
        else {
            float2* s_pulse = reinterpret_cast<float2*>(smem_raw);
            for(int i = threadIdx.x; i < P.red.range_axis.n + 2; i += kThreads) s_pulse[i] = P.pulse[i];
            __syncthreads();
            gather_rows_1d(P.sorted, P.offsets, P.win, P.ranges, s_pulse, P.red, P.out, (int)item.y * kWarps);
        }
    }
}

template <int TR, int TB>
rtacx_status prepare_fused_shape(std::string& error, size_t smem, int sm_count, uint32_t& grid)
{
    if(raise_smem_limit((const void*)k_batch_fused<TR, TB>, smem) != cudaSuccess) {
        cudaGetLastError();
        error = "shared memory of the fused batched kernel (" + std::to_string(smem) + " B) not available";
        return RTACX_ERR_UNSUPPORTED;
    }
    int per_sm = 0;
    if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_fused<TR, TB>, kThreads, smem) != cudaSuccess ||
       per_sm < 1) {
        cudaGetLastError();
        error = "the fused batched kernel does not fit on an SM";
        return RTACX_ERR_UNSUPPORTED;
    }
    grid = (uint32_t)sm_count * (uint32_t)per_sm;
    return RTACX_OK;
}

template <int TR, int TB>
rtacx_status launch_fused_shape(std::string& error, const FusedBatch& fb, size_t smem, uint32_t grid,
                                cudaStream_t stream)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_batch_fused<TR, TB>, fb);
    if(e != cudaSuccess) {
        cudaGetLastError();
        error = std::string("k_batch_fused: ") + cudaGetErrorString(e);
        return RTACX_ERR_CUDA;
    }
    return RTACX_OK;
}

} // namespace

rtacx_status prepare_fused_batch(std::string& error, int shape, size_t smem, int sm_count, uint32_t& grid)
{
    if(shape == 2) return prepare_fused_shape<32, 128>(error, smem, sm_count, grid);
    if(shape == 1) return prepare_fused_shape<16, 128>(error, smem, sm_count, grid);
    return prepare_fused_shape<16, 64>(error, smem, sm_count, grid);
}

rtacx_status launch_fused_batch(std::string& error, int shape, const FusedBatch& fb, size_t smem, uint32_t grid,
                                cudaStream_t stream)
{
    if(shape == 2) return launch_fused_shape<32, 128>(error, fb, smem, grid, stream);
    if(shape == 1) return launch_fused_shape<16, 128>(error, fb, smem, grid, stream);
    return launch_fused_shape<16, 64>(error, fb, smem, grid, stream);
}

// Batched gather tile shapes: 0 = 16 x 64, 1 = 16 x 128, 2 = 32 x 128.
int gather_shape_rows(int shape) { return shape == 2 ? 32 : 16; }
int gather_shape_bearings(int shape) { return shape == 0 ? 64 : 128; }

size_t gather_batch_smem(int shape, uint32_t H, uint32_t W)
{
    const size_t base = shape == 2 ? sizeof(GatherSmem<32, 128>)
                      : shape == 1 ? sizeof(GatherSmem<16, 128>) : sizeof(GatherSmem<16, 64>);
    return base + (H + 2) * sizeof(float2) + (W + 2) * sizeof(float);
}

template <int TR, int TB>
rtacx_status prepare_batch_shape(std::string& error, size_t smem)
{
    if(raise_smem_limit((const void*)k_gather_batch<TR, TB>, smem) != cudaSuccess) {
        error = "PSF tables too large for the batched gather";
        return RTACX_ERR_UNSUPPORTED;
    }
    return RTACX_OK;
}

template <int TR, int TB>
rtacx_status launch_batch_shape(std::string& error, const PingDev* pings, const uint4* items, uint32_t n_items,
                                uint32_t* counter, size_t smem, uint32_t grid, cudaStream_t stream)
{
    k_gather_batch<TR, TB><<<grid, kThreads, smem, stream>>>(pings, items, n_items, counter);
    const cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) { error = std::string("k_gather_batch: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    return RTACX_OK;
}

rtacx_status prepare_gather_batch(std::string& error, int shape, size_t smem)
{
    if(shape == 2) return prepare_batch_shape<32, 128>(error, smem);
    if(shape == 1) return prepare_batch_shape<16, 128>(error, smem);
    return prepare_batch_shape<16, 64>(error, smem);
}

rtacx_status launch_gather_batch(std::string& error, int shape, const PingDev* pings, const uint4* items,
                                 uint32_t n_items, uint32_t* counter, size_t smem, uint32_t grid, cudaStream_t stream)
{
    if(shape == 2) return launch_batch_shape<32, 128>(error, pings, items, n_items, counter, smem, grid, stream);
    if(shape == 1) return launch_batch_shape<16, 128>(error, pings, items, n_items, counter, smem, grid, stream);
    return launch_batch_shape<16, 64>(error, pings, items, n_items, counter, smem, grid, stream);
}

size_t gather_smem_bytes(uint32_t range_tile, uint32_t bearing_tile, uint32_t H, uint32_t W)
{
    size_t base = range_tile == 32 ? sizeof(GatherSmem<32, 128>)
                : bearing_tile == 128 ? sizeof(GatherSmem<16, 128>) : sizeof(GatherSmem<16, 64>);
    return base + (H + 2) * sizeof(float2) + (W + 2) * sizeof(float);
}

rtacx_status run_reduce(Context& ctx, float* out_f, cudaStream_t stream)
{
    float2* out = reinterpret_cast<float2*>(out_f);
    if(ctx.dims == 1 && ctx.psf_tex) {
        k_gather_tex_1d<<<(ctx.nR + kWarps - 1) / kWarps, kThreads, 0, stream>>>(
            ctx.d_sorted, ctx.d_offsets, ctx.d_win, ctx.d_ranges, ctx.psf_tex, ctx.tex_yscale, ctx.nR, out);
        const cudaError_t e = cudaGetLastError();
        if(e != cudaSuccess) { ctx.error = std::string("k_gather_tex_1d: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
        return RTACX_OK;
    }
    if(ctx.dims == 1) {
        const size_t smem = (ctx.H + 2) * sizeof(float2);
        if(smem > 48 * 1024) raise_smem_limit((const void*)k_gather_1d, smem);
        k_gather_1d<<<(ctx.nR + kWarps - 1) / kWarps, kThreads, smem, stream>>>(
            ctx.d_sorted, ctx.d_offsets, ctx.d_win, ctx.d_ranges, ctx.d_pulse, ctx.red, out);
        const cudaError_t e = cudaGetLastError();
        if(e != cudaSuccess) { ctx.error = std::string("k_gather_1d: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
        return RTACX_OK;
    }
    if(ctx.psf_tex) {
        const uint64_t warps = (uint64_t)ctx.nR * ctx.nB;
        k_gather_tex<<<(uint32_t)((warps + kWarps - 1) / kWarps), kThreads, 0, stream>>>(
            ctx.d_sorted, ctx.d_offsets, ctx.d_win, ctx.d_ranges, ctx.d_bearings, ctx.psf_tex, ctx.tex_xscale,
            ctx.tex_yscale, ctx.nR, ctx.nB, out);
        const cudaError_t e = cudaGetLastError();
        if(e != cudaSuccess) { ctx.error = std::string("k_gather_tex: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
        return RTACX_OK;
    }
    if(!(ctx.flags & RTACX_FLAG_SIMT_GATHER) && ctx.d_tile_parts) return launch_2d_tc(ctx, out, stream);
    if(ctx.range_tile == 32) return launch_2d<32, 128>(ctx, out, stream);
    if(ctx.bearing_tile == 128) return launch_2d<16, 128>(ctx, out, stream);
    return launch_2d<16, 64>(ctx, out, stream);
}

} // namespace rtacx
