// Precision (tensor-core) form: bin first, contract over bearings on the
// tensor cores, filter in range.
//
//   k_prec_clear       zeroes the pair cells and the non-empty bitmap.
//   k_prec_accumulate  one pass over the samples (read once, 16 B each):
//   (_staged)          range key (Binner::Key, bit-exact), optional FP64
//                      echo pre-step, linear split between the two table
//                      bearings around the sample bearing, one 16-byte vector
//                      float atomic (red.global.add.v4.f32) into the pair
//                      cell P[j][k]; non-empty range bins in a bitmap. No sort.
//   k_prec_filter      row r's window by the reference rule
//                      (src/Binner.cu:90-102) on the non-empty bitmap, then
//                      G'[r][k] = sum_t taps[t] G[r + t - c][k] over that
//                      window, written as the bf16 A operand [hi | hi | lo]
//                      of the three-term split product.
//   gemm_tn            out = A x B^T on tcgen05 (rtacx_umma.cu), B the
//                      [hi | lo | hi] split of the complex directivity laid
//                      out so that output column 2b is Re(out(r, b)) and
//                      2b + 1 is Im(out(r, b)): the GEMM writes the
//                      complex64 ping directly.
// FP16 form (RTACX_PRECISION_FP16_ROWSCALE): the filter writes the fp32
// filtered grid and per-row maxima, k_prec_split_f16 scales each row by a
// power of two and writes the fp16 split, and the GEMM (fp16 operands)
// undoes the row and column scales in its epilogue.
#include "rtacx_internal.cuh"

#include <cuda_fp16.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

namespace rtacx {

namespace {

constexpr int kMaxBearingsSmem = 2048;

__device__ __forceinline__ void red_add_v4(float4* addr, float4 v)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

// The same reduction without the "memory" clobber: the pair cells are not
// read by the kernels that issue it, so loads may be scheduled across it.
__device__ __forceinline__ void red_add_v4_unordered(float4* addr, float4 v)
{
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w));
}

// Pair cells: P[j][k] = {contribution to bearing k, contribution to bearing
// k + 1} of the samples of range bin j whose bearing lies in [theta_k,
// theta_k+1). One 16-byte vector atomic per sample; the filter kernel forms
// G[j][k] = P[j][k].xy + P[j][k - 1].zw. Non-empty range bins are collected
// in a shared-memory bitmap per CTA and OR-ed into the global bitmap once.
// The bearing cell k is the largest k in [0, nB - 2] with theta_k <= theta,
// i.e. the number of interior table bearings theta_1 .. theta_nB-2 at or
// below theta. It comes from a uniform lookup grid over the table: grid cell
// c(theta) = (int)clamp((theta - origin) * scale, 0, cells - 1) in float, the
// same expression on the host and the device. c is non-decreasing in theta,
// so an interior bearing whose own grid cell lies below c(theta) is below
// theta and one whose cell lies above is above it. Grid entry c holds {the
// count of interior bearings in cells below c, the interior bearing in cell
// c or +inf}; when no cell holds two interior bearings (checked on the host:
// the lookup is then exact), k = count + (theta >= bearing) with no search.
// Otherwise the count is corrected by comparisons with the table.
// Shared memory (dynamic, sized by nB and nR): per table bearing an 8-byte
// cell {theta_k, 1 / (theta_k+1 - theta_k)}; the bitmap; the grid as 8-byte
// entries. Two 8-byte shared loads per sample in the exact case.
constexpr int kMaxRangeWords = 8192 / 32 * 4;   // bitmap words for up to 32768 range bins
constexpr int kLutCells = 4096;
constexpr int kAccThreads = 256;
// Hot range interval (RTACX_PRECISION_HOT_RANGE): kHotRows consecutive range
// rows whose pair cells are replicated kHotReplicas times; samples in them
// reduce into the replica of their warp, and k_hot_fold adds the replicas
// back into the grid before the range filter.
constexpr int kHotRows = 256, kHotReplicas = 8;
constexpr int kAccLoads = 4;                     // independent record loads per thread in flight
constexpr int kAccEchoModels = 6;                // echo models of k_prec_accumulate_exact

// Lookup-grid cell of a bearing; one expression for the host (building the
// grid) and the device (reading it), so both agree on every float input.
// NaN bearings fall in cell 0.
__host__ __device__ __forceinline__ int bearing_grid_cell(float th, float origin, float scale, uint32_t cells)
{
    return (int)fminf(fmaxf((th - origin) * scale, 0.0f), (float)(cells - 1));
}

size_t accumulate_smem_bytes(uint32_t nB, uint32_t nR, uint32_t lut_cells)
{
    return (size_t)nB * sizeof(float2) + (size_t)lut_cells * sizeof(float2) + (size_t)((nR + 31) / 32) * sizeof(uint32_t);
}

__global__ void __launch_bounds__(kAccThreads)
k_prec_accumulate(const float* __restrict__ samples, uint64_t n, BinParams p,
                  const float* __restrict__ bearings, uint32_t nB, const float2* __restrict__ lut,
                  uint32_t lut_cells, float lut_origin, float lut_scale, int lut_exact,
                  float4* __restrict__ P, uint32_t* __restrict__ nonempty, const int2* __restrict__ hot,
                  float4* __restrict__ rep)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    float2* s_cell = reinterpret_cast<float2*>(s_raw);
    int hot_lo = 0, hot_len = 0;
    if(hot) { const int2 h = *hot; hot_lo = h.x; hot_len = h.y; }
    const uint32_t rsel = (blockIdx.x + (threadIdx.x >> 5)) & (kHotReplicas - 1);   // by CTA and warp
    // Pair-cell row of range bin j: the grid's, or this warp's replica of a hot row.
    auto cell_row = [&](uint32_t j) -> float4* {
        const uint32_t hj = j - (uint32_t)hot_lo;
        return hj < (uint32_t)hot_len ? rep + ((size_t)hj * kHotReplicas + rsel) * nB : P + (size_t)j * nB;
    };
    const uint32_t words = (p.key.nR + 31) / 32;
    float2* s_lut = s_cell + nB;
    uint32_t* s_bits = reinterpret_cast<uint32_t*>(s_lut + lut_cells);
    for(uint32_t i = threadIdx.x; i < nB; i += blockDim.x) {
        const float th = bearings[i];
        s_cell[i] = make_float2(th, i + 1 >= nB ? 0.0f : 1.0f / (bearings[i + 1] - th));
    }
    for(uint32_t i = threadIdx.x; i < lut_cells; i += blockDim.x) s_lut[i] = lut[i];
    for(uint32_t i = threadIdx.x; i < words; i += blockDim.x) s_bits[i] = 0u;
    __syncthreads();
    const int kmax = (int)nB - 2;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for(uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < n; i0 += stride * kAccLoads) {
        float4 rec[kAccLoads];
#pragma unroll
        for(int u = 0; u < kAccLoads; u++) {
            const uint64_t i = i0 + (uint64_t)u * stride;
            rec[u] = i < n ? load_record(samples, i, p) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for(int u = 0; u < kAccLoads; u++) {
            if(i0 + (uint64_t)u * stride >= n) continue;
            int side;
            const uint32_t j = range_key(p.key, rec[u].z, side);
            if(j == kOutOfRange) continue;
            const float2 v = apply_echo(p, make_float2(rec[u].x, rec[u].y), rec[u].z);
            atomicOr(&s_bits[j >> 5], 1u << (j & 31));
            if(nB == 1) { red_add_v4(cell_row(j), make_float4(v.x, v.y, 0.f, 0.f)); continue; }
            const float th = rec[u].w;
            const float2 e = s_lut[bearing_grid_cell(th, lut_origin, lut_scale, lut_cells)];
            int k = __float_as_int(e.x);
            if(lut_exact) k += (th >= e.y) ? 1 : 0;
            else {
                while(k < kmax && s_cell[k + 1].x <= th) ++k;
                while(k > 0 && !(s_cell[k].x <= th)) --k;
            }
            const float2 c = s_cell[k];
            float w = (th - c.x) * c.y;
            w = fminf(fmaxf(w, 0.0f), 1.0f);          // NaN bearings -> 0
            const float w0 = 1.0f - w;
            red_add_v4(cell_row(j) + k, make_float4(w0 * v.x, w0 * v.y, w * v.x, w * v.y));
        }
    }
    __syncthreads();
    for(uint32_t i = threadIdx.x; i < words; i += blockDim.x)
        if(s_bits[i]) atomicOr(&nonempty[i], s_bits[i]);
}

// k_prec_accumulate for the common case: 16-byte aligned records, an exact
// bearing lookup grid, more than one bearing, no hot range, and the echo
// model kEcho fixed at compile time. The records reach shared memory by bulk
// copies (cp.async.bulk, the TMA engine) into a ring of kStages stages of
// kStageRecs records, so the bytes in flight per SM depend neither on
// registers nor on how long the threads compute. Each thread computes the
// key, value, cell and weights of its records of a stage without branches
// (out-of-range and tail records only clear their predicate), then issues
// the bitmap bits and the vector reductions; the results are those of
// k_prec_accumulate. The bearing lookup is one 16-byte grid entry per sample
// (no cell table): the weight's reciprocal 1 / (theta_k+1 - theta_k) is
// computed per sample with the correctly rounded __frcp_rn, the same value
// as the general kernel's table entry 1.0f / (theta_k+1 - theta_k). One persistent CTA
// takes stages c = blockIdx.x, blockIdx.x + gridDim.x, ...; thread 0 issues
// the copy of the stage kStages ahead as soon as every thread has read the
// stage it refills. Each wait is bounded (kAccWaitCycles); a timeout sets
// kErrAccumulateTimeout in the error word, the CTA stops, and thread 0 waits
// (bounded again) for its copies still in flight before the CTA exits.
constexpr int kStageRecs = 1024;                 // 16 KB of records per stage
constexpr int kStages = 4;
constexpr int kStagedThreads = 512;
constexpr int kStagedPerThread = kStageRecs / kStagedThreads;
constexpr long long kAccWaitCycles = 2000000000ll;   // about one second

size_t staged_smem_bytes(uint32_t nB, uint32_t nR, uint32_t lut_cells)
{
    return (size_t)kStages * kStageRecs * sizeof(float4) + (size_t)lut_cells * sizeof(float4) +
           (size_t)((nR + 31) / 32) * sizeof(uint32_t);
}

template <uint32_t kEcho>
__global__ void __launch_bounds__(kStagedThreads)
k_prec_accumulate_staged(const float4* __restrict__ samples, uint64_t n, BinParams p,
                         const float* __restrict__ bearings, uint32_t nB, const float2* __restrict__ lut,
                         uint32_t lut_cells, float lut_origin, float lut_scale,
                         float4* __restrict__ P, uint32_t* __restrict__ nonempty, uint32_t* __restrict__ err,
                         uint32_t drop_stage)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ __align__(8) uint64_t s_full[kStages];
    __shared__ int s_abort;
    float4* s_ring = reinterpret_cast<float4*>(s_raw);
    float4* s_lut = s_ring + kStages * kStageRecs;
    uint32_t* s_bits = reinterpret_cast<uint32_t*>(s_lut + lut_cells);
    const uint32_t words = (p.key.nR + 31) / 32;
    const uint64_t stages = (n + kStageRecs - 1) / kStageRecs;
    auto issue = [&](uint64_t c, int slot) {
        if(c == drop_stage) return;      // failure-path test: this stage's copy never comes
        const uint64_t first = c * kStageRecs;
        const uint64_t left = n - first;
        const uint32_t bytes = (uint32_t)(left < (uint64_t)kStageRecs ? left : (uint64_t)kStageRecs) * (uint32_t)sizeof(float4);
        const uint32_t bar = smem_u32(&s_full[slot]);
        mbar_expect_tx(bar, bytes);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(smem_u32(s_ring + slot * kStageRecs)), "l"(samples + first), "r"(bytes), "r"(bar)
                     : "memory");
    };
    if(threadIdx.x == 0) {
        for(int i = 0; i < kStages; i++) mbar_init(smem_u32(&s_full[i]), 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for(int i = 0; i < kStages; i++) {
            const uint64_t c = blockIdx.x + (uint64_t)i * gridDim.x;
            if(c < stages) issue(c, i);
        }
    }
    // Grid entry c: {count k_lo, the interior bearing theta_b in the cell or
    // +inf, theta_k_lo, the next bearing the weight needs: theta_k_lo+2 when
    // theta_b is finite (samples at or above it take k_lo + 1), else
    // theta_k_lo+1}.
    for(uint32_t i = threadIdx.x; i < lut_cells; i += blockDim.x) {
        const float2 e = lut[i];
        const int k = __float_as_int(e.x);
        const bool has_b = e.y != INFINITY;
        s_lut[i] = make_float4(e.x, e.y, bearings[k], bearings[has_b ? k + 2 : k + 1]);
    }
    for(uint32_t i = threadIdx.x; i < words; i += blockDim.x) s_bits[i] = 0u;
    __syncthreads();
    int it = 0;
    bool aborted = false;
    for(uint64_t c = blockIdx.x; c < stages; c += gridDim.x, it++) {
        const int slot = it % kStages;
        const bool ready = mbar_wait_bounded(smem_u32(&s_full[slot]), (uint32_t)(it / kStages) & 1u, &s_abort,
                                             kAccWaitCycles);
        const uint64_t left = n - c * kStageRecs;
        const uint32_t count = left < (uint64_t)kStageRecs ? (uint32_t)left : (uint32_t)kStageRecs;
        uint32_t row[kStagedPerThread];
        int cell[kStagedPerThread];
        float4 add[kStagedPerThread];
#pragma unroll
        for(int u = 0; u < kStagedPerThread; u++) {
            const uint32_t idx = threadIdx.x + (uint32_t)u * kStagedThreads;
            const float4 rec = s_ring[slot * kStageRecs + min(idx, (uint32_t)kStageRecs - 1u)];
            const uint32_t j = range_key_select(p.key, rec.z);
            row[u] = (ready && idx < count) ? j : kOutOfRange;
            const float2 v = apply_echo(p, make_float2(rec.x, rec.y), rec.z, kEcho);
            const float th = rec.w;
            const float4 e = s_lut[bearing_grid_cell(th, lut_origin, lut_scale, lut_cells)];
            const bool up = th >= e.y;
            const int k = __float_as_int(e.x) + (up ? 1 : 0);
            const float tk = up ? e.y : e.z;
            const float tk1 = (up || e.y == INFINITY) ? e.w : e.y;
            const float w = fminf(fmaxf((th - tk) * __frcp_rn(tk1 - tk), 0.0f), 1.0f);   // NaN bearings -> 0
            const float w0 = 1.0f - w;
            cell[u] = k;
            add[u] = make_float4(w0 * v.x, w0 * v.y, w * v.x, w * v.y);
        }
        // Every thread has read the slot: refill it kStages stages ahead.
        aborted = __syncthreads_or(!ready) != 0;
        if(threadIdx.x == 0 && !aborted) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const uint64_t next = c + (uint64_t)kStages * gridDim.x;
            if(next < stages) issue(next, slot);
        }
#pragma unroll
        for(int u = 0; u < kStagedPerThread; u++) {
            const uint32_t j = row[u];
            if(j != kOutOfRange) {
                atomicOr(&s_bits[j >> 5], 1u << (j & 31));
                red_add_v4_unordered(P + (size_t)j * nB + cell[u], add[u]);
            }
        }
        if(aborted) break;
    }
    if(aborted && threadIdx.x == 0) {
        atomicOr(err, kErrAccumulateTimeout);
        // Let the copies still in flight land before the CTA's shared memory
        // is released: those of iterations it .. it + kStages - 1 (the refill
        // of the aborted iteration was not issued).
        // Each wait is bounded on its own; a copy that was never issued (or
        // never lands) costs one more timeout.
        for(int i = it; i < it + kStages; i++) {
            if(blockIdx.x + (uint64_t)i * gridDim.x >= stages) break;
            volatile int keep_waiting = 0;
            mbar_wait_bounded(smem_u32(&s_full[i % kStages]), (uint32_t)(i / kStages) & 1u, &keep_waiting,
                              kAccWaitCycles);
        }
    }
    __syncthreads();
    for(uint32_t i = threadIdx.x; i < words; i += blockDim.x)
        if(s_bits[i]) atomicOr(&nonempty[i], s_bits[i]);
}

// Echo models of the specialised accumulation (RTACX_ECHO_PHASE_COMPENSATED
// only matters with RTACX_ECHO_PHASE).
constexpr uint32_t kEchoP = RTACX_ECHO_PHASE, kEchoS = RTACX_ECHO_SPREADING, kEchoC = RTACX_ECHO_PHASE_COMPENSATED;
constexpr uint32_t kEchoModels[kAccEchoModels] = {0u, kEchoP, kEchoS, kEchoP | kEchoS, kEchoP | kEchoC,
                                                 kEchoP | kEchoS | kEchoC};

const void* accumulate_staged_kernel(int model)
{
    switch(model) {
    case 0: return (const void*)k_prec_accumulate_staged<0u>;
    case 1: return (const void*)k_prec_accumulate_staged<kEchoP>;
    case 2: return (const void*)k_prec_accumulate_staged<kEchoS>;
    case 3: return (const void*)k_prec_accumulate_staged<kEchoP | kEchoS>;
    case 4: return (const void*)k_prec_accumulate_staged<kEchoP | kEchoC>;
    default: return (const void*)k_prec_accumulate_staged<kEchoP | kEchoS | kEchoC>;
    }
}

// Index into kEchoModels of an echo flag word.
int accumulate_echo_model(uint32_t flags)
{
    flags &= kEchoP | kEchoS | kEchoC;
    if(!(flags & kEchoP)) flags &= ~kEchoC;
    for(int m = 0; m < kAccEchoModels; m++)
        if(kEchoModels[m] == flags) return m;
    return 0;
}

// Zeroes the pair cells (16-byte stores, grid-stride) and the non-empty
// bitmap of a new ping in one launch.
__global__ void k_prec_clear(float4* __restrict__ P, uint64_t cells, uint32_t* __restrict__ bits, uint32_t words)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for(uint64_t i = i0; i < cells; i += stride) P[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for(uint64_t i = i0; i < words; i += stride) bits[i] = 0u;
}

// Hot-range detection (RTACX_PRECISION_HOT_RANGE): range-bin counts of a
// strided subsample of the ping, then one CTA picks the kHotRows-row window
// with the largest count. The window is hot when it holds at least a tenth of
// the counted samples and four times its uniform share; otherwise its length
// is 0 and every sample reduces into the grid. The counts are zeroed for the
// next ping.
__global__ void k_hot_count(const float* __restrict__ samples, uint64_t n, BinParams p, uint64_t step,
                            uint32_t* __restrict__ cnt)
{
    const uint64_t m = (n + step - 1) / step;
    for(uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < m; s += (uint64_t)gridDim.x * blockDim.x) {
        const float4 rec = load_record(samples, s * step, p);
        int side;
        const uint32_t j = range_key(p.key, rec.z, side);
        if(j != kOutOfRange) atomicAdd(&cnt[j], 1u);
    }
}

constexpr int kHotPickThreads = 1024;

// Exclusive block scan of one value per thread (blockDim.x a multiple of 32).
__device__ __forceinline__ uint32_t block_exclusive_scan_hot(uint32_t v, uint32_t* s_warp, uint32_t& total)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for(int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if(lane >= (unsigned)o) x += y;
    }
    if(lane == 31) s_warp[warp] = x;
    __syncthreads();
    const unsigned nw = blockDim.x >> 5;
    if(warp == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
        for(int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if(lane >= (unsigned)o) w += y;
        }
        if(lane < nw) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[nw - 1];
    const uint32_t before = warp ? s_warp[warp - 1] : 0u;
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kHotPickThreads) k_hot_pick(uint32_t* __restrict__ cnt, uint32_t nR,
                                                               int2* __restrict__ hot)
{
    extern __shared__ uint32_t s_pre[];           // [nR + 1] inclusive prefix: s_pre[j + 1] = sum cnt[0..j]
    __shared__ unsigned long long s_best;
    const uint32_t per = (nR + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = min(threadIdx.x * per, nR), b1 = min(b0 + per, nR);
    uint32_t sum = 0;
    for(uint32_t b = b0; b < b1; b++) sum += cnt[b];
    __shared__ uint32_t s_warp[32];
    uint32_t total;
    uint32_t run = block_exclusive_scan_hot(sum, s_warp, total);
    if(threadIdx.x == 0) { s_pre[0] = 0; s_best = 0ull; }
    for(uint32_t b = b0; b < b1; b++) { run += cnt[b]; s_pre[b + 1] = run; cnt[b] = 0u; }
    __syncthreads();
    const uint32_t H = min((uint32_t)kHotRows, nR);
    unsigned long long best = 0ull;   // (window count << 32) | (0xFFFFFFFF - start): ties go to the lowest start
    for(uint32_t s = threadIdx.x; s + H <= nR; s += blockDim.x) {
        const uint32_t w = s_pre[s + H] - s_pre[s];
        const unsigned long long key = ((unsigned long long)w << 32) | (0xFFFFFFFFu - s);
        best = key > best ? key : best;
    }
    atomicMax(&s_best, best);
    __syncthreads();
    if(threadIdx.x == 0) {
        const uint32_t w = (uint32_t)(s_best >> 32), s = 0xFFFFFFFFu - (uint32_t)(s_best & 0xFFFFFFFFu);
        const bool dense = nR > 2u * H && (double)w >= 0.1 * total && (double)w * nR >= 4.0 * H * (double)total;
        *hot = dense && total > 0 ? make_int2((int)s, (int)H) : make_int2(0, 0);
    }
}

// Adds the replicas of the hot rows into the grid once every sample is in
// (nothing when the interval is empty).
__global__ void k_hot_fold(const int2* __restrict__ hot, uint32_t nB, const float4* __restrict__ rep,
                           float4* __restrict__ P)
{
    const int2 h = *hot;
    const uint64_t cells = (uint64_t)h.y * nB;
    for(uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cells; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t row = i / nB, k = i % nB;
        const float4* rb = rep + row * kHotReplicas * nB + k;
        float4 acc = P[((uint64_t)h.x + row) * nB + k];
        for(int r = 0; r < kHotReplicas; r++) {
            const float4 e = rb[(uint64_t)r * nB];
            acc.x += e.x; acc.y += e.y; acc.z += e.z; acc.w += e.w;
        }
        P[((uint64_t)h.x + row) * nB + k] = acc;
    }
}

// Zeroes the replicas of the hot rows (nothing when the interval is empty).
__global__ void k_hot_zero(const int2* __restrict__ hot, uint32_t nB, float4* __restrict__ rep)
{
    const uint64_t cells = (uint64_t)hot->y * kHotReplicas * nB;
    for(uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cells; i += (uint64_t)gridDim.x * blockDim.x)
        rep[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ bool bit_set(const uint32_t* bits, long long j)
{
    return (bits[j >> 5] >> (j & 31)) & 1u;
}

// Window of range row r by the reference rule (src/Binner.cu:90-102) on the
// non-empty bitmap: [max(0, r - ov), min(nR - 1, r + ov)] shrunk to its first
// and last non-empty bins; {1, 0} (empty) when fewer than two are non-empty.
__device__ __noinline__ int2 row_window(const uint32_t* __restrict__ nonempty, uint32_t nR, int ov, int r)
{
    const int lo = max(0, r - ov);
    const int hi = (int)min((long long)nR - 1, (long long)r + ov);
    int a = lo;
    while(a <= hi && !bit_set(nonempty, a)) a++;
    if(a >= hi) return make_int2(1, 0);
    int z = hi;
    while(z > a && !bit_set(nonempty, z)) z--;
    return a < z ? make_int2(a, z) : make_int2(1, 0);
}

// Round-to-nearest-even fp32 -> bf16 (bit pattern).
__device__ __forceinline__ uint16_t bf16_bits(float x)
{
    uint32_t u = __float_as_uint(x);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

__device__ __forceinline__ float bf16_value(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

constexpr int kFiltRows = 64, kFiltCols = 64, kFiltTapsMax = 64, kFiltThreads = 256;

size_t filter_smem_bytes(uint32_t ntaps)
{
    const size_t nt = std::min<uint32_t>(std::max<uint32_t>(ntaps, 1u), (uint32_t)kFiltTapsMax);
    return (kFiltRows + nt - 1) * kFiltCols * sizeof(float2) + kFiltTapsMax * sizeof(float2) + kFiltRows * sizeof(int2);
}

// Range filter + split. One CTA per 64 rows x 64 bearings. Per chunk of up
// to 64 taps, the binned grid rows the chunk needs are staged in shared
// memory once: each warp reads a row's pair cells with one 16-byte load per
// cell and forms G[j][k] = P[j][k].xy + P[j][k - 1].zw with the neighbour
// lane's cell (lane 0 loads its left neighbour). Each thread then filters 8
// rows x 2 adjacent bearings and writes the bf16 A operand [hi | hi | lo],
// two bearings per 4-byte store.
// kF32Out: write the filtered grid as fp32 complex (Gf [nR][nB]) and each
// row's largest |component| (rowmax, float bits, atomicMax) for the FP16
// per-row-scaled split instead of the bf16 A operand.
template <bool kF32Out>
__global__ void __launch_bounds__(kFiltThreads, 4)
k_prec_filter(const float4* __restrict__ P, const uint32_t* __restrict__ nonempty, int ov, const float2* __restrict__ taps,
              uint32_t ntaps, uint32_t center, uint32_t nR, uint32_t nB, uint32_t Kp, uint16_t* __restrict__ A,
              float2* __restrict__ Gf, uint32_t* __restrict__ rowmax)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int ntc = min((int)max(ntaps, 1u), kFiltTapsMax);
    float2* sG = reinterpret_cast<float2*>(s_raw);                    // [kFiltRows + ntc - 1][kFiltCols]
    float2* sT = sG + (size_t)(kFiltRows + ntc - 1) * kFiltCols;       // [kFiltTapsMax]
    int2* sW = reinterpret_cast<int2*>(sT + kFiltTapsMax);              // [kFiltRows]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = blockIdx.y * kFiltRows, k0 = blockIdx.x * kFiltCols;
    if(tid < kFiltRows) sW[tid] = (r0 + tid < (int)nR) ? row_window(nonempty, nR, ov, r0 + tid) : make_int2(1, 0);
    float2 acc[8][2];
#pragma unroll
    for(int q = 0; q < 8; q++) { acc[q][0] = make_float2(0.f, 0.f); acc[q][1] = make_float2(0.f, 0.f); }

    for(int tc = 0; tc < (int)ntaps; tc += ntc) {
        const int nt = min(ntc, (int)ntaps - tc);
        const int jlo = r0 + tc - (int)center;          // bin of sG row 0
        const int rows_s = kFiltRows + nt - 1;
        __syncthreads();
        if(tid < nt) sT[tid] = taps[tc + tid];
#pragma unroll 2
        for(int rr = warp; rr < rows_s; rr += kFiltThreads / 32) {
            const int j = jlo + rr;
            const bool jok = j >= 0 && j < (int)nR;
            const float4* row = P + (size_t)(jok ? j : 0) * nB;
            float4 c[2];
#pragma unroll
            for(int h = 0; h < 2; h++) {
                const int k = k0 + 32 * h + lane;
                c[h] = (jok && k < (int)nB) ? row[k] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            const float4 lead = (jok && lane == 0 && k0 > 0) ? row[k0 - 1] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for(int h = 0; h < 2; h++) {
                float zx = __shfl_up_sync(0xffffffffu, c[h].z, 1), zy = __shfl_up_sync(0xffffffffu, c[h].w, 1);
                const float ex = __shfl_sync(0xffffffffu, c[0].z, 31), ey = __shfl_sync(0xffffffffu, c[0].w, 31);
                if(lane == 0) {
                    zx = h == 0 ? lead.z : ex;
                    zy = h == 0 ? lead.w : ey;
                }
                const int k = k0 + 32 * h + lane;
                float2 g = make_float2(c[h].x, c[h].y);
                if(k > 0) { g.x += zx; g.y += zy; }
                // column cc = 32 h + lane is stored at (cc & 1) * 32 + cc / 2: the
                // compute loop's lane reads columns 2 lane and 2 lane + 1 from two
                // conflict-free 32-float2 planes
                sG[rr * kFiltCols + (lane & 1) * 32 + 16 * h + (lane >> 1)] = g;
            }
        }
        __syncthreads();
        // Fast path (every row of this warp's eight takes all nt taps of the
        // chunk): a sliding window of eight staged rows per column in
        // registers, one shared load per tap and column instead of one per
        // tap, row and column. Same operations in the same tap order as the
        // general path.
        bool full = true;
#pragma unroll
        for(int q = 0; q < 8; q++) {
            const int rr = warp * 8 + q, r = r0 + rr;
            const int2 w = sW[rr];
            if(w.x > w.y || w.x - r + (int)center > tc || w.y - r + (int)center < tc + nt - 1) full = false;
        }
        if(full) {
#pragma unroll
            for(int h = 0; h < 2; h++) {
                const float2* col = sG + h * 32 + lane + warp * 8 * kFiltCols;
                float2 g[8];
#pragma unroll
                for(int i = 0; i < 7; i++) g[i] = col[i * kFiltCols];
                // Blocks of eight taps with the window rotated at compile time:
                // at step i of a block, staged row tt + i + q sits in slot
                // (q + i) & 7 and the new row goes to the slot of the row just
                // dropped; after eight steps the window is back in order.
                int tt = 0;
                for(; tt + 8 <= nt; tt += 8) {
#pragma unroll
                    for(int i = 0; i < 8; i++) {
                        g[(i + 7) & 7] = col[(tt + i + 7) * kFiltCols];
                        const float2 c = sT[tt + i];
#pragma unroll
                        for(int q = 0; q < 8; q++) {
                            const float2 gq = g[(q + i) & 7];
                            acc[q][h].x = fmaf(c.x, gq.x, fmaf(-c.y, gq.y, acc[q][h].x));
                            acc[q][h].y = fmaf(c.x, gq.y, fmaf(c.y, gq.x, acc[q][h].y));
                        }
                    }
                }
                for(; tt < nt; tt++) {
                    g[7] = col[(tt + 7) * kFiltCols];
                    const float2 c = sT[tt];
#pragma unroll
                    for(int q = 0; q < 8; q++) {
                        acc[q][h].x = fmaf(c.x, g[q].x, fmaf(-c.y, g[q].y, acc[q][h].x));
                        acc[q][h].y = fmaf(c.x, g[q].y, fmaf(c.y, g[q].x, acc[q][h].y));
                    }
#pragma unroll
                    for(int i = 0; i < 7; i++) g[i] = g[i + 1];
                }
            }
        }
        else {
#pragma unroll
            for(int q = 0; q < 8; q++) {
                const int rr = warp * 8 + q, r = r0 + rr;
                const int2 w = sW[rr];
                if(w.x > w.y) continue;
                // taps t (absolute) with bin j = r + t - center inside the window
                const int tlo = max(tc, w.x - r + (int)center), thi = min(tc + nt - 1, w.y - r + (int)center);
                for(int t = tlo; t <= thi; t++) {
                    const float2 c = sT[t - tc];
#pragma unroll
                    for(int h = 0; h < 2; h++) {
                        const float2 g = sG[(rr + t - tc) * kFiltCols + h * 32 + lane];
                        acc[q][h].x = fmaf(c.x, g.x, fmaf(-c.y, g.y, acc[q][h].x));
                        acc[q][h].y = fmaf(c.x, g.y, fmaf(c.y, g.x, acc[q][h].y));
                    }
                }
            }
        }
    }
    const int k = k0 + 2 * lane;
    if constexpr(kF32Out) {
#pragma unroll
        for(int q = 0; q < 8; q++) {
            const int r = r0 + warp * 8 + q;
            if(r >= (int)nR) continue;     // warp-uniform
            float m = 0.0f;
#pragma unroll
            for(int h = 0; h < 2; h++) {
                if(k + h >= (int)nB) continue;
                Gf[(size_t)r * nB + k + h] = acc[q][h];
                m = fmaxf(m, fmaxf(fabsf(acc[q][h].x), fabsf(acc[q][h].y)));
            }
            for(int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if(lane == 0 && m > 0.0f) atomicMax(&rowmax[r], __float_as_uint(m));
        }
        return;
    }
    const bool packed = (nB & 1u) == 0u && k + 1 < (int)nB;
#pragma unroll
    for(int q = 0; q < 8; q++) {
        const int r = r0 + warp * 8 + q;
        if(r >= (int)nR || k >= (int)nB) continue;
        uint16_t* row = A + (size_t)r * Kp;
        uint16_t hr[2], hi[2], lr[2], li[2];
#pragma unroll
        for(int h = 0; h < 2; h++) {
            const float2 v = acc[q][h];
            hr[h] = bf16_bits(v.x); hi[h] = bf16_bits(v.y);
            lr[h] = bf16_bits(v.x - bf16_value(hr[h])); li[h] = bf16_bits(v.y - bf16_value(hi[h]));
        }
        if(packed) {
            auto put = [&](uint32_t off, const uint16_t* v2) {
                *reinterpret_cast<uint32_t*>(row + off + k) = (uint32_t)v2[0] | ((uint32_t)v2[1] << 16);
            };
            put(0, hr); put(nB, hi); put(2 * nB, hr); put(3 * nB, hi); put(4 * nB, lr); put(5 * nB, li);
        }
        else {
#pragma unroll
            for(int h = 0; h < 2; h++) {
                if(k + h >= (int)nB) continue;
                row[k + h] = hr[h];            row[nB + k + h] = hi[h];
                row[2 * nB + k + h] = hr[h];   row[3 * nB + k + h] = hi[h];
                row[4 * nB + k + h] = lr[h];   row[5 * nB + k + h] = li[h];
            }
        }
    }
}

// FP16 per-row-scaled split: row r of the filtered grid is scaled by
// 2^(14 - e), e = floor(log2(rowmax[r])), so that its largest component lies
// in [2^14, 2^15), then split into fp16 [hi | hi | lo] (lo = x - hi, so
// hi + lo carries 22 significant bits); row_scale[r] = 2^(e - 14) undoes the
// scaling exactly in the GEMM epilogue. One CTA per row.
__device__ __forceinline__ int scale_exponent(uint32_t maxbits)
{
    if(maxbits == 0u) return 0;                       // zero row: scale 1
    const int e = (int)((maxbits >> 23) & 0xffu) - 127;
    return min(max(14 - e, -126), 127);
}

__global__ void k_prec_split_f16(const float2* __restrict__ Gf, const uint32_t* __restrict__ rowmax, uint32_t nR,
                                 uint32_t nB, uint32_t Kp, uint16_t* __restrict__ A, float* __restrict__ row_scale)
{
    const uint32_t r = blockIdx.x;
    if(r >= nR) return;
    const int se = scale_exponent(rowmax[r]);
    const float s = __uint_as_float((uint32_t)(se + 127) << 23);
    if(threadIdx.x == 0) row_scale[r] = __uint_as_float((uint32_t)(127 - se) << 23);
    uint16_t* row = A + (size_t)r * Kp;
    for(uint32_t k = threadIdx.x; k < nB; k += blockDim.x) {
        const float2 v = Gf[(size_t)r * nB + k];
        const float xr = v.x * s, xi = v.y * s;
        const __half hr = __float2half_rn(xr), hi = __float2half_rn(xi);
        const __half lr = __float2half_rn(xr - __half2float(hr)), li = __float2half_rn(xi - __half2float(hi));
        row[k] = __half_as_ushort(hr);            row[nB + k] = __half_as_ushort(hi);
        row[2 * nB + k] = __half_as_ushort(hr);   row[3 * nB + k] = __half_as_ushort(hi);
        row[4 * nB + k] = __half_as_ushort(lr);   row[5 * nB + k] = __half_as_ushort(li);
    }
}

// Round-to-nearest-even float -> IEEE-754 binary16 bit pattern (from the
// format definition: 10-bit mantissa, exponent bias 15, subnormal unit 2^-24).
uint16_t host_f16_bits(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    const uint32_t sign = (u >> 16) & 0x8000u, a = u & 0x7fffffffu;
    if(a >= 0x7f800000u) return (uint16_t)(sign | 0x7c00u | (a > 0x7f800000u ? 0x200u : 0u));
    if(a >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);          // >= 65520 rounds to infinity
    if(a <= 0x33000000u) return (uint16_t)sign;                      // <= 2^-25 rounds to zero
    const int e = (int)(a >> 23) - 127;
    const uint32_t m = (a & 0x7fffffu) | 0x800000u;
    if(e >= -14) {
        uint32_t h = ((uint32_t)(e + 15) << 10) | ((m >> 13) & 0x3ffu);
        const uint32_t rem = m & 0x1fffu;
        if(rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    const int shift = -e - 1;                                        // 14 .. 24
    uint32_t h = m >> shift;
    const uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
    if(rem > half || (rem == half && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

float host_f16_value(uint16_t h)
{
    const uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    float v;
    if(e == 0u) v = std::ldexp((float)m, -24);
    else if(e == 31u) v = m ? NAN : INFINITY;
    else v = std::ldexp((float)(m | 0x400u), (int)e - 25);
    return (h & 0x8000u) ? -v : v;
}

uint16_t host_bf16_bits(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

float host_bf16_value(uint16_t b)
{
    uint32_t u = (uint32_t)b << 16;
    float x;
    std::memcpy(&x, &u, 4);
    return x;
}

double host_lerp(const float* tab, int n, int comps, int comp, double x)
{
    const double fl = std::floor(x);
    if(!(fl >= -1.0 && fl <= (double)(n - 1))) return 0.0;
    const int i = (int)fl;
    const double a = x - fl;
    const double lo = i >= 0 ? tab[(size_t)i * comps + comp] : 0.0;
    const double hi = i + 1 < n ? tab[(size_t)(i + 1) * comps + comp] : 0.0;
    return lo * (1.0 - a) + hi * a;
}

#define RTACX_CUDA(call)                                                         \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if(e_ != cudaSuccess) {                                                  \
            ctx.error = std::string(#call) + ": " + cudaGetErrorString(e_);      \
            return RTACX_ERR_CUDA;                                               \
        }                                                                        \
    } while(0)

template <typename T>
void free_dev(T*& p)
{
    if(p) cudaFree(p);
    p = nullptr;
}

} // namespace

void free_precision(Context& c)
{
    free_dev(c.d_G); free_dev(c.d_flags); free_dev(c.d_A); free_dev(c.d_B);
    free_dev(c.d_C); free_dev(c.d_taps); free_dev(c.d_lut);
    free_dev(c.d_Gf); free_dev(c.d_rowmax); free_dev(c.d_row_scale); free_dev(c.d_col_scale);
    free_dev(c.d_hot); free_dev(c.d_hotcnt); free_dev(c.d_rep);
    c.prec_f16 = false;
    c.prec_hot = false;
    c.prec_configured = false;
}

rtacx_status configure_precision(Context& ctx, const rtacx_precision_desc* d)
{
    if(!ctx.configured || ctx.dims != 2) { ctx.error = "the precision form needs a configured 2D sensor"; return RTACX_ERR_NOT_CONFIGURED; }
    if(!d) { ctx.error = "null precision descriptor"; return RTACX_ERR_INVALID_ARGUMENT; }
    const uint32_t nB = ctx.nB, nR = ctx.nR;
    if(nB > (uint32_t)kMaxBearingsSmem) { ctx.error = "too many bearings for the precision form"; return RTACX_ERR_UNSUPPORTED; }
    for(uint32_t b = 1; b < nB; b++)
        if(!(ctx.bearings[b] > ctx.bearings[b - 1])) {
            ctx.error = "the precision form needs strictly increasing bearings";
            return RTACX_ERR_INVALID_ARGUMENT;
        }
    free_precision(ctx);

    // Directivity D[k][b] (complex), given or derived from the beam table.
    std::vector<float> D((size_t)nB * nB * 2, 0.0f);
    if(d->directivity) {
        std::memcpy(D.data(), d->directivity, D.size() * sizeof(float));
    }
    else {
        const double kx = (double)(1.0f / ctx.span) * ctx.W, cx = 0.5 * ctx.W - 0.5;
        for(uint32_t k = 0; k < nB; k++)
            for(uint32_t b = 0; b < nB; b++) {
                const float e = ctx.bearings[k] - ctx.bearings[b];
                D[((size_t)k * nB + b) * 2] = (float)host_lerp(ctx.beam.data(), (int)ctx.W, 1, 0, (double)e * kx + cx);
            }
    }
    for(float v : D) if(!std::isfinite(v)) { ctx.error = "non-finite directivity"; return RTACX_ERR_INVALID_ARGUMENT; }

    // Range taps, given or derived from the pulse table at bin offsets.
    std::vector<float> taps;
    uint32_t center;
    if(d->range_taps) {
        if(d->tap_count == 0 || d->tap_center >= d->tap_count) { ctx.error = "bad tap_count / tap_center"; return RTACX_ERR_INVALID_ARGUMENT; }
        taps.assign(d->range_taps, d->range_taps + 2 * (size_t)d->tap_count);
        center = d->tap_center;
    }
    else {
        const int ov = std::max(0, ctx.overlap);
        const double res = (nR > 1) ? (double)((ctx.rmax - ctx.rmin) / (float)(nR - 1u)) : 0.0;
        const float pscale = host_pulse_scale(ctx.duration, ctx.c, false);
        const double ky = (double)pscale * ctx.H, cy = 0.5 * ctx.H - 0.5;
        int first = ov + 1, last = -ov - 1;
        std::vector<float> full((size_t)(2 * ov + 1) * 2);
        for(int t = -ov; t <= ov; t++) {
            const double x = t * res * ky + cy;
            const float re = (float)host_lerp(ctx.pulse.data(), (int)ctx.H, 2, 0, x);
            const float im = (float)host_lerp(ctx.pulse.data(), (int)ctx.H, 2, 1, x);
            full[(size_t)(t + ov) * 2] = re; full[(size_t)(t + ov) * 2 + 1] = im;
            if(re != 0.0f || im != 0.0f) { first = std::min(first, t); last = std::max(last, t); }
        }
        if(first > last) { first = 0; last = 0; }
        taps.assign(full.begin() + (size_t)(first + ov) * 2, full.begin() + (size_t)(last + ov + 1) * 2);
        center = (uint32_t)(-first);
    }
    for(float v : taps) if(!std::isfinite(v)) { ctx.error = "non-finite range taps"; return RTACX_ERR_INVALID_ARGUMENT; }
    ctx.taps = (uint32_t)(taps.size() / 2);
    ctx.tap_center = center;
    if(nR > (uint32_t)kMaxRangeWords * 32) { ctx.error = "too many range bins for the precision form"; return RTACX_ERR_UNSUPPORTED; }

    // Bearing lookup grid (see k_prec_accumulate): entry c = {number of
    // interior bearings theta_1 .. theta_nB-2 in grid cells below c, the
    // interior bearing in cell c or +inf}; exact when no cell holds two.
    const uint32_t cells = std::min<uint32_t>(4 * nB, (uint32_t)kLutCells);
    const float origin = ctx.bearings[0];
    const float width = (nB > 1) ? ctx.bearings[nB - 1] - ctx.bearings[0] : 1.0f;
    const float lscale = (float)cells / width;
    std::vector<int> in_cell(cells, 0);
    std::vector<float> lut_bearing(cells, INFINITY);
    for(uint32_t b = 1; b + 1 < nB; b++) {
        const int cidx = bearing_grid_cell(ctx.bearings[b], origin, lscale, cells);
        in_cell[cidx]++;
        lut_bearing[cidx] = ctx.bearings[b];
    }
    std::vector<float2> lut(cells);
    bool exact = true;
    for(uint32_t cidx = 0, below = 0; cidx < cells; cidx++) {
        exact = exact && in_cell[cidx] <= 1;
        float count_bits;
        std::memcpy(&count_bits, &below, sizeof(float));
        lut[cidx] = make_float2(count_bits, lut_bearing[cidx]);
        below += (uint32_t)in_cell[cidx];
    }
    ctx.lut_exact = exact ? 1 : 0;
    ctx.lut_cells = cells;
    ctx.lut_origin = origin;
    ctx.lut_scale = lscale;
    ctx.acc_smem = accumulate_smem_bytes(nB, nR, cells);
    int acc_blocks = 0;
    if(raise_smem_limit((const void*)k_prec_accumulate, ctx.acc_smem) != cudaSuccess ||
       cudaOccupancyMaxActiveBlocksPerMultiprocessor(&acc_blocks, k_prec_accumulate, kAccThreads, ctx.acc_smem) !=
           cudaSuccess ||
       acc_blocks < 1) {
        cudaGetLastError();
        ctx.error = "cannot reserve shared memory for the accumulation tables";
        return RTACX_ERR_CUDA;
    }
    ctx.acc_blocks_per_sm = (uint32_t)acc_blocks;
    ctx.acc_staged_smem = staged_smem_bytes(nB, nR, cells);
    for(int m = 0; m < kAccEchoModels; m++) {
        const void* fs = accumulate_staged_kernel(m);
        int bs = 0;
        if(raise_smem_limit(fs, ctx.acc_staged_smem) != cudaSuccess ||
           cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, fs, kStagedThreads, ctx.acc_staged_smem) != cudaSuccess)
            bs = 0;
        cudaGetLastError();
        ctx.acc_staged_blocks[m] = (uint32_t)std::max(bs, 0);
    }
    if(raise_smem_limit((const void*)k_prec_filter<false>, filter_smem_bytes(kFiltTapsMax)) != cudaSuccess ||
       raise_smem_limit((const void*)k_prec_filter<true>, filter_smem_bytes(kFiltTapsMax)) != cudaSuccess) {
        ctx.error = "cannot reserve shared memory for the range filter";
        return RTACX_ERR_CUDA;
    }

    // GEMM operand shapes.
    ctx.Mpad = (nR + 127) / 128 * 128;
    ctx.Npad = (2 * nB + 255) / 256 * 256;
    ctx.Kp = (6 * nB + 63) / 64 * 64;

    // B operand: row n = 2b (real) / 2b + 1 (imag); K blocks [hi | lo | hi]
    // of [real part of G pairs | imaginary part of G pairs]. FP16 form: each
    // row n is first scaled by 2^(14 - e_n) (largest |value| in [2^14, 2^15))
    // and col_scale[n] = 2^(e_n - 14) undoes it in the GEMM epilogue.
    const bool f16 = (d->flags & RTACX_PRECISION_FP16_ROWSCALE) != 0;
    const bool hot = (d->flags & RTACX_PRECISION_HOT_RANGE) != 0;
    if(d->flags & ~(RTACX_PRECISION_FP16_ROWSCALE | RTACX_PRECISION_HOT_RANGE)) {
        ctx.error = "unknown precision flags";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint16_t> B((size_t)ctx.Npad * ctx.Kp, 0);
    std::vector<float> col_scale(ctx.Npad, 1.0f);
    for(uint32_t b = 0; b < nB; b++)
        for(int o = 0; o < 2; o++) {
            auto value = [&](uint32_t k, int h) {
                const float dr = D[((size_t)k * nB + b) * 2], di = D[((size_t)k * nB + b) * 2 + 1];
                const float vals[2][2] = {{dr, -di}, {di, dr}};     // [re/im output][G real / G imag]
                return vals[o][h];
            };
            float scale = 1.0f;
            if(f16) {
                float mx = 0.0f;
                for(uint32_t k = 0; k < nB; k++) mx = std::max(mx, std::max(std::fabs(value(k, 0)), std::fabs(value(k, 1))));
                if(mx > 0.0f) {
                    const int se = std::min(std::max(14 - std::ilogb(mx), -126), 127);
                    scale = std::ldexp(1.0f, se);
                    col_scale[2 * b + o] = std::ldexp(1.0f, -se);
                }
            }
            uint16_t* row = B.data() + (size_t)(2 * b + o) * ctx.Kp;
            for(uint32_t k = 0; k < nB; k++)
                for(int h = 0; h < 2; h++) {
                    const float v = value(k, h) * scale;
                    uint16_t bh, bl;
                    if(f16) { bh = host_f16_bits(v); bl = host_f16_bits(v - host_f16_value(bh)); }
                    else { bh = host_bf16_bits(v); bl = host_bf16_bits(v - host_bf16_value(bh)); }
                    row[h * nB + k] = bh;
                    row[2 * nB + h * nB + k] = bl;
                    row[4 * nB + h * nB + k] = bh;
                }
        }

    const bool direct = (ctx.Mpad == nR) && (ctx.Npad == 2 * nB);
    auto alloc = [&](auto*& p, size_t bytes) {
        if(cudaMalloc(&p, bytes) != cudaSuccess) { cudaGetLastError(); p = nullptr; return false; }
        return true;
    };
    if(!alloc(ctx.d_G, (size_t)nR * nB * sizeof(float4)) || !alloc(ctx.d_flags, (size_t)(nR + 31) / 32 * 4) ||
       !alloc(ctx.d_lut, (size_t)cells * sizeof(float2)) ||
!alloc(ctx.d_A, (size_t)ctx.Mpad * ctx.Kp * 2) ||
       !alloc(ctx.d_B, B.size() * 2) || !alloc(ctx.d_taps, taps.size() * sizeof(float)) ||
       (!direct && !alloc(ctx.d_C, (size_t)ctx.Mpad * ctx.Npad * sizeof(float))) ||
       (f16 && (!alloc(ctx.d_Gf, (size_t)nR * nB * sizeof(float2)) || !alloc(ctx.d_rowmax, (size_t)nR * 4) ||
                !alloc(ctx.d_row_scale, (size_t)ctx.Mpad * sizeof(float)) ||
                !alloc(ctx.d_col_scale, (size_t)ctx.Npad * sizeof(float)))) ||
       (hot && (!alloc(ctx.d_hot, sizeof(int2)) || !alloc(ctx.d_hotcnt, (size_t)nR * 4) ||
                !alloc(ctx.d_rep, (size_t)kHotRows * kHotReplicas * nB * sizeof(float4))))) {
        free_precision(ctx);
        ctx.error = "out of device memory for the precision form";
        return RTACX_ERR_OUT_OF_MEMORY;
    }
    if(cudaMemset(ctx.d_A, 0, (size_t)ctx.Mpad * ctx.Kp * 2) != cudaSuccess ||
       cudaMemcpy(ctx.d_B, B.data(), B.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(ctx.d_taps, taps.data(), taps.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(ctx.d_lut, lut.data(), lut.size() * sizeof(float2), cudaMemcpyHostToDevice) != cudaSuccess ||
       (f16 && (cudaMemcpy(ctx.d_col_scale, col_scale.data(), col_scale.size() * sizeof(float),
                           cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemset(ctx.d_row_scale, 0, (size_t)ctx.Mpad * sizeof(float)) != cudaSuccess)) ||
       (hot && (cudaMemset(ctx.d_hot, 0, sizeof(int2)) != cudaSuccess ||
                cudaMemset(ctx.d_hotcnt, 0, (size_t)nR * 4) != cudaSuccess))) {
        cudaGetLastError();
        free_precision(ctx);
        ctx.error = "uploading the precision tables failed";
        return RTACX_ERR_CUDA;
    }
    if(gemm_smem_bytes() > 227 * 1024) { ctx.error = "GEMM tile exceeds shared memory"; return RTACX_ERR_UNSUPPORTED; }
    if(hot && raise_smem_limit((const void*)k_hot_pick, (nR + 1) * sizeof(uint32_t)) != cudaSuccess) {
        free_precision(ctx);
        ctx.error = "cannot reserve shared memory for the hot-range scan";
        return RTACX_ERR_CUDA;
    }
    ctx.prec_f16 = f16;
    ctx.prec_hot = hot;
    ctx.prec_configured = true;
    return RTACX_OK;
}

// Zeroes the pair cells and the non-empty bitmap of a new ping.
rtacx_status precision_begin(Context& ctx, cudaStream_t stream)
{
    const uint64_t cells = (uint64_t)ctx.nR * ctx.nB;
    const uint32_t blocks = (uint32_t)std::min<uint64_t>((cells + 255) / 256, (uint64_t)ctx.sm_count * 32);
    k_prec_clear<<<blocks, 256, 0, stream>>>(ctx.d_G, cells, ctx.d_flags, (ctx.nR + 31) / 32);
    RTACX_CUDA(cudaGetLastError());
    return RTACX_OK;
}

// Adds n samples to the ping's pair cells (order-independent, so a ping may
// be accumulated in any number of chunks).
rtacx_status precision_accumulate(Context& ctx, const void* samples, uint64_t n, cudaStream_t stream)
{
    if(!n) return RTACX_OK;
    const uint64_t want = (n + kAccThreads * kAccLoads - 1) / (kAccThreads * kAccLoads);
    if(ctx.lut_exact && ctx.nB > 1 && !ctx.prec_hot && ctx.bin.vec4 &&
       (reinterpret_cast<uintptr_t>(samples) & 15u) == 0) {
        const int m = accumulate_echo_model(ctx.bin.echo_flags);
        if(ctx.acc_staged_blocks[m] > 0) {
            const uint64_t stages = (n + kStageRecs - 1) / kStageRecs;
            const uint32_t blocks = (uint32_t)std::min<uint64_t>(stages, (uint64_t)ctx.sm_count * ctx.acc_staged_blocks[m]);
            void* args[] = {(void*)&samples, (void*)&n, (void*)&ctx.bin, (void*)&ctx.d_bearings, (void*)&ctx.nB,
                            (void*)&ctx.d_lut, (void*)&ctx.lut_cells, (void*)&ctx.lut_origin, (void*)&ctx.lut_scale,
                            (void*)&ctx.d_G, (void*)&ctx.d_flags, (void*)&ctx.d_err, (void*)&ctx.diag_drop_stage};
            RTACX_CUDA(cudaLaunchKernel(accumulate_staged_kernel(m), dim3(blocks), dim3(kStagedThreads), args,
                                        ctx.acc_staged_smem, stream));
            return RTACX_OK;
        }
    }
    const uint32_t blocks = (uint32_t)std::min<uint64_t>(want, (uint64_t)ctx.sm_count * ctx.acc_blocks_per_sm);
    k_prec_accumulate<<<blocks, kAccThreads, ctx.acc_smem, stream>>>(static_cast<const float*>(samples), n, ctx.bin,
                                                                     ctx.d_bearings, ctx.nB, ctx.d_lut, ctx.lut_cells,
                                                                     ctx.lut_origin, ctx.lut_scale, ctx.lut_exact,
                                                                     ctx.d_G, ctx.d_flags,
                                                                     ctx.prec_hot ? ctx.d_hot : nullptr, ctx.d_rep);
    RTACX_CUDA(cudaGetLastError());
    return RTACX_OK;
}

// Hot-range detection on (a strided subsample of) these samples and zeroing
// of the hot rows' replicas; nothing without RTACX_PRECISION_HOT_RANGE.
rtacx_status precision_hot_scan(Context& ctx, const void* samples, uint64_t n, cudaStream_t stream)
{
    if(!ctx.prec_hot) return RTACX_OK;
    const uint64_t step = std::max<uint64_t>(1, n / 131072);
    const uint64_t m = n ? (n + step - 1) / step : 0;
    if(m) {
        const uint32_t blocks = (uint32_t)std::min<uint64_t>((m + 255) / 256, (uint64_t)ctx.sm_count * 4);
        k_hot_count<<<blocks, 256, 0, stream>>>(static_cast<const float*>(samples), n, ctx.bin, step, ctx.d_hotcnt);
        RTACX_CUDA(cudaGetLastError());
    }
    k_hot_pick<<<1, kHotPickThreads, (ctx.nR + 1) * sizeof(uint32_t), stream>>>(ctx.d_hotcnt, ctx.nR, ctx.d_hot);
    RTACX_CUDA(cudaGetLastError());
    k_hot_zero<<<ctx.sm_count * 4, 256, 0, stream>>>(ctx.d_hot, ctx.nB, ctx.d_rep);
    RTACX_CUDA(cudaGetLastError());
    return RTACX_OK;
}

rtacx_status precision_finish(Context& ctx, float* out, cudaStream_t stream);

rtacx_status run_precision(Context& ctx, const void* samples, uint64_t n, float* out, cudaStream_t stream)
{
    ctx.mark(5, false, stream);
    rtacx_status st = precision_begin(ctx, stream);
    ctx.mark(5, true, stream);
    ctx.mark(0, false, stream);
    if(st == RTACX_OK) st = precision_hot_scan(ctx, samples, n, stream);
    if(st == RTACX_OK) st = precision_accumulate(ctx, samples, n, stream);
    if(st != RTACX_OK) return st;
    ctx.mark(0, true, stream);
    return precision_finish(ctx, out, stream);
}

// Windows, range filter + split, tensor-core contraction into `out`.
rtacx_status precision_finish(Context& ctx, float* out, cudaStream_t stream)
{
    const uint32_t nR = ctx.nR, nB = ctx.nB;
    if(ctx.prec_hot) {
        k_hot_fold<<<ctx.sm_count * 4, 256, 0, stream>>>(ctx.d_hot, nB, ctx.d_rep, ctx.d_G);
        RTACX_CUDA(cudaGetLastError());
    }
    ctx.mark(2, false, stream);
    const dim3 fgrid((nB + kFiltCols - 1) / kFiltCols, (nR + kFiltRows - 1) / kFiltRows);
    if(!ctx.prec_f16) {
        k_prec_filter<false><<<fgrid, kFiltThreads, filter_smem_bytes(ctx.taps), stream>>>(
            ctx.d_G, ctx.d_flags, ctx.overlap, ctx.d_taps, ctx.taps, ctx.tap_center, nR, nB, ctx.Kp, ctx.d_A, nullptr, nullptr);
        RTACX_CUDA(cudaGetLastError());
    }
    else {
        RTACX_CUDA(cudaMemsetAsync(ctx.d_rowmax, 0, (size_t)nR * 4, stream));
        k_prec_filter<true><<<fgrid, kFiltThreads, filter_smem_bytes(ctx.taps), stream>>>(
            ctx.d_G, ctx.d_flags, ctx.overlap, ctx.d_taps, ctx.taps, ctx.tap_center, nR, nB, ctx.Kp, nullptr, ctx.d_Gf, ctx.d_rowmax);
        RTACX_CUDA(cudaGetLastError());
        k_prec_split_f16<<<nR, 256, 0, stream>>>(ctx.d_Gf, ctx.d_rowmax, nR, nB, ctx.Kp, ctx.d_A, ctx.d_row_scale);
        RTACX_CUDA(cudaGetLastError());
    }
    ctx.mark(2, true, stream);
    ctx.mark(3, false, stream);
    const bool direct = ctx.d_C == nullptr;
    float* C = direct ? out : ctx.d_C;
    rtacx_status st = gemm_tn(ctx.error, ctx.d_A, ctx.d_B, C, (int)ctx.Mpad, (int)ctx.Npad, (int)ctx.Kp,
                              (int)ctx.Npad, stream, ctx.d_err, ctx.prec_f16, ctx.prec_f16 ? ctx.d_row_scale : nullptr,
                              ctx.prec_f16 ? ctx.d_col_scale : nullptr);
    if(st != RTACX_OK) return st;
    ctx.mark(3, true, stream);
    ctx.mark(4, false, stream);
    if(!direct)
        RTACX_CUDA(cudaMemcpy2DAsync(out, (size_t)2 * nB * sizeof(float), ctx.d_C, (size_t)ctx.Npad * sizeof(float),
                                     (size_t)2 * nB * sizeof(float), nR, cudaMemcpyDeviceToDevice, stream));
    ctx.mark(4, true, stream);
    return RTACX_OK;
}

} // namespace rtacx
