// Precision (tensor-core) form: bin onto a grid first, contract over
// bearings on the tensor cores, then filter in range.
//
//   k_prec_clear       zeroes the binned grid and the non-empty bitmap.
//   k_prec_accumulate  one pass over the samples (read once, 16 B each):
//   (_staged)          reference range key (Binner::Key, bit-exact) into the
//                      non-empty bitmap, optional FP64 echo pre-step, then a
//                      bilinear split onto the grid: linear in range between
//                      the two range nodes around the travel (one node every
//                      two output bins), linear in bearing between the two
//                      grid bearings around the sample bearing. The grid is
//                      stored by bearing interval: entry (node, q) holds the
//                      interval's shares of grid bearings q and q + 1, so each
//                      sample is exactly two 16-byte vector reductions; node
//                      rows are stored in pairs, so that lane pairs send a
//                      sample's two reductions as one 32-byte sector request
//                      when its nodes share a pair. No sort.
//   k_prec_split       grid bearing q of a node = left share of interval q +
//                      right share of interval q - 1, as the bf16 A operand
//                      [hi | hi | lo] of the three-term split product
//                      (k_prec_split_f16: fp16 with a power-of-two scale per
//                      row).
//   gemm_tn            C = A x B^T on tcgen05 (rtacx_umma.cu), B the
//                      [hi | lo | hi] split of the complex directivity laid
//                      out so that column 2b of C is the real and 2b + 1 the
//                      imaginary part of the grid contracted onto bearing b.
//   k_prec_filter      the range taps of each output-row parity over C's
//                      node rows, rows whose reference window
//                      (src/Binner.cu:90-102) is empty set to zero: the
//                      complex64 ping.
// The range filter runs after the contraction (the two commute): it then
// works on bearing_count columns instead of the grid's.
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
constexpr int kMaxRangeWords = 8192 / 32 * 4;   // bitmap words for up to 32768 range bins
constexpr uint32_t kMaxGridCells = 16384;
constexpr int kAccThreads = 256;
// Hot range interval (RTACX_PRECISION_HOT_RANGE): kHotRows consecutive grid
// rows replicated kHotReplicas times; samples in them reduce into the replica
// of their CTA and warp, and k_hot_fold adds the replicas back into the grid
// before the contraction.
constexpr int kHotRows = 128, kHotReplicas = 8;
constexpr int kAccLoads = 4;                     // independent record loads per thread in flight
constexpr int kAccEchoModels = 6;                // echo models of the staged accumulation
// Grid rows are stored cells + kRowPad entries apart (128 bytes of padding,
// so that the row pitch is not a power of two): 4 % faster accumulation on
// the clustered 2^27-sample stress ping, no change on the uniform one.
constexpr uint32_t kRowPad = 8;

// L2 eviction priorities (createpolicy): the sample stream is read once
// and marked evict-first, the grid's reductions evict-last, so that the
// grid (68 MB on the 512 x 4096 ping) stays in L2 while 268 MB of samples
// stream past it.
__device__ __forceinline__ uint64_t policy_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t policy_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ void red_add_v4(float4* addr, float4 v, uint64_t pol)
{
    asm volatile("red.global.add.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;"
                 ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "l"(pol));
}

// Grid layout: node rows in pairs. Entry (node row j, bearing interval q)
// is float4 ((j >> 1) pitch + q) 2 + (j & 1), so the two rows of a pair share
// the 32-byte sector of each interval: a sample's two deposits (rows jg and
// jg + 1, one interval) fall into one sector when jg is even.
__host__ __device__ __forceinline__ size_t grid_at(int j, int q, uint32_t pitch)
{
    return ((size_t)(j >> 1) * pitch + (size_t)q) * 2 + (size_t)(j & 1);
}

// Grid entries of `rows` node rows (an odd last row keeps its pair's space).
__host__ __device__ __forceinline__ size_t grid_quads(uint32_t rows, uint32_t pitch)
{
    return (size_t)((rows + 1) >> 1) * pitch * 2;
}

// Adds a sample's share v of one range node to one bearing interval entry:
// (1 - w) v to the interval's left bearing, w v to its right bearing, in one
// 16-byte vector reduction. The grid is never read by the kernels that
// reduce into it, so the reductions carry no memory clobber.
__device__ __forceinline__ void deposit(float4* entry, float w, float2 v, uint64_t pol)
{
    const float w0 = 1.0f - w;
    red_add_v4(entry, make_float4(w0 * v.x, w0 * v.y, w * v.x, w * v.y), pol);
}

size_t accumulate_smem_bytes(uint32_t nR)
{
    return (size_t)((nR + 31) / 32) * sizeof(uint32_t);
}

// General accumulation: any record alignment, echo model read at run time,
// the hot-range replicas. Grid-stride over the samples, kAccLoads records per
// thread in flight; non-empty range bins (reference keys) in a shared bitmap
// OR-ed into the global one once per CTA.
__global__ void __launch_bounds__(kAccThreads)
k_prec_accumulate(const float* __restrict__ samples, uint64_t n, BinParams p, GridParams g,
                  float4* __restrict__ G, uint32_t* __restrict__ nonempty, const int2* __restrict__ hot,
                  float4* __restrict__ rep)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    uint32_t* s_bits = reinterpret_cast<uint32_t*>(s_raw);
    int hot_lo = 0, hot_len = 0;
    if(hot) { const int2 h = *hot; hot_lo = h.x; hot_len = h.y; }
    const uint32_t rsel = (blockIdx.x + (threadIdx.x >> 5)) & (kHotReplicas - 1);   // by CTA and warp
    const uint32_t pitch = g.pitch;
    // Entry (jg, q): the grid's, or in this warp's replica of a hot row
    // (replica rows are plain rows of `pitch` entries).
    auto entry = [&](int jg, int q) -> float4* {
        const uint32_t hj = (uint32_t)(jg - hot_lo);
        return hj < (uint32_t)hot_len ? rep + ((size_t)hj * kHotReplicas + rsel) * pitch + q : G + grid_at(jg, q, pitch);
    };
    const uint32_t words = (p.key.nR + 31) / 32;
    const uint64_t keep = policy_evict_last();
    for(uint32_t i = threadIdx.x; i < words; i += blockDim.x) s_bits[i] = 0u;
    __syncthreads();
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
            atomicOr(&s_bits[j >> 5], 1u << (j & 31));
            int jg, q;
            float alpha, w;
            if(!grid_coords(g, rec[u].z, rec[u].w, jg, alpha, q, w)) continue;
            const float2 v = apply_echo(p, make_float2(rec[u].x, rec[u].y), rec[u].z);
            const float a0 = 1.0f - alpha;
            deposit(entry(jg, q), w, make_float2(a0 * v.x, a0 * v.y), keep);
            deposit(entry(jg + 1, q), w, make_float2(alpha * v.x, alpha * v.y), keep);
        }
    }
    __syncthreads();
    for(uint32_t i = threadIdx.x; i < words; i += blockDim.x)
        if(s_bits[i]) atomicOr(&nonempty[i], s_bits[i]);
}

// The accumulation for the common case: 16-byte aligned records, no hot
// range, and the echo model kEcho fixed at compile time. The records reach
// shared memory by bulk copies (cp.async.bulk, the TMA engine) into a ring of
// kStages stages of kStageRecs records, so the bytes in flight per SM depend
// neither on registers nor on how long the threads compute. Each thread
// computes the key, grid coordinates and weighted values of its records of a
// stage without branches (invalid and tail records only clear a predicate),
// then issues the bitmap bits and the reductions; the results are those of
// k_prec_accumulate. One persistent CTA takes stages c = blockIdx.x,
// blockIdx.x + gridDim.x, ...; thread 0 issues the copy of the stage kStages
// ahead as soon as every thread has read the stage it refills. Each wait is
// bounded (kAccWaitCycles); a timeout sets kErrAccumulateTimeout in the error
// word, the CTA stops, and thread 0 waits (bounded again) for its copies
// still in flight before the CTA exits.
constexpr int kStageRecs = 1024;                 // 16 KB of records per stage
constexpr int kStages = 4;
constexpr int kStagedThreads = 512;
constexpr int kStagedPerThread = kStageRecs / kStagedThreads;
constexpr long long kAccWaitCycles = 2000000000ll;   // about one second

size_t staged_smem_bytes(uint32_t nR)
{
    return (size_t)kStages * kStageRecs * sizeof(float4) + (size_t)((nR + 31) / 32) * sizeof(uint32_t);
}

template <uint32_t kEcho>
__global__ void __launch_bounds__(kStagedThreads, 3)
k_prec_accumulate_staged(const float4* __restrict__ samples, uint64_t n, BinParams p, GridParams g,
                         float4* __restrict__ G, uint32_t* __restrict__ nonempty, uint32_t* __restrict__ err,
                         uint32_t drop_stage)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ __align__(8) uint64_t s_full[kStages];
    __shared__ int s_abort;
    float4* s_ring = reinterpret_cast<float4*>(s_raw);
    uint32_t* s_bits = reinterpret_cast<uint32_t*>(s_ring + kStages * kStageRecs);
    const uint32_t words = (p.key.nR + 31) / 32;
    const uint64_t stages = (n + kStageRecs - 1) / kStageRecs;
    const uint32_t pitch = g.pitch;
    const uint64_t stream_pol = policy_evict_first(), keep = policy_evict_last();
    auto issue = [&](uint64_t c, int slot) {
        if(c == drop_stage) return;      // failure-path test: this stage's copy never comes
        const uint64_t first = c * kStageRecs;
        const uint64_t left = n - first;
        const uint32_t bytes = (uint32_t)(left < (uint64_t)kStageRecs ? left : (uint64_t)kStageRecs) * (uint32_t)sizeof(float4);
        const uint32_t bar = smem_u32(&s_full[slot]);
        mbar_expect_tx(bar, bytes);
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
                     " [%0], [%1], %2, [%3], %4;"
                     ::"r"(smem_u32(s_ring + slot * kStageRecs)), "l"(samples + first), "r"(bytes), "r"(bar),
                       "l"(stream_pol)
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
        uint32_t key[kStagedPerThread];
        int row[kStagedPerThread], cell[kStagedPerThread];
        float wgt[kStagedPerThread];
        float4 add[kStagedPerThread];
#pragma unroll
        for(int u = 0; u < kStagedPerThread; u++) {
            const uint32_t idx = threadIdx.x + (uint32_t)u * kStagedThreads;
            const float4 rec = s_ring[slot * kStageRecs + min(idx, (uint32_t)kStageRecs - 1u)];
            const uint32_t k = range_key_select(p.key, rec.z);
            const bool live = ready && idx < count && k != kOutOfRange;
            key[u] = live ? k : kOutOfRange;
            int jg, q;
            float alpha, w;
            const bool ok = grid_coords(g, rec.z, rec.w, jg, alpha, q, w) && live;
            const float2 v = apply_echo(p, make_float2(rec.x, rec.y), rec.z, kEcho);
            row[u] = ok ? jg : -1;
            cell[u] = q;
            wgt[u] = w;
            const float a0 = 1.0f - alpha;
            add[u] = make_float4(a0 * v.x, a0 * v.y, alpha * v.x, alpha * v.y);
        }
        // Every thread has read the slot: refill it kStages stages ahead.
        aborted = __syncthreads_or(!ready) != 0;
        if(threadIdx.x == 0 && !aborted) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const uint64_t next = c + (uint64_t)kStages * gridDim.x;
            if(next < stages) issue(next, slot);
        }
        // Lanes 2k and 2k + 1 deposit together: first the even lane's
        // sample (row jg from the even lane, jg + 1 from the odd one), then
        // the odd lane's, so each reduction instruction sends a sample's two
        // rows of an interval as one sector when jg is even.
        const bool odd = (threadIdx.x & 1u) != 0u;
#pragma unroll
        for(int u = 0; u < kStagedPerThread; u++) {
            if(key[u] != kOutOfRange) atomicOr(&s_bits[key[u] >> 5], 1u << (key[u] & 31));
            const int row_p = __shfl_xor_sync(0xffffffffu, row[u], 1);
            const int cell_p = __shfl_xor_sync(0xffffffffu, cell[u], 1);
            const float wgt_p = __shfl_xor_sync(0xffffffffu, wgt[u], 1);
            float4 add_p;
            add_p.x = __shfl_xor_sync(0xffffffffu, add[u].x, 1);
            add_p.y = __shfl_xor_sync(0xffffffffu, add[u].y, 1);
            add_p.z = __shfl_xor_sync(0xffffffffu, add[u].z, 1);
            add_p.w = __shfl_xor_sync(0xffffffffu, add[u].w, 1);
#pragma unroll
            for(int h = 0; h < 2; h++) {
                // h = 0: the even lane's sample; h = 1: the odd lane's.
                const bool mine = odd == (h == 1);
                const int r = mine ? row[u] : row_p;
                if(r >= 0) {
                    const float4 a = mine ? add[u] : add_p;
                    deposit(G + grid_at(r + (odd ? 1 : 0), mine ? cell[u] : cell_p, pitch), mine ? wgt[u] : wgt_p,
                            odd ? make_float2(a.z, a.w) : make_float2(a.x, a.y), keep);
                }
            }
        }
        if(aborted) break;
    }
    if(aborted && threadIdx.x == 0) {
        atomicOr(err, kErrAccumulateTimeout);
        // Let the copies still in flight land before the CTA's shared memory
        // is released: those of iterations it .. it + kStages - 1 (the refill
        // of the aborted iteration was not issued). Each wait is bounded on
        // its own; a copy that was never issued (or never lands) costs one
        // more timeout.
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

// Zeroes the grid (16-byte stores, grid-stride) and the non-empty bitmap of
// a new ping in one launch.
__global__ void k_prec_clear(float4* __restrict__ G, uint64_t quads, uint32_t* __restrict__ bits, uint32_t words)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for(uint64_t i = i0; i < quads; i += stride) G[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for(uint64_t i = i0; i < words; i += stride) bits[i] = 0u;
}

// Hot-range detection (RTACX_PRECISION_HOT_RANGE): grid-row counts of a
// strided subsample of the ping, then one CTA picks the kHotRows-row window
// with the largest count. The window is hot when it holds at least a tenth of
// the counted samples and four times its uniform share; otherwise its length
// is 0 and every sample reduces into the grid. The counts are zeroed for the
// next ping.
__global__ void k_hot_count(const float* __restrict__ samples, uint64_t n, BinParams p, GridParams g, uint64_t step,
                            uint32_t* __restrict__ cnt)
{
    const uint64_t m = (n + step - 1) / step;
    for(uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < m; s += (uint64_t)gridDim.x * blockDim.x) {
        const float4 rec = load_record(samples, s * step, p);
        int side;
        if(range_key(p.key, rec.z, side) == kOutOfRange) continue;
        int jg, q;
        float alpha, w;
        if(grid_coords(g, rec.z, rec.w, jg, alpha, q, w)) atomicAdd(&cnt[jg], 1u);
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
// (nothing when the interval is empty). Replica rows of `pitch` entries.
__global__ void k_hot_fold(const int2* __restrict__ hot, uint32_t pitch, const float4* __restrict__ rep,
                           float4* __restrict__ G)
{
    const int2 h = *hot;
    const uint64_t total = (uint64_t)h.y * pitch;
    for(uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t row = i / pitch, k = i % pitch;
        const float4* rb = rep + row * kHotReplicas * pitch + k;
        float4* g = G + grid_at(h.x + (int)row, (int)k, pitch);
        float4 acc = *g;
        for(int r = 0; r < kHotReplicas; r++) {
            const float4 e = rb[(uint64_t)r * pitch];
            acc.x += e.x; acc.y += e.y; acc.z += e.z; acc.w += e.w;
        }
        *g = acc;
    }
}

// Zeroes the replicas of the hot rows (nothing when the interval is empty).
__global__ void k_hot_zero(const int2* __restrict__ hot, uint32_t pitch, float4* __restrict__ rep)
{
    const uint64_t total = (uint64_t)hot->y * kHotReplicas * pitch;
    for(uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x)
        rep[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ bool bit_set(const uint32_t* bits, long long j)
{
    return (bits[j >> 5] >> (j & 31)) & 1u;
}

// Does row r's reference window hold at least two non-empty range bins?
// The window of src/Binner.cu:90-102 covers [max(0, r - ov), min(nR - 1,
// r + ov)] shrunk to its first and last non-empty bins, and it is an empty
// view when fewer than two bins are non-empty.
__device__ __noinline__ bool row_has_window(const uint32_t* __restrict__ nonempty, uint32_t nR, int ov, int r)
{
    if(ov < 0) return false;
    const int lo = max(0, r - ov);
    const int hi = (int)min((long long)nR - 1, (long long)r + ov);
    int seen = 0;
    for(int j = lo; j <= hi && seen < 2; j++) seen += bit_set(nonempty, j) ? 1 : 0;
    return seen >= 2;
}

// Round-to-nearest-even fp32 -> bf16 (bit pattern).
__device__ __forceinline__ uint16_t bf16_bits(float x)
{
    uint32_t u = __float_as_uint(x);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

__device__ __forceinline__ float bf16_value(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

// Grid bearings q of both node rows of pair m: for each row the left share
// of bearing interval q plus the right share of interval q - 1 (interval
// cells - 1 is never written). Entries (2m, q) and (2m + 1, q) are adjacent.
__device__ __forceinline__ void pair_values(const float4* __restrict__ G, uint32_t m, uint32_t q, uint32_t pitch,
                                            float2& v0, float2& v1)
{
    const float4* e = G + grid_at((int)(2 * m), (int)q, pitch);
    const float4 a0 = e[0], a1 = e[1];
    if(q == 0) { v0 = make_float2(a0.x, a0.y); v1 = make_float2(a1.x, a1.y); return; }
    const float4 b0 = e[-2], b1 = e[-1];
    v0 = make_float2(a0.x + b0.z, a0.y + b0.w);
    v1 = make_float2(a1.x + b1.z, a1.y + b1.w);
}

// The A operand of the three-term split product: node row r (cells complex
// values) becomes A row r = [hi(Re) | hi(Im) | hi(Re) | hi(Im) | lo(Re) |
// lo(Im)], each block `cells` wide, lo = bf16(x - hi). One thread per pair of
// grid bearings of a pair of node rows: their entries are read once (six
// 16-byte loads), twelve 4-byte stores.
__device__ __forceinline__ void split_store(uint16_t* row, uint32_t cells, float2 n0, float2 n1)
{
    const float x[4] = {n0.x, n0.y, n1.x, n1.y};     // re0, im0, re1, im1
    uint16_t h[4], l[4];
#pragma unroll
    for(int i = 0; i < 4; i++) { h[i] = bf16_bits(x[i]); l[i] = bf16_bits(x[i] - bf16_value(h[i])); }
    const uint32_t hr = (uint32_t)h[0] | ((uint32_t)h[2] << 16), hi = (uint32_t)h[1] | ((uint32_t)h[3] << 16);
    const uint32_t lr = (uint32_t)l[0] | ((uint32_t)l[2] << 16), li = (uint32_t)l[1] | ((uint32_t)l[3] << 16);
    *reinterpret_cast<uint32_t*>(row) = hr;
    *reinterpret_cast<uint32_t*>(row + cells) = hi;
    *reinterpret_cast<uint32_t*>(row + 2 * cells) = hr;
    *reinterpret_cast<uint32_t*>(row + 3 * cells) = hi;
    *reinterpret_cast<uint32_t*>(row + 4 * cells) = lr;
    *reinterpret_cast<uint32_t*>(row + 5 * cells) = li;
}

__global__ void k_prec_split(const float4* __restrict__ G, uint32_t rows, uint32_t cells, uint32_t pitch, uint32_t Kp,
                             uint16_t* __restrict__ A)
{
    const uint32_t m = blockIdx.y;                   // node rows 2m, 2m + 1
    const uint32_t k2 = blockIdx.x * blockDim.x + threadIdx.x;
    if(2 * m >= rows || 2 * k2 >= cells) return;
    float2 a0, a1, b0, b1;                           // rows 2m, 2m + 1 at grid bearings 2 k2, 2 k2 + 1
    pair_values(G, m, 2 * k2, pitch, a0, b0);
    pair_values(G, m, 2 * k2 + 1, pitch, a1, b1);
    split_store(A + (size_t)(2 * m) * Kp + 2 * k2, cells, a0, a1);
    if(2 * m + 1 < rows) split_store(A + (size_t)(2 * m + 1) * Kp + 2 * k2, cells, b0, b1);
}

// FP16 per-row-scaled split: grid row r is scaled by 2^(14 - e), e =
// floor(log2(max |component|)), so that its largest component lies in
// [2^14, 2^15), then split into fp16 [hi | hi | lo] (lo = x - hi, so hi + lo
// carries 22 significant bits); row_scale[r] = 2^(e - 14) undoes the scaling
// exactly in the GEMM epilogue. One CTA per pair of node rows: both rows'
// maxima, then the split.
__device__ __forceinline__ int scale_exponent(uint32_t maxbits)
{
    if(maxbits == 0u) return 0;                       // zero row: scale 1
    const int e = (int)((maxbits >> 23) & 0xffu) - 127;
    return min(max(14 - e, -126), 127);
}

constexpr int kSplitF16Threads = 256;

__global__ void __launch_bounds__(kSplitF16Threads)
k_prec_split_f16(const float4* __restrict__ G, uint32_t rows, uint32_t cells, uint32_t pitch, uint32_t Kp,
                 uint16_t* __restrict__ A, float* __restrict__ row_scale)
{
    __shared__ float s_max[2][kSplitF16Threads / 32];
    const uint32_t m = blockIdx.x;                   // node rows 2m, 2m + 1
    if(2 * m >= rows) return;
    const bool second = 2 * m + 1 < rows;
    float mx0 = 0.0f, mx1 = 0.0f;
    for(uint32_t k = threadIdx.x; k < cells; k += blockDim.x) {
        float2 v0, v1;
        pair_values(G, m, k, pitch, v0, v1);
        mx0 = fmaxf(mx0, fmaxf(fabsf(v0.x), fabsf(v0.y)));
        mx1 = fmaxf(mx1, fmaxf(fabsf(v1.x), fabsf(v1.y)));
    }
    for(int o = 16; o > 0; o >>= 1) {
        mx0 = fmaxf(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
        mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
    }
    if((threadIdx.x & 31) == 0) { s_max[0][threadIdx.x >> 5] = mx0; s_max[1][threadIdx.x >> 5] = mx1; }
    __syncthreads();
    mx0 = 0.0f; mx1 = 0.0f;
    for(int w = 0; w < kSplitF16Threads / 32; w++) { mx0 = fmaxf(mx0, s_max[0][w]); mx1 = fmaxf(mx1, s_max[1][w]); }
    const int se0 = scale_exponent(__float_as_uint(mx0)), se1 = scale_exponent(__float_as_uint(mx1));
    const float sc0 = __uint_as_float((uint32_t)(se0 + 127) << 23), sc1 = __uint_as_float((uint32_t)(se1 + 127) << 23);
    if(threadIdx.x == 0) {
        row_scale[2 * m] = __uint_as_float((uint32_t)(127 - se0) << 23);
        if(second) row_scale[2 * m + 1] = __uint_as_float((uint32_t)(127 - se1) << 23);
    }
    auto store = [&](uint16_t* row, uint32_t k, float2 v, float sc) {
        const float xr = v.x * sc, xi = v.y * sc;
        const __half hr = __float2half_rn(xr), hi = __float2half_rn(xi);
        const __half lr = __float2half_rn(xr - __half2float(hr)), li = __float2half_rn(xi - __half2float(hi));
        row[k] = __half_as_ushort(hr);             row[cells + k] = __half_as_ushort(hi);
        row[2 * cells + k] = __half_as_ushort(hr); row[3 * cells + k] = __half_as_ushort(hi);
        row[4 * cells + k] = __half_as_ushort(lr); row[5 * cells + k] = __half_as_ushort(li);
    };
    uint16_t* row0 = A + (size_t)(2 * m) * Kp;
    uint16_t* row1 = row0 + Kp;
    for(uint32_t k = threadIdx.x; k < cells; k += blockDim.x) {
        float2 v0, v1;
        pair_values(G, m, k, pitch, v0, v1);
        store(row0, k, v0, sc0);
        if(second) store(row1, k, v1, sc1);
    }
}

constexpr int kFiltRows = 64, kFiltCols = 64, kFiltTapsMax = 64, kFiltThreads = 512;

size_t filter_smem_bytes(uint32_t ntaps)
{
    const size_t nt = std::min<uint32_t>(std::max<uint32_t>(ntaps, 1u), (uint32_t)kFiltTapsMax);
    return (kFiltRows + nt - 1) * kFiltCols * sizeof(float2) + 2 * kFiltTapsMax * sizeof(float2) +
           2 * kFiltRows * sizeof(int);
}

// Range filter on the contracted grid: out(r, b) = sum_t taps[r % 2][t]
// C[r / 2 + t + 1][b] (C row j holds range node j - tap_center - 1), or 0
// when row r's reference window is empty. One CTA per 64 node rows x 64
// bearings, both output-row parities (warps 0-7 the even rows 2 m, warps
// 8-15 the odd rows 2 m + 1, from the same staged node rows). Per chunk of
// up to 64 taps the C rows it needs are staged in shared memory once,
// row-major: every warp first loads all of its rows (up to 8, two 256-byte
// row segments each, the GEMM's K partials added) and only then stores
// them, so the loads are in flight together. Lane l owns columns l and
// l + 32; each warp filters 8 node rows of its parity with a sliding window
// of eight staged rows per column in registers (one shared load per tap and
// column).
constexpr int kFiltWarps = kFiltThreads / 32;
constexpr int kFiltRowsPerWarp = (kFiltRows + kFiltTapsMax - 1 + kFiltWarps - 1) / kFiltWarps;

template <int kParts>
__global__ void __launch_bounds__(kFiltThreads, 1)
k_prec_filter(const float2* __restrict__ C, uint32_t ldc2, uint32_t c_rows, size_t part2,
              const uint32_t* __restrict__ nonempty, int ov, const float2* __restrict__ taps, uint32_t ntaps,
              uint32_t nR, uint32_t nB, float2* __restrict__ out)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int ntc = min((int)max(ntaps, 1u), kFiltTapsMax);
    float2* sG = reinterpret_cast<float2*>(s_raw);                    // [kFiltRows + ntc - 1][kFiltCols]
    float2* sT = sG + (size_t)(kFiltRows + ntc - 1) * kFiltCols;       // [2][kFiltTapsMax]
    int* sW = reinterpret_cast<int*>(sT + 2 * kFiltTapsMax);            // [2][kFiltRows]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int par = warp >> 3, wl = warp & 7;                           // parity, warp within it
    const int r0 = blockIdx.y * kFiltRows, k0 = blockIdx.x * kFiltCols;
    if(tid < 2 * kFiltRows) {
        const int p = tid / kFiltRows, m = tid % kFiltRows;
        const int r = 2 * (r0 + m) + p;
        sW[tid] = r < (int)nR ? (row_has_window(nonempty, nR, ov, r) ? 1 : 0) : 0;
    }
    float2 acc[8][2];
#pragma unroll
    for(int q = 0; q < 8; q++) { acc[q][0] = make_float2(0.f, 0.f); acc[q][1] = make_float2(0.f, 0.f); }

    for(int tc = 0; tc < (int)ntaps; tc += ntc) {
        const int nt = min(ntc, (int)ntaps - tc);
        const int rows_s = kFiltRows + nt - 1;
        __syncthreads();
        if(tid < 2 * nt) sT[(tid / nt) * kFiltTapsMax + tid % nt] = taps[(size_t)(tid / nt) * ntaps + tc + tid % nt];
        float2 v[kFiltRowsPerWarp][2];
#pragma unroll
        for(int i = 0; i < kFiltRowsPerWarp; i++) {
            const int rr = warp + kFiltWarps * i;
            const uint32_t j = (uint32_t)(r0 + tc + rr + 1);        // C row of staged row rr
            const bool live = rr < rows_s && j < c_rows;
            const float2* row = C + (size_t)(live ? j : 0) * ldc2;
#pragma unroll
            for(int h = 0; h < 2; h++) {
                const int k = k0 + 32 * h + lane;
                float2 x = make_float2(0.f, 0.f);
                if(live && k < (int)nB) {
                    float2 y[kParts];
#pragma unroll
                    for(int z = 0; z < kParts; z++) y[z] = __ldg(row + (size_t)z * part2 + k);
#pragma unroll
                    for(int z = 0; z < kParts; z++) { x.x += y[z].x; x.y += y[z].y; }
                }
                v[i][h] = x;
            }
        }
#pragma unroll
        for(int i = 0; i < kFiltRowsPerWarp; i++) {
            const int rr = warp + kFiltWarps * i;
            if(rr < rows_s) {
                sG[rr * kFiltCols + lane] = v[i][0];
                sG[rr * kFiltCols + 32 + lane] = v[i][1];
            }
        }
        __syncthreads();
        const float2* tp = sT + par * kFiltTapsMax;
#pragma unroll
        for(int h = 0; h < 2; h++) {
            const float2* col = sG + h * 32 + lane + wl * 8 * kFiltCols;
            float2 g[8];
#pragma unroll
            for(int i = 0; i < 7; i++) g[i] = col[i * kFiltCols];
            // Blocks of eight taps with the window rotated at compile time: at
            // step i of a block, staged row tt + i + q sits in slot (q + i) & 7
            // and the new row goes to the slot of the row just dropped; after
            // eight steps the window is back in order.
            int tt = 0;
            for(; tt + 8 <= nt; tt += 8) {
#pragma unroll
                for(int i = 0; i < 8; i++) {
                    g[(i + 7) & 7] = col[(tt + i + 7) * kFiltCols];
                    const float2 c = tp[tt + i];
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
                const float2 c = tp[tt];
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
#pragma unroll
    for(int q = 0; q < 8; q++) {
        const int r = 2 * (r0 + wl * 8 + q) + par;
        if(r >= (int)nR) continue;
        const bool on = sW[par * kFiltRows + wl * 8 + q] != 0;
#pragma unroll
        for(int h = 0; h < 2; h++) {
            const int k = k0 + 32 * h + lane;
            if(k < (int)nB) out[(size_t)r * nB + k] = on ? acc[q][h] : make_float2(0.f, 0.f);
        }
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


// Derived directivity of the binned model: for each output bearing b, the
// least-squares (L2) projection of its response beam(theta - theta_b) (the
// texture-equivalent lerp of the beam table) onto the hat functions of the
// bearing grid g: the coefficients whose linear interpolation between grid
// bearings is closest in mean square to the per-sample response. The Gram
// system of the hat functions is tridiagonal (h_q / 6 off the diagonal,
// (h_q-1 + h_q) / 3 on it); its right-hand side integrates hat x beam over
// every grid interval, split at the beam table's knots, with the three-point
// Gauss-Legendre rule (exact for these quadratic pieces). Output D[q][b]
// (double, cells x nB).
void project_directivity(const std::vector<float>& g, const std::vector<float>& bearings, const std::vector<float>& beam,
                         float span, std::vector<double>& D)
{
    const size_t cells = g.size(), nB = bearings.size();
    const int W = (int)beam.size();
    const double kx = (double)(1.0f / span) * W, cx = 0.5 * W - 0.5;
    const double gx[3] = {-std::sqrt(0.6), 0.0, std::sqrt(0.6)}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    D.assign(cells * nB, 0.0);
    std::vector<double> f(cells), cp(cells), dp(cells), h(cells - 1);
    for(size_t q = 0; q + 1 < cells; q++) h[q] = (double)g[q + 1] - (double)g[q];
    for(size_t b = 0; b < nB; b++) {
        const double tb = bearings[b];
        std::fill(f.begin(), f.end(), 0.0);
        for(size_t q = 0; q + 1 < cells; q++) {
            const double g0 = g[q], g1 = g[q + 1];
            const double xa = (g0 - tb) * kx + cx, xb = (g1 - tb) * kx + cx;
            const double k0 = std::floor(xa) + 1.0;
            for(int m = 0;; m++) {
                const double lo = m == 0 ? xa : std::min(k0 + (m - 1), xb);
                const double hi = std::min(k0 + m, xb);
                if(!(lo < xb)) break;
                const double half = 0.5 * (hi - lo), mid = 0.5 * (hi + lo);
                if(!(half > 0.0)) continue;
                for(int i = 0; i < 3; i++) {
                    const double x = mid + half * gx[i];
                    const double th = tb + (x - cx) / kx;
                    const double wq = gw[i] * half / kx * host_lerp(beam.data(), W, 1, 0, x);
                    f[q] += wq * (g1 - th) / h[q];
                    f[q + 1] += wq * (th - g0) / h[q];
                }
            }
        }
        // Thomas algorithm on the tridiagonal Gram system.
        for(size_t q = 0; q < cells; q++) {
            const double sub = q > 0 ? h[q - 1] / 6.0 : 0.0;
            const double sup = q + 1 < cells ? h[q] / 6.0 : 0.0;
            const double diag = ((q > 0 ? h[q - 1] : 0.0) + (q + 1 < cells ? h[q] : 0.0)) / 3.0;
            const double den = diag - (q > 0 ? sub * cp[q - 1] : 0.0);
            cp[q] = sup / den;
            dp[q] = (f[q] - (q > 0 ? sub * dp[q - 1] : 0.0)) / den;
        }
        for(size_t q = cells; q-- > 0;) {
            const double x = dp[q] - (q + 1 < cells ? cp[q] * D[(q + 1) * nB + b] : 0.0);
            D[q * nB + b] = x;
        }
    }
}

// Range nodes of the binned model's output rows: one node every two output
// bins (node m at range_min + m * 2 * resolution; output row r uses node
// r / 2 and the taps of its parity r % 2).
uint32_t range_nodes(uint32_t nR) { return ((nR - 1u) >> 1) + 1u; }

// Derived range taps: for output row r = 2 m + p the pulse response
// P(x - R_r), seen from node m, is P(x - p res); its least-squares (L2)
// projection onto the hat functions of the nodes (spacing h = 2 res) gives
// taps[p][t], the weight of node m + t - center. P is the texture-equivalent
// lerp of the pulse table (border addressing; coordinate y ky + cy). Each
// right-hand side integrates hat x P over the two halves of the hat, split
// at the pulse table's knots, with the three-point Gauss-Legendre rule
// (exact for these linear x linear pieces); the Gram system of the uniform
// hats (h / 6, 2 h / 3, h / 6) is solved (Thomas) on the nodes the pulse
// reaches widened by kTapPad + kSolvePad on each side, and the nodes widened
// by kTapPad are kept. Output: taps complex [2][L] as float pairs.
constexpr int kTapPad = 6, kSolvePad = 10;

void project_range_taps(const std::vector<float>& pulse, uint32_t H, float res_f, float pscale,
                        std::vector<float>& taps, uint32_t& center)
{
    const double res = res_f, hr = (double)(2.0f * res_f);
    const double ky = (double)pscale * H, cy = 0.5 * H - 0.5;
    const double y_lo = (-1.0 - cy) / ky, y_hi = (H - cy) / ky;
    const int dmin = (int)std::floor(y_lo / hr) - 1;
    const int dmax = (int)std::ceil((y_hi + res) / hr) + 1;
    const int s0 = dmin - kTapPad - kSolvePad, s1 = dmax + kTapPad + kSolvePad;
    const int ns = s1 - s0 + 1, L = dmax - dmin + 1 + 2 * kTapPad;
    const double gx[3] = {-std::sqrt(0.6), 0.0, std::sqrt(0.6)}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    taps.assign((size_t)4 * L, 0.0f);
    std::vector<double> fr(ns), fi(ns), cp(ns), dr(ns), di(ns), xr(ns), xi(ns);
    for(int p = 0; p < 2; p++) {
        const double off = p * res;
        for(int i = 0; i < ns; i++) {
            const int dd = s0 + i;
            double sr = 0.0, si = 0.0;
            for(int half_i = 0; half_i < 2; half_i++) {
                const double a = (dd - 1 + half_i) * hr, b = (dd + half_i) * hr;
                std::vector<double> pts{a};
                const long long k_lo = (long long)std::ceil((a - off) * ky + cy), k_hi = (long long)std::floor((b - off) * ky + cy);
                for(long long k = k_lo; k <= k_hi; k++) {
                    const double x = off + ((double)k - cy) / ky;
                    if(x >= a && x <= b) pts.push_back(x);
                }
                pts.push_back(b);
                std::sort(pts.begin(), pts.end());
                for(size_t e = 0; e + 1 < pts.size(); e++) {
                    const double half = 0.5 * (pts[e + 1] - pts[e]), mid = 0.5 * (pts[e + 1] + pts[e]);
                    if(!(half > 0.0)) continue;
                    for(int g = 0; g < 3; g++) {
                        const double x = mid + half * gx[g];
                        const double xt = (x - off) * ky + cy;
                        const double lam = half_i == 0 ? (x - a) / hr : (b - x) / hr;
                        const double wq = gw[g] * half * lam;
                        sr += wq * host_lerp(pulse.data(), (int)H, 2, 0, xt);
                        si += wq * host_lerp(pulse.data(), (int)H, 2, 1, xt);
                    }
                }
            }
            fr[i] = sr; fi[i] = si;
        }
        // Thomas algorithm: sub = sup = h / 6, diag = 2 h / 3 on every row.
        const double sub = hr / 6.0, diag = 2.0 * hr / 3.0;
        for(int i = 0; i < ns; i++) {
            const double den = diag - (i > 0 ? sub * cp[i - 1] : 0.0);
            cp[i] = sub / den;
            dr[i] = (fr[i] - (i > 0 ? sub * dr[i - 1] : 0.0)) / den;
            di[i] = (fi[i] - (i > 0 ? sub * di[i - 1] : 0.0)) / den;
        }
        for(int i = ns; i-- > 0;) {
            xr[i] = dr[i] - (i + 1 < ns ? cp[i] * xr[i + 1] : 0.0);
            xi[i] = di[i] - (i + 1 < ns ? cp[i] * xi[i + 1] : 0.0);
        }
        for(int t = 0; t < L; t++) {
            const int i = (dmin - kTapPad + t) - s0;
            taps[((size_t)p * L + t) * 2] = (float)xr[i];
            taps[((size_t)p * L + t) * 2 + 1] = (float)xi[i];
        }
    }
    center = (uint32_t)(kTapPad - dmin);
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
    free_dev(c.d_C); free_dev(c.d_taps);
    free_dev(c.d_row_scale); free_dev(c.d_col_scale);
    free_dev(c.d_hot); free_dev(c.d_hotcnt); free_dev(c.d_rep);
    c.prec_f16 = false;
    c.prec_hot = false;
    c.prec_configured = false;
}

// Default grid size: four grid bearings per output bearing, rounded up to a
// multiple of 32.
uint32_t default_grid_cells(uint32_t nB) { return (4u * nB + 31u) / 32u * 32u; }

rtacx_status configure_precision(Context& ctx, const rtacx_precision_desc* d)
{
    if(!ctx.configured || ctx.dims != 2) { ctx.error = "the precision form needs a configured 2D sensor"; return RTACX_ERR_NOT_CONFIGURED; }
    if(!d) { ctx.error = "null precision descriptor"; return RTACX_ERR_INVALID_ARGUMENT; }
    const uint32_t nB = ctx.nB, nR = ctx.nR;
    if(nB > (uint32_t)kMaxBearingsSmem) { ctx.error = "too many bearings for the precision form"; return RTACX_ERR_UNSUPPORTED; }
    if(nR < 2) { ctx.error = "the precision form needs at least two range bins"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(nR > (uint32_t)kMaxRangeWords * 32) { ctx.error = "too many range bins for the precision form"; return RTACX_ERR_UNSUPPORTED; }
    if(d->flags & ~(RTACX_PRECISION_FP16_ROWSCALE | RTACX_PRECISION_HOT_RANGE)) {
        ctx.error = "unknown precision flags";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    // Bearing grid.
    const uint32_t cells = d->grid_count ? d->grid_count : default_grid_cells(nB);
    if(cells < 2 || (cells & 1u)) { ctx.error = "grid_count must be even and at least 2"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(cells > kMaxGridCells) { ctx.error = "grid_count above 16384"; return RTACX_ERR_UNSUPPORTED; }
    float first = d->grid_first, last = d->grid_last;
    if(first == last) {
        first = *std::min_element(ctx.bearings.begin(), ctx.bearings.end());
        last = *std::max_element(ctx.bearings.begin(), ctx.bearings.end());
    }
    if(!(std::isfinite(first) && std::isfinite(last) && last > first)) {
        ctx.error = "the bearing grid needs finite grid_first < grid_last";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    const float step = (last - first) / (float)(cells - 1u);
    if(!(step > 0.0f) || !std::isfinite(1.0f / step)) { ctx.error = "degenerate bearing grid"; return RTACX_ERR_INVALID_ARGUMENT; }
    free_precision(ctx);

    // Range taps (two phases: even and odd output rows), given or projected
    // from the pulse table.
    std::vector<float> taps;
    uint32_t center;
    if(d->range_taps) {
        if(d->tap_count == 0 || d->tap_center >= d->tap_count) { ctx.error = "bad tap_count / tap_center"; return RTACX_ERR_INVALID_ARGUMENT; }
        if(d->tap_count > 1024) { ctx.error = "tap_count above 1024"; return RTACX_ERR_UNSUPPORTED; }
        taps.assign(d->range_taps, d->range_taps + 4 * (size_t)d->tap_count);
        center = d->tap_center;
    }
    else {
        project_range_taps(ctx.pulse, ctx.H, (ctx.rmax - ctx.rmin) / (float)(nR - 1u),
                           host_pulse_scale(ctx.duration, ctx.c, false), taps, center);
    }
    for(float v : taps) if(!std::isfinite(v)) { ctx.error = "non-finite range taps"; return RTACX_ERR_INVALID_ARGUMENT; }
    const uint32_t ntaps = (uint32_t)(taps.size() / 4);
    ctx.taps = ntaps;
    ctx.tap_center = center;

    // Grid parameters (the oracle computes the same floats).
    GridParams& g = ctx.grid;
    const uint32_t nodes = range_nodes(nR);
    g.rmin = ctx.rmin;
    g.res = 2.0f * ((ctx.rmax - ctx.rmin) / (float)(nR - 1u));
    g.inv_res = 1.0f / g.res;
    g.first = first;
    g.step = step;
    g.inv_step = 1.0f / step;
    g.cells = cells;
    g.pitch = cells + kRowPad;
    g.row_lo = -(int)center - 1;
    g.row_hi = (int)nodes + (int)ntaps - (int)center - 2;
    g.row_shift = (int)center + 1;
    if(!(g.res > 0.0f) || !std::isfinite(g.inv_res)) { ctx.error = "degenerate range axis"; return RTACX_ERR_INVALID_ARGUMENT; }
    ctx.grid_rows = nodes + ntaps + 1;

    // Directivity D[q][b] (complex), given or projected from the beam table.
    std::vector<float> D((size_t)cells * nB * 2, 0.0f);
    if(d->directivity) {
        std::memcpy(D.data(), d->directivity, D.size() * sizeof(float));
    }
    else {
        std::vector<float> gp(cells);
        for(uint32_t q = 0; q < cells; q++) gp[q] = first + (float)q * step;
        std::vector<double> Dd;
        project_directivity(gp, ctx.bearings, ctx.beam, ctx.span, Dd);
        for(size_t e = 0; e < Dd.size(); e++) D[2 * e] = (float)Dd[e];
    }
    for(float v : D) if(!std::isfinite(v)) { ctx.error = "non-finite directivity"; return RTACX_ERR_INVALID_ARGUMENT; }

    ctx.acc_smem = accumulate_smem_bytes(nR);
    int acc_blocks = 0;
    if(raise_smem_limit((const void*)k_prec_accumulate, ctx.acc_smem) != cudaSuccess ||
       cudaOccupancyMaxActiveBlocksPerMultiprocessor(&acc_blocks, k_prec_accumulate, kAccThreads, ctx.acc_smem) !=
           cudaSuccess ||
       acc_blocks < 1) {
        cudaGetLastError();
        ctx.error = "cannot reserve shared memory for the accumulation";
        return RTACX_ERR_CUDA;
    }
    ctx.acc_blocks_per_sm = (uint32_t)acc_blocks;
    ctx.acc_staged_smem = staged_smem_bytes(nR);
    for(int m = 0; m < kAccEchoModels; m++) {
        const void* fs = accumulate_staged_kernel(m);
        int bs = 0;
        if(raise_smem_limit(fs, ctx.acc_staged_smem) != cudaSuccess ||
           cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bs, fs, kStagedThreads, ctx.acc_staged_smem) != cudaSuccess)
            bs = 0;
        cudaGetLastError();
        ctx.acc_staged_blocks[m] = (uint32_t)std::max(bs, 0);
    }
    if(raise_smem_limit((const void*)k_prec_filter<1>, filter_smem_bytes(kFiltTapsMax)) != cudaSuccess ||
       raise_smem_limit((const void*)k_prec_filter<2>, filter_smem_bytes(kFiltTapsMax)) != cudaSuccess) {
        ctx.error = "cannot reserve shared memory for the range filter";
        return RTACX_ERR_CUDA;
    }

    // GEMM operand shapes: M = grid rows, N = 2 nB (re / im of each bearing),
    // K = 6 cells (the three split products of [Re | Im] grid values).
    ctx.Mpad = (ctx.grid_rows + 127) / 128 * 128;
    ctx.Npad = (2 * nB + 255) / 256 * 256;
    ctx.Kp = (6 * cells + 63) / 64 * 64;
    // Split K in two when the 128 x 256 output tiles cover at most half of
    // the SMs (the node grid of a 4096-range ping: 68 tiles on 152 SMs): twice
    // the CTAs, each over half of K; the range filter adds the two partials.
    ctx.ksplit = ((uint64_t)(ctx.Npad / 256) * (ctx.Mpad / 128) * 2 <= (uint64_t)ctx.sm_count &&
                  (ctx.Kp / 64) % 2 == 0) ? 2u : 1u;

    // B operand: row n = 2b (real) / 2b + 1 (imag); K blocks [hi | lo | hi]
    // of [real part of G | imaginary part of G]. FP16 form: each row n is
    // first scaled by 2^(14 - e_n) (largest |value| in [2^14, 2^15)) and
    // col_scale[n] = 2^(e_n - 14) undoes it in the GEMM epilogue.
    const bool f16 = (d->flags & RTACX_PRECISION_FP16_ROWSCALE) != 0;
    const bool hot = (d->flags & RTACX_PRECISION_HOT_RANGE) != 0;
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
                for(uint32_t k = 0; k < cells; k++) mx = std::max(mx, std::max(std::fabs(value(k, 0)), std::fabs(value(k, 1))));
                if(mx > 0.0f) {
                    const int se = std::min(std::max(14 - std::ilogb(mx), -126), 127);
                    scale = std::ldexp(1.0f, se);
                    col_scale[2 * b + o] = std::ldexp(1.0f, -se);
                }
            }
            uint16_t* row = B.data() + (size_t)(2 * b + o) * ctx.Kp;
            for(uint32_t k = 0; k < cells; k++)
                for(int h = 0; h < 2; h++) {
                    const float v = value(k, h) * scale;
                    uint16_t bh, bl;
                    if(f16) { bh = host_f16_bits(v); bl = host_f16_bits(v - host_f16_value(bh)); }
                    else { bh = host_bf16_bits(v); bl = host_bf16_bits(v - host_bf16_value(bh)); }
                    row[h * cells + k] = bh;
                    row[2 * cells + h * cells + k] = bl;
                    row[4 * cells + h * cells + k] = bh;
                }
        }

    auto alloc = [&](auto*& p, size_t bytes) {
        if(cudaMalloc(&p, bytes) != cudaSuccess) { cudaGetLastError(); p = nullptr; return false; }
        return true;
    };
    const size_t grid_bytes = grid_quads(ctx.grid_rows, g.pitch) * sizeof(float4);
    if(!alloc(ctx.d_G, grid_bytes) || !alloc(ctx.d_flags, (size_t)(nR + 31) / 32 * 4) ||
       !alloc(ctx.d_A, (size_t)ctx.Mpad * ctx.Kp * 2) || !alloc(ctx.d_B, B.size() * 2) ||
       !alloc(ctx.d_taps, taps.size() * sizeof(float)) || !alloc(ctx.d_C, (size_t)ctx.ksplit * ctx.Mpad * ctx.Npad * sizeof(float)) ||
       (f16 && (!alloc(ctx.d_row_scale, (size_t)ctx.Mpad * sizeof(float)) ||
                !alloc(ctx.d_col_scale, (size_t)ctx.Npad * sizeof(float)))) ||
       (hot && (!alloc(ctx.d_hot, sizeof(int2)) || !alloc(ctx.d_hotcnt, (size_t)ctx.grid_rows * 4) ||
                !alloc(ctx.d_rep, (size_t)kHotRows * kHotReplicas * g.pitch * sizeof(float4))))) {
        free_precision(ctx);
        ctx.error = "out of device memory for the precision form";
        return RTACX_ERR_OUT_OF_MEMORY;
    }
    if(cudaMemset(ctx.d_A, 0, (size_t)ctx.Mpad * ctx.Kp * 2) != cudaSuccess ||
       cudaMemcpy(ctx.d_B, B.data(), B.size() * 2, cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaMemcpy(ctx.d_taps, taps.data(), taps.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
       (f16 && (cudaMemcpy(ctx.d_col_scale, col_scale.data(), col_scale.size() * sizeof(float),
                           cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemset(ctx.d_row_scale, 0, (size_t)ctx.Mpad * sizeof(float)) != cudaSuccess)) ||
       (hot && (cudaMemset(ctx.d_hot, 0, sizeof(int2)) != cudaSuccess ||
                cudaMemset(ctx.d_hotcnt, 0, (size_t)ctx.grid_rows * 4) != cudaSuccess))) {
        cudaGetLastError();
        free_precision(ctx);
        ctx.error = "uploading the precision tables failed";
        return RTACX_ERR_CUDA;
    }
    if(gemm_smem_bytes() > 227 * 1024) { ctx.error = "GEMM tile exceeds shared memory"; return RTACX_ERR_UNSUPPORTED; }
    if(hot && raise_smem_limit((const void*)k_hot_pick, (ctx.grid_rows + 1) * sizeof(uint32_t)) != cudaSuccess) {
        free_precision(ctx);
        ctx.error = "cannot reserve shared memory for the hot-range scan";
        return RTACX_ERR_CUDA;
    }
    ctx.prec_f16 = f16;
    ctx.prec_hot = hot;
    ctx.prec_configured = true;
    return RTACX_OK;
}

// Zeroes the grid and the non-empty bitmap of a new ping.
rtacx_status precision_begin(Context& ctx, cudaStream_t stream)
{
    const uint64_t quads = grid_quads(ctx.grid_rows, ctx.grid.pitch);
    const uint32_t blocks = (uint32_t)std::min<uint64_t>((quads + 255) / 256, (uint64_t)ctx.sm_count * 32);
    k_prec_clear<<<blocks, 256, 0, stream>>>(ctx.d_G, quads, ctx.d_flags, (ctx.nR + 31) / 32);
    RTACX_CUDA(cudaGetLastError());
    return RTACX_OK;
}

// Adds n samples to the ping's grid (order-independent, so a ping may be
// accumulated in any number of chunks).
rtacx_status precision_accumulate(Context& ctx, const void* samples, uint64_t n, cudaStream_t stream)
{
    if(!n) return RTACX_OK;
    const uint64_t want = (n + kAccThreads * kAccLoads - 1) / (kAccThreads * kAccLoads);
    if(!ctx.prec_hot && ctx.bin.vec4 && (reinterpret_cast<uintptr_t>(samples) & 15u) == 0) {
        const int m = accumulate_echo_model(ctx.bin.echo_flags);
        if(ctx.acc_staged_blocks[m] > 0) {
            const uint64_t stages = (n + kStageRecs - 1) / kStageRecs;
            const uint32_t blocks = (uint32_t)std::min<uint64_t>(stages, (uint64_t)ctx.sm_count * ctx.acc_staged_blocks[m]);
            void* args[] = {(void*)&samples, (void*)&n, (void*)&ctx.bin, (void*)&ctx.grid, (void*)&ctx.d_G,
                            (void*)&ctx.d_flags, (void*)&ctx.d_err, (void*)&ctx.diag_drop_stage};
            RTACX_CUDA(cudaLaunchKernel(accumulate_staged_kernel(m), dim3(blocks), dim3(kStagedThreads), args,
                                        ctx.acc_staged_smem, stream));
            return RTACX_OK;
        }
    }
    const uint32_t blocks = (uint32_t)std::min<uint64_t>(want, (uint64_t)ctx.sm_count * ctx.acc_blocks_per_sm);
    k_prec_accumulate<<<blocks, kAccThreads, ctx.acc_smem, stream>>>(static_cast<const float*>(samples), n, ctx.bin,
                                                                     ctx.grid, ctx.d_G, ctx.d_flags,
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
        k_hot_count<<<blocks, 256, 0, stream>>>(static_cast<const float*>(samples), n, ctx.bin, ctx.grid, step,
                                                ctx.d_hotcnt);
        RTACX_CUDA(cudaGetLastError());
    }
    k_hot_pick<<<1, kHotPickThreads, (ctx.grid_rows + 1) * sizeof(uint32_t), stream>>>(ctx.d_hotcnt, ctx.grid_rows,
                                                                                        ctx.d_hot);
    RTACX_CUDA(cudaGetLastError());
    k_hot_zero<<<ctx.sm_count * 4, 256, 0, stream>>>(ctx.d_hot, ctx.grid.pitch, ctx.d_rep);
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

// Operand split, tensor-core contraction, range filter into `out`.
rtacx_status precision_finish(Context& ctx, float* out, cudaStream_t stream)
{
    const uint32_t nR = ctx.nR, nB = ctx.nB, cells = ctx.grid.cells;
    if(ctx.prec_hot) {
        k_hot_fold<<<ctx.sm_count * 4, 256, 0, stream>>>(ctx.d_hot, ctx.grid.pitch, ctx.d_rep, ctx.d_G);
        RTACX_CUDA(cudaGetLastError());
    }
    ctx.mark(1, false, stream);
    if(!ctx.prec_f16) {
        const dim3 sgrid((cells / 2 + 255) / 256, (ctx.grid_rows + 1) / 2);
        k_prec_split<<<sgrid, 256, 0, stream>>>(ctx.d_G, ctx.grid_rows, cells, ctx.grid.pitch, ctx.Kp, ctx.d_A);
    }
    else {
        k_prec_split_f16<<<(ctx.grid_rows + 1) / 2, kSplitF16Threads, 0, stream>>>(ctx.d_G, ctx.grid_rows, cells, ctx.grid.pitch,
                                                                         ctx.Kp, ctx.d_A, ctx.d_row_scale);
    }
    RTACX_CUDA(cudaGetLastError());
    ctx.mark(1, true, stream);
    ctx.mark(3, false, stream);
    rtacx_status st = gemm_tn(ctx.error, ctx.d_A, ctx.d_B, ctx.d_C, (int)ctx.Mpad, (int)ctx.Npad, (int)ctx.Kp,
                              (int)ctx.Npad, stream, ctx.d_err, ctx.prec_f16, ctx.prec_f16 ? ctx.d_row_scale : nullptr,
                              ctx.prec_f16 ? ctx.d_col_scale : nullptr, (int)ctx.ksplit);
    if(st != RTACX_OK) return st;
    ctx.mark(3, true, stream);
    ctx.mark(2, false, stream);
    const dim3 fgrid((nB + kFiltCols - 1) / kFiltCols, (range_nodes(nR) + kFiltRows - 1) / kFiltRows);
    auto filter = ctx.ksplit == 2 ? k_prec_filter<2> : k_prec_filter<1>;
    filter<<<fgrid, kFiltThreads, filter_smem_bytes(ctx.taps), stream>>>(
        reinterpret_cast<const float2*>(ctx.d_C), ctx.Npad / 2, ctx.grid_rows, (size_t)ctx.Mpad * ctx.Npad / 2,
        ctx.d_flags, ctx.overlap, ctx.d_taps, ctx.taps, nR, nB, reinterpret_cast<float2*>(out));
    RTACX_CUDA(cudaGetLastError());
    ctx.mark(2, true, stream);
    return RTACX_OK;
}

} // namespace rtacx
