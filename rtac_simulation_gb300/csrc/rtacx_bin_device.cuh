// Device-side building blocks of the counting sort (shared by the per-ping
// binning kernels and the fused batched kernel): the tiled pass over a chunk
// of samples, the count and scatter passes of one chunk, the block scan and
// the reference windows. Internal linkage: every translation unit that
// includes this header gets its own copy.
#pragma once

#include "rtacx_internal.cuh"

#include <climits>

namespace rtacx {

namespace {

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

constexpr int kTileLoads = 4;        // independent record loads per thread and tile

// Block-uniform pass over chunk `c` of `nc` equal chunks of the input in
// tiles of blockDim.x * kTileLoads samples: the loads of tile t + 1 are
// issued before tile t is processed, then the keys are computed and
// f(valid[], record[], key[], side[]) is called -- the same number of times
// in every thread, so f may synchronise the block.
template <typename F>
__device__ __forceinline__ void for_chunk(const float* samples, uint64_t n, const BinParams& p,
                                          uint32_t c, uint32_t nc, F&& f)
{
    const uint64_t chunk = (n + nc - 1) / nc;
    const uint64_t begin = (uint64_t)c * chunk;
    const uint64_t end = min(begin + chunk, n);
    const uint64_t tile = (uint64_t)blockDim.x * kTileLoads;
    float4 next[kTileLoads];
    auto load_tile = [&](uint64_t t0) {
#pragma unroll
        for(int u = 0; u < kTileLoads; u++) {
            const uint64_t i = t0 + (uint64_t)u * blockDim.x + threadIdx.x;
            next[u] = i < end ? load_record(samples, i, p) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    if(begin < end) load_tile(begin);
    for(uint64_t t0 = begin; t0 < end; t0 += tile) {
        bool valid[kTileLoads];
        float4 rec[kTileLoads];
        uint32_t key[kTileLoads];
        int side[kTileLoads];
#pragma unroll
        for(int u = 0; u < kTileLoads; u++) {
            valid[u] = t0 + (uint64_t)u * blockDim.x + threadIdx.x < end;
            rec[u] = next[u];
        }
        if(t0 + tile < end) load_tile(t0 + tile);
#pragma unroll
        for(int u = 0; u < kTileLoads; u++) {
            key[u] = kOutOfRange;
            side[u] = 0;
            if(valid[u]) key[u] = sample_key(p, rec[u].z, rec[u].w, side[u]);
        }
        f(valid, rec, key, side);
    }
}

// Count pass of chunk c of nc (shared-memory histogram sh of p.nBins
// words), added into totals[0, nBins) (zeroed by the caller).
__device__ __forceinline__ void count_chunk(const float* __restrict__ samples, uint64_t n, const BinParams& p, uint32_t c,
                            uint32_t nc, uint32_t* __restrict__ totals, unsigned long long* __restrict__ oor,
                            uint32_t* sh, unsigned long long* s_oor)
{
    for(uint32_t b = threadIdx.x; b < p.nBins; b += blockDim.x) sh[b] = 0u;
    if(threadIdx.x < 2) s_oor[threadIdx.x] = 0ull;
    __syncthreads();

    uint32_t low = 0, high = 0;
    for_chunk(samples, n, p, c, nc, [&](const bool* valid, const float4*, const uint32_t* key, const int* side) {
#pragma unroll
        for(int u = 0; u < kTileLoads; u++) {
            if(valid[u] && key[u] != kOutOfRange) atomicAdd(&sh[key[u]], 1u);
            else if(valid[u]) {
                if(side[u] < 0) low++; else high++;
            }
        }
    });
    for(int o = 16; o > 0; o >>= 1) {
        low += __shfl_down_sync(0xffffffffu, low, o);
        high += __shfl_down_sync(0xffffffffu, high, o);
    }
    if(lane_id() == 0 && (low | high)) {
        atomicAdd(&s_oor[0], (unsigned long long)low);
        atomicAdd(&s_oor[1], (unsigned long long)high);
    }
    __syncthreads();
    if(threadIdx.x == 0) {
        if(s_oor[0]) atomicAdd(&oor[0], s_oor[0]);
        if(s_oor[1]) atomicAdd(&oor[1], s_oor[1]);
    }
    for(uint32_t b = threadIdx.x; b < p.nBins; b += blockDim.x)
        if(sh[b]) atomicAdd(&totals[b], sh[b]);
    // Per-block sums of kScanBlock bins (totals[nBins + blk]) for the
    // parallel bin scan: one warp per block of bins.
    const uint32_t blocks = (p.nBins + kScanBlock - 1) / kScanBlock;
    for(uint32_t blk = threadIdx.x >> 5; blk < blocks; blk += blockDim.x >> 5) {
        uint32_t s = 0;
        for(uint32_t b = blk * kScanBlock + lane_id(); b < min((blk + 1) * kScanBlock, p.nBins); b += 32) s += sh[b];
        for(int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if(lane_id() == 0 && s) atomicAdd(&totals[p.nBins + blk], s);
    }
}

// Exclusive block scan of one value per thread (any blockDim.x that is a
// multiple of 32, at most 1024).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t& total)
{
    const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t x = v;
    for(int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if(lane >= (unsigned)o) x += y;
    }
    if(lane == 31) s_warp[warp] = x;
    __syncthreads();
    const unsigned nw = blockDim.x >> 5;
    if(warp == 0) {
        uint32_t w = lane < nw ? s_warp[lane] : 0u;
        for(int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
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

// Scatter pass of chunk c of nc. Per tile: rank of each sample among the
// tile's samples of its bin (shared-memory histogram sh of p.nBins words,
// zero between tiles); the first sample of each (tile, bin) reserves the
// bin's run with one atomicAdd on the shared cursor and leaves the run's
// base in sh; every sample is written at base + rank.
__device__ __forceinline__ void scatter_chunk(const float* __restrict__ samples, uint64_t n, const BinParams& p, uint32_t c,
                              uint32_t nc, uint32_t* __restrict__ cursor, const uint32_t* __restrict__ offsets,
                              float4* __restrict__ sorted, uint32_t* __restrict__ err, uint32_t* sh)
{
    for(uint32_t b = threadIdx.x; b < p.nBins; b += blockDim.x) sh[b] = 0u;
    const uint32_t total = offsets[p.nBins];
    __syncthreads();

    for_chunk(samples, n, p, c, nc, [&](const bool* valid, const float4* rec, const uint32_t* key, const int*) {
        uint32_t rank[kTileLoads];
#pragma unroll
        for(int u = 0; u < kTileLoads; u++)
            rank[u] = (valid[u] && key[u] != kOutOfRange) ? atomicAdd(&sh[key[u]], 1u) : UINT_MAX;
        __syncthreads();
#pragma unroll
        for(int u = 0; u < kTileLoads; u++)
            if(rank[u] == 0u) sh[key[u]] = atomicAdd(&cursor[cursor_word(key[u])], sh[key[u]]);
        __syncthreads();
#pragma unroll
        for(int u = 0; u < kTileLoads; u++) {
            if(rank[u] == UINT_MAX) continue;
            const uint32_t pos = sh[key[u]] + rank[u];
            float4 out = rec[u];
            if(p.echo_flags) {
                const float2 v = apply_echo(p, make_float2(out.x, out.y), out.z);
                out.x = v.x; out.y = v.y;
            }
            if(pos < total) sorted[pos] = out;
            else atomicOr(err, kErrScatterOverflow);
        }
        __syncthreads();
#pragma unroll
        for(int u = 0; u < kTileLoads; u++)
            if(rank[u] == 0u) sh[key[u]] = 0u;
        __syncthreads();
    });
}

__device__ __forceinline__ uint32_t bin_count(const uint32_t* off, uint32_t nBB, int j)
{
    return off[(size_t)(j + 1) * nBB] - off[(size_t)j * nBB];
}

// First / last non-empty range bin of row r's reference window
// [max(0, r - ov), min(nR - 1, r + ov)]; returns false for the empty view
// (no non-empty bin, or istart >= iend: src/Binner.cu:90-102).
__device__ __forceinline__ bool ref_window(const uint32_t* off, uint32_t nBB, uint32_t nR, int ov, int r,
                                           int& f, int& l)
{
    const long long lo = max(0ll, (long long)r - ov);
    const long long hi = min((long long)nR - 1, (long long)r + ov);
    long long a = lo;
    while(a <= hi && bin_count(off, nBB, (int)a) == 0u) a++;
    if(a >= hi) return false;
    long long z = hi;
    while(z > a && bin_count(off, nBB, (int)z) == 0u) z--;
    if(a >= z) return false;
    f = (int)a; l = (int)z;
    return true;
}

// Effective window of output row r: the reference window's first / last
// non-empty bins intersected with the row's PSF support.
__device__ __forceinline__ void window_row(const uint32_t* __restrict__ off, uint32_t nBB, uint32_t nR, int ov,
                           const int2* __restrict__ support, int2* __restrict__ win, int r)
{
    if(r >= (int)nR) return;
    int f, l;
    int2 w = make_int2(1, 0);
    if(ref_window(off, nBB, nR, ov, r, f, l)) {
        const int2 s = support[r];
        w = make_int2(max(f, s.x), min(l, s.y));
    }
    win[r] = w;
}

// Exclusive scan of bins [blk kScanBlock, (blk + 1) kScanBlock) of
// totals[0, nBins), offset by the count of every bin before the block: the
// sum of the block sums before it (totals[nBins + j], j < blk, accumulated by
// the count pass) when block_sums, else the sum of totals[0, blk kScanBlock)
// taken by the whole CTA. Writes offsets (and offsets[nBins] from the block
// holding the last bin) and the scatter's per-bin cursors. Each thread scans
// kScanBlock / blockDim.x consecutive bins; blockDim.x divides kScanBlock.
__device__ __forceinline__ void scan_bin_block(const uint32_t* __restrict__ totals, uint32_t nBins, uint32_t blk,
                                               uint32_t* __restrict__ offsets, uint32_t* __restrict__ cursor,
                                               uint32_t* s_warp, uint32_t* s_prefix, bool block_sums = true)
{
    if(block_sums) {
        if(threadIdx.x < 32) {
            uint32_t s = 0;
            for(uint32_t j = threadIdx.x; j < blk; j += 32) s += totals[nBins + j];
            for(int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if(threadIdx.x == 0) *s_prefix = s;
        }
    }
    else {
        if(threadIdx.x == 0) *s_prefix = 0u;
        __syncthreads();
        uint32_t s = 0;
        for(uint32_t i = threadIdx.x; i < blk * kScanBlock; i += blockDim.x) s += totals[i];
        for(int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if(lane_id() == 0 && s) atomicAdd(s_prefix, s);
    }
    const uint32_t per = kScanBlock / blockDim.x;
    const uint32_t b0 = blk * kScanBlock + threadIdx.x * per;
    uint32_t sum = 0;
    for(uint32_t u = 0; u < per; u++) sum += b0 + u < nBins ? totals[b0 + u] : 0u;
    uint32_t blk_total;
    uint32_t o = block_exclusive_scan(sum, s_warp, blk_total);   // synchronises: s_prefix is visible
    o += *s_prefix;
    for(uint32_t u = 0; u < per; u++) {
        const uint32_t b = b0 + u;
        if(b >= nBins) break;
        const uint32_t v = totals[b];
        offsets[b] = o;
        cursor[cursor_word(b)] = o;
        o += v;
        if(b == nBins - 1) offsets[nBins] = o;
    }
}

// Count pass of chunk c of nc straight into totals[0, nBins) with one global
// atomic per sample (no shared histogram: the fused batched kernel keeps its
// shared memory for the gather). Out-of-range counts as count_chunk.
__device__ __forceinline__ void count_chunk_global(const float* __restrict__ samples, uint64_t n, const BinParams& p,
                                                   uint32_t c, uint32_t nc, uint32_t* __restrict__ totals,
                                                   unsigned long long* __restrict__ oor, unsigned long long* s_oor)
{
    if(threadIdx.x < 2) s_oor[threadIdx.x] = 0ull;
    __syncthreads();
    uint32_t low = 0, high = 0;
    for_chunk(samples, n, p, c, nc, [&](const bool* valid, const float4*, const uint32_t* key, const int* side) {
#pragma unroll
        for(int u = 0; u < kTileLoads; u++) {
            if(valid[u] && key[u] != kOutOfRange) atomicAdd(&totals[key[u]], 1u);
            else if(valid[u]) {
                if(side[u] < 0) low++; else high++;
            }
        }
    });
    for(int o = 16; o > 0; o >>= 1) {
        low += __shfl_down_sync(0xffffffffu, low, o);
        high += __shfl_down_sync(0xffffffffu, high, o);
    }
    if(lane_id() == 0 && (low | high)) {
        atomicAdd(&s_oor[0], (unsigned long long)low);
        atomicAdd(&s_oor[1], (unsigned long long)high);
    }
    __syncthreads();
    if(threadIdx.x == 0) {
        if(s_oor[0]) atomicAdd(&oor[0], s_oor[0]);
        if(s_oor[1]) atomicAdd(&oor[1], s_oor[1]);
    }
}

// Scatter pass of chunk c of nc with one global atomic per sample on its
// bin's cursor (no shared histogram); positions past the counted total set
// kErrScatterOverflow instead of being written.
__device__ __forceinline__ void scatter_chunk_global(const float* __restrict__ samples, uint64_t n, const BinParams& p,
                                                     uint32_t c, uint32_t nc, uint32_t* __restrict__ cursor,
                                                     const uint32_t* __restrict__ offsets, float4* __restrict__ sorted,
                                                     uint32_t* __restrict__ err)
{
    const uint32_t total = offsets[p.nBins];
    for_chunk(samples, n, p, c, nc, [&](const bool* valid, const float4* rec, const uint32_t* key, const int*) {
#pragma unroll
        for(int u = 0; u < kTileLoads; u++) {
            if(!valid[u] || key[u] == kOutOfRange) continue;
            const uint32_t pos = atomicAdd(&cursor[cursor_word(key[u])], 1u);
            float4 out = rec[u];
            if(p.echo_flags) {
                const float2 v = apply_echo(p, make_float2(out.x, out.y), out.z);
                out.x = v.x; out.y = v.y;
            }
            if(pos < total) sorted[pos] = out;
            else atomicOr(err, kErrScatterOverflow);
        }
    });
}

} // namespace

} // namespace rtacx
