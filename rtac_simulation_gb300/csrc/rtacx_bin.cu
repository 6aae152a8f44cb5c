// Sort + bin: a counting sort of echo samples by (range bin, bearing bin).
//
// Replaces sort() (src/Receiver.cu:9-42: thrust merge sort of the AoS
// samples by travel) and Binner::compute (src/Binner.cu:24-136: key
// transform, segment search, window construction). Only the multiset of
// samples per range bin matters downstream -- the reference's reduction sums
// a window of consecutive bins in any order -- so a counting sort on the
// integer key gives the reference's segments and windows exactly without a
// comparison sort.
//
// Passes (persistent CTAs, each owning one contiguous chunk of the input,
// processed in tiles of kTileLoads independent record loads per thread):
//   k_count           key of every sample, per-CTA histogram in shared
//                     memory, added into the zeroed bin totals and per-1024-bin
//                     block sums; out-of-range counts.
//   k_binscan_blocks  one CTA per 1024 bins: exclusive scan of the totals ->
//                     bin offsets, and one shared write cursor per bin
//                     initialised to its offset (binscan_cta: the
//                     single-CTA scan of the staged batched form).
//   k_scatter_pipe    re-reads the chunk in tiles of 7680 records, sorts each
//                     tile by bin in shared memory, reserves one run per
//                     (tile, bin) with a global atomicAdd on the bin's cursor
//                     and writes the float4 {re, im, travel, bearing} records
//                     of each run with consecutive lanes, while the next
//                     tile's loads are in flight (k_scatter_staged: the same
//                     without the pipelining, for more bins; k_scatter: the
//                     reservation without staging, when the per-bin tables do
//                     not fit next to a tile, and in the batched form).
//   k_windows         reference windows (do_make_bins, src/Binner.cu:82-106)
//                     as range-bin intervals, intersected with each row's PSF
//                     support.
// Every bin has one write frontier shared by all CTAs, so the partially
// written 128-byte lines of the sorted array number about one per bin and
// complete in L2 before eviction (per-CTA sub-ranges inside each bin would
// keep CTAs x bins lines open for the whole pass and turn the scattered
// 16-byte stores into partial-line write-backs).
#include "rtacx_bin_device.cuh"

#include <algorithm>
#include <climits>

namespace rtacx {

namespace {

constexpr int kScanThreads = 1024;

__global__ void k_count(const float* __restrict__ samples, uint64_t n, BinParams p,
                        uint32_t* __restrict__ totals, unsigned long long* __restrict__ oor)
{
    extern __shared__ uint32_t sh[];
    __shared__ unsigned long long s_oor[2];
    count_chunk(samples, n, p, blockIdx.x, gridDim.x, totals, oor, sh, s_oor);
}

// Exclusive scan of totals[0, nBins) into offsets[0, nBins] by one CTA of
// kScanThreads threads; cursor (optional) receives offsets[0, nBins).
// The totals pass through shared memory in segments of kScanSeg bins
// (coalesced loads and stores; each thread scans 8 consecutive bins of the
// segment, padded against bank conflicts), carrying the running total.
constexpr uint32_t kScanPer = 8, kScanSeg = kScanThreads * kScanPer;

__device__ __forceinline__ uint32_t scan_pad(uint32_t i) { return i + i / 32; }

__device__ void binscan_cta(const uint32_t* __restrict__ totals, uint32_t nBins, uint32_t* __restrict__ offsets,
                            uint32_t* __restrict__ cursor)
{
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_seg[kScanSeg + kScanSeg / 32];
    uint32_t carry = 0;
    for(uint32_t s0 = 0; s0 < nBins; s0 += kScanSeg) {
        const uint32_t len = min(kScanSeg, nBins - s0);
        for(uint32_t i = threadIdx.x; i < kScanSeg; i += blockDim.x) s_seg[scan_pad(i)] = i < len ? totals[s0 + i] : 0u;
        __syncthreads();
        const uint32_t q0 = threadIdx.x * kScanPer;
        uint32_t v[kScanPer], sum = 0;
#pragma unroll
        for(uint32_t u = 0; u < kScanPer; u++) { v[u] = s_seg[scan_pad(q0 + u)]; sum += v[u]; }
        uint32_t seg_total;
        uint32_t run = carry + block_exclusive_scan(sum, s_warp, seg_total);
#pragma unroll
        for(uint32_t u = 0; u < kScanPer; u++) { s_seg[scan_pad(q0 + u)] = run; run += v[u]; }
        __syncthreads();
        for(uint32_t i = threadIdx.x; i < len; i += blockDim.x) {
            const uint32_t o = s_seg[scan_pad(i)];
            offsets[s0 + i] = o;
            if(cursor) cursor[cursor_word(s0 + i)] = o;
        }
        carry += seg_total;
        __syncthreads();
    }
    if(threadIdx.x == 0) offsets[nBins] = carry;
}

// Parallel exclusive scan of the bin totals: CTA i scans bins
// [i kScanBlock, (i + 1) kScanBlock) and adds the sum of the block sums
// before it (totals[nBins + j], accumulated by the count pass). Writes
// offsets[0, nBins] and the scatter's per-bin cursors.
__global__ void __launch_bounds__(kScanBlock) k_binscan_blocks(const uint32_t* __restrict__ totals, uint32_t nBins,
                                                               uint32_t* __restrict__ offsets,
                                                               uint32_t* __restrict__ cursor)
{
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_prefix;
    scan_bin_block(totals, nBins, blockIdx.x, offsets, cursor, s_warp, &s_prefix);
}

__global__ void k_scatter(const float* __restrict__ samples, uint64_t n, BinParams p,
                          uint32_t* __restrict__ cursor, const uint32_t* __restrict__ offsets,
                          float4* __restrict__ sorted, uint32_t* __restrict__ err)
{
    extern __shared__ uint32_t sh[];
    scatter_chunk(samples, n, p, blockIdx.x, gridDim.x, cursor, offsets, sorted, err, sh);
}

// Staged scatter (single ping; one 1024-thread CTA per SM): tiles of
// 1024 * U records are sorted by bin in shared memory before they are
// written, so consecutive lanes store consecutive slots of each bin's run and
// the stores coalesce into whole sectors. Per tile:
//   pass 1   load records, key, rank among the tile's samples of the bin
//            (shared histogram);
//   scan     block exclusive scan of the histogram = local run starts; one
//            atomicAdd per non-empty (tile, bin) on the bin's shared cursor
//            reserves the run; delta = global base - local start;
//   pass 2   reload the tile (L2-resident since pass 1) into its sorted
//            shared-memory slot;
//   write    slot j goes to j + delta[key(j)] (the key recomputed from the
//            record's travel and bearing, as in pass 1).
// Shared memory: 16 B x NT U records + 8 B per bin. Used as 1024 x 4 where
// the bin tables leave no room for the pipelined scatter's tile.
size_t staged_smem_bytes(int NT, int U, uint32_t nBins) { return (size_t)NT * U * sizeof(float4) + (size_t)nBins * 8; }

template <int NT, int U>
__global__ void __launch_bounds__(NT, 1024 / NT)
k_scatter_staged(const float* __restrict__ samples, uint64_t n, BinParams p, uint32_t* __restrict__ cursor,
                 const uint32_t* __restrict__ offsets, float4* __restrict__ sorted, uint32_t* __restrict__ err)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ uint32_t s_warp[32];
    const uint32_t nb = p.nBins;
    float4* s_rec = reinterpret_cast<float4*>(s_raw);
    uint32_t* s_start = reinterpret_cast<uint32_t*>(s_rec + NT * U);     // histogram, then local run starts
    uint32_t* s_delta = s_start + nb;                                     // global base - local start
    const uint32_t tid = threadIdx.x;
    const uint32_t per = (nb + NT - 1) / NT, b0 = min(tid * per, nb), b1 = min(b0 + per, nb);
    const uint32_t total = offsets[nb];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t begin = (uint64_t)blockIdx.x * chunk, end = min(begin + chunk, n);
    for(uint32_t b = tid; b < nb; b += NT) s_start[b] = 0u;
    __syncthreads();
    for(uint64_t t0 = begin; t0 < end; t0 += (uint64_t)NT * U) {
        uint32_t key[U], rank[U];
#pragma unroll
        for(int u = 0; u < U; u++) {
            const uint64_t i = t0 + (uint64_t)u * NT + tid;
            key[u] = kOutOfRange;
            if(i < end) {
                const float4 rec = load_record(samples, i, p);
                int side;
                key[u] = sample_key(p, rec.z, rec.w, side);
            }
        }
#pragma unroll
        for(int u = 0; u < U; u++) rank[u] = key[u] != kOutOfRange ? atomicAdd(&s_start[key[u]], 1u) : 0u;
        __syncthreads();
        uint32_t sum = 0;
        for(uint32_t b = b0; b < b1; b++) sum += s_start[b];
        uint32_t tile_total;
        uint32_t run = block_exclusive_scan(sum, s_warp, tile_total);
        for(uint32_t b = b0; b < b1; b++) {
            const uint32_t c = s_start[b];
            s_start[b] = run;
            if(c) s_delta[b] = atomicAdd(&cursor[cursor_word(b)], c) - run;
            run += c;
        }
        __syncthreads();
#pragma unroll
        for(int u = 0; u < U; u++) {
            if(key[u] == kOutOfRange) continue;
            float4 rec = load_record(samples, t0 + (uint64_t)u * NT + tid, p);
            if(p.echo_flags) {
                const float2 v = apply_echo(p, make_float2(rec.x, rec.y), rec.z);
                rec.x = v.x; rec.y = v.y;
            }
            s_rec[s_start[key[u]] + rank[u]] = rec;
        }
        __syncthreads();
        for(uint32_t j = tid; j < tile_total; j += NT) {
            const float4 rec = s_rec[j];
            int side;
            const uint32_t k = sample_key(p, rec.z, rec.w, side);
            const uint32_t pos = j + s_delta[k];
            if(pos < total) sorted[pos] = rec;
            else atomicOr(err, kErrScatterOverflow);
        }
        __syncthreads();
        for(uint32_t b = b0; b < b1; b++) s_start[b] = 0u;
        __syncthreads();
    }
}

__global__ void k_windows(const uint32_t* __restrict__ off, uint32_t nBB, uint32_t nR, int ov,
                          const int2* __restrict__ support, int2* __restrict__ win)
{
    window_row(off, nBB, nR, ov, support, win, blockIdx.x * blockDim.x + threadIdx.x);
}

// Reference-coordinate outputs of rtacx_bin: the reference's sorted array
// puts the below-range out-of-range samples first, then the bins in order.
__global__ void k_ref_outputs(const uint32_t* __restrict__ off, uint32_t nBB, uint32_t nR, int ov,
                              const unsigned long long* __restrict__ oor,
                              uint32_t* __restrict__ segments, uint32_t* __restrict__ windows,
                              uint32_t* __restrict__ counts)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if(r >= (int)nR) return;
    const uint32_t lowc = (uint32_t)oor[0];
    const uint32_t cnt = bin_count(off, nBB, r);
    if(counts) counts[r] = cnt;
    if(segments) {
        uint2 s = make_uint2(0u, 0u);
        if(cnt) s = make_uint2(lowc + off[(size_t)r * nBB], lowc + off[(size_t)(r + 1) * nBB]);
        reinterpret_cast<uint2*>(segments)[r] = s;
    }
    if(windows) {
        int f, l;
        uint2 w = make_uint2(0u, 0u);
        if(ref_window(off, nBB, nR, ov, r, f, l))
            w = make_uint2(lowc + off[(size_t)f * nBB], off[(size_t)(l + 1) * nBB] - off[(size_t)f * nBB]);
        reinterpret_cast<uint2*>(windows)[r] = w;
    }
}

__global__ void k_range_keys(const float* __restrict__ samples, uint64_t n, BinParams p, uint32_t* __restrict__ keys)
{
    for(uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const float t = __ldg(samples + i * p.stride + 2);
        int side;
        keys[i] = range_key(p.key, t, side);
    }
}

__global__ void k_oor_out(const unsigned long long* __restrict__ src, uint64_t* __restrict__ dst)
{
    if(threadIdx.x < 2) dst[threadIdx.x] = src[threadIdx.x];
}

// ---- batched stages (one launch per stage over every ping of a batch) -----

__global__ void k_count_batch(const PingDev* __restrict__ pings, const uint2* __restrict__ map)
{
    extern __shared__ uint32_t sh[];
    __shared__ unsigned long long s_oor[2];
    const uint2 m = map[blockIdx.x];
    const PingDev& P = pings[m.x];
    count_chunk(P.samples, P.n, P.bin, m.y, P.chunks, P.totals, P.oor, sh, s_oor);
}

// Zeroes every ping's bin totals and block sums (one thread per (ping, bin)).
__global__ void k_zero_totals_batch(const PingDev* __restrict__ pings, const uint2* __restrict__ map)
{
    const uint2 m = map[blockIdx.x];
    const PingDev& P = pings[m.x];
    const uint32_t b = m.y * blockDim.x + threadIdx.x;
    if(b < P.bin.nBins) P.totals[b] = 0u;
    if(b < (P.bin.nBins + kScanBlock - 1) / kScanBlock) P.totals[P.bin.nBins + b] = 0u;
}

__global__ void __launch_bounds__(kScanThreads) k_binscan_batch(const PingDev* __restrict__ pings)
{
    const PingDev& P = pings[blockIdx.x];
    binscan_cta(P.totals, P.bin.nBins, P.offsets, P.hist);
}

__global__ void k_scatter_batch(const PingDev* __restrict__ pings, const uint2* __restrict__ map)
{
    extern __shared__ uint32_t sh[];
    const uint2 m = map[blockIdx.x];
    const PingDev& P = pings[m.x];
    scatter_chunk(P.samples, P.n, P.bin, m.y, P.chunks, P.hist, P.offsets, P.sorted, P.err, sh);   // hist = cursors
}

__global__ void k_windows_batch(const PingDev* __restrict__ pings, const uint2* __restrict__ map)
{
    const uint2 m = map[blockIdx.x];
    const PingDev& P = pings[m.x];
    window_row(P.offsets, P.bin.nBB, P.nR, P.overlap, P.support, P.win, m.y * blockDim.x + threadIdx.x);
}

__global__ void k_reset_batch(const PingDev* __restrict__ pings, uint32_t n_pings)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i < n_pings) { pings[i].oor[0] = 0ull; pings[i].oor[1] = 0ull; }
}

uint32_t hist_grid(uint32_t ctas, uint64_t n)
{
    // At least ~1024 samples per CTA so that the per-CTA histogram set-up
    // stays small relative to the data.
    const uint64_t want = std::max<uint64_t>(1, (n + 1023) / 1024);
    return (uint32_t)std::min<uint64_t>(ctas, want);
}

#define RTACX_CUDA(call)                                                         \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if(e_ != cudaSuccess) {                                                  \
            ctx.error = std::string(#call) + ": " + cudaGetErrorString(e_);      \
            return RTACX_ERR_CUDA;                                               \
        }                                                                        \
    } while(0)

} // namespace

bool ensure_capacity(Context& ctx, uint64_t n)
{
    if(n <= ctx.capacity) return true;
    uint64_t cap = std::max<uint64_t>(n, 1024);
    float4* p = nullptr;
    if(cudaMalloc(&p, cap * sizeof(float4)) != cudaSuccess) {
        cudaGetLastError();
        return ctx.fail("out of device memory for " + std::to_string(cap) + " sorted samples");
    }
    if(ctx.d_sorted) cudaFree(ctx.d_sorted);
    ctx.d_sorted = p;
    ctx.capacity = cap;
    return true;
}

namespace {

// Pipelined staged scatter (single ping; one CTA of NT threads per SM). The
// records of tile t are loaded into registers (U per thread) while the
// sorted slots of tile t - 1 are written out from shared memory, so each SM
// reads and writes HBM at the same time instead of in alternating phases,
// and every record is read from memory once (it goes from its registers
// straight into its sorted slot). Per tile:
//   load     U records per thread into registers (tile t)
//   write    sorted slot j of tile t - 1 -> j + delta[key(j)]
//   rank     key of every record of tile t, rank among the tile's samples of
//            the bin (shared histogram)
//   reserve  block exclusive scan of the histogram = local run starts; one
//            64-bit atomicAdd per (tile, pair of bins) with a non-empty bin on
//            the pair's shared cursor word, up to kReserveBatch / 2 of them in
//            flight per thread; with at most
//            kReserveBatch bins per thread (ONE_BATCH) they stay in flight
//            during the placement
//   place    records -> sorted shared-memory slots (echo pre-step applied;
//            instantiated with and without it, which keeps the echo-free
//            form's registers below the launch bound)
// Shared memory: 16 B x NT U records + 8 B per bin.
constexpr int kReserveBatch = 8;

// Bins per thread of the pipelined scatter's reservation: even, so that each
// thread's bins start a cursor pair.
__host__ __device__ __forceinline__ uint32_t pipe_bins_per_thread(uint32_t nb, uint32_t nt)
{
    return ((nb + nt - 1) / nt + 1u) & ~1u;
}

// Reserves c0 slots in even bin b and c1 in bin b + 1 with one 64-bit atomic
// on their shared cursor word; returns the old cursors (low: b, high: b + 1).
__device__ __forceinline__ unsigned long long reserve_pair(uint32_t* cursor, uint32_t b, uint32_t c0, uint32_t c1)
{
    if(!(c0 | c1)) return 0ull;
    return atomicAdd(reinterpret_cast<unsigned long long*>(cursor + cursor_word(b)),
                     (unsigned long long)c1 << 32 | c0);
}

// Placement of one thread's records into their sorted shared-memory slots
// (echo pre-step applied when ECHO); rank kOutOfRange marks a skipped record.
template <int U, bool ECHO>
__device__ __forceinline__ void place_records(const BinParams& p, const float4 (&rec)[U], const uint32_t (&rank)[U],
                                              const uint32_t* s_start, float4* s_rec)
{
#pragma unroll
    for(int u = 0; u < U; u++) {
        if(rank[u] == kOutOfRange) continue;
        float4 r = rec[u];
        int side;
        const uint32_t k = sample_key(p, r.z, r.w, side);
        if(ECHO) {
            const float2 v = apply_echo(p, make_float2(r.x, r.y), r.z);
            r.x = v.x; r.y = v.y;
        }
        s_rec[s_start[k] + rank[u]] = r;
    }
}

template <int NT, int U, bool ECHO, bool ONE_BATCH>
__global__ void __launch_bounds__(NT, 1)
k_scatter_pipe(const float* __restrict__ samples, uint64_t n, BinParams p, uint32_t* __restrict__ cursor,
               const uint32_t* __restrict__ offsets, float4* __restrict__ sorted, uint32_t* __restrict__ err)
{
    extern __shared__ __align__(16) unsigned char s_raw[];
    __shared__ uint32_t s_warp[32];
    const uint32_t nb = p.nBins;
    float4* s_rec = reinterpret_cast<float4*>(s_raw);
    uint32_t* s_start = reinterpret_cast<uint32_t*>(s_rec + NT * U);     // histogram, then local run starts
    uint32_t* s_delta = s_start + nb;                                     // global base - local start
    const uint32_t tid = threadIdx.x;
    const uint32_t per = pipe_bins_per_thread(nb, NT), b0 = min(tid * per, nb), b1 = min(b0 + per, nb);
    const uint32_t total = offsets[nb];
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t begin = (uint64_t)blockIdx.x * chunk, end = min(begin + chunk, n);
    for(uint32_t b = b0; b < b1; b++) s_start[b] = 0u;
    uint32_t prev = 0;                       // sorted slots of the previous tile
    for(uint64_t t0 = begin;; t0 += (uint64_t)NT * U) {
        const bool more = t0 < end;
        float4 rec[U];
        if(more) {
#pragma unroll
            for(int u = 0; u < U; u++) {
                const uint64_t i = t0 + (uint64_t)u * NT + tid;
                rec[u] = i < end ? load_record(samples, i, p) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        for(uint32_t j = tid; j < prev; j += NT) {
            const float4 r = s_rec[j];
            int side;
            const uint32_t pos = j + s_delta[sample_key(p, r.z, r.w, side)];
            if(pos < total) sorted[pos] = r;
            else atomicOr(err, kErrScatterOverflow);
        }
        if(!more) break;
        __syncthreads();                     // slots and deltas of tile t - 1 consumed, histogram zeroed
        uint32_t rank[U];
#pragma unroll
        for(int u = 0; u < U; u++) {
            int side;
            const bool in = t0 + (uint64_t)u * NT + tid < end;
            const uint32_t k = in ? sample_key(p, rec[u].z, rec[u].w, side) : kOutOfRange;
            rank[u] = k != kOutOfRange ? atomicAdd(&s_start[k], 1u) : kOutOfRange;
        }
        __syncthreads();
        uint32_t sum = 0;
        for(uint32_t b = b0; b < b1; b++) sum += s_start[b];
        uint32_t tile_total;
        uint32_t run = block_exclusive_scan(sum, s_warp, tile_total);
        if(ONE_BATCH) {
            // The thread's bins (at most kReserveBatch) in one batch: local
            // run starts now, the cursor reservations in flight during the
            // placement, the deltas after it.
            uint32_t base[kReserveBatch], nonempty = 0;
#pragma unroll
            for(int q = 0; q < kReserveBatch; q += 2) {
                const uint32_t b = b0 + q;
                const uint32_t c0 = b < b1 ? s_start[b] : 0u, c1 = b + 1 < b1 ? s_start[b + 1] : 0u;
                const unsigned long long old = reserve_pair(cursor, b, c0, c1);
                base[q] = (uint32_t)old;
                base[q + 1] = (uint32_t)(old >> 32);
                nonempty |= (c0 ? 1u : 0u) << q | (c1 ? 1u : 0u) << (q + 1);
                if(b < b1) s_start[b] = run;
                if(b + 1 < b1) s_start[b + 1] = run + c0;
                run += c0 + c1;
            }
            __syncthreads();
            place_records<U, ECHO>(p, rec, rank, s_start, s_rec);
#pragma unroll
            for(int q = 0; q < kReserveBatch; q++)
                if(nonempty & (1u << q)) s_delta[b0 + q] = base[q] - s_start[b0 + q];
        }
        else {
            for(uint32_t g = b0; g < b1; g += kReserveBatch) {
                uint32_t c[kReserveBatch];
                unsigned long long old[kReserveBatch / 2];
#pragma unroll
                for(int q = 0; q < kReserveBatch; q++) c[q] = g + q < b1 ? s_start[g + q] : 0u;
#pragma unroll
                for(int q = 0; q < kReserveBatch; q += 2) old[q / 2] = reserve_pair(cursor, g + q, c[q], c[q + 1]);
#pragma unroll
                for(int q = 0; q < kReserveBatch; q++) {
                    if(g + q < b1) {
                        s_start[g + q] = run;
                        if(c[q]) s_delta[g + q] = (uint32_t)(old[q / 2] >> (32 * (q & 1))) - run;
                        run += c[q];
                    }
                }
            }
            __syncthreads();
            place_records<U, ECHO>(p, rec, rank, s_start, s_rec);
        }
        __syncthreads();
        for(uint32_t b = b0; b < b1; b++) s_start[b] = 0u;   // the next rank follows a barrier
        prev = tile_total;
    }
}

using ScatterFn = void (*)(const float*, uint64_t, BinParams, uint32_t*, const uint32_t*, float4*, uint32_t*);
struct ScatterShape {
    ScatterFn fn[2][2];         // [echo pre-step][one reservation batch per thread]
    int nt, u;
};
// In order of preference: pipelined 768 x 10 (bins up to ~13K), unpipelined
// 1024 x 4 (up to ~20K); more bins take the per-tile k_scatter.
const ScatterShape kScatterShapes[] = {
    {{{k_scatter_pipe<768, 10, false, false>, k_scatter_pipe<768, 10, false, true>},
      {k_scatter_pipe<768, 10, true, false>, k_scatter_pipe<768, 10, true, true>}}, 768, 10},
    {{{k_scatter_staged<1024, 4>, k_scatter_staged<1024, 4>}, {k_scatter_staged<1024, 4>, k_scatter_staged<1024, 4>}},
     1024, 4},
};
constexpr int kNumScatterShapes = sizeof(kScatterShapes) / sizeof(kScatterShapes[0]);

} // namespace

void configure_hist_launch(Context& ctx);

rtacx_status run_binning(Context& ctx, const void* samples, uint64_t n, cudaStream_t stream)
{
    const BinParams& p = ctx.bin;
    RTACX_CUDA(cudaMemsetAsync(ctx.d_oor, 0, 2 * sizeof(unsigned long long), stream));
    if(n == 0) {
        RTACX_CUDA(cudaMemsetAsync(ctx.d_offsets, 0, (p.nBins + 1) * sizeof(uint32_t), stream));
    }
    else {
        const uint32_t grid = hist_grid(ctx.hist_ctas, n);
        const size_t smem = (size_t)p.nBins * sizeof(uint32_t);
        const float* s = static_cast<const float*>(samples);
        ctx.mark(1, false, stream);
        const uint32_t scan_blocks = (p.nBins + kScanBlock - 1) / kScanBlock;
        RTACX_CUDA(cudaMemsetAsync(ctx.d_totals, 0, (p.nBins + scan_blocks) * sizeof(uint32_t), stream));
        ctx.mark(1, true, stream);
        ctx.mark(0, false, stream);
        k_count<<<grid, ctx.hist_threads, smem, stream>>>(s, n, p, ctx.d_totals, ctx.d_oor);
        RTACX_CUDA(cudaGetLastError());
        ctx.mark(0, true, stream);
        ctx.mark(2, false, stream);
        // d_hist holds the per-bin write cursors of the scatter.
        k_binscan_blocks<<<scan_blocks, kScanBlock, 0, stream>>>(ctx.d_totals, p.nBins, ctx.d_offsets, ctx.d_hist);
        RTACX_CUDA(cudaGetLastError());
        ctx.mark(2, true, stream);
        ctx.mark(3, false, stream);
        if(ctx.scatter_shape) {
            const ScatterShape& sh = kScatterShapes[ctx.scatter_shape - 1];
            const uint32_t g = hist_grid((uint32_t)ctx.sm_count, n);
            const bool one_batch = pipe_bins_per_thread(p.nBins, sh.nt) <= (uint32_t)kReserveBatch;
            const ScatterFn fn = sh.fn[p.echo_flags ? 1 : 0][one_batch ? 1 : 0];
            fn<<<g, sh.nt, staged_smem_bytes(sh.nt, sh.u, p.nBins), stream>>>(s, n, p, ctx.d_hist, ctx.d_offsets,
                                                                           ctx.d_sorted, ctx.d_err);
        }
        else {
            k_scatter<<<hist_grid(ctx.scatter_ctas, n), ctx.hist_threads, smem, stream>>>(s, n, p, ctx.d_hist,
                                                                                           ctx.d_offsets, ctx.d_sorted,
                                                                                           ctx.d_err);
        }
        RTACX_CUDA(cudaGetLastError());
        ctx.mark(3, true, stream);
    }
    ctx.mark(4, false, stream);
    k_windows<<<(ctx.nR + 255) / 256, 256, 0, stream>>>(ctx.d_offsets, p.nBB, ctx.nR, ctx.overlap,
                                                         ctx.d_support, ctx.d_win);
    RTACX_CUDA(cudaGetLastError());
    ctx.mark(4, true, stream);
    return RTACX_OK;
}

rtacx_status run_bin_outputs(Context& ctx, const void* samples, uint64_t n,
                             uint32_t* keys, uint32_t* segments, uint32_t* windows,
                             uint32_t* counts, uint64_t* oor, cudaStream_t stream)
{
    const BinParams& p = ctx.bin;
    if(keys && n) {
        const uint32_t blocks = (uint32_t)std::min<uint64_t>((n + 255) / 256, (uint64_t)ctx.sm_count * 16);
        k_range_keys<<<blocks, 256, 0, stream>>>(static_cast<const float*>(samples), n, p, keys);
        RTACX_CUDA(cudaGetLastError());
    }
    if(segments || windows || counts) {
        k_ref_outputs<<<(ctx.nR + 255) / 256, 256, 0, stream>>>(ctx.d_offsets, p.nBB, ctx.nR, ctx.overlap,
                                                                 ctx.d_oor, segments, windows, counts);
        RTACX_CUDA(cudaGetLastError());
    }
    if(oor) {
        k_oor_out<<<1, 32, 0, stream>>>(ctx.d_oor, oor);
        RTACX_CUDA(cudaGetLastError());
    }
    return RTACX_OK;
}

rtacx_status prepare_bin_batch(std::string& error, uint32_t max_bins)
{
    const size_t smem = std::max<size_t>((size_t)max_bins * sizeof(uint32_t), 1);
    if(raise_smem_limit((const void*)k_count_batch, smem) != cudaSuccess ||
       raise_smem_limit((const void*)k_scatter_batch, smem) != cudaSuccess) {
        error = "cannot reserve shared memory for the batched histograms";
        return RTACX_ERR_CUDA;
    }
    return RTACX_OK;
}

rtacx_status launch_bin_batch(std::string& error, const PingDev* pings, uint32_t n_pings,
                              const uint2* chunk_map, uint32_t n_chunks, const uint2* col_map, uint32_t n_col,
                              const uint2* win_map, uint32_t n_win, uint32_t max_bins, cudaStream_t stream)
{
    const size_t smem = (size_t)max_bins * sizeof(uint32_t);
    k_reset_batch<<<(n_pings + 255) / 256, 256, 0, stream>>>(pings, n_pings);
    k_zero_totals_batch<<<n_col, 256, 0, stream>>>(pings, col_map);
    k_count_batch<<<n_chunks, 512, smem, stream>>>(pings, chunk_map);
    k_binscan_batch<<<n_pings, kScanThreads, 0, stream>>>(pings);
    k_scatter_batch<<<n_chunks, 512, smem, stream>>>(pings, chunk_map);
    k_windows_batch<<<n_win, 256, 0, stream>>>(pings, win_map);
    const cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) { error = std::string("batched binning: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    return RTACX_OK;
}

// Launch shape of the count / scatter passes for the configured bin count.
void configure_hist_launch(Context& ctx)
{
    const size_t smem = (size_t)ctx.bin.nBins * sizeof(uint32_t);
    raise_smem_limit((const void*)k_count, std::max<size_t>(smem, 1));
    raise_smem_limit((const void*)k_scatter, std::max<size_t>(smem, 1));
    // 512-thread CTAs when two histograms fit in one SM's shared memory, one
    // 1024-thread CTA otherwise; each pass gets as many CTAs as are resident
    // at once (registers and shared memory), so that the scatter's per-tile
    // reservation phases of different CTAs overlap and no CTA waits for a
    // second wave.
    const size_t per_sm = 200u * 1024u;
    ctx.hist_threads = per_sm / (smem + 1024) >= 2 ? 512 : 1024;
    auto resident = [&](const void* fn) {
        int nb = 0;
        if(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, (int)ctx.hist_threads, std::max<size_t>(smem, 1)) !=
               cudaSuccess || nb < 1)
            nb = 1;
        return (uint32_t)ctx.sm_count * (uint32_t)std::min(nb, 4);
    };
    ctx.hist_ctas = resident((const void*)k_count);
    ctx.scatter_ctas = resident((const void*)k_scatter);
    // Staged scatter: the first shape of kScatterShapes whose shared memory
    // fits.
    ctx.scatter_shape = 0;
    int optin = 0, smem_sm = 0;
    if(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx.device) != cudaSuccess) optin = 0;
    if(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx.device) != cudaSuccess) smem_sm = 0;
    for(int c = 0; c < kNumScatterShapes && !ctx.scatter_shape; c++) {
        const ScatterShape& sh = kScatterShapes[c];
        const size_t need = staged_smem_bytes(sh.nt, sh.u, ctx.bin.nBins);
        bool ok = need + 1024 <= (size_t)optin && need + 1024 <= (size_t)smem_sm;
        for(int e = 0; e < 2 && ok; e++)
            for(int b = 0; b < 2 && ok; b++) ok = raise_smem_limit((const void*)sh.fn[e][b], need) == cudaSuccess;
        if(ok) ctx.scatter_shape = c + 1;
    }
    cudaGetLastError();
}

} // namespace rtacx
