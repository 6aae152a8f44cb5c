// Batched plain form: many pings from heterogeneous sensors in one CUDA graph.
//
// A batch holds up to thousands of pings, each bound to its own configured
// context (1D or 2D). rtacx_batch_plan builds, once:
//   * a device descriptor per ping (PingDev: its samples, scratch, tables);
//   * (ping, index) maps of the binning work of every ping (totals to zero,
//     count / scatter chunks, bin-scan blocks, window row groups);
//   * the gather work list: 2D output tiles and 1D row groups of every ping,
//     heaviest first;
// then captures the batch into a CUDA graph. By default the graph holds one
// kernel: k_batch_fused, a cooperative persistent launch (one or two CTAs per
// SM, all resident) that runs every phase of every ping, taking work from
// atomic queues and separating the phases with bounded grid barriers (and a
// 24-byte memset node that resets the barrier and the queues). With
// RTACX_BATCH_STAGED the graph holds one launch per binning stage and a
// persistent gather kernel instead. rtacx_batch_run replays the graph with one
// cudaGraphLaunch. With RTACX_BATCH_AUTOTUNE the plan times every candidate
// (gather tile shape x samples per binning chunk) on the real batch and keeps
// the fastest.
#include "rtacx_internal.cuh"

#include <algorithm>
#include <cmath>
#include <set>
#include <vector>

namespace rtacx {

namespace {

struct Candidate {
    int shape;
    uint32_t per_cta;
};

uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

} // namespace

struct Batch {
    int device = 0;
    int sm_count = 0;
    std::string error;
    cudaStream_t stream = nullptr;
    std::vector<rtacx_ping_desc> pings;
    // Device arrays of the current plan.
    PingDev* d_pings = nullptr;
    uint2* d_chunk_map = nullptr;
    uint2* d_col_map = nullptr;
    uint2* d_win_map = nullptr;
    uint2* d_scan_map = nullptr;
    uint4* d_items = nullptr;
    uint32_t* d_counter = nullptr;
    BatchSync* d_sync = nullptr;
    uint32_t* d_status = nullptr;
    uint32_t n_chunks = 0, n_col = 0, n_win = 0, n_scan = 0, n_items = 0, max_bins = 0;
    size_t gather_smem = 0;
    uint32_t gather_grid = 0;
    bool staged = false;            // RTACX_BATCH_STAGED
    FusedBatch fb{};
    size_t fused_smem = 0;
    uint32_t fused_grid = 0;
    uint32_t graph_kernels = 0;     // kernel nodes of the captured graph
    uint32_t diag_extra = 0;        // extra barrier arrivals (diagnostic)
    uint32_t wait_ms = 1000;        // bound of one grid-barrier wait
    Candidate chosen{2, 4096};
    float tuned_ms = 0.0f;
    cudaGraphExec_t exec = nullptr;

    template <typename T>
    void drop(T*& p) { if(p) cudaFree(p); p = nullptr; }

    void free_plan()
    {
        if(exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        drop(d_pings); drop(d_chunk_map); drop(d_col_map); drop(d_win_map); drop(d_scan_map); drop(d_items);
        graph_kernels = 0;
    }

    template <typename T>
    bool put(T*& dst, const std::vector<T>& src)
    {
        drop(dst);
        const size_t bytes = std::max<size_t>(1, src.size()) * sizeof(T);
        if(cudaMalloc(&dst, bytes) != cudaSuccess) { cudaGetLastError(); error = "cudaMalloc failed"; return false; }
        if(!src.empty() && cudaMemcpy(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            error = "cudaMemcpy failed";
            return false;
        }
        return true;
    }

    // Descriptors, maps and work items for one candidate; captures the graph.
    rtacx_status build(const Candidate& cand)
    {
        free_plan();
        const int TR = gather_shape_rows(cand.shape), TB = gather_shape_bearings(cand.shape);
        std::vector<PingDev> descs;
        std::vector<uint2> chunk_map, col_map, win_map, scan_map;
        struct Item { uint4 v; double cost; };
        std::vector<Item> items;
        max_bins = 1;
        gather_smem = 0;
        for(uint32_t i = 0; i < pings.size(); i++) {
            Context& c = pings[i].ctx->impl;
            const uint64_t n = pings[i].n;
            PingDev d{};
            d.samples = static_cast<const float*>(pings[i].samples);
            d.n = n;
            d.bin = c.bin;
            d.bin.vec4 = (c.dims == 2 && reinterpret_cast<uintptr_t>(pings[i].samples) % 16 == 0) ? 1 : 0;
            d.chunks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(c.hist_ctas, ceil_div(n, cand.per_cta)));
            d.hist = c.d_hist; d.totals = c.d_totals; d.offsets = c.d_offsets; d.oor = c.d_oor; d.err = c.d_err;
            d.sorted = c.d_sorted;
            d.nR = c.nR; d.overlap = c.overlap; d.support = c.d_support; d.win = c.d_win;
            d.red = c.red; d.bb_tiles = c.d_bb_tiles; d.ranges = c.d_ranges; d.bearings = c.d_bearings;
            d.pulse = c.d_pulse; d.beam = c.d_beam; d.out = reinterpret_cast<float2*>(pings[i].out);
            if(c.dims == 2) d.bb_tiles = (TB == 64) ? c.d_bb_tiles64 : c.d_bb_tiles128;   // ranges for width TB
            descs.push_back(d);
            for(uint32_t k = 0; k < d.chunks; k++) chunk_map.push_back(make_uint2(i, k));
            for(uint32_t k = 0; k < ceil_div(c.bin.nBins, 256); k++) col_map.push_back(make_uint2(i, k));
            for(uint32_t k = 0; k < ceil_div(c.nR, 256); k++) win_map.push_back(make_uint2(i, k));
            for(uint32_t k = 0; k < ceil_div(c.bin.nBins, kScanBlock); k++) scan_map.push_back(make_uint2(i, k));
            max_bins = std::max(max_bins, c.bin.nBins);
            const double density = (double)n / c.nR;     // samples per range bin
            if(c.dims == 2) {
                const uint32_t tb = (c.nB + TB - 1) / TB, tr = (c.nR + TR - 1) / TR;
                for(uint32_t y = 0; y < tr; y++)
                    for(uint32_t x = 0; x < tb; x++) items.push_back({make_uint4(i, x, y, 0), density * TR * TB});
                gather_smem = std::max(gather_smem, gather_batch_smem(cand.shape, c.H, c.W));
            }
            else {
                for(uint32_t g = 0; g < ceil_div(c.nR, 8); g++) items.push_back({make_uint4(i, g, 0, 1), density * 8.0});
                gather_smem = std::max(gather_smem, (size_t)(c.H + 2) * sizeof(float2));
            }
        }
        std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& b) { return a.cost > b.cost; });
        std::vector<uint4> iv(items.size());
        for(size_t k = 0; k < items.size(); k++) iv[k] = items[k].v;
        n_chunks = (uint32_t)chunk_map.size(); n_col = (uint32_t)col_map.size();
        n_win = (uint32_t)win_map.size(); n_scan = (uint32_t)scan_map.size(); n_items = (uint32_t)iv.size();
        if(!put(d_pings, descs) || !put(d_chunk_map, chunk_map) || !put(d_col_map, col_map) ||
           !put(d_win_map, win_map) || !put(d_scan_map, scan_map) || !put(d_items, iv))
            return RTACX_ERR_OUT_OF_MEMORY;
        if(gather_smem > 227 * 1024) { error = "PSF tables too large for the batched gather"; return RTACX_ERR_UNSUPPORTED; }
        if(staged && (size_t)max_bins * 4 > 227 * 1024) { error = "histograms too large for the batched binning"; return RTACX_ERR_UNSUPPORTED; }
        chosen = cand;
        return staged ? capture_staged(cand, (uint32_t)descs.size()) : capture_fused(cand);
    }

    // Graph of the fused form: reset of the barrier and queues, one
    // cooperative launch.
    rtacx_status capture_fused(const Candidate& cand)
    {
        fused_smem = gather_smem;
        rtacx_status prep = prepare_fused_batch(error, cand.shape, fused_smem, sm_count, fused_grid);
        if(prep != RTACX_OK) return prep;
        fb = FusedBatch{};
        fb.pings = d_pings;
        fb.col_map = d_col_map; fb.n_col = n_col;
        fb.chunk_map = d_chunk_map; fb.n_chunks = n_chunks;
        fb.scan_map = d_scan_map; fb.n_scan = n_scan;
        fb.win_map = d_win_map; fb.n_win = n_win;
        fb.items = d_items; fb.n_items = n_items;
        fb.sync = d_sync;
        fb.status = d_status;
        fb.arrivals = fused_grid + diag_extra;
        fb.wait_ns = (unsigned long long)wait_ms * 1000000ull;
        cudaGraph_t graph = nullptr;
        if(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            error = "cudaStreamBeginCapture failed";
            return RTACX_ERR_CUDA;
        }
        rtacx_status st = RTACX_OK;
        if(cudaMemsetAsync(d_sync, 0, sizeof(BatchSync), stream) != cudaSuccess) st = RTACX_ERR_CUDA;
        if(st == RTACX_OK) st = launch_fused_batch(error, cand.shape, fb, fused_smem, fused_grid, stream);
        return finish_capture(st, graph);
    }

    // Graph of the staged form: reset of the work counter, five binning
    // launches, one persistent gather.
    rtacx_status capture_staged(const Candidate& cand, uint32_t n_pings)
    {
        gather_grid = (uint32_t)sm_count * (gather_smem <= 100 * 1024 ? 2u : 1u);
        rtacx_status prep = prepare_bin_batch(error, max_bins);
        if(prep == RTACX_OK) prep = prepare_gather_batch(error, cand.shape, gather_smem);
        if(prep != RTACX_OK) return prep;
        cudaGraph_t graph = nullptr;
        if(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            error = "cudaStreamBeginCapture failed";
            return RTACX_ERR_CUDA;
        }
        rtacx_status st = RTACX_OK;
        if(cudaMemsetAsync(d_counter, 0, sizeof(uint32_t), stream) != cudaSuccess) st = RTACX_ERR_CUDA;
        if(st == RTACX_OK)
            st = launch_bin_batch(error, d_pings, n_pings, d_chunk_map, n_chunks, d_col_map, n_col,
                                  d_win_map, n_win, max_bins, stream);
        if(st == RTACX_OK)
            st = launch_gather_batch(error, cand.shape, d_pings, d_items, n_items, d_counter, gather_smem, gather_grid,
                                     stream);
        return finish_capture(st, graph);
    }

    rtacx_status finish_capture(rtacx_status st, cudaGraph_t graph)
    {
        const cudaError_t ec = cudaStreamEndCapture(stream, &graph);
        if(st != RTACX_OK || ec != cudaSuccess) {
            cudaGetLastError();
            if(graph) cudaGraphDestroy(graph);
            if(st == RTACX_OK) { error = std::string("stream capture failed: ") + cudaGetErrorString(ec); st = RTACX_ERR_CUDA; }
            return st;
        }
        size_t n_nodes = 0;
        graph_kernels = 0;
        if(cudaGraphGetNodes(graph, nullptr, &n_nodes) == cudaSuccess && n_nodes) {
            std::vector<cudaGraphNode_t> nodes(n_nodes);
            if(cudaGraphGetNodes(graph, nodes.data(), &n_nodes) == cudaSuccess)
                for(size_t k = 0; k < n_nodes; k++) {
                    cudaGraphNodeType t;
                    if(cudaGraphNodeGetType(nodes[k], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) graph_kernels++;
                }
        }
        cudaGetLastError();
        const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if(ei != cudaSuccess) {
            cudaGetLastError();
            exec = nullptr;
            error = std::string("cudaGraphInstantiate failed: ") + cudaGetErrorString(ei);
            return RTACX_ERR_CUDA;
        }
        return RTACX_OK;
    }

    // Median device time of `reps` replays of the current graph.
    bool time_plan(int reps, float& ms)
    {
        cudaEvent_t a, b;
        if(cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) { cudaGetLastError(); return false; }
        std::vector<float> t;
        bool ok = cudaGraphLaunch(exec, stream) == cudaSuccess;   // warm-up
        for(int r = 0; ok && r < reps; r++) {
            float x = 0.0f;
            ok = cudaEventRecord(a, stream) == cudaSuccess && cudaGraphLaunch(exec, stream) == cudaSuccess &&
                 cudaEventRecord(b, stream) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess &&
                 cudaEventElapsedTime(&x, a, b) == cudaSuccess;
            t.push_back(x);
        }
        cudaEventDestroy(a); cudaEventDestroy(b);
        if(!ok) { cudaGetLastError(); return false; }
        std::sort(t.begin(), t.end());
        ms = t[t.size() / 2];
        return true;
    }
};

} // namespace rtacx

struct rtacx_batch {
    rtacx::Batch impl;
};

using namespace rtacx;

extern "C" {

rtacx_status rtacx_batch_create(rtacx_batch** out, int device)
{
    if(!out) return RTACX_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if(cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return RTACX_ERR_CUDA; }
    rtacx_batch* b = new rtacx_batch();
    Batch& B = b->impl;
    B.device = device;
    if(cudaDeviceGetAttribute(&B.sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
       cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking) != cudaSuccess ||
       cudaMalloc(&B.d_counter, sizeof(uint32_t)) != cudaSuccess ||
       cudaMalloc(&B.d_sync, sizeof(BatchSync)) != cudaSuccess ||
       cudaMalloc(&B.d_status, sizeof(uint32_t)) != cudaSuccess ||
       cudaMemset(B.d_status, 0, sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        rtacx_batch_destroy(b);
        return RTACX_ERR_CUDA;
    }
    *out = b;
    return RTACX_OK;
}

void rtacx_batch_destroy(rtacx_batch* b)
{
    if(!b) return;
    Batch& B = b->impl;
    cudaSetDevice(B.device);
    B.free_plan();
    B.drop(B.d_counter);
    B.drop(B.d_sync);
    B.drop(B.d_status);
    if(B.stream) cudaStreamDestroy(B.stream);
    delete b;
}

const char* rtacx_batch_last_error(const rtacx_batch* b)
{
    return b ? b->impl.error.c_str() : "null batch";
}

rtacx_status rtacx_batch_plan(rtacx_batch* b, const rtacx_ping_desc* pings, uint32_t count, uint32_t flags)
{
    if(!b) return RTACX_ERR_INVALID_ARGUMENT;
    Batch& B = b->impl;
    if(!pings || count == 0) { B.error = "empty batch"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(cudaSetDevice(B.device) != cudaSuccess) { cudaGetLastError(); B.error = "cudaSetDevice failed"; return RTACX_ERR_CUDA; }
    std::set<const rtacx_ctx*> seen;
    for(uint32_t i = 0; i < count; i++) {
        const rtacx_ping_desc& p = pings[i];
        if(!p.ctx || !p.samples || !p.out || p.n == 0) { B.error = "ping " + std::to_string(i) + ": null pointer or no samples"; return RTACX_ERR_INVALID_ARGUMENT; }
        Context& c = p.ctx->impl;
        if(!c.configured) { B.error = "ping " + std::to_string(i) + ": context not configured"; return RTACX_ERR_NOT_CONFIGURED; }
        if(c.psf_tex) { B.error = "ping " + std::to_string(i) + ": RTACX_FLAG_TEXTURE_PSF is not supported in batches"; return RTACX_ERR_UNSUPPORTED; }
        if(c.device != B.device) { B.error = "ping " + std::to_string(i) + ": context on another device"; return RTACX_ERR_INVALID_ARGUMENT; }
        if(!seen.insert(p.ctx).second) { B.error = "ping " + std::to_string(i) + ": every ping needs its own context"; return RTACX_ERR_INVALID_ARGUMENT; }
        if(p.n >= (1ull << 32)) { B.error = "at most 2^32 - 1 samples per ping"; return RTACX_ERR_UNSUPPORTED; }
        if(reinterpret_cast<uintptr_t>(p.samples) % 4 != 0) { B.error = "sample buffers must be 4-byte aligned"; return RTACX_ERR_INVALID_ARGUMENT; }
        if(reinterpret_cast<uintptr_t>(p.out) % 8 != 0) { B.error = "pings must be 8-byte aligned"; return RTACX_ERR_INVALID_ARGUMENT; }
        if(!ensure_capacity(c, p.n)) { B.error = c.error; return RTACX_ERR_OUT_OF_MEMORY; }
    }
    B.pings.assign(pings, pings + count);
    B.staged = (flags & RTACX_BATCH_STAGED) != 0;
    if(!(flags & RTACX_BATCH_AUTOTUNE)) {
        const rtacx_status st = B.build(Candidate{2, 4096});
        B.tuned_ms = 0.0f;
        return st;
    }
    // Autotune: every candidate is built, captured and timed on this batch.
    Candidate best{2, 4096};
    float best_ms = 1e30f;
    for(int shape = 0; shape < 3; shape++)
        for(uint32_t per : {2048u, 4096u, 8192u}) {
            const Candidate cand{shape, per};
            if(B.build(cand) != RTACX_OK) continue;
            float ms;
            if(B.time_plan(3, ms) && ms < best_ms) { best_ms = ms; best = cand; }
        }
    if(best_ms >= 1e30f) { if(B.error.empty()) B.error = "no batch plan could be built"; return RTACX_ERR_CUDA; }
    const rtacx_status st = B.build(best);
    B.tuned_ms = best_ms;
    return st;
}

rtacx_status rtacx_batch_run(rtacx_batch* b, void* stream)
{
    if(!b) return RTACX_ERR_INVALID_ARGUMENT;
    Batch& B = b->impl;
    if(!B.exec) { B.error = "plan the batch first"; return RTACX_ERR_NOT_CONFIGURED; }
    if(cudaSetDevice(B.device) != cudaSuccess ||
       cudaGraphLaunch(B.exec, static_cast<cudaStream_t>(stream)) != cudaSuccess) {
        cudaGetLastError();
        B.error = "cudaGraphLaunch failed";
        return RTACX_ERR_CUDA;
    }
    return RTACX_OK;
}

rtacx_status rtacx_batch_status(rtacx_batch* b, void* stream)
{
    if(!b) return RTACX_ERR_INVALID_ARGUMENT;
    Batch& B = b->impl;
    if(cudaSetDevice(B.device) != cudaSuccess) { cudaGetLastError(); B.error = "cudaSetDevice failed"; return RTACX_ERR_CUDA; }
    const cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if(e != cudaSuccess) { B.error = std::string("stream: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    uint32_t word = 0;
    if(cudaMemcpy(&word, B.d_status, sizeof(word), cudaMemcpyDeviceToHost) != cudaSuccess ||
       cudaMemset(B.d_status, 0, sizeof(word)) != cudaSuccess) {
        cudaGetLastError();
        B.error = "reading the batch status word failed";
        return RTACX_ERR_CUDA;
    }
    if(word) {
        B.error = "batch status word " + std::to_string(word) +
                  ((word & kErrBatchWaitTimeout) ? " (a grid-barrier wait expired; the batch's pings are incomplete)" : "");
        return RTACX_ERR_DEVICE;
    }
    return RTACX_OK;
}

rtacx_status rtacx_batch_graph_kernels(const rtacx_batch* b, uint32_t* kernels)
{
    if(!b || !kernels) return RTACX_ERR_INVALID_ARGUMENT;
    *kernels = b->impl.exec ? b->impl.graph_kernels : 0u;
    return RTACX_OK;
}

rtacx_status rtacx_diag_batch_barrier(rtacx_batch* b, uint32_t extra_arrivals, uint32_t wait_ms)
{
    if(!b || wait_ms == 0 || wait_ms > 10000 || extra_arrivals > 1) return RTACX_ERR_INVALID_ARGUMENT;
    b->impl.diag_extra = extra_arrivals;
    b->impl.wait_ms = wait_ms;
    return RTACX_OK;
}

rtacx_status rtacx_batch_tuning(const rtacx_batch* b, uint32_t* tile_rows, uint32_t* tile_bearings,
                                uint32_t* samples_per_cta, float* tuned_ms)
{
    if(!b) return RTACX_ERR_INVALID_ARGUMENT;
    const Batch& B = b->impl;
    if(tile_rows) *tile_rows = (uint32_t)gather_shape_rows(B.chosen.shape);
    if(tile_bearings) *tile_bearings = (uint32_t)gather_shape_bearings(B.chosen.shape);
    if(samples_per_cta) *samples_per_cta = B.chosen.per_cta;
    if(tuned_ms) *tuned_ms = B.tuned_ms;
    return RTACX_OK;
}

} // extern "C"
