// Precision form from host memory: the end-to-end call a host-side caller
// makes. The samples are copied to the device in chunks through two staging
// buffers on an internal copy stream; chunk i + 1 is copied while chunk i is
// accumulated (the accumulation is order-independent, so a ping may be
// accumulated chunk by chunk), then the ping is formed on the device and
// copied back. The copy stream is forked from and joined to the caller's
// stream with events, so the call is stream-ordered and graph-capturable.
#include "rtacx_internal.cuh"

namespace rtacx {

namespace {

#define RTACX_CUDA(call)                                                         \
    do {                                                                         \
        cudaError_t e_ = (call);                                                 \
        if(e_ != cudaSuccess) {                                                  \
            c.error = std::string(#call) + ": " + cudaGetErrorString(e_);        \
            return RTACX_ERR_CUDA;                                               \
        }                                                                        \
    } while(0)

rtacx_status ensure_streaming(Context& c, size_t record_bytes)
{
    if(!c.copy_stream) RTACX_CUDA(cudaStreamCreateWithFlags(&c.copy_stream, cudaStreamNonBlocking));
    for(cudaEvent_t& e : c.stream_ev)
        if(!e) RTACX_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    const size_t stage = (size_t)RTACX_STREAM_CHUNK * record_bytes;
    if(c.stage_bytes < stage) {
        for(unsigned char*& p : c.d_stage) { if(p) cudaFree(p); p = nullptr; }
        c.stage_bytes = 0;
        for(unsigned char*& p : c.d_stage) RTACX_CUDA(cudaMalloc(&p, stage));
        c.stage_bytes = stage;
    }
    const size_t ping = (size_t)c.nR * c.nB * 2;
    if(c.ping_floats < ping) {
        if(c.d_ping) cudaFree(c.d_ping);
        c.d_ping = nullptr;
        c.ping_floats = 0;
        RTACX_CUDA(cudaMalloc(&c.d_ping, ping * sizeof(float)));
        c.ping_floats = ping;
    }
    return RTACX_OK;
}

} // namespace

void free_streaming(Context& c)
{
    for(unsigned char*& p : c.d_stage) { if(p) cudaFree(p); p = nullptr; }
    c.stage_bytes = 0;
    if(c.d_ping) cudaFree(c.d_ping);
    c.d_ping = nullptr;
    c.ping_floats = 0;
    for(cudaEvent_t& e : c.stream_ev) { if(e) cudaEventDestroy(e); e = nullptr; }
    if(c.copy_stream) cudaStreamDestroy(c.copy_stream);
    c.copy_stream = nullptr;
}

rtacx_status reduce_precision_host(Context& c, const void* samples, uint64_t n, float* out, cudaStream_t s)
{
    const size_t rec = (size_t)c.bin.stride * sizeof(float);
    rtacx_status st = ensure_streaming(c, rec);
    if(st != RTACX_OK) return st;
    c.bin.vec4 = c.bin.stride == 4 ? 1 : 0;        // staging buffers are 256-byte aligned
    const unsigned char* host = static_cast<const unsigned char*>(samples);
    cudaEvent_t fork = c.stream_ev[0], copied[2] = {c.stream_ev[1], c.stream_ev[2]},
                used[2] = {c.stream_ev[3], c.stream_ev[4]};

    c.mark(5, false, s);
    if((st = precision_begin(c, s)) != RTACX_OK) return st;
    c.mark(5, true, s);
    c.mark(0, false, s);
    RTACX_CUDA(cudaEventRecord(fork, s));
    RTACX_CUDA(cudaStreamWaitEvent(c.copy_stream, fork, 0));
    const uint64_t chunks = (n + RTACX_STREAM_CHUNK - 1) / RTACX_STREAM_CHUNK;
    for(uint64_t i = 0; i < chunks; i++) {
        const int b = (int)(i & 1);
        const uint64_t first = i * (uint64_t)RTACX_STREAM_CHUNK;
        const uint64_t cnt = std::min<uint64_t>(RTACX_STREAM_CHUNK, n - first);
        if(i >= 2) RTACX_CUDA(cudaStreamWaitEvent(c.copy_stream, used[b], 0));
        RTACX_CUDA(cudaMemcpyAsync(c.d_stage[b], host + first * rec, cnt * rec, cudaMemcpyHostToDevice, c.copy_stream));
        RTACX_CUDA(cudaEventRecord(copied[b], c.copy_stream));
        RTACX_CUDA(cudaStreamWaitEvent(s, copied[b], 0));
        if(i == 0 && (st = precision_hot_scan(c, c.d_stage[0], cnt, s)) != RTACX_OK) return st;
        if((st = precision_accumulate(c, c.d_stage[b], cnt, s)) != RTACX_OK) return st;
        RTACX_CUDA(cudaEventRecord(used[b], s));
    }
    if(chunks == 0 && (st = precision_hot_scan(c, nullptr, 0, s)) != RTACX_OK) return st;
    if(chunks == 0) {   // join the forked copy stream
        RTACX_CUDA(cudaEventRecord(copied[0], c.copy_stream));
        RTACX_CUDA(cudaStreamWaitEvent(s, copied[0], 0));
    }
    c.mark(0, true, s);
    if((st = precision_finish(c, c.d_ping, s)) != RTACX_OK) return st;
    RTACX_CUDA(cudaMemcpyAsync(out, c.d_ping, (size_t)c.nR * c.nB * 2 * sizeof(float), cudaMemcpyDeviceToHost, s));
    return RTACX_OK;
}

} // namespace rtacx

using namespace rtacx;

extern "C" rtacx_status rtacx_reduce_precision_host(rtacx_ctx* ctx, const void* samples, uint64_t n, float* out,
                                                    void* stream)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    Context& c = ctx->impl;
    if(!c.prec_configured) { c.error = "call rtacx_configure_precision first"; return RTACX_ERR_NOT_CONFIGURED; }
    if(!out) { c.error = "null output buffer"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(n && !samples) { c.error = "null sample buffer"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(n >= (1ull << 32)) { c.error = "at most 2^32 - 1 samples per ping"; return RTACX_ERR_UNSUPPORTED; }
    if(cudaSetDevice(c.device) != cudaSuccess) { cudaGetLastError(); c.error = "cudaSetDevice failed"; return RTACX_ERR_CUDA; }
    for(bool& t : c.traced) t = false;
    return reduce_precision_host(c, samples, n, out, static_cast<cudaStream_t>(stream));
}
