// Echo-sample epilogue and receiver directivity tables on the device.
//
// k_make_samples restates, per ray-cast hit, what the reference's ray
// generator and receiver do before the receiver path starts
// (src/RayCaster.cu:49-81, include/rtac_simulation/Receiver.h:51-60,
// include/rtac_simulation/Sample.h:144-153):
//   distance < 1e-4          -> null sample (value 0, travel -1)
//   value *= exp(i 4 pi f d / c) / d^2        (carrier phase reduced by one
//                                              FP64 fused multiply-add)
//   localDir = R^T * dir                      (receiver frame)
//   value *= directivity(atan2(ly, lx) / pi, atan2(lz, lx) / pi)
//   bearing = atan2(-ly, lx)
// The directivity lookup is the reference's float texture with normalized
// coordinates, linear filtering and mirror addressing
// (src/Directivity.cpp:21-25, include/rtac_simulation/Directivity.h:30-34),
// evaluated with exact bilinear weights.
//
// k_directivity_rect / k_directivity_disk build the receiver directivity
// tables of Directivity::rectangle_antenna / disk_antenna
// (src/Directivity.cpp:59-101, 109-166) on the device, with the reference's float /
// double arithmetic.
#include "rtacx_internal.cuh"

#include <cmath>
#include <vector>

namespace rtacx {

namespace {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ float mirror_coord(float u)
{
    const float t = u - 2.0f * floorf(0.5f * u);   // [0, 2)
    return t <= 1.0f ? t : 2.0f - t;
}

__device__ __forceinline__ int mirror_index(int i, int n)
{
    if(i < 0) return min(-i - 1, n - 1);
    if(i >= n) return max(2 * n - i - 1, 0);
    return i;
}

// Bilinear lookup of a [h][w] table at normalized (u, v), mirror addressing.
__device__ __forceinline__ float directivity_lookup(const float* __restrict__ tab, int w, int h, float u, float v)
{
    const float x = mirror_coord(u) * (float)w - 0.5f, y = mirror_coord(v) * (float)h - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    const int x0 = mirror_index((int)fx, w), x1 = mirror_index((int)fx + 1, w);
    const int y0 = mirror_index((int)fy, h), y1 = mirror_index((int)fy + 1, h);
    const float t00 = __ldg(tab + (size_t)y0 * w + x0), t01 = __ldg(tab + (size_t)y0 * w + x1);
    const float t10 = __ldg(tab + (size_t)y1 * w + x0), t11 = __ldg(tab + (size_t)y1 * w + x1);
    const float top = fmaf(ax, t01 - t00, t00), bot = fmaf(ax, t11 - t10, t10);
    return fmaf(ay, bot - top, top);
}

struct ReceiverParams {
    float R[9];                 // row-major, world = R * receiver
    int dir_w, dir_h;           // 0: uniform directivity
    uint32_t flags;
    double cycles;              // 2 f / c
    float cycles_hi;            // (float)cycles
    int dims;
};

__global__ void k_make_samples(const rtacx_echo* __restrict__ hits, uint64_t n, ReceiverParams rp,
                               const float* __restrict__ dir_tab, float* __restrict__ out)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for(uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        const rtacx_echo e = hits[i];
        float re = 0.0f, im = 0.0f, travel = -1.0f, bearing = 0.0f;
        const float d = e.distance;
        if(d >= 1.0e-4f) {
            float2 v = make_float2(e.re, e.im);
            if(rp.flags & RTACX_ECHO_PHASE) {
                // Below 2^22 cycles the float-rounded cycle count is within
                // one of the nearest integer and the one-FMA reduction lands in
                // [-0.5, 0.5]; longer (or infinite) travels take the full FP64
                // reduction. |phase| <= pi: the hardware sine / cosine are
                // accurate to ~4e-7 there.
                float frac;
                if(d * rp.cycles_hi < 4194304.0f) frac = carrier_fraction_f64(d, rp.cycles, rp.cycles_hi);
                else {
                    const double cyc = (double)d * rp.cycles;
                    frac = (float)(cyc - rint(cyc));
                }
                float sn, cs;
                __sincosf(frac * 6.28318530717958647692f, &sn, &cs);
                v = make_float2(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
            }
            if(rp.flags & RTACX_ECHO_SPREADING) {
                const float inv = __fdividef(1.0f, d * d);
                v = make_float2(v.x * inv, v.y * inv);
            }
            // receiver frame: R^T * dir (column k of R dotted with dir)
            const float lx = fmaf(rp.R[0], e.dir_x, fmaf(rp.R[3], e.dir_y, rp.R[6] * e.dir_z));
            const float ly = fmaf(rp.R[1], e.dir_x, fmaf(rp.R[4], e.dir_y, rp.R[7] * e.dir_z));
            const float lz = fmaf(rp.R[2], e.dir_x, fmaf(rp.R[5], e.dir_y, rp.R[8] * e.dir_z));
            // atan2 is odd in its first argument: atan2(-ly, lx) = -atan2(ly, lx).
            const float az = atan2f(ly, lx);
            if(rp.dir_w > 0) {
                const float g = directivity_lookup(dir_tab, rp.dir_w, rp.dir_h, az * 0.318309886183790671538f,
                                                   atan2f(lz, lx) * 0.318309886183790671538f);
                v = make_float2(v.x * g, v.y * g);
            }
            re = v.x; im = v.y; travel = d;
            bearing = -az;
        }
        if(rp.dims == 2) reinterpret_cast<float4*>(out)[i] = make_float4(re, im, travel, bearing);
        else { out[3 * i] = re; out[3 * i + 1] = im; out[3 * i + 2] = travel; }
    }
}

__global__ void k_directivity_rect(float width, float height, float wavelength, int baffle, uint32_t Nw, uint32_t Nh,
                                   float* __restrict__ out)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if(idx >= Nw * Nh) return;
    const uint32_t h = idx / Nw, w = idx % Nw;
    const double elevation = kPi * h / Nh;
    const double ke = kPi * (double)height / (double)wavelength;
    float eValue = (float)(sin(ke * sin(elevation)) / (ke * sin(elevation)));
    if(h == 0) eValue = 1.0f;
    const double bearing = kPi * w / Nw;
    const double kb = kPi * (double)width / (double)wavelength;
    float bValue = (float)(sin(kb * sin(bearing)) / (kb * sin(bearing)));
    if(w == 0) bValue = 1.0f;
    float v = eValue * bValue;
    if(baffle == 1 && (h > Nh / 2 || w > Nw / 2)) v = 0.0f;
    out[idx] = v;
}

__global__ void k_directivity_disk(float diameter, float wavelength, int baffle, uint32_t N, float* __restrict__ out)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if(idx >= N * N) return;
    const uint32_t h = idx / N, w = idx % N;
    const double elevation = kPi * h / N;
    double cose2 = cos(elevation); cose2 *= cose2;
    double sine2 = sin(elevation); sine2 *= sine2;
    const double bearing = kPi * w / N;
    double cosb2 = cos(bearing); cosb2 *= cosb2;
    double sinb2 = sin(bearing); sinb2 *= sinb2;
    const double denom = 1.0 - sine2 * sinb2;
    const double y2 = cose2 * sinb2 / denom, z2 = sine2 * cosb2 / denom;
    // The reference takes sqrt(1 - y2 - z2) as is: where the two terms
    // cancel (elevation or bearing at pi/2) the host libm's last bit decides
    // between a NaN and a tiny x, and 0/0 gives a NaN at (N/2, N/2). Here the
    // exact-math limit is kept instead: a degenerate x is 0 (value 0).
    const double s = 1.0 - y2 - z2;
    double x = (denom > 0.0 && s > 0.0) ? sqrt(s) : 0.0;
    float v;
    if(fabs(x) < 1.0e-2) v = 0.0f;
    else {
        if(elevation > 0.5 * kPi || bearing > (double)0.5f * kPi) x = -x;
        const double a = (kPi * (double)diameter / (double)wavelength) * sin(atan2(sqrt(y2 + z2), x));
        v = (fabs(a) < 1.0e-3) ? 1.0f : (float)(2.0 * j1(a) / a);
    }
    if(baffle == 1 && (h > N / 2 || w > N / 2)) v = 0.0f;
    out[idx] = v;
}

} // namespace

rtacx_status configure_receiver(Context& c, const rtacx_receiver* r)
{
    if(!c.configured) { c.error = "configure the sensor first"; return RTACX_ERR_NOT_CONFIGURED; }
    if(!r) { c.error = "null receiver"; return RTACX_ERR_INVALID_ARGUMENT; }
    for(float v : r->rotation) if(!std::isfinite(v)) { c.error = "non-finite rotation"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(r->flags & ~(RTACX_ECHO_PHASE | RTACX_ECHO_SPREADING)) { c.error = "unknown echo flags"; return RTACX_ERR_INVALID_ARGUMENT; }
    if((r->flags & RTACX_ECHO_PHASE) && !(std::isfinite(r->carrier_hz) && r->carrier_hz > 0.0)) {
        c.error = "carrier_hz must be positive"; return RTACX_ERR_INVALID_ARGUMENT;
    }
    if(c.d_dir) { cudaFree(c.d_dir); c.d_dir = nullptr; }
    c.dir_w = c.dir_h = 0;
    if(r->directivity) {
        if(r->directivity_width == 0 || r->directivity_height == 0) { c.error = "empty directivity table"; return RTACX_ERR_INVALID_ARGUMENT; }
        // Entries are used as given: the reference's disk_antenna table holds
        // a NaN at (N/2, N/2) and propagates it to the hits that sample it.
        const size_t cnt = (size_t)r->directivity_width * r->directivity_height;
        if(cudaMalloc(&c.d_dir, cnt * sizeof(float)) != cudaSuccess ||
           cudaMemcpy(c.d_dir, r->directivity, cnt * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            c.error = "uploading the directivity table failed";
            return RTACX_ERR_OUT_OF_MEMORY;
        }
        c.dir_w = r->directivity_width; c.dir_h = r->directivity_height;
    }
    std::copy(r->rotation, r->rotation + 9, c.rx_rotation);
    c.rx_flags = r->flags;
    c.rx_hz = (r->flags & RTACX_ECHO_PHASE) ? r->carrier_hz : 0.0;
    c.rx_configured = true;
    return RTACX_OK;
}

rtacx_status make_samples(Context& c, const rtacx_echo* hits, uint64_t n, void* samples, cudaStream_t stream)
{
    if(!c.rx_configured) { c.error = "call rtacx_configure_receiver first"; return RTACX_ERR_NOT_CONFIGURED; }
    if(n && (!hits || !samples)) { c.error = "null buffer"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(c.dims == 2 && reinterpret_cast<uintptr_t>(samples) % 16) { c.error = "2D samples must be 16-byte aligned"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(reinterpret_cast<uintptr_t>(hits) % 4) { c.error = "hits must be 4-byte aligned"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(!n) return RTACX_OK;
    ReceiverParams rp{};
    std::copy(c.rx_rotation, c.rx_rotation + 9, rp.R);
    rp.dir_w = (int)c.dir_w; rp.dir_h = (int)c.dir_h;
    rp.flags = c.rx_flags;
    rp.cycles = 2.0 * c.rx_hz / (double)c.c;
    rp.cycles_hi = (float)rp.cycles;
    rp.dims = c.dims;
    const uint32_t blocks = (uint32_t)std::min<uint64_t>((n + 255) / 256, (uint64_t)c.sm_count * 16);
    k_make_samples<<<blocks, 256, 0, stream>>>(hits, n, rp, c.d_dir, static_cast<float*>(samples));
    const cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) { c.error = std::string("k_make_samples: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    return RTACX_OK;
}

} // namespace rtacx

using namespace rtacx;

extern "C" rtacx_status rtacx_directivity_table(int kind, const float* params, float* out, uint32_t* width,
                                                uint32_t* height, void* stream)
{
    if(!params || !width || !height) return RTACX_ERR_INVALID_ARGUMENT;
    // Table sides are formed in double and bounded before the conversion to
    // unsigned (an out-of-range conversion is undefined): at most 2^26 texels.
    constexpr double kMaxSide = (double)(1u << 26);
    uint32_t W, H;
    if(kind == RTACX_DIRECTIVITY_RECTANGLE) {
        const float w = params[0], h = params[1], l = params[2], os = params[4];
        if(!(w > 0.0f && h > 0.0f && l > 0.0f && os >= 1.0f)) return RTACX_ERR_INVALID_ARGUMENT;
        if(!(os < 65536.0f)) return RTACX_ERR_UNSUPPORTED;
        const unsigned int o = (unsigned int)os;
        // Nw = 2 * (unsigned)(0.5f * oversampling * 2 * M_PI * width / wavelength + 1)
        const double hw = (double)(0.5f * o * 2) * kPi * w / l + 1, hh = (double)(0.5f * o * 2) * kPi * h / l + 1;
        if(!(hw < kMaxSide && hh < kMaxSide)) return RTACX_ERR_UNSUPPORTED;
        W = 2u * (unsigned int)hw;
        H = 2u * (unsigned int)hh;
    }
    else if(kind == RTACX_DIRECTIVITY_DISK) {
        const float dia = params[0], l = params[1], os = params[3];
        if(!(dia > 0.0f && l > 0.0f && os >= 1.0f)) return RTACX_ERR_INVALID_ARGUMENT;
        if(!(os < 65536.0f)) return RTACX_ERR_UNSUPPORTED;
        const float period = 2.0f * l / dia;
        const double q = (unsigned int)os * kPi / period;
        if(!(q < kMaxSide)) return RTACX_ERR_UNSUPPORTED;
        W = H = std::max(64u, 8u * (unsigned int)q);
    }
    else return RTACX_ERR_INVALID_ARGUMENT;
    if((uint64_t)W * H > (1u << 26)) return RTACX_ERR_UNSUPPORTED;
    *width = W; *height = H;
    if(!out) return RTACX_OK;
    const int baffle = (kind == RTACX_DIRECTIVITY_RECTANGLE) ? (int)params[3] : (int)params[2];
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t blocks = (W * H + 255) / 256;
    if(kind == RTACX_DIRECTIVITY_RECTANGLE)
        k_directivity_rect<<<blocks, 256, 0, s>>>(params[0], params[1], params[2], baffle, W, H, out);
    else
        k_directivity_disk<<<blocks, 256, 0, s>>>(params[0], params[1], baffle, W, out);
    return cudaGetLastError() == cudaSuccess ? RTACX_OK : RTACX_ERR_CUDA;
}

extern "C" rtacx_status rtacx_configure_receiver(rtacx_ctx* ctx, const rtacx_receiver* r)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    if(cudaSetDevice(ctx->impl.device) != cudaSuccess) { cudaGetLastError(); return RTACX_ERR_CUDA; }
    return configure_receiver(ctx->impl, r);
}

extern "C" rtacx_status rtacx_make_samples(rtacx_ctx* ctx, const rtacx_echo* hits, uint64_t n, void* samples,
                                           void* stream)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    if(cudaSetDevice(ctx->impl.device) != cudaSuccess) { cudaGetLastError(); return RTACX_ERR_CUDA; }
    return make_samples(ctx->impl, hits, n, samples, static_cast<cudaStream_t>(stream));
}
