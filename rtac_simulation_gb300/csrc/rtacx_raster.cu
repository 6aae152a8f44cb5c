// Rasterised echo samples: the OpenGL ray caster's shader math on CUDA.
//
// The reference's GL path (src/RayCasterGL.cpp:5-63, src/SimulationGL.cu:
// 82-171) draws the mesh from the sensor, runs this fragment arithmetic per
// pixel and copies the RGBA float framebuffer into the receiver's SimSample2D
// buffer:
//   vertex:   clip = worldToScreen (p, 1); delta = (worldToLocal (p - origin, 0)).xyz
//             reflected = |normalize((worldToLocal (n, 0)).xyz).z|
//   fragment: a = reflected / |delta|^2; range = |delta|
//             bearing = atan(delta.x, -delta.z); elevation = atan(delta.y, -delta.z)
//             phase = range * 4 pi f / c + pi / 2; a /= cos(bearing) cos(elevation)
//             out = (a cos phase, a sin phase, range, bearing)
// No graphics stack is needed here. The rasteriser:
//   k_rast_vertices   transform, snap window coordinates to 1/256 pixel
//   k_rast_triangles  integer edge functions (exact coverage, top-left rule),
//                     depth test as a 64-bit atomicMin of (depth, triangle)
//                     into a visibility buffer; large triangles go to a list
//   k_rast_large      one CTA per large triangle
//   k_rast_resolve    per pixel: perspective-correct interpolation of the
//                     winning triangle's varyings, the fragment arithmetic
//                     (phase reduced in FP64), one float4 sample per pixel,
//                     rows bottom-up as glReadPixels returns them.
// Triangles with a vertex behind the eye (w <= 1e-6) or outside a +/-64 NDC
// guard band are skipped (the GL pipeline would clip them).
#include "rtacx_internal.cuh"

#include <cmath>

namespace rtacx {

namespace {

constexpr unsigned long long kEmpty = 0xFFFFFFFFFFFFFFFFull;
constexpr int kSub = 256;                 // sub-pixel steps per pixel
constexpr uint32_t kSmallPixels = 256;    // bbox pixels a single thread rasterises

// The receiver-frame delta is kept in FP64: the carrier phase multiplies the
// range by 2 f / c (1600 cycles per metre at 1.2 MHz), so float deltas alone
// would move the phase by ~1e-2 rad at 20 m.
struct RasterVertex {
    int X, Y;             // window coordinates x 256
    float z;              // NDC depth
    float inv_w;
    double dx, dy, dz;    // delta (receiver frame)
    float refl;           // reflected
    float pad;
};
static_assert(sizeof(RasterVertex) == 48, "vertex record");

struct RasterParams {
    float L[16], S[16];
    float origin[3];
    int width, height;
    double cycles;      // 2 f / c
    uint32_t n_vertices, n_triangles;
};

__global__ void k_rast_vertices(const float* __restrict__ vtx, const float* __restrict__ nrm, RasterParams p,
                                RasterVertex* __restrict__ out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= p.n_vertices) return;
    // Coverage must not depend on FMA contraction: the snapped window
    // coordinates use explicitly rounded operations (restated on the host).
    const float x = vtx[3 * i], y = vtx[3 * i + 1], z = vtx[3 * i + 2];
    const float cx = fmaf(p.S[0], x, fmaf(p.S[1], y, fmaf(p.S[2], z, p.S[3])));
    const float cy = fmaf(p.S[4], x, fmaf(p.S[5], y, fmaf(p.S[6], z, p.S[7])));
    const float cz = fmaf(p.S[8], x, fmaf(p.S[9], y, fmaf(p.S[10], z, p.S[11])));
    const float cw = fmaf(p.S[12], x, fmaf(p.S[13], y, fmaf(p.S[14], z, p.S[15])));
    RasterVertex v;
    v.inv_w = 0.0f;
    v.X = v.Y = 0;
    v.z = 0.0f;
    if(cw > 1.0e-6f) {
        const float iw = __fdiv_rn(1.0f, cw);
        const float nx = __fmul_rn(cx, iw), ny = __fmul_rn(cy, iw);
        if(fabsf(nx) <= 64.0f && fabsf(ny) <= 64.0f) {
            v.inv_w = iw;
            v.X = __float2int_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.0f), 0.5f), (float)p.width), (float)kSub));
            v.Y = __float2int_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fadd_rn(ny, 1.0f), 0.5f), (float)p.height), (float)kSub));
            v.z = __fmul_rn(cz, iw);
        }
    }
    const double ox = (double)x - p.origin[0], oy = (double)y - p.origin[1], oz = (double)z - p.origin[2];
    v.dx = (double)p.L[0] * ox + (double)p.L[1] * oy + (double)p.L[2] * oz;
    v.dy = (double)p.L[4] * ox + (double)p.L[5] * oy + (double)p.L[6] * oz;
    v.dz = (double)p.L[8] * ox + (double)p.L[9] * oy + (double)p.L[10] * oz;
    v.pad = 0.0f;
    const float n0 = nrm[3 * i], n1 = nrm[3 * i + 1], n2 = nrm[3 * i + 2];
    const float mx = p.L[0] * n0 + p.L[1] * n1 + p.L[2] * n2;
    const float my = p.L[4] * n0 + p.L[5] * n1 + p.L[6] * n2;
    const float mz = p.L[8] * n0 + p.L[9] * n1 + p.L[10] * n2;
    v.refl = fabsf(mz * rsqrtf(mx * mx + my * my + mz * mz));
    out[i] = v;
}

struct Tri {
    long long X[3], Y[3];
    float z[3];
    long long area;
    float gx, gy, d0;     // depth plane: depth = d0 + gx (px - X0) + gy (py - Y0)
    bool ok;
};

// Depth plane of a triangle, anchored at vertex 0. The window depth
// 0.5 zn + 0.5, with zn the barycentric interpolation of the vertices' NDC
// depths (e0 z0 + e1 z1 + e2 z2) / (e0 + e1 + e2), is linear in the pixel
// position; its slopes and its value at vertex 0 are formed once per
// triangle in float with explicitly rounded operations (the coordinate
// differences are integers below 2^24, exact in float), so each pixel
// evaluates it with two float FMAs; the host oracle restates the same
// operations. o1, o2: the CCW order of vertices 1 and 2.
__device__ __forceinline__ void depth_plane(Tri& T, int o1, int o2)
{
    const float A = __ll2float_rn(T.area > 0 ? T.area : -T.area);
    const float z0 = T.z[0], z1 = T.z[o1], z2 = T.z[o2];
    const float dy21 = (float)(T.Y[o2] - T.Y[o1]), dy02 = (float)(T.Y[0] - T.Y[o2]), dy10 = (float)(T.Y[o1] - T.Y[0]);
    const float dx21 = (float)(T.X[o2] - T.X[o1]), dx02 = (float)(T.X[0] - T.X[o2]), dx10 = (float)(T.X[o1] - T.X[0]);
    const float sx = __fadd_rn(__fadd_rn(__fmul_rn(dy21, z0), __fmul_rn(dy02, z1)), __fmul_rn(dy10, z2));
    const float sy = __fadd_rn(__fadd_rn(__fmul_rn(dx21, z0), __fmul_rn(dx02, z1)), __fmul_rn(dx10, z2));
    T.gx = __fmul_rn(-0.5f, __fdiv_rn(sx, A));
    T.gy = __fmul_rn(0.5f, __fdiv_rn(sy, A));
    T.d0 = __fadd_rn(__fmul_rn(0.5f, z0), 0.5f);
}

__device__ __forceinline__ Tri load_tri(const RasterVertex* __restrict__ V, const uint32_t* __restrict__ tris, uint32_t t,
                                        uint32_t nv)
{
    Tri T;
    T.ok = false;
    uint32_t id[3] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
    for(int k = 0; k < 3; k++) {
        if(id[k] >= nv) return T;
        const RasterVertex v = V[id[k]];
        if(!(v.inv_w > 0.0f)) return T;
        T.X[k] = v.X; T.Y[k] = v.Y; T.z[k] = v.z;
    }
    T.area = (T.X[1] - T.X[0]) * (T.Y[2] - T.Y[0]) - (T.Y[1] - T.Y[0]) * (T.X[2] - T.X[0]);
    T.ok = T.area != 0;
    if(T.ok) depth_plane(T, T.area > 0 ? 1 : 2, T.area > 0 ? 2 : 1);
    return T;
}

// Edge function of edge a -> b at point (px, py), positive inside a CCW triangle.
__device__ __forceinline__ long long edge(long long ax, long long ay, long long bx, long long by, long long px, long long py)
{
    return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
}

// Top-left rule for a CCW triangle in y-up window coordinates.
__device__ __forceinline__ bool top_left(long long ax, long long ay, long long bx, long long by)
{
    const long long dx = bx - ax, dy = by - ay;
    return (dy == 0 && dx < 0) || dy < 0;
}

// Coverage and depth of pixel (i, j); returns the packed visibility word or
// kEmpty. Vertex order is made CCW by the caller (sign of area).
__device__ __forceinline__ unsigned long long shade_test(const Tri& T, int o0, int o1, int o2, int i, int j, uint32_t t)
{
    const long long px = (long long)i * kSub + kSub / 2, py = (long long)j * kSub + kSub / 2;
    const long long e0 = edge(T.X[o1], T.Y[o1], T.X[o2], T.Y[o2], px, py);
    const long long e1 = edge(T.X[o2], T.Y[o2], T.X[o0], T.Y[o0], px, py);
    const long long e2 = edge(T.X[o0], T.Y[o0], T.X[o1], T.Y[o1], px, py);
    if(e0 < 0 || e1 < 0 || e2 < 0) return kEmpty;
    if(e0 == 0 && !top_left(T.X[o1], T.Y[o1], T.X[o2], T.Y[o2])) return kEmpty;
    if(e1 == 0 && !top_left(T.X[o2], T.Y[o2], T.X[o0], T.Y[o0])) return kEmpty;
    if(e2 == 0 && !top_left(T.X[o0], T.Y[o0], T.X[o1], T.Y[o1])) return kEmpty;
    const float d = fmaf(T.gx, (float)(px - T.X[0]), fmaf(T.gy, (float)(py - T.Y[0]), T.d0));
    if(!(d >= 0.0f && d <= 1.0f)) return kEmpty;
    return ((unsigned long long)__float_as_uint(d) << 32) | t;
}

__device__ __forceinline__ void tri_bbox(const Tri& T, int width, int height, int& i0, int& i1, int& j0, int& j1)
{
    const long long minX = min(T.X[0], min(T.X[1], T.X[2])), maxX = max(T.X[0], max(T.X[1], T.X[2]));
    const long long minY = min(T.Y[0], min(T.Y[1], T.Y[2])), maxY = max(T.Y[0], max(T.Y[1], T.Y[2]));
    // pixel i has its centre at i * 256 + 128
    i0 = (int)max(0ll, (minX - kSub / 2 + kSub - 1) / kSub);
    i1 = (int)min((long long)width - 1, (maxX - kSub / 2) >= 0 ? (maxX - kSub / 2) / kSub : -1ll);
    j0 = (int)max(0ll, (minY - kSub / 2 + kSub - 1) / kSub);
    j1 = (int)min((long long)height - 1, (maxY - kSub / 2) >= 0 ? (maxY - kSub / 2) / kSub : -1ll);
}

__global__ void k_rast_triangles(const RasterVertex* __restrict__ V, const uint32_t* __restrict__ tris, RasterParams p,
                                 unsigned long long* __restrict__ vis, uint32_t* __restrict__ large,
                                 uint32_t* __restrict__ n_large)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= p.n_triangles) return;
    const Tri T = load_tri(V, tris, t, p.n_vertices);
    if(!T.ok) return;
    int i0, i1, j0, j1;
    tri_bbox(T, p.width, p.height, i0, i1, j0, j1);
    if(i0 > i1 || j0 > j1) return;
    if((uint64_t)(i1 - i0 + 1) * (uint64_t)(j1 - j0 + 1) > kSmallPixels) {
        large[atomicAdd(n_large, 1u)] = t;
        return;
    }
    const int o1 = T.area > 0 ? 1 : 2, o2 = T.area > 0 ? 2 : 1;
    for(int j = j0; j <= j1; j++)
        for(int i = i0; i <= i1; i++) {
            const unsigned long long w = shade_test(T, 0, o1, o2, i, j, t);
            if(w != kEmpty) atomicMin(&vis[(size_t)j * p.width + i], w);
        }
}

__global__ void k_rast_large(const RasterVertex* __restrict__ V, const uint32_t* __restrict__ tris, RasterParams p,
                             unsigned long long* __restrict__ vis, const uint32_t* __restrict__ large,
                             const uint32_t* __restrict__ n_large)
{
    for(uint32_t q = blockIdx.x; q < *n_large; q += gridDim.x) {
        const uint32_t t = large[q];
        const Tri T = load_tri(V, tris, t, p.n_vertices);
        int i0, i1, j0, j1;
        tri_bbox(T, p.width, p.height, i0, i1, j0, j1);
        const int o1 = T.area > 0 ? 1 : 2, o2 = T.area > 0 ? 2 : 1;
        const int w = i1 - i0 + 1;
        const long long count = (long long)w * (j1 - j0 + 1);
        for(long long k = threadIdx.x; k < count; k += blockDim.x) {
            const int i = i0 + (int)(k % w), j = j0 + (int)(k / w);
            const unsigned long long v = shade_test(T, 0, o1, o2, i, j, t);
            if(v != kEmpty) atomicMin(&vis[(size_t)j * p.width + i], v);
        }
    }
}

__global__ void k_rast_resolve(const RasterVertex* __restrict__ V, const uint32_t* __restrict__ tris, RasterParams p,
                               const unsigned long long* __restrict__ vis, float4* __restrict__ out)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if(idx >= (uint32_t)(p.width * p.height)) return;
    const unsigned long long w = vis[idx];
    float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
    if(w != kEmpty) {
        const uint32_t t = (uint32_t)(w & 0xFFFFFFFFu);
        const int i = idx % p.width, j = idx / p.width;
        const uint32_t id[3] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
        const RasterVertex a = V[id[0]], b = V[id[1]], c = V[id[2]];
        const long long px = (long long)i * kSub + kSub / 2, py = (long long)j * kSub + kSub / 2;
        const double l0 = (double)edge(b.X, b.Y, c.X, c.Y, px, py);
        const double l1 = (double)edge(c.X, c.Y, a.X, a.Y, px, py);
        const double l2 = (double)edge(a.X, a.Y, b.X, b.Y, px, py);
        // perspective-correct weights, normalised by one reciprocal; the
        // receiver-frame delta in FP64 (the carrier phase needs the range to
        // ~1e-8 relative), the reflectance in float
        const double w0 = l0 * a.inv_w, w1 = l1 * b.inv_w, w2 = l2 * c.inv_w;
        const double rs = __drcp_rn(w0 + w1 + w2);
        const double b0 = w0 * rs, b1 = w1 * rs, b2 = w2 * rs;
        const double dx = fma(b0, a.dx, fma(b1, b.dx, b2 * c.dx));
        const double dy = fma(b0, a.dy, fma(b1, b.dy, b2 * c.dy));
        const double dz = fma(b0, a.dz, fma(b1, b.dz, b2 * c.dz));
        const float refl = fmaf((float)b0, a.refl, fmaf((float)b1, b.refl, (float)b2 * c.refl));
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double range = sqrt(r2);
        const float fx = (float)dx, fy = (float)dy, fz = (float)dz;
        const float bearing = atan2f(fx, -fz);
        const float elevation = atan2f(fy, -fz);
        // phase = range * 4 pi f / c + pi / 2, reduced modulo one cycle in FP64
        const double cyc = range * p.cycles + 0.25;
        const float frac = (float)(cyc - rint(cyc));
        float sn, cs;
        sincosf(frac * 6.28318530717958647692f, &sn, &cs);
        const float amp = refl / (float)r2 / cosf(bearing) / cosf(elevation);
        res = make_float4(amp * cs, amp * sn, (float)range, bearing);
    }
    out[idx] = res;
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
bool grow(Context& ctx, T*& p, size_t& cap, size_t n)
{
    if(n <= cap) return true;
    T* q = nullptr;
    if(cudaMalloc(&q, n * sizeof(T)) != cudaSuccess) { cudaGetLastError(); return ctx.fail("cudaMalloc failed"); }
    if(p) cudaFree(p);
    p = q;
    cap = n;
    return true;
}

} // namespace

rtacx_status rasterize(Context& ctx, const rtacx_mesh* m, const rtacx_raster_view* v, float* samples, cudaStream_t s)
{
    if(!m || !v || !samples) { ctx.error = "null argument"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(!m->vertices || !m->normals || !m->triangles || m->n_vertices == 0 || m->n_triangles == 0) {
        ctx.error = "empty mesh";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    if(v->width == 0 || v->height == 0 || (uint64_t)v->width * v->height > (1u << 26)) {
        ctx.error = "render target must be 1 .. 2^26 pixels";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    if(v->width > (1u << 16) || v->height > (1u << 16)) { ctx.error = "render target side above 65536"; return RTACX_ERR_UNSUPPORTED; }
    if(!(v->sound_celerity > 0.0f) || !(v->carrier_hz >= 0.0)) { ctx.error = "bad carrier / celerity"; return RTACX_ERR_INVALID_ARGUMENT; }
    if(reinterpret_cast<uintptr_t>(samples) % 16) { ctx.error = "samples must be 16-byte aligned"; return RTACX_ERR_INVALID_ARGUMENT; }
    RasterParams p{};
    for(int k = 0; k < 16; k++) { p.L[k] = v->world_to_local[k]; p.S[k] = v->world_to_screen[k]; }
    for(int k = 0; k < 3; k++) p.origin[k] = v->origin[k];
    p.width = (int)v->width; p.height = (int)v->height;
    p.cycles = 2.0 * v->carrier_hz / (double)v->sound_celerity;
    p.n_vertices = m->n_vertices; p.n_triangles = m->n_triangles;
    const size_t pixels = (size_t)v->width * v->height;
    if(!grow(ctx, ctx.d_rast_v, ctx.rast_v_cap, m->n_vertices * sizeof(RasterVertex)) ||
       !grow(ctx, ctx.d_rast_vis, ctx.rast_vis_cap, pixels) ||
       !grow(ctx, ctx.d_rast_large, ctx.rast_large_cap, (size_t)m->n_triangles + 1))
        return RTACX_ERR_OUT_OF_MEMORY;
    RasterVertex* V = reinterpret_cast<RasterVertex*>(ctx.d_rast_v);
    uint32_t* n_large = ctx.d_rast_large + m->n_triangles;
    RTACX_CUDA(cudaMemsetAsync(ctx.d_rast_vis, 0xFF, pixels * sizeof(unsigned long long), s));
    RTACX_CUDA(cudaMemsetAsync(n_large, 0, sizeof(uint32_t), s));
    k_rast_vertices<<<(m->n_vertices + 255) / 256, 256, 0, s>>>(m->vertices, m->normals, p, V);
    k_rast_triangles<<<(m->n_triangles + 255) / 256, 256, 0, s>>>(V, m->triangles, p, ctx.d_rast_vis, ctx.d_rast_large,
                                                                  n_large);
    k_rast_large<<<ctx.sm_count * 4, 256, 0, s>>>(V, m->triangles, p, ctx.d_rast_vis, ctx.d_rast_large, n_large);
    k_rast_resolve<<<(uint32_t)((pixels + 255) / 256), 256, 0, s>>>(V, m->triangles, p, ctx.d_rast_vis,
                                                                     reinterpret_cast<float4*>(samples));
    RTACX_CUDA(cudaGetLastError());
    return RTACX_OK;
}

} // namespace rtacx

extern "C" rtacx_status rtacx_rasterize(rtacx_ctx* ctx, const rtacx_mesh* mesh, const rtacx_raster_view* view,
                                        float* samples, void* stream)
{
    if(!ctx) return RTACX_ERR_INVALID_ARGUMENT;
    if(cudaSetDevice(ctx->impl.device) != cudaSuccess) { cudaGetLastError(); return RTACX_ERR_CUDA; }
    return rtacx::rasterize(ctx->impl, mesh, view, samples, static_cast<cudaStream_t>(stream));
}
