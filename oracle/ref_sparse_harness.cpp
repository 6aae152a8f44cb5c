// Launch harness for the reference's own 2D reduction kernel
// (do_sparse_convolve_2d_f, src/SensorInstance2D.cu:44-83), compiled by
// oracle/ref_build.sh into oracle/_ref/ref_sparse2d.cubin against the
// stand-ins of oracle/ref_stubs_cuda. Test infrastructure only: it records
// golden pings (tests/golden/make_ref_pings.py); nothing in the library uses
// it.
//
// The harness does what SensorInstance2D::do_reduce (src/SensorInstance2D.cu:
// 85-104) and the sensor set-up do around the kernel:
//   * the PSF texture of generate_psf_data (src/SensorInstance2D.cu:20-33):
//     a W x H float2 image, linear filter, border addressing, normalized
//     coordinates (src/SensorInstance2D.cu:14-15);
//   * KernelView2D scalings {1 / span, 0.5} and {1 / (duration c), 0.5}
//     (src/SensorInstance2D.cu:35-42);
//   * one CTA per output cell (grid nB x nR), 512 threads, 512 floats of
//     dynamic shared memory.
// Before the launch it checks every bin view against the sample buffer and
// the kernel's parameter offsets and sizes (cuFuncGetParamInfo) against its
// own argument structures.
//
// Input file (little endian): u32 magic 'RPNG', nB, nR, W, H, u64 n;
// f32 rmin, rmax, xscale, yscale; f32 bearings[nB]; float2 psf[H][W];
// f32 samples[n][4] (travel-sorted); u64 views[nR][2] {start, size}.
// Output file: float2 ping[nR][nB].
//
// With magic 'RPN1' it runs the reference's 1D kernel instead
// (do_sparse_convolve_1d_f, src/SensorInstance1D.cu:35-72, compiled into
// oracle/_ref/ref_sparse1d.cubin), launched as SensorInstance1D::do_reduce
// does (src/SensorInstance1D.cu:74-86: one 512-thread CTA per output range,
// 512 floats of dynamic shared memory). Input: u32 'RPN1', nR, H, address
// mode (0 border, 1 clamp), u64 n; f32 rmin, rmax, scaling; float2
// pulse[H]; f32 samples[n][3] (travel-sorted); u64 views[nR][2]. Output:
// float2 ping[nR]. The reference builds its pulse texture with rtac_base's
// Texture2D (a W x 1 image) and sets neither filter nor address mode
// (src/SensorInstance1D.cu:15-25), so both are rtac_base defaults, which are
// not vendored. The harness takes the texture as a 1D float2 array of the H
// taps with linear filtering and normalized coordinates (KernelView1D adds
// 0.5 to the scaled coordinate, ReductionKernel.h:44-55) and the address
// mode given; a tex1D fetch from a 2D array is not a defined combination,
// so it is not reproduced.
// With a repetition count REPS > 0 it also times the kernel: one untimed
// launch, then REPS launches between two CUDA events on the launching
// stream; it prints "ref_kernel_ms <mean per launch>".
#include <cuda.h>
#include <cuda_runtime.h>

#include <rtac_base/containers/Image.h>
#include <rtac_base/cuda/CudaVector.h>
#include <rtac_base/cuda/TextureVector.h>
#include <rtac_base/types/Complex.h>
#include <rtac_base/types/Linspace.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Sample2D { float re, im, travel, bearing; };           // SimSample2D layout
struct KernelView2DArgs { float2 x; float2 y; cudaTextureObject_t tex; };   // KernelView2D<Complex<float>> layout
static_assert(sizeof(KernelView2DArgs) == 24, "KernelView2D layout");
static_assert(sizeof(rtac::VectorView<const Sample2D>) == 16, "VectorView layout");

bool fail(const std::string& m) { std::fprintf(stderr, "ref_sparse_harness: %s\n", m.c_str()); return false; }

bool cu_ok(CUresult r, const char* what)
{
    if(r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    return fail(std::string(what) + ": " + (s ? s : "?"));
}

bool rt_ok(cudaError_t e, const char* what)
{
    return e == cudaSuccess || fail(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T> bool get(FILE* f, T* p, size_t n) { return std::fread(p, sizeof(T), n, f) == n; }

bool run_1d(const char* cubin, FILE* f, const char* out_path, int reps);

bool run(const char* cubin, const char* in_path, const char* out_path, int reps)
{
    FILE* f = std::fopen(in_path, "rb");
    if(!f) return fail("cannot open input");
    uint32_t magic = 0;
    if(!get(f, &magic, 1)) { std::fclose(f); return fail("bad header"); }
    if(magic == 0x314E5052u) return run_1d(cubin, f, out_path, reps);
    uint32_t hdr[5];
    hdr[0] = magic;
    uint64_t n = 0;
    float par[4];
    if(!get(f, hdr + 1, 4) || !get(f, &n, 1) || !get(f, par, 4) || hdr[0] != 0x474E5052u) { std::fclose(f); return fail("bad header"); }
    const uint32_t nB = hdr[1], nR = hdr[2], W = hdr[3], H = hdr[4];
    if(!nB || !nR || !W || !H || nB > 65535u || nR > 65535u || n > (1ull << 28)) { std::fclose(f); return fail("bad sizes"); }
    std::vector<float> bearings(nB);
    std::vector<float2> psf((size_t)W * H);
    std::vector<Sample2D> samples(n);
    std::vector<uint64_t> views(2 * (size_t)nR);
    const bool ok = get(f, bearings.data(), nB) && get(f, psf.data(), psf.size()) &&
                    (n == 0 || get(f, samples.data(), n)) && get(f, views.data(), views.size());
    std::fclose(f);
    if(!ok) return fail("short input");
    for(uint32_t r = 0; r < nR; r++)
        if(views[2 * r] > n || views[2 * r + 1] > n - views[2 * r]) return fail("bin view outside the samples");

    if(!rt_ok(cudaSetDevice(0), "cudaSetDevice") || !rt_ok(cudaFree(nullptr), "context")) return false;

    // PSF texture as the reference sensor configures it.
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float2>();
    cudaArray_t arr = nullptr;
    if(!rt_ok(cudaMallocArray(&arr, &ch, W, H), "cudaMallocArray") ||
       !rt_ok(cudaMemcpy2DToArray(arr, 0, 0, psf.data(), W * sizeof(float2), W * sizeof(float2), H,
                                  cudaMemcpyHostToDevice), "psf upload"))
        return false;
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeBorder;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    cudaTextureObject_t tex = 0;
    if(!rt_ok(cudaCreateTextureObject(&tex, &rd, &td, nullptr), "texture")) return false;

    float* d_bear = nullptr;
    Sample2D* d_smp = nullptr;
    rtac::VectorView<const Sample2D>* d_views = nullptr;
    float2* d_out = nullptr;
    std::vector<rtac::VectorView<const Sample2D>> hv(nR);
    if(!rt_ok(cudaMalloc(&d_bear, nB * sizeof(float)), "malloc") ||
       !rt_ok(cudaMalloc(&d_smp, (n ? n : 1) * sizeof(Sample2D)), "malloc") ||
       !rt_ok(cudaMalloc(&d_views, nR * sizeof(hv[0])), "malloc") ||
       !rt_ok(cudaMalloc(&d_out, (size_t)nR * nB * sizeof(float2)), "malloc"))
        return false;
    for(uint32_t r = 0; r < nR; r++) hv[r] = rtac::VectorView<const Sample2D>{views[2 * r + 1], d_smp + views[2 * r]};
    if(!rt_ok(cudaMemcpy(d_bear, bearings.data(), nB * sizeof(float), cudaMemcpyHostToDevice), "copy") ||
       (n && !rt_ok(cudaMemcpy(d_smp, samples.data(), n * sizeof(Sample2D), cudaMemcpyHostToDevice), "copy")) ||
       !rt_ok(cudaMemcpy(d_views, hv.data(), nR * sizeof(hv[0]), cudaMemcpyHostToDevice), "copy") ||
       !rt_ok(cudaMemset(d_out, 0xFF, (size_t)nR * nB * sizeof(float2)), "memset"))
        return false;

    // The reference kernel from the cubin, found by name.
    CUmodule mod = nullptr;
    unsigned int count = 0;
    if(!cu_ok(cuModuleLoad(&mod, cubin), "cuModuleLoad") || !cu_ok(cuModuleGetFunctionCount(&count, mod), "count"))
        return false;
    std::vector<CUfunction> fns(count);
    if(!cu_ok(cuModuleEnumerateFunctions(fns.data(), count, mod), "enumerate")) return false;
    CUfunction fn = nullptr;
    for(CUfunction c : fns) {
        const char* name = nullptr;
        if(cuFuncGetName(&name, c) == CUDA_SUCCESS && name && std::strstr(name, "do_sparse_convolve_2d_f")) {
            if(fn) return fail("more than one do_sparse_convolve_2d_f in the cubin");
            fn = c;
        }
    }
    if(!fn) return fail("do_sparse_convolve_2d_f not found in the cubin");

    rtac::ImageView<rtac::Complex<float>> out_view{nB, nR, reinterpret_cast<rtac::Complex<float>*>(d_out)};
    rtac::cuda::TextureVectorView<float> bear_view{nB, d_bear};
    rtac::Linspace<float> ranges{par[0], par[1], nR};
    const rtac::VectorView<const Sample2D>* bins = d_views;
    KernelView2DArgs kv{make_float2(par[2], 0.5f), make_float2(par[3], 0.5f), tex};
    void* args[] = {&out_view, &bear_view, &ranges, &bins, &kv};
    const size_t sizes[] = {sizeof(out_view), sizeof(bear_view), sizeof(ranges), sizeof(bins), sizeof(kv)};
    const size_t aligns[] = {alignof(decltype(out_view)), alignof(decltype(bear_view)), alignof(decltype(ranges)),
                             alignof(decltype(bins)), alignof(decltype(kv))};
    size_t expect = 0;
    for(size_t i = 0; i < 5; i++) {
        size_t off = 0, sz = 0;
        if(!cu_ok(cuFuncGetParamInfo(fn, i, &off, &sz), "cuFuncGetParamInfo")) return false;
        const size_t align = aligns[i];
        expect = (expect + align - 1) / align * align;
        if(sz != sizes[i] || off != expect)
            return fail("kernel parameter " + std::to_string(i) + " layout differs from the harness");
        expect += sz;
    }
    size_t off5 = 0, sz5 = 0;
    if(cuFuncGetParamInfo(fn, 5, &off5, &sz5) == CUDA_SUCCESS) return fail("kernel has more than five parameters");

    if(!cu_ok(cuLaunchKernel(fn, nB, nR, 1, 512, 1, 1, 512 * sizeof(float), nullptr, args, nullptr), "launch") ||
       !cu_ok(cuCtxSynchronize(), "kernel"))
        return false;
    std::vector<float2> out((size_t)nR * nB);
    if(!rt_ok(cudaMemcpy(out.data(), d_out, out.size() * sizeof(float2), cudaMemcpyDeviceToHost), "copy back"))
        return false;
    if(reps > 0) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if(!rt_ok(cudaEventCreate(&e0), "event") || !rt_ok(cudaEventCreate(&e1), "event")) return false;
        bool ok = cu_ok(cuLaunchKernel(fn, nB, nR, 1, 512, 1, 1, 512 * sizeof(float), nullptr, args, nullptr), "launch") &&
                  rt_ok(cudaEventRecord(e0, nullptr), "record");
        for(int i = 0; ok && i < reps; i++)
            ok = cu_ok(cuLaunchKernel(fn, nB, nR, 1, 512, 1, 1, 512 * sizeof(float), nullptr, args, nullptr), "launch");
        float ms = 0.0f;
        ok = ok && rt_ok(cudaEventRecord(e1, nullptr), "record") && rt_ok(cudaEventSynchronize(e1), "kernel") &&
             rt_ok(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if(!ok) return false;
        std::printf("ref_kernel_ms %.6f\n", ms / reps);
    }
    FILE* o = std::fopen(out_path, "wb");
    if(!o) return fail("cannot open output");
    const bool wrote = std::fwrite(out.data(), sizeof(float2), out.size(), o) == out.size();
    std::fclose(o);
    cudaDestroyTextureObject(tex);
    cudaFreeArray(arr);
    cudaFree(d_bear); cudaFree(d_smp); cudaFree(d_views); cudaFree(d_out);
    cuModuleUnload(mod);
    return wrote || fail("short output");
}

struct Sample1D { float re, im, travel; };                     // SimSample1D layout
struct KernelView1DArgs { float2 scaling; cudaTextureObject_t tex; }; // KernelView1D<Complex<float>> layout
static_assert(sizeof(KernelView1DArgs) == 16, "KernelView1D layout");
static_assert(sizeof(rtac::VectorView<const Sample1D>) == 16, "VectorView layout");

bool run_1d(const char* cubin, FILE* f, const char* out_path, int reps)
{
    uint32_t hdr[3];
    uint64_t n = 0;
    float par[3];
    if(!get(f, hdr, 3) || !get(f, &n, 1) || !get(f, par, 3)) { std::fclose(f); return fail("bad 1D header"); }
    const uint32_t nR = hdr[0], H = hdr[1], mode = hdr[2];
    if(!nR || !H || nR > (1u << 20) || H > (1u << 20) || mode > 1u || n > (1ull << 28)) { std::fclose(f); return fail("bad 1D sizes"); }
    std::vector<float2> pulse(H);
    std::vector<Sample1D> samples(n);
    std::vector<uint64_t> views(2 * (size_t)nR);
    const bool ok = get(f, pulse.data(), H) && (n == 0 || get(f, samples.data(), n)) && get(f, views.data(), views.size());
    std::fclose(f);
    if(!ok) return fail("short 1D input");
    for(uint32_t r = 0; r < nR; r++)
        if(views[2 * r] > n || views[2 * r + 1] > n - views[2 * r]) return fail("bin view outside the samples");

    if(!rt_ok(cudaSetDevice(0), "cudaSetDevice") || !rt_ok(cudaFree(nullptr), "context")) return false;
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float2>();
    cudaArray_t arr = nullptr;
    if(!rt_ok(cudaMallocArray(&arr, &ch, H, 0), "cudaMallocArray (1D)") ||
       !rt_ok(cudaMemcpy2DToArray(arr, 0, 0, pulse.data(), H * sizeof(float2), H * sizeof(float2), 1,
                                  cudaMemcpyHostToDevice), "pulse upload"))
        return false;
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = mode == 0 ? cudaAddressModeBorder : cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    cudaTextureObject_t tex = 0;
    if(!rt_ok(cudaCreateTextureObject(&tex, &rd, &td, nullptr), "texture")) return false;

    Sample1D* d_smp = nullptr;
    rtac::VectorView<const Sample1D>* d_views = nullptr;
    float2* d_out = nullptr;
    std::vector<rtac::VectorView<const Sample1D>> hv(nR);
    if(!rt_ok(cudaMalloc(&d_smp, (n ? n : 1) * sizeof(Sample1D)), "malloc") ||
       !rt_ok(cudaMalloc(&d_views, nR * sizeof(hv[0])), "malloc") ||
       !rt_ok(cudaMalloc(&d_out, (size_t)nR * sizeof(float2)), "malloc"))
        return false;
    for(uint32_t r = 0; r < nR; r++) hv[r] = rtac::VectorView<const Sample1D>{views[2 * r + 1], d_smp + views[2 * r]};
    if((n && !rt_ok(cudaMemcpy(d_smp, samples.data(), n * sizeof(Sample1D), cudaMemcpyHostToDevice), "copy")) ||
       !rt_ok(cudaMemcpy(d_views, hv.data(), nR * sizeof(hv[0]), cudaMemcpyHostToDevice), "copy") ||
       !rt_ok(cudaMemset(d_out, 0xFF, (size_t)nR * sizeof(float2)), "memset"))
        return false;

    CUmodule mod = nullptr;
    unsigned int count = 0;
    if(!cu_ok(cuModuleLoad(&mod, cubin), "cuModuleLoad") || !cu_ok(cuModuleGetFunctionCount(&count, mod), "count"))
        return false;
    std::vector<CUfunction> fns(count);
    if(!cu_ok(cuModuleEnumerateFunctions(fns.data(), count, mod), "enumerate")) return false;
    CUfunction fn = nullptr;
    for(CUfunction c : fns) {
        const char* name = nullptr;
        if(cuFuncGetName(&name, c) == CUDA_SUCCESS && name && std::strstr(name, "do_sparse_convolve_1d_f")) {
            if(fn) return fail("more than one do_sparse_convolve_1d_f in the cubin");
            fn = c;
        }
    }
    if(!fn) return fail("do_sparse_convolve_1d_f not found in the cubin");

    rtac::VectorView<rtac::Complex<float>> out_view{nR, reinterpret_cast<rtac::Complex<float>*>(d_out)};
    rtac::Linspace<float> ranges{par[0], par[1], nR};
    const rtac::VectorView<const Sample1D>* bins = d_views;
    KernelView1DArgs kv{make_float2(par[2], 0.5f), tex};
    void* args[] = {&out_view, &ranges, &bins, &kv};
    const size_t sizes[] = {sizeof(out_view), sizeof(ranges), sizeof(bins), sizeof(kv)};
    const size_t aligns[] = {alignof(decltype(out_view)), alignof(decltype(ranges)), alignof(decltype(bins)),
                             alignof(decltype(kv))};
    size_t expect = 0;
    for(size_t i = 0; i < 4; i++) {
        size_t off = 0, sz = 0;
        if(!cu_ok(cuFuncGetParamInfo(fn, i, &off, &sz), "cuFuncGetParamInfo")) return false;
        expect = (expect + aligns[i] - 1) / aligns[i] * aligns[i];
        if(sz != sizes[i] || off != expect)
            return fail("1D kernel parameter " + std::to_string(i) + " layout differs from the harness");
        expect += sz;
    }
    size_t off4 = 0, sz4 = 0;
    if(cuFuncGetParamInfo(fn, 4, &off4, &sz4) == CUDA_SUCCESS) return fail("1D kernel has more than four parameters");

    if(!cu_ok(cuLaunchKernel(fn, nR, 1, 1, 512, 1, 1, 512 * sizeof(float), nullptr, args, nullptr), "launch") ||
       !cu_ok(cuCtxSynchronize(), "kernel"))
        return false;
    std::vector<float2> out(nR);
    if(!rt_ok(cudaMemcpy(out.data(), d_out, out.size() * sizeof(float2), cudaMemcpyDeviceToHost), "copy back"))
        return false;
    if(reps > 0) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if(!rt_ok(cudaEventCreate(&e0), "event") || !rt_ok(cudaEventCreate(&e1), "event")) return false;
        bool okr = rt_ok(cudaEventRecord(e0, nullptr), "record");
        for(int i = 0; okr && i < reps; i++)
            okr = cu_ok(cuLaunchKernel(fn, nR, 1, 1, 512, 1, 1, 512 * sizeof(float), nullptr, args, nullptr), "launch");
        float ms = 0.0f;
        okr = okr && rt_ok(cudaEventRecord(e1, nullptr), "record") && rt_ok(cudaEventSynchronize(e1), "kernel") &&
              rt_ok(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if(!okr) return false;
        std::printf("ref_kernel_ms %.6f\n", ms / reps);
    }
    FILE* o = std::fopen(out_path, "wb");
    if(!o) return fail("cannot open output");
    const bool wrote = std::fwrite(out.data(), sizeof(float2), out.size(), o) == out.size();
    std::fclose(o);
    cudaDestroyTextureObject(tex);
    cudaFreeArray(arr);
    cudaFree(d_smp); cudaFree(d_views); cudaFree(d_out);
    cuModuleUnload(mod);
    return wrote || fail("short output");
}

} // namespace

int main(int argc, char** argv)
{
    if(argc != 4 && argc != 5) {
        std::fprintf(stderr, "usage: %s REF_SPARSE2D_OR_1D.cubin INPUT OUTPUT [REPS]\n", argv[0]);
        return 2;
    }
    const int reps = argc == 5 ? std::atoi(argv[4]) : 0;
    if(reps < 0 || reps > 1000) {
        std::fprintf(stderr, "REPS must be in [0, 1000]\n");
        return 2;
    }
    return run(argv[1], argv[2], argv[3], reps) ? 0 : 1;
}
