// rtacx oracle -- CPU restatement of rtac_simulation's receiver-side reduction.
//
// TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline / reference arm may load this library, and only as the checker
// or as the timed CPU rendition of the reference algorithm. The product path
// (librtacx.so) never links or calls it.
//
// Parity status: PINNED for the range key, the pulse table and the 2D
// reduction. Binner::Key and Waveform_Sine are pinned against golden vectors
// produced by compiling the reference's own headers (oracle/ref_probe.cpp,
// tests/golden/ref_keys.json, ref_waveforms.json). The 2D reduction
// (segments, windows, PSF lookup, accumulation) is pinned against pings of
// the reference's own do_sparse_convolve_2d_f kernel, compiled from the
// reference tree and run on a GB300 (oracle/ref_sparse_harness.cpp,
// tests/golden/ref_pings_2d.npz): mode 2 below, which emulates the texture
// unit's fixed-point weights, reproduces them to 1e-7 relative L2. The 1D
// reduction is restated from the cited sources only (the reference's 1D
// texture set-up is not reproducible).
//
// Arithmetic contract (shared with the CUDA path):
//   * Key parameters are computed in float exactly as the Key constructor does
//     (include/rtac_simulation/Binner.h:34-45). The key itself is
//     (int)fmaf(a, travel, b) with CUDA's float->int conversion (round toward
//     zero, saturating, NaN -> 0), then the unit-mixing bound tests of
//     include/rtac_simulation/Binner.h:47-53.
//   * binOverlap = (int)(margin / ((max - min) / (binCount - 1))) in float
//     (src/Binner.cu:112-113).
//   * Segments and windows follow do_make_segments / do_make_bins literally
//     (src/Binner.cu:51-69, 82-106) on travel-sorted samples
//     (src/Receiver.cu:9-42), including the "istart >= iend -> empty view" rule.
//   * PSF lookup: the reference samples a float2 texture with normalized
//     coordinates, linear filtering and border addressing
//     (src/SensorInstance2D.cu:14-15, 35-42; ReductionKernel.h:44-73). With
//     u = scale * delta + 0.5 the texel coordinate is x = u * n - 0.5 and the
//     value is (1 - frac(x)) T[floor(x)] + frac(x) T[floor(x) + 1], T = 0
//     outside [0, n). The separable table PSF[h][w] = pulse[h] * beam[w]
//     (src/SensorInstance2D.cu:20-33) makes the bilinear fetch the product of
//     two 1D lerps. The coordinate deltas delta = travel - range_r and
//     bearing_s - bearing_b are float subtractions as in the reference kernel
//     (src/SensorInstance2D.cu:56-65); everything after them is exact (FP64)
//     in FP64 mode. The hardware's 9-bit filter weights are NOT reproduced.
//   * Output range r is Linspace[r] = min + r * ((max - min) / (n - 1)) in float
//     (rtac_base Linspace, not vendored; r = 0 for n = 1).

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kOutOfRange = 0xFFFFFFFFu;

// CUDA's cvt.rzi.s32.f32: truncate toward zero, saturate, NaN -> 0.
inline int cuda_f2i_rz(float f)
{
    if(std::isnan(f)) return 0;
    if(f >= 2147483648.0f)  return std::numeric_limits<int>::max();
    if(f <= -2147483648.0f) return std::numeric_limits<int>::min();
    return (int)f;
}

struct KeyParams {
    uint32_t bin_count;
    float a, b, lower, upper;
};

KeyParams make_key(uint32_t binCount, float minBin, float maxBin, float margin)
{
    // include/rtac_simulation/Binner.h:34-45
    KeyParams k;
    k.bin_count = binCount;
    float resolution = (maxBin - minBin) / (float)binCount;
    float m = minBin - 0.5f * resolution;
    float M = maxBin + 0.5f * resolution;
    k.a = (float)(binCount - 1u) / (M - m);
    float ma = -m * k.a;
    k.b = ma + 0.5f;
    k.lower = m - margin;
    k.upper = M + margin;
    return k;
}

inline uint32_t range_key(const KeyParams& k, float travel, int* side = nullptr)
{
    // include/rtac_simulation/Binner.h:47-53
    int res = cuda_f2i_rz(std::fmaf(k.a, travel, k.b));
    if(side) *side = 0;
    if(res < 0) {
        if((float)res >= k.lower) return 0;
        if(side) *side = -1;
        return kOutOfRange;
    }
    if((uint32_t)res >= k.bin_count) {
        if((float)res <= k.upper) return k.bin_count - 1;
        if(side) *side = 1;
        return kOutOfRange;
    }
    return (uint32_t)res;
}

int bin_overlap(float rmin, float rmax, uint32_t n, float margin)
{
    // src/Binner.cu:112-113: float resolution = length / (count - 1);
    // int binOverlap = margin_ / resolution;
    float resolution = (rmax - rmin) / (float)(n - 1u);
    return cuda_f2i_rz(margin / resolution);
}

float linspace_at(float rmin, float rmax, uint32_t n, uint32_t r)
{
    if(n <= 1) return rmin;
    float res = (rmax - rmin) / (float)(n - 1u);
    float prod = res * (float)r;
    return rmin + prod;
}

// Texture-equivalent 1D linear lookup with border addressing, exact weights.
template <typename T>
inline T lerp_border(const T* table, int n, double x)
{
    double fl = std::floor(x);
    if(!(fl >= -1.0 && fl <= (double)(n - 1))) return T(0);
    int i = (int)fl;
    double alpha = x - fl;
    T lo = (i >= 0)    ? table[i]     : T(0);
    T hi = (i + 1 < n) ? table[i + 1] : T(0);
    return lo * (1.0 - alpha) + hi * alpha;
}

// FP32 reference-arithmetic lookup: the float expressions of the reference
// kernel (u = fmaf(scale, delta, 0.5f)) followed by a float texel coordinate.
template <typename T>
inline T lerp_border_f32(const T* table, int n, float u)
{
    float x = u * (float)n - 0.5f;
    float fl = std::floor(x);
    if(!(fl >= -1.0f && fl <= (float)(n - 1))) return T(0);
    int i = (int)fl;
    float alpha = x - fl;
    T lo = (i >= 0)    ? table[i]     : T(0);
    T hi = (i + 1 < n) ? table[i + 1] : T(0);
    return lo * (1.0f - alpha) + hi * alpha;
}

// Linear texture fetch as the texture unit performs it. CUDA's programming
// guide (texture fetching appendix): x = u * n - 0.5 for a normalized
// coordinate u, i = floor(x), weight frac(x) in 9-bit fixed point with 8
// fractional bits. The remaining details were measured on GB300 with
// in-bounds probe fetches (2e5 coordinates each; every one reproduced):
//  * per axis (ramps T[i] = i, n = 2, 64, 164, 500, 3495): u is truncated to
//    21 fractional bits before the scaling, and the weight k = frac(x) * 256
//    is rounded half up to an integer in [0, 256];
//  * bilinear (a unit texel of a 4 x 4 texture at random (u, v)): with
//    per-axis weights a (x) and b (y), the corner weights in 1/256 are
//    w11 = round_half_up(a b / 256), w10 = a - w11, w01 = b - w11,
//    w00 = 256 - a - b + w11 (they sum to 256).
// Border addressing: texels outside [0, n) are 0. Returns i and k.
inline int texel_weight(float u, int n, int& k)
{
    const double uq = std::floor((double)u * 2097152.0) / 2097152.0;
    const double x = uq * n - 0.5;
    const double fl = std::floor(x);
    k = (int)std::floor((x - fl) * 256.0 + 0.5);
    return (int)std::max(-2.0, std::min(fl, (double)n + 1.0));
}

struct Sensor {
    uint32_t dims;          // 1 or 2
    float rmin, rmax;
    uint32_t nR;
    float margin;
    float pulse_scale;      // 1 / (duration * c) (2D), see the 1D quirk flag
    uint32_t pulse_len;
    const float* pulse;     // 2 * pulse_len floats (complex)
    // 2D
    float beam_scale;       // 1 / span
    uint32_t beam_len;
    const float* beam;      // beam_len floats
    uint32_t nB;
    const float* bearings;  // nB floats
};

struct SortedSample { float re, im, travel, bearing; uint32_t index; };

// Travel sort + keys + reference segments + reference windows on the host.
struct BinResult {
    std::vector<SortedSample> sorted;
    std::vector<uint32_t> keys;       // per sorted sample
    std::vector<uint32_t> segments;   // nR * 2 {start, end}
    std::vector<uint32_t> windows;    // nR * 2 {offset, size}
    int overlap;
};

void do_bin(const float* samples, uint64_t n, uint32_t stride, uint32_t dims,
            const KeyParams& key, float rmin, float rmax, uint32_t nR, float margin,
            BinResult& out)
{
    out.sorted.resize(n);
    for(uint64_t i = 0; i < n; i++) {
        const float* s = samples + i * stride;
        out.sorted[i] = SortedSample{s[0], s[1], s[2], dims == 2 ? s[3] : 0.0f, (uint32_t)i};
    }
    // src/Receiver.cu:9-42 sorts by travel; the order among equal travels is
    // unspecified there, a stable order is one valid outcome.
    std::stable_sort(out.sorted.begin(), out.sorted.end(),
                     [](const SortedSample& l, const SortedSample& r) { return l.travel < r.travel; });
    out.keys.resize(n);
    for(uint64_t i = 0; i < n; i++) out.keys[i] = range_key(key, out.sorted[i].travel);

    // src/Binner.cu:51-80 (memset, then do_make_segments)
    out.segments.assign((size_t)nR * 2, 0u);
    for(uint64_t tid = 0; tid < n; tid++) {
        uint32_t k = out.keys[tid];
        if(k == kOutOfRange) continue;
        if(tid == 0) out.segments[0] = 0;
        else if(out.keys[tid - 1] != k) out.segments[(size_t)k * 2] = (uint32_t)tid;
        if(tid == n - 1) out.segments[(size_t)k * 2 + 1] = (uint32_t)n;
        else if(k != out.keys[tid + 1]) out.segments[(size_t)k * 2 + 1] = (uint32_t)(tid + 1);
    }

    // src/Binner.cu:82-136 (do_make_bins)
    int ov = bin_overlap(rmin, rmax, nR, margin);
    out.overlap = ov;
    out.windows.assign((size_t)nR * 2, 0u);
    for(int tid = 0; tid < (int)nR; tid++) {
        int istart = std::max(0, tid - ov);
        int iend = std::min((int)nR - 1, tid + ov);
        auto empty = [&](int i) { return out.segments[2 * i + 1] == out.segments[2 * i]; };
        for(; istart < iend && empty(istart); istart++);
        for(; iend > istart && empty(iend); iend--);
        if(istart >= iend) {
            out.windows[2 * tid] = 0; out.windows[2 * tid + 1] = 0;
        }
        else {
            out.windows[2 * tid] = out.segments[2 * istart];
            out.windows[2 * tid + 1] = out.segments[2 * iend + 1] - out.segments[2 * istart];
        }
    }
}

template <typename F>
void parallel_rows(uint32_t row_begin, uint32_t row_end, int nthreads, F&& f)
{
    if(nthreads <= 1 || row_end - row_begin < 2) {
        for(uint32_t r = row_begin; r < row_end; r++) f(r);
        return;
    }
    std::atomic<uint32_t> next{row_begin};
    std::vector<std::thread> pool;
    for(int t = 0; t < nthreads; t++) {
        pool.emplace_back([&]() {
            for(uint32_t r = next.fetch_add(1); r < row_end; r = next.fetch_add(1)) f(r);
        });
    }
    for(auto& th : pool) th.join();
}

// One output row of the reduction in FP64 (mode 0) or FP32 reference
// arithmetic (mode 1). out points at nB complex values (doubles or floats).
void reduce_row(const Sensor& S, const BinResult& B, uint32_t r, int mode, void* out_row)
{
    const uint32_t nB = (S.dims == 2) ? S.nB : 1u;
    const float R = linspace_at(S.rmin, S.rmax, S.nR, r);
    const uint32_t off = B.windows[2 * r], size = B.windows[2 * r + 1];
    const std::complex<float>* pulse_f = reinterpret_cast<const std::complex<float>*>(S.pulse);
    const int H = (int)S.pulse_len, W = (int)S.beam_len;
    if(mode == 0) {
        std::vector<std::complex<double>> pulse_d(pulse_f, pulse_f + H);
        std::vector<double> beam_d(S.beam, S.beam + (S.dims == 2 ? W : 0));
        std::complex<double>* o = static_cast<std::complex<double>*>(out_row);
        const double ky = (double)S.pulse_scale * H, cy = 0.5 * H - 0.5;
        const double kx = (double)S.beam_scale * W, cx = 0.5 * W - 0.5;
        // Range factor does not depend on the bearing: evaluate once per sample.
        std::vector<std::complex<double>> u(size);
        for(uint32_t i = 0; i < size; i++) {
            const SortedSample& s = B.sorted[off + i];
            float d = s.travel - R;
            u[i] = std::complex<double>(s.re, s.im) * lerp_border(pulse_d.data(), H, (double)d * ky + cy);
        }
        bool sorted_bearings = S.dims == 2;
        for(uint32_t b = 1; sorted_bearings && b < nB; b++) sorted_bearings = S.bearings[b] > S.bearings[b - 1];
        if(S.dims == 2 && sorted_bearings) {
            // Only bearings inside the beam support can receive a non-zero
            // weight (|e| < span/2 (1 + 1/W)); visit a superset of them.
            for(uint32_t b = 0; b < nB; b++) o[b] = std::complex<double>(0.0, 0.0);
            const double hs = 0.5 / (double)S.beam_scale * (1.0 + 1.0 / W) * (1.0 + 1e-6) + 1e-9;
            for(uint32_t i = 0; i < size; i++) {
                const float th_s = B.sorted[off + i].bearing;
                const float* lo = std::lower_bound(S.bearings, S.bearings + nB, (float)((double)th_s - hs));
                const float* hi = std::upper_bound(S.bearings, S.bearings + nB, (float)((double)th_s + hs));
                for(const float* q = lo; q < hi; q++) {
                    const float e = th_s - *q;
                    o[q - S.bearings] += u[i] * lerp_border(beam_d.data(), W, (double)e * kx + cx);
                }
            }
        }
        else {
            for(uint32_t b = 0; b < nB; b++) {
                std::complex<double> acc(0.0, 0.0);
                if(S.dims == 2) {
                    const float th = S.bearings[b];
                    for(uint32_t i = 0; i < size; i++) {
                        float e = B.sorted[off + i].bearing - th;
                        acc += u[i] * lerp_border(beam_d.data(), W, (double)e * kx + cx);
                    }
                }
                else {
                    for(uint32_t i = 0; i < size; i++) acc += u[i];
                }
                o[b] = acc;
            }
        }
    }
    else if((mode == 2 || mode == 3) && S.dims == 1) {
        // Texture-unit emulation (1D): the reference's tex1D fetch of its
        // one-row pulse texture (include/rtac_simulation/ReductionKernel.h:
        // 44-55) at the kernel's coordinate fmaf(scale, delta, 0.5), linear
        // filter, normalized coordinates, border (mode 2) or clamp (mode 3)
        // addressing -- the reference's 1D texture takes rtac_base's
        // defaults (src/SensorInstance1D.cu:15-25), which are not vendored.
        // Measured on GB300 (the reference's own kernel, recorded in
        // tests/golden/ref_pings_1d.npz): the fetch filters the missing
        // second axis as a one-texel axis sampled at its texel edge, so the
        // pulse row is blended half-and-half with the row beyond it. With
        // clamp addressing that row is the pulse row again (a plain linear
        // fetch); with border addressing it is zero and the value is halved.
        // The bilinear corner weights follow texel_weight's rule with the
        // second axis' weight b = 128; accumulation in double.
        std::complex<double>* o = static_cast<std::complex<double>*>(out_row);
        auto texel = [&](int j) -> std::complex<double> {
            if(mode == 3) j = std::min(std::max(j, 0), H - 1);
            else if(j < 0 || j >= H) return std::complex<double>(0.0, 0.0);
            return std::complex<double>(pulse_f[j].real(), pulse_f[j].imag());
        };
        std::complex<double> acc(0.0, 0.0);
        for(uint32_t k = 0; k < size; k++) {
            const SortedSample& s = B.sorted[off + k];
            const float uy = std::fmaf(S.pulse_scale, s.travel - R, 0.5f);
            int a;
            const int j = texel_weight(uy, H, a);
            std::complex<double> w;
            if(mode == 3) {
                w = ((double)(256 - a) * texel(j) + (double)a * texel(j + 1)) / 256.0;
            }
            else {
                const int b = 128, w11 = (a * b + 128) >> 8, w01 = b - w11;   // the pulse row's corners
                w = ((double)w01 * texel(j) + (double)w11 * texel(j + 1)) / 256.0;
            }
            acc += std::complex<double>(s.re, s.im) * w;
        }
        o[0] = acc;
    }
    else if(mode == 2) {
        // Texture-unit emulation (2D): the bilinear fetch of the W x H table
        // PSF[h][w] = pulse[h] * beam[w] (rounded to float, as
        // generate_psf_data builds it, src/SensorInstance2D.cu:20-33) with
        // the texture unit's weights (texel_weight), at the kernel's
        // coordinates fmaf(scale, delta, 0.5)
        // (include/rtac_simulation/ReductionKernel.h:63-69); the weighted
        // texel sum and the accumulation in double.
        std::complex<double>* o = static_cast<std::complex<double>*>(out_row);
        std::vector<std::complex<float>> psf((size_t)W * H);
        for(int h = 0; h < H; h++)
            for(int w = 0; w < W; w++) psf[(size_t)h * W + w] = pulse_f[h] * S.beam[w];
        auto texel = [&](int i, int j) -> std::complex<double> {
            if(i < 0 || i >= W || j < 0 || j >= H) return std::complex<double>(0.0, 0.0);
            const std::complex<float> t = psf[(size_t)j * W + i];
            return std::complex<double>(t.real(), t.imag());
        };
        for(uint32_t b = 0; b < nB; b++) {
            std::complex<double> acc(0.0, 0.0);
            const float th = S.bearings[b];
            for(uint32_t k = 0; k < size; k++) {
                const SortedSample& s = B.sorted[off + k];
                const float uy = std::fmaf(S.pulse_scale, s.travel - R, 0.5f);
                const float ux = std::fmaf(S.beam_scale, s.bearing - th, 0.5f);
                int a, c;
                const int i = texel_weight(ux, W, a), j = texel_weight(uy, H, c);
                const int w11 = (a * c + 128) >> 8, w10 = a - w11, w01 = c - w11, w00 = 256 - a - c + w11;
                const std::complex<double> w = ((double)w00 * texel(i, j) + (double)w10 * texel(i + 1, j) +
                                                (double)w01 * texel(i, j + 1) + (double)w11 * texel(i + 1, j + 1)) /
                                               256.0;
                acc += std::complex<double>(s.re, s.im) * w;
            }
            o[b] = acc;
        }
    }
    else {
        // Literal per-(sample, output) loop of do_sparse_convolve_2d_f /
        // do_sparse_convolve_1d_f in float: one fused PSF evaluation per pair.
        std::complex<float>* o = static_cast<std::complex<float>*>(out_row);
        for(uint32_t b = 0; b < nB; b++) {
            std::complex<float> acc(0.0f, 0.0f);
            const float th = (S.dims == 2) ? S.bearings[b] : 0.0f;
            for(uint32_t i = 0; i < size; i++) {
                const SortedSample& s = B.sorted[off + i];
                float uy = std::fmaf(S.pulse_scale, s.travel - R, 0.5f);
                std::complex<float> w = lerp_border_f32(pulse_f, H, uy);
                if(S.dims == 2) {
                    float ux = std::fmaf(S.beam_scale, s.bearing - th, 0.5f);
                    w *= lerp_border_f32(S.beam, W, ux);
                }
                acc += std::complex<float>(s.re, s.im) * w;
            }
            o[b] = acc;
        }
    }
}

struct GridAxes {
    float rmin, res, inv_res;
    float first, step, inv_step;
    uint32_t cells;
    int row_lo, row_hi;        // accepted absolute rows j: [row_lo, row_hi]
};

// Range grid of the binned model: one node every two output bins (node m at
// rmin + m * hr, hr = 2 res), rows for the nodes of output rows 0 .. nR - 1
// (m = r / 2) widened by the taps.
uint32_t range_nodes(uint32_t nR) { return ((nR - 1u) >> 1) + 1u; }

GridAxes make_grid_axes(float rmin, float rmax, uint32_t nR, float first, float last, uint32_t cells,
                        uint32_t ntaps, uint32_t center)
{
    GridAxes g;
    g.rmin = rmin;
    const float res = (rmax - rmin) / (float)(nR - 1u);
    g.res = 2.0f * res;
    g.inv_res = 1.0f / g.res;
    g.first = first;
    g.step = (last - first) / (float)(cells - 1u);
    g.inv_step = 1.0f / g.step;
    g.cells = cells;
    g.row_lo = -(int)center - 1;
    g.row_hi = (int)range_nodes(nR) + (int)ntaps - (int)center - 2;
    return g;
}

// Grid coordinates of one sample; false when it contributes nothing.
inline bool grid_coords(const GridAxes& g, float t, float th, int& jg, float& alpha, int& q, float& w, int center)
{
    if(!std::isfinite(t) || !std::isfinite(th)) return false;
    const float jf = std::floor((t - g.rmin) * g.inv_res);
    if(!(jf >= (float)g.row_lo && jf <= (float)g.row_hi)) return false;
    const int j = (int)jf;
    const float rj = g.rmin + (float)j * g.res;
    alpha = (t - rj) * g.inv_res;
    jg = j + center + 1;
    const float qf = std::fmin(std::fmax(std::floor((th - g.first) * g.inv_step), 0.0f), (float)(g.cells - 2u));
    q = (int)qf;
    const float gq = g.first + (float)q * g.step;
    w = std::fmin(std::fmax((th - gq) * g.inv_step, 0.0f), 1.0f);
    return true;
}

} // namespace

extern "C" {

// ---- range key (Binner::Key) ------------------------------------------------

void rtacx_oracle_key_params(uint32_t binCount, float minBin, float maxBin, float margin,
                             float* a, float* b, float* lower, float* upper)
{
    KeyParams k = make_key(binCount, minBin, maxBin, margin);
    *a = k.a; *b = k.b; *lower = k.lower; *upper = k.upper;
}

// keys[i] = Key(travel[i * stride]); side[i] (optional) = -1 / 0 / +1 for
// below-range out-of-range, in range, above-range out-of-range.
void rtacx_oracle_range_keys(uint32_t binCount, float minBin, float maxBin, float margin,
                             const float* travel, uint64_t n, uint32_t stride,
                             uint32_t* keys, int8_t* side)
{
    KeyParams k = make_key(binCount, minBin, maxBin, margin);
    for(uint64_t i = 0; i < n; i++) {
        int sd;
        keys[i] = range_key(k, travel[i * stride], &sd);
        if(side) side[i] = (int8_t)sd;
    }
}

int rtacx_oracle_bin_overlap(float rmin, float rmax, uint32_t n, float margin)
{
    return bin_overlap(rmin, rmax, n, margin);
}

float rtacx_oracle_linspace_at(float rmin, float rmax, uint32_t n, uint32_t r)
{
    return linspace_at(rmin, rmax, n, r);
}

// Bearing sub-bin of the (range-bin, bearing-bin) sort key used by the GPU
// path (an extension: the reference keys by range only). With
// q = fmaf(scale, bearing, offset): 0 if !(q >= 1) (NaN included),
// count - 1 if q >= count, else (int)q. scale/offset are floats computed by the
// caller.
void rtacx_oracle_bearing_bins(float scale, float offset, uint32_t count,
                               const float* bearing, uint64_t n, uint32_t stride, uint32_t* out)
{
    for(uint64_t i = 0; i < n; i++) {
        float q = std::fmaf(scale, bearing[i * stride], offset);
        uint32_t kb;
        if(!(q >= 1.0f)) kb = 0;
        else if(q >= (float)count) kb = count - 1;
        else kb = (uint32_t)(int)q;
        out[i] = kb;
    }
}

// Reference segments (binIndexes_) and windows (bins_ as {offset, size}) for a
// sample buffer; samples are AoS with `stride` floats per sample
// (3 = SimSample1D, 4 = SimSample2D). Also returns the low/high out-of-range
// counts and the overlap.
int rtacx_oracle_bin(const float* samples, uint64_t n, uint32_t stride, uint32_t dims,
                     float rmin, float rmax, uint32_t nR, float margin,
                     uint32_t* segments, uint32_t* windows, uint32_t* counts,
                     uint64_t* low_oor, uint64_t* high_oor)
{
    KeyParams key = make_key(nR, rmin, rmax, margin);
    BinResult B;
    do_bin(samples, n, stride, dims, key, rmin, rmax, nR, margin, B);
    if(segments) std::memcpy(segments, B.segments.data(), B.segments.size() * 4);
    if(windows) std::memcpy(windows, B.windows.data(), B.windows.size() * 4);
    if(counts || low_oor || high_oor) {
        uint64_t lo = 0, hi = 0;
        if(counts) std::memset(counts, 0, (size_t)nR * 4);
        for(uint64_t i = 0; i < n; i++) {
            int sd; uint32_t k = range_key(key, samples[i * stride + 2], &sd);
            if(k != kOutOfRange) { if(counts) counts[k]++; }
            else if(sd < 0) lo++;
            else hi++;
        }
        if(low_oor) *low_oor = lo;
        if(high_oor) *high_oor = hi;
    }
    return B.overlap;
}

// Full reduction. mode 0: FP64 (out = 2 doubles per cell), mode 1: FP32
// reference arithmetic (out = 2 floats per cell), mode 2 (2D): the PSF
// fetched as the texture unit does, accumulated in FP64 (2 doubles per cell). Rows [row_begin, row_end)
// only; nthreads worker threads. Returns the wall time of the sort+bin step
// in seconds through bin_seconds (optional).
void rtacx_oracle_reduce(uint32_t dims, const float* samples, uint64_t n,
                         float rmin, float rmax, uint32_t nR, float margin,
                         float pulse_scale, const float* pulse, uint32_t pulse_len,
                         float beam_scale, const float* beam, uint32_t beam_len,
                         const float* bearings, uint32_t nB,
                         int mode, uint32_t row_begin, uint32_t row_end, int nthreads,
                         void* out)
{
    Sensor S{dims, rmin, rmax, nR, margin, pulse_scale, pulse_len, pulse,
             beam_scale, beam_len, beam, nB, bearings};
    KeyParams key = make_key(nR, rmin, rmax, margin);
    BinResult B;
    do_bin(samples, n, dims == 2 ? 4u : 3u, dims, key, rmin, rmax, nR, margin, B);
    const uint32_t nb = (dims == 2) ? nB : 1u;
    const size_t cell = (mode == 1) ? 8 : 16;
    row_end = std::min(row_end, nR);
    parallel_rows(row_begin, row_end, nthreads, [&](uint32_t r) {
        reduce_row(S, B, r, mode, static_cast<char*>(out) + (size_t)(r - row_begin) * nb * cell);
    });
}

// Echo-sample epilogue of the ray generator (src/RayCaster.cu:37-39, 69-71):
// value *= exp(i * 4 pi f d / c) / d^2, applied in place to AoS samples
// (`stride` floats per sample, travel at offset 2). mode 0: exact (the phase
// reduced in double, products in double, rounded to float once); mode 1: the
// reference's own arithmetic (float phase = (float)((4 pi f / c) * d), float
// cos/sin, float product and division). flags: 1 phase, 2 spreading.
void rtacx_oracle_apply_echo(float* samples, uint64_t n, uint32_t stride, double carrier_hz, float c,
                             uint32_t flags, int mode)
{
    const double pi = 3.14159265358979323846;
    for(uint64_t i = 0; i < n; i++) {
        float* s = samples + i * stride;
        const float d = s[2];
        if(mode == 0) {
            std::complex<double> v(s[0], s[1]);
            if(flags & 1u) {
                const double cyc = (double)d * (2.0 * carrier_hz / (double)c);
                const double ph = 2.0 * pi * (cyc - std::nearbyint(cyc));
                v *= std::complex<double>(std::cos(ph), std::sin(ph));
            }
            if(flags & 2u) v /= (double)d * (double)d;
            s[0] = (float)v.real(); s[1] = (float)v.imag();
        }
        else {
            std::complex<float> v(s[0], s[1]);
            if(flags & 1u) {
                const float ph = (float)((4.0 * pi * (double)(float)carrier_hz / (double)c) * (double)d);
                v *= std::complex<float>(std::cos(ph), std::sin(ph));
            }
            if(flags & 2u) { const float dd = d * d; v = std::complex<float>(v.real() / dd, v.imag() / dd); }
            s[0] = v.real(); s[1] = v.imag();
        }
    }
}

// FP64 oracle of the binned (precision) model -- see rtacx_reduce_precision
// in include/rtacx.h. Per sample (in-range reference key, finite travel and
// bearing), with the float arithmetic of the device spelled out so that the
// grid coordinates agree bit for bit:
//   range    res = (rmax - rmin) / (nR - 1) (the Linspace resolution of the
//            output ranges), hr = 2 res, inv_hr = 1 / hr;
//            j = floor((t - rmin) * inv_hr), alpha = (t - (rmin + j * hr)) *
//            inv_hr: weight 1 - alpha on range node j, alpha on node j + 1;
//   bearing  step = (last - first) / (cells - 1), inv_step = 1 / step;
//            q = clamp(floor((theta - first) * inv_step), 0, cells - 2),
//            w = clamp((theta - (first + q * step)) * inv_step, 0, 1): weight
//            1 - w on grid bearing q, w on q + 1.
// Node j is stored at row jg = j + center + 1 of (nR - 1) / 2 + 1 + ntaps + 1
// rows; samples whose rows fall outside reach no output row and are dropped.
// Output row r is zero when its reference window (do_make_bins rule on the
// keyed non-empty bins) is empty, else out(r, b) = sum_t taps[r % 2][t]
// sum_q G[r / 2 + t + 1][q] D[q][b] (taps: two phases of ntaps complex
// values). Rows [row_begin, row_end) into out (complex double).
void rtacx_oracle_reduce_binned(const float* samples, uint64_t n, float rmin, float rmax, uint32_t nR,
                                float margin, uint32_t nB, float grid_first, float grid_last, uint32_t cells,
                                const float* D, const float* taps, uint32_t ntaps, uint32_t center,
                                uint32_t row_begin, uint32_t row_end, int nthreads, void* out)
{
    using cd = std::complex<double>;
    if(nR < 2 || cells < 2 || ntaps == 0) return;
    KeyParams key = make_key(nR, rmin, rmax, margin);
    const GridAxes ax = make_grid_axes(rmin, rmax, nR, grid_first, grid_last, cells, ntaps, center);
    const size_t rows = (size_t)range_nodes(nR) + ntaps + 1;
    std::vector<cd> G(rows * cells, cd(0.0, 0.0));
    std::vector<uint8_t> nonempty(nR, 0);
    for(uint64_t i = 0; i < n; i++) {
        const float* s = samples + i * 4;
        const uint32_t k = range_key(key, s[2]);
        if(k == kOutOfRange) continue;
        nonempty[k] = 1;
        int jg, q;
        float alpha, w;
        if(!grid_coords(ax, s[2], s[3], jg, alpha, q, w, (int)center)) continue;
        const cd v(s[0], s[1]);
        const double a = alpha, b = w;
        cd* r0 = G.data() + (size_t)jg * cells + q;
        cd* r1 = r0 + cells;
        r0[0] += (1.0 - a) * (1.0 - b) * v;
        r0[1] += (1.0 - a) * b * v;
        r1[0] += a * (1.0 - b) * v;
        r1[1] += a * b * v;
    }
    const int ov = bin_overlap(rmin, rmax, nR, margin);
    std::vector<cd> tv(2 * (size_t)ntaps);
    for(uint32_t t = 0; t < 2 * ntaps; t++) tv[t] = cd(taps[2 * t], taps[2 * t + 1]);
    std::vector<cd> Dd((size_t)cells * nB);
    for(size_t e = 0; e < Dd.size(); e++) Dd[e] = cd(D[2 * e], D[2 * e + 1]);
    row_end = std::min(row_end, nR);
    parallel_rows(row_begin, row_end, nthreads, [&](uint32_t r) {
        cd* o = static_cast<cd*>(out) + (size_t)(r - row_begin) * nB;
        for(uint32_t b = 0; b < nB; b++) o[b] = cd(0.0, 0.0);
        if(ov < 0) return;
        const long long lo = std::max(0ll, (long long)r - ov), hi = std::min((long long)nR - 1, (long long)r + ov);
        int nonempty_bins = 0;
        for(long long jj = lo; jj <= hi && nonempty_bins < 2; jj++) nonempty_bins += nonempty[jj];
        if(nonempty_bins < 2) return;          // the reference's empty view (src/Binner.cu:90-102)
        std::vector<cd> g(cells, cd(0.0, 0.0));
        const cd* tp = tv.data() + (size_t)(r & 1u) * ntaps;
        for(uint32_t t = 0; t < ntaps; t++) {
            const cd* row = G.data() + ((size_t)(r >> 1) + t + 1) * cells;
            for(uint32_t q = 0; q < cells; q++) g[q] += tp[t] * row[q];
        }
        for(uint32_t q = 0; q < cells; q++) {
            if(g[q] == cd(0.0, 0.0)) continue;
            const cd* dq = Dd.data() + (size_t)q * nB;
            for(uint32_t b = 0; b < nB; b++) o[b] += g[q] * dq[b];
        }
    });
}

// Echo-sample epilogue (see rtacx_make_samples): hits are n x 6 floats
// {re, im, distance, dir_x, dir_y, dir_z}; R row-major; table [h][w] (or
// w = 0 for uniform); out: n x (dims == 2 ? 4 : 3). Exact arithmetic after
// the float inputs: FP64 phase and exact bilinear weights with mirror
// addressing on normalized coordinates.
void rtacx_oracle_make_samples(const float* hits, uint64_t n, const float* R, const float* tab, uint32_t w,
                               uint32_t h, double carrier_hz, float c, uint32_t flags, uint32_t dims, float* out)
{
    const double pi = 3.14159265358979323846;
    auto mirror = [](double u) { double t = u - 2.0 * std::floor(0.5 * u); return t <= 1.0 ? t : 2.0 - t; };
    auto midx = [](long long i, long long n_) { if(i < 0) return std::min(-i - 1, n_ - 1); if(i >= n_) return std::max(2 * n_ - i - 1, 0ll); return i; };
    for(uint64_t i = 0; i < n; i++) {
        const float* e = hits + 6 * i;
        float* o = out + (dims == 2 ? 4 : 3) * i;
        const double d = e[2];
        if(!(e[2] >= 1.0e-4f)) {
            o[0] = 0.0f; o[1] = 0.0f; o[2] = -1.0f; if(dims == 2) o[3] = 0.0f;
            continue;
        }
        std::complex<double> v(e[0], e[1]);
        if(flags & 1u) {
            const double cyc = d * (2.0 * carrier_hz / (double)c);
            const double ph = 2.0 * pi * (cyc - std::nearbyint(cyc));
            v *= std::complex<double>(std::cos(ph), std::sin(ph));
        }
        if(flags & 2u) v /= d * d;
        const double lx = (double)R[0] * e[3] + (double)R[3] * e[4] + (double)R[6] * e[5];
        const double ly = (double)R[1] * e[3] + (double)R[4] * e[4] + (double)R[7] * e[5];
        const double lz = (double)R[2] * e[3] + (double)R[5] * e[4] + (double)R[8] * e[5];
        if(w > 0) {
            const double x = mirror(std::atan2(ly, lx) / pi) * w - 0.5, y = mirror(std::atan2(lz, lx) / pi) * h - 0.5;
            const double fx = std::floor(x), fy = std::floor(y), ax = x - fx, ay = y - fy;
            const long long x0 = midx((long long)fx, w), x1 = midx((long long)fx + 1, w);
            const long long y0 = midx((long long)fy, h), y1 = midx((long long)fy + 1, h);
            const double t00 = tab[y0 * w + x0], t01 = tab[y0 * w + x1], t10 = tab[y1 * w + x0], t11 = tab[y1 * w + x1];
            v *= (1 - ay) * ((1 - ax) * t00 + ax * t01) + ay * ((1 - ax) * t10 + ax * t11);
        }
        o[0] = (float)v.real(); o[1] = (float)v.imag(); o[2] = e[2];
        if(dims == 2) o[3] = (float)std::atan2(-ly, lx);
    }
}

// Rasteriser oracle (see rtacx_rasterize): identical integer coverage,
// top-left rule, the same float depth plane (slopes and anchor value formed
// per triangle in float, two float FMAs per pixel) and (depth, triangle)
// ties as the kernel; varyings and the fragment arithmetic in double. out: W*H*4
// floats, rows bottom-up; winner (optional): triangle per pixel or -1.
void rtacx_oracle_rasterize(const float* vtx, const float* nrm, const uint32_t* tris, uint32_t nv, uint32_t nt,
                            const float* L, const float* S, const float* origin, uint32_t W, uint32_t H,
                            double carrier_hz, float c, float* out, int32_t* winner)
{
    struct V { long long X, Y; float z, iw; double d[3]; double refl; bool ok; };
    std::vector<V> vs(nv);
    for(uint32_t i = 0; i < nv; i++) {
        const float x = vtx[3 * i], y = vtx[3 * i + 1], z = vtx[3 * i + 2];
        const float cx = std::fma(S[0], x, std::fma(S[1], y, std::fma(S[2], z, S[3])));
        const float cy = std::fma(S[4], x, std::fma(S[5], y, std::fma(S[6], z, S[7])));
        const float cz = std::fma(S[8], x, std::fma(S[9], y, std::fma(S[10], z, S[11])));
        const float cw = std::fma(S[12], x, std::fma(S[13], y, std::fma(S[14], z, S[15])));
        V& v = vs[i];
        v.ok = false; v.X = v.Y = 0; v.z = 0.0f; v.iw = 0.0f;
        if(cw > 1.0e-6f) {
            const float iw = 1.0f / cw;
            const float nx = cx * iw, ny = cy * iw;
            if(std::fabs(nx) <= 64.0f && std::fabs(ny) <= 64.0f) {
                float fx = nx + 1.0f; fx = fx * 0.5f; fx = fx * (float)W; fx = fx * 256.0f;
                float fy = ny + 1.0f; fy = fy * 0.5f; fy = fy * (float)H; fy = fy * 256.0f;
                v.X = (long long)std::nearbyint(fx); v.Y = (long long)std::nearbyint(fy);
                v.z = cz * iw; v.iw = iw; v.ok = true;
            }
        }
        const double o[3] = {(double)x - origin[0], (double)y - origin[1], (double)z - origin[2]};
        double m[3];
        for(int r = 0; r < 3; r++) {
            v.d[r] = L[4 * r] * o[0] + L[4 * r + 1] * o[1] + L[4 * r + 2] * o[2];
            m[r] = L[4 * r] * (double)nrm[3 * i] + L[4 * r + 1] * (double)nrm[3 * i + 1] + L[4 * r + 2] * (double)nrm[3 * i + 2];
        }
        v.refl = std::fabs(m[2] / std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]));
    }
    auto edge = [](long long ax, long long ay, long long bx, long long by, long long px, long long py) {
        return (bx - ax) * (py - ay) - (by - ay) * (px - ax);
    };
    auto top_left = [](long long ax, long long ay, long long bx, long long by) {
        const long long dx = bx - ax, dy = by - ay;
        return (dy == 0 && dx < 0) || dy < 0;
    };
    std::vector<unsigned long long> vis((size_t)W * H, ~0ull);
    for(uint32_t t = 0; t < nt; t++) {
        const uint32_t id[3] = {tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]};
        if(id[0] >= nv || id[1] >= nv || id[2] >= nv) continue;
        const V* p[3] = {&vs[id[0]], &vs[id[1]], &vs[id[2]]};
        if(!p[0]->ok || !p[1]->ok || !p[2]->ok) continue;
        const long long area = (p[1]->X - p[0]->X) * (p[2]->Y - p[0]->Y) - (p[1]->Y - p[0]->Y) * (p[2]->X - p[0]->X);
        if(area == 0) continue;
        const int o0 = 0, o1 = area > 0 ? 1 : 2, o2 = area > 0 ? 2 : 1;
        // depth plane anchored at vertex 0 (the kernel's depth_plane), in float
        const float A = (float)(area > 0 ? area : -area);
        const float z0 = p[0]->z, z1 = p[o1]->z, z2 = p[o2]->z;
        const float dy21 = (float)(p[o2]->Y - p[o1]->Y), dy02 = (float)(p[0]->Y - p[o2]->Y), dy10 = (float)(p[o1]->Y - p[0]->Y);
        const float dx21 = (float)(p[o2]->X - p[o1]->X), dx02 = (float)(p[0]->X - p[o2]->X), dx10 = (float)(p[o1]->X - p[0]->X);
        float sx = dy21 * z0; sx = sx + dy02 * z1; sx = sx + dy10 * z2;
        float sy = dx21 * z0; sy = sy + dx02 * z1; sy = sy + dx10 * z2;
        const float gx = -0.5f * (sx / A), gy = 0.5f * (sy / A);
        const float d0 = 0.5f * z0 + 0.5f;
        long long minX = std::min({p[0]->X, p[1]->X, p[2]->X}), maxX = std::max({p[0]->X, p[1]->X, p[2]->X});
        long long minY = std::min({p[0]->Y, p[1]->Y, p[2]->Y}), maxY = std::max({p[0]->Y, p[1]->Y, p[2]->Y});
        const long long i0 = std::max(0ll, (minX - 128 + 255) / 256);
        const long long i1 = std::min((long long)W - 1, (maxX - 128) >= 0 ? (maxX - 128) / 256 : -1ll);
        const long long j0 = std::max(0ll, (minY - 128 + 255) / 256);
        const long long j1 = std::min((long long)H - 1, (maxY - 128) >= 0 ? (maxY - 128) / 256 : -1ll);
        for(long long j = j0; j <= j1; j++)
            for(long long i = i0; i <= i1; i++) {
                const long long px = i * 256 + 128, py = j * 256 + 128;
                const long long e0 = edge(p[o1]->X, p[o1]->Y, p[o2]->X, p[o2]->Y, px, py);
                const long long e1 = edge(p[o2]->X, p[o2]->Y, p[o0]->X, p[o0]->Y, px, py);
                const long long e2 = edge(p[o0]->X, p[o0]->Y, p[o1]->X, p[o1]->Y, px, py);
                if(e0 < 0 || e1 < 0 || e2 < 0) continue;
                if(e0 == 0 && !top_left(p[o1]->X, p[o1]->Y, p[o2]->X, p[o2]->Y)) continue;
                if(e1 == 0 && !top_left(p[o2]->X, p[o2]->Y, p[o0]->X, p[o0]->Y)) continue;
                if(e2 == 0 && !top_left(p[o0]->X, p[o0]->Y, p[o1]->X, p[o1]->Y)) continue;
                const float d = std::fma(gx, (float)(px - p[0]->X), std::fma(gy, (float)(py - p[0]->Y), d0));
                if(!(d >= 0.0f && d <= 1.0f)) continue;
                uint32_t bits;
                std::memcpy(&bits, &d, 4);
                const unsigned long long w = ((unsigned long long)bits << 32) | t;
                unsigned long long& slot = vis[(size_t)j * W + i];
                if(w < slot) slot = w;
            }
    }
    const double pi = 3.14159265358979323846;
    for(size_t idx = 0; idx < (size_t)W * H; idx++) {
        float* o = out + 4 * idx;
        o[0] = o[1] = o[2] = o[3] = 0.0f;
        if(winner) winner[idx] = -1;
        if(vis[idx] == ~0ull) continue;
        const uint32_t t = (uint32_t)(vis[idx] & 0xFFFFFFFFu);
        if(winner) winner[idx] = (int32_t)t;
        const V* p[3] = {&vs[tris[3 * t]], &vs[tris[3 * t + 1]], &vs[tris[3 * t + 2]]};
        const long long i = (long long)(idx % W), j = (long long)(idx / W);
        const long long px = i * 256 + 128, py = j * 256 + 128;
        const double l[3] = {(double)edge(p[1]->X, p[1]->Y, p[2]->X, p[2]->Y, px, py),
                             (double)edge(p[2]->X, p[2]->Y, p[0]->X, p[0]->Y, px, py),
                             (double)edge(p[0]->X, p[0]->Y, p[1]->X, p[1]->Y, px, py)};
        double wsum = 0.0, d[3] = {0, 0, 0}, refl = 0.0;
        for(int k = 0; k < 3; k++) {
            const double w = l[k] * (double)p[k]->iw;
            wsum += w;
            for(int r = 0; r < 3; r++) d[r] += w * p[k]->d[r];
            refl += w * p[k]->refl;
        }
        for(int r = 0; r < 3; r++) d[r] /= wsum;
        refl /= wsum;
        const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const double range = std::sqrt(r2);
        const double bearing = std::atan2(d[0], -d[2]), elevation = std::atan2(d[1], -d[2]);
        const double cyc = range * (2.0 * carrier_hz / (double)c) + 0.25;
        const double ph = 2.0 * pi * (cyc - std::nearbyint(cyc));
        const double a = refl / r2 / std::cos(bearing) / std::cos(elevation);
        o[0] = (float)(a * std::cos(ph)); o[1] = (float)(a * std::sin(ph));
        o[2] = (float)range; o[3] = (float)bearing;
    }
}

} // extern "C"
