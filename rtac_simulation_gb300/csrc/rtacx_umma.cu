// 16-bit tensor-core GEMM on sm_103a: C[M][N] (fp32) =
// row_scale[M] * col_scale[N] * (A[M][K] * B[N][K]^T), A and B both bf16 or
// both fp16 (the scales are optional).
//
// Used by the precision form for the dense complex bearing-directivity
// contraction, written as one real GEMM (see rtacx_precision.cu). Both
// operands are K-major ("TN"); M % 128 == 0, N % 256 == 0, K % 64 == 0
// (callers pad).
//
// One CTA computes a 128 x BN tile with four warps (BN = 256 with a 4-stage
// ring, one CTA per SM; BN = 128 with a 3-stage ring, two CTAs per SM, when N
// is a multiple of 128 but not of 256):
//   warp 0, lane 0  TMA producer: cp.async.bulk.tensor 2D loads of a 128x64
//                   A tile and a BNx64 B tile per stage (128-byte swizzle)
//                   into the shared-memory ring guarded by mbarriers;
//   warp 1, lane 0  MMA issuer: four tcgen05.mma.kind::f16 (K = 16 each) per
//                   stage into a 128-lane x BN-column fp32 TMEM accumulator,
//                   tcgen05.commit frees the stage;
//   warps 0-3       epilogue: tcgen05.ld 32x32b of their TMEM lane quadrant,
//                   optional row / column scaling, fp32 stores of whole
//                   128-byte row segments.
// Every mbarrier wait is bounded (about two seconds); a timeout sets an
// error bit and the CTA skips its remaining work, still waiting (bounded) for
// issued MMAs and freeing its TMEM.
#include "rtacx_internal.cuh"
#include "rtacx_tcgen05.cuh"

#include <atomic>
#include <cuda.h>
#include <cuda_bf16.h>

namespace rtacx {

namespace {

constexpr int BM = 128, BK = 64;
constexpr int kThreads = 128;
constexpr uint32_t A_BYTES = BM * BK * 2;

template <int BN_, int STAGES_>
struct Tile {
    static constexpr int BN = BN_, STAGES = STAGES_;
    static constexpr uint32_t B_BYTES = BN * BK * 2;
    static constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
    static constexpr uint32_t TMEM_COLS = BN;           // power of two >= 32
    static constexpr size_t SMEM_BYTES = (size_t)STAGES * STAGE_BYTES + 1024 + 256;
    static constexpr int CTAS_PER_SM = BN == 128 ? 2 : 1;
};
using TileWide = Tile<256, 4>;
using TileNarrow = Tile<128, 3>;
constexpr long long kWaitCycles = 4000000000ll;

// Instruction descriptor of tcgen05.mma.kind::f16: D = f32 (bits 4-5 = 1),
// A and B format at bits 7-9 and 10-12 (0 = f16, 1 = bf16; always the same
// type for both), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22,
// M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_for(bool f16, int bn)
{
    return (1u << 4) | ((f16 ? 0u : 1u) << 7) | ((f16 ? 0u : 1u) << 10) | ((uint32_t)(bn >> 3) << 17) |
           ((uint32_t)(BM >> 4) << 24);
}

// Bounded wait of the GEMM (about two seconds).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag)
{
    return mbar_wait_bounded(bar, parity, abort_flag, kWaitCycles);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];"
                 ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
                 : "memory");
}

template <bool kF16, int BN>
__device__ __forceinline__ void umma_16bit(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc_for(kF16, BN)), "r"(accumulate)
                 : "memory");
}

template <bool kF16, typename T>
__global__ void __launch_bounds__(kThreads, T::CTAS_PER_SM)
k_gemm_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
          float* __restrict__ C, int M, int N, int K, int ldc, const float* __restrict__ row_scale,
          const float* __restrict__ col_scale, uint32_t* __restrict__ err)
{
    constexpr int BN = T::BN, STAGES = T::STAGES;
    constexpr uint32_t STAGE_BYTES = T::STAGE_BYTES, TMEM_COLS = T::TMEM_COLS;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    unsigned char* base = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + STAGES * STAGE_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * BN, m0 = blockIdx.y * BM;
    // Split K: CTA z multiplies K blocks [z nkb, (z + 1) nkb) into its own
    // partial product C + z M ldc (the caller sums the partials).
    const int nkb = K / BK / (int)gridDim.z, kb0 = (int)blockIdx.z * nkb;
    C += (size_t)blockIdx.z * (size_t)M * ldc;
    auto full_bar = [&](int s) { return smem_u32(bars + s); };
    auto empty_bar = [&](int s) { return smem_u32(bars + STAGES + s); };
    const uint32_t accum_bar = smem_u32(bars + 2 * STAGES);

    if(threadIdx.x == 0) {
        for(int s = 0; s < STAGES; s++) { mbar_init(full_bar(s), 1); mbar_init(empty_bar(s), 1); }
        mbar_init(accum_bar, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    }
    if(warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if(warp == 0 && lane == 0) {
        // TMA producer.
        for(int kb = 0; kb < nkb; kb++) {
            const int s = kb % STAGES;
            if(kb >= STAGES && !mbar_wait(empty_bar(s), ((kb / STAGES) - 1) & 1, abort_flag)) break;
            unsigned char* a = base + s * STAGE_BYTES;
            mbar_expect_tx(full_bar(s), STAGE_BYTES);
            tma_load_2d(smem_u32(a), &tmA, (kb0 + kb) * BK, m0, full_bar(s));
            tma_load_2d(smem_u32(a + A_BYTES), &tmB, (kb0 + kb) * BK, n0, full_bar(s));
        }
    }
    else if(warp == 1 && lane == 0) {
        // MMA issuer.
        for(int kb = 0; kb < nkb; kb++) {
            const int s = kb % STAGES;
            if(!mbar_wait(full_bar(s), (kb / STAGES) & 1, abort_flag)) break;
            tc_fence_after();
            const uint32_t a = smem_u32(base + s * STAGE_BYTES);
            const uint64_t ad = smem_desc(a), bd = smem_desc(a + A_BYTES);
#pragma unroll
            for(int kk = 0; kk < BK / 16; kk++)   // 32 bytes of K per MMA: +2 in descriptor units
                umma_16bit<kF16, BN>(tmem, ad + 2 * kk, bd + 2 * kk, (kb > 0 || kk > 0) ? 1u : 0u);
            umma_commit(empty_bar(s));
        }
        umma_commit(accum_bar);   // arrives once every MMA issued above has completed
    }
    __syncwarp();

    // Epilogue: TMEM lane quadrant of this warp -> rows m0 + 32 warp + lane.
    const bool ok = mbar_wait(accum_bar, 0, abort_flag);
    __syncwarp();
    tc_fence_after();
    if(__all_sync(0xffffffffu, ok ? 1 : 0)) {
        const int row = m0 + warp * 32 + lane;
        float* crow = C + (size_t)row * ldc + n0;
        const float rs = (row_scale && row < M) ? row_scale[row] : 1.0f;
#pragma unroll 1
        for(int c = 0; c < BN / 32; c++) {
            uint32_t r[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), r);
            if(row < M && n0 + c * 32 < N) {
                float v[32];
#pragma unroll
                for(int q = 0; q < 32; q++) v[q] = __uint_as_float(r[q]);
                if(row_scale) {
#pragma unroll
                    for(int q = 0; q < 32; q++) v[q] *= rs;
                }
                if(col_scale) {
                    const float4* cs = reinterpret_cast<const float4*>(col_scale + n0 + c * 32);
#pragma unroll
                    for(int q = 0; q < 8; q++) {
                        const float4 s4 = __ldg(cs + q);
                        v[4 * q] *= s4.x; v[4 * q + 1] *= s4.y; v[4 * q + 2] *= s4.z; v[4 * q + 3] *= s4.w;
                    }
                }
                float4* dst = reinterpret_cast<float4*>(crow + c * 32);
#pragma unroll
                for(int q = 0; q < 8; q++) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
    }
    else if(lane == 0 && err) {
        atomicOr(err, kErrGemmTimeout);
    }
    tc_fence_before();
    __syncthreads();
    if(warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if(!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
           q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            cudaGetLastError();
    }
    return fn;
}

bool make_map(CUtensorMap* map, const void* ptr, uint64_t rows, uint64_t k, uint32_t box_rows, bool f16)
{
    EncodeTiledFn enc = encode_fn();
    if(!enc) return false;
    cuuint64_t dims[2] = {k, rows};
    cuuint64_t strides[1] = {k * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, box_rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
               const_cast<void*>(ptr), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

} // namespace

size_t gemm_smem_bytes() { return std::max(TileWide::SMEM_BYTES, TileNarrow::SMEM_BYTES); }

// C = row_scale * col_scale * (A * B^T); A [M][K], B [N][K] both bf16 or
// both fp16 (16-byte aligned, row stride K), C [M][ldc] fp32, scales
// optional (row_scale [M], col_scale [N], 16-byte aligned). Shapes must be
// multiples of the tile (128, 128, 64). ksplit > 1 splits K into that many
// parts with partial products at C + z M ldc, z = 0 .. ksplit - 1, for the
// caller to sum.
rtacx_status gemm_tn(std::string& error, const void* A, const void* B, float* C, int M, int N, int K, int ldc,
                     cudaStream_t stream, uint32_t* err, bool f16, const float* row_scale, const float* col_scale,
                     int ksplit)
{
    if(M <= 0 || N <= 0 || K <= 0 || M % BM || N % 128 || K % BK || ldc < N || ldc % 4) {
        error = "gemm shape must be multiples of 128 x 128 x 64";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    if(ksplit < 1 || ksplit > 8 || (K / BK) % ksplit) {
        error = "gemm K split must divide the K blocks (1 to 8 parts)";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    // 128 x 256 tiles when N allows them and they cover more than half of
    // the SMs; 128 x 128 tiles (two CTAs per SM) otherwise. Measured on the
    // 4096 x 1024 x 3072 contraction (128 wide tiles): 27 us wide, 30 us
    // narrow (the narrow grid re-reads A twice as often through L2); with
    // half the SMs or fewer, wide tiles leave the tensor cores of the rest
    // idle for the whole launch.
    int dev_sms = 0;
    {
        int d0 = 0;
        if(cudaGetDevice(&d0) != cudaSuccess || cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, d0) != cudaSuccess) {
            cudaGetLastError();
            dev_sms = 0;
        }
    }
    const bool wide = N % 256 == 0 && 2ll * (N / 256) * (M / BM) * ksplit > (long long)dev_sms;
    const int bn = wide ? TileWide::BN : TileNarrow::BN;
    if((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) % 16 || reinterpret_cast<uintptr_t>(C) % 16 ||
       reinterpret_cast<uintptr_t>(col_scale) % 16) {
        error = "gemm operands must be 16-byte aligned";
        return RTACX_ERR_INVALID_ARGUMENT;
    }
    CUtensorMap ma, mb;
    if(!make_map(&ma, A, (uint64_t)M, (uint64_t)K, BM, f16) || !make_map(&mb, B, (uint64_t)N, (uint64_t)K, bn, f16)) {
        error = "cuTensorMapEncodeTiled failed";
        return RTACX_ERR_CUDA;
    }
    // Function attributes belong to a device's context: set them once per device.
    static std::atomic<uint64_t> attr_done{0};
    int dev = 0;
    if(cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        error = "cannot query the current device";
        return RTACX_ERR_CUDA;
    }
    if(!(attr_done.load() & (1ull << dev))) {
        if(cudaFuncSetAttribute(k_gemm_tn<false, TileWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TileWide::SMEM_BYTES) != cudaSuccess ||
           cudaFuncSetAttribute(k_gemm_tn<true, TileWide>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TileWide::SMEM_BYTES) != cudaSuccess ||
           cudaFuncSetAttribute(k_gemm_tn<false, TileNarrow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TileNarrow::SMEM_BYTES) != cudaSuccess ||
           cudaFuncSetAttribute(k_gemm_tn<true, TileNarrow>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TileNarrow::SMEM_BYTES) != cudaSuccess) {
            cudaGetLastError();
            error = "cannot reserve shared memory for the tensor-core GEMM";
            return RTACX_ERR_CUDA;
        }
        attr_done.fetch_or(1ull << dev);
    }
    dim3 grid(N / bn, M / BM, ksplit);
    if(wide) {
        if(f16) k_gemm_tn<true, TileWide><<<grid, kThreads, TileWide::SMEM_BYTES, stream>>>(ma, mb, C, M, N, K, ldc, row_scale, col_scale, err);
        else k_gemm_tn<false, TileWide><<<grid, kThreads, TileWide::SMEM_BYTES, stream>>>(ma, mb, C, M, N, K, ldc, row_scale, col_scale, err);
    }
    else {
        if(f16) k_gemm_tn<true, TileNarrow><<<grid, kThreads, TileNarrow::SMEM_BYTES, stream>>>(ma, mb, C, M, N, K, ldc, row_scale, col_scale, err);
        else k_gemm_tn<false, TileNarrow><<<grid, kThreads, TileNarrow::SMEM_BYTES, stream>>>(ma, mb, C, M, N, K, ldc, row_scale, col_scale, err);
    }
    const cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) { error = std::string("k_gemm_tn: ") + cudaGetErrorString(e); return RTACX_ERR_CUDA; }
    return RTACX_OK;
}

} // namespace rtacx

namespace {
__device__ uint32_t g_gemm_check_err;
}

// Diagnostic entry point (include/rtacx.h): synchronous C = A * B^T.
extern "C" rtacx_status rtacx_gemm_bf16_tn(const void* A, const void* B, float* C, int M, int N, int K, void* stream)
{
    std::string error;
    uint32_t* err = nullptr;
    if(cudaGetSymbolAddress(reinterpret_cast<void**>(&err), g_gemm_check_err) != cudaSuccess) {
        cudaGetLastError();
        return RTACX_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if(cudaMemsetAsync(err, 0, sizeof(uint32_t), s) != cudaSuccess) { cudaGetLastError(); return RTACX_ERR_CUDA; }
    rtacx_status st = rtacx::gemm_tn(error, A, B, C, M, N, K, N, s, err, false, nullptr, nullptr, 1);
    if(st != RTACX_OK) return st;
    uint32_t word = 0;
    if(cudaStreamSynchronize(s) != cudaSuccess ||
       cudaMemcpyFromSymbol(&word, g_gemm_check_err, sizeof(word)) != cudaSuccess) {
        cudaGetLastError();
        return RTACX_ERR_CUDA;
    }
    return word ? RTACX_ERR_DEVICE : RTACX_OK;
}
