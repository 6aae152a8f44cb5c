// tcgen05 building blocks shared by the tensor-core kernels (the GEMM of the
// precision form, the tensor-core gather of the plain form): shared-memory
// matrix descriptors of the 128-byte-swizzle K-major layout, MMA commit,
// the thread-sync fences around tcgen05 operations and TMEM loads.
#pragma once

#include "rtacx_internal.cuh"

namespace rtacx {

namespace {

// Shared-memory matrix descriptor, K-major operand in the 128-byte swizzle
// layout written by TMA: start address >> 4 (bits 0-13), leading byte offset
// 16 B (unused for this layout), stride byte offset 1024 B between 8-row
// groups (bits 32-45), fixed version bits 46-48 = 0b001, swizzle mode 2
// (128 B) at bits 61-63. The tile base is 1024-byte aligned (base offset 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                 "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                   "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Byte offset of element (row, k) of 4-byte elements in a K-major operand
// tile stored in the 128-byte swizzle layout: 128-byte rows, eight-row atoms
// of 1024 bytes; the 16-byte chunk k / 4 of row r sits at chunk (k / 4) ^ (r % 8).
__device__ __forceinline__ uint32_t sw128_offset_b32(uint32_t row, uint32_t k)
{
    return row * 128u + ((((k >> 2) ^ row) & 7u) << 4) + ((k & 3u) << 2);
}

} // namespace

} // namespace rtacx
