// Inline-PTX helpers for the 5th-generation tensor cores (tcgen05) on sm_103a: tensor
// memory allocation, shared-memory matrix and instruction descriptors, single-thread
// MMA issue with completion on an mbarrier, and accumulator loads.
//
// Operands live in shared memory in the K-major layout without swizzle: 8 x 16-byte
// "core matrices" (8 rows of 8 bf16), element (r, k) of a tile at
//     (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2 bytes.
// The accumulator D (M = 128 rows, fp32) lives in tensor memory: row i in lane i,
// column j in column base + j.  A warp w of the CTA reads lanes 32 (w % 4) ... + 31.
#pragma once

#include <cstdint>

#include "tma.cuh"

namespace emsim_gb300 {
namespace umma {

// ---- tensor memory -------------------------------------------------------------------
// executed by all 32 threads of one warp; the allocated base address lands in *dst_smem
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t n_cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tma::smem_u32(dst_smem)),
                 "r"(n_cols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t n_cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(n_cols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- descriptors -------------------------------------------------------------------
// shared-memory matrix descriptor: K-major, no swizzle, LBO / SBO in bytes
__device__ __forceinline__ uint64_t smem_desc(const void* base, uint32_t lbo, uint32_t sbo) {
    const uint32_t a = tma::smem_u32(base);
    uint64_t d = 0;
    d |= (uint64_t)((a >> 4) & 0x3FFFu);           // start address
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;    // leading-dimension byte offset
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;    // stride-dimension byte offset
    d |= (uint64_t)1 << 46;                          // descriptor version of this architecture
    // base offset 0, LBO mode 0, layout type 0 (no swizzle)
    return d;
}

// instruction descriptor of kind::f16 with bf16 A and B, fp32 D, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4)                        // D format: f32
           | (1u << 7)                      // A format: bf16
           | (1u << 10)                     // B format: bf16
           | ((uint32_t)(N >> 3) << 17)     // N / 8
           | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// ---- MMA -----------------------------------------------------------------------------
// D (tensor memory) (+)= A (smem, M x 16) * B (smem, N x 16)^T ; one thread issues
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive once on `bar` when every MMA this thread issued before has completed
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     tma::smem_u32(bar))
                 : "memory");
}

// ---- accumulator loads -------------------------------------------------------------
// 8 consecutive fp32 columns of this thread's lane
__device__ __forceinline__ void ld_x8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// tensor-memory address of lane `lane`, column `col` relative to the allocation base
__device__ __forceinline__ uint32_t taddr(uint32_t base, uint32_t lane, uint32_t col) {
    return base + (lane << 16) + col;
}

// byte offset of element (r, k) in a K-major no-swizzle tile with K_BYTES bytes per row
// (core matrices adjacent in K are contiguous: LBO = 128, SBO = 8 * K_BYTES)
template <int K_BYTES>
__host__ __device__ constexpr uint32_t kmajor_offset(int r, int k) {
    return (uint32_t)((r >> 3) * (8 * K_BYTES) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

}  // namespace umma
}  // namespace emsim_gb300
