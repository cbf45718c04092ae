// Fifth-generation tensor cores (tcgen05) for sm_103a, written as inline PTX:
// tensor-memory (TMEM) allocation, shared-memory matrix descriptors in the
// K-major layout without swizzling, the instruction descriptor of
// kind::tf32 / kind::f16 products, MMA issue and commit to an mbarrier,
// bounded mbarrier waits, and TMEM loads of the accumulator.
//
// Operand layout (both A and B K-major, no swizzle): the matrix is cut into
// core matrices of 8 rows x 16 bytes (8 x 4 tf32 values); the 16-byte rows of
// a core matrix are contiguous (128 bytes per core matrix).  Core matrix
// (r, c) -- rows 8r..8r+7, K elements 4c..4c+3 -- starts at
//     base + r * SBO + c * LBO,   LBO = 128 bytes (K-adjacent core matrices
//     contiguous), SBO = 128 * (K / 4) bytes (one 8-row band after another).
// smem_kmajor_offset() gives the byte offset of element (row, k) in that
// layout; an MMA of K = 8 reads two K-adjacent core matrices per 8-row band,
// and the descriptor of K step s starts 2 * 128 * s bytes after the base.
//
// Accumulator: D (M = 128 rows x N columns, fp32) in TMEM, row i in lane i,
// column j in column j of the allocation.  A warp reads the 32 lanes of its
// quarter (warp % 4) with tcgen05.ld.32x32b: thread t of the warp gets row
// 32 (warp % 4) + t.
//
// Every wait is bounded: a wait that gives up returns false and the caller
// records an error instead of spinning forever.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nqcd {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Byte offset of element (row, k) of a K-major, unswizzled operand whose K
// extent is kdim (a multiple of 4) and whose elements are 4 bytes.
__host__ __device__ __forceinline__ uint32_t smem_kmajor_offset(int row, int k, int kdim) {
    return (uint32_t)((row >> 3) * (kdim * 32) + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// Shared-memory matrix descriptor (tcgen05): start address >> 4 in bits
// 0-13, leading-dimension byte offset >> 4 in 16-29, stride-dimension byte
// offset >> 4 in 32-45, the fixed value 1 in bits 46-47, base offset 0,
// relative leading-dimension mode, swizzle mode 0 (none) in bits 61-63.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::tf32 (atype = btype = 2) or kind::f16 with
// bf16 operands (atype = btype = 1): fp32 accumulator (bits 4-5 = 1), A and B
// K-major, N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc_f32acc(int atype, int m, int n) {
    return (1u << 4) | ((uint32_t)atype << 7) | ((uint32_t)atype << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}
constexpr int kTypeBF16 = 1;
constexpr int kTypeTF32 = 2;

// TMEM allocation by one whole warp; the address lands in *slot (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Generic-proxy shared-memory writes become visible to the tensor cores.
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Wait until the phase with the given parity has completed; false after
// max_polls unsuccessful polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < max_polls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// D[tmem] (+)= A * B, issued by one thread.
template <int KIND>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate) {
    const uint32_t acc = accumulate ? 1u : 0u;
    if constexpr (KIND == kTypeTF32) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
            : "memory");
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
            "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
            : "memory");
    }
}

// Arrive on the mbarrier once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// 8 consecutive fp32 columns of this thread's TMEM lane, read and written.
__device__ __forceinline__ void ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ void st8(uint32_t taddr, const float (&v)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}

__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Round to tf32 (nearest, ties away), returned in an fp32 container.
// Round to the nearest tf32 value, ties away from zero (cvt.rna.tf32.f32's rounding), with two
// integer instructions: add half a tf32 unit to the magnitude bits and clear the 13 low bits.
// Exact for every finite float whose rounding stays finite; symmetric in the sign, so an
// antisymmetric matrix stays antisymmetric.
__device__ __forceinline__ float to_tf32(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xffffe000u);
}

}  // namespace tc
}  // namespace nqcd
