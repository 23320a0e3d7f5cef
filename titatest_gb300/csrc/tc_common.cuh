// tcgen05 building blocks shared by the tensor-core kernels (band factor,
// Jacobian contraction): kind::tf32 MMAs on K-major shared-memory operands
// without swizzle, TMEM loads/stores and the tf32 hi/lo split.
#pragma once

#include <cstdint>

#include "bulk.cuh"

namespace crgpu {
namespace tc {

// float index of element (row, k) of a [rows x 8] K-major operand
__device__ __forceinline__ int kmaj(int row, int k) { return ((row >> 3) * 2 + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3); }

__device__ __forceinline__ uint64_t smem_desc(const void *p) {
    const uint64_t addr = smem_u32(p);
    uint64_t d = (addr >> 4) & 0x3FFFull;   // start address
    d |= (uint64_t)(128 >> 4) << 16;        // leading (K) byte offset between core matrices
    d |= (uint64_t)(256 >> 4) << 32;        // stride (M/N) byte offset between 8-row groups
    d |= 1ull << 46;                        // descriptor version of sm_100
    return d;                               // base offset 0, no swizzle
}

// kind::tf32 instruction descriptor: D f32, A/B tf32, both K-major, N, M
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// D (+)= A B^T; acc = 0 overwrites D
__device__ __forceinline__ void tc_mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc = 1) {
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r0, r1, r2, r3, r4, r5, r6, r7;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3), "=r"(r4), "=r"(r5), "=r"(r6), "=r"(r7)
        : "r"(taddr)
        : "memory");
    v[0] = __uint_as_float(r0);
    v[1] = __uint_as_float(r1);
    v[2] = __uint_as_float(r2);
    v[3] = __uint_as_float(r3);
    v[4] = __uint_as_float(r4);
    v[5] = __uint_as_float(r5);
    v[6] = __uint_as_float(r6);
    v[7] = __uint_as_float(r7);
}

__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};\n"
        "tcgen05.wait::st.sync.aligned;\n" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
        : "memory");
}

// tf32 split x = hi + lo: hi is x rounded to the nearest tf32 (10 mantissa
// bits), so |lo| <= 2^-11 |x| and the tensor core's truncation of lo to tf32
// costs at most ~2^-22 |x|; the dropped lo.lo product is below 2^-22 too.
__device__ __forceinline__ float tf32_hi(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

__device__ __forceinline__ void put_row8(float *op, int row, const float (&v)[8]) {
    *(float4 *)&op[kmaj(row, 0)] = make_float4(v[0], v[1], v[2], v[3]);
    *(float4 *)&op[kmaj(row, 4)] = make_float4(v[4], v[5], v[6], v[7]);
}

}  // namespace tc
}  // namespace crgpu
