// Asynchronous global -> shared copies (cp.async, sm_80+) used to stream band
// rows ahead of the sequential sweeps.  A thread waits only for its own
// copies (wait_group); a __syncwarp/__syncthreads after the wait publishes
// them to the other threads.
#pragma once

#include <cuda_runtime.h>

namespace crgpu {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename T>
__device__ __forceinline__ void cp_async_elem(T *dst, const T *src);
template <>
__device__ __forceinline__ void cp_async_elem<float2>(float2 *dst, const float2 *src) {
    cp_async8(dst, src);
}
template <>
__device__ __forceinline__ void cp_async_elem<double2>(double2 *dst, const double2 *src) {
    cp_async16(dst, src);
}

}  // namespace crgpu
