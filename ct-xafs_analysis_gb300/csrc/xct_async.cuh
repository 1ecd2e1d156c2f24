// xct_async.cuh -- asynchronous global -> shared copies (cp.async, zero-filled past
// src_bytes) and shared loads at a constant offset, for the kernels that stage windows.
#pragma once
#include <cuda_runtime.h>

__device__ __forceinline__ void cp_async16(unsigned dst, const void *src, unsigned src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async4(unsigned dst, const void *src, unsigned src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int kOff>
__device__ __forceinline__ float lds_f1_at(unsigned addr)
{
    float v;
    asm volatile("ld.shared.f32 %0, [%1+%2];" : "=f"(v) : "r"(addr), "n"(kOff));
    return v;
}
template <int kOff>
__device__ __forceinline__ void lds_f2_at(unsigned addr, float &a, float &b)
{
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];" : "=f"(a), "=f"(b) : "r"(addr), "n"(kOff));
}
