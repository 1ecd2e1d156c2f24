// xct_f32x2.cuh -- Blackwell packed FP32 pairs (PTX add/sub/mul/fma .f32x2, sm_100+).
//
// One instruction computes two IEEE single-precision results with the stated rounding,
// lane for lane identical to the scalar instruction; it halves the issue slots of the
// coordinate and bin arithmetic of the projectors.
#pragma once
#include <cuda_runtime.h>

typedef unsigned long long f2x;  // (lo, hi) float pair in one 64-bit register pair

__device__ __forceinline__ f2x f2_pack(float lo, float hi)
{
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2x v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ void f2_unpack_bits(f2x v, int &lo, int &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(v));
}
__device__ __forceinline__ f2x f2_add(f2x a, f2x b)
{
    f2x r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2_add_rd(f2x a, f2x b)
{
    f2x r;
    asm("add.rm.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b)
{
    f2x r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b)
{
    f2x r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2x f2_fma(f2x a, f2x b, f2x c)
{
    f2x r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
