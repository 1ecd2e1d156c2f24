// xct_device.cuh -- device arithmetic shared by the plain and tiled kernels.
//
// The library is compiled with --fmad=false: every multiply-add that should be fused is
// an explicit fmaf(), everything else rounds separately, so each expression below has
// exactly one IEEE result.  The oracle's GPU order (oracle/xct_oracle_body.h) restates
// the same expressions, so forward samples and backprojection bins agree bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#include "xct_internal.h"

// One bilinear sample of the reference forward model (OSEM.cl:56-62 with the
// CLK_FILTER_LINEAR | CLK_ADDRESS_CLAMP sampler of reconstShare.cl:32): the sample at
// texel-centre coordinates (x, y) = (u - 0.5, v - 0.5), zero outside the image.
// Coordinates are formed as x = fma(Yc, s, ax), y = fma(Yc, c, ay) from the per-ray
// bases ax = fma(Xc, c, nx/2), ay = fma(Xc, -s, ny/2); the filter is three FMA lerps.
__device__ __forceinline__ float xct_lerp(float a, float t0, float t1) { return fmaf(a, t1 - t0, t0); }

__device__ __forceinline__ float xct_bilinear_global(const float *__restrict__ img, int nx, int ny, float x, float y)
{
    const float fi = floorf(x), fj = floorf(y);
    const float a = x - fi, b = y - fj;
    const int i = (int)fi, j = (int)fj;
    const bool i0 = (unsigned)i < (unsigned)nx, i1 = (unsigned)(i + 1) < (unsigned)nx;
    const bool j0 = (unsigned)j < (unsigned)ny, j1 = (unsigned)(j + 1) < (unsigned)ny;
    const float *r0 = img + (size_t)j * nx + i;
    const float t00 = (i0 && j0) ? __ldg(r0) : 0.0f;
    const float t10 = (i1 && j0) ? __ldg(r0 + 1) : 0.0f;
    const float t01 = (i0 && j1) ? __ldg(r0 + nx) : 0.0f;
    const float t11 = (i1 && j1) ? __ldg(r0 + nx + 1) : 0.0f;
    const float q0 = xct_lerp(a, t00, t10);
    const float q1 = xct_lerp(a, t01, t11);
    return xct_lerp(b, q0, q1);
}

// Detector bin of pixel (X, Y) at angle (c, s) exactly as OSEM2 evaluates it
// (OSEM.cl:95): ((Xc*c - Yc*s) + PRJ_IMAGESIZE*0.5f) + 0.5f, no contraction, then the
// nearest sampler's floor.  q = Yc*s is passed in (one product per row and angle).
__device__ __forceinline__ float xct_bin_coord(float Xc, float c, float q, float cx)
{
    return ((Xc * c - q) + cx) + 0.5f;
}

// floor(t) for |t| < 2^22 without the conversion pipe: adding 1.5*2^23 rounding toward
// -inf leaves floor(t) in the low mantissa bits.  Returns floor(t) + 0x4B400000.
__device__ __forceinline__ int xct_floor_bits(float t)
{
    return __float_as_int(__fadd_rd(t, 12582912.0f));
}
#define XCT_FLOOR_BIAS 0x4B400000

// OSEM1 measured value (OSEM.cl:64-65): read at integer (X, th); see XCT_FETCH_*.
__device__ __forceinline__ float xct_measured(const float *__restrict__ meas, int px, int pa, int X, int th, int fetch)
{
    if (fetch == XCT_FETCH_EXACT) return __ldg(meas + (size_t)th * px + X);
    // 0.25 * (t(X-1,th-1) + t(X,th-1) + t(X-1,th) + t(X,th)), zero border, summed in
    // that order (X < px and th < pa hold for every caller)
    (void)pa;
    const float a = (X >= 1 && th >= 1) ? __ldg(meas + (size_t)(th - 1) * px + X - 1) : 0.0f;
    const float b = (th >= 1) ? __ldg(meas + (size_t)(th - 1) * px + X) : 0.0f;
    const float c = (X >= 1) ? __ldg(meas + (size_t)th * px + X - 1) : 0.0f;
    const float d = __ldg(meas + (size_t)th * px + X);
    return 0.25f * (((a + b) + c) + d);
}

// OSEM1 epilogue (OSEM.cl:64-66): m = max(1e-6, y) with NaN -> 1e-6, then
// r = (prj < 1e-4) ? m : m / prj (IEEE division).
__device__ __forceinline__ float xct_ratio(float y, float prj)
{
    const float m = (y > 1.0e-6f) ? y : 1.0e-6f;
    return (prj < 0.0001f) ? m : __fdiv_rn(m, prj);
}

// OSEM2 update (OSEM.cl:102-103): ((x * b) * SS) / PRJ_ANGLESIZE, NaN -> 1e-6.
__device__ __forceinline__ float xct_update(float x, float b, float ssf, float paf)
{
    const float v = __fdiv_rn((x * b) * ssf, paf);
    return (v != v) ? 1.0e-6f : v;
}
