// xct_fista.cu -- kernels of the FISTA reconstruction with compressed sensing (FISTA_ocl /
// FISTA_execution, CT_reconstruction/GPU.cpp:1755-2299; FISTA.cl, AART.cl).
//
//   * the power iteration that estimates each subset operator's Lipschitz constant
//     (powerIteration, GPU.cpp:2079-2188): its backprojection powerIter2 (FISTA.cl:79-111:
//     integer half sizes, the nearest sampler's floor, no +0.5), the squared L2 norm of the
//     candidate over the columns and rows the reference's work-groups visit
//     (imageL2AbsX/Y, FISTA.cl:133-208; summed in double here) and the normalisation
//     powerIter3 (FISTA.cl:114-130).  Its forward projection powerIter1 is the tiled forward
//     projector with the geometry shifted by half a texel (powerIter1 adds no +0.5);
//   * the AART1 residual (AART.cl:38-70): y - A x on the subset's rows, a NaN measurement read
//     as 0, applied in place to the forward projection;
//   * FISTAbackProjection (FISTA.cl:211-246): x + b alpha ss/pa/D/L[sub] 0.5 with b the
//     floor-rule nearest-bin backprojection of the residual (no +0.5, unlike OSEM2).
// Element-wise or gather kernels; the proximal steps are xct_cs.cu's.
#include <math.h>

#include <algorithm>

#include "xct_device.cuh"
#include "xct_internal.h"

namespace {

// powerIter2 for subset `sub`: cnd = (sum over its pa/ss rows of prj[th][floor(t)]) * scale,
// t = ((X - nx/2) c - (Y - ny/2) s) + px/2 with integer halves (FISTA.cl:100).
__global__ void pi_bp_kernel(const float *__restrict__ prj, float *__restrict__ cnd, const float2 *__restrict__ trig,
                             KGeom g, int sub, int step, int nrows, float scale)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int Y = blockIdx.y * blockDim.y + threadIdx.y;
    if (X >= g.nx || Y >= g.ny) return;
    const float Xc = (float)(X - g.nx / 2), Yc = (float)(Y - g.ny / 2), c0 = (float)(g.px / 2);
    float b = 0.0f;
    for (int k = 0; k < nrows; ++k) {
        const int th = sub + k * step;
        const float2 cs = __ldg(trig + th);
        const float t = (Xc * cs.x - Yc * cs.y) + c0;
        const int bin = (int)floorf(t);
        if (bin >= 0 && bin < g.px) b += __ldg(prj + (size_t)th * g.px + bin);
    }
    cnd[(size_t)Y * g.nx + X] = b * scale;
}

// imageL2AbsX/Y: the squares of the candidate (rounded as the kernel's val*val) summed in
// double over columns [0, nxe) and rows [0, nye).
__global__ void pi_l2_kernel(const float *__restrict__ cnd, int nx, int nxe, int nye, double *__restrict__ out)
{
    __shared__ double red[256 / 32];
    double acc = 0.0;
    const long long total = (long long)nxe * nye;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int Y = (int)(i / nxe), X = (int)(i - (long long)Y * nxe);
        const float v = __ldg(cnd + (size_t)Y * nx + X);
        acc += (double)(v * v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        atomicAdd(out, s);
    }
}

// powerIter3: img = cnd read at integer coordinates with the linear sampler (exact texel, or
// the 2x2 average, XCT_FETCH_*) over sqrt(L2) in float.
__global__ void pi_norm_kernel(const float *__restrict__ cnd, float *__restrict__ img, int nx, int ny,
                               const double *__restrict__ l2, int fetch)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int Y = blockIdx.y * blockDim.y + threadIdx.y;
    if (X >= nx || Y >= ny) return;
    const float n = sqrtf((float)*l2);
    float v;
    if (fetch == XCT_FETCH_EXACT) {
        v = __ldg(cnd + (size_t)Y * nx + X);
    } else {
        auto t = [&](int i, int j) { return (i >= 0 && j >= 0) ? __ldg(cnd + (size_t)j * nx + i) : 0.0f; };
        v = 0.25f * (((t(X - 1, Y - 1) + t(X, Y - 1)) + t(X - 1, Y)) + t(X, Y));
    }
    img[(size_t)Y * nx + X] = __fdiv_rn(v, n);
}

// AART1's residual in place on the subset's rows of dN sinograms: out = m - out, m the
// measured value (XCT_FETCH_*) with NaN read as 0.
__global__ void residual_kernel(const float *__restrict__ meas, float *__restrict__ out, KGeom g, int sub, int step)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y, z = blockIdx.z;
    if (X >= g.px) return;
    const int th = sub + k * step;
    float m = xct_measured(meas + (size_t)z * g.pa * g.px, g.px, g.pa, X, th, g.fetch);
    m = (m != m) ? 0.0f : m;
    float *o = out + ((size_t)z * g.pa + th) * g.px + X;
    *o = m - *o;
}

// FISTAbackProjection for subset `sub` on dN slices: v = x + ((((b alpha) ss) / pa) / D) / L 0.5,
// b the sum over th = sub, sub + ss, ... < pa of res[th][floor(((X - nx/2) c - (Y - ny/2) s) + cx)]
// (float halves, FISTA.cl:237), 0 off the detector.
__global__ void fista_bp_kernel(const float *__restrict__ x, float *__restrict__ v, const float *__restrict__ res,
                                const float2 *__restrict__ trig, KGeom g, int sub, float alpha, float L)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int Y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    if (X >= g.nx || Y >= g.ny) return;
    const float *rz = res + (size_t)z * g.pa * g.px;
    const float Xc = (float)X - g.hx, Yc = (float)Y - g.hy;
    float b = 0.0f;
    for (int th = sub; th < g.pa; th += g.ss) {
        const float2 cs = __ldg(trig + th);
        const float t = (Xc * cs.x - Yc * cs.y) + g.cx;
        const int bin = (int)floorf(t);
        if (bin >= 0 && bin < g.px) b += __ldg(rz + (size_t)th * g.px + bin);
    }
    float d = b * alpha;
    d = d * (float)g.ss;
    d = __fdiv_rn(d, (float)g.pa);
    d = __fdiv_rn(d, (float)g.depth);
    d = __fdiv_rn(d, L);
    d = d * 0.5f;
    const size_t o = ((size_t)z * g.ny + Y) * g.nx + X;
    v[o] = __ldg(x + o) + d;
}

}  // namespace

int launch_pi_bp(const KGeom &g, const float2 *trig, const float *prj, float *cnd, int sub, int step, int nrows,
                 float scale, cudaStream_t st)
{
    dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8);
    pi_bp_kernel<<<grid, dim3(32, 8), 0, st>>>(prj, cnd, trig, g, sub, step, nrows, scale);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_pi_l2(const float *cnd, int nx, int nxe, int nye, double *out, int sm_count, cudaStream_t st)
{
    XCT_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double), st));
    if (nxe <= 0 || nye <= 0) return XCT_OK;
    const long long total = (long long)nxe * nye;
    const int grid = (int)std::max(1LL, std::min((total + 255) / 256, (long long)sm_count * 8));
    pi_l2_kernel<<<grid, 256, 0, st>>>(cnd, nx, nxe, nye, out);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_pi_norm(const float *cnd, float *img, int nx, int ny, const double *l2, int fetch, cudaStream_t st)
{
    dim3 grid((nx + 31) / 32, (ny + 7) / 8);
    pi_norm_kernel<<<grid, dim3(32, 8), 0, st>>>(cnd, img, nx, ny, l2, fetch);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_residual(const KGeom &g, const float *meas, float *out, int dN, int sub, int step, int nrows,
                    cudaStream_t st)
{
    if (nrows <= 0 || dN <= 0) return XCT_OK;
    dim3 grid((g.px + 127) / 128, nrows, dN);
    residual_kernel<<<grid, 128, 0, st>>>(meas, out, g, sub, step);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_fista_bp(const KGeom &g, const float2 *trig, const float *x, float *v, const float *res, int dN, int sub,
                    float alpha, float L, cudaStream_t st)
{
    if (dN <= 0) return XCT_OK;
    dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, dN);
    fista_bp_kernel<<<grid, dim3(32, 8), 0, st>>>(x, v, res, trig, g, sub, alpha, L);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}
