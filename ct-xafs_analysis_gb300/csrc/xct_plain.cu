// xct_plain.cu -- the plain per-slice kernels: one thread per ray for the forward
// projector, one thread per pixel for the backprojector, the launch shape of the
// reference (OSEM1 global (px, pa/ss, dN), OSEM2 global (ox, oy, dN), GPU.cpp:169-170).
//
// These are the "plain path" the tiled kernels are measured against, and the fallback
// for shapes the tiled kernels do not take.  They read the image straight from global
// memory through the read-only cache.
#include <algorithm>

#include "xct_device.cuh"

namespace {

constexpr int kFwdThreads = 128;

// OSEM1 (OSEM.cl:38-68) when meas != nullptr, projection (reconstShare.cl:213-241)
// otherwise.  Samples are summed in Y order, as in the reference work-item.
__global__ void __launch_bounds__(kFwdThreads) fwd_plain_kernel(const float *__restrict__ img,
                                                                const float *__restrict__ meas,
                                                                float *__restrict__ out,
                                                                const float2 *__restrict__ trig, KGeom g, int sub,
                                                                int step)
{
    const int X = blockIdx.x * kFwdThreads + threadIdx.x;
    const int k = blockIdx.y;
    const int z = blockIdx.z;
    if (X >= g.px) return;
    const int th = sub + k * step;
    const float2 cs = trig[th];
    const float *im = img + (size_t)z * g.nx * g.ny;
    const float Xc = (float)X - g.cx;
    const float ax = fmaf(Xc, cs.x, g.hx);
    const float ay = fmaf(Xc, -cs.y, g.hy);
    float acc = 0.0f;
    for (int Y = 0; Y < g.depth; ++Y) {
        const float Yc = (float)Y - g.hd;
        const float x = fmaf(Yc, cs.y, ax);
        const float y = fmaf(Yc, cs.x, ay);
        acc += xct_bilinear_global(im, g.nx, g.ny, x, y);
    }
    const size_t o = ((size_t)z * g.pa + th) * g.px + X;
    if (meas != nullptr) {
        const float yv = xct_measured(meas + (size_t)z * g.pa * g.px, g.px, g.pa, X, th, g.fetch);
        out[o] = xct_ratio(yv, acc);
    } else {
        out[o] = acc;
    }
}

// OSEM2 (OSEM.cl:71-105): b = sum over th = sub, sub+ss, ... of ratio[th][bin]; the
// image is updated in place (each pixel only reads itself).
__global__ void __launch_bounds__(256) bp_update_plain_kernel(float *__restrict__ img,
                                                              const float *__restrict__ ratio,
                                                              const float2 *__restrict__ trig, KGeom g, int sub)
{
    const int X = blockIdx.x * 32 + threadIdx.x;
    const int Y = blockIdx.y * 8 + threadIdx.y;
    const int z = blockIdx.z;
    if (X >= g.nx || Y >= g.ny) return;
    const float *rt = ratio + (size_t)z * g.pa * g.px;
    const float Xc = (float)X - g.hx;
    const float Yc = (float)Y - g.hy;
    float b = 0.0f;
    for (int th = sub; th < g.pa; th += g.ss) {
        const float2 cs = trig[th];
        const float t = xct_bin_coord(Xc, cs.x, Yc * cs.y, g.cx);
        const int bin = (int)floorf(t);
        b += ((unsigned)bin < (unsigned)g.px) ? __ldg(rt + (size_t)th * g.px + bin) : 0.0f;
    }
    float *p = img + ((size_t)z * g.ny + Y) * g.nx + X;
    *p = xct_update(*p, b, (float)g.ss, (float)g.pa);
}

// backProjection (reconstShare.cl:245-275): integer halves (IMAGESIZE_X/2 etc.), NaN
// samples -> 0, result b * SS / PRJ_ANGLESIZE / DEPTHSIZE.
__global__ void __launch_bounds__(256) bp_ref_plain_kernel(float *__restrict__ img, const float *__restrict__ prj,
                                                           const float2 *__restrict__ trig, KGeom g, int sub,
                                                           int step)
{
    const int X = blockIdx.x * 32 + threadIdx.x;
    const int Y = blockIdx.y * 8 + threadIdx.y;
    const int z = blockIdx.z;
    if (X >= g.nx || Y >= g.ny) return;
    const float *pr = prj + (size_t)z * g.pa * g.px;
    const float Xc = (float)(X - g.nx / 2);
    const float Yc = (float)(Y - g.ny / 2);
    const float ch = (float)(g.px / 2);
    float b = 0.0f;
    for (int th = sub; th < g.pa; th += step) {
        const float2 cs = trig[th];
        const float t = ((Xc * cs.x - Yc * cs.y) + ch) + 0.5f;
        const int bin = (int)floorf(t);
        float v = ((unsigned)bin < (unsigned)g.px) ? __ldg(pr + (size_t)th * g.px + bin) : 0.0f;
        v = (v != v) ? 0.0f : v;
        b += v;
    }
    img[((size_t)z * g.ny + Y) * g.nx + X] = ((b * (float)step) / (float)g.pa) / (float)g.depth;
}

// sinogramCorrection (reconstShare.cl:35-70), modes 1..4.  The transcendental factors
// are tabulated on the host (ang_fac[2*th] = cos(angle_pr), ang_fac[2*th+1] = sinfactor,
// bin_fac[X] = cos(asin(theta))), so the kernel is pure multiplies/compares.
__device__ __forceinline__ float sino_corrected(float v, int X, int th, int px, const float *__restrict__ ang_fac,
                                                const float *__restrict__ bin_fac, int mode)
{
    const float ca = ang_fac[2 * th], sf = ang_fac[2 * th + 1];
    const float theta = 2.0f * fabsf((float)X - (float)px / 2.0f) / (float)px;
    switch (mode) {
    case 4: return (theta * theta < sf * sf) ? v : 0.0f;
    case 3: return v * (bin_fac[X] * ca);
    case 2: return v * ca;
    case 1: return v * bin_fac[X];
    default: return v;
    }
}

__global__ void sino_correction_kernel(const float *__restrict__ src, float *__restrict__ dst,
                                       const float *__restrict__ ang_fac, const float *__restrict__ bin_fac, KGeom g,
                                       int mode)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int th = blockIdx.y;
    const int z = blockIdx.z;
    if (X >= g.px) return;
    const size_t o = ((size_t)z * g.pa + th) * g.px + X;
    dst[o] = sino_corrected(src[o], X, th, g.px, ang_fac, bin_fac, mode);
}

// The same for every item of a batch with a correction: block (x, th, item).
__global__ void sino_correction_batched_kernel(const XctItemDev *__restrict__ items)
{
    const XctItemDev &it = items[blockIdx.z];  // items: this launch's first item
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int th = blockIdx.y;
    if (it.corr_mode <= 0 || X >= it.g.px || th >= it.g.pa) return;
    const size_t o = (size_t)th * it.g.px + X;
    it.corr[o] = sino_corrected(it.sino_in[o], X, th, it.g.px, it.corr_ang, it.corr_bin, it.corr_mode);
}

}  // namespace

int launch_fwd_plain(const KGeom &g, const float2 *trig, const float *img, const float *meas, float *out, int dN,
                     int sub, int step, int nrows, cudaStream_t st)
{
    if (nrows <= 0 || dN <= 0) return XCT_OK;
    dim3 grid((g.px + kFwdThreads - 1) / kFwdThreads, nrows, dN);
    fwd_plain_kernel<<<grid, kFwdThreads, 0, st>>>(img, meas, out, trig, g, sub, step);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_bp_update_plain(const KGeom &g, const float2 *trig, float *img, const float *ratio, int dN, int sub,
                           cudaStream_t st)
{
    if (dN <= 0) return XCT_OK;
    dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, dN);
    bp_update_plain_kernel<<<grid, dim3(32, 8), 0, st>>>(img, ratio, trig, g, sub);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_bp_ref_plain(const KGeom &g, const float2 *trig, const float *prj, float *img, int dN, int sub, int step,
                        cudaStream_t st)
{
    if (dN <= 0) return XCT_OK;
    dim3 grid((g.nx + 31) / 32, (g.ny + 7) / 8, dN);
    bp_ref_plain_kernel<<<grid, dim3(32, 8), 0, st>>>(img, prj, trig, g, sub, step);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_sino_correction(const KGeom &g, const float *src, float *dst, const float *ang_fac, const float *bin_fac,
                           int mode, int dN, cudaStream_t st)
{
    if (dN <= 0) return XCT_OK;
    dim3 grid((g.px + 127) / 128, g.pa, dN);
    sino_correction_kernel<<<grid, 128, 0, st>>>(src, dst, ang_fac, bin_fac, g, mode);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

// One launch per 65535 items (the grid's z limit); captured, so counted per replay.
int launch_sino_correction_batched(const XctItemDev *items, int n, int max_px, int max_pa, cudaStream_t st)
{
    if (max_pa > 65535) return xct_fail(XCT_E_UNSUPPORTED, "sinogram correction in a batch: more than 65535 angles");
    for (int first = 0; first < n; first += 65535) {
        dim3 grid((max_px + 127) / 128, max_pa, std::min(65535, n - first));
        sino_correction_batched_kernel<<<grid, 128, 0, st>>>(items + first);
        XCT_CUDA_TRY(cudaGetLastError());
    }
    return XCT_OK;
}
