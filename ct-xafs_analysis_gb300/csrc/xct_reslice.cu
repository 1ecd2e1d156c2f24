// xct_reslice.cu -- projection stack -> sinograms on the device (Reslice/).
//
// Replaces reslice() (Reslice/reslice_ocl.cpp:153-208) and denoiseSinogram()
// (:211-255) over the kernels reslice (reslice.cl:52-71) and denoiseSinogram
// (reslice.cl:223-248).  The reference uploads one projection at a time into an image,
// reslices it into an image array of (num_angle/iter) rows per layer and reads every layer
// back to host memory; here the whole projection stack (or a chunk of angles) is resident in
// HBM and the sinograms are written in the layout the OS-EM plans read directly: slice Y's
// sinogram [A][W] at d_sino + Y*A*W, so rows Y0..Y0+dN-1 are a ready dN-slice batch.
//
// Both kernels are HBM-bound element maps: X is the fastest index of the projections and of
// the sinograms, so reads and writes are coalesced along X and the angle/row transpose
// happens at whole-row granularity.  The arithmetic is the reference's, operation for
// operation (the sampler's bilinear sum as the OpenCL filtering formula writes it).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "xct_internal.h"

struct xct_reslice_plan {
    xct_ctx *ctx = nullptr;
    int W = 0, H = 0, A = 0;
    float baseup = 0.0f;
    int correction = 0;
    float *d_xs = nullptr;    // [A] per-angle x shift
    float *d_ys = nullptr;    // [A] per-angle y (z-drift) shift
    float *d_corr = nullptr;  // [W] cos(asin(2|X - W/2|/W)) when correction == 1
};

namespace {

__device__ __forceinline__ float tex2(const float *__restrict__ im, int W, int H, int i, int j)
{
    return (i >= 0 && j >= 0 && i < W && j < H) ? __ldg(im + (size_t)j * W + i) : 0.0f;
}

constexpr int kRowsPerThread = 8;  // output rows a thread walks (reslice: Y; denoise: th)

constexpr int kColsPerThread = 1;  // reslice: columns per thread (2 measured slower: fewer threads in flight)

// grid: (ceil(W/(256*kColsPerThread)), ceil(H/8), n); prj[Y][th0 + th][X] for projection th
// of the chunk.  A thread serves 8 rows Y of kColsPerThread columns X (256 apart).  The
// sampler rows j(Y) = floor(Y + sy) are the same for every column and consecutive unless
// rounding says otherwise (checked):
// then the 9 texel rows the 8 outputs need are loaded at once -- every load in flight
// together, each texel read once -- and each output is formed from registers with the
// reference's arithmetic; otherwise each row loads its own 2x2 footprint.
__global__ void __launch_bounds__(256) reslice_kernel(const float *__restrict__ mt, float *__restrict__ prj, int W,
                                                      int H, int A, int th0, const float *__restrict__ xs,
                                                      const float *__restrict__ ys, float baseup,
                                                      const float *__restrict__ corr)
{
    const int Yb = blockIdx.y * kRowsPerThread, th = blockIdx.z;
    const float *im = mt + (size_t)th * H * W;
    const float sx = __ldg(xs + th0 + th), sy = __ldg(ys + th0 + th);
    const int n = min(kRowsPerThread, H - Yb);
    int j[kRowsPerThread];
    float b[kRowsPerThread];
    bool run = true;
#pragma unroll
    for (int r = 0; r < kRowsPerThread; ++r) {
        const float vv = (((float)(Yb + r) + sy) + 0.5f) - 0.5f;
        const float fj = floorf(vv);
        b[r] = vv - fj;
        j[r] = (int)fj;
        if (r > 0 && r < n && j[r] != j[r - 1] + 1) run = false;
    }
    const size_t ostep = (size_t)A * W;
#pragma unroll
    for (int cc = 0; cc < kColsPerThread; ++cc) {
        const int X = blockIdx.x * (blockDim.x * kColsPerThread) + cc * blockDim.x + threadIdx.x;
        if (X >= W) break;
        const float uu = (((float)X + sx) + 0.5f) - 0.5f;
        const float fi = floorf(uu);
        const float a = uu - fi;
        const int i = (int)fi;
        const float cf = corr != nullptr ? __ldg(corr + X) : 1.0f;
        float *out = prj + ((size_t)Yb * A + th0 + th) * W + X;
        if (run) {
            // zero border: the column tests once per column, the row test once per row
            const bool in0 = (unsigned)i < (unsigned)W, in1 = (unsigned)(i + 1) < (unsigned)W;
            const float *col = im + i;
            float c0[kRowsPerThread + 1], c1[kRowsPerThread + 1];
#pragma unroll
            for (int r = 0; r <= kRowsPerThread; ++r) {
                const int jr = j[0] + r;
                const bool rok = r <= n && (unsigned)jr < (unsigned)H;
                const float *p = col + (size_t)(rok ? jr : 0) * W;
                c0[r] = (rok && in0) ? __ldg(p) : 0.0f;
                c1[r] = (rok && in1) ? __ldg(p + 1) : 0.0f;
            }
#pragma unroll
            for (int r = 0; r < kRowsPerThread; ++r) {
                if (r < n) {
                    float t = (1.0f - a) * (1.0f - b[r]) * c0[r] + a * (1.0f - b[r]) * c1[r] +
                              (1.0f - a) * b[r] * c0[r + 1] + a * b[r] * c1[r + 1];
                    t += baseup;
                    if (corr != nullptr) t *= cf;
                    out[r * ostep] = t;
                }
            }
        } else {
            for (int r = 0; r < n; ++r) {
                float t = (1.0f - a) * (1.0f - b[r]) * tex2(im, W, H, i, j[r]) +
                          a * (1.0f - b[r]) * tex2(im, W, H, i + 1, j[r]) +
                          (1.0f - a) * b[r] * tex2(im, W, H, i, j[r] + 1) +
                          a * b[r] * tex2(im, W, H, i + 1, j[r] + 1);
                t += baseup;
                if (corr != nullptr) t *= cf;
                out[r * ostep] = t;
            }
        }
    }
}

// grid: (ceil(W/256), ceil(A/8), H) over sinograms [H][A][W]; a thread walks 8 angles of one
// column with the three angle rows in registers; neighbours clamped to the edge.
__global__ void __launch_bounds__(256) denoise_kernel(const float *__restrict__ src, float *__restrict__ dst, int W,
                                                      int A, float thr)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int t0 = blockIdx.y * kRowsPerThread, Y = blockIdx.z;
    if (X >= W) return;
    const float *base = src + (size_t)Y * A * W + X;
    // rows t0-1 .. t0+8 (clamped), all loads first
    float f[kRowsPerThread + 2];
#pragma unroll
    for (int r = 0; r < kRowsPerThread + 2; ++r) f[r] = __ldg(base + (size_t)min(max(t0 - 1 + r, 0), A - 1) * W);
    float *out = dst + ((size_t)Y * A + t0) * W + X;
#pragma unroll
    for (int r = 0; r < kRowsPerThread; ++r) {
        if (t0 + r < A) {
            const float f3 = f[r], f1 = f[r + 1], f2 = f[r + 2];
            const float d1 = f2 - f1, d2 = f1 - f3;
            const float c = (f2 + f3) * 0.5f;  // == (f2 + f3) / 2.0f exactly (a power of two)
            out[(size_t)r * W] = ((d1 > thr && d2 < -thr) || (d1 < -thr && d2 > thr)) ? c : f1;
        }
    }
}

void reslice_free(xct_reslice_plan *p)
{
    if (!p) return;
    cudaFree(p->d_xs);
    cudaFree(p->d_ys);
    cudaFree(p->d_corr);
    delete p;
}

}  // namespace

extern "C" {

int xct_reslice_plan_create(xct_ctx *ctx, int width, int height, int n_angles, const float *xshift,
                            const float *yshift, float baseup, int correction, xct_reslice_plan **out)
{
    if (!ctx || !out) return xct_fail(XCT_E_INVALID, "xct_reslice_plan_create: null argument");
    *out = nullptr;
    if (width <= 0 || height <= 0 || n_angles <= 0 || width > 65536 || height > 65535 || n_angles > 65535)
        return xct_fail(XCT_E_INVALID, "xct_reslice_plan_create: width 1..65536, height and angles 1..65535");
    if (correction != 0 && correction != 1)
        return xct_fail(XCT_E_INVALID, "xct_reslice_plan_create: correction must be 0 or 1");
    if (!(fabsf(baseup) < 1.0e30f)) return xct_fail(XCT_E_INVALID, "xct_reslice_plan_create: baseup not finite");
    std::vector<float> xs(n_angles, 0.0f), ys(n_angles, 0.0f);
    for (int i = 0; i < n_angles; ++i) {
        if (xshift) xs[i] = xshift[i];
        if (yshift) ys[i] = yshift[i];
        if (!(fabsf(xs[i]) < 1.0e6f) || !(fabsf(ys[i]) < 1.0e6f))
            return xct_fail(XCT_E_INVALID, "xct_reslice_plan_create: shifts must be finite and below 1e6 pixels");
    }
    XCT_CUDA_TRY(cudaSetDevice(ctx->device));
    xct_reslice_plan *p = new (std::nothrow) xct_reslice_plan();
    if (!p) return xct_fail(XCT_E_NOMEM, "xct_reslice_plan_create: host allocation failed");
    p->ctx = ctx;
    p->W = width;
    p->H = height;
    p->A = n_angles;
    p->baseup = baseup;
    p->correction = correction;
    auto fail = [&](cudaError_t e, const char *what) {
        int r = xct_cuda_fail(e, what);
        reslice_free(p);
        return r;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&p->d_xs, sizeof(float) * n_angles)) != cudaSuccess) return fail(e, "cudaMalloc xshift");
    if ((e = cudaMalloc(&p->d_ys, sizeof(float) * n_angles)) != cudaSuccess) return fail(e, "cudaMalloc yshift");
    if ((e = cudaMemcpy(p->d_xs, xs.data(), sizeof(float) * n_angles, cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e, "upload xshift");
    if ((e = cudaMemcpy(p->d_ys, ys.data(), sizeof(float) * n_angles, cudaMemcpyHostToDevice)) != cudaSuccess)
        return fail(e, "upload yshift");
    if (correction == 1) {
        // theta = 2.0f*fabs((float)X - IMAGESIZE_X/2.0f)/IMAGESIZE_X; cos(asin(theta)) in float
        // (reslice.cl:65-67), each function correctly rounded
        std::vector<float> cf(width);
        for (int X = 0; X < width; ++X) {
            const float theta = 2.0f * fabsf((float)X - (float)width / 2.0f) / (float)width;
            cf[X] = (float)cos((double)(float)asin((double)theta));
        }
        if ((e = cudaMalloc(&p->d_corr, sizeof(float) * width)) != cudaSuccess) return fail(e, "cudaMalloc corr");
        if ((e = cudaMemcpy(p->d_corr, cf.data(), sizeof(float) * width, cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "upload corr");
    }
    *out = p;
    return XCT_OK;
}

int xct_reslice_plan_destroy(xct_reslice_plan *p)
{
    if (p) cudaSetDevice(p->ctx->device);
    reslice_free(p);
    return XCT_OK;
}

int xct_reslice(xct_reslice_plan *p, int first_angle, int n, const float *d_proj, float *d_sino, void *stream)
{
    if (!p) return xct_fail(XCT_E_INVALID, "xct_reslice: plan is null");
    if (!d_proj || !d_sino) return xct_fail(XCT_E_INVALID, "xct_reslice: null device pointer");
    if (n <= 0 || first_angle < 0 || first_angle + n > p->A) {
        char b[160];
        snprintf(b, sizeof b, "xct_reslice: angles [%d, %d) outside the plan's %d", first_angle, first_angle + n, p->A);
        return xct_fail(XCT_E_INVALID, b);
    }
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    dim3 grid((p->W + 256 * kColsPerThread - 1) / (256 * kColsPerThread), (p->H + kRowsPerThread - 1) / kRowsPerThread,
              n);
    reslice_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_proj, d_sino, p->W, p->H, p->A, first_angle, p->d_xs,
                                                           p->d_ys, p->baseup, p->d_corr);
    XCT_CUDA_TRY(cudaGetLastError());
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

int xct_denoise_sinogram(int width, int n_angles, int n_rows, float threshold, const float *d_src, float *d_dst,
                         void *stream)
{
    if (!d_src || !d_dst) return xct_fail(XCT_E_INVALID, "xct_denoise_sinogram: null device pointer");
    if (width <= 0 || n_angles <= 0 || n_rows <= 0 || n_angles > 65535 || n_rows > 65535)
        return xct_fail(XCT_E_INVALID, "xct_denoise_sinogram: sizes must be > 0 (angles, rows <= 65535)");
    const size_t bytes = sizeof(float) * (size_t)width * n_angles * n_rows;
    const char *s = (const char *)d_src, *d = (const char *)d_dst;
    if (s < d + bytes && d < s + bytes)
        return xct_fail(XCT_E_INVALID, "xct_denoise_sinogram: source and destination overlap");
    dim3 grid((width + 255) / 256, (n_angles + kRowsPerThread - 1) / kRowsPerThread, n_rows);
    denoise_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_src, d_dst, width, n_angles, threshold);
    XCT_CUDA_TRY(cudaGetLastError());
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

}  // extern "C"
