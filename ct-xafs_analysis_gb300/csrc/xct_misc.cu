// xct_misc.cu -- device micro-benchmark used for the roofline denominator of the
// forward/backward projectors, which are bound by the FP32 and shared-memory pipes rather
// than by HBM or the tensor cores.
#include "xct_internal.h"

namespace {

// 8 independent FMA chains per thread, 256 threads per CTA: enough independent work to
// keep every SMSP's FMA pipe busy.  The result is stored so nothing is dead code.
__global__ void __launch_bounds__(256) fma_peak_kernel(float *out, int iters, float a, float b)
{
    float v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = (float)(threadIdx.x + i);
    for (int n = 0; n < iters; ++n) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = fmaf(v[i], a, b);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += v[i];
    if (s == 1.2345f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int xct_fp32_peak(int device, float *tflops)
{
    if (!tflops) return xct_fail(XCT_E_INVALID, "xct_fp32_peak: null");
    XCT_CUDA_TRY(cudaSetDevice(device));
    cudaDeviceProp p;
    XCT_CUDA_TRY(cudaGetDeviceProperties(&p, device));
    const int blocks = p.multiProcessorCount * 8, threads = 256, iters = 4096;
    float *out = nullptr;
    XCT_CUDA_TRY(cudaMalloc(&out, sizeof(float) * blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 0.0f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        fma_peak_kernel<<<blocks, threads>>>(out, iters, 0.999999f, 1.0e-6f);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flop = 2.0 * 8 * 16 * (double)iters * blocks * threads;
        if (ms > 0.0f) best = fmaxf(best, (float)(flop / (ms * 1.0e-3) / 1.0e12));
    }
    g_xct_launches.fetch_add(4, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return xct_cuda_fail(e, "fma_peak_kernel");
    *tflops = best;
    return XCT_OK;
}

extern "C" int xct_check_report(xct_ctx *ctx, long long *count, int *site, long long *index, long long *lo,
                                long long *hi)
{
    if (!ctx || !count) return xct_fail(XCT_E_INVALID, "xct_check_report: null argument");
#ifdef XCT_CHECKED
    XCT_CUDA_TRY(cudaSetDevice(ctx->device));
    XCT_CUDA_TRY(cudaDeviceSynchronize());
    int (*const readers[])(XctCheckWord *, bool) = {xct_check_read_tiled, xct_check_read_fbp};
    long long total = 0;
    XctCheckWord first = {};
    for (auto rd : readers) {
        XctCheckWord w = {};
        if (rd(&w, true) != 0) return xct_fail(XCT_E_CUDA, "xct_check_report: reading a check word failed");
        if (w.count != 0 && total == 0) first = w;
        total += (long long)w.count;
    }
    *count = total;
    if (site) *site = first.site;
    if (index) *index = first.value;
    if (lo) *lo = first.lo;
    if (hi) *hi = first.hi;
    return XCT_OK;
#else
    (void)site;
    (void)index;
    (void)lo;
    (void)hi;
    *count = -1;
    return xct_fail(XCT_E_UNSUPPORTED, "xct_check_report: this library was built without bounds checks "
                                       "(the checked build is libxct_checked.so)");
#endif
}
