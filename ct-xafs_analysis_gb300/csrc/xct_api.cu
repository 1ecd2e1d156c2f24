// xct_api.cu -- the C ABI of libxct (include/xct.h): device context, OS-EM plans, the
// subset/iteration loop and the operator entry points.
//
// Replaces, for the OS-EM path of CT_reconstruction:
//   OCL_platform_device (share source/OCL_platform_device_class.cpp:55-208)  -> xct_ctx_*
//   OSEM_programBuild   (CT_reconstruction/GPU.cpp:513-559)                  -> xct_osem_plan_create
//   OSEM_execution      (GPU.cpp:125-240) + OSEM_thread copies (:440-463)    -> xct_osem_run[_device]
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <mutex>
#include <new>
#include <string>

#include "xct_internal.h"

std::atomic<long long> g_xct_launches{0};

namespace {
thread_local std::string t_last_error;
}

int xct_fail(int code, const std::string &msg)
{
    t_last_error = msg;
    return code;
}

int xct_cuda_fail(cudaError_t e, const char *what)
{
    char buf[512];
    snprintf(buf, sizeof buf, "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    t_last_error = buf;
    return e == cudaErrorMemoryAllocation ? XCT_E_NOMEM : XCT_E_CUDA;
}

// Per-angle (cos, sin): angle_pr = angle[th]*PI/180.0f with PI a double literal
// (OSEM.cl:2,57), stored to float; then the float cos/sin of that float, correctly
// rounded.  The oracle builds the identical table (oracle/xct_oracle.c, xo_trig_f32).
void xct_trig_table(const float *ang_deg, int pa, std::vector<float2> &cs)
{
    cs.resize(pa);
    for (int th = 0; th < pa; ++th) {
        const float phi = (float)(((double)ang_deg[th] * 3.14159265358979323846) / 180.0);
        cs[th].x = (float)cos((double)phi);
        cs[th].y = (float)sin((double)phi);
    }
}

// sinogramCorrection factors (reconstShare.cl:44-64): angle_pr = angle/180*PI (float
// division, then a double PI, stored to float); a = b = 0.5 (GPU.cpp:182-183); per angle
// cos(angle_pr) and the sine factor a + b cos, per bin cos(asin(theta)).
void xct_corr_tables(const float *ang_deg, int pa, int px, std::vector<float> &af, std::vector<float> &bf)
{
    af.assign(2 * (size_t)pa, 0.0f);
    bf.assign((size_t)px, 0.0f);
    for (int th = 0; th < pa; ++th) {
        const float q = ang_deg[th] / 180.0f;
        const float apr = (float)((double)q * 3.14159265358979323846);
        const float ca = (float)cos((double)apr);
        af[2 * th] = ca;
        af[2 * th + 1] = 0.5f + 0.5f * ca;
    }
    for (int X = 0; X < px; ++X) {
        const float theta = 2.0f * fabsf((float)X - (float)px / 2.0f) / (float)px;
        const float as = (float)asin((double)theta);
        bf[X] = (float)cos((double)as);
    }
}

// Subset order of OSEM_ocl (GPU.cpp:564-582): a power-of-two ss gives the bit-reversal
// permutation (0, ss/2, ss/4, 3ss/4, ...); any other ss the identity.  Entry k alone:
int xct_subset_at(int ss, int k)
{
    if (ss <= 0 || (ss & (ss - 1)) != 0) return k;
    int bits = 0;
    while ((1 << bits) < ss) ++bits;
    int r = 0;
    for (int b = 0; b < bits; ++b)
        if (k & (1 << b)) r |= 1 << (bits - 1 - b);
    return r;
}

// ... and the whole order.
void xct_subset_order_host(int ss, int *sub)
{
    for (int j = 0; j < ss; ++j) sub[j] = xct_subset_at(ss, j);
}

// The kernels' lambda: -D LAMBDA_FISTA is the float CSlambda written by an ostream (six
// significant digits, GPU.cpp:549) and compiled as a double literal; lambda =
// LAMBDA_FISTA/L[sub]*0.5f with L[sub] = 0.5 for every subset (GPU.cpp:343, FISTA.cl:426).
float xct_cs_kernel_lambda(float cs_lambda)
{
    char b[64];
    snprintf(b, sizeof b, "%g", (double)cs_lambda);
    const double d = strtod(b, nullptr);
    return (float)(d / (double)0.5f * 0.5);
}

extern "C" {

const char *xct_last_error(void) { return t_last_error.c_str(); }
int xct_abi_version(void) { return XCT_ABI_VERSION; }
long long xct_launch_count(void) { return g_xct_launches.load(); }

int xct_subset_order(int ss, int *sub)
{
    if (ss <= 0 || sub == nullptr) return xct_fail(XCT_E_INVALID, "xct_subset_order: ss must be > 0");
    xct_subset_order_host(ss, sub);
    return XCT_OK;
}

int xct_device_count(int *count)
{
    if (!count) return xct_fail(XCT_E_INVALID, "xct_device_count: null");
    XCT_CUDA_TRY(cudaGetDeviceCount(count));
    return XCT_OK;
}

int xct_device_name(int device, char *buf, int buflen)
{
    if (!buf || buflen <= 0) return xct_fail(XCT_E_INVALID, "xct_device_name: bad buffer");
    cudaDeviceProp p;
    XCT_CUDA_TRY(cudaGetDeviceProperties(&p, device));
    snprintf(buf, buflen, "%s", p.name);
    return XCT_OK;
}

int xct_ctx_create(int device, xct_ctx **out)
{
    if (!out) return xct_fail(XCT_E_INVALID, "xct_ctx_create: out is null");
    *out = nullptr;
    int n = 0;
    XCT_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) {
        char b[128];
        snprintf(b, sizeof b, "xct_ctx_create: device %d out of range (%d devices)", device, n);
        return xct_fail(XCT_E_INVALID, b);
    }
    cudaDeviceProp p;
    XCT_CUDA_TRY(cudaGetDeviceProperties(&p, device));
    if (!(p.major == 10 && p.minor == 3)) {
        char b[512];
        snprintf(b, sizeof b, "libxct is built for sm_103a (GB300); device %d (%s) is sm_%d%d", device, p.name,
                 p.major, p.minor);
        return xct_fail(XCT_E_UNSUPPORTED, b);
    }
    XCT_CUDA_TRY(cudaSetDevice(device));
    xct_ctx *c = new (std::nothrow) xct_ctx();
    if (!c) return xct_fail(XCT_E_NOMEM, "xct_ctx_create: host allocation failed");
    c->device = device;
    c->sm_count = p.multiProcessorCount;
    c->max_smem_optin = (int)p.sharedMemPerBlockOptin;
    snprintf(c->name, sizeof c->name, "%s", p.name);
    *out = c;
    return XCT_OK;
}

int xct_ctx_destroy(xct_ctx *ctx)
{
    delete ctx;
    return XCT_OK;
}

static void plan_free(xct_plan *p)
{
    if (!p) return;
    cudaFree(p->d_trig);
    cudaFree(p->d_sino);
    cudaFree(p->d_img);
    cudaFree(p->d_ratio);
    cudaFree(p->d_corr);
    cudaFree(p->d_corr_ang);
    cudaFree(p->d_corr_bin);
    cudaFree(p->d_acc);
    cudaFree(p->d_min_keys);
    cudaFree(p->d_red);
    cudaFree(p->d_rc_prm);
    cudaFree(p->d_fi);
    cudaFree(p->d_cs);
    cudaFree(p->d_fista);
    cudaFree(p->d_pi);
    cudaFree(p->d_pi_l2);
    cudaFree(p->d_sino2);
    cudaFree(p->d_img2);
    if (p->s_h2d) cudaStreamDestroy(p->s_h2d);
    if (p->s_d2h) cudaStreamDestroy(p->s_d2h);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    if (p->s_aux) cudaStreamDestroy(p->s_aux);
    if (p->ev_fork) cudaEventDestroy(p->ev_fork);
    if (p->ev_join) cudaEventDestroy(p->ev_join);
    delete p;
}

static int check_geom(const xct_geom *g)
{
    if (!g) return xct_fail(XCT_E_INVALID, "geometry is null");
    if (g->nx <= 0 || g->ny <= 0 || g->px <= 0 || g->pa <= 0 || g->ss <= 0 || g->it < 0)
        return xct_fail(XCT_E_INVALID, "geometry: nx, ny, px, pa, ss must be > 0 and it >= 0");
    if (g->ox != g->nx || g->oy != g->ny)
        return xct_fail(XCT_E_INVALID,
                        "geometry: output ROI smaller than the reconstruction (ox < nx) is not supported; the "
                        "reference's own ROI path updates a different region than it reads back (GPU.cpp:152-170)");
    if (g->ss > g->pa) return xct_fail(XCT_E_INVALID, "geometry: more subsets than angles");
    if (!(g->center_bin < 2.0f * (float)g->px))
        return xct_fail(XCT_E_INVALID, "geometry: center_bin must be finite and below 2*px (< 0 selects px/2)");
    if (!g->angles_deg) return xct_fail(XCT_E_INVALID, "geometry: angles_deg is null");
    if (g->nx > 16384 || g->ny > 16384 || g->px > 65536 || g->pa > 65536)
        return xct_fail(XCT_E_INVALID, "geometry: size beyond the supported maximum (16384 px image, 65536 bins)");
    if (g->measured_fetch_mode != XCT_FETCH_EXACT && g->measured_fetch_mode != XCT_FETCH_AVG2X2)
        return xct_fail(XCT_E_INVALID, "geometry: measured_fetch_mode must be XCT_FETCH_EXACT or XCT_FETCH_AVG2X2");
    if (g->subset_mode != XCT_SUBSETS_REF && g->subset_mode != XCT_SUBSETS_COVER)
        return xct_fail(XCT_E_INVALID, "geometry: subset_mode must be XCT_SUBSETS_REF or XCT_SUBSETS_COVER");
    if (g->correction_mode < 0 || g->correction_mode > 4)
        return xct_fail(XCT_E_INVALID, "geometry: correction_mode must be 0..4");
    if (g->max_batch <= 0) return xct_fail(XCT_E_INVALID, "geometry: max_batch must be > 0");
    if (g->kernels != XCT_KERNELS_TILED && g->kernels != XCT_KERNELS_PLAIN)
        return xct_fail(XCT_E_INVALID, "geometry: kernels must be XCT_KERNELS_TILED or XCT_KERNELS_PLAIN");
    for (int i = 0; i < g->pa; ++i)
        if (!(fabsf(g->angles_deg[i]) < 1.0e6f)) return xct_fail(XCT_E_INVALID, "geometry: non-finite angle");
    return XCT_OK;
}

int xct_osem_plan_create(xct_ctx *ctx, const xct_geom *geom, xct_plan **out)
{
    if (!ctx || !out) return xct_fail(XCT_E_INVALID, "xct_osem_plan_create: null argument");
    *out = nullptr;
    int rc = check_geom(geom);
    if (rc) return rc;
    XCT_CUDA_TRY(cudaSetDevice(ctx->device));
    xct_plan *p = new (std::nothrow) xct_plan();
    if (!p) return xct_fail(XCT_E_NOMEM, "xct_osem_plan_create: host allocation failed");
    p->ctx = ctx;
    p->g = *geom;
    p->angles.assign(geom->angles_deg, geom->angles_deg + geom->pa);
    p->g.angles_deg = nullptr;
    p->sub_default.resize(geom->ss);
    xct_subset_order_host(geom->ss, p->sub_default.data());
    KGeom &k = p->kg;
    k.nx = geom->nx;
    k.ny = geom->ny;
    k.px = geom->px;
    k.pa = geom->pa;
    k.ss = geom->ss;
    k.depth = std::max(geom->nx, geom->ny);
    k.hx = (float)geom->nx * 0.5f;
    k.hy = (float)geom->ny * 0.5f;
    k.hd = (float)k.depth * 0.5f;
    k.cx = geom->center_bin < 0.0f ? (float)geom->px * 0.5f : geom->center_bin;
    k.fetch = geom->measured_fetch_mode;
    xct_plan_default_tuning(p);  // cached choice for this shape, else the default rule

    auto fail = [&](cudaError_t e, const char *what) {
        int r = xct_cuda_fail(e, what);
        plan_free(p);
        return r;
    };
    const size_t nb = (size_t)geom->max_batch;
    const size_t nimg = (size_t)geom->nx * geom->ny, nprj = (size_t)geom->px * geom->pa;
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
    if ((e = cudaEventCreate(&p->ev0)) != cudaSuccess) return fail(e, "event");
    if ((e = cudaEventCreate(&p->ev1)) != cudaSuccess) return fail(e, "event");
    if ((e = cudaStreamCreateWithFlags(&p->s_aux, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
    if ((e = cudaEventCreateWithFlags(&p->ev_fork, cudaEventDisableTiming)) != cudaSuccess) return fail(e, "event");
    if ((e = cudaEventCreateWithFlags(&p->ev_join, cudaEventDisableTiming)) != cudaSuccess) return fail(e, "event");
    if ((e = cudaMalloc(&p->d_trig, sizeof(float2) * geom->pa)) != cudaSuccess) return fail(e, "cudaMalloc trig");
    if ((e = cudaMalloc(&p->d_sino, sizeof(float) * nb * nprj)) != cudaSuccess) return fail(e, "cudaMalloc sino");
    if ((e = cudaMalloc(&p->d_img, sizeof(float) * nb * nimg)) != cudaSuccess) return fail(e, "cudaMalloc img");
    if ((e = cudaMalloc(&p->d_ratio, sizeof(float) * nb * nprj)) != cudaSuccess) return fail(e, "cudaMalloc ratio");
    if ((e = cudaMalloc(&p->d_min_keys, sizeof(int) * nb)) != cudaSuccess) return fail(e, "cudaMalloc min keys");
    if ((e = cudaMalloc(&p->d_red, sizeof(double) * 2 * nb)) != cudaSuccess) return fail(e, "cudaMalloc red");
    if ((e = cudaMemsetAsync(p->d_red, 0, sizeof(double) * 2 * nb, p->stream)) != cudaSuccess)
        return fail(e, "memset red");
    if ((e = cudaMalloc(&p->d_rc_prm, sizeof(float) * 16 * nb)) != cudaSuccess) return fail(e, "cudaMalloc prm");
    if ((e = cudaMalloc(&p->d_fi, sizeof(float) * nb)) != cudaSuccess) return fail(e, "cudaMalloc findex");
    if ((e = cudaMemsetAsync(p->d_ratio, 0, sizeof(float) * nb * nprj, p->stream)) != cudaSuccess)
        return fail(e, "memset ratio");
    if (geom->kernels == XCT_KERNELS_TILED) {
        // ray-sum accumulator for the largest subset (OSEM2 reads ceil(pa/ss) rows)
        p->acc_rows = (geom->pa + geom->ss - 1) / geom->ss;
        const size_t n = nb * (size_t)p->acc_rows * geom->px;
        if ((e = cudaMalloc(&p->d_acc, sizeof(double) * n)) != cudaSuccess) return fail(e, "cudaMalloc acc");
        if ((e = cudaMemsetAsync(p->d_acc, 0, sizeof(double) * n, p->stream)) != cudaSuccess)
            return fail(e, "memset acc");
    }
    std::vector<float2> cs;
    xct_trig_table(p->angles.data(), geom->pa, cs);
    if ((e = cudaMemcpyAsync(p->d_trig, cs.data(), sizeof(float2) * geom->pa, cudaMemcpyHostToDevice, p->stream)) !=
        cudaSuccess)
        return fail(e, "upload trig");
    if (geom->correction_mode > 0) {
        // sinogramCorrection factors (reconstShare.cl:44-64): angle_pr = angle/180*PI
        // (float division, then a double PI, stored to float); a = b = 0.5
        // (GPU.cpp:182-183).
        std::vector<float> af, bf;
        xct_corr_tables(p->angles.data(), geom->pa, geom->px, af, bf);
        if ((e = cudaMalloc(&p->d_corr, sizeof(float) * nb * nprj)) != cudaSuccess) return fail(e, "cudaMalloc corr");
        if ((e = cudaMalloc(&p->d_corr_ang, sizeof(float) * af.size())) != cudaSuccess) return fail(e, "corr ang");
        if ((e = cudaMalloc(&p->d_corr_bin, sizeof(float) * bf.size())) != cudaSuccess) return fail(e, "corr bin");
        if ((e = cudaMemcpy(p->d_corr_ang, af.data(), sizeof(float) * af.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            return fail(e, "upload corr ang");
        if ((e = cudaMemcpy(p->d_corr_bin, bf.data(), sizeof(float) * bf.size(), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            return fail(e, "upload corr bin");
    }
    if ((e = cudaStreamSynchronize(p->stream)) != cudaSuccess) return fail(e, "plan sync");
    *out = p;
    return XCT_OK;
}

int xct_osem_plan_destroy(xct_plan *plan)
{
    if (plan) cudaSetDevice(plan->ctx->device);
    plan_free(plan);
    return XCT_OK;
}

// Rows OSEM1 forward-projects for subset `sub` (GPU.cpp:169: pa/ss rows), or every row
// OSEM2 reads (ceil((pa - sub)/ss)) in XCT_SUBSETS_COVER mode.
static inline int subset_rows(const xct_plan *p, int sub)
{
    const int pa = p->g.pa, ss = p->g.ss;
    return p->g.subset_mode == XCT_SUBSETS_COVER ? (pa - sub + ss - 1) / ss : pa / ss;
}

// First-half size of a batch that runs as two halves on two streams.  With the
// slice-interleaved forward projector on, the cut falls on a multiple of its slice group, so
// that each half keeps whole groups (10 slices: 8 | 2; 16: 8 | 8; 20: 8 | 12; 8: 8 | 0, no
// split); otherwise in the middle.
static int xct_osem_split(const xct_plan *p, int dN)
{
    const int G = fwd_ms_slices();
    if (p->g.kernels == XCT_KERNELS_TILED && p->kg.ms_chunk > 0 && dN >= G) return G * ((dN / G + 1) / 2);
    return (dN + 1) / 2;
}

// One subset step (OSEM1 then OSEM2) of dN slices with the given plan buffers (ratio
// [dN][pa][px], accumulator [dN][rows][px]) on one stream.
static int subset_step(xct_plan *p, int dN, const float *meas, float *d_img, float *ratio, double *acc, int s,
                       cudaStream_t st)
{
    const KGeom &g = p->kg;
    int rc;
    if (p->g.kernels == XCT_KERNELS_TILED) {
        rc = launch_fwd_tiled(g, p->d_trig, d_img, meas, ratio, acc, dN, s, g.ss, subset_rows(p, s), st);
        if (rc) return rc;
        return launch_bp_update_tiled(g, p->d_trig, d_img, ratio, dN, s, st);
    }
    rc = launch_fwd_plain(g, p->d_trig, d_img, meas, ratio, dN, s, g.ss, subset_rows(p, s), st);
    if (rc) return rc;
    return launch_bp_update_plain(g, p->d_trig, d_img, ratio, dN, s, st);
}

// The subset/iteration loop over dN slices with the given plan buffers on one stream.
static int osem_loop_range(xct_plan *p, int dN, const float *meas, float *d_img, float *ratio, double *acc,
                           const int *sub, int it, cudaStream_t st)
{
    for (int i = 0; i < it; ++i)
        for (int k = 0; k < p->g.ss; ++k) {
            const int rc = subset_step(p, dN, meas, d_img, ratio, acc, sub[k], st);
            if (rc) return rc;
        }
    return XCT_OK;
}

// One subset step of a batch of two or more slices as two halves on two streams (the
// caller's and the plan's s_aux), joined back into the caller's stream.
static int subset_step_split(xct_plan *p, int dN, const float *meas, float *d_img, int s, cudaStream_t st)
{
    const KGeom &g = p->kg;
    const int d0 = xct_osem_split(p, dN);
    if (d0 >= dN) return subset_step(p, dN, meas, d_img, p->d_ratio, p->d_acc, s, st);
    const size_t nimg = (size_t)g.nx * g.ny, nprj = (size_t)g.px * g.pa;
    double *acc1 = p->d_acc ? p->d_acc + (size_t)d0 * p->acc_rows * g.px : nullptr;
    XCT_CUDA_TRY(cudaEventRecord(p->ev_fork, st));
    XCT_CUDA_TRY(cudaStreamWaitEvent(p->s_aux, p->ev_fork, 0));
    int rc = subset_step(p, d0, meas, d_img, p->d_ratio, p->d_acc, s, st);
    if (rc == XCT_OK)
        rc = subset_step(p, dN - d0, meas + d0 * nprj, d_img + d0 * nimg, p->d_ratio + d0 * nprj, acc1, s, p->s_aux);
    const cudaError_t e1 = cudaEventRecord(p->ev_join, p->s_aux);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(st, p->ev_join, 0) : e1;
    if (rc) return rc;
    if (e2 != cudaSuccess) return xct_cuda_fail(e2, "subset step: join");
    return XCT_OK;
}

// The subset/iteration loop of OSEM_execution (GPU.cpp:199-229) for dN slices already on
// the device.  The dest image and its copy-back (GPU.cpp:165, 226) are folded away: the
// backprojection update is done in place, which is equivalent because each pixel's new
// value depends only on its own old value and the ratio image.  The slices are independent,
// so a batch of two or more runs as two halves on two streams (the caller's and the plan's
// s_aux, joined back into the caller's by events): the kernels of one half fill the SMs that
// the other half's last waves of CTAs leave idle (measured +3.7 % on 10 slices of 2048^2).
static int osem_loop(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it,
                     cudaStream_t st, bool correct = true)
{
    const KGeom &g = p->kg;
    const float *meas = d_sino;
    if (correct && p->g.correction_mode > 0) {
        int rc = launch_sino_correction(g, d_sino, p->d_corr, p->d_corr_ang, p->d_corr_bin, p->g.correction_mode, dN,
                                        st);
        if (rc) return rc;
        meas = p->d_corr;
    }
    const int d0 = xct_osem_split(p, dN), d1 = dN - d0;
    if (dN < 2 || it == 0 || d1 == 0) return osem_loop_range(p, dN, meas, d_img, p->d_ratio, p->d_acc, sub, it, st);
    const size_t nimg = (size_t)g.nx * g.ny, nprj = (size_t)g.px * g.pa;
    double *acc1 = p->d_acc ? p->d_acc + (size_t)d0 * p->acc_rows * g.px : nullptr;
    XCT_CUDA_TRY(cudaEventRecord(p->ev_fork, st));
    XCT_CUDA_TRY(cudaStreamWaitEvent(p->s_aux, p->ev_fork, 0));
    int rc = osem_loop_range(p, d0, meas, d_img, p->d_ratio, p->d_acc, sub, it, st);
    if (rc == XCT_OK)
        rc = osem_loop_range(p, d1, meas + d0 * nprj, d_img + d0 * nimg, p->d_ratio + d0 * nprj, acc1, sub, it,
                             p->s_aux);
    // join in every case, so that the caller's stream never runs ahead of work still queued
    const cudaError_t e1 = cudaEventRecord(p->ev_join, p->s_aux);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(st, p->ev_join, 0) : e1;
    if (rc) return rc;
    if (e2 != cudaSuccess) return xct_cuda_fail(e2, "osem_loop: join");
    return XCT_OK;
}

// ---- tracing: XCT_TRACE=<file> (or 1 for stderr) ------------------------------------
// Every xct_osem_run_device / xct_osem_run call of a plan without a sinogram correction then
// runs with CUDA events around each launch, synchronously, and appends one JSON line: the
// shape, dN, iterations, the summed milliseconds and launch counts per kernel kind, and per
// subset step [forward, finalize, backprojection] milliseconds in launch order.
static std::mutex g_trace_mu;
static FILE *trace_file()
{
    static FILE *f = nullptr;
    static bool init = false;
    std::lock_guard<std::mutex> lk(g_trace_mu);
    if (!init) {
        init = true;
        const char *v = getenv("XCT_TRACE");
        if (v && *v && strcmp(v, "0") != 0) {
            if (strcmp(v, "1") == 0 || strcmp(v, "stderr") == 0) f = stderr;
            else f = fopen(v, "a");
        }
    }
    return f;
}
static int osem_loop_timed(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *so, int it,
                           cudaStream_t st, float *ms, long long *launches, std::vector<float> *per_launch);
// osem_loop, traced when XCT_TRACE is set
static int osem_loop_maybe_traced(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *so, int it,
                                  cudaStream_t st, const char *call)
{
    FILE *f = trace_file();
    if (!f || p->g.correction_mode > 0) return osem_loop(p, dN, d_sino, d_img, so, it, st);
    float ms[4];
    long long n[4];
    std::vector<float> per;
    int rc = osem_loop_timed(p, dN, d_sino, d_img, so, it, st, ms, n, &per);
    if (rc) return rc;
    std::string line;
    char b[512];
    snprintf(b, sizeof b,
             "{\"call\": \"%s\", \"device\": %d, \"nx\": %d, \"ny\": %d, \"px\": %d, \"pa\": %d, "
             "\"ss\": %d, \"it\": %d, \"dN\": %d, \"kernels\": \"%s\", \"fwd_tile\": %d, \"ang_chunk\": %d, "
             "\"ms\": {\"fwd\": %.4f, \"finalize\": %.4f, \"bp\": %.4f, \"total\": %.4f}, "
             "\"launches\": %lld, \"slice_iters_per_s\": %.4f, \"subset_ms\": [",
             call, p->ctx->device, p->g.nx, p->g.ny, p->g.px, p->g.pa, p->g.ss, it, dN,
             p->g.kernels == XCT_KERNELS_TILED ? "tiled" : "plain", p->kg.fwd_T, p->kg.fwd_chunk, ms[0], ms[1], ms[2],
             ms[3], n[3], ms[3] > 0.0f ? dN * it / (ms[3] * 1e-3) : 0.0);
    line = b;
    for (size_t j = 0; j + 2 < per.size(); j += 3) {
        snprintf(b, sizeof b, "%s[%.4f, %.4f, %.4f]", j ? ", " : "", per[j], per[j + 1], per[j + 2]);
        line += b;
    }
    line += "]}\n";
    std::lock_guard<std::mutex> lk(g_trace_mu);
    fputs(line.c_str(), f);
    fflush(f);
    return XCT_OK;
}

static int check_run(xct_plan *p, int dN, const int *sub, int it)
{
    if (!p) return xct_fail(XCT_E_INVALID, "plan is null");
    if (dN <= 0 || dN > p->g.max_batch) {
        char b[160];
        snprintf(b, sizeof b, "dN=%d outside [1, max_batch=%d] of the plan", dN, p->g.max_batch);
        return xct_fail(XCT_E_INVALID, b);
    }
    if (it < 0) return xct_fail(XCT_E_INVALID, "iterations must be >= 0");
    if (sub)
        for (int k = 0; k < p->g.ss; ++k)
            if (sub[k] < 0 || sub[k] >= p->g.ss) return xct_fail(XCT_E_INVALID, "subset order entry out of range");
    return XCT_OK;
}

int xct_osem_run_device(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it, void *stream)
{
    XCT_RANGE("xct_osem_run_device");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_osem_run_device: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    return osem_loop_maybe_traced(p, dN, d_sino, d_img, sub ? sub : p->sub_default.data(), it, st,
                                  "xct_osem_run_device");
}

// A blocking host-buffer call on a batch of two or more independent slices: the batch's two
// halves each carry their own copies and kernels (run_half(first, count, stream), using the
// plan's work buffers from slice `first` on) on their own stream -- the plan's stream and
// s_aux -- enqueued so that one half's uploads and downloads overlap the other half's kernels.
// Copies from pageable host memory return only when done, so the host order is: upload A,
// kernels A, upload B (while A runs), kernels B, download A (while B runs), download B.
// ev0..ev1 spans the first kernel to the later half's last (ev_fork, after its first use for
// the fork, marks the end of A).
static int host_run_split(xct_plan *p, int dN, int d0, const float *const *sino_host, float *const *img_host,
                          bool upload_img, const std::function<int(int, int, cudaStream_t)> &run_half)
{
    const size_t nimg = (size_t)p->g.nx * p->g.ny, nprj = (size_t)p->g.px * p->g.pa;
    const int first[2] = {0, d0}, count[2] = {d0, dN - d0};
    cudaStream_t sts[2] = {p->stream, p->s_aux};
    XCT_CUDA_TRY(cudaEventRecord(p->ev_fork, sts[0]));
    XCT_CUDA_TRY(cudaStreamWaitEvent(sts[1], p->ev_fork, 0));
    auto upload_and_run = [&](int h) -> int {
        cudaStream_t st = sts[h];
        cudaError_t e;
        for (int i = first[h]; i < first[h] + count[h]; ++i) {
            if ((e = cudaMemcpyAsync(p->d_sino + i * nprj, sino_host[i], sizeof(float) * nprj, cudaMemcpyHostToDevice,
                                     st)) != cudaSuccess)
                return xct_cuda_fail(e, "upload sinogram");
            if (upload_img && (e = cudaMemcpyAsync(p->d_img + i * nimg, img_host[i], sizeof(float) * nimg,
                                                   cudaMemcpyHostToDevice, st)) != cudaSuccess)
                return xct_cuda_fail(e, "upload image");
        }
        if (h == 0 && (e = cudaEventRecord(p->ev0, st)) != cudaSuccess) return xct_cuda_fail(e, "event");
        const int r = run_half(first[h], count[h], st);
        if (r) return r;
        if (h == 0) e = cudaEventRecord(p->ev_fork, st);
        else if ((e = cudaStreamWaitEvent(st, p->ev_fork, 0)) == cudaSuccess) e = cudaEventRecord(p->ev1, st);
        return e == cudaSuccess ? XCT_OK : xct_cuda_fail(e, "event");
    };
    auto download = [&](int h) -> int {
        for (int i = first[h]; i < first[h] + count[h]; ++i) {
            const cudaError_t e = cudaMemcpyAsync(img_host[i], p->d_img + i * nimg, sizeof(float) * nimg,
                                                  cudaMemcpyDeviceToHost, sts[h]);
            if (e != cudaSuccess) return xct_cuda_fail(e, "download image");
        }
        return XCT_OK;
    };
    int rc = upload_and_run(0);
    if (rc == XCT_OK) rc = upload_and_run(1);
    if (rc == XCT_OK) rc = download(0);
    if (rc == XCT_OK) rc = download(1);
    // join in every case, so that nothing of this call is still queued when it returns
    const cudaError_t e1 = cudaEventRecord(p->ev_join, sts[1]);
    const cudaError_t e2 = e1 == cudaSuccess ? cudaStreamWaitEvent(sts[0], p->ev_join, 0) : e1;
    const cudaError_t e3 = cudaStreamSynchronize(sts[0]);
    if (rc) return rc;
    if (e2 != cudaSuccess) return xct_cuda_fail(e2, "join");
    if (e3 != cudaSuccess) return xct_cuda_fail(e3, "synchronize");
    XCT_CUDA_TRY(cudaEventElapsedTime(&p->last_ms, p->ev0, p->ev1));
    return XCT_OK;
}

// xct_osem_run's halves: the sinogram correction (if any) and the subset/iteration loop on
// the plan's buffers from slice `first` on.
static int osem_host_split(xct_plan *p, int dN, const float *const *sino_host, float *const *img_host,
                           const int *sub, int it)
{
    const KGeom &g = p->kg;
    const size_t nimg = (size_t)g.nx * g.ny, nprj = (size_t)g.px * g.pa;
    return host_run_split(p, dN, xct_osem_split(p, dN), sino_host, img_host, true,
                          [&](int first, int count, cudaStream_t st) {
        const float *meas = p->d_sino + first * nprj;
        if (p->g.correction_mode > 0) {
            const int r = launch_sino_correction(g, meas, p->d_corr + first * nprj, p->d_corr_ang, p->d_corr_bin,
                                                 p->g.correction_mode, count, st);
            if (r) return r;
            meas = p->d_corr + first * nprj;
        }
        double *acc = p->d_acc ? p->d_acc + (size_t)first * p->acc_rows * g.px : nullptr;
        return osem_loop_range(p, count, meas, p->d_img + first * nimg, p->d_ratio + first * nprj, acc, sub, it, st);
    });
}

int xct_osem_run(xct_plan *p, int dN, const float *const *sino_host, float *const *img_host, const int *sub, int it)
{
    XCT_RANGE("xct_osem_run");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!sino_host || !img_host) return xct_fail(XCT_E_INVALID, "xct_osem_run: null host array");
    for (int i = 0; i < dN; ++i)
        if (!sino_host[i] || !img_host[i]) return xct_fail(XCT_E_INVALID, "xct_osem_run: null slice pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    // two or more slices: halves with their own copies on two streams (a traced call keeps
    // the one-stream order below, whose launches the trace times)
    const bool traced = trace_file() != nullptr && p->g.correction_mode == 0;
    if (dN >= 2 && it > 0 && !traced)
        return osem_host_split(p, dN, sino_host, img_host, sub ? sub : p->sub_default.data(), it);
    const size_t nimg = (size_t)p->g.nx * p->g.ny, nprj = (size_t)p->g.px * p->g.pa;
    cudaStream_t st = p->stream;
    // host -> device (OSEM_thread, GPU.cpp:440-445)
    for (int i = 0; i < dN; ++i) {
        XCT_CUDA_TRY(cudaMemcpyAsync(p->d_sino + i * nprj, sino_host[i], sizeof(float) * nprj,
                                     cudaMemcpyHostToDevice, st));
        XCT_CUDA_TRY(
            cudaMemcpyAsync(p->d_img + i * nimg, img_host[i], sizeof(float) * nimg, cudaMemcpyHostToDevice, st));
    }
    XCT_CUDA_TRY(cudaEventRecord(p->ev0, st));
    rc = osem_loop_maybe_traced(p, dN, p->d_sino, p->d_img, sub ? sub : p->sub_default.data(), it, st, "xct_osem_run");
    if (rc) return rc;
    XCT_CUDA_TRY(cudaEventRecord(p->ev1, st));
    // device -> host (GPU.cpp:460-463)
    for (int i = 0; i < dN; ++i)
        XCT_CUDA_TRY(
            cudaMemcpyAsync(img_host[i], p->d_img + i * nimg, sizeof(float) * nimg, cudaMemcpyDeviceToHost, st));
    XCT_CUDA_TRY(cudaStreamSynchronize(st));
    XCT_CUDA_TRY(cudaEventElapsedTime(&p->last_ms, p->ev0, p->ev1));
    return XCT_OK;
}

int xct_osem1(xct_plan *p, int dN, int sub, const float *d_img, const float *d_sino, float *d_ratio, void *stream)
{
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_img || !d_sino || !d_ratio) return xct_fail(XCT_E_INVALID, "xct_osem1: null device pointer");
    if (sub < 0 || sub >= p->g.ss) return xct_fail(XCT_E_INVALID, "xct_osem1: subset out of range");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    const int rows = subset_rows(p, sub);
    if (p->g.kernels == XCT_KERNELS_TILED)
        return launch_fwd_tiled(p->kg, p->d_trig, d_img, d_sino, d_ratio, p->d_acc, dN, sub, p->g.ss, rows, st);
    return launch_fwd_plain(p->kg, p->d_trig, d_img, d_sino, d_ratio, dN, sub, p->g.ss, rows, st);
}

int xct_osem2(xct_plan *p, int dN, int sub, float *d_img, const float *d_ratio, void *stream)
{
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_img || !d_ratio) return xct_fail(XCT_E_INVALID, "xct_osem2: null device pointer");
    if (sub < 0 || sub >= p->g.ss) return xct_fail(XCT_E_INVALID, "xct_osem2: subset out of range");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    if (p->g.kernels == XCT_KERNELS_TILED) return launch_bp_update_tiled(p->kg, p->d_trig, d_img, d_ratio, dN, sub, st);
    return launch_bp_update_plain(p->kg, p->d_trig, d_img, d_ratio, dN, sub, st);
}

int xct_fwd(xct_plan *p, int dN, const float *d_img, float *d_sino, void *stream)
{
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_img || !d_sino) return xct_fail(XCT_E_INVALID, "xct_fwd: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    if (p->g.kernels != XCT_KERNELS_TILED)
        return launch_fwd_plain(p->kg, p->d_trig, d_img, nullptr, d_sino, dN, 0, 1, p->g.pa, st);
    // all angles, in chunks of the accumulator's row capacity
    for (int r0 = 0; r0 < p->g.pa; r0 += p->acc_rows) {
        const int n = std::min(p->acc_rows, p->g.pa - r0);
        int rc = launch_fwd_tiled(p->kg, p->d_trig, d_img, nullptr, d_sino, p->d_acc, dN, r0, 1, n, st);
        if (rc) return rc;
    }
    return XCT_OK;
}

int xct_bp_ref(xct_plan *p, int dN, const float *d_sino, float *d_img, void *stream)
{
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_img || !d_sino) return xct_fail(XCT_E_INVALID, "xct_bp_ref: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    return launch_bp_ref_plain(p->kg, p->d_trig, d_sino, d_img, dN, 0, 1, st);
}

int xct_adj(xct_plan *p, int dN, const float *d_sino, float *d_img, void *stream)
{
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_img || !d_sino) return xct_fail(XCT_E_INVALID, "xct_adj: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return launch_adj_tiled(p->kg, p->d_trig, d_sino, d_img, dN, (cudaStream_t)stream);
}

// OS-EM of the plan's tiled or plain kernels with a CUDA event pair around every launch
// (forward, finalize, backprojection per subset); synchronous.  per_launch receives each
// launch's milliseconds in launch order (the plain kernels' finalize slot stays 0).
static int osem_loop_timed(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *so, int it,
                           cudaStream_t st, float *ms, long long *launches, std::vector<float> *per_launch)
{
    const bool tiled = p->g.kernels == XCT_KERNELS_TILED;
    const int nk = 3;
    const int nlaunch = it * p->g.ss * nk;
    std::vector<cudaEvent_t> ev(2 * (size_t)nlaunch + 2, nullptr);
    for (auto &e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) {
            for (auto &f : ev)
                if (f) cudaEventDestroy(f);
            return xct_fail(XCT_E_CUDA, "osem timing: event create");
        }
    int rc = XCT_OK, q = 0;
    cudaEventRecord(ev[ev.size() - 2], st);
    for (int i = 0; i < it && rc == 0; ++i)
        for (int k = 0; k < p->g.ss && rc == 0; ++k) {
            const int s = so[k];
            const int rows = subset_rows(p, s);
            for (int kind = 0; kind < nk && rc == 0; ++kind) {
                cudaEventRecord(ev[2 * q], st);
                if (tiled) {
                    if (kind == 0) rc = launch_fwd_tiled_main(p->kg, p->d_trig, d_img, p->d_acc, dN, s, p->g.ss, rows, st);
                    else if (kind == 1)
                        rc = launch_fwd_finalize(p->kg, d_sino, p->d_ratio, p->d_acc, dN, s, p->g.ss, rows, st);
                    else rc = launch_bp_update_tiled(p->kg, p->d_trig, d_img, p->d_ratio, dN, s, st);
                } else {
                    if (kind == 0)
                        rc = launch_fwd_plain(p->kg, p->d_trig, d_img, d_sino, p->d_ratio, dN, s, p->g.ss, rows, st);
                    else if (kind == 2) rc = launch_bp_update_plain(p->kg, p->d_trig, d_img, p->d_ratio, dN, s, st);
                }
                cudaEventRecord(ev[2 * q + 1], st);
                ++q;
            }
        }
    cudaEventRecord(ev[ev.size() - 1], st);
    cudaError_t e = cudaEventSynchronize(ev[ev.size() - 1]);
    if (rc == 0 && e != cudaSuccess) rc = xct_cuda_fail(e, "osem timing: sync");
    if (rc == 0) {
        for (int kk = 0; kk < 4; ++kk) {
            ms[kk] = 0.0f;
            launches[kk] = 0;
        }
        if (per_launch) per_launch->assign(q, 0.0f);
        for (int j = 0; j < q; ++j) {
            float t = 0.0f;
            cudaEventElapsedTime(&t, ev[2 * j], ev[2 * j + 1]);
            ms[j % nk] += t;
            if (per_launch) (*per_launch)[j] = t;
            if (tiled || j % nk != 1) launches[j % nk] += 1;
        }
        cudaEventElapsedTime(&ms[3], ev[ev.size() - 2], ev[ev.size() - 1]);
        launches[3] = launches[0] + launches[1] + launches[2];
    }
    for (auto &f : ev) cudaEventDestroy(f);
    return rc;
}

int xct_osem_profile(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it, void *stream,
                     float *ms, long long *launches)
{
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!d_sino || !d_img || !ms || !launches) return xct_fail(XCT_E_INVALID, "xct_osem_profile: null argument");
    if (p->g.correction_mode > 0)
        return xct_fail(XCT_E_UNSUPPORTED, "xct_osem_profile: plans with a sinogram correction are not profiled");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return osem_loop_timed(p, dN, d_sino, d_img, sub ? sub : p->sub_default.data(), it, (cudaStream_t)stream, ms,
                           launches, nullptr);
}

// ---------------------------------------------------------------------------- FBP
// FBP_execution (GPU.cpp:665-819) on dN slices already on the device: the plan's sinogram
// correction when it has one (GPU.cpp:711-723, applied into the correction buffer), the
// ramp filter into the ratio buffer, backProjectionFBP into d_img.  The ratio buffer is
// cleared afterwards: OS-EM relies on the rows it never writes being 0.
// FBP of dN slices; the plan's work buffers (corrected sinograms, filtered sinograms, minima)
// are used from slice `first` on, so the halves of a batch can run side by side.
static int fbp_device(xct_plan *p, int dN, int zp, const float *d_sino, float *d_img, bool with_min,
                      const float **meas_out, cudaStream_t st, int first = 0)
{
    const KGeom &g = p->kg;
    const size_t nprj = (size_t)g.pa * g.px;
    float *fprj = p->d_ratio + first * nprj;
    const float *meas = d_sino;
    if (p->g.correction_mode > 0) {
        int rc = launch_sino_correction(g, d_sino, p->d_corr + first * nprj, p->d_corr_ang, p->d_corr_bin,
                                        p->g.correction_mode, dN, st);
        if (rc) return rc;
        meas = p->d_corr + first * nprj;
    }
    int rc = launch_fbp_filter(g, meas, fprj, dN, zp, st);
    if (rc) return rc;
    rc = launch_fbp_bp(g, p->d_trig, fprj, d_img, dN, with_min ? p->d_min_keys + first : nullptr, st);
    if (rc) return rc;
    XCT_CUDA_TRY(cudaMemsetAsync(fprj, 0, sizeof(float) * dN * nprj, st));
    if (meas_out) *meas_out = meas;
    return XCT_OK;
}

int xct_fbp_filter(xct_plan *p, int dN, int zp, const float *d_sino, float *d_fprj, void *stream)
{
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_sino || !d_fprj) return xct_fail(XCT_E_INVALID, "xct_fbp_filter: null device pointer");
    if ((rc = xct_fbp_check_zp(p->g.px, zp))) return rc;
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return launch_fbp_filter(p->kg, d_sino, d_fprj, dN, zp, (cudaStream_t)stream);
}

int xct_fbp_backproject(xct_plan *p, int dN, const float *d_fprj, float *d_img, void *stream)
{
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_fprj || !d_img) return xct_fail(XCT_E_INVALID, "xct_fbp_backproject: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return launch_fbp_bp(p->kg, p->d_trig, d_fprj, d_img, dN, nullptr, (cudaStream_t)stream);
}

int xct_fbp_run_device(xct_plan *p, int dN, int zp, const float *d_sino, float *d_img, void *stream)
{
    XCT_RANGE("xct_fbp_run_device");
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if (!d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_fbp_run_device: null device pointer");
    if ((rc = xct_fbp_check_zp(p->g.px, zp))) return rc;
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return fbp_device(p, dN, zp, d_sino, d_img, false, nullptr, (cudaStream_t)stream);
}

static int cs_loop(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it, float lambda,
                   cudaStream_t st, bool correct = true);

// hybrid_thread (GPU.cpp:1458-1600): FBP_execution with the sinogram correction, the
// base-up of FBPcorrection = 1 (slice minimum, then baseUp with baseupOrder), then
// OSEM_execution -- or FISTA_OSEM_execution when CSitBool is set (:1569-1574) -- on the
// corrected sinogram without correcting it again.
static int hybrid_device(xct_plan *p, int dN, int zp, int order, const float *d_sino, float *d_img, const int *sub,
                         int it, cudaStream_t st, bool cs = false, float lambda = 0.0f)
{
    const float *meas = nullptr;
    int rc = fbp_device(p, dN, zp, d_sino, d_img, true, &meas, st);
    if (rc) return rc;
    rc = launch_base_up(p->kg, d_img, dN, order, p->d_min_keys, p->ctx->sm_count, st);
    if (rc) return rc;
    if (cs) return cs_loop(p, dN, meas, d_img, sub ? sub : p->sub_default.data(), it, lambda, st, false);
    return osem_loop(p, dN, meas, d_img, sub ? sub : p->sub_default.data(), it, st, false);
}

// One half of a host-buffer hybrid batch: FBP, base-up and OS-EM of `count` slices on the
// plan's buffers from slice `first` on, on one stream (no inner split: the halves already
// run side by side).
static int hybrid_half(xct_plan *p, int first, int count, int zp, int order, const int *sub, int it,
                       cudaStream_t st)
{
    const KGeom &g = p->kg;
    const size_t nimg = (size_t)g.nx * g.ny, nprj = (size_t)g.px * g.pa;
    float *img = p->d_img + first * nimg;
    const float *meas = nullptr;
    int rc = fbp_device(p, count, zp, p->d_sino + first * nprj, img, true, &meas, st, first);
    if (rc) return rc;
    rc = launch_base_up(g, img, count, order, p->d_min_keys + first, p->ctx->sm_count, st);
    if (rc) return rc;
    double *acc = p->d_acc ? p->d_acc + (size_t)first * p->acc_rows * g.px : nullptr;
    return osem_loop_range(p, count, meas, img, p->d_ratio + first * nprj, acc, sub ? sub : p->sub_default.data(), it,
                           st);
}

int xct_hybrid_run_device(xct_plan *p, int dN, int zp, int baseup_order, const float *d_sino, float *d_img,
                          const int *sub, int it, void *stream)
{
    XCT_RANGE("xct_hybrid_run_device");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_hybrid_run_device: null device pointer");
    if (baseup_order < 0 || baseup_order > 64) return xct_fail(XCT_E_INVALID, "xct_hybrid_run_device: order 0..64");
    if ((rc = xct_fbp_check_zp(p->g.px, zp))) return rc;
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return hybrid_device(p, dN, zp, baseup_order, d_sino, d_img, sub, it, (cudaStream_t)stream);
}

// Host-buffer forms (FBP_thread GPU.cpp:822-893, hybrid_thread): copies in, run, copies out.
static int host_run(xct_plan *p, int dN, const float *const *sino_host, float *const *img_host, bool upload_img,
                    const std::function<int(cudaStream_t)> &run)
{
    if (!sino_host || !img_host) return xct_fail(XCT_E_INVALID, "null host array");
    for (int i = 0; i < dN; ++i)
        if (!sino_host[i] || !img_host[i]) return xct_fail(XCT_E_INVALID, "null slice pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    const size_t nimg = (size_t)p->g.nx * p->g.ny, nprj = (size_t)p->g.px * p->g.pa;
    cudaStream_t st = p->stream;
    for (int i = 0; i < dN; ++i) {
        XCT_CUDA_TRY(cudaMemcpyAsync(p->d_sino + i * nprj, sino_host[i], sizeof(float) * nprj,
                                     cudaMemcpyHostToDevice, st));
        if (upload_img)
            XCT_CUDA_TRY(cudaMemcpyAsync(p->d_img + i * nimg, img_host[i], sizeof(float) * nimg,
                                         cudaMemcpyHostToDevice, st));
    }
    XCT_CUDA_TRY(cudaEventRecord(p->ev0, st));
    int rc = run(st);
    if (rc) return rc;
    XCT_CUDA_TRY(cudaEventRecord(p->ev1, st));
    for (int i = 0; i < dN; ++i)
        XCT_CUDA_TRY(
            cudaMemcpyAsync(img_host[i], p->d_img + i * nimg, sizeof(float) * nimg, cudaMemcpyDeviceToHost, st));
    XCT_CUDA_TRY(cudaStreamSynchronize(st));
    XCT_CUDA_TRY(cudaEventElapsedTime(&p->last_ms, p->ev0, p->ev1));
    return XCT_OK;
}

int xct_fbp_run(xct_plan *p, int dN, int zp, const float *const *sino_host, float *const *img_host)
{
    XCT_RANGE("xct_fbp_run");
    int rc = check_run(p, dN, nullptr, 0);
    if (rc) return rc;
    if ((rc = xct_fbp_check_zp(p->g.px, zp))) return rc;
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    if (dN >= 2) {  // halves with their own copies on two streams
        const size_t nimg = (size_t)p->g.nx * p->g.ny, nprj = (size_t)p->g.px * p->g.pa;
        return host_run_split(p, dN, (dN + 1) / 2, sino_host, img_host, false,
                              [&](int first, int count, cudaStream_t st) {
            return fbp_device(p, count, zp, p->d_sino + first * nprj, p->d_img + first * nimg, false, nullptr, st,
                              first);
        });
    }
    return host_run(p, dN, sino_host, img_host, false,
                    [&](cudaStream_t st) { return fbp_device(p, dN, zp, p->d_sino, p->d_img, false, nullptr, st); });
}

int xct_hybrid_run(xct_plan *p, int dN, int zp, int baseup_order, const float *const *sino_host,
                   float *const *img_host, const int *sub, int it)
{
    XCT_RANGE("xct_hybrid_run");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (baseup_order < 0 || baseup_order > 64) return xct_fail(XCT_E_INVALID, "xct_hybrid_run: order 0..64");
    if ((rc = xct_fbp_check_zp(p->g.px, zp))) return rc;
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    if (dN >= 2)  // halves with their own copies on two streams
        return host_run_split(p, dN, (dN + 1) / 2, sino_host, img_host, false,
                              [&](int first, int count, cudaStream_t st) {
            return hybrid_half(p, first, count, zp, baseup_order, sub, it, st);
        });
    return host_run(p, dN, sino_host, img_host, false, [&](cudaStream_t st) {
        return hybrid_device(p, dN, zp, baseup_order, p->d_sino, p->d_img, sub, it, st);
    });
}

// The hybrid with CSitBool: FBP, base-up, then the compressed-sensing OS-EM.
int xct_hybrid_cs_run_device(xct_plan *p, int dN, int zp, int baseup_order, const float *d_sino, float *d_img,
                             const int *sub, int it, float cs_lambda, void *stream)
{
    XCT_RANGE("xct_hybrid_cs_run_device");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_hybrid_cs_run_device: null device pointer");
    if (baseup_order < 0 || baseup_order > 64)
        return xct_fail(XCT_E_INVALID, "xct_hybrid_cs_run_device: order 0..64");
    if (!(cs_lambda >= 0.0f && cs_lambda < 1.0e30f))
        return xct_fail(XCT_E_INVALID, "xct_hybrid_cs_run_device: cs_lambda must be finite and >= 0");
    if ((rc = xct_fbp_check_zp(p->g.px, zp))) return rc;
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return hybrid_device(p, dN, zp, baseup_order, d_sino, d_img, sub, it, (cudaStream_t)stream, true,
                         xct_cs_kernel_lambda(cs_lambda));
}

int xct_hybrid_cs_run(xct_plan *p, int dN, int zp, int baseup_order, const float *const *sino_host,
                      float *const *img_host, const int *sub, int it, float cs_lambda)
{
    XCT_RANGE("xct_hybrid_cs_run");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (baseup_order < 0 || baseup_order > 64) return xct_fail(XCT_E_INVALID, "xct_hybrid_cs_run: order 0..64");
    if (!(cs_lambda >= 0.0f && cs_lambda < 1.0e30f))
        return xct_fail(XCT_E_INVALID, "xct_hybrid_cs_run: cs_lambda must be finite and >= 0");
    if ((rc = xct_fbp_check_zp(p->g.px, zp))) return rc;
    const float lam = xct_cs_kernel_lambda(cs_lambda);
    return host_run(p, dN, sino_host, img_host, false, [&](cudaStream_t st) {
        return hybrid_device(p, dN, zp, baseup_order, p->d_sino, p->d_img, sub, it, st, true, lam);
    });
}

// --------------------------------------------------------------- streamed full volume
// OS-EM of n slices held in host memory, max_batch slices per device batch, two staging sets
// on the device: batch b computes on the plan stream while batch b+1's sinograms and initial
// images go up on an upload stream and batch b-1's images come down on a download stream;
// events order each staging set's reuse.  The volume never needs to fit in HBM.
int xct_osem_run_volume(xct_plan *p, int n, const float *const *sino_host, float *const *img_host, const int *sub,
                        int it)
{
    XCT_RANGE("xct_osem_run_volume");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, 1, sub, it);
    if (rc) return rc;
    if (n <= 0 || !sino_host || !img_host) return xct_fail(XCT_E_INVALID, "xct_osem_run_volume: bad arguments");
    for (int i = 0; i < n; ++i)
        if (!sino_host[i] || !img_host[i]) return xct_fail(XCT_E_INVALID, "xct_osem_run_volume: null slice pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    const size_t nimg = (size_t)p->g.nx * p->g.ny, nprj = (size_t)p->g.px * p->g.pa, nb = (size_t)p->g.max_batch;
    if (!p->d_sino2) {
        XCT_CUDA_TRY(cudaMalloc(&p->d_sino2, sizeof(float) * nb * nprj));
        cudaError_t e = cudaMalloc(&p->d_img2, sizeof(float) * nb * nimg);
        if (e != cudaSuccess) {
            cudaFree(p->d_sino2);
            p->d_sino2 = nullptr;
            return xct_cuda_fail(e, "cudaMalloc volume staging");
        }
        XCT_CUDA_TRY(cudaStreamCreateWithFlags(&p->s_h2d, cudaStreamNonBlocking));
        XCT_CUDA_TRY(cudaStreamCreateWithFlags(&p->s_d2h, cudaStreamNonBlocking));
    }
    float *dsino[2] = {p->d_sino, p->d_sino2}, *dimg[2] = {p->d_img, p->d_img2};
    const int *so = sub ? sub : p->sub_default.data();
    cudaEvent_t up[2], done[2], down[2];
    for (int k = 0; k < 2; ++k) {
        XCT_CUDA_TRY(cudaEventCreateWithFlags(&up[k], cudaEventDisableTiming));
        XCT_CUDA_TRY(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
        XCT_CUDA_TRY(cudaEventCreateWithFlags(&down[k], cudaEventDisableTiming));
    }
    auto cleanup = [&]() {
        for (int k = 0; k < 2; ++k) {
            cudaEventDestroy(up[k]);
            cudaEventDestroy(done[k]);
            cudaEventDestroy(down[k]);
        }
    };
    auto upload = [&](int b) -> int {
        const int s = b & 1, z0 = b * p->g.max_batch, dn = std::min(p->g.max_batch, n - z0);
        if (b >= 2) XCT_CUDA_TRY(cudaStreamWaitEvent(p->s_h2d, down[s], 0));  // set s is free again
        for (int i = 0; i < dn; ++i) {
            XCT_CUDA_TRY(cudaMemcpyAsync(dsino[s] + i * nprj, sino_host[z0 + i], sizeof(float) * nprj,
                                         cudaMemcpyHostToDevice, p->s_h2d));
            XCT_CUDA_TRY(cudaMemcpyAsync(dimg[s] + i * nimg, img_host[z0 + i], sizeof(float) * nimg,
                                         cudaMemcpyHostToDevice, p->s_h2d));
        }
        XCT_CUDA_TRY(cudaEventRecord(up[s], p->s_h2d));
        return XCT_OK;
    };
    const int nbatch = (int)((n + nb - 1) / nb);
    XCT_CUDA_TRY(cudaEventRecord(p->ev0, p->stream));
    rc = upload(0);
    for (int b = 0; b < nbatch && rc == XCT_OK; ++b) {
        const int s = b & 1, z0 = b * p->g.max_batch, dn = std::min(p->g.max_batch, n - z0);
        if (b + 1 < nbatch && (rc = upload(b + 1))) break;
        cudaError_t e = cudaStreamWaitEvent(p->stream, up[s], 0);
        if (e != cudaSuccess) {
            rc = xct_cuda_fail(e, "volume wait");
            break;
        }
        if ((rc = osem_loop(p, dn, dsino[s], dimg[s], so, it, p->stream))) break;
        cudaEventRecord(done[s], p->stream);
        cudaStreamWaitEvent(p->s_d2h, done[s], 0);
        for (int i = 0; i < dn && rc == XCT_OK; ++i) {
            e = cudaMemcpyAsync(img_host[z0 + i], dimg[s] + i * nimg, sizeof(float) * nimg, cudaMemcpyDeviceToHost,
                                p->s_d2h);
            if (e != cudaSuccess) rc = xct_cuda_fail(e, "volume download");
        }
        cudaEventRecord(down[s], p->s_d2h);
    }
    cudaError_t e1 = cudaStreamSynchronize(p->s_d2h), e2 = cudaStreamSynchronize(p->stream),
                e3 = cudaStreamSynchronize(p->s_h2d);
    if (rc == XCT_OK && (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess))
        rc = xct_cuda_fail(e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3), "xct_osem_run_volume: sync");
    if (rc == XCT_OK) {
        cudaEventRecord(p->ev1, p->stream);
        cudaEventSynchronize(p->ev1);
        cudaEventElapsedTime(&p->last_ms, p->ev0, p->ev1);
    }
    cleanup();
    return rc;
}

// ------------------------------------------------------ compressed-sensing OS-EM (FISTA)
// FISTA_OSEM_execution (GPU.cpp:243-405) on dN slices on the device.  Per subset: OSEM1 and
// OSEM2 (in place: the image becomes v, the OS-EM update), then FISTA3D(w, v, beta) writes x'
// (then copied into the image), w' and beta' (in place).  The first cycle runs ISTA3D on the
// image as it was BEFORE that subset's OS-EM step -- the reference passes reconst_img, not the
// updated dest image, to ISTA3D (:335-336, :388) -- so its OS-EM step is dead work and is
// skipped here (the ratio rows it would write are rewritten before every later read).
static int cs_loop(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it, float lambda,
                   cudaStream_t st, bool correct)
{
    const KGeom &g = p->kg;
    const size_t nimg = (size_t)g.nx * g.ny, nb = (size_t)p->g.max_batch;
    if (!p->d_cs) {
        cudaError_t e = cudaMalloc(&p->d_cs, sizeof(float) * 3 * nb * nimg);
        if (e != cudaSuccess) {
            p->d_cs = nullptr;
            return xct_cuda_fail(e, "cudaMalloc compressed-sensing buffers");
        }
    }
    float *w = p->d_cs, *beta = p->d_cs + nb * nimg, *xn = p->d_cs + 2 * nb * nimg;
    const size_t bytes = sizeof(float) * dN * nimg;
    const float *meas = d_sino;
    if (correct && p->g.correction_mode > 0) {
        int rc = launch_sino_correction(g, d_sino, p->d_corr, p->d_corr_ang, p->d_corr_bin, p->g.correction_mode, dN,
                                        st);
        if (rc) return rc;
        meas = p->d_corr;
    }
    XCT_CUDA_TRY(cudaMemcpyAsync(w, d_img, bytes, cudaMemcpyDeviceToDevice, st));  // w = x (:344)
    XCT_CUDA_TRY(cudaMemsetAsync(beta, 0, bytes, st));                             // beta = 0 (:342)
    bool first = true;
    for (int i = 0; i < it; ++i)
        for (int k = 0; k < p->g.ss; ++k) {
            const int s = sub[k];
            int rc;
            if (first) {
                rc = launch_ista3d(d_img, xn, g.nx, g.ny, dN, lambda, p->ctx->sm_count, st);
                first = false;
            } else {
                // the OS-EM step of the two halves on two streams; the proximal step after the
                // join couples neighbouring slices
                rc = dN >= 2 ? subset_step_split(p, dN, meas, d_img, s, st)
                             : subset_step(p, dN, meas, d_img, p->d_ratio, p->d_acc, s, st);
                if (!rc) rc = launch_fista3d(w, w, d_img, beta, xn, g.nx, g.ny, dN, lambda, p->ctx->sm_count, st);
            }
            if (rc) return rc;
            XCT_CUDA_TRY(cudaMemcpyAsync(d_img, xn, bytes, cudaMemcpyDeviceToDevice, st));
        }
    return XCT_OK;
}

int xct_cs_osem_run_device(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it,
                           float cs_lambda, void *stream)
{
    XCT_RANGE("xct_cs_osem_run_device");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_cs_osem_run_device: null device pointer");
    if (!(cs_lambda >= 0.0f && cs_lambda < 1.0e30f))
        return xct_fail(XCT_E_INVALID, "xct_cs_osem_run_device: cs_lambda must be finite and >= 0");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return cs_loop(p, dN, d_sino, d_img, sub ? sub : p->sub_default.data(), it, xct_cs_kernel_lambda(cs_lambda),
                   (cudaStream_t)stream);
}

int xct_cs_osem_run(xct_plan *p, int dN, const float *const *sino_host, float *const *img_host, const int *sub, int it,
                    float cs_lambda)
{
    XCT_RANGE("xct_cs_osem_run");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!(cs_lambda >= 0.0f && cs_lambda < 1.0e30f))
        return xct_fail(XCT_E_INVALID, "xct_cs_osem_run: cs_lambda must be finite and >= 0");
    const float lam = xct_cs_kernel_lambda(cs_lambda);
    return host_run(p, dN, sino_host, img_host, true, [&](cudaStream_t st) {
        return cs_loop(p, dN, p->d_sino, p->d_img, sub ? sub : p->sub_default.data(), it, lam, st);
    });
}

// ------------------------------------------------------------ rotation-centre search
static int check_shifts(int n, float start, float step)
{
    if (n <= 0) return xct_fail(XCT_E_INVALID, "rotation-centre search: n must be > 0");
    if (!(fabsf(start) < 1.0e6f) || !(fabsf(step) < 1.0e6f) || !(fabsf(start) + fabsf(step) * (float)n < 1.0e6f))
        return xct_fail(XCT_E_INVALID, "rotation-centre search: shifts must be finite and below 1e6 bins");
    return XCT_OK;
}

int xct_rot_center_shift(xct_plan *p, int n, float shift_start, float shift_step, const float *d_sino,
                         float *d_shifted, void *stream)
{
    if (!p) return xct_fail(XCT_E_INVALID, "plan is null");
    int rc = check_shifts(n, shift_start, shift_step);
    if (rc) return rc;
    if (!d_sino || !d_shifted) return xct_fail(XCT_E_INVALID, "xct_rot_center_shift: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    return launch_rot_shift(d_sino, d_shifted, p->g.px, p->g.pa, n, 0, shift_start, shift_step, p->ctx->sm_count,
                            (cudaStream_t)stream);
}

// Focus indices of images [off, off + c) of a shift sequence into d_findex (device).
static int focus_chunk(xct_plan *p, const float *d_imgs, int off, int c, float start, float step, float ang_ini,
                       float ang_fin, float *d_findex, cudaStream_t st)
{
    std::vector<float> prm(16 * (size_t)c);
    for (int i = 0; i < c; ++i)
        xct_mask_params(p->g.nx, p->g.ny, xct_shift_value(start, step, off + i), ang_ini, ang_fin, &prm[16 * i]);
    XCT_CUDA_TRY(cudaMemcpyAsync(p->d_rc_prm, prm.data(), sizeof(float) * prm.size(), cudaMemcpyHostToDevice, st));
    return launch_focus_index(d_imgs, p->g.nx, p->g.ny, c, p->d_rc_prm, p->d_red, d_findex, st);
}

int xct_focus_index(xct_plan *p, int n, int shift_offset, float shift_start, float shift_step, float ang_ini_deg,
                    float ang_fin_deg, const float *d_imgs, float *d_findex, void *stream)
{
    if (!p) return xct_fail(XCT_E_INVALID, "plan is null");
    int rc = check_shifts(n + std::max(shift_offset, 0), shift_start, shift_step);
    if (rc) return rc;
    if (shift_offset < 0) return xct_fail(XCT_E_INVALID, "xct_focus_index: shift_offset must be >= 0");
    if (!d_imgs || !d_findex) return xct_fail(XCT_E_INVALID, "xct_focus_index: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nimg = (size_t)p->g.nx * p->g.ny;
    for (int off = 0; off < n; off += p->g.max_batch) {
        const int c = std::min(p->g.max_batch, n - off);
        rc = focus_chunk(p, d_imgs + off * nimg, shift_offset + off, c, shift_start, shift_step, ang_ini_deg,
                         ang_fin_deg, d_findex + off, st);
        if (rc) return rc;
    }
    return XCT_OK;
}

// rotationCenterSearch (rotationCenterSearch_ocl.cpp:419-540) from the resliced sinogram on:
// per batch of max_batch shifts, rotCenterShift, a uniform initial image (g_ini), one OS-EM
// iteration with the plan's subsets and sinogram correction (OSEM_execution(..., 1, true),
// :307), and the focus index; the estimate is the first shift with the smallest index
// (:505-513).
int xct_rot_center_search(xct_plan *p, int n, float shift_start, float shift_step, float ang_ini_deg,
                          float ang_fin_deg, float init_value, const float *d_sino, float *d_imgs, float *findex,
                          int *best, void *stream)
{
    XCT_RANGE("xct_rot_center_search");
    if (!p) return xct_fail(XCT_E_INVALID, "plan is null");
    int rc = check_shifts(n, shift_start, shift_step);
    if (rc) return rc;
    if (!d_sino || !d_imgs || !findex || !best) return xct_fail(XCT_E_INVALID, "xct_rot_center_search: null argument");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const size_t nimg = (size_t)p->g.nx * p->g.ny;
    for (int off = 0; off < n; off += p->g.max_batch) {
        const int c = std::min(p->g.max_batch, n - off);
        float *imgs = d_imgs + off * nimg;
        if ((rc = launch_rot_shift(d_sino, p->d_sino, p->g.px, p->g.pa, c, off, shift_start, shift_step,
                                   p->ctx->sm_count, st)))
            return rc;
        if ((rc = launch_fill(imgs, (long long)c * nimg, init_value, p->ctx->sm_count, st))) return rc;
        if ((rc = osem_loop(p, c, p->d_sino, imgs, p->sub_default.data(), 1, st))) return rc;
        if ((rc = focus_chunk(p, imgs, off, c, shift_start, shift_step, ang_ini_deg, ang_fin_deg, p->d_fi, st)))
            return rc;
        XCT_CUDA_TRY(cudaMemcpyAsync(findex + off, p->d_fi, sizeof(float) * c, cudaMemcpyDeviceToHost, st));
    }
    XCT_CUDA_TRY(cudaStreamSynchronize(st));
    float m = 3.402823466e38f;
    int b = 0;
    for (int i = 0; i < n; ++i)
        if (m > findex[i]) {
            m = findex[i];
            b = i;
        }
    *best = b;
    return XCT_OK;
}

// ------------------------------------------------- FISTA with compressed sensing (FISTA_ocl)
// powerIteration (GPU.cpp:2079-2188): per subset z, the estimate image (all 1 at first) is
// forward-projected on z's rows (powerIter1: the tiled projector with the half-texel shift of
// its coordinates), backprojected (powerIter2), its squared norm taken over the columns and
// rows the reference's work-groups visit (imageL2AbsX/Y) and the image normalised
// (powerIter3); L[z] is the last norm.  powerIter1 never sets the layer of its sampling
// coordinate (FISTA.cl:60), so by default every subset projects layer 0's estimate -- then
// only layer 0's iterate matters, and the other subsets are evaluated on its final state
// alone (the same values, ss times less work); XCT_PI_OWN_LAYER projects each subset's own.
int xct_fista_power_iteration(xct_plan *p, int trials, int work_group, int flags, float *L_out, void *stream)
{
    XCT_RANGE("xct_fista_power_iteration");
    if (!p) return xct_fail(XCT_E_INVALID, "xct_fista_power_iteration: plan is null");
    if (trials < 1 || trials > 100000) return xct_fail(XCT_E_INVALID, "xct_fista_power_iteration: trials must be >= 1");
    if (work_group < 1) return xct_fail(XCT_E_INVALID, "xct_fista_power_iteration: work_group must be >= 1");
    if (flags & ~XCT_PI_OWN_LAYER) return xct_fail(XCT_E_INVALID, "xct_fista_power_iteration: unknown flags");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const KGeom &g = p->kg;
    const int ss = g.ss, rows = g.pa / g.ss;
    const bool own = (flags & XCT_PI_OWN_LAYER) != 0;
    const int layers = own ? ss : 1;
    const size_t nimg = (size_t)g.nx * g.ny, nprj = (size_t)g.px * g.pa;
    if (p->pi_layers < layers) {
        cudaFree(p->d_pi);
        p->d_pi = nullptr;
        p->pi_layers = 0;
        cudaError_t e = cudaMalloc(&p->d_pi, sizeof(float) * ((size_t)(layers + 1) * nimg + nprj));
        if (e != cudaSuccess) {
            p->d_pi = nullptr;
            return xct_cuda_fail(e, "cudaMalloc power-iteration buffers");
        }
        p->pi_layers = layers;
    }
    if (!p->d_pi_l2) {
        cudaError_t e = cudaMalloc(&p->d_pi_l2, sizeof(double) * (size_t)std::max(ss, 1));
        if (e != cudaSuccess) {
            p->d_pi_l2 = nullptr;
            return xct_cuda_fail(e, "cudaMalloc power-iteration norms");
        }
    }
    float *img = p->d_pi, *cnd = p->d_pi + (size_t)p->pi_layers * nimg, *prj = cnd + nimg;
    int rc = launch_fill(img, (long long)layers * (long long)nimg, 1.0f, p->ctx->sm_count, st);  // GPU.cpp:2122
    if (rc) return rc;
    // powerIter1's coordinates: (X - px/2) c + (Y - D/2) s + nx/2 in integer halves, read by the
    // linear sampler at that minus 0.5 (no +0.5 as in OSEM1)
    KGeom gs = g;
    gs.hx = (float)(g.nx / 2) - 0.5f;
    gs.hy = (float)(g.ny / 2) - 0.5f;
    gs.cx = (float)(g.px / 2);
    gs.hd = (float)(g.depth / 2);
    gs.ms_chunk = 0;
    const int wg = std::min(work_group, g.nx);  // min(CL_DEVICE_MAX_WORK_GROUP_SIZE, g_ox)
    const int nxe = (g.nx / wg) * wg, nye = (g.ny / wg) * wg;
    const float scale = ((float)ss / (float)g.pa) / (float)g.depth;
    for (int t = 0; t < trials; ++t) {
        const bool last = t == trials - 1;
        for (int z = 0; z < ss; ++z) {
            if (!own && !last && z > 0) continue;  // only layer 0's iterate is ever projected
            float *im = img + (own ? (size_t)z * nimg : 0);
            if (p->g.kernels == XCT_KERNELS_TILED)
                rc = launch_fwd_tiled(gs, p->d_trig, im, nullptr, prj, p->d_acc, 1, z, ss, rows, st);
            else rc = launch_fwd_plain(gs, p->d_trig, im, nullptr, prj, 1, z, ss, rows, st);
            if (!rc) rc = launch_pi_bp(g, p->d_trig, prj, cnd, z, ss, rows, scale, st);
            if (!rc) rc = launch_pi_l2(cnd, g.nx, nxe, nye, p->d_pi_l2 + z, p->ctx->sm_count, st);
            // on the last trial every subset reads the same state; no further normalisation
            if (!rc && !last) rc = launch_pi_norm(cnd, im, g.nx, g.ny, p->d_pi_l2 + z, g.fetch, st);
            if (rc) return rc;
        }
    }
    std::vector<double> l2(ss);
    XCT_CUDA_TRY(cudaMemcpyAsync(l2.data(), p->d_pi_l2, sizeof(double) * ss, cudaMemcpyDeviceToHost, st));
    XCT_CUDA_TRY(cudaStreamSynchronize(st));
    p->lip.assign(ss, 0.0f);
    for (int z = 0; z < ss; ++z) p->lip[z] = (float)l2[z];
    if (L_out)
        for (int z = 0; z < ss; ++z) L_out[z] = p->lip[z];
    return XCT_OK;
}

int xct_fista_set_lipschitz(xct_plan *p, const float *L)
{
    if (!p || !L) return xct_fail(XCT_E_INVALID, "xct_fista_set_lipschitz: null argument");
    for (int z = 0; z < p->g.ss; ++z)
        if (!(L[z] > 0.0f && L[z] < 3.0e38f))
            return xct_fail(XCT_E_INVALID, "xct_fista_set_lipschitz: every L must be finite and > 0");
    p->lip.assign(L, L + p->g.ss);
    return XCT_OK;
}

// FISTA_execution (GPU.cpp:1755-1924) on dN slices on the device, with the reference's kernel
// argument bindings: the sinogram correction if the plan has one (the uncorrected sinogram
// stays in the residual image, :1812-1816); x = the plain backprojection of subset sub[0]
// (:1853-1858), w = x, beta = 0; per subset AART1 (the residual of x in the first cycle, of w
// after), the gradient step v (FISTAbackProjection, or with XCT_FISTA_ADJOINT the exact
// adjoint), then ISTA3D(v) into dest in the first cycle and FISTA3D(x, v, beta) after --
// whose x_{t+1} the reference writes into the beta image, where beta_{t+1} overwrites it
// (:1867-1868), so dest keeps the first cycle's result; XCT_FISTA_UPDATE_X stores x_{t+1} in
// dest instead -- and x = dest.  The residual image is the plan's ratio buffer.
static int fista_loop(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it, float alpha,
                      double lambda_d, int flags, cudaStream_t st)
{
    const KGeom &g = p->kg;
    const size_t nimg = (size_t)g.nx * g.ny, nprj = (size_t)g.px * g.pa, nb = (size_t)p->g.max_batch;
    if (!p->d_fista) {
        cudaError_t e = cudaMalloc(&p->d_fista, sizeof(float) * 4 * nb * nimg);
        if (e != cudaSuccess) {
            p->d_fista = nullptr;
            return xct_cuda_fail(e, "cudaMalloc FISTA buffers");
        }
    }
    float *v = p->d_fista, *w = v + nb * nimg, *beta = w + nb * nimg, *dest = beta + nb * nimg;
    float *res = p->d_ratio;
    const size_t ibytes = sizeof(float) * dN * nimg, pbytes = sizeof(float) * dN * nprj;
    const float *meas = d_sino;
    int rc;
    if (p->g.correction_mode > 0) {
        rc = launch_sino_correction(g, d_sino, p->d_corr, p->d_corr_ang, p->d_corr_bin, p->g.correction_mode, dN, st);
        if (rc) return rc;
        meas = p->d_corr;
        XCT_CUDA_TRY(cudaMemcpyAsync(res, d_sino, pbytes, cudaMemcpyDeviceToDevice, st));
    } else {
        XCT_CUDA_TRY(cudaMemsetAsync(res, 0, pbytes, st));
    }
    rc = launch_bp_ref_plain(g, p->d_trig, meas, dest, dN, sub[0], g.ss, st);
    if (rc) return rc;
    XCT_CUDA_TRY(cudaMemcpyAsync(d_img, dest, ibytes, cudaMemcpyDeviceToDevice, st));
    XCT_CUDA_TRY(cudaMemcpyAsync(w, d_img, ibytes, cudaMemcpyDeviceToDevice, st));
    XCT_CUDA_TRY(cudaMemsetAsync(beta, 0, ibytes, st));
    const float *X = d_img;
    bool first = true;
    for (int i = 0; i < it; ++i)
        for (int k = 0; k < g.ss; ++k) {
            const int s = sub[k];
            const int rows = subset_rows(p, s);
            const float L = p->lip[s];
            // AART1: the forward projection into the subset's residual rows, then y - A x there
            if (p->g.kernels == XCT_KERNELS_TILED)
                rc = launch_fwd_tiled(g, p->d_trig, X, nullptr, res, p->d_acc, dN, s, g.ss, rows, st);
            else rc = launch_fwd_plain(g, p->d_trig, X, nullptr, res, dN, s, g.ss, rows, st);
            if (!rc) rc = launch_residual(g, meas, res, dN, s, g.ss, rows, st);
            if (rc) return rc;
            if (flags & XCT_FISTA_ADJOINT) {
                const float coef = ((((alpha * (float)g.ss) / (float)g.pa) / (float)g.depth) / L) * 0.5f;
                rc = launch_adj_subset(g, p->d_trig, res, v, dN, s, g.ss, (g.pa - s + g.ss - 1) / g.ss, X, coef, st);
            } else {
                rc = launch_fista_bp(g, p->d_trig, X, v, res, dN, s, alpha, L, st);
            }
            if (rc) return rc;
            const float lam = (float)(lambda_d / (double)L * 0.5);  // LAMBDA_FISTA/L[sub]*0.5f
            if (first) {
                rc = launch_ista3d(v, dest, g.nx, g.ny, dN, lam, p->ctx->sm_count, st);
                X = w;
                first = false;
            } else {
                rc = launch_fista3d(d_img, w, v, beta, (flags & XCT_FISTA_UPDATE_X) ? dest : nullptr, g.nx, g.ny, dN,
                                    lam, p->ctx->sm_count, st);
            }
            if (rc) return rc;
            XCT_CUDA_TRY(cudaMemcpyAsync(d_img, dest, ibytes, cudaMemcpyDeviceToDevice, st));
        }
    return XCT_OK;
}

static int check_fista(xct_plan *p, float alpha, float cs_lambda, int flags, cudaStream_t st)
{
    if (!(alpha > -1.0e30f && alpha < 1.0e30f)) return xct_fail(XCT_E_INVALID, "FISTA: alpha must be finite");
    if (!(cs_lambda >= 0.0f && cs_lambda < 1.0e30f))
        return xct_fail(XCT_E_INVALID, "FISTA: cs_lambda must be finite and >= 0");
    if (flags & ~(XCT_FISTA_UPDATE_X | XCT_FISTA_ADJOINT)) return xct_fail(XCT_E_INVALID, "FISTA: unknown flags");
    // FISTA_ocl estimates the Lipschitz constants before reconstructing (GPU.cpp:2250-2256)
    if ((int)p->lip.size() != p->g.ss) return xct_fista_power_iteration(p, 30, 1024, 0, nullptr, st);
    return XCT_OK;
}

// -D LAMBDA_FISTA: the float CSlambda streamed with six significant digits (FISTA_programBuild,
// GPU.cpp:2044), compiled as a double literal.
static double fista_lambda_literal(float cs_lambda)
{
    char b[64];
    snprintf(b, sizeof b, "%g", (double)cs_lambda);
    return strtod(b, nullptr);
}

int xct_fista_run_device(xct_plan *p, int dN, const float *d_sino, float *d_img, const int *sub, int it, float alpha,
                         float cs_lambda, int flags, void *stream)
{
    XCT_RANGE("xct_fista_run_device");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    if (!d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_fista_run_device: null device pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    rc = check_fista(p, alpha, cs_lambda, flags, st);
    if (rc) return rc;
    return fista_loop(p, dN, d_sino, d_img, sub ? sub : p->sub_default.data(), it, alpha,
                      fista_lambda_literal(cs_lambda), flags, st);
}

int xct_fista_run(xct_plan *p, int dN, const float *const *sino_host, float *const *img_host, const int *sub, int it,
                  float alpha, float cs_lambda, int flags)
{
    XCT_RANGE("xct_fista_run");
    if (p && it < 0) it = p->g.it;
    int rc = check_run(p, dN, sub, it);
    if (rc) return rc;
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    rc = check_fista(p, alpha, cs_lambda, flags, p->stream);
    if (rc) return rc;
    const double lam = fista_lambda_literal(cs_lambda);
    // the images' initial contents are not read: the backprojection of subset sub[0] replaces them
    return host_run(p, dN, sino_host, img_host, false, [&](cudaStream_t st) {
        return fista_loop(p, dN, p->d_sino, p->d_img, sub ? sub : p->sub_default.data(), it, alpha, lam, flags, st);
    });
}

int xct_plan_sync(xct_plan *p)
{
    if (!p) return xct_fail(XCT_E_INVALID, "plan is null");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    XCT_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return XCT_OK;
}

int xct_plan_last_ms(xct_plan *p, float *ms)
{
    if (!p || !ms) return xct_fail(XCT_E_INVALID, "null argument");
    *ms = p->last_ms;
    return XCT_OK;
}

}  // extern "C"

// geometry validation shared with the batched plans (xct_batch.cu)
int xct_check_geom(const xct_geom *g) { return check_geom(g); }
