// xct_noalloc.cu -- OS-EM for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: an acquisition loop that must never stall on the
// allocator (cudaMalloc can synchronise the device), a host application whose device memory
// is all owned by its own pool, or code that runs where allocation is forbidden.  For them,
// xct_osem_run_static reconstructs from the caller's own sinograms and images and allocates
// nothing.  The scratch that the tiled kernels need -- the (cos, sin) table, the ratio image
// and the ray-sum accumulator -- lives in ONE file-scope __device__ array of
// XCT_STATIC_SCRATCH_BYTES bytes.  Every GPU that loads this library holds that array until
// the process exits, so it is kept modest; problems that need more are rejected.
//
// In host code the array's name is only a host-side stand-in for the symbol, not a device
// address: its device address is fetched with cudaGetSymbolAddress once per device (with
// that device current) on the first call made on that device, and passed to the kernels.
// That address belongs to the device's current context: after a cudaDeviceReset the module
// is loaded anew and the cached address is stale, so this entry point must not be used on a
// device after it has been reset.
//
// The (cos, sin) table is uploaded on every call from a stack buffer (pageable memory), so a
// call cannot be captured into a CUDA graph: a replay would read a stack buffer that no
// longer exists.  Calls made while the stream is capturing are rejected.
#include <math.h>
#include <stdio.h>

#include <mutex>

#include "xct_internal.h"

namespace {

__device__ __align__(256) unsigned char g_static_scratch[XCT_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};  // device address of g_static_scratch, per device

size_t round256(size_t n) { return (n + 255) & ~(size_t)255; }

// Device address of the static scratch on the current device (set up on first use).
int scratch_address(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess) return xct_cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
        g_scratch_addr[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_scratch_addr[dev]);
    return XCT_OK;
}

}  // namespace

extern "C" int xct_osem_run_static(const xct_geom *g, int dN, const float *d_sino, float *d_img, const int *sub,
                                   int it, void *stream)
{
    XCT_RANGE("xct_osem_run_static");
    if (!g || !d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_osem_run_static: null argument");
    if (g->nx <= 0 || g->ny <= 0 || g->px <= 0 || g->pa <= 0 || g->ss <= 0 || g->ss > g->pa || !g->angles_deg)
        return xct_fail(XCT_E_INVALID, "xct_osem_run_static: invalid geometry");
    if (g->ox != g->nx || g->oy != g->ny)
        return xct_fail(XCT_E_INVALID, "xct_osem_run_static: the output ROI must equal the reconstruction size");
    if (g->nx > 16384 || g->ny > 16384 || g->px > 65536 || g->pa > 65536)
        return xct_fail(XCT_E_INVALID, "xct_osem_run_static: size beyond the supported maximum");
    if (g->measured_fetch_mode != XCT_FETCH_EXACT && g->measured_fetch_mode != XCT_FETCH_AVG2X2)
        return xct_fail(XCT_E_INVALID, "xct_osem_run_static: invalid measured_fetch_mode");
    if (g->subset_mode != XCT_SUBSETS_REF && g->subset_mode != XCT_SUBSETS_COVER)
        return xct_fail(XCT_E_INVALID, "xct_osem_run_static: invalid subset_mode");
    if (g->correction_mode != 0)
        return xct_fail(XCT_E_UNSUPPORTED,
                        "xct_osem_run_static: sinogram correction needs a corrected-sinogram buffer; use a plan");
    if (dN <= 0) return xct_fail(XCT_E_INVALID, "xct_osem_run_static: dN must be > 0");
    if (it < 0) it = g->it;
    if (it < 0) return xct_fail(XCT_E_INVALID, "xct_osem_run_static: iterations must be >= 0");
    if (sub)
        for (int k = 0; k < g->ss; ++k)
            if (sub[k] < 0 || sub[k] >= g->ss)
                return xct_fail(XCT_E_INVALID, "xct_osem_run_static: subset order entry out of range");
    for (int i = 0; i < g->pa; ++i)
        if (!(fabsf(g->angles_deg[i]) < 1.0e6f)) return xct_fail(XCT_E_INVALID, "xct_osem_run_static: bad angle");

    // scratch layout: trig [pa] float2 | accumulator [dN][ceil(pa/ss)][px] f64 | ratio [dN][pa][px] f32
    const int rows = (g->pa + g->ss - 1) / g->ss;
    const size_t trig_bytes = round256(sizeof(float2) * (size_t)g->pa);
    const size_t acc_bytes = round256(sizeof(double) * (size_t)dN * rows * g->px);
    const size_t ratio_bytes = sizeof(float) * (size_t)dN * g->pa * g->px;
    const size_t need = trig_bytes + acc_bytes + ratio_bytes;
    if (need > (size_t)XCT_STATIC_SCRATCH_BYTES) {
        char b[320];
        snprintf(b, sizeof b,
                 "xct_osem_run_static: this problem needs %zu bytes of scratch; the static scratch holds %u bytes "
                 "(XCT_STATIC_SCRATCH_BYTES). Use fewer slices per call or a plan (xct_osem_run_device).",
                 need, (unsigned)XCT_STATIC_SCRATCH_BYTES);
        return xct_fail(XCT_E_INVALID, b);
    }

    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    // the per-call pageable upload of the angle table cannot be replayed from a graph
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    const cudaError_t ce = cudaStreamIsCapturing(st, &cap);
    if (ce != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        if (ce != cudaSuccess) (void)cudaGetLastError();  // not a sticky error: clear it
        return xct_fail(XCT_E_UNSUPPORTED,
                        "xct_osem_run_static: the stream is being captured; this entry point uploads its angle table "
                        "from host memory on every call and cannot be captured into a CUDA graph (use a plan)");
    }

    int dev = 0;
    XCT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return xct_fail(XCT_E_INVALID, "xct_osem_run_static: device index too large");
    unsigned char *base = nullptr;
    int rc = scratch_address(dev, &base);
    if (rc) return rc;
    float2 *d_trig = reinterpret_cast<float2 *>(base);
    double *d_acc = reinterpret_cast<double *>(base + trig_bytes);
    float *d_ratio = reinterpret_cast<float *>(base + trig_bytes + acc_bytes);
    // (cos, sin) table, computed exactly as for a plan, staged through a small stack buffer
    // (a pageable copy returns once the source has been read)
    float2 chunk[256];
    for (int t0 = 0; t0 < g->pa; t0 += 256) {
        const int n = (g->pa - t0) < 256 ? (g->pa - t0) : 256;
        for (int i = 0; i < n; ++i) {
            const float phi = (float)(((double)g->angles_deg[t0 + i] * 3.14159265358979323846) / 180.0);
            chunk[i].x = (float)cos((double)phi);
            chunk[i].y = (float)sin((double)phi);
        }
        XCT_CUDA_TRY(cudaMemcpyAsync(d_trig + t0, chunk, sizeof(float2) * n, cudaMemcpyHostToDevice, st));
    }
    // the previous call's contents stay in the array: the accumulator must start at zero,
    // and ratio rows that OSEM1 never writes must read as zero
    XCT_CUDA_TRY(cudaMemsetAsync(d_acc, 0, acc_bytes, st));
    XCT_CUDA_TRY(cudaMemsetAsync(d_ratio, 0, ratio_bytes, st));

    KGeom k;
    k.nx = g->nx;
    k.ny = g->ny;
    k.px = g->px;
    k.pa = g->pa;
    k.ss = g->ss;
    k.depth = g->nx > g->ny ? g->nx : g->ny;
    k.hx = (float)g->nx * 0.5f;
    k.hy = (float)g->ny * 0.5f;
    k.hd = (float)k.depth * 0.5f;
    k.cx = g->center_bin < 0.0f ? (float)g->px * 0.5f : g->center_bin;
    k.fetch = g->measured_fetch_mode;
    k.fwd_T = 92;  // the default tiles; this path keeps no per-shape state
    k.fwd_chunk = fwd_tiled_rows_cap();

    for (int i = 0; i < it; ++i)
        for (int kk = 0; kk < g->ss; ++kk) {
            const int s = sub ? sub[kk] : xct_subset_at(g->ss, kk);
            const int nrows = g->subset_mode == XCT_SUBSETS_COVER ? (g->pa - s + g->ss - 1) / g->ss : g->pa / g->ss;
            rc = launch_fwd_tiled(k, d_trig, d_img, d_sino, d_ratio, d_acc, dN, s, g->ss, nrows, st);
            if (rc) return rc;
            rc = launch_bp_update_tiled(k, d_trig, d_img, d_ratio, dN, s, st);
            if (rc) return rc;
        }
    return XCT_OK;
}
