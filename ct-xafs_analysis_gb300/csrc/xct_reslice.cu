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
//
// Reslice has two kernels with the same arithmetic.  reslice_tma_kernel (widths that are a
// multiple of 4, 16-byte aligned projections) is persistent: a CTA walks output tiles of 16
// rows x 128 columns of one projection through a 4-stage ring.  Warp 0 describes each tile
// once in the stage's slot -- the 16 sampler rows and weights (one lane each), whether they
// are consecutive, the window origin -- and issues the 3-D tensor copy (TMA) of its sampler
// window (19 rows x 136 columns) on the stage's mbarrier, three tiles ahead; the 256
// threads then form 8 outputs each from shared memory.  The row-walking reslice_kernel
// recomputes the rows in every thread and reads texels through the LSU (0.39 ms for 1500 x
// 64 x 2048 on a GB300 against 0.26 ms here).  The copy's zero fill outside the projection
// is the sampler's zero border.  reslice_kernel serves every other shape.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <string>
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
    int *d_err = nullptr;     // set by reslice_tma_kernel when a copy wait gave up
    int tma_grid = 0;         // persistent CTAs of reslice_tma_kernel (0: not set up)
    long long wait_clocks = 0;  // limit of its waits for staged copies (SM clocks)
};

namespace {

__device__ __forceinline__ float tex2(const float *__restrict__ im, int W, int H, int i, int j)
{
    return (i >= 0 && j >= 0 && i < W && j < H) ? __ldg(im + (size_t)j * W + i) : 0.0f;
}

constexpr int kRowsPerThread = 8;  // output rows a thread walks (reslice: Y; denoise: th)

constexpr int kColsPerThread = 1;  // reslice: columns per thread (2 measured slower: fewer threads in flight)

// The sampler rows j(Y) = floor(Y + sy) and weights of rows Yb .. Yb+n-1 (n <= 8); run is
// true when the rows are consecutive (rounding can break that, and is checked).
__device__ __forceinline__ bool reslice_rows(int Yb, int n, float sy, int (&j)[kRowsPerThread],
                                             float (&b)[kRowsPerThread])
{
    bool run = true;
#pragma unroll
    for (int r = 0; r < kRowsPerThread; ++r) {
        const float vv = (((float)(Yb + r) + sy) + 0.5f) - 0.5f;
        const float fj = floorf(vv);
        b[r] = vv - fj;
        j[r] = (int)fj;
        if (r > 0 && r < n && j[r] != j[r - 1] + 1) run = false;
    }
    return run;
}

// The sampler column i(X) = floor(X + sx) and weight a.
__device__ __forceinline__ int reslice_col(int X, float sx, float &a)
{
    const float uu = (((float)X + sx) + 0.5f) - 0.5f;
    const float fi = floorf(uu);
    a = uu - fi;
    return (int)fi;
}

// The reference's filtering sum of one output from its 2x2 texels, plus base-up and the
// optional correction factor.
__device__ __forceinline__ float reslice_value(float a, float b, float t00, float t10, float t01, float t11,
                                               float baseup, bool corr, float cf)
{
    float t = (1.0f - a) * (1.0f - b) * t00 + a * (1.0f - b) * t10 + (1.0f - a) * b * t01 + a * b * t11;
    t += baseup;
    if (corr) t *= cf;
    return t;
}

// Rows Yb .. Yb+n-1 of column X of projection im from global memory; out = the row-Yb output
// of this column, successive rows ostep apart.  When the sampler rows are consecutive the 9
// texel rows the 8 outputs need are loaded at once -- every load in flight together, each
// texel read once -- and each output is formed from registers; otherwise each row loads its
// own 2x2 footprint.
__device__ __forceinline__ void reslice_column_global(const float *__restrict__ im, int W, int H, int X, int n,
                                                      float a, int i, const int (&j)[kRowsPerThread],
                                                      const float (&b)[kRowsPerThread], bool run, float baseup,
                                                      bool corr, float cf, float *out, size_t ostep)
{
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
        for (int r = 0; r < kRowsPerThread; ++r)
            if (r < n) out[r * ostep] = reslice_value(a, b[r], c0[r], c1[r], c0[r + 1], c1[r + 1], baseup, corr, cf);
    } else {
        for (int r = 0; r < n; ++r)
            out[r * ostep] = reslice_value(a, b[r], tex2(im, W, H, i, j[r]), tex2(im, W, H, i + 1, j[r]),
                                           tex2(im, W, H, i, j[r] + 1), tex2(im, W, H, i + 1, j[r] + 1), baseup,
                                           corr, cf);
    }
}

// grid: (ceil(W/(256*kColsPerThread)), ceil(H/8), n); prj[Y][th0 + th][X] for projection th
// of the chunk.  A thread serves 8 rows Y of kColsPerThread columns X (256 apart).
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
    const bool run = reslice_rows(Yb, n, sy, j, b);
    const size_t ostep = (size_t)A * W;
#pragma unroll
    for (int cc = 0; cc < kColsPerThread; ++cc) {
        const int X = blockIdx.x * (blockDim.x * kColsPerThread) + cc * blockDim.x + threadIdx.x;
        if (X >= W) break;
        float a;
        const int i = reslice_col(X, sx, a);
        const float cf = corr != nullptr ? __ldg(corr + X) : 1.0f;
        float *out = prj + ((size_t)Yb * A + th0 + th) * W + X;
        reslice_column_global(im, W, H, X, n, a, i, j, b, run, baseup, corr != nullptr, cf, out, ostep);
    }
}

// ------------------------------------------------------------ TMA-staged reslice
constexpr int kTmaCols = 128;                  // output columns per tile (one per thread)
constexpr int kTmaRows = 2 * kRowsPerThread;   // output rows per tile (two threads per column)
constexpr int kTmaThreads = kTmaCols * 2;
// Staged window: columns from the sampler column of the tile's first column, less one,
// rounded down to a multiple of 4 (a tensor copy's x must be 16-byte aligned), 136 wide;
// rows from the first row's sampler row less one, 19 high.  Every thread checks that its
// texels lie inside and reads global memory for a column that rounding pushed outside.
constexpr int kTmaBoxW = kTmaCols + 8;
constexpr int kTmaBoxH = kTmaRows + 3;
constexpr int kTmaStages = 4;
constexpr unsigned kTmaBoxBytes = (unsigned)(kTmaBoxW * kTmaBoxH * sizeof(float));
constexpr unsigned kTmaStagePitch = (kTmaBoxBytes + 1023u) / 1024u * 1024u;
constexpr size_t kTmaSlotBytes = 512;  // one TmaTileInfo per stage
constexpr size_t kTmaBarBytes = (8 * kTmaStages + 15) / 16 * 16;
constexpr size_t kTmaSmem = 1024 + (size_t)kTmaStages * kTmaStagePitch + kTmaBarBytes + kTmaStages * kTmaSlotBytes;
// A copy normally lands in microseconds; a wait gives up after ~2^31 SM clocks (about a
// second; xct_reslice_plan_set_wait_limit changes the tile waits, not the final drain),
// flags the plan and the CTA finishes its tiles from global memory.
constexpr long long kTmaWaitClocks = 1ll << 31;

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for phase `parity` of the barrier to complete, at most `limit` SM clocks; a negative
// limit gives up at once (the plan's diagnostic setting).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity, long long limit)
{
    if (limit < 0) return false;
    if (mbar_test(bar, parity)) return true;
    const long long t0 = clock64();
    for (;;) {
        __nanosleep(32);
        if (mbar_test(bar, parity)) return true;
        if (clock64() - t0 > limit) return false;
    }
}
// Box (x, y, z) of the tensor map into shared memory at dst; completion counted on bar.
__device__ __forceinline__ void tma_load_box(unsigned dst, const CUtensorMap *map, int x, int y, int z, unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"((unsigned long long)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// Per-stage description of the tile whose window the stage holds, written by warp 0 when it
// issues the copy and read by every thread after the barrier that follows.
struct __align__(16) TmaTileInfo {
    float b[kTmaRows], ob[kTmaRows];  // weight b and 1 - b of each output row (float4 reads)
    int X0, Y0, th;  // first output column and row, projection within the call
    int xs0, ys0;    // window origin (column, row) in the projection
    float sx;        // the projection's x shift
    int run[2];      // rows [0, 8) / [8, 16) of the tile have consecutive sampler rows
    int j[kTmaRows];  // sampler row of each output row
};

static_assert(sizeof(TmaTileInfo) <= kTmaSlotBytes && kTmaSlotBytes % 16 == 0, "tile slot size");

// The reference's filtering sum with 1 - a and 1 - b precomputed (the same roundings).
__device__ __forceinline__ float reslice_value_w(float a, float oa, float b, float ob, float t00, float t10,
                                                 float t01, float t11, float baseup, bool corr, float cf)
{
    float t = oa * ob * t00 + a * ob * t10 + oa * b * t01 + a * b * t11;
    t += baseup;
    if (corr) t *= cf;
    return t;
}

// Persistent: CTA c takes tiles c, c + gridDim.x, ... in the order (column block, row block,
// projection), column block fastest.  Tensor map: projections [n][H][W] as a 3-D tensor
// (W, H, n) of floats, box (kTmaBoxW, kTmaBoxH, 1), zero fill.
__global__ void __launch_bounds__(kTmaThreads, 4) reslice_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                                  const float *__restrict__ mt,
                                                                  float *__restrict__ prj, int W, int H, int A,
                                                                  int th0, int n, const float *__restrict__ xs,
                                                                  const float *__restrict__ ys, float baseup,
                                                                  const float *__restrict__ corr, int *err,
                                                                  long long wait_clocks)
{
    extern __shared__ unsigned char smem_raw[];
    const unsigned raw = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned sbase = (raw + 1023u) & ~1023u;
    const unsigned bars = sbase + kTmaStages * kTmaStagePitch;  // kTmaStages 8-byte barriers
    unsigned char *const sgen = smem_raw + (sbase - raw);
    const float *stage_ptr0 = reinterpret_cast<const float *>(sgen);
    // slots after the barriers, 16-byte aligned (the stages are 1024-aligned)
    TmaTileInfo *info = reinterpret_cast<TmaTileInfo *>(sgen + kTmaStages * kTmaStagePitch + kTmaBarBytes);
    const int nxb = (W + kTmaCols - 1) / kTmaCols, nyb = (H + kTmaRows - 1) / kTmaRows;
    const long long ntiles = (long long)nxb * nyb * n;
    const long long first = blockIdx.x, stride = gridDim.x;
    const long long nmine = first < ntiles ? (ntiles - 1 - first) / stride + 1 : 0;
    const int tid = threadIdx.x, lane = tid & 31;
    const bool producer = tid < 32;  // warp 0 describes and issues the copies

    if (tid == 0) {
        for (int s = 0; s < kTmaStages; ++s) mbar_init(bars + 8u * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();

    // warp 0: coordinates of the next tile to issue, advanced by the grid stride with carries
    int qx = 0, qy = 0, qt = 0, dx = 0, dy = 0, dt = 0;
    if (producer) {
        const long long per = (long long)nxb * nyb;
        qt = (int)(first / per);
        const int q = (int)(first - (long long)qt * per);
        qy = q / nxb;
        qx = q - qy * nxb;
        dt = (int)(stride / per);
        const int r = (int)(stride - (long long)dt * per);
        dy = r / nxb;
        dx = r - dy * nxb;
    }
    // warp 0 (all lanes): describe the next tile in stage s's slot and, with copy, issue its
    // window copy (after a wait gave up, tiles are still described but not copied).  The
    // shifts of the tile after it are fetched here, a whole tile ahead of their use.
    float nsx = 0.0f, nsy = 0.0f;
    if (producer && nmine > 0) {
        nsx = __ldg(xs + th0 + qt);
        nsy = __ldg(ys + th0 + qt);
    }
    auto issue = [&](unsigned s, bool copy, bool more) {
        TmaTileInfo &ti = info[s];
        const float sx = nsx, sy = nsy;
        const int X0 = qx * kTmaCols, Y0 = qy * kTmaRows;
        int jl = 0;
        if (lane < kTmaRows) {
            const float vv = (((float)(Y0 + lane) + sy) + 0.5f) - 0.5f;  // as reslice_rows
            const float fj = floorf(vv);
            const float bb = vv - fj;
            jl = (int)fj;
            ti.j[lane] = jl;
            ti.b[lane] = bb;
            ti.ob[lane] = 1.0f - bb;
        }
        const int prev = __shfl_up_sync(0xffffffffu, jl, 1);
        const bool broken = lane < kTmaRows && (lane % kRowsPerThread) != 0 && Y0 + lane < H && jl != prev + 1;
        const unsigned bad = __ballot_sync(0xffffffffu, broken);
        const int j0 = __shfl_sync(0xffffffffu, jl, 0);
        if (lane == 0) {
            float a;
            const int i0 = reslice_col(X0, sx, a);
            const int xs0 = (i0 - 1) & ~3;  // floor to a multiple of 4, negative values included
            const int ys0 = j0 - 1;
            ti.X0 = X0;
            ti.Y0 = Y0;
            ti.th = qt;
            ti.xs0 = xs0;
            ti.ys0 = ys0;
            ti.sx = sx;
            ti.run[0] = (bad & 0x00ffu) == 0;
            ti.run[1] = (bad & 0xff00u) == 0;
            if (copy) {
                const unsigned bar = bars + 8u * s;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive_expect_tx(bar, kTmaBoxBytes);
                tma_load_box(sbase + s * kTmaStagePitch, &map, xs0, ys0, qt, bar);
            }
        }
        qx += dx;
        if (qx >= nxb) { qx -= nxb; ++qy; }
        qy += dy;
        if (qy >= nyb) { qy -= nyb; ++qt; }
        qt += dt;
        if (more) {  // a next tile exists: qt is one of this call's projections
            nsx = __ldg(xs + th0 + qt);
            nsy = __ldg(ys + th0 + qt);
        }
    };
    long long issued = nmine < kTmaStages ? nmine : kTmaStages;  // the same count in every thread
    if (producer)
        for (long long k = 0; k < issued; ++k) issue((unsigned)k, true, k + 1 < nmine);

    bool alive = true;  // false once a wait gave up: no more copies, global memory from then on
    long long consumed = 0;
    const int col = tid % kTmaCols, half = tid / kTmaCols;
    const size_t ostep = (size_t)A * W;
    for (long long k = 0; k < nmine; ++k) {
        const unsigned s = (unsigned)(k % kTmaStages), parity = (unsigned)((k / kTmaStages) & 1);
        bool ok = alive && mbar_wait_bounded(bars + 8u * s, parity, wait_clocks);
        // one barrier per tile: makes the outcome uniform, publishes the slots written since
        // the last one, and frees the previous tile's stage and slot
        ok = __syncthreads_and(ok) != 0;
        if (alive && !ok) {
            alive = false;
            if (tid == 0) atomicAdd(err, 1);
        }
        if (ok) consumed = k + 1;
        if (k >= 1 && k - 1 + kTmaStages < nmine) {
            if (producer) issue((unsigned)((k - 1) % kTmaStages), alive, k + kTmaStages < nmine);
            if (alive) issued = k - 1 + kTmaStages + 1;
        }

        const TmaTileInfo &ti = info[s];
        const int X = ti.X0 + col, Yb = ti.Y0 + half * kRowsPerThread;
        const int nr = min(kRowsPerThread, H - Yb);
        if (X >= W || nr <= 0) continue;
        const int r0 = half * kRowsPerThread;
        float a;
        const int i = reslice_col(X, ti.sx, a);
        const float oa = 1.0f - a;
        const float cf = corr != nullptr ? __ldg(corr + X) : 1.0f;
        float *out = prj + ((size_t)Yb * A + th0 + ti.th) * W + X;
        const int ci = i - ti.xs0, rj = ti.j[r0] - ti.ys0;
        const bool run = ti.run[half] != 0;
        const bool inside = ok && run && ci >= 0 && ci + 1 < kTmaBoxW && rj >= 0 && rj + nr < kTmaBoxH;
        if (inside) {
            const float *w = stage_ptr0 + (size_t)s * (kTmaStagePitch / 4) + rj * kTmaBoxW + ci;
            float bw[kRowsPerThread], obw[kRowsPerThread];
#pragma unroll
            for (int q = 0; q < kRowsPerThread; q += 4) {
                const float4 v = *reinterpret_cast<const float4 *>(&ti.b[r0 + q]);
                const float4 o = *reinterpret_cast<const float4 *>(&ti.ob[r0 + q]);
                bw[q] = v.x, bw[q + 1] = v.y, bw[q + 2] = v.z, bw[q + 3] = v.w;
                obw[q] = o.x, obw[q + 1] = o.y, obw[q + 2] = o.z, obw[q + 3] = o.w;
            }
            float c0[kRowsPerThread + 1], c1[kRowsPerThread + 1];
            if (nr == kRowsPerThread) {  // every tile but a last, partial row block
#pragma unroll
                for (int r = 0; r <= kRowsPerThread; ++r) {
                    c0[r] = w[r * kTmaBoxW];
                    c1[r] = w[r * kTmaBoxW + 1];
                }
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r)
                    out[r * ostep] = reslice_value_w(a, oa, bw[r], obw[r], c0[r], c1[r], c0[r + 1], c1[r + 1],
                                                     baseup, corr != nullptr, cf);
            } else {
#pragma unroll
                for (int r = 0; r <= kRowsPerThread; ++r) {
                    c0[r] = r <= nr ? w[r * kTmaBoxW] : 0.0f;
                    c1[r] = r <= nr ? w[r * kTmaBoxW + 1] : 0.0f;
                }
#pragma unroll
                for (int r = 0; r < kRowsPerThread; ++r)
                    if (r < nr)
                        out[r * ostep] = reslice_value_w(a, oa, bw[r], obw[r], c0[r], c1[r], c0[r + 1], c1[r + 1],
                                                         baseup, corr != nullptr, cf);
            }
        } else {
            int j[kRowsPerThread];
            float b[kRowsPerThread];
#pragma unroll
            for (int r = 0; r < kRowsPerThread; ++r) {
                j[r] = ti.j[r0 + r];
                b[r] = ti.b[r0 + r];
            }
            reslice_column_global(mt + (size_t)ti.th * H * W, W, H, X, nr, a, i, j, b, run, baseup, corr != nullptr,
                                  cf, out, ostep);
        }
    }
    // copies issued but never waited for (only after a wait gave up; at most one per stage):
    // let them land before the CTA's shared memory is released, each wait again bounded
    if (tid == 0)
        for (long long k = consumed; k < issued; ++k)
            (void)mbar_wait_bounded(bars + 8u * (unsigned)(k % kTmaStages), (unsigned)((k / kTmaStages) & 1),
                                    kTmaWaitClocks);
}

constexpr int kDenoiseRows = 16;  // angles a denoise thread walks

// grid: (ceil(W/256), ceil(A/16), H) over sinograms [H][A][W]; a thread walks 16 angles of one
// column with the angle rows in registers (18 loads for 16 outputs, all in flight at once);
// neighbours clamped to the edge.
__global__ void __launch_bounds__(256) denoise_kernel(const float *__restrict__ src, float *__restrict__ dst, int W,
                                                      int A, float thr)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int t0 = blockIdx.y * kDenoiseRows, Y = blockIdx.z;
    if (X >= W) return;
    const float *base = src + (size_t)Y * A * W + X;
    // rows t0-1 .. t0+16 (clamped), all loads first
    float f[kDenoiseRows + 2];
#pragma unroll
    for (int r = 0; r < kDenoiseRows + 2; ++r) f[r] = __ldg(base + (size_t)min(max(t0 - 1 + r, 0), A - 1) * W);
    float *out = dst + ((size_t)Y * A + t0) * W + X;
#pragma unroll
    for (int r = 0; r < kDenoiseRows; ++r) {
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
    cudaFree(p->d_err);
    delete p;
}

// cuTensorMapEncodeTiled from the driver, looked up once (no link-time libcuda dependency).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(ptr);
        (void)cudaGetLastError();
    });
    return fn;
}

// Tensor map of projections [n][H][W] (floats) with the staged window as its box.
bool encode_projection_map(CUtensorMap *map, const float *d_proj, int W, int H, int n)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)n};
    const cuuint64_t strides[2] = {(cuuint64_t)W * sizeof(float), (cuuint64_t)W * H * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)kTmaBoxW, (cuuint32_t)kTmaBoxH, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(d_proj), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
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
    p->wait_clocks = kTmaWaitClocks;
    auto fail = [&](cudaError_t e, const char *what) {
        int r = xct_cuda_fail(e, what);
        reslice_free(p);
        return r;
    };
    cudaError_t e;
    if ((e = cudaMalloc(&p->d_err, sizeof(int))) != cudaSuccess) return fail(e, "cudaMalloc error word");
    if ((e = cudaMemset(p->d_err, 0, sizeof(int))) != cudaSuccess) return fail(e, "clear error word");
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
    if (width % 4 == 0 && tensor_map_encoder()) {
        int per_sm = 0;
        if ((e = cudaFuncSetAttribute(reslice_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kTmaSmem)) != cudaSuccess)
            return fail(e, "reslice kernel attributes");
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reslice_tma_kernel, kTmaThreads,
                                                               kTmaSmem)) != cudaSuccess)
            return fail(e, "reslice kernel occupancy");
        p->tma_grid = std::max(1, per_sm) * ctx->sm_count;
    }
    *out = p;
    return XCT_OK;
}

int xct_reslice_plan_destroy(xct_reslice_plan *p)
{
    if (!p) return XCT_OK;
    cudaSetDevice(p->ctx->device);
    int err = 0;
    const bool read = cudaDeviceSynchronize() == cudaSuccess &&
                      cudaMemcpy(&err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
    reslice_free(p);
    if (read && err != 0)
        return xct_fail(XCT_E_TIMEOUT, "xct_reslice: " + std::to_string(err) +
                                           " tile copies did not land within the wait limit; those tiles were "
                                           "read from global memory instead (results are complete)");
    return XCT_OK;
}

int xct_reslice(xct_reslice_plan *p, int first_angle, int n, const float *d_proj, float *d_sino, void *stream)
{
    XCT_RANGE("xct_reslice");
    if (!p) return xct_fail(XCT_E_INVALID, "xct_reslice: plan is null");
    if (!d_proj || !d_sino) return xct_fail(XCT_E_INVALID, "xct_reslice: null device pointer");
    if (n <= 0 || first_angle < 0 || first_angle + n > p->A) {
        char b[160];
        snprintf(b, sizeof b, "xct_reslice: angles [%d, %d) outside the plan's %d", first_angle, first_angle + n, p->A);
        return xct_fail(XCT_E_INVALID, b);
    }
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    CUtensorMap map;
    if (p->tma_grid > 0 && ((uintptr_t)d_proj & 15u) == 0 && encode_projection_map(&map, d_proj, p->W, p->H, n)) {
        const long long tiles = (long long)((p->W + kTmaCols - 1) / kTmaCols) * ((p->H + kTmaRows - 1) / kTmaRows) * n;
        const int grid = (int)std::min<long long>(tiles, p->tma_grid);
        reslice_tma_kernel<<<grid, kTmaThreads, kTmaSmem, (cudaStream_t)stream>>>(
            map, d_proj, d_sino, p->W, p->H, p->A, first_angle, n, p->d_xs, p->d_ys, p->baseup, p->d_corr, p->d_err,
            p->wait_clocks);
    } else {
        dim3 grid((p->W + 256 * kColsPerThread - 1) / (256 * kColsPerThread),
                  (p->H + kRowsPerThread - 1) / kRowsPerThread, n);
        reslice_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_proj, d_sino, p->W, p->H, p->A, first_angle,
                                                               p->d_xs, p->d_ys, p->baseup, p->d_corr);
    }
    XCT_CUDA_TRY(cudaGetLastError());
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

int xct_reslice_plan_set_wait_limit(xct_reslice_plan *p, long long sm_clocks)
{
    if (!p) return xct_fail(XCT_E_INVALID, "xct_reslice_plan_set_wait_limit: plan is null");
    p->wait_clocks = sm_clocks;
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
    dim3 grid((width + 255) / 256, (n_angles + kDenoiseRows - 1) / kDenoiseRows, n_rows);
    denoise_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(d_src, d_dst, width, n_angles, threshold);
    XCT_CUDA_TRY(cudaGetLastError());
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

}  // extern "C"
