// xct_tiled.cu -- the optimised OS-EM kernels for sm_103a.
//
// Forward projector (OSEM1 / projection, OSEM.cl:38-68, reconstShare.cl:213-241),
// tile-stationary:
//   * one CTA owns an image tile: the taps whose base texel (floor(x), floor(y)) lies in
//     [x0, x0+T) x [y0, y0+T), with x0 = -1 + bx*T (base texel -1 still reaches texel 0).
//     It stages texels [x0, x0+T] x [y0, y0+T] (zero outside the image: the sampler's
//     CLK_ADDRESS_CLAMP border) in shared memory ONCE and serves every angle of its angle
//     chunk from there, so the image is read from L2 once per subset instead of once per
//     angle;
//   * a warp takes one angle and 32 consecutive rays; each lane computes the exact range of
//     sample indices Y whose base texel is in the tile (the sample coordinates are monotone
//     in Y, so the range is an interval), then sums those bilinear samples from shared
//     memory with the same arithmetic as the plain kernel;
//   * the per-tile partial ray sums are added into a double-precision accumulator with
//     atomics (one per ray and tile; ~1 per 50-130 samples).
// A finalize/ratio kernel turns the accumulator into the OSEM1 ratio (or the raw
// projection) and clears it for the next subset.
//
// Backprojector (OSEM2, OSEM.cl:71-105), footprint-staged:
//   * one CTA owns a 32x32 pixel tile; for each angle of the subset it stages the window of
//     ratio bins that the tile's pixels hit (bin coordinates are monotone in X and in Y, so
//     the four corners bound the window exactly; <= 46 bins for 32x32) into shared memory
//     with coalesced loads, then every thread gathers its 4 pixels' bins from there, in
//     angle order, with the reference's own bin arithmetic (no contraction);
//   * the multiplicative update is fused into the same kernel.
#include "xct_device.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kFwdTile = 64;           // owned base texels per tile side
constexpr int kFwdPitch = kFwdTile + 1; // staged texels per row (T + 1)
constexpr int kAngChunk = 128;          // angles per CTA (forward) / per staging pass (back)
constexpr int kBpTile = 32;             // pixels per backprojection tile side
constexpr int kBpWin = 48;              // staged bins per angle (>= 31*(|c|+|s|) + 3)

// ---------------------------------------------------------------------- ray intervals
// Sample coordinate along a ray: u(Y) = fma(Y - hd, sl, a), monotone in Y.
__device__ __forceinline__ float ray_coord(int Y, float hd, float sl, float a)
{
    return fmaf((float)Y - hd, sl, a);
}

// First Y in [0, D] where the monotone predicate P(Y) holds (D if none):
//   sl > 0: P(Y) = u(Y) >= b ;  sl < 0: P(Y) = u(Y) < b.
// Estimate from the real crossing point, correct with a few exact evaluations, and fall
// back to a binary search (11-12 steps) when the slope is too small for the estimate.
__device__ int first_true(float b, float a, float sl, float inv_sl, float hd, int D)
{
    const bool up = sl > 0.0f;
    auto P = [&](int Y) {
        const float u = ray_coord(Y, hd, sl, a);
        return up ? (u >= b) : (u < b);
    };
    float e = fmaf(b - a, inv_sl, hd);
    e = fminf(fmaxf(e, -1.0f), (float)D + 1.0f);  // also maps +-inf; NaN -> -1
    int Y = (int)ceilf(e);
    Y = Y < 0 ? 0 : (Y > D ? D : Y);
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (Y > 0 && P(Y - 1)) --Y;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if (Y < D && !P(Y)) ++Y;
    const bool ok = (Y == 0 || !P(Y - 1)) && (Y == D || P(Y));
    if (!ok) {
        int lo = 0, hi = D;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (P(mid)) hi = mid;
            else lo = mid + 1;
        }
        Y = lo;
    }
    return Y;
}

// Y range [ya, yb) of samples whose coordinate u lies in [lo, hi).
__device__ __forceinline__ void coord_range(float lo, float hi, float a, float sl, float inv_sl, float hd, int D,
                                            int &ya, int &yb)
{
    if (sl > 0.0f) {
        ya = first_true(lo, a, sl, inv_sl, hd, D);
        yb = first_true(hi, a, sl, inv_sl, hd, D);
    } else if (sl < 0.0f) {
        ya = first_true(hi, a, sl, inv_sl, hd, D);
        yb = first_true(lo, a, sl, inv_sl, hd, D);
    } else {  // constant coordinate: fma(Yc, 0, a) == a for every Y
        const bool in = (a >= lo) && (a < hi);
        ya = 0;
        yb = in ? D : 0;
    }
}

// ----------------------------------------------------------------- forward projector
// grid: (ntx*nty tiles, angle chunks, dN).  acc: [dN][rows][px] doubles.
__global__ void __launch_bounds__(kThreads) fwd_tiled_kernel(const float *__restrict__ img,
                                                             double *__restrict__ acc,
                                                             const float2 *__restrict__ trig, KGeom g, int sub,
                                                             int step, int nrows, int ntx)
{
    __shared__ float tile[kFwdPitch * kFwdPitch];
    __shared__ float2 scs[kAngChunk];

    const int bx = blockIdx.x % ntx, by = blockIdx.x / ntx;
    const int z = blockIdx.z;
    const int k0 = blockIdx.y * kAngChunk;
    const int kn = min(kAngChunk, nrows - k0);
    const int x0 = -1 + bx * kFwdTile, y0 = -1 + by * kFwdTile;
    const float *im = img + (size_t)z * g.nx * g.ny;

    for (int i = threadIdx.x; i < kFwdPitch * kFwdPitch; i += kThreads) {
        const int r = i / kFwdPitch, c = i - r * kFwdPitch;
        const int gx = x0 + c, gy = y0 + r;
        float v = 0.0f;
        if ((unsigned)gx < (unsigned)g.nx && (unsigned)gy < (unsigned)g.ny) v = __ldg(im + (size_t)gy * g.nx + gx);
        tile[i] = v;
    }
    for (int k = threadIdx.x; k < kn; k += kThreads) scs[k] = trig[sub + (k0 + k) * step];
    __syncthreads();

    // owned base-texel ranges (the union over tiles is [-1, n-1]: base texel -1 reaches
    // texel 0, base texel n-1 still reads texel n-1)
    const float xlo = (float)x0, xhi = (float)min(x0 + kFwdTile, g.nx);
    const float ylo = (float)y0, yhi = (float)min(y0 + kFwdTile, g.ny);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int D = g.depth;

    for (int k = warp; k < kn; k += kWarps) {
        const float c = scs[k].x, s = scs[k].y;
        const float inv_s = 1.0f / s, inv_c = 1.0f / c;
        // rays that can reach the tile: project the (expanded) tile corners on the
        // detector axis, X = (x - nx/2) c - (y - ny/2) s + cx
        float pmin = 3.0e38f, pmax = -3.0e38f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float px_ = (q & 1) ? xhi + 2.0f : xlo - 2.0f;
            const float py_ = (q & 2) ? yhi + 2.0f : ylo - 2.0f;
            const float p = (px_ - g.hx) * c - (py_ - g.hy) * s + g.cx;
            pmin = fminf(pmin, p);
            pmax = fmaxf(pmax, p);
        }
        const int Xlo = max(0, (int)floorf(pmin) - 1);
        const int Xhi = min(g.px - 1, (int)ceilf(pmax) + 1);
        for (int base = Xlo; base <= Xhi; base += 32) {
            const int X = base + lane;
            int ya = 0, yb = 0;
            float ax = 0.0f, ay = 0.0f;
            if (X <= Xhi) {
                const float Xc = (float)X - g.cx;
                ax = fmaf(Xc, c, g.hx);
                ay = fmaf(Xc, -s, g.hy);
                int a0, a1, b0, b1;
                coord_range(xlo, xhi, ax, s, inv_s, g.hd, D, a0, a1);
                coord_range(ylo, yhi, ay, c, inv_c, g.hd, D, b0, b1);
                ya = max(a0, b0);
                yb = min(a1, b1);
            }
            float sum = 0.0f;
            for (int Y = ya; Y < yb; ++Y) {
                const float Yc = (float)Y - g.hd;
                const float x = fmaf(Yc, s, ax);
                const float y = fmaf(Yc, c, ay);
                const int bxs = xct_floor_bits(x), bys = xct_floor_bits(y);
                const float fx = x - (__int_as_float(bxs) - 12582912.0f);
                const float fy = y - (__int_as_float(bys) - 12582912.0f);
                const int col = bxs - XCT_FLOOR_BIAS - x0;
                const int row = bys - XCT_FLOOR_BIAS - y0;
                const float *t = tile + row * kFwdPitch + col;
                const float q0 = xct_lerp(fx, t[0], t[1]);
                const float q1 = xct_lerp(fx, t[kFwdPitch], t[kFwdPitch + 1]);
                sum += xct_lerp(fy, q0, q1);
            }
            if (yb > ya) atomicAdd(acc + ((size_t)z * nrows + k0 + k) * g.px + X, (double)sum);
        }
    }
}

// acc -> OSEM1 ratio (meas != nullptr) or raw projection, rows th = sub + k*step; clears acc.
__global__ void fwd_finalize_kernel(double *__restrict__ acc, const float *__restrict__ meas,
                                    float *__restrict__ out, KGeom g, int sub, int step, int nrows)
{
    const int X = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = blockIdx.y, z = blockIdx.z;
    if (X >= g.px) return;
    double *a = acc + ((size_t)z * nrows + k) * g.px + X;
    const float p = (float)*a;
    *a = 0.0;
    const int th = sub + k * step;
    const size_t o = ((size_t)z * g.pa + th) * g.px + X;
    if (meas != nullptr) {
        const float yv = xct_measured(meas + (size_t)z * g.pa * g.px, g.px, g.pa, X, th, g.fetch);
        out[o] = xct_ratio(yv, p);
    } else {
        out[o] = p;
    }
}

// ------------------------------------------------------------------- backprojector
// grid: (ntx*nty tiles, 1, dN).  Angles th = sub + k*ss for k < nang (as OSEM2 loops).
__global__ void __launch_bounds__(kThreads) bp_tiled_kernel(float *__restrict__ img,
                                                            const float *__restrict__ ratio,
                                                            const float2 *__restrict__ trig, KGeom g, int sub,
                                                            int nang, int ntx, float ssf, float paf)
{
    __shared__ float win[kAngChunk * kBpWin];
    __shared__ float2 scs[kAngChunk];
    __shared__ int sbase[kAngChunk];

    const int bx = blockIdx.x % ntx, by = blockIdx.x / ntx;
    const int z = blockIdx.z;
    const int X0 = bx * kBpTile, Y0 = by * kBpTile;
    const int X1 = min(X0 + kBpTile, g.nx) - 1, Y1 = min(Y0 + kBpTile, g.ny) - 1;
    const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;  // 8 x 4 pixels per row, 32 rows
    const int Y = Y0 + ty;
    // threads past the image edge of a partial tile gather for the edge pixel (inside the
    // staged window) and write nothing
    const float Yc = (float)min(Y, Y1) - g.hy;
    float Xc[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        Xc[i] = (float)min(X0 + tx * 4 + i, X1) - g.hx;
        b[i] = 0.0f;
    }
    const float *rt = ratio + (size_t)z * g.pa * g.px;

    for (int k0 = 0; k0 < nang; k0 += kAngChunk) {
        const int kn = min(kAngChunk, nang - k0);
        __syncthreads();  // previous chunk's gathers are done with win/scs/sbase
        for (int k = threadIdx.x; k < kn; k += kThreads) {
            const float2 cs = trig[sub + (k0 + k) * g.ss];
            scs[k] = cs;
            // bin coordinate is monotone in X and in Y: the corners bound the window
            const float xa = (float)X0 - g.hx, xb = (float)X1 - g.hx;
            const float yA = (float)Y0 - g.hy, yB = (float)Y1 - g.hy;
            const float qa = yA * cs.y, qb = yB * cs.y;
            int lo = xct_floor_bits(xct_bin_coord(xa, cs.x, qa, g.cx));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qa, g.cx)));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xa, cs.x, qb, g.cx)));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qb, g.cx)));
            sbase[k] = lo - XCT_FLOOR_BIAS;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kn * kBpWin; i += kThreads) {
            const int k = i / kBpWin, j = i - k * kBpWin;
            const int bin = sbase[k] + j;
            const int th = sub + (k0 + k) * g.ss;
            win[i] = ((unsigned)bin < (unsigned)g.px) ? __ldg(rt + (size_t)th * g.px + bin) : 0.0f;
        }
        __syncthreads();
        for (int k = 0; k < kn; ++k) {
            const float c = scs[k].x;
            const float q = Yc * scs[k].y;
            const int off = k * kBpWin - (sbase[k] + XCT_FLOOR_BIAS);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int bits = xct_floor_bits(xct_bin_coord(Xc[i], c, q, g.cx));
                b[i] += win[bits + off];
            }
        }
    }
    if (Y <= Y1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int X = X0 + tx * 4 + i;
            if (X <= X1) {
                float *p = img + ((size_t)z * g.ny + Y) * g.nx + X;
                *p = xct_update(*p, b[i], ssf, paf);
            }
        }
    }
}

}  // namespace

int fwd_tiled_rows_cap() { return kAngChunk; }

int launch_fwd_tiled(const KGeom &g, const float2 *trig, const float *img, const float *meas, float *out,
                     double *acc, int dN, int sub, int step, int nrows, cudaStream_t st)
{
    if (nrows <= 0 || dN <= 0) return XCT_OK;
    const int ntx = (g.nx + 1 + kFwdTile - 1) / kFwdTile;  // base texels -1 .. nx-1
    const int nty = (g.ny + 1 + kFwdTile - 1) / kFwdTile;
    const int nch = (nrows + kAngChunk - 1) / kAngChunk;
    dim3 grid(ntx * nty, nch, dN);
    fwd_tiled_kernel<<<grid, kThreads, 0, st>>>(img, acc, trig, g, sub, step, nrows, ntx);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return launch_fwd_finalize(g, meas, out, acc, dN, sub, step, nrows, st);
}

int launch_fwd_tiled_main(const KGeom &g, const float2 *trig, const float *img, double *acc, int dN, int sub, int step,
                          int nrows, cudaStream_t st)
{
    if (nrows <= 0 || dN <= 0) return XCT_OK;
    const int ntx = (g.nx + 1 + kFwdTile - 1) / kFwdTile;
    const int nty = (g.ny + 1 + kFwdTile - 1) / kFwdTile;
    const int nch = (nrows + kAngChunk - 1) / kAngChunk;
    dim3 grid(ntx * nty, nch, dN);
    fwd_tiled_kernel<<<grid, kThreads, 0, st>>>(img, acc, trig, g, sub, step, nrows, ntx);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_fwd_finalize(const KGeom &g, const float *meas, float *out, double *acc, int dN, int sub, int step,
                        int nrows, cudaStream_t st)
{
    if (nrows <= 0 || dN <= 0) return XCT_OK;
    dim3 g2((g.px + 127) / 128, nrows, dN);
    fwd_finalize_kernel<<<g2, 128, 0, st>>>(acc, meas, out, g, sub, step, nrows);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_bp_update_tiled(const KGeom &g, const float2 *trig, float *img, const float *ratio, int dN, int sub,
                           cudaStream_t st)
{
    if (dN <= 0) return XCT_OK;
    const int nang = (g.pa - sub + g.ss - 1) / g.ss;  // OSEM2's angle loop (OSEM.cl:93)
    const int ntx = (g.nx + kBpTile - 1) / kBpTile, nty = (g.ny + kBpTile - 1) / kBpTile;
    dim3 grid(ntx * nty, 1, dN);
    bp_tiled_kernel<<<grid, kThreads, 0, st>>>(img, ratio, trig, g, sub, nang, ntx, (float)g.ss, (float)g.pa);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}
