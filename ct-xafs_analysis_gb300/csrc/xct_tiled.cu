// xct_tiled.cu -- the optimised OS-EM kernels for sm_103a.
//
// Forward projector (OSEM1 / projection, OSEM.cl:38-68, reconstShare.cl:213-241),
// tile-stationary:
//   * one CTA owns an image tile: the samples whose base texel (floor(x), floor(y)) lies in
//     [x0, x0+T) x [y0, y0+T), with x0 = -1 + bx*T (base texel -1 still reaches texel 0).
//     It stages the tile ONCE per subset in shared memory as (t, t[x+1] - t) pairs, so
//     the x-lerp of a bilinear sample is one FMA and its 2x2 footprint is two 64-bit
//     loads, and serves every angle of its angle chunk from there;
//   * a warp takes one angle and 8 consecutive rays, 4 lanes per ray; the exact interval of
//     sample indices Y whose base texel lies in the tile (the coordinates are monotone in Y)
//     comes from four boundary searches, one per lane of the ray's group; the 4 lanes then
//     take every 4th sample of the interval, with packed f32x2 coordinate/floor/fraction
//     arithmetic, and their partial sums are combined with two shuffles;
//   * per-tile partial ray sums go into a double-precision accumulator with one atomic per
//     ray and tile.
// A finalize kernel turns the accumulator into the OSEM1 ratio (or the raw projection)
// and clears it for the next subset.
//
// Backprojector (OSEM2, OSEM.cl:71-105), footprint-staged:
//   * one CTA owns a 64x64 pixel tile; per angle it stages the window of ratio bins its
//     pixels hit (bin coordinates are monotone in X and in Y, so the tile corners bound the
//     window exactly) into shared memory with coalesced loads;
//   * each thread gathers 8 pixels (8 apart) of four rows (16 apart; 128 threads) or, for launches with
//     few tiles, of two rows (32 apart; 256 threads) per angle, in angle order, evaluating the
//     reference's bin expression ((Xc*c - Yc*s) + cx) + 0.5 -- the products Xc*c once for
//     all its rows, the rest with packed f32x2 instructions (each lane rounds exactly like the
//     scalar expression) and the nearest rule as a round-down add;
//   * the multiplicative update is fused.
#include <stdint.h>

#include <atomic>
#include <type_traits>

#include "xct_async.cuh"
#include "xct_check.cuh"
#include "xct_device.cuh"
#include "xct_f32x2.cuh"

namespace {

constexpr int kThreads = 256;
// forward projector: 12 warps per CTA so that 3 CTAs (3 x 69 KB of shared memory) give 36
// resident warps per SM to hide the shared-memory load latency
constexpr int kFwdThreads = 384;
constexpr int kFwdWarps = kFwdThreads / 32;
constexpr int kAngChunk = 128;  // most subset angles one forward-projector CTA serves

// A warp works on 8 consecutive rays of one angle with 4 lanes per ray, the 4 lanes taking
// every 4th sample (lane k: samples ya+k, ya+k+4, ...).  A half-warp then reads a compact
// 4x4 patch of footprints, and with an element pitch of 4 (mod 8) most such patches fall in
// distinct 64-bit bank pairs; 8 neighbouring rays also have similar lengths inside a tile,
// so few lanes idle.  (A CPU model of the access pattern: 0.232 shared wavefronts and 90 %
// active lanes per sample, against 0.293 and 73 % for one lane per ray with an odd pitch.)
// Tile side T (owned base texels per side) is a template parameter chosen per plan by the
// autotuner from {44, 60, 76, 92}; every candidate has an element pitch of T = 4 (mod 8).
template <int T>
struct FwdTile {
    static_assert(T % 8 == 4, "tile pitch must be 4 (mod 8)");
    static constexpr int P = T;         // element pitch
    static constexpr int Rows = T + 1;  // a base row r reads element rows r and r+1
    static constexpr size_t Smem = (size_t)P * Rows * sizeof(float2) + kAngChunk * sizeof(float2);
    // CTAs per SM: 4 (48 warps, <= 40 registers, no spills) where four tiles fit in the
    // 227 KB of shared memory (T <= 76), else 3 (56 registers)
    static constexpr int MinBlocks = Smem * 4 <= 227u * 1024u ? 4 : 3;
};
constexpr int kLanesPerRay = 4;
constexpr int kRaysPerWarp = 32 / kLanesPerRay;

constexpr int kBpTX = 64, kBpTY = 64;  // backprojection tile (pixels)
// A backprojector thread takes 8 pixels of R rows (kBpTY / R apart): R = 4 shares the
// products Xc*c over four rows (128 threads, 80 registers); R = 2 (256 threads, 64 registers)
// fills the SMs better when a launch has few tiles.
template <int R>
struct BpCfg {
    static constexpr int Threads = (kBpTX / 8) * (kBpTY / R);
    static constexpr int Stride = kBpTY / R;
};
constexpr int kBpW = 96;               // staged bins per angle (>= 63|c| + 63|s| + 3 = 92.1)
constexpr int kBpChunk = 64;           // angles per staging pass of the backprojector

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23

// ---------------------------------------------------------------------- ray intervals
__device__ __forceinline__ float ray_coord(int Y, float hd, float sl, float a)
{
    return fmaf((float)Y - hd, sl, a);
}

// First Y in [0, D] where the monotone predicate P holds (D if none), with the sentinels
// P(-1) = false, P(D) = true:  sl > 0: P(Y) = u(Y) >= b;  sl < 0: P(Y) = u(Y) < b,
// u(Y) = fma(Y - hd, sl, a).  The estimate from the real crossing point is checked with
// two exact evaluations; a binary search settles the rare cases it misses.
__device__ __noinline__ int first_true_search(float b, float a, float sl, float hd, int D)
{
    const bool up = sl > 0.0f;
    int lo = 0, hi = D;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const float u = ray_coord(mid, hd, sl, a);
        if (up ? (u >= b) : (u < b)) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

__device__ __forceinline__ int first_true(float b, float a, float sl, float inv_sl, float hd, int D)
{
    const bool up = sl > 0.0f;
    float e = fmaf(b - a, inv_sl, hd);
    e = fminf(fmaxf(e, -1.0f), (float)D + 1.0f);  // also maps +-inf; NaN -> -1
    int Y = (int)ceilf(e);
    Y = min(max(Y, 0), D);
    const float ul = ray_coord(Y - 1, hd, sl, a);
    const float uh = ray_coord(Y, hd, sl, a);
    const bool pl = (Y > 0) && (up ? (ul >= b) : (ul < b));
    const bool ph = (Y >= D) || (up ? (uh >= b) : (uh < b));
    if (!pl && ph) return Y;
    return first_true_search(b, a, sl, hd, D);
}

__device__ __forceinline__ void lds_f2(unsigned addr, float &a, float &b)
{
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(a), "=f"(b) : "r"(addr));
}
template <int P>
__device__ __forceinline__ void lds_f2_next_row(unsigned addr, float &a, float &b)
{
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2+%3];" : "=f"(a), "=f"(b) : "r"(addr), "n"(P * 8));
}
__device__ __forceinline__ float lds_f1(unsigned addr)
{
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

// ----------------------------------------------------------------- forward projector
// One bilinear sample at Yc (both halves of yc2): coordinates (fma(Yc,s,ax), fma(Yc,c,ay)),
// floor as a round-down add of 1.5*2^23 (the low mantissa bits), fraction = coordinate -
// floor, the footprint as two 64-bit loads of (t, t[x+1] - t), three FMA lerps.  [alo, ahi]:
// the byte addresses the first load may take (checked in the bounds-checked build only).
template <int P>
__device__ __forceinline__ float fwd_sample(f2x yc2, f2x sc, f2x axy, f2x MM, unsigned base2, unsigned alo,
                                            unsigned ahi)
{
    const f2x xy = f2_fma(yc2, sc, axy);
    const f2x tb = f2_add_rd(xy, MM);
    const f2x fr = f2_sub(xy, f2_sub(tb, MM));
    int ixb, iyb;
    f2_unpack_bits(tb, ixb, iyb);
    float fx, fy;
    f2_unpack(fr, fx, fy);
    const unsigned addr = (unsigned)iyb * (unsigned)(P * 8) + (unsigned)ixb * 8u + base2;
    if (!XCT_IN(addr, alo, ahi, XCT_SITE_FWD_TAP)) return 0.0f;
    float t00, d0, t01, d1;
    lds_f2(addr, t00, d0);
    lds_f2_next_row<P>(addr, t01, d1);
    const float r0 = fmaf(fx, d0, t00);
    const float r1 = fmaf(fx, d1, t01);
    return fmaf(fy, r1 - r0, r0);
}

// The work of one CTA: tile (bx, by) of one slice (image im, accumulator acc [nrows][px])
// for the subset angles k0 .. k0+chunk-1 (chunk <= kAngChunk).  Starts and ends with all
// threads in step.
template <int T>
__device__ __forceinline__ void fwd_tile(const KGeom &g, const float *__restrict__ im, double *__restrict__ acc,
                                         const float2 *__restrict__ trig, int sub, int step, int nrows, int bx,
                                         int by, int k0, int chunk, unsigned char *smem_raw)
{
    constexpr int kFwdT = T, kFwdP = FwdTile<T>::P, kFwdRows = FwdTile<T>::Rows;
    float2 *tile = reinterpret_cast<float2 *>(smem_raw);
    float2 *scs = reinterpret_cast<float2 *>(smem_raw + (size_t)kFwdP * kFwdRows * sizeof(float2));
    const int kn = min(chunk, nrows - k0);
    if (kn <= 0) return;
    const int x0 = -1 + bx * kFwdT, y0 = -1 + by * kFwdT;

    // element (c, r) = (t(x0+c, y0+r), t(x0+c+1, y0+r) - t(x0+c, y0+r)), zero border
    for (int i = threadIdx.x; i < kFwdT * kFwdRows; i += kFwdThreads) {
        const int r = i / kFwdT, c = i - r * kFwdT;
        const int gx = x0 + c, gy = y0 + r;
        float t0 = 0.0f, t1 = 0.0f;
        if ((unsigned)gy < (unsigned)g.ny) {
            const float *row = im + (size_t)gy * g.nx;
            if ((unsigned)gx < (unsigned)g.nx) t0 = __ldg(row + gx);
            if ((unsigned)(gx + 1) < (unsigned)g.nx) t1 = __ldg(row + gx + 1);
        }
        tile[r * kFwdP + c] = make_float2(t0, t1 - t0);
    }
    for (int k = threadIdx.x; k < kn; k += kFwdThreads) scs[k] = trig[sub + (k0 + k) * step];
    __syncthreads();

    // owned base-texel ranges (the union over tiles is [-1, n-1])
    const float xlo = (float)x0, xhi = (float)min(x0 + kFwdT, g.nx);
    const float ylo = (float)y0, yhi = (float)min(y0 + kFwdT, g.ny);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int D = g.depth;
    // shared address of element (col, row) from the floor bits (col + BIAS + x0, ...):
    // base2 + iy_bits * 8P + ix_bits * 8, with the biases folded into base2 (mod 2^32)
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(tile);
    const unsigned bias = (unsigned)XCT_FLOOR_BIAS;
    const unsigned base2 = sbase - (((bias + (unsigned)y0) * (unsigned)kFwdP + bias + (unsigned)x0) * 8u);
    const f2x MM = f2_pack(kMagic, kMagic);
    const f2x step2 = f2_pack((float)kLanesPerRay, (float)kLanesPerRay);
    // a footprint's first element may be any but the last row's (the second load reads the row below)
    const unsigned alo = sbase, ahi = sbase + (unsigned)((kFwdP * (kFwdRows - 1) - 1) * 8);
    const int ray = lane / kLanesPerRay;  // ray within the warp's 8
    const int ph = lane % kLanesPerRay;   // sample phase of this lane
    const int grp = lane & ~(kLanesPerRay - 1);
    // lane phase 0/1 bound the x coordinate, 2/3 the y coordinate (lower / upper Y limit)
    const bool bound_x = ph < 2;
    const bool upper = (ph & 1) != 0;

    for (int k = warp; k < kn; k += kFwdWarps) {
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
        const f2x sc = f2_pack(s, c);
        for (int base = Xlo; base <= Xhi; base += kRaysPerWarp) {
            const int X = base + ray;
            const bool live = X <= Xhi;
            const float Xc = (float)X - g.cx;
            const float ax = fmaf(Xc, c, g.hx);
            const float ay = fmaf(Xc, -s, g.hy);
            // the four interval limits of this ray, one per lane of its group: the lower (even
            // phase) or upper (odd phase) Y limit from the x (phase 0/1) or y (2/3) coordinate
            int v = 0;
            if (live) {
                const float a = bound_x ? ax : ay, sl = bound_x ? s : c, isl = bound_x ? inv_s : inv_c;
                const float lo = bound_x ? xlo : ylo, hi = bound_x ? xhi : yhi;
                if (sl != 0.0f) {
                    // sl > 0: [first(u >= lo), first(u >= hi)); sl < 0: [first(u < hi), first(u < lo))
                    const float b = ((sl > 0.0f) != upper) ? lo : hi;
                    v = first_true(b, a, sl, isl, g.hd, D);
                } else {  // constant coordinate: all samples or none
                    v = upper ? ((a >= lo && a < hi) ? D : 0) : 0;
                }
            }
            const int v0 = __shfl_sync(0xffffffffu, v, grp + 0), v1 = __shfl_sync(0xffffffffu, v, grp + 1);
            const int v2 = __shfl_sync(0xffffffffu, v, grp + 2), v3 = __shfl_sync(0xffffffffu, v, grp + 3);
            const int ya = max(v0, v2), yb = min(v1, v3);
            const int n = yb - ya > ph ? (yb - ya - ph + kLanesPerRay - 1) / kLanesPerRay : 0;
            const float yc0 = (float)(ya + ph) - g.hd;
            f2x yc2 = f2_pack(yc0, yc0);
            const f2x axy = f2_pack(ax, ay);
            // two samples per iteration into two accumulators (independent load/FMA chains)
            float sum = 0.0f, sum_b = 0.0f;
            int i = 0;
            for (; i + 1 < n; i += 2) {
                const f2x yb2 = f2_add(yc2, step2);
                sum += fwd_sample<kFwdP>(yc2, sc, axy, MM, base2, alo, ahi);
                sum_b += fwd_sample<kFwdP>(yb2, sc, axy, MM, base2, alo, ahi);
                yc2 = f2_add(yb2, step2);
            }
            if (i < n) sum += fwd_sample<kFwdP>(yc2, sc, axy, MM, base2, alo, ahi);
            sum += sum_b;
            // the ray's partial sum over this tile: the 4 phases, then one atomic
            sum += __shfl_xor_sync(0xffffffffu, sum, 1);
            sum += __shfl_xor_sync(0xffffffffu, sum, 2);
            if (ph == 0 && live && yb > ya &&
                XCT_IN((long long)(k0 + k) * g.px + X, 0, (long long)nrows * g.px - 1, XCT_SITE_FWD_ACC))
                atomicAdd(acc + (size_t)(k0 + k) * g.px + X, (double)sum);
        }
    }
}

// grid: (ntx*nty tiles, angle chunks, dN).  acc: [dN][nrows][px] doubles.
template <int T>
__global__ void __launch_bounds__(kFwdThreads, FwdTile<T>::MinBlocks) fwd_tiled_kernel(const float *__restrict__ img,
                                                                   double *__restrict__ acc,
                                                                   const float2 *__restrict__ trig, KGeom g, int sub,
                                                                   int step, int nrows, int ntx)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int z = blockIdx.z;
    fwd_tile<T>(g, img + (size_t)z * g.nx * g.ny, acc + (size_t)z * nrows * g.px, trig, sub, step, nrows,
                (int)blockIdx.x % ntx, (int)blockIdx.x / ntx, (int)blockIdx.y * g.fwd_chunk, g.fwd_chunk, smem_raw);
}

// ------------------------------------------- forward projector, eight slices per tile
// For a batch of slices of one geometry (the reference's dN image-array layers, OSEM1 over
// global size (px, pa/ss, dN)), eight slices share every sample position.  A CTA of 28 warps
// (the most whose registers fit one SM: 71 a thread; the tile fills shared memory, one CTA
// per SM; 28 warps hide the shared-memory latency better than 16: 2.08 against 2.24 ms per
// launch of 8 slices x 100 angles of 2048^2) owns a T x T tile of base texels of eight
// slices; shared memory holds, per base texel, one
// 16-byte element per slice -- (t00, t10 - t00, t01 - t00, (t11 - t01) - (t10 - t00)), the
// whole 2x2 footprint -- and a texel's eight elements are one 128-byte record.  A warp takes
// eight rays of one angle, a quarter-warp (eight lanes) per pair of consecutive rays: lanes
// 0-3 of the quarter walk the first ray's samples in the tile, lanes 4-7 the second's, lane j
// of a ray taking its samples j, j + 4, ...  For each sample a lane finds the coordinates,
// floor and record once and then reads the eight slices' elements starting at slot p (its
// lane in the quarter) and wrapping, so at every load the quarter's eight lanes read eight
// different 16-byte bank groups: no load has a bank conflict whatever the geometry, the
// coordinate work is spread over eight slice-samples, and a quarter whose rays are done
// costs no shared-memory wavefronts.  The bilinear value of one slice,
// t00 + fy dy + fx (dx + fy dxy), is two packed-pair FMAs: (t00, dx) + fy (dy, dxy), then
// added into the slot's pair of partial sums with weights (1, fx).  Slot r of lane p
// accumulates slice (r + p) mod 8; eight shuffles give lane p the quarter's totals for slice
// p of both rays, which it adds to the double accumulator with one atomic per ray.  Work
// items (angle, eight rays) are taken from a shared counter, so warps finish within one item
// of each other.
constexpr int kMsSlices = 8;
constexpr int kMsThreads = 896;
constexpr int kMsRays = 2 * 32 / kMsSlices;  // rays per warp (a pair per quarter-warp)
constexpr int kMsLanesPerRay = kMsSlices / 2;
constexpr int kMsTile = 42;              // base texels per tile side: 42^2 x 128 B = 221 KB
constexpr int kMsStageRows = 6;          // element rows per staging strip

template <int T>
struct FwdMsTile {
    static constexpr size_t TileBytes = (size_t)T * T * kMsSlices * sizeof(float4);
    // per chunk angle: (c, s), (1/c, 1/s), first and last ray, ray-group prefix; then the
    // group total and the work counter
    static constexpr size_t Smem = TileBytes + (size_t)kAngChunk * (2 * sizeof(float2) + 3 * sizeof(int)) + 16;
    static_assert(Smem <= 227u * 1024u, "eight-slice tile exceeds shared memory");
};

// float -> double for the accumulator without the FP64 pipe (GB300 runs FP64 at a small
// fraction of the FP32 rate): normal numbers and zero by re-biasing the exponent in integer
// arithmetic, the rare others through the conversion instruction.
__device__ __forceinline__ double f32_to_f64(float v)
{
    const unsigned u = __float_as_uint(v);
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u < 254u) {
        const unsigned hi = (u & 0x80000000u) | ((e + (1023u - 127u)) << 20) | ((u >> 3) & 0xfffffu);
        return __hiloint2double((int)hi, (int)(u << 29));
    }
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)v;
}

// One slice element (t00, dx | dy, dxy) of a record as two packed pairs.
__device__ __forceinline__ void lds_2f2(unsigned addr, f2x &lo, f2x &hi)
{
    asm volatile("ld.shared.v2.b64 {%0, %1}, [%2];" : "=l"(lo), "=l"(hi) : "r"(addr));
}

// The eight slices' elements of the record at byte address rec, slot r from offset off[r],
// added to the slots' partial sums: part[r] += (1, fx) * ((t00, dx) + fy * (dy, dxy)).
__device__ __forceinline__ void ms_tap(unsigned rec, const unsigned (&off)[kMsSlices], unsigned alo, unsigned ahi,
                                       float fx, float fy, f2x (&part)[kMsSlices])
{
    if (!XCT_IN(rec, alo, ahi, XCT_SITE_FWD_MS_TAP)) return;
    f2x lo[kMsSlices], hi[kMsSlices];
#pragma unroll
    for (int r = 0; r < kMsSlices; ++r) lds_2f2(rec + off[r], lo[r], hi[r]);
    const f2x fy2 = f2_pack(fy, fy), wx = f2_pack(1.0f, fx);
#pragma unroll
    for (int r = 0; r < kMsSlices; ++r) part[r] = f2_fma(wx, f2_fma(fy2, hi[r], lo[r]), part[r]);
}

// grid: (ntx*nty tiles, angle chunks, dN / 8 slice groups); acc [dN][nrows][px] doubles.
template <int T>
__global__ void __launch_bounds__(kMsThreads, 1) fwd_ms_kernel(const float *__restrict__ img,
                                                               double *__restrict__ acc,
                                                               const float2 *__restrict__ trig, KGeom g, int sub,
                                                               int step, int nrows, int ntx, int chunk)
{
    // 128-byte records, read with 128-bit loads
    extern __shared__ __align__(128) unsigned char ms_smem[];
    float4 *tile = reinterpret_cast<float4 *>(ms_smem);
    float2 *scs = reinterpret_cast<float2 *>(ms_smem + FwdMsTile<T>::TileBytes);
    float2 *inv_s = scs + kAngChunk;
    int *xlo_s = reinterpret_cast<int *>(inv_s + kAngChunk);
    int *xhi_s = xlo_s + kAngChunk;
    int *gpre = xhi_s + kAngChunk;
    int *tail = gpre + kAngChunk;  // [0] ray groups of the chunk, [1] work counter
    const int k0 = (int)blockIdx.y * chunk;
    const int kn = min(chunk, nrows - k0);
    if (kn <= 0) return;
    const int bx = (int)blockIdx.x % ntx, by = (int)blockIdx.x / ntx;
    const int x0 = -1 + bx * T, y0 = -1 + by * T;
    const int z0 = (int)blockIdx.z * kMsSlices;
    const size_t nimg = (size_t)g.nx * g.ny;
    const float *im0 = img + (size_t)z0 * nimg;

    // element (c, r) of slice z at tile[(r*T + c)*8 + z]; texels outside the image are 0.
    // A warp stages a strip of four columns x eight slices (lane 8*cl + z: column 4u + cl of
    // slice z) over kMsStageRows element rows, walking down the texel rows: each texel is
    // loaded once, its right neighbour comes from the next column's lane (the strip's last
    // column loads it), and the quarter-warps store whole records (no bank conflict).
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int cl = lane >> 3, z = lane & (kMsSlices - 1);
        const float *im = im0 + (size_t)z * nimg;
        constexpr int kStrips = (T + 3) / 4, kBands = (T + kMsStageRows - 1) / kMsStageRows;
        for (int u = warp; u < kStrips * kBands; u += kMsThreads / 32) {
            const int c = (u % kStrips) * 4 + cl, r0 = (u / kStrips) * kMsStageRows;
            const int gx = x0 + c;
            const bool c0 = (unsigned)gx < (unsigned)g.nx, c1 = (unsigned)(gx + 1) < (unsigned)g.nx;
            float tp = 0.0f, trp = 0.0f;
#pragma unroll
            for (int j = 0; j <= kMsStageRows; ++j) {
                const int r = r0 + j, gy = y0 + r;
                const bool rv = (unsigned)gy < (unsigned)g.ny && r <= T;
                const long long o = (long long)gy * g.nx + gx;
                const float t = (rv && c0) ? __ldg(im + o) : 0.0f;
                float tr = __shfl_down_sync(0xffffffffu, t, 8);
                if (cl == 3) tr = (rv && c1) ? __ldg(im + o + 1) : 0.0f;
                if (j > 0 && c < T && r - 1 < T) {
                    const float d0 = trp - tp, d1 = tr - t;
                    tile[((r - 1) * T + c) * kMsSlices + z] = make_float4(tp, d0, t - tp, d1 - d0);
                }
                tp = t;
                trp = tr;
            }
        }
    }
    // owned base-texel ranges (the union over tiles is [-1, n-1])
    const float xlo = (float)x0, xhi = (float)min(x0 + T, g.nx);
    const float ylo = (float)y0, yhi = (float)min(y0 + T, g.ny);
    for (int k = threadIdx.x; k < kn; k += kMsThreads) {
        const float2 cs = trig[sub + (k0 + k) * step];
        scs[k] = cs;
        inv_s[k] = make_float2(1.0f / cs.x, 1.0f / cs.y);
        // rays that can reach the tile: the (expanded) tile corners on the detector axis
        float pmin = 3.0e38f, pmax = -3.0e38f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float px_ = (q & 1) ? xhi + 2.0f : xlo - 2.0f;
            const float py_ = (q & 2) ? yhi + 2.0f : ylo - 2.0f;
            const float p = (px_ - g.hx) * cs.x - (py_ - g.hy) * cs.y + g.cx;
            pmin = fminf(pmin, p);
            pmax = fmaxf(pmax, p);
        }
        xlo_s[k] = max(0, (int)floorf(pmin) - 1);
        xhi_s[k] = min(g.px - 1, (int)ceilf(pmax) + 1);
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive prefix of the ray groups per angle (warp 0)
        const int lane = threadIdx.x;
        int carry = 0;
        for (int b = 0; b < kn; b += 32) {
            const int k = b + lane;
            const int n = k < kn ? max(0, (xhi_s[k] - xlo_s[k] + kMsRays) / kMsRays) : 0;
            int v = n;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += t;
            }
            if (k < kn) gpre[k] = carry + v - n;
            carry += __shfl_sync(0xffffffffu, v, 31);
        }
        if (lane == 0) {
            tail[0] = carry;
            tail[1] = 0;
        }
    }
    __syncthreads();

    const int total = tail[0];
    const int lane = threadIdx.x & 31;
    const int ph = lane & (kMsSlices - 1);    // lane of the quarter; also this lane's first slot
    const int qb = lane & ~(kMsSlices - 1);   // first lane of the quarter
    const int pair = lane >> 3;               // ray pair of the warp's four
    const int half = ph / kMsLanesPerRay;     // 0: the pair's first ray, 1: its second
    const int jr = ph % kMsLanesPerRay;       // this lane's phase in its ray's samples
    const int D = g.depth;
    // byte address of the record of base texel (col, row) from the floor bits:
    // (iy_bits * T + ix_bits) * 128 + base2, the biases folded into base2 (mod 2^32)
    const unsigned sbase = (unsigned)__cvta_generic_to_shared(tile);
    const unsigned bias = (unsigned)XCT_FLOOR_BIAS;
    const unsigned base2 =
        sbase - ((bias + (unsigned)y0) * (unsigned)T + bias + (unsigned)x0) * (unsigned)(kMsSlices * 16);
    const unsigned alo = sbase, ahi = sbase + (unsigned)((T * T - 1) * kMsSlices * 16);
    // slot r of this lane holds slice (r + ph) mod 8, read at byte offset 16 * that
    unsigned off[kMsSlices];
#pragma unroll
    for (int r = 0; r < kMsSlices; ++r) off[r] = 16u * (unsigned)((r + ph) & (kMsSlices - 1));
    const f2x MM = f2_pack(kMagic, kMagic);
    // the four lanes of a ray find its four interval limits: the lower (even jr) or upper
    // (odd jr) Y limit from the x (jr < 2) or the y coordinate
    const bool bound_x = jr < 2;
    const bool upper = (jr & 1) != 0;
    int *counter = tail + 1;
    int k = 0;  // the warp's current angle: items only grow, so the search runs forward

    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        while (k + 1 < kn && gpre[k + 1] <= item) ++k;  // the last k with gpre[k] <= item
        const float c = scs[k].x, s = scs[k].y;
        // the quarter's two consecutive rays XA and XA + 1; this lane's ray X
        const int XA = xlo_s[k] + (item - gpre[k]) * kMsRays + 2 * pair;
        const int X = XA + half;
        const float Xc = (float)X - g.cx;
        const float ax = fmaf(Xc, c, g.hx);
        const float ay = fmaf(Xc, -s, g.hy);
        int v = 0;
        if (X <= xhi_s[k]) {
            const float a = bound_x ? ax : ay, sl = bound_x ? s : c;
            const float isl = bound_x ? inv_s[k].y : inv_s[k].x;
            const float lo_ = bound_x ? xlo : ylo, hi_ = bound_x ? xhi : yhi;
            if (sl != 0.0f) {
                // sl > 0: [first(u >= lo), first(u >= hi)); sl < 0: [first(u < hi), first(u < lo))
                const float b = ((sl > 0.0f) != upper) ? lo_ : hi_;
                v = first_true(b, a, sl, isl, g.hd, D);
            } else {  // constant coordinate: all samples or none
                v = upper ? ((a >= lo_ && a < hi_) ? D : 0) : 0;
            }
        }
        // the ray's limits: lower ones (even jr) max-combined, upper ones min-combined across
        // the x and y limits (xor 2), then exchanged within the pair of lanes (xor 1)
        const int w = __shfl_xor_sync(0xffffffffu, v, 2);
        const int m = upper ? min(v, w) : max(v, w);
        const int u = __shfl_xor_sync(0xffffffffu, m, 1);
        const int ya = upper ? u : m, yb = upper ? m : u;
        const int L = max(yb - ya, 0);
        const int Lo = __shfl_xor_sync(0xffffffffu, L, kMsLanesPerRay);  // the other ray's
        // samples ya + jr, ya + jr + 4, ... of this lane's ray; Yc = Y - hd is tracked as a
        // float (exact small integers)
        const int n = L > jr ? (L - jr + kMsLanesPerRay - 1) / kMsLanesPerRay : 0;
        float yc = (float)(ya + jr) - g.hd;
        const f2x sc = f2_pack(s, c);
        const f2x axy = f2_pack(ax, ay);
        f2x part[kMsSlices];
#pragma unroll
        for (int r = 0; r < kMsSlices; ++r) part[r] = 0ull;
        for (int i = 0; i < n; ++i, yc += (float)kMsLanesPerRay) {
            const f2x xy = f2_fma(f2_pack(yc, yc), sc, axy);
            const f2x tb = f2_add_rd(xy, MM);
            const f2x fr = f2_sub(xy, f2_sub(tb, MM));
            int ixb, iyb;
            float fx, fy;
            f2_unpack_bits(tb, ixb, iyb);
            f2_unpack(fr, fx, fy);
            ms_tap(((unsigned)iyb * (unsigned)T + (unsigned)ixb) * (unsigned)(kMsSlices * 16) + base2, off, alo, ahi,
                   fx, fy, part);
        }
        // lane p gathers slice p's partial sums from lanes (p - d) mod 8 of its quarter, slot
        // d: lanes 0-3 hold the first ray's, lanes 4-7 the second's
        float tot0 = 0.0f, tot1 = 0.0f;
#pragma unroll
        for (int d = 0; d < kMsSlices; ++d) {
            const int sp = (ph - d) & (kMsSlices - 1);
            float plo, phi;
            f2_unpack(part[d], plo, phi);
            const float pv = __shfl_sync(0xffffffffu, plo + phi, qb + sp);
            if (sp < kMsLanesPerRay) tot0 += pv;
            else tot1 += pv;
        }
        const int L0 = half ? Lo : L, L1 = half ? L : Lo;
        double *accz = acc + ((size_t)(z0 + ph) * nrows + k0 + k) * g.px;
        if (L0 > 0 && XCT_IN((long long)k * g.px + XA, 0, (long long)(nrows - k0) * g.px - 1, XCT_SITE_FWD_ACC))
            atomicAdd(accz + XA, f32_to_f64(tot0));
        if (L1 > 0 && XCT_IN((long long)k * g.px + XA + 1, 0, (long long)(nrows - k0) * g.px - 1, XCT_SITE_FWD_ACC))
            atomicAdd(accz + XA + 1, f32_to_f64(tot1));
    }
}

// ------------------------------------------------------------------- exact adjoint
// A^T of the forward projector: img[t] = sum over samples of w_t(sample) * sino[th][X], with
// the bilinear weights w00 = (1-fx)(1-fy), w10 = fx(1-fy), w01 = (1-fx)fy, w11 = fx fy of the
// sample's 2x2 footprint.  A CTA owns a T x T texel tile; it visits every sample whose base
// texel lies in [x0-1, x0+T) x [y0-1, y0+T) (exactly those whose footprint touches the
// tile), scatters its four weighted values into a shared (T+2)^2 accumulator with shared
// atomics (fixed-point integers per window of angles, below), and writes its own T x T
// texels once -- no global atomics, no overlap between tiles.  grid: (ntx*nty tiles, 1, dN).
// tile side: 64, or 32 when a launch of 64-texel tiles would leave fewer than three CTAs per
// SM (one slice of 1024^2 makes only 256 tiles of 64)
constexpr int kAdjT = 64, kAdjTSmall = 32;
constexpr int kAdjWarps = kThreads / 32;  // one angle per warp and window

// Accumulation: the warps take one angle each per window of kAdjWarps angles; within a window
// the contributions are scattered as 32-bit fixed-point integers (shared-memory integer atomics
// run ~6x the rate of float ones on this GPU), with a power-of-two scale chosen from the
// window's largest |ray value| vmax: every contribution is at most vmax * scale <= 2^22, so
// it converts to an integer with one add of 1.5*2^23 (its low bits hold the rounded value --
// no conversion instruction), and no texel can overflow: it receives at most six taps per
// angle (the half-open 2x2 cell around it holds at most five samples of the rotated unit
// lattice, one more allowed for coordinate rounding), 48 * 2^22 < 2^28 per window.  After the
// window every thread adds its texels' integers, unscaled, to the float total in window order
// -- so the result does not depend on the order of the atomics -- and clears them.  One
// integer unit is at most 2^-21 of vmax, each contribution rounds by at most 2^-22 of it; only
// rays with |value| >= vmax * 2^-6 take the integer path (so each of their contributions
// rounds by at most 2^-16 of the ray's value, below the weight error of float32 sample
// coordinates), smaller ones -- and every ray of a window with a non-finite value or one above
// 1e30 -- scatter float atomics, which keep full relative precision.
// The angles are th = sub + k*step for k < nang (all: 0, 1, pa); with base non-null the
// output is base + scale * (A^T sino) (a gradient step).
template <int T>
__global__ void __launch_bounds__(kThreads) adj_tiled_kernel(const float *__restrict__ sino,
                                                             float *__restrict__ img,
                                                             const float2 *__restrict__ trig, KGeom g, int ntx,
                                                             int sub, int step, int nang,
                                                             const float *__restrict__ base, float scale)
{
    constexpr int kAdjT = T, kAdjP = T + 2;  // this launch's tile side and pitch
    __shared__ float accs[kAdjP * kAdjP];
    __shared__ int acci[kAdjP * kAdjP];
    __shared__ float wmax[kAdjWarps];
    const int bx = blockIdx.x % ntx, by = blockIdx.x / ntx;
    const int z = blockIdx.z;
    const int x0 = bx * kAdjT, y0 = by * kAdjT;  // owned texels [x0, x0+T) x [y0, y0+T)
    for (int i = threadIdx.x; i < kAdjP * kAdjP; i += kThreads) {
        accs[i] = 0.0f;
        acci[i] = 0;
    }
    __syncthreads();
    const float *sn = sino + (size_t)z * g.pa * g.px;
    // base texels whose footprint touches the tile
    const float xlo = (float)(x0 - 1), xhi = (float)min(x0 + kAdjT, g.nx);
    const float ylo = (float)(y0 - 1), yhi = (float)min(y0 + kAdjT, g.ny);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int D = g.depth;
    for (int w0 = 0; w0 < nang; w0 += kAdjWarps) {
        const bool active = w0 + warp < nang;
        const int th = active ? sub + (w0 + warp) * step : 0;
        float c = 1.0f, s = 0.0f;
        int Xlo = 0, Xhi = -1;
        if (active) {
            const float2 cs = trig[th];
            c = cs.x;
            s = cs.y;
            float pmin = 3.0e38f, pmax = -3.0e38f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float px_ = (q & 1) ? xhi + 2.0f : xlo - 2.0f;
                const float py_ = (q & 2) ? yhi + 2.0f : ylo - 2.0f;
                const float p = (px_ - g.hx) * c - (py_ - g.hy) * s + g.cx;
                pmin = fminf(pmin, p);
                pmax = fmaxf(pmax, p);
            }
            Xlo = max(0, (int)floorf(pmin) - 1);
            Xhi = min(g.px - 1, (int)ceilf(pmax) + 1);
        }
        // the window's largest |ray value| (NaN and inf make it non-finite)
        float m = 0.0f;
        for (int X = Xlo + lane; X <= Xhi; X += 32) {
            const float v = fabsf(__ldg(sn + (size_t)th * g.px + X));
            m = (v == v && m == m) ? fmaxf(m, v) : __int_as_float(0x7fc00000);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float t = __shfl_xor_sync(0xffffffffu, m, o);
            m = (t == t && m == m) ? fmaxf(m, t) : __int_as_float(0x7fc00000);
        }
        if (lane == 0) wmax[warp] = m;
        __syncthreads();
        float vmax = 0.0f;
#pragma unroll
        for (int k = 0; k < kAdjWarps; ++k) {
            const float t = wmax[k];
            vmax = (t == t && vmax == vmax) ? fmaxf(vmax, t) : __int_as_float(0x7fc00000);
        }
        // false for NaN and inf, and for finite windows above 1e30: those scatter float atomics
        const bool fixed = vmax < 1.0e30f;
        // scale = 2^(22 - e) with vmax < 2^e: every contribution is below 2^22 in magnitude
        float scale = 0.0f, inv = 0.0f;
        if (fixed && vmax > 0.0f) {
            int e;
            frexpf(vmax, &e);  // vmax < 2^e
            e = max(e, -78);   // keep the scale <= 2^100 (a finite float)
            scale = ldexpf(1.0f, 22 - e);
            inv = ldexpf(1.0f, e - 22);
        }
        if (active && (!fixed || vmax > 0.0f)) {
            // the forward projector's lane mapping: 8 consecutive rays, 4 lanes per ray taking
            // every 4th sample of the ray's interval in the tile, whose four limits come from
            // one boundary search per lane -- the same samples the forward visits
            const float inv_s = 1.0f / s, inv_c = 1.0f / c;
            const int ray = lane / kLanesPerRay, ph = lane % kLanesPerRay, grp = lane & ~(kLanesPerRay - 1);
            const bool bound_x = ph < 2, upper = (ph & 1) != 0;
            for (int base = Xlo; base <= Xhi; base += kRaysPerWarp) {
                const int X = base + ray;
                const bool live = X <= Xhi;
                const float v = live ? __ldg(sn + (size_t)th * g.px + X) : 0.0f;
                const float Xc = (float)X - g.cx;
                const float ax = fmaf(Xc, c, g.hx);
                const float ay = fmaf(Xc, -s, g.hy);
                int lim = 0;
                if (live) {
                    const float a = bound_x ? ax : ay, sl = bound_x ? s : c, isl = bound_x ? inv_s : inv_c;
                    const float lo = bound_x ? xlo : ylo, hi = bound_x ? xhi : yhi;
                    if (sl != 0.0f) {
                        const float bnd = ((sl > 0.0f) != upper) ? lo : hi;
                        lim = first_true(bnd, a, sl, isl, g.hd, D);
                    } else {
                        lim = upper ? ((a >= lo && a < hi) ? D : 0) : 0;
                    }
                }
                const int l0 = __shfl_sync(0xffffffffu, lim, grp + 0), l1 = __shfl_sync(0xffffffffu, lim, grp + 1);
                const int l2 = __shfl_sync(0xffffffffu, lim, grp + 2), l3 = __shfl_sync(0xffffffffu, lim, grp + 3);
                const int ya = max(l0, l2);
                const int yb = (live && v != 0.0f) ? min(l1, l3) : ya;  // a zero ray contributes nothing
                const float vs = v * scale;
                const bool as_int = fixed && fabsf(v) >= vmax * 0.015625f;  // |v| >= vmax * 2^-6
                for (int Y = ya + ph; Y < yb; Y += kLanesPerRay) {
                    const float Yc = (float)Y - g.hd;
                    const float x = fmaf(Yc, s, ax), y = fmaf(Yc, c, ay);
                    const float fi = floorf(x), fj = floorf(y);
                    const float fx = x - fi, fy = y - fj;
                    const int col = (int)fi - (x0 - 1), row = (int)fj - (y0 - 1);
                    const float gx = 1.0f - fx, gy = 1.0f - fy;
                    if (!XCT_IN(row * kAdjP + col, 0, kAdjP * kAdjP - kAdjP - 2, XCT_SITE_ADJ)) continue;
                    const int o = row * kAdjP + col;
                    if (as_int) {
                        // round(x) for |x| < 2^22: the low bits of x + 1.5*2^23
                        const float p0 = vs * gy, p1 = vs * fy;
                        atomicAdd(acci + o, __float_as_int(gx * p0 + kMagic) - 0x4B400000);
                        atomicAdd(acci + o + 1, __float_as_int(fx * p0 + kMagic) - 0x4B400000);
                        atomicAdd(acci + o + kAdjP, __float_as_int(gx * p1 + kMagic) - 0x4B400000);
                        atomicAdd(acci + o + kAdjP + 1, __float_as_int(fx * p1 + kMagic) - 0x4B400000);
                    } else {
                        atomicAdd(accs + o, gx * gy * v);
                        atomicAdd(accs + o + 1, fx * gy * v);
                        atomicAdd(accs + o + kAdjP, gx * fy * v);
                        atomicAdd(accs + o + kAdjP + 1, fx * fy * v);
                    }
                }
            }
        }
        __syncthreads();
        if (fixed && vmax > 0.0f) {
            for (int i = threadIdx.x; i < kAdjP * kAdjP; i += kThreads) {
                const int q = acci[i];
                if (q != 0) {
                    accs[i] += (float)q * inv;
                    acci[i] = 0;
                }
            }
        }
        __syncthreads();  // the integers are clear and wmax may be rewritten
    }
    float *im = img + (size_t)z * g.nx * g.ny;
    const float *bz = base ? base + (size_t)z * g.nx * g.ny : nullptr;
    for (int i = threadIdx.x; i < kAdjT * kAdjT; i += kThreads) {
        const int r = i / kAdjT, cc = i - r * kAdjT;
        const int X = x0 + cc, Y = y0 + r;
        if (X < g.nx && Y < g.ny) {
            const float a = accs[(r + 1) * kAdjP + cc + 1];
            const size_t o = (size_t)Y * g.nx + X;
            im[o] = bz ? fmaf(scale, a, __ldg(bz + o)) : a;
        }
    }
}

// The exact adjoint over S slices of one geometry at once: adj_tiled_kernel's samples,
// windows, fixed-point scales (one per slice and window) and epilogue, with each sample's
// coordinates, weights and accumulator offset found once for the S slices.  Tile 32 texels;
// the (T+2)^2 accumulators of a slice are kept at a pitch of 37 (a CPU model of the 32 lanes'
// footprints over all angles gives 2.0 bank wavefronts per atomic instruction at this pitch,
// 3.0 at pitch 34).  grid: (ntx*nty tiles, 1, dN / S slice groups); dynamic shared memory
// AdjMs<S>::Smem.
constexpr int kAdjMsT = 32, kAdjMsP = 37, kAdjMsR = kAdjMsT + 2;
constexpr int kAdjMsSlices = 4;  // slices per adjoint group
constexpr int kAdjMsN = kAdjMsR * kAdjMsP;  // accumulator entries per slice
template <int S>
struct AdjMs {
    static constexpr size_t Smem = (size_t)S * kAdjMsN * (sizeof(float) + sizeof(int)) + kAdjWarps * S * sizeof(float);
};

template <int S>
__global__ void __launch_bounds__(kThreads) adj_ms_kernel(const float *__restrict__ sino, float *__restrict__ img,
                                                          const float2 *__restrict__ trig, KGeom g, int ntx, int sub,
                                                          int step, int nang, const float *__restrict__ base,
                                                          float scale_out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *accs = reinterpret_cast<float *>(smem_raw);
    int *acci = reinterpret_cast<int *>(accs + S * kAdjMsN);
    float *wmax = reinterpret_cast<float *>(acci + S * kAdjMsN);
    const int bx = (int)blockIdx.x % ntx, by = (int)blockIdx.x / ntx;
    const int z0 = (int)blockIdx.z * S;
    const size_t nprj = (size_t)g.pa * g.px, nimg = (size_t)g.nx * g.ny;
    const int x0 = bx * kAdjMsT, y0 = by * kAdjMsT;  // owned texels [x0, x0+T) x [y0, y0+T)
    for (int i = threadIdx.x; i < S * kAdjMsN; i += kThreads) {
        accs[i] = 0.0f;
        acci[i] = 0;
    }
    __syncthreads();
    const float *sn = sino + (size_t)z0 * nprj;
    // base texels whose footprint touches the tile
    const float xlo = (float)(x0 - 1), xhi = (float)min(x0 + kAdjMsT, g.nx);
    const float ylo = (float)(y0 - 1), yhi = (float)min(y0 + kAdjMsT, g.ny);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int D = g.depth;
    for (int w0 = 0; w0 < nang; w0 += kAdjWarps) {
        const bool active = w0 + warp < nang;
        const int th = active ? sub + (w0 + warp) * step : 0;
        float c = 1.0f, s = 0.0f;
        int Xlo = 0, Xhi = -1;
        if (active) {
            const float2 cs = trig[th];
            c = cs.x;
            s = cs.y;
            float pmin = 3.0e38f, pmax = -3.0e38f;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float px_ = (q & 1) ? xhi + 2.0f : xlo - 2.0f;
                const float py_ = (q & 2) ? yhi + 2.0f : ylo - 2.0f;
                const float p = (px_ - g.hx) * c - (py_ - g.hy) * s + g.cx;
                pmin = fminf(pmin, p);
                pmax = fmaxf(pmax, p);
            }
            Xlo = max(0, (int)floorf(pmin) - 1);
            Xhi = min(g.px - 1, (int)ceilf(pmax) + 1);
        }
        const float *row = sn + (size_t)th * g.px;
        // each slice's largest |ray value| over the window (NaN and inf make it non-finite)
        float m[S];
#pragma unroll
        for (int z = 0; z < S; ++z) m[z] = 0.0f;
        for (int X = Xlo + lane; X <= Xhi; X += 32) {
#pragma unroll
            for (int z = 0; z < S; ++z) {
                const float v = fabsf(__ldg(row + (size_t)z * nprj + X));
                m[z] = (v == v && m[z] == m[z]) ? fmaxf(m[z], v) : __int_as_float(0x7fc00000);
            }
        }
#pragma unroll
        for (int z = 0; z < S; ++z) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float t = __shfl_xor_sync(0xffffffffu, m[z], o);
                m[z] = (t == t && m[z] == m[z]) ? fmaxf(m[z], t) : __int_as_float(0x7fc00000);
            }
        }
        if (lane == 0) {
#pragma unroll
            for (int z = 0; z < S; ++z) wmax[warp * S + z] = m[z];
        }
        __syncthreads();
        float vmax[S], sc[S], inv[S];
        unsigned fixed = 0;  // bit z: slice z's window takes the fixed-point path
#pragma unroll
        for (int z = 0; z < S; ++z) {
            float vm = 0.0f;
#pragma unroll
            for (int k = 0; k < kAdjWarps; ++k) {
                const float t = wmax[k * S + z];
                vm = (t == t && vm == vm) ? fmaxf(vm, t) : __int_as_float(0x7fc00000);
            }
            vmax[z] = vm;
            sc[z] = 0.0f;
            inv[z] = 0.0f;
            // false for NaN and inf, and for finite windows above 1e30: those scatter float atomics
            if (vm < 1.0e30f && vm > 0.0f) {
                int e;
                frexpf(vm, &e);  // vmax < 2^e
                e = max(e, -78);  // keep the scale <= 2^100 (a finite float)
                sc[z] = ldexpf(1.0f, 22 - e);
                inv[z] = ldexpf(1.0f, e - 22);
                fixed |= 1u << z;
            }
        }
        if (active) {
            // the forward projector's lane mapping: 8 consecutive rays, 4 lanes per ray
            const float inv_s = 1.0f / s, inv_c = 1.0f / c;
            const int ray = lane / kLanesPerRay, ph = lane % kLanesPerRay, grp = lane & ~(kLanesPerRay - 1);
            const bool bound_x = ph < 2, upper = (ph & 1) != 0;
            for (int b0 = Xlo; b0 <= Xhi; b0 += kRaysPerWarp) {
                const int X = b0 + ray;
                const bool live = X <= Xhi;
                float v[S];
                bool any = false;
#pragma unroll
                for (int z = 0; z < S; ++z) {
                    v[z] = live ? __ldg(row + (size_t)z * nprj + X) : 0.0f;
                    any |= v[z] != 0.0f;
                }
                const float Xc = (float)X - g.cx;
                const float ax = fmaf(Xc, c, g.hx);
                const float ay = fmaf(Xc, -s, g.hy);
                int lim = 0;
                if (live) {
                    const float a = bound_x ? ax : ay, sl = bound_x ? s : c, isl = bound_x ? inv_s : inv_c;
                    const float lo = bound_x ? xlo : ylo, hi = bound_x ? xhi : yhi;
                    if (sl != 0.0f) {
                        const float bnd = ((sl > 0.0f) != upper) ? lo : hi;
                        lim = first_true(bnd, a, sl, isl, g.hd, D);
                    } else {
                        lim = upper ? ((a >= lo && a < hi) ? D : 0) : 0;
                    }
                }
                const int l0 = __shfl_sync(0xffffffffu, lim, grp + 0), l1 = __shfl_sync(0xffffffffu, lim, grp + 1);
                const int l2 = __shfl_sync(0xffffffffu, lim, grp + 2), l3 = __shfl_sync(0xffffffffu, lim, grp + 3);
                const int ya = max(l0, l2);
                const int yb = (live && any) ? min(l1, l3) : ya;  // a ray zero in every slice adds nothing
                float vs[S];
                unsigned as_int = 0;  // bit z: |v| >= vmax * 2^-6 in a fixed-point window
#pragma unroll
                for (int z = 0; z < S; ++z) {
                    vs[z] = v[z] * sc[z];
                    if (((fixed >> z) & 1u) && fabsf(v[z]) >= vmax[z] * 0.015625f) as_int |= 1u << z;
                }
                for (int Y = ya + ph; Y < yb; Y += kLanesPerRay) {
                    const float Yc = (float)Y - g.hd;
                    const float x = fmaf(Yc, s, ax), y = fmaf(Yc, c, ay);
                    const float fi = floorf(x), fj = floorf(y);
                    const float fx = x - fi, fy = y - fj;
                    const int col = (int)fi - (x0 - 1), rr = (int)fj - (y0 - 1);
                    const float gx = 1.0f - fx, gy = 1.0f - fy;
                    if (!XCT_IN(rr * kAdjMsP + col, 0, (kAdjMsR - 2) * kAdjMsP + kAdjMsR - 2, XCT_SITE_ADJ)) continue;
                    const int o = rr * kAdjMsP + col;
#pragma unroll
                    for (int z = 0; z < S; ++z) {
                        int *ai = acci + z * kAdjMsN + o;
                        float *af = accs + z * kAdjMsN + o;
                        if ((as_int >> z) & 1u) {
                            // round(x) for |x| < 2^22: the low bits of x + 1.5*2^23
                            const float p0 = vs[z] * gy, p1 = vs[z] * fy;
                            atomicAdd(ai, __float_as_int(gx * p0 + kMagic) - 0x4B400000);
                            atomicAdd(ai + 1, __float_as_int(fx * p0 + kMagic) - 0x4B400000);
                            atomicAdd(ai + kAdjMsP, __float_as_int(gx * p1 + kMagic) - 0x4B400000);
                            atomicAdd(ai + kAdjMsP + 1, __float_as_int(fx * p1 + kMagic) - 0x4B400000);
                        } else if (v[z] != 0.0f) {
                            atomicAdd(af, gx * gy * v[z]);
                            atomicAdd(af + 1, fx * gy * v[z]);
                            atomicAdd(af + kAdjMsP, gx * fy * v[z]);
                            atomicAdd(af + kAdjMsP + 1, fx * fy * v[z]);
                        }
                    }
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int z = 0; z < S; ++z) {
            if ((fixed >> z) & 1u) {
                for (int i = threadIdx.x; i < kAdjMsN; i += kThreads) {
                    const int q = acci[z * kAdjMsN + i];
                    if (q != 0) {
                        accs[z * kAdjMsN + i] += (float)q * inv[z];
                        acci[z * kAdjMsN + i] = 0;
                    }
                }
            }
        }
        __syncthreads();  // the integers are clear and wmax may be rewritten
    }
    for (int z = 0; z < S; ++z) {
        float *im = img + (size_t)(z0 + z) * nimg;
        const float *bz = base ? base + (size_t)(z0 + z) * nimg : nullptr;
        for (int i = threadIdx.x; i < kAdjMsT * kAdjMsT; i += kThreads) {
            const int r = i / kAdjMsT, cc = i - r * kAdjMsT;
            const int X = x0 + cc, Y = y0 + r;
            if (X < g.nx && Y < g.ny) {
                const float a = accs[z * kAdjMsN + (r + 1) * kAdjMsP + cc + 1];
                const size_t o = (size_t)Y * g.nx + X;
                im[o] = bz ? fmaf(scale_out, a, __ldg(bz + o)) : a;
            }
        }
    }
}

// The exact adjoint over eight or ten slices as a gather, without atomics.  Every sample (ray X,
// index Y) of the forward projector has one base texel (floor of its coordinates); its value
// v goes to that base texel's four footprint texels with the weights gx gy, fx gy, gx fy,
// fx fy.  A thread owns one base texel (i, j) and keeps four accumulators per slice -- the
// parts its samples give to (i, j), (i+1, j), (i, j+1), (i+1, j+1) -- so each sample is
// handled by exactly one thread.  Per angle the thread finds its samples: a half-open unit
// square holds at most two points of the rotated unit sample lattice, which lie on the at
// most two rays whose lattice coordinate is within 0.717 of the square's centre, each at
// most two sample indices within 0.717 of the centre's projection on the ray; each of those
// four candidates is evaluated with the forward projector's own arithmetic (fma
// coordinates, round-down floor) and kept when its base texel is (i, j), the ray is on the
// detector and the index within [0, D).  A CTA owns 32 x BY base texels (BY = 16 for eight
// slices, 20 for ten) and writes the 31 x (BY - 1) texels whose four base texels it holds,
// texel (i, j) = A00(i, j) + A10(i-1, j) + A01(i, j-1) + A11(i-1, j-1), after staging the
// four parts in shared memory.
// The rays' values of 16 angles at a time are staged by asynchronous copies into one of two
// windows: the next chunk's copies run while this chunk is accumulated.  Most squares hold
// one sample per angle, about 9 % two and 9 % none, so a warp whose lanes each added all
// their samples at once would run two accumulation passes at almost every angle; with ten
// slices a second sample instead waits in a four-slot queue per thread in shared memory
// (window address and fractions) and the queues are emptied at the end of the chunk -- about
// 1.2 passes per angle instead of 1.8.  Float sums in a fixed order given by the geometry:
// deterministic, and no fixed-point rounding.
constexpr int kAdjGBX = 32;                          // base texels per CTA row
constexpr int kAdjGW = 44;  // staged rays per angle (a 32 x 20 block needs at most 43)
constexpr int kAdjGChunk = 16;                       // angles per staging pass
template <int S>
struct AdjG {
    // base texel rows per CTA (one thread per base texel): 16 at two CTAs per SM (eight
    // slices, 64 registers), 20 at one (ten slices, 94 registers)
    static constexpr int BY = S <= 8 ? 16 : 20;
    static constexpr int Threads = kAdjGBX * BY;
    static constexpr unsigned QStride = 16u * Threads;  // bytes between a queue's slots
    // two windows: [slice pair][angle][ray] of float2, then the queues: [slot][thread] of
    // (window address, fx, fy); later the parts: [corner][slice][thread]; three slots of
    // (cos, sin) and first staged ray per angle
    static constexpr unsigned PairBytes = (unsigned)(kAdjGChunk * kAdjGW * 8);
    static constexpr unsigned WinBytes = (unsigned)(S / 2) * PairBytes;
    static constexpr size_t CombBytes = (size_t)4 * S * Threads * 4;
    // queued samples per thread: four where the registers allow (one CTA per SM); none at
    // two CTAs per SM, whose 64 registers a thread would then exceed
    static constexpr int Queue = S > 8 ? 4 : 0;
    static constexpr size_t QueueBytes = (size_t)Queue * QStride;
    static constexpr size_t SlotBytes = (size_t)3 * kAdjGChunk * 12;
    static constexpr size_t Front = 2 * (size_t)WinBytes + QueueBytes;
    static constexpr size_t Smem = (Front > CombBytes ? Front : CombBytes) + SlotBytes;
};

__device__ __forceinline__ f2x lds_f2x(unsigned addr)
{
    f2x v;
    asm volatile("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
    return v;
}

// A queued sample: window address and fractions (fx, fy) in one 16-byte slot.
__device__ __forceinline__ void sts_q(unsigned addr, unsigned ad, f2x fr)
{
    asm volatile("{ .reg .b32 lo, hi; mov.b64 {lo, hi}, %2; st.shared.v4.b32 [%0], {%1, lo, hi, %1}; }"
                 :: "r"(addr), "r"(ad), "l"(fr) : "memory");
}
__device__ __forceinline__ void lds_q(unsigned addr, unsigned &ad, f2x &fr)
{
    asm volatile("{ .reg .b32 lo, hi, pad; ld.shared.v4.b32 {%0, lo, hi, pad}, [%2]; mov.b64 %1, {lo, hi}; }"
                 : "=r"(ad), "=l"(fr) : "r"(addr) : "memory");
}

// S (even) slices per CTA; the library launches S = 8 and S = 10 (one CTA per SM).
template <int S>
__global__ void __launch_bounds__(AdjG<S>::Threads, S <= 8 ? 2 : 1) adj_gather_kernel(const float *__restrict__ sino,
                                                                     float *__restrict__ img,
                                                                     const float2 *__restrict__ trig, KGeom g,
                                                                     int ntx, int sub, int step, int nang,
                                                                     const float *__restrict__ base, float scale_out)
{
    constexpr int P = S / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *part = reinterpret_cast<float *>(smem_raw);  // the window, later the parts
    float2 *scs = reinterpret_cast<float2 *>(smem_raw + AdjG<S>::Smem - AdjG<S>::SlotBytes);
    int *sxw = reinterpret_cast<int *>(scs + 3 * kAdjGChunk);
    const int tx = threadIdx.x % kAdjGBX, ty = threadIdx.x / kAdjGBX;
    const int bx = (int)blockIdx.x % ntx, by = (int)blockIdx.x / ntx;
    const int z0 = (int)blockIdx.z * S;
    const size_t nprj = (size_t)g.pa * g.px, nimg = (size_t)g.nx * g.ny;
    const float *sz = sino + (size_t)z0 * nprj;
    // base texels [bi0, bi0 + 32) x [bj0, bj0 + 16); output texels from bi0 + 1, bj0 + 1
    const int bi0 = bx * (kAdjGBX - 1) - 1, bj0 = by * (AdjG<S>::BY - 1) - 1;
    const int i = bi0 + tx, j = bj0 + ty;
    const int ibits = i + XCT_FLOOR_BIAS, jbits = j + XCT_FLOOR_BIAS;
    const float ci = (float)i + 0.5f, cj = (float)j + 0.5f;  // the square's centre
    const float di = ci - g.hx, dj = cj - g.hy;
    const int D = g.depth;
    const unsigned wbase = (unsigned)__cvta_generic_to_shared(part);
    const f2x MM = f2_pack(kMagic, kMagic), one2 = f2_pack(1.0f, 1.0f);
    const f2x hxy = f2_pack(g.hx, g.hy);
    f2x acc[4][P];  // [corner 00, 10, 01, 11][slice pair]
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int h = 0; h < P; ++h) acc[q][h] = 0ull;

    // one sample: fractions (fx, fy) of its base texel, window byte address ad of its ray;
    // the four bilinear weights (gx gy, fx gy, gx fy, fx fy) times the slices' ray values
    const f2x bxy = f2_pack(__int_as_float(ibits) - kMagic, __int_as_float(jbits) - kMagic);
    auto add = [&](unsigned ad, f2x fr, unsigned wb) {
        const f2x gr = f2_sub(one2, fr);
        float fx, fy, gx, gy;
        f2_unpack(fr, fx, fy);
        f2_unpack(gr, gx, gy);
        const float w[4] = {gx * gy, fx * gy, gx * fy, fx * fy};
        if (!XCT_IN(ad, wb, wb + AdjG<S>::WinBytes - 8, XCT_SITE_ADJ)) return;
        f2x v[P];
#pragma unroll
        for (int h = 0; h < P; ++h) v[h] = lds_f2x(ad + (unsigned)h * AdjG<S>::PairBytes);
#pragma unroll
        for (int cq = 0; cq < 4; ++cq) {
            const f2x ww = f2_pack(w[cq], w[cq]);
#pragma unroll
            for (int h = 0; h < P; ++h) acc[cq][h] = f2_fma(ww, v[h], acc[cq][h]);
        }
    };
    // this thread's queue of samples left for the end of the chunk: slot i at qb + i * stride
    const unsigned qb = wbase + 2u * AdjG<S>::WinBytes + 16u * threadIdx.x;
    int qn = 0;

    // Software pipeline over chunks of 16 angles: the rays of chunk ch + 1 are copied into the
    // other window while chunk ch is accumulated; the angles' (cos, sin) and first staged ray
    // sit in three slots (chunks ch, ch + 1, ch + 2), the (cos, sin) of chunk ch + 3 in the
    // registers of threads 0..15.
    const int nch = (nang + kAdjGChunk - 1) / kAdjGChunk;
    auto trig_of = [&](int ch) -> float2 {
        const int a = ch * kAdjGChunk + (int)threadIdx.x;
        return (ch < nch && (int)threadIdx.x < kAdjGChunk && a < nang) ? __ldg(trig + sub + a * step)
                                                                        : make_float2(0.0f, 0.0f);
    };
    auto prep = [&](int ch, float2 cs) {
        if (ch >= nch || (int)threadIdx.x >= kAdjGChunk) return;
        const int at = (ch % 3) * kAdjGChunk + (int)threadIdx.x;
        scs[at] = cs;
        // rays whose lattice coordinate meets the block's base squares
        float umin = 3.0e38f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float px_ = (float)(bi0 + ((q & 1) ? kAdjGBX : 0)) - g.hx;
            const float py_ = (float)(bj0 + ((q & 2) ? AdjG<S>::BY : 0)) - g.hy;
            umin = fminf(umin, px_ * cs.x - py_ * cs.y + g.cx);
        }
        sxw[at] = (int)floorf(umin) - 2;
    };
    // window (pair p, angle k, ray sxw + r) = (slice 2p, slice 2p + 1), 0 off the detector
    auto stage = [&](int ch) {
        if (ch >= nch) return;
        const int k0 = ch * kAdjGChunk, kn = min(kAdjGChunk, nang - k0), sl = (ch % 3) * kAdjGChunk;
        const unsigned wb = wbase + (unsigned)(ch & 1) * AdjG<S>::WinBytes;
        for (int e = threadIdx.x; e < kn * S * kAdjGW; e += AdjG<S>::Threads) {
            const int r = e % kAdjGW, t2 = e / kAdjGW;
            const int z = t2 % S, k = t2 / S;
            const int X = sxw[sl + k] + r;
            const float *row = sz + (size_t)z * nprj + (size_t)(sub + (k0 + k) * step) * g.px;
            const bool in = (unsigned)X < (unsigned)g.px;
            const unsigned dst = wb + (unsigned)(z >> 1) * AdjG<S>::PairBytes + 8u * (unsigned)(k * kAdjGW + r) +
                                 4u * (unsigned)(z & 1);
            cp_async4(dst, in ? (const void *)(row + X) : (const void *)row, in ? 4u : 0u);
        }
    };
    prep(0, trig_of(0));
    prep(1, trig_of(1));
    float2 csr = trig_of(2);
    __syncthreads();
    stage(0);
    for (int ch = 0; ch < nch; ++ch) {
        // this chunk's copies have landed; every thread is past chunk ch - 1, whose window
        // and slot are reused below
        cp_async_wait_all();
        __syncthreads();
        prep(ch + 2, csr);
        csr = trig_of(ch + 3);
        stage(ch + 1);
        const int k0 = ch * kAdjGChunk, kn = min(kAdjGChunk, nang - k0), sl = (ch % 3) * kAdjGChunk;
        const unsigned wb = wbase + (unsigned)(ch & 1) * AdjG<S>::WinBytes;
        for (int k = 0; k < kn; ++k) {
            const float c = scs[sl + k].x, s = scs[sl + k].y;
            const f2x cs2 = f2_pack(c, -s), sc2 = f2_pack(s, c);
            const unsigned wk = wb + 8u * (unsigned)(k * kAdjGW - sxw[sl + k]);
            // the candidates: rays Xa, Xa + 1 (lattice coordinate of the cell centre u0 - 0.717
            // and up); on each, indices Ya, Ya + 1 (the centre's coordinate along the rays, w0,
            // is the same on every ray)
            const float u0 = fmaf(di, c, fmaf(-dj, s, g.cx));
            const float w0 = fmaf(di, s, dj * c) + g.hd;
            const int Xa = (xct_floor_bits(u0 - 0.717f) - XCT_FLOOR_BIAS) + 1;
            const int Ya = (xct_floor_bits(w0 - 0.717f) - XCT_FLOOR_BIAS) + 1;
            // Y - hd is exact (hd is a multiple of 0.5), so the second index is the first + 1
            const float Yc0 = (float)Ya - g.hd;
            const f2x yy[2] = {f2_pack(Yc0, Yc0), f2_pack(Yc0 + 1.0f, Yc0 + 1.0f)};
            const bool yin[2] = {(unsigned)Ya < (unsigned)D, (unsigned)(Ya + 1) < (unsigned)D};
            f2x cxy[4];
            unsigned valid = 0;
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const int X = Xa + a;
                const float Xc = (float)X - g.cx;
                const f2x axy = f2_fma(f2_pack(Xc, Xc), cs2, hxy);  // (ax, ay) as the forward
                const bool xin = (unsigned)X < (unsigned)g.px;
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    const f2x xy = f2_fma(yy[b], sc2, axy);  // (x, y) as the forward
                    int xb, yb;
                    f2_unpack_bits(f2_add_rd(xy, MM), xb, yb);
                    const int q = 2 * a + b;
                    cxy[q] = xy;
                    if (xb == ibits && yb == jbits && xin && yin[b]) valid |= 1u << q;
                }
            }
            // a unit square holds at most two samples.  The first is added now; a second one
            // (and, never seen but kept for float-rounded coordinates at the square's corners,
            // any further) waits in the queue, or is added now when the queue is full
            unsigned now = valid & (0u - valid), rest = valid ^ now;
            while (rest != 0 && qn < AdjG<S>::Queue) {
                const int q = __ffs(rest) - 1;
                rest &= rest - 1;
                const f2x xy = q == 1 ? cxy[1] : q == 2 ? cxy[2] : cxy[3];
                const int X = Xa + (q >> 1);
                sts_q(qb + (unsigned)qn * AdjG<S>::QStride, wk + 8u * (unsigned)X, f2_sub(xy, bxy));
                ++qn;
            }
            now |= rest;
            while (now != 0) {
                const int q = __ffs(now) - 1;
                now &= now - 1;
                const f2x xy = q == 0 ? cxy[0] : q == 1 ? cxy[1] : q == 2 ? cxy[2] : cxy[3];
                const int X = Xa + (q >> 1);
                add(wk + 8u * (unsigned)X, f2_sub(xy, bxy), wb);
            }
        }
        // the queued samples, while this chunk's window is still in place
        for (int i = 0; i < qn; ++i) {
            unsigned ad;
            f2x fr;
            lds_q(qb + (unsigned)i * AdjG<S>::QStride, ad, fr);
            add(ad, fr, wb);
        }
        qn = 0;
    }
    // the parts: part[corner][slice][thread]
    __syncthreads();
#pragma unroll
    for (int cq = 0; cq < 4; ++cq)
#pragma unroll
        for (int h = 0; h < P; ++h) {
            float a0, a1;
            f2_unpack(acc[cq][h], a0, a1);
            part[(cq * S + 2 * h) * AdjG<S>::Threads + threadIdx.x] = a0;
            part[(cq * S + 2 * h + 1) * AdjG<S>::Threads + threadIdx.x] = a1;
        }
    __syncthreads();
    if (tx == 0 || ty == 0 || i >= g.nx || j >= g.ny) return;
    const int t = threadIdx.x;
#pragma unroll
    for (int z = 0; z < S; ++z) {
        const float a = part[(0 * S + z) * AdjG<S>::Threads + t] + part[(1 * S + z) * AdjG<S>::Threads + t - 1] +
                        part[(2 * S + z) * AdjG<S>::Threads + t - kAdjGBX] +
                        part[(3 * S + z) * AdjG<S>::Threads + t - kAdjGBX - 1];
        const size_t o = (size_t)(z0 + z) * nimg + (size_t)j * g.nx + i;
        img[o] = base ? fmaf(scale_out, a, __ldg(base + o)) : a;
    }
}

// Launch of adj_gather_kernel<S> over `groups` groups of S slices (its shared memory opted in
// once per device).
template <int S>
static int launch_adj_gather(const KGeom &g, const float2 *trig, const float *sino, float *img, int groups, int sub,
                             int step, int nang, const float *base, float scale, cudaStream_t st)
{
    static std::atomic<bool> done[64];
    int dev = 0;
    XCT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return xct_fail(XCT_E_INVALID, "device index out of range");
    if (!done[dev].load(std::memory_order_acquire)) {
        XCT_CUDA_TRY(cudaFuncSetAttribute((const void *)adj_gather_kernel<S>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AdjG<S>::Smem));
        done[dev].store(true, std::memory_order_release);
    }
    const int ntx = (g.nx + kAdjGBX - 2) / (kAdjGBX - 1), nty = (g.ny + AdjG<S>::BY - 2) / (AdjG<S>::BY - 1);
    adj_gather_kernel<S><<<dim3(ntx * nty, 1, groups), AdjG<S>::Threads, AdjG<S>::Smem, st>>>(sino, img, trig, g, ntx, sub,
                                                                                         step, nang, base, scale);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
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

// The same for 4 consecutive bins per thread (px % 4 == 0, exact measured fetch, 16-byte
// aligned sinograms): float4 / double2 accesses, each bin's arithmetic unchanged.
__global__ void __launch_bounds__(256) fwd_finalize4_kernel(double *__restrict__ acc, const float *__restrict__ meas,
                                                            float *__restrict__ out, KGeom g, int sub, int step,
                                                            int nrows)
{
    const int X = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
    const int k = blockIdx.y, z = blockIdx.z;
    if (X >= g.px) return;
    double2 *a = reinterpret_cast<double2 *>(acc + ((size_t)z * nrows + k) * g.px + X);
    const double2 a0 = a[0], a1 = a[1];
    a[0] = make_double2(0.0, 0.0);
    a[1] = make_double2(0.0, 0.0);
    const float p0 = (float)a0.x, p1 = (float)a0.y, p2 = (float)a1.x, p3 = (float)a1.y;
    const int th = sub + k * step;
    const size_t o = ((size_t)z * g.pa + th) * g.px + X;
    float4 r;
    if (meas != nullptr) {
        const float4 y = __ldg(reinterpret_cast<const float4 *>(meas + o));
        r = make_float4(xct_ratio(y.x, p0), xct_ratio(y.y, p1), xct_ratio(y.z, p2), xct_ratio(y.w, p3));
    } else {
        r = make_float4(p0, p1, p2, p3);
    }
    *reinterpret_cast<float4 *>(out + o) = r;
}

// ------------------------------------------------------------------- backprojector
struct BpShared {
    float win[kBpChunk * kBpW];
    float2 scs[kBpChunk];     // (c, s)
    int slo[kBpChunk];        // first staged bin of the angle's window
    unsigned soff[kBpChunk];  // byte address of window entry (bits - BIAS - lo)
};

// The work of one CTA: pixel tile (bx, by) of one slice (image img, ratio rt [pa][px]),
// angles th = sub + k*ss for k < nang (as OSEM2 loops).  Starts/ends with threads in step.
template <int kBpRows>
__device__ __forceinline__ void bp_tile(const KGeom &g, float *__restrict__ img, const float *__restrict__ rt,
                                        const float2 *__restrict__ trig, int sub, int nang, int bx, int by,
                                        float ssf, float paf, BpShared &sh)
{
    float *win = sh.win;
    float2 *scs = sh.scs;
    int *slo = sh.slo;
    unsigned *soff = sh.soff;
    const int X0 = bx * kBpTX, Y0 = by * kBpTY;
    const int X1 = min(X0 + kBpTX, g.nx) - 1, Y1 = min(Y0 + kBpTY, g.ny) - 1;
    // 8 threads x 8 pixels across, thread tx taking X0 + tx + 8i (the 8 lanes of a row read
    // neighbouring bins and write neighbouring pixels); thread row ty covers rows
    // ty + r * (kBpTY / kBpRows)
    constexpr int kStride = BpCfg<kBpRows>::Stride, kBpThreads = BpCfg<kBpRows>::Threads;
    const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;
    // threads past the image edge of a partial tile gather for the edge pixel (inside the
    // staged window) and write nothing
    float Ycr[kBpRows];
#pragma unroll
    for (int r = 0; r < kBpRows; ++r) Ycr[r] = (float)min(Y0 + ty + r * kStride, Y1) - g.hy;
    f2x xcp[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float a = (float)min(X0 + tx + 16 * j, X1) - g.hx;
        const float b = (float)min(X0 + tx + 16 * j + 8, X1) - g.hx;
        xcp[j] = f2_pack(a, b);
    }
    f2x acc[kBpRows][4];  // pixel pairs of each row, packed adds (each lane an IEEE add)
#pragma unroll
    for (int r = 0; r < kBpRows; ++r)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[r][j] = f2_pack(0.0f, 0.0f);
    const f2x cxp = f2_pack(g.cx, g.cx);
    const f2x hp = f2_pack(0.5f, 0.5f);
    const f2x MM = f2_pack(kMagic, kMagic);
    const unsigned wbase = (unsigned)__cvta_generic_to_shared(win);

    for (int k0 = 0; k0 < nang; k0 += kBpChunk) {
        const int kn = min(kBpChunk, nang - k0);
        __syncthreads();  // the previous chunk's gathers are done with the shared arrays
        for (int k = threadIdx.x; k < kn; k += kBpThreads) {
            const float2 cs = trig[sub + (k0 + k) * g.ss];
            scs[k] = cs;
            // the bin coordinate is monotone in X and in Y: the corners bound the window
            const float xa = (float)X0 - g.hx, xb = (float)X1 - g.hx;
            const float yA = (float)Y0 - g.hy, yB = (float)Y1 - g.hy;
            const float qa = yA * cs.y, qb = yB * cs.y;
            int lo = xct_floor_bits(xct_bin_coord(xa, cs.x, qa, g.cx));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qa, g.cx)));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xa, cs.x, qb, g.cx)));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qb, g.cx)));
            slo[k] = lo - XCT_FLOOR_BIAS;
            // entry for floor bits fb: wbase + 4*(k*W + fb - lo)  (mod 2^32)
            soff[k] = wbase + 4u * (unsigned)(k * kBpW) - 4u * (unsigned)lo;
        }
        __syncthreads();
        // element j of angle k holds ratio[th][lo_k + j] (0 off the detector)
        for (int i = threadIdx.x; i < kn * kBpW; i += kBpThreads) {
            const int k = i / kBpW, j = i - k * kBpW;
            const int bin = slo[k] + j;
            const int th = sub + (k0 + k) * g.ss;
            win[i] = ((unsigned)bin < (unsigned)g.px) ? __ldg(rt + (size_t)th * g.px + bin) : 0.0f;
        }
        __syncthreads();
        const unsigned wlo = wbase, whi = wbase + 4u * (unsigned)(kn * kBpW - 1);
        (void)wlo;
        (void)whi;
        for (int k = 0; k < kn; ++k) {
            const float c = scs[k].x, s = scs[k].y;
            const unsigned off = soff[k];
            float q[kBpRows];
#pragma unroll
            for (int r = 0; r < kBpRows; ++r) q[r] = Ycr[r] * s;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                // Xc*c - q in scalar: ptxas contracts a packed multiply feeding a packed
                // subtract into one fused operation whatever the rounding modifiers, and the
                // reference rounds the product and the difference separately.  The products
                // serve every row; the three additions that follow are packed:
                // ((.) + cx) + 0.5, then floor.
                float xa, xb;
                f2_unpack(xcp[j], xa, xb);
                const float pa_ = xa * c, pb_ = xb * c;
#pragma unroll
                for (int r = 0; r < kBpRows; ++r) {
                    const f2x t = f2_add_rd(f2_add(f2_add(f2_pack(pa_ - q[r], pb_ - q[r]), cxp), hp), MM);
                    int b0, b1;
                    f2_unpack_bits(t, b0, b1);
                    const unsigned ad0 = (unsigned)b0 * 4u + off, ad1 = (unsigned)b1 * 4u + off;
                    const float v0 = XCT_IN(ad0, wlo, whi, XCT_SITE_BP_WIN) ? lds_f1(ad0) : 0.0f;
                    const float v1 = XCT_IN(ad1, wlo, whi, XCT_SITE_BP_WIN) ? lds_f1(ad1) : 0.0f;
                    acc[r][j] = f2_add(acc[r][j], f2_pack(v0, v1));
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kBpRows; ++r) {
        const int Y = Y0 + ty + r * kStride;
        if (Y > Y1) continue;
        float *row = img + (size_t)Y * g.nx;
        float v[8];
#pragma unroll
        for (int j = 0; j < 4; ++j) f2_unpack(acc[r][j], v[2 * j], v[2 * j + 1]);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int X = X0 + tx + 8 * i;
            if (X <= X1) row[X] = xct_update(row[X], v[i], ssf, paf);
        }
    }
    __syncthreads();  // the shared arrays may be restaged by the caller's next tile
}

// grid: (ntx*nty tiles, 1, dN).
template <int R>
__global__ void __launch_bounds__(BpCfg<R>::Threads) bp_tiled_kernel(float *__restrict__ img,
                                                            const float *__restrict__ ratio,
                                                            const float2 *__restrict__ trig, KGeom g, int sub,
                                                            int nang, int ntx, float ssf, float paf)
{
    __shared__ BpShared sh;
    const int z = blockIdx.z;
    bp_tile<R>(g, img + (size_t)z * g.nx * g.ny, ratio + (size_t)z * g.pa * g.px, trig, sub, nang,
            (int)blockIdx.x % ntx, (int)blockIdx.x / ntx, ssf, paf, sh);
}

// --------------------------------------------- backprojector, eight slices per tile
// For the slices of one OS-EM call (one geometry) a (pixel, angle) pair reads the same bin in
// all eight slices of a group, so the bin expression is evaluated once for eight gathers.  A
// CTA of 256 threads owns a 32 x 32 pixel tile of eight slices and stages, per angle and
// slice, the window of the tile's bins (< 48, bounded exactly by the tile corners as in
// bp_tiled_kernel, its start rounded down to a multiple of 4) with asynchronous 16-byte copies
// (zero-filled off the detector), 24 angles at a time.  A thread takes 4 pixels of one row (8
// apart), a warp 8 adjacent pixels in each of 4 rows: the bins one load instruction touches
// span fewer than 32 consecutive words, so no load has a bank conflict.  Per pixel and angle:
// the literal bin expression of bp_tiled_kernel, one address, eight 4-byte loads at constant
// offsets (one per slice), four packed adds -- in angle order, so each slice's sum is
// bp_tiled_kernel's bit for bit -- and the update at the end.
constexpr int kBpMsT = 32;
constexpr int kBpMsThreads = 256;
constexpr int kBpMsW = 52;      // staged bins per angle and slice (>= 31|c| + 31|s| + 3 + 3 = 49.9)
constexpr int kBpMsChunk = 24;  // angles per staging pass
constexpr int kBpMsPix = 4;     // pixels per thread, 8 apart
constexpr unsigned kBpMsSliceBytes = (unsigned)(kBpMsChunk * kBpMsW * 4);  // one slice's windows

template <int S>
struct BpMsShared {
    float win[S * kBpMsChunk * kBpMsW];          // [slice][angle][bin]
    float2 scs[kBpMsChunk];                      // (c, s)
    int slo[kBpMsChunk];                         // first staged bin (a multiple of 4)
    unsigned soff[kBpMsChunk];                   // byte address of slice 0's entry (bits - BIAS - lo)
};

// grid: (ntx*nty tiles of 32 x 32, 1, dN / S slice groups), S = 8 or 2.  vec: 16-byte staging
// copies (px a multiple of 4 and a 16-byte aligned ratio array).
template <int S>
__global__ void __launch_bounds__(kBpMsThreads) bp_ms_kernel(float *__restrict__ img, const float *__restrict__ ratio,
                                                             const float2 *__restrict__ trig, KGeom g, int sub,
                                                             int nang, int ntx, float ssf, float paf, int vec)
{
    __shared__ __align__(16) BpMsShared<S> sh;
    const int bx = (int)blockIdx.x % ntx, by = (int)blockIdx.x / ntx;
    const int z0 = (int)blockIdx.z * S;
    const size_t nimg = (size_t)g.nx * g.ny, nprj = (size_t)g.pa * g.px;
    const float *rz = ratio + (size_t)z0 * nprj;
    const int X0 = bx * kBpMsT, Y0 = by * kBpMsT;
    const int X1 = min(X0 + kBpMsT, g.nx) - 1, Y1 = min(Y0 + kBpMsT, g.ny) - 1;
    const int t = threadIdx.x;
    const int tx = t & 7, ty = t >> 3;
    // pixel i of this thread: (X0 + tx + 8i, Y0 + ty); threads past the image edge of a partial
    // tile gather for the edge pixel (inside the staged window) and write nothing
    const float Yc = (float)min(Y0 + ty, Y1) - g.hy;
    float xc[kBpMsPix];
#pragma unroll
    for (int i = 0; i < kBpMsPix; ++i) xc[i] = (float)min(X0 + tx + 8 * i, X1) - g.hx;
    f2x acc[kBpMsPix][S / 2];  // slice pairs of each pixel
#pragma unroll
    for (int i = 0; i < kBpMsPix; ++i)
#pragma unroll
        for (int h = 0; h < S / 2; ++h) acc[i][h] = 0ull;
    const f2x cxp = f2_pack(g.cx, g.cx);
    const f2x hp = f2_pack(0.5f, 0.5f);
    const f2x MM = f2_pack(kMagic, kMagic);
    const unsigned wbase = (unsigned)__cvta_generic_to_shared(sh.win);

    for (int k0 = 0; k0 < nang; k0 += kBpMsChunk) {
        const int kn = min(kBpMsChunk, nang - k0);
        __syncthreads();  // the previous chunk's gathers are done with the shared arrays
        for (int k = t; k < kn; k += kBpMsThreads) {
            const float2 cs = trig[sub + (k0 + k) * g.ss];
            sh.scs[k] = cs;
            // the bin coordinate is monotone in X and in Y: the corners bound the window
            const float xa = (float)X0 - g.hx, xb = (float)X1 - g.hx;
            const float yA = (float)Y0 - g.hy, yB = (float)Y1 - g.hy;
            const float qa = yA * cs.y, qb = yB * cs.y;
            int lo = xct_floor_bits(xct_bin_coord(xa, cs.x, qa, g.cx));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qa, g.cx)));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xa, cs.x, qb, g.cx)));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qb, g.cx)));
            lo &= ~3;  // the bias is a multiple of 4: this rounds the bin down to one
            sh.slo[k] = lo - XCT_FLOOR_BIAS;
            // slice 0's entry for floor bits fb: wbase + 4*(k*W + fb - lo)  (mod 2^32)
            sh.soff[k] = wbase + 4u * (unsigned)(k * kBpMsW) - 4u * (unsigned)lo;
        }
        __syncthreads();
        // window (z, k) = ratio[z0 + z][th_k][lo_k .. lo_k + W), 0 off the detector
        if (vec) {
            constexpr int kQ = kBpMsW / 4;
            for (int i = t; i < kn * S * kQ; i += kBpMsThreads) {
                const int q = i % kQ, r = i / kQ;
                const int z = r % S, k = r / S;
                const int bin = sh.slo[k] + 4 * q;
                const int th = sub + (k0 + k) * g.ss;
                const float *row = rz + (size_t)z * nprj + (size_t)th * g.px;
                const int nb = bin < 0 ? 0 : min(4, g.px - bin);
                const unsigned dst = wbase + (unsigned)z * kBpMsSliceBytes + 4u * (unsigned)(k * kBpMsW + 4 * q);
                cp_async16(dst, nb > 0 ? (const void *)(row + bin) : (const void *)row, nb > 0 ? 4u * (unsigned)nb : 0u);
            }
        } else {
            for (int i = t; i < kn * S * kBpMsW; i += kBpMsThreads) {
                const int j = i % kBpMsW, r = i / kBpMsW;
                const int z = r % S, k = r / S;
                const int bin = sh.slo[k] + j;
                const int th = sub + (k0 + k) * g.ss;
                const float *row = rz + (size_t)z * nprj + (size_t)th * g.px;
                const bool in = (unsigned)bin < (unsigned)g.px;
                const unsigned dst = wbase + (unsigned)z * kBpMsSliceBytes + 4u * (unsigned)(k * kBpMsW + j);
                cp_async4(dst, in ? (const void *)(row + bin) : (const void *)row, in ? 4u : 0u);
            }
        }
        cp_async_wait_all();
        __syncthreads();
        const unsigned wlo = wbase, whi = wbase + 4u * (unsigned)(kn * kBpMsW - 1);
        (void)wlo;
        (void)whi;
        for (int k = 0; k < kn; ++k) {
            const float c = sh.scs[k].x, s = sh.scs[k].y;
            const unsigned off = sh.soff[k];
            const float q = Yc * s;
#pragma unroll
            for (int j = 0; j < kBpMsPix / 2; ++j) {
                // the literal bin expression of bp_tiled_kernel for pixels 2j and 2j+1
                const float pa_ = xc[2 * j] * c, pb_ = xc[2 * j + 1] * c;
                const f2x tt = f2_add_rd(f2_add(f2_add(f2_pack(pa_ - q, pb_ - q), cxp), hp), MM);
                int b0, b1;
                f2_unpack_bits(tt, b0, b1);
                const unsigned ad[2] = {(unsigned)b0 * 4u + off, (unsigned)b1 * 4u + off};
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    float v[S];
                    if (XCT_IN(ad[u], wlo, whi, XCT_SITE_BP_WIN)) {
                        v[0] = lds_f1_at<0 * kBpMsSliceBytes>(ad[u]);
                        v[1] = lds_f1_at<1 * kBpMsSliceBytes>(ad[u]);
                        if constexpr (S == 8) {
                            v[2] = lds_f1_at<2 * kBpMsSliceBytes>(ad[u]);
                            v[3] = lds_f1_at<3 * kBpMsSliceBytes>(ad[u]);
                            v[4] = lds_f1_at<4 * kBpMsSliceBytes>(ad[u]);
                            v[5] = lds_f1_at<5 * kBpMsSliceBytes>(ad[u]);
                            v[6] = lds_f1_at<6 * kBpMsSliceBytes>(ad[u]);
                            v[7] = lds_f1_at<7 * kBpMsSliceBytes>(ad[u]);
                        }
                    } else {
#pragma unroll
                        for (int z = 0; z < S; ++z) v[z] = 0.0f;
                    }
#pragma unroll
                    for (int h = 0; h < S / 2; ++h)
                        acc[2 * j + u][h] = f2_add(acc[2 * j + u][h], f2_pack(v[2 * h], v[2 * h + 1]));
                }
            }
        }
    }
    const int Y = Y0 + ty;
    if (Y > Y1) return;
#pragma unroll
    for (int i = 0; i < kBpMsPix; ++i) {
        const int X = X0 + tx + 8 * i;
        if (X > X1) continue;
#pragma unroll
        for (int h = 0; h < S / 2; ++h) {
            float v0, v1;
            f2_unpack(acc[i][h], v0, v1);
            float *p0 = img + (size_t)(z0 + 2 * h) * nimg + (size_t)Y * g.nx + X;
            *p0 = xct_update(*p0, v0, ssf, paf);
            float *p1 = p0 + nimg;
            *p1 = xct_update(*p1, v1, ssf, paf);
        }
    }
}

// ----------------------------------------------------------------- batched launches
// One subset step of many slices of different shapes in one persistent launch per kernel:
// CTAs take (slice, tile) work units from a device queue (an atomic counter) until the
// units run out.  Units of slice i are [base[i], base[i+1]); they are independent within a
// launch, so there is no waiting on other CTAs.
__device__ __forceinline__ int queue_take(int *queue, int *s_unit)
{
    if (threadIdx.x == 0) *s_unit = atomicAdd(queue, 1);
    __syncthreads();
    const int u = *s_unit;
    __syncthreads();
    return u;
}

// Slice owning unit u: the last i with base[i] <= u (binary search, one thread).
__device__ __forceinline__ int unit_item(const int *__restrict__ base, int n, int u, int *s_item)
{
    if (threadIdx.x == 0) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (base[mid] <= u) lo = mid;
            else hi = mid - 1;
        }
        *s_item = lo;
    }
    __syncthreads();
    const int i = *s_item;
    __syncthreads();
    return i;
}

template <int T>
__global__ void __launch_bounds__(kFwdThreads, FwdTile<T>::MinBlocks) fwd_batched_kernel(const XctItemDev *__restrict__ items,
                                                                     const int *__restrict__ base, int n, int sub,
                                                                     int *queue)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_unit, s_item;
    const int total = base[n];
    for (;;) {
        const int u = queue_take(queue, &s_unit);
        if (u >= total) break;
        const int i = unit_item(base, n, u, &s_item);
        const XctItemDev &it = items[i];
        const KGeom &g = it.g;
        const int nrows = it.cover ? (g.pa - sub + g.ss - 1) / g.ss : g.pa / g.ss;
        const int local = u - base[i];
        const int tiles = it.fwd_ntx * it.fwd_nty;
        const int t = local % tiles, ch = local / tiles;
        fwd_tile<T>(g, it.img, it.acc, it.trig, sub, g.ss, nrows, t % it.fwd_ntx, t / it.fwd_ntx, ch * g.fwd_chunk,
                    g.fwd_chunk, smem_raw);
        __syncthreads();  // the tile in shared memory is restaged by the next unit
    }
}

// grid: one CTA per finalize unit (a ratio row of an item's largest subset), base[n] of them.
__global__ void fwd_finalize_batched_kernel(const XctItemDev *__restrict__ items, const int *__restrict__ base,
                                            int n, int sub)
{
    __shared__ int s_item;
    const int u = blockIdx.x;
    const int i = unit_item(base, n, u, &s_item);
    const XctItemDev &it = items[i];
    const KGeom &g = it.g;
    const int nrows = it.cover ? (g.pa - sub + g.ss - 1) / g.ss : g.pa / g.ss;
    const int k = u - base[i];  // one unit per ratio row of the largest subset
    if (k >= nrows) return;
    const int th = sub + k * g.ss;
    for (int X = threadIdx.x; X < g.px; X += blockDim.x) {
        double *a = it.acc + (size_t)k * g.px + X;
        const float p = (float)*a;
        *a = 0.0;
        const float yv = xct_measured(it.sino, g.px, g.pa, X, th, g.fetch);
        it.ratio[(size_t)th * g.px + X] = xct_ratio(yv, p);
    }
}

__global__ void __launch_bounds__(BpCfg<4>::Threads) bp_batched_kernel(const XctItemDev *__restrict__ items,
                                                              const int *__restrict__ base, int n, int sub,
                                                              int *queue)
{
    __shared__ BpShared sh;
    __shared__ int s_unit, s_item;
    const int total = base[n];
    for (;;) {
        const int u = queue_take(queue, &s_unit);
        if (u >= total) break;
        const int i = unit_item(base, n, u, &s_item);
        const XctItemDev &it = items[i];
        const KGeom &g = it.g;
        const int nang = (g.pa - sub + g.ss - 1) / g.ss;
        const int t = u - base[i];
        bp_tile<4>(g, it.img, it.ratio, it.trig, sub, nang, t % it.bp_ntx, t / it.bp_ntx, (float)g.ss, (float)g.pa,
                sh);
    }
}

}  // namespace

// ---------------------------------------------------------------- tile-size dispatch
bool xct_fwd_tile_valid(int T) { return T == 44 || T == 60 || T == 76 || T == 92; }

// Raises a kernel's dynamic shared-memory limit once per device.  Host threads may race on
// the first call of a device: the flags are atomic, and setting the attribute twice is
// harmless.  Devices beyond the table set it on every call.
template <int T>
static int fwd_smem_attr(const void *fn, std::atomic<bool> *done)
{
    int dev = 0;
    XCT_CUDA_TRY(cudaGetDevice(&dev));
    const bool cached = dev >= 0 && dev < 64;
    if (!cached || !done[dev].load(std::memory_order_acquire)) {
        XCT_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FwdTile<T>::Smem));
        if (cached) done[dev].store(true, std::memory_order_release);
    }
    return XCT_OK;
}

// Calls f(std::integral_constant<int, T>) for the plan's tile side T.
template <class F>
static int with_tile(int T, F &&f)
{
    switch (T) {
    case 44: return f(std::integral_constant<int, 44>{});
    case 60: return f(std::integral_constant<int, 60>{});
    case 76: return f(std::integral_constant<int, 76>{});
    case 92: return f(std::integral_constant<int, 92>{});
    default: return xct_fail(XCT_E_INVALID, "forward tile side must be 44, 60, 76 or 92");
    }
}

void xct_batched_units(const KGeom &g, int &fwd_ntx, int &fwd_nty, int &fwd_units, int &fin_units, int &bp_ntx,
                       int &bp_units)
{
    fwd_ntx = (g.nx + 1 + g.fwd_T - 1) / g.fwd_T;
    fwd_nty = (g.ny + 1 + g.fwd_T - 1) / g.fwd_T;
    const int rows = (g.pa + g.ss - 1) / g.ss;  // the largest subset (cover mode)
    fwd_units = fwd_ntx * fwd_nty * ((rows + g.fwd_chunk - 1) / g.fwd_chunk);
    fin_units = rows;
    bp_ntx = (g.nx + kBpTX - 1) / kBpTX;
    bp_units = bp_ntx * ((g.ny + kBpTY - 1) / kBpTY);
}

int xct_batched_grids(int device, int sm_count, int fwd_T, int grids[3])
{
    (void)device;
    int a = 0, c = 0;
    int rc = with_tile(fwd_T, [&](auto tc) -> int {
        constexpr int T = decltype(tc)::value;
        static std::atomic<bool> done[64];
        int r = fwd_smem_attr<T>((const void *)fwd_batched_kernel<T>, done);
        if (r) return r;
        XCT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, fwd_batched_kernel<T>, kFwdThreads,
                                                                   FwdTile<T>::Smem));
        return XCT_OK;
    });
    if (rc) return rc;
    XCT_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, bp_batched_kernel, BpCfg<4>::Threads, 0));
    grids[0] = sm_count * (a > 0 ? a : 1);
    grids[1] = 0;  // the finalize grid is the plan's unit count
    grids[2] = sm_count * (c > 0 ? c : 1);
    return XCT_OK;
}

int launch_osem_step_batched(const XctItemDev *items, const int *bases /*[3][n+1]*/, int n, int sub,
                             int *queues /*[3]*/, const int grids[3], int fwd_T, cudaStream_t st)
{
    int rc = with_tile(fwd_T, [&](auto tc) -> int {
        constexpr int T = decltype(tc)::value;
        fwd_batched_kernel<T><<<grids[0], kFwdThreads, FwdTile<T>::Smem, st>>>(items, bases, n, sub, queues);
        XCT_CUDA_TRY(cudaGetLastError());
        return XCT_OK;
    });
    if (rc) return rc;
    if (grids[1] > 0) {
        fwd_finalize_batched_kernel<<<grids[1], 256, 0, st>>>(items, bases + (n + 1), n, sub);
        XCT_CUDA_TRY(cudaGetLastError());
    }
    bp_batched_kernel<<<grids[2], BpCfg<4>::Threads, 0, st>>>(items, bases + 2 * (n + 1), n, sub, queues + 2);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;  // launches are counted when the captured graph is replayed
}

// The forward launch of one batched subset step alone (the autotuner times it).
int launch_fwd_batched(const XctItemDev *items, const int *bases, int n, int sub, int *queue, int grid, int fwd_T,
                       cudaStream_t st)
{
    return with_tile(fwd_T, [&](auto tc) -> int {
        constexpr int T = decltype(tc)::value;
        fwd_batched_kernel<T><<<grid, kFwdThreads, FwdTile<T>::Smem, st>>>(items, bases, n, sub, queue);
        XCT_CUDA_TRY(cudaGetLastError());
        return XCT_OK;
    });
}

int fwd_tiled_rows_cap() { return kAngChunk; }

int fwd_ms_slices() { return kMsSlices; }
int fwd_ms_tile() { return kMsTile; }

// The slice-interleaved forward projector over groups*8 slices (slice-group g of the grid is
// slices 8g .. 8g+7 of img / acc).
int launch_fwd_ms(const KGeom &g, const float2 *trig, const float *img, double *acc, int groups, int sub, int step,
                  int nrows, int chunk, cudaStream_t st)
{
    if (nrows <= 0 || groups <= 0) return XCT_OK;
    if (chunk <= 0 || chunk > kAngChunk) return xct_fail(XCT_E_INVALID, "slice-interleaved angle chunk out of range");
    constexpr int T = kMsTile;
    static std::atomic<bool> done[64];
    int dev = 0;
    XCT_CUDA_TRY(cudaGetDevice(&dev));
    const bool cached = dev >= 0 && dev < 64;
    if (!cached || !done[dev].load(std::memory_order_acquire)) {
        XCT_CUDA_TRY(cudaFuncSetAttribute((const void *)fwd_ms_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)FwdMsTile<T>::Smem));
        if (cached) done[dev].store(true, std::memory_order_release);
    }
    const int ntx = (g.nx + 1 + T - 1) / T, nty = (g.ny + 1 + T - 1) / T;
    const int nch = (nrows + chunk - 1) / chunk;
    dim3 grid(ntx * nty, nch, groups);
    fwd_ms_kernel<T><<<grid, kMsThreads, FwdMsTile<T>::Smem, st>>>(img, acc, trig, g, sub, step, nrows, ntx, chunk);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

// The forward projection of dN slices into the accumulator: with the slice-interleaved
// kernel enabled (g.ms_chunk > 0), its groups of eight slices first, then the rest with the
// per-slice tiled kernel.
int launch_fwd_tiled_main(const KGeom &g, const float2 *trig, const float *img, double *acc, int dN, int sub, int step,
                          int nrows, cudaStream_t st)
{
    if (nrows <= 0 || dN <= 0) return XCT_OK;
    const int ms = g.ms_chunk > 0 ? (dN / kMsSlices) * kMsSlices : 0;
    if (ms > 0) {
        const int rc = launch_fwd_ms(g, trig, img, acc, ms / kMsSlices, sub, step, nrows, g.ms_chunk, st);
        if (rc || ms == dN) return rc;
        img += (size_t)ms * g.nx * g.ny;
        acc += (size_t)ms * nrows * g.px;
        dN -= ms;
    }
    if (g.fwd_chunk <= 0 || g.fwd_chunk > kAngChunk) return xct_fail(XCT_E_INVALID, "forward angle chunk out of range");
    return with_tile(g.fwd_T, [&](auto tc) -> int {
        constexpr int T = decltype(tc)::value;
        static std::atomic<bool> done[64];
        int r = fwd_smem_attr<T>((const void *)fwd_tiled_kernel<T>, done);
        if (r) return r;
        const int ntx = (g.nx + 1 + T - 1) / T;  // base texels -1 .. nx-1
        const int nty = (g.ny + 1 + T - 1) / T;
        const int nch = (nrows + g.fwd_chunk - 1) / g.fwd_chunk;
        dim3 grid(ntx * nty, nch, dN);
        fwd_tiled_kernel<T><<<grid, kFwdThreads, FwdTile<T>::Smem, st>>>(img, acc, trig, g, sub, step, nrows, ntx);
        g_xct_launches.fetch_add(1, std::memory_order_relaxed);
        XCT_CUDA_TRY(cudaGetLastError());
        return XCT_OK;
    });
}

int launch_fwd_finalize(const KGeom &g, const float *meas, float *out, double *acc, int dN, int sub, int step,
                        int nrows, cudaStream_t st)
{
    if (nrows <= 0 || dN <= 0) return XCT_OK;
    const bool vec = g.px % 4 == 0 && g.fetch == XCT_FETCH_EXACT && (((uintptr_t)meas | (uintptr_t)out) & 15u) == 0 &&
                     ((uintptr_t)acc & 15u) == 0;
    if (vec) {
        dim3 g4((g.px / 4 + 255) / 256, nrows, dN);
        fwd_finalize4_kernel<<<g4, 256, 0, st>>>(acc, meas, out, g, sub, step, nrows);
    } else {
        dim3 g2((g.px + 127) / 128, nrows, dN);
        fwd_finalize_kernel<<<g2, 128, 0, st>>>(acc, meas, out, g, sub, step, nrows);
    }
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_fwd_tiled(const KGeom &g, const float2 *trig, const float *img, const float *meas, float *out,
                     double *acc, int dN, int sub, int step, int nrows, cudaStream_t st)
{
    int rc = launch_fwd_tiled_main(g, trig, img, acc, dN, sub, step, nrows, st);
    if (rc) return rc;
    return launch_fwd_finalize(g, meas, out, acc, dN, sub, step, nrows, st);
}

int launch_adj_tiled(const KGeom &g, const float2 *trig, const float *sino, float *img, int dN, cudaStream_t st)
{
    return launch_adj_subset(g, trig, sino, img, dN, 0, 1, g.pa, nullptr, 0.0f, st);
}

// Launch of adj_ms_kernel<S> over groups of S slices (its shared memory opted in once per
// device).
template <int S>
static int launch_adj_ms(const KGeom &g, const float2 *trig, const float *sino, float *img, int groups, int sub,
                         int step, int nang, const float *base, float scale, cudaStream_t st)
{
    static std::atomic<bool> done[64];
    int dev = 0;
    XCT_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return xct_fail(XCT_E_INVALID, "device index out of range");
    if (!done[dev].load(std::memory_order_acquire)) {
        XCT_CUDA_TRY(cudaFuncSetAttribute((const void *)adj_ms_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)AdjMs<S>::Smem));
        done[dev].store(true, std::memory_order_release);
    }
    const int ntx = (g.nx + kAdjMsT - 1) / kAdjMsT, nty = (g.ny + kAdjMsT - 1) / kAdjMsT;
    adj_ms_kernel<S><<<dim3(ntx * nty, 1, groups), kThreads, AdjMs<S>::Smem, st>>>(sino, img, trig, g, ntx, sub, step,
                                                                                  nang, base, scale);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

int launch_adj_subset(const KGeom &g, const float2 *trig, const float *sino, float *img, int dN, int sub, int step,
                      int nang, const float *base, float scale, cudaStream_t st)
{
    if (dN <= 0) return XCT_OK;
    // with the slice-interleaved kernels on, groups of eight or ten slices take the gather
    // form (its candidate search is shared by the group; for fewer slices the scatter forms
    // cost less) -- the most groups of ten that leave a multiple of eight (a slice costs less
    // in a group of ten), then groups of eight -- and groups of four the scatter form with
    // shared sample work
    if (g.ms_chunk > 0 && dN >= 8) {
        const size_t np = (size_t)g.pa * g.px, ni = (size_t)g.nx * g.ny;
        int rc = XCT_OK;
        auto advance = [&](int n) {
            sino += n * np;
            img += n * ni;
            if (base) base += n * ni;
            dN -= n;
        };
        int tens = dN / 10;
        while (tens > 0 && (dN - 10 * tens) % 8 != 0) --tens;
        if (tens > 0) {
            if ((rc = launch_adj_gather<10>(g, trig, sino, img, tens, sub, step, nang, base, scale, st))) return rc;
            advance(tens * 10);
        }
        const int groups = dN / 8;
        if (groups > 0) {
            if ((rc = launch_adj_gather<8>(g, trig, sino, img, groups, sub, step, nang, base, scale, st))) return rc;
            advance(groups * 8);
        }
        if (dN == 0) return XCT_OK;
    }
    if (g.ms_chunk > 0 && dN >= kAdjMsSlices) {
        const int groups = dN / kAdjMsSlices, ms = groups * kAdjMsSlices;
        const int rc = launch_adj_ms<kAdjMsSlices>(g, trig, sino, img, groups, sub, step, nang, base, scale, st);
        if (rc || ms == dN) return rc;
        sino += (size_t)ms * g.pa * g.px;
        img += (size_t)ms * g.nx * g.ny;
        if (base) base += (size_t)ms * g.nx * g.ny;
        dN -= ms;
    }
    const long long big = (long long)((g.nx + kAdjT - 1) / kAdjT) * ((g.ny + kAdjT - 1) / kAdjT) * dN;
    if (big >= 3LL * device_sm_count()) {
        const int ntx = (g.nx + kAdjT - 1) / kAdjT, nty = (g.ny + kAdjT - 1) / kAdjT;
        adj_tiled_kernel<kAdjT><<<dim3(ntx * nty, 1, dN), kThreads, 0, st>>>(sino, img, trig, g, ntx, sub, step, nang,
                                                                            base, scale);
    } else {
        const int ntx = (g.nx + kAdjTSmall - 1) / kAdjTSmall, nty = (g.ny + kAdjTSmall - 1) / kAdjTSmall;
        adj_tiled_kernel<kAdjTSmall><<<dim3(ntx * nty, 1, dN), kThreads, 0, st>>>(sino, img, trig, g, ntx, sub, step,
                                                                                  nang, base, scale);
    }
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

// SM count of the current device, cached per device (152 if it cannot be read).
int device_sm_count()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        int n = 0;
        v = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0 ? n : 152;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

int launch_bp_update_tiled(const KGeom &g, const float2 *trig, float *img, const float *ratio, int dN, int sub,
                           cudaStream_t st)
{
    if (dN <= 0) return XCT_OK;
    const int nang = (g.pa - sub + g.ss - 1) / g.ss;  // OSEM2's angle loop (OSEM.cl:93)
    // with the slice-interleaved kernels on, whole groups of eight slices go through the
    // eight-slice backprojector, pairs of the rest through its two-slice form, and a last
    // single slice through the per-slice one
    if (g.ms_chunk > 0 && dN >= 2) {
        const int mtx = (g.nx + kBpMsT - 1) / kBpMsT, mty = (g.ny + kBpMsT - 1) / kBpMsT;
        const int vec = g.px % 4 == 0 && ((uintptr_t)ratio & 15u) == 0;
        const int g8 = dN / kMsSlices, g2 = (dN - g8 * kMsSlices) / 2;
        if (g8 > 0) {
            bp_ms_kernel<kMsSlices><<<dim3(mtx * mty, 1, g8), kBpMsThreads, 0, st>>>(
                img, ratio, trig, g, sub, nang, mtx, (float)g.ss, (float)g.pa, vec);
            g_xct_launches.fetch_add(1, std::memory_order_relaxed);
            XCT_CUDA_TRY(cudaGetLastError());
            img += (size_t)g8 * kMsSlices * g.nx * g.ny;
            ratio += (size_t)g8 * kMsSlices * g.pa * g.px;
            dN -= g8 * kMsSlices;
        }
        if (g2 > 0) {
            bp_ms_kernel<2><<<dim3(mtx * mty, 1, g2), kBpMsThreads, 0, st>>>(img, ratio, trig, g, sub, nang, mtx,
                                                                             (float)g.ss, (float)g.pa, vec);
            g_xct_launches.fetch_add(1, std::memory_order_relaxed);
            XCT_CUDA_TRY(cudaGetLastError());
            img += (size_t)g2 * 2 * g.nx * g.ny;
            ratio += (size_t)g2 * 2 * g.pa * g.px;
            dN -= g2 * 2;
        }
        if (dN == 0) return XCT_OK;
    }
    const int ntx = (g.nx + kBpTX - 1) / kBpTX, nty = (g.ny + kBpTY - 1) / kBpTY;
    dim3 grid(ntx * nty, 1, dN);
    // four rows per thread once the grid gives three waves of its resident CTAs (6 per SM)
    if ((long long)ntx * nty * dN >= 3LL * 6 * device_sm_count())
        bp_tiled_kernel<4><<<grid, BpCfg<4>::Threads, 0, st>>>(img, ratio, trig, g, sub, nang, ntx, (float)g.ss,
                                                                (float)g.pa);
    else
        bp_tiled_kernel<2><<<grid, BpCfg<2>::Threads, 0, st>>>(img, ratio, trig, g, sub, nang, ntx, (float)g.ss,
                                                                (float)g.pa);
    g_xct_launches.fetch_add(1, std::memory_order_relaxed);
    XCT_CUDA_TRY(cudaGetLastError());
    return XCT_OK;
}

XCT_CHECK_READER(xct_check_read_tiled)
