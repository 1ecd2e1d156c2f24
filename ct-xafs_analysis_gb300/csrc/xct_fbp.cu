// xct_fbp.cu -- filtered backprojection and the base-up step of the FBP + OS-EM hybrid.
//
// Replaces, for CT_reconstruction:
//   FBP_execution (GPU.cpp:665-819) over the kernels of FBP.cl:
//     spinFactor .. outputImage (FBP.cl:34-160)  -> fbp_filter_kernel (one launch)
//     backProjectionFBP (FBP.cl:164-188)          -> fbp_bp_kernel
//   hybrid_thread's base-up (GPU.cpp:1538-1566):
//     findMinimumX/findMinimumY (reconstShare.cl:111-177) -> folded into fbp_bp_kernel
//     baseUp (reconstShare.cl:87-109)                     -> base_up_kernel
//
// Ramp filter.  The reference zero-pads each sinogram row to ZP_SIZE bins, runs a radix-2
// FFT in global memory (one launch per butterfly stage), multiplies by the ramp
// |k| * PI/ZP_SIZE, runs the inverse FFT the same way and keeps the real part.  Here one
// CTA filters two rows a, b at once in shared memory: z = a + i b, Z = FFT(z),
// Y = Z * H / zp, y = IFFT(Y) = filt(a) + i filt(b), which holds because the ramp H is real
// and even.  The transform is a Stockham autosort FFT (radix 8, then 4 or 2), the inverse is
// taken as conj(FFT(conj(Y))).  The reference moves bin px/2 to index 0 before the
// transform (FBP.cl:53-56); a circular shift commutes with a circular convolution, so the
// bins stay in place here and the filtered row is the same in exact arithmetic.  The
// rounding differs from the reference's radix-2 float FFT at the 1e-6 relative level.
//
// FBP backprojection.  Same pixel tiling as the OS-EM backprojector (64 x 64 pixels, 8 per
// thread in two or four rows, per-angle windows of the filtered row staged in shared
// memory), with the
// reference's linear sampler along the row and its per-pixel expression order, so the
// image is bit-identical to FBP.cl's for the same filtered sinogram.
#include <math.h>
#include <stdio.h>

#include <algorithm>

#include "xct_async.cuh"
#include "xct_check.cuh"
#include "xct_device.cuh"
#include "xct_f32x2.cuh"
#include "xct_internal.h"

namespace {

// backprojection: 64 x 64 pixel tiles (each thread 8 pixels of two rows 32 apart), windows of
// kFbpW >= 63|c| + 63|s| + 4 bins staged kFbpChunk angles at a time
// (40 angles of 96 bin pairs: 31 KB of shared memory, so the register-limited six CTAs of the
// four-row kernel still fit on an SM)
constexpr int kFbpTX = 64, kFbpTY = 64, kFbpThreads = 256, kFbpChunk = 40, kFbpW = 96;

// ------------------------------------------------------------------ ramp filter (FFT)
__device__ __forceinline__ int fpad(int i) { return i + (i >> 4); }  // 16-entry rows + 1

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }  // a * (-i)

// Forward DFT of R points in registers: y[k] = sum_r v[r] exp(-2 pi i r k / R).
__device__ __forceinline__ void dft2(float2 &a, float2 &b)
{
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}
__device__ __forceinline__ void dft4(float2 &v0, float2 &v1, float2 &v2, float2 &v3)
{
    const float2 t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), t3 = cmul_mi(csub(v1, v3));
    v0 = cadd(t0, t2);
    v2 = csub(t0, t2);
    v1 = cadd(t1, t3);
    v3 = csub(t1, t3);
}
template <int R>
__device__ __forceinline__ void dft(float2 *v)
{
    if constexpr (R == 2) {
        dft2(v[0], v[1]);
    } else if constexpr (R == 4) {
        dft4(v[0], v[1], v[2], v[3]);
    } else {
        // 8 = 2 x 4: DFT4 of the even and the odd samples, then the W8^k combination
        float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
        float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
        dft4(e0, e1, e2, e3);
        dft4(o0, o1, o2, o3);
        const float h = 0.70710678118654752f;
        o1 = make_float2((o1.x + o1.y) * h, (o1.y - o1.x) * h);   // * (1 - i)/sqrt2
        o2 = cmul_mi(o2);                                         // * (-i)
        o3 = make_float2((o3.y - o3.x) * h, -(o3.x + o3.y) * h);  // * (-1 - i)/sqrt2
        v[0] = cadd(e0, o0);
        v[4] = csub(e0, o0);
        v[1] = cadd(e1, o1);
        v[5] = csub(e1, o1);
        v[2] = cadd(e2, o2);
        v[6] = csub(e2, o2);
        v[3] = cadd(e3, o3);
        v[7] = csub(e3, o3);
    }
}

// One Stockham pass of radix R over xs[zp] (padded): butterfly j < zp/R reads
// xs[j + r*zp/R], twiddles by exp(-2 pi i r k / (Ns R)) with k = j mod Ns, transforms, and
// writes xs[(j - k) R + k + r Ns].  Each thread owns VPT/R butterflies; all reads finish
// before the barrier, so the pass is in place.
template <int R, int VPT>
__device__ __forceinline__ void stockham_pass(float2 *xs, int zp, int Ns, float tscale)
{
    constexpr int B = VPT / R;
    const int T = blockDim.x, stride = zp / R;
    float2 v[B][R];
#pragma unroll
    for (int q = 0; q < B; ++q) {
        const int j = threadIdx.x + q * T;
        const int k = j & (Ns - 1);
#pragma unroll
        for (int r = 0; r < R; ++r) v[q][r] = xs[fpad(j + r * stride)];
        if (Ns > 1) {
            // angle 2 pi r k / (Ns R) = pi * (2 r k zp/(Ns R)) / zp; tscale = 2 / (Ns R)
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float s, c;
                sincospif((float)(r * k) * tscale, &s, &c);
                v[q][r] = cmul(v[q][r], make_float2(c, -s));
            }
        }
        dft<R>(v[q]);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < B; ++q) {
        const int j = threadIdx.x + q * T;
        const int k = j & (Ns - 1);
        const int d = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) xs[fpad(d + r * Ns)] = v[q][r];
    }
    __syncthreads();
}

template <int VPT>
__device__ __forceinline__ void fft_forward(float2 *xs, int zp, int logzp)
{
    int Ns = 1, rem = logzp;
    while (rem > 0) {
        if (VPT >= 8 && rem >= 3) {
            stockham_pass<(VPT >= 8 ? 8 : 2), VPT>(xs, zp, Ns, 2.0f / (float)(Ns * 8));
            Ns <<= 3;
            rem -= 3;
        } else if (VPT >= 4 && rem >= 2) {
            stockham_pass<(VPT >= 4 ? 4 : 2), VPT>(xs, zp, Ns, 2.0f / (float)(Ns * 4));
            Ns <<= 2;
            rem -= 2;
        } else {
            stockham_pass<2, VPT>(xs, zp, Ns, 2.0f / (float)(Ns * 2));
            Ns <<= 1;
            rem -= 1;
        }
    }
}

// grid: ceil(nrows / 2) CTAs of zp / VPT threads (at least 32); rows 2c and 2c+1 of the
// flattened [nrows][px] sinogram stack.  h = PI/zp as the reference stores it (a float).
template <int VPT>
__global__ void __launch_bounds__(1024) fbp_filter_kernel(const float *__restrict__ sino, float *__restrict__ out,
                                                          long long nrows, int px, int zp, int logzp, float h)
{
    extern __shared__ float2 xs[];
    const int T = blockDim.x;
    const long long r0 = 2LL * blockIdx.x;
    const bool has_b = r0 + 1 < nrows;
    const float *ra = sino + r0 * px;
    for (int n = threadIdx.x; n < zp; n += T) {
        float a = 0.0f, b = 0.0f;
        if (n < px) {
            a = __ldg(ra + n);
            if (has_b) b = __ldg(ra + px + n);
        }
        xs[fpad(n)] = make_float2(a, b);
    }
    __syncthreads();
    fft_forward<VPT>(xs, zp, logzp);
    // ramp (FBP.cl:132-133: X*h below zp/2, (zp - X)*h above), then conj for the inverse
    for (int k = threadIdx.x; k < zp; k += T) {
        const float f = (float)min(k, zp - k) * h;
        const float2 v = xs[fpad(k)];
        xs[fpad(k)] = make_float2(v.x * f, -(v.y * f));
    }
    __syncthreads();
    fft_forward<VPT>(xs, zp, logzp);
    // y = conj(F) / zp (a power of two: the scaling is exact)
    const float inv = 1.0f / (float)zp;
    float *oa = out + r0 * px;
    for (int n = threadIdx.x; n < px; n += T) {
        const float2 v = xs[fpad(n)];
        oa[n] = v.x * inv;
        if (has_b) oa[px + n] = -v.y * inv;
    }
}

// ------------------------------------------------------------ FBP backprojection
struct FbpShared {
    float2 win[kFbpChunk * kFbpW];  // entry j of angle k: (t[lo+j], t[lo+j+1]), the lerp's two bins
    float2 scs[kFbpChunk];
    int slo[kFbpChunk];
    unsigned soff[kFbpChunk];  // shared address of angle k's entry for floor bits fb: soff[k] + 8*fb
    float red[kFbpThreads / 32];
};

__device__ __forceinline__ void fbp_lds2(unsigned addr, float &t0, float &t1)
{
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(t0), "=f"(t1) : "r"(addr));
}

// Monotone integer key of a float (atomicMin on keys orders as the floats do).
__device__ __forceinline__ int fkey(float f)
{
    const int b = __float_as_int(f);
    return b >= 0 ? b : b ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float fkey_decode(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF); }

// grid: (ntx * nty, 1, dN).  img[Y][X] = (1/(2 pa)) sum_th lin(fprj[th], u) for pixels with
// r < nx/2, else 0 (FBP.cl:178-187); u = ((Xc c - Yc s) + cx) + 0.5, sampled by the linear
// sampler at (u, th + 0.5): i = floor(u - 0.5), a = (u - 0.5) - i,
// (1 - a) t[i] + a t[i+1], zero off the detector.  min_keys (optional): the per-slice
// minimum of the written image, as keys.
// R rows per thread (kFbpTY / R apart, 512 / R threads): R = 4 shares the products Xc*c over
// four rows; R = 2 fills the SMs better when a launch has few tiles.
template <int R>
__global__ void __launch_bounds__(512 / R, R == 4 ? 6 : 4) fbp_bp_kernel(const float *__restrict__ fprj, float *__restrict__ img,
                                                         const float2 *__restrict__ trig, KGeom g, int ntx,
                                                         int *__restrict__ min_keys)
{
    constexpr int kThr = 512 / R, kStride = kFbpTY / R;
    __shared__ FbpShared sh;
    const int z = blockIdx.z;
    const float *rt = fprj + (size_t)z * g.pa * g.px;
    const int bx = (int)blockIdx.x % ntx, by = (int)blockIdx.x / ntx;
    const int X0 = bx * kFbpTX, Y0 = by * kFbpTY;
    const int X1 = min(X0 + kFbpTX, g.nx) - 1, Y1 = min(Y0 + kFbpTY, g.ny) - 1;
    // thread tx takes the pixels X0 + tx + 8i (i < 8): the 8 lanes of a row read neighbouring
    // bins and write neighbouring pixels
    const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;
    float Ycr[R];
#pragma unroll
    for (int r = 0; r < R; ++r) Ycr[r] = (float)min(Y0 + ty + r * kStride, Y1) - g.hy;
    float xc[8];
    f2x acc2[R][4];  // pixel pairs of each row, packed adds (each lane an IEEE add)
#pragma unroll
    for (int i = 0; i < 8; ++i) xc[i] = (float)min(X0 + tx + 8 * i, X1) - g.hx;
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc2[r][j] = f2_pack(0.0f, 0.0f);
    const unsigned wbase = (unsigned)__cvta_generic_to_shared(sh.win);
    const f2x cxp = f2_pack(g.cx, g.cx), hp = f2_pack(0.5f, 0.5f), MM = f2_pack(12582912.0f, 12582912.0f);
    const f2x one2 = f2_pack(1.0f, 1.0f);
    for (int k0 = 0; k0 < g.pa; k0 += kFbpChunk) {
        const int kn = min(kFbpChunk, g.pa - k0);
        __syncthreads();
        for (int k = threadIdx.x; k < kn; k += kThr) {
            const float2 cs = trig[k0 + k];
            sh.scs[k] = cs;
            // u is monotone in X and in Y (every step rounds monotonically): the corners
            // bound the window of floor(u - 0.5)
            const float xa = (float)X0 - g.hx, xb = (float)X1 - g.hx;
            const float qa = ((float)Y0 - g.hy) * cs.y, qb = ((float)Y1 - g.hy) * cs.y;
            int lo = xct_floor_bits(xct_bin_coord(xa, cs.x, qa, g.cx) - 0.5f);
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qa, g.cx) - 0.5f));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xa, cs.x, qb, g.cx) - 0.5f));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qb, g.cx) - 0.5f));
            sh.slo[k] = lo - XCT_FLOOR_BIAS;
            // entry for floor bits fb: k*W + fb - lo  (mod 2^32), 8 bytes each
            sh.soff[k] = wbase + 8u * (unsigned)(k * kFbpW) - 8u * (unsigned)lo;
        }
        __syncthreads();
        for (int i = threadIdx.x; i < kn * kFbpW; i += kThr) {
            const int k = i / kFbpW, j = i - k * kFbpW;
            const int bin = sh.slo[k] + j;
            const float *rk = rt + (size_t)(k0 + k) * g.px;
            sh.win[i] = make_float2(((unsigned)bin < (unsigned)g.px) ? __ldg(rk + bin) : 0.0f,
                                    ((unsigned)(bin + 1) < (unsigned)g.px) ? __ldg(rk + bin + 1) : 0.0f);
        }
        __syncthreads();
        // any entry of the staged windows (each holds both bins of its lerp)
        const unsigned wlo = wbase, whi = wbase + 8u * (unsigned)(kn * kFbpW - 1);
        (void)wlo;
        (void)whi;
        for (int k = 0; k < kn; ++k) {
            const float c = sh.scs[k].x, s = sh.scs[k].y;
            const unsigned off = sh.soff[k];
            float q[R];
#pragma unroll
            for (int r = 0; r < R; ++r) q[r] = Ycr[r] * s;
            // one row's pixel pair from the shared products Xc*c: the additions, the
            // round-down floor and the fraction packed over the pair, each lane rounding as
            // the scalar expression uu = (((Xc*c - q) + cx) + 0.5) - 0.5, fi = floor(uu),
            // a = uu - fi; then acc += (1 - a) t[fi] + a t[fi+1] with the products in scalar
            // (ptxas fuses a packed multiply feeding a packed add or subtract, and the
            // reference rounds each operation)
            auto pair = [&](float p0, float p1, float qq, f2x &acc) {
                const f2x d = f2_pack(p0 - qq, p1 - qq);
                const f2x uu = f2_sub(f2_add(f2_add(d, cxp), hp), hp);
                const f2x tb = f2_add_rd(uu, MM);
                const f2x a2 = f2_sub(uu, f2_sub(tb, MM));
                const f2x w2 = f2_sub(one2, a2);
                int e0, e1;
                f2_unpack_bits(tb, e0, e1);
                float a0, a1, w0, w1;
                f2_unpack(a2, a0, a1);
                f2_unpack(w2, w0, w1);
                const unsigned ad0 = (unsigned)e0 * 8u + off, ad1 = (unsigned)e1 * 8u + off;
                const bool in0 = XCT_IN(ad0, wlo, whi, XCT_SITE_FBP_WIN), in1 = XCT_IN(ad1, wlo, whi, XCT_SITE_FBP_WIN);
                float t00 = 0.0f, t01 = 0.0f, t10 = 0.0f, t11 = 0.0f;
                if (in0) fbp_lds2(ad0, t00, t01);
                if (in1) fbp_lds2(ad1, t10, t11);
                const float p00 = w0 * t00, p01 = a0 * t01;
                const float p10 = w1 * t10, p11 = a1 * t11;
                acc = f2_add(acc, f2_add(f2_pack(p00, p10), f2_pack(p01, p11)));
            };
#pragma unroll
            for (int i = 0; i < 8; i += 2) {
                const float p0 = xc[i] * c, p1 = xc[i + 1] * c;
#pragma unroll
                for (int r = 0; r < R; ++r) pair(p0, p1, q[r], acc2[r][i / 2]);
            }
        }
    }
    const float two_pa = (float)g.pa * 2.0f;
    float vmin = INFINITY;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int Y = Y0 + ty + r * kStride;
        const float Yc = Ycr[r];
        if (Y > Y1) continue;
        float acc[8];
#pragma unroll
        for (int j = 0; j < 4; ++j) f2_unpack(acc2[r][j], acc[2 * j], acc[2 * j + 1]);
        float *row = img + ((size_t)z * g.ny + Y) * g.nx;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int X = X0 + tx + 8 * i;
            if (X <= X1) {
                const float rr = sqrtf(xc[i] * xc[i] + Yc * Yc);
                const float v = (rr < g.hx) ? __fdiv_rn(acc[i], two_pa) : 0.0f;
                row[X] = v;
                vmin = fminf(vmin, v);
            }
        }
    }
    if (min_keys != nullptr) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        if ((threadIdx.x & 31) == 0) sh.red[threadIdx.x >> 5] = vmin;
        __syncthreads();
        if (threadIdx.x == 0) {
            float m = sh.red[0];
            for (int i = 1; i < kThr / 32; ++i) m = fminf(m, sh.red[i]);
            atomicMin(min_keys + z, fkey(m));
        }
    }
}

// ---------------------------------------- FBP backprojection, eight slices per tile
// For the slices of one call (one geometry) a (pixel, angle) pair reads the same two bins in
// all eight slices of a group, so the bin coordinate, floor and fraction are found once for
// eight lerps.  A CTA of 256 threads owns a 32 x 32 pixel tile of eight slices and stages,
// per angle and pair of slices, the window of the tile's bins (< 49 with the lerp's second
// bin, bounded exactly by the tile corners as in fbp_bp_kernel, its start rounded down to a
// multiple of 4) as (t_z, t_z+1) pairs by asynchronous copies, 24 angles at a time.  A
// thread takes 4 pixels of one row (8 apart); per pixel and angle: the literal expression of
// fbp_bp_kernel for u, floor and fraction, two 8-byte loads per slice pair (bins i and
// i + 1), the products in scalar and their sum and the accumulation packed over the slice
// pair -- each slice's sum is fbp_bp_kernel's bit for bit.  The epilogue (field-of-view mask,
// 1/(2 pa), the slice minimum for the base-up) is fbp_bp_kernel's.
constexpr int kFbpMsT = 32, kFbpMsThreads = 256, kFbpMsW = 52, kFbpMsChunk = 24, kFbpMsPix = 4, kFbpMsSlices = 8;
constexpr unsigned kFbpMsPairBytes = (unsigned)(kFbpMsChunk * kFbpMsW * 8);  // one slice pair's windows

template <int S>
struct FbpMsShared {
    float2 win[(S / 2) * kFbpMsChunk * kFbpMsW];  // [pair][angle][bin]: (t_z, t_z+1)
    float2 scs[kFbpMsChunk];
    int slo[kFbpMsChunk];
    unsigned soff[kFbpMsChunk];  // shared address of angle k's entry for floor bits fb: soff[k] + 8*fb
    float red[kFbpMsThreads / 32][S];
};

// grid: (ntx * nty tiles of 32 x 32, 1, dN / S slice groups), S = 8 or 2.
template <int S>
__global__ void __launch_bounds__(kFbpMsThreads) fbp_bp_ms_kernel(const float *__restrict__ fprj,
                                                                  float *__restrict__ img,
                                                                  const float2 *__restrict__ trig, KGeom g, int ntx,
                                                                  int *__restrict__ min_keys)
{
    constexpr int P = S / 2;
    __shared__ __align__(16) FbpMsShared<S> sh;
    const int z0 = (int)blockIdx.z * S;
    const size_t nprj = (size_t)g.pa * g.px, nimg = (size_t)g.nx * g.ny;
    const float *rz = fprj + (size_t)z0 * nprj;
    const int bx = (int)blockIdx.x % ntx, by = (int)blockIdx.x / ntx;
    const int X0 = bx * kFbpMsT, Y0 = by * kFbpMsT;
    const int X1 = min(X0 + kFbpMsT, g.nx) - 1, Y1 = min(Y0 + kFbpMsT, g.ny) - 1;
    const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;
    const float Yc = (float)min(Y0 + ty, Y1) - g.hy;
    float xc[kFbpMsPix];
#pragma unroll
    for (int i = 0; i < kFbpMsPix; ++i) xc[i] = (float)min(X0 + tx + 8 * i, X1) - g.hx;
    f2x acc[kFbpMsPix][P];
#pragma unroll
    for (int i = 0; i < kFbpMsPix; ++i)
#pragma unroll
        for (int h = 0; h < P; ++h) acc[i][h] = 0ull;
    const unsigned wbase = (unsigned)__cvta_generic_to_shared(sh.win);
    const f2x cxp = f2_pack(g.cx, g.cx), hp = f2_pack(0.5f, 0.5f), MM = f2_pack(12582912.0f, 12582912.0f);
    const f2x one2 = f2_pack(1.0f, 1.0f);
    for (int k0 = 0; k0 < g.pa; k0 += kFbpMsChunk) {
        const int kn = min(kFbpMsChunk, g.pa - k0);
        __syncthreads();
        for (int k = threadIdx.x; k < kn; k += kFbpMsThreads) {
            const float2 cs = trig[k0 + k];
            sh.scs[k] = cs;
            const float xa = (float)X0 - g.hx, xb = (float)X1 - g.hx;
            const float qa = ((float)Y0 - g.hy) * cs.y, qb = ((float)Y1 - g.hy) * cs.y;
            int lo = xct_floor_bits(xct_bin_coord(xa, cs.x, qa, g.cx) - 0.5f);
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qa, g.cx) - 0.5f));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xa, cs.x, qb, g.cx) - 0.5f));
            lo = min(lo, xct_floor_bits(xct_bin_coord(xb, cs.x, qb, g.cx) - 0.5f));
            lo &= ~3;  // the bias is a multiple of 4: this rounds the bin down to one
            sh.slo[k] = lo - XCT_FLOOR_BIAS;
            sh.soff[k] = wbase + 8u * (unsigned)(k * kFbpMsW) - 8u * (unsigned)lo;
        }
        __syncthreads();
        // window (pair p, angle k, bin lo_k + r) = (t_{2p}, t_{2p+1}), 0 off the detector
        for (int e = threadIdx.x; e < kn * S * kFbpMsW; e += kFbpMsThreads) {
            const int r = e % kFbpMsW, t2 = e / kFbpMsW;
            const int z = t2 % S, k = t2 / S;
            const int bin = sh.slo[k] + r;
            const float *row = rz + (size_t)z * nprj + (size_t)(k0 + k) * g.px;
            const bool in = (unsigned)bin < (unsigned)g.px;
            const unsigned dst =
                wbase + (unsigned)(z >> 1) * kFbpMsPairBytes + 8u * (unsigned)(k * kFbpMsW + r) + 4u * (unsigned)(z & 1);
            cp_async4(dst, in ? (const void *)(row + bin) : (const void *)row, in ? 4u : 0u);
        }
        cp_async_wait_all();
        __syncthreads();
        // any entry whose next entry (the lerp's second bin) is staged
        const unsigned wlo = wbase, whi = wbase + 8u * (unsigned)(kn * kFbpMsW - 2);
        (void)wlo;
        (void)whi;
        for (int k = 0; k < kn; ++k) {
            const float c = sh.scs[k].x, s = sh.scs[k].y;
            const unsigned off = sh.soff[k];
            const float q = Yc * s;
#pragma unroll
            for (int j = 0; j < kFbpMsPix / 2; ++j) {
                // fbp_bp_kernel's expression for pixels 2j and 2j+1
                const float p0 = xc[2 * j] * c, p1 = xc[2 * j + 1] * c;
                const f2x d = f2_pack(p0 - q, p1 - q);
                const f2x uu = f2_sub(f2_add(f2_add(d, cxp), hp), hp);
                const f2x tb = f2_add_rd(uu, MM);
                const f2x a2 = f2_sub(uu, f2_sub(tb, MM));
                const f2x w2 = f2_sub(one2, a2);
                int e0, e1;
                f2_unpack_bits(tb, e0, e1);
                float a[2], w[2];
                f2_unpack(a2, a[0], a[1]);
                f2_unpack(w2, w[0], w[1]);
                const unsigned ad[2] = {(unsigned)e0 * 8u + off, (unsigned)e1 * 8u + off};
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    if (!XCT_IN(ad[u], wlo, whi, XCT_SITE_FBP_WIN)) continue;
#pragma unroll
                    for (int h = 0; h < P; ++h) {
                        float t0a, t0b, t1a, t1b;  // (slice 2h, 2h+1) at bins i and i + 1
                        if (h == 0) {
                            lds_f2_at<0>(ad[u], t0a, t0b);
                            lds_f2_at<8>(ad[u], t1a, t1b);
                        } else if (h == 1) {
                            lds_f2_at<1 * kFbpMsPairBytes>(ad[u], t0a, t0b);
                            lds_f2_at<1 * kFbpMsPairBytes + 8>(ad[u], t1a, t1b);
                        } else if (h == 2) {
                            lds_f2_at<2 * kFbpMsPairBytes>(ad[u], t0a, t0b);
                            lds_f2_at<2 * kFbpMsPairBytes + 8>(ad[u], t1a, t1b);
                        } else {
                            lds_f2_at<3 * kFbpMsPairBytes>(ad[u], t0a, t0b);
                            lds_f2_at<3 * kFbpMsPairBytes + 8>(ad[u], t1a, t1b);
                        }
                        const float pa0 = w[u] * t0a, pb0 = w[u] * t0b, pa1 = a[u] * t1a, pb1 = a[u] * t1b;
                        acc[2 * j + u][h] = f2_add(acc[2 * j + u][h], f2_add(f2_pack(pa0, pb0), f2_pack(pa1, pb1)));
                    }
                }
            }
        }
    }
    const float two_pa = (float)g.pa * 2.0f;
    const int Y = Y0 + ty;
    float vmin[S];
#pragma unroll
    for (int z = 0; z < S; ++z) vmin[z] = INFINITY;
    if (Y <= Y1) {
#pragma unroll
        for (int i = 0; i < kFbpMsPix; ++i) {
            const int X = X0 + tx + 8 * i;
            if (X > X1) continue;
            const float rr = sqrtf(xc[i] * xc[i] + Yc * Yc);
#pragma unroll
            for (int h = 0; h < P; ++h) {
                float v2[2];
                f2_unpack(acc[i][h], v2[0], v2[1]);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int z = 2 * h + u;
                    const float v = (rr < g.hx) ? __fdiv_rn(v2[u], two_pa) : 0.0f;
                    img[(size_t)(z0 + z) * nimg + (size_t)Y * g.nx + X] = v;
                    vmin[z] = fminf(vmin[z], v);
                }
            }
        }
    }
    if (min_keys != nullptr) {
#pragma unroll
        for (int z = 0; z < S; ++z) {
            float m = vmin[z];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, o));
            if ((threadIdx.x & 31) == 0) sh.red[threadIdx.x >> 5][z] = m;
        }
        __syncthreads();
        if (threadIdx.x < S) {
            float m = sh.red[0][threadIdx.x];
            for (int i = 1; i < kFbpMsThreads / 32; ++i) m = fminf(m, sh.red[i][threadIdx.x]);
            atomicMin(min_keys + z0 + threadIdx.x, fkey(m));
        }
    }
}

// baseUp (reconstShare.cl:87-109) over dN slices of n pixels, in place, a = the slice
// minimum: b1 = (v - a)/a (0 when a == 0); g = sum_{i<=order} (-1)^(i+1) b1^i / i in float;
// v -= a * exp(g).
__global__ void base_up_kernel(float *__restrict__ img, long long n, int dN, int order,
                               const int *__restrict__ min_keys)
{
    const long long total = n * dN;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const float a = fkey_decode(__ldg(min_keys + idx / n));
        const float v = img[idx];
        float gs = 0.0f;
        const float b1 = (a != 0.0f) ? __fdiv_rn(v - a, a) : 0.0f;
        float b2 = 1.0f, flag = -1.0f;
        for (int i = 1; i <= order; ++i) {
            b2 *= b1;
            flag *= -1.0f;
            gs += __fdiv_rn(flag * b2, (float)i);
        }
        img[idx] = v - a * expf(gs);
    }
}

int fbp_vpt(int zp) { return zp >= 16384 ? 16 : (zp >= 256 ? 8 : zp / 32); }

template <int VPT>
int launch_filter_vpt(const float *sino, float *out, long long nrows, int px, int zp, int logzp, float h,
                      cudaStream_t st)
{
    const int threads = zp / VPT;
    const size_t smem = sizeof(float2) * (size_t)(zp + zp / 16);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fbp_filter_kernel<VPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return xct_cuda_fail(e, "fbp_filter smem attribute");
    }
    const long long ctas = (nrows + 1) / 2;
    if (ctas > 0x7FFFFFFFLL) return xct_fail(XCT_E_INVALID, "fbp filter: too many rows in one call");
    fbp_filter_kernel<VPT><<<(unsigned)ctas, threads, smem, st>>>(sino, out, nrows, px, zp, logzp, h);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "fbp_filter_kernel launch");
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

}  // namespace

int xct_fbp_check_zp(int px, int &zp)
{
    if (zp == 0) {
        zp = 1;
        while (zp < 2 * px) zp *= 2;
    }
    if (zp < 64 || zp > 16384 || (zp & (zp - 1)) != 0 || zp < px) {
        char b[200];
        snprintf(b, sizeof b,
                 "fbp: zero padding %d must be a power of two in [64, 16384] and >= the detector width %d", zp, px);
        return xct_fail(XCT_E_INVALID, b);
    }
    return XCT_OK;
}

int launch_fbp_filter(const KGeom &g, const float *sino, float *out, int dN, int zp, cudaStream_t st)
{
    int logzp = 0;
    while ((1 << logzp) < zp) ++logzp;
    const float h = (float)(3.14159265358979323846 / zp);  // FBP.cl:132
    const long long nrows = (long long)dN * g.pa;
    switch (fbp_vpt(zp)) {
    case 2: return launch_filter_vpt<2>(sino, out, nrows, g.px, zp, logzp, h, st);
    case 4: return launch_filter_vpt<4>(sino, out, nrows, g.px, zp, logzp, h, st);
    case 8: return launch_filter_vpt<8>(sino, out, nrows, g.px, zp, logzp, h, st);
    default: return launch_filter_vpt<16>(sino, out, nrows, g.px, zp, logzp, h, st);
    }
}

int launch_fbp_bp(const KGeom &g, const float2 *trig, const float *fprj, float *img, int dN, int *min_keys,
                  cudaStream_t st)
{
    const int ntx = (g.nx + kFbpTX - 1) / kFbpTX, nty = (g.ny + kFbpTY - 1) / kFbpTY;
    if (min_keys != nullptr) {
        cudaError_t e = cudaMemsetAsync(min_keys, 0x7F, sizeof(int) * dN, st);  // key of a huge float
        if (e != cudaSuccess) return xct_cuda_fail(e, "fbp min reset");
    }
    // with the slice-interleaved kernels on, groups of eight slices go through the
    // eight-slice backprojector, pairs of the rest through its two-slice form, and a last
    // single slice through the per-slice one
    if (g.ms_chunk > 0 && dN >= 2) {
        const int mtx = (g.nx + kFbpMsT - 1) / kFbpMsT, mty = (g.ny + kFbpMsT - 1) / kFbpMsT;
        const int g8 = dN / kFbpMsSlices, g2 = (dN - g8 * kFbpMsSlices) / 2;
        auto advance = [&](int n) {
            fprj += (size_t)n * g.pa * g.px;
            img += (size_t)n * g.nx * g.ny;
            if (min_keys != nullptr) min_keys += n;
            dN -= n;
        };
        if (g8 > 0) {
            fbp_bp_ms_kernel<kFbpMsSlices><<<dim3(mtx * mty, 1, g8), kFbpMsThreads, 0, st>>>(fprj, img, trig, g, mtx,
                                                                                             min_keys);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return xct_cuda_fail(e, "fbp_bp_ms_kernel launch");
            g_xct_launches.fetch_add(1);
            advance(g8 * kFbpMsSlices);
        }
        if (g2 > 0) {
            fbp_bp_ms_kernel<2><<<dim3(mtx * mty, 1, g2), kFbpMsThreads, 0, st>>>(fprj, img, trig, g, mtx, min_keys);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return xct_cuda_fail(e, "fbp_bp_ms_kernel launch");
            g_xct_launches.fetch_add(1);
            advance(g2 * 2);
        }
        if (dN == 0) return XCT_OK;
    }
    dim3 grid(ntx * nty, 1, dN);
    // four rows per thread once the grid gives three waves of its resident CTAs (6 per SM)
    if ((long long)grid.x * grid.z >= 3LL * 6 * device_sm_count())
        fbp_bp_kernel<4><<<grid, 128, 0, st>>>(fprj, img, trig, g, ntx, min_keys);
    else
        fbp_bp_kernel<2><<<grid, 256, 0, st>>>(fprj, img, trig, g, ntx, min_keys);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "fbp_bp_kernel launch");
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

int launch_base_up(const KGeom &g, float *img, int dN, int order, const int *min_keys, int sm_count, cudaStream_t st)
{
    const long long n = (long long)g.nx * g.ny;
    const long long want = (n * dN + 255) / 256;
    const int blocks = (int)std::min<long long>(want, (long long)sm_count * 8);
    base_up_kernel<<<blocks, 256, 0, st>>>(img, n, dN, order, min_keys);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "base_up_kernel launch");
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

XCT_CHECK_READER(xct_check_read_fbp)
