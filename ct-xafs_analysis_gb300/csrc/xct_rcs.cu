// xct_rcs.cu -- the rotation-centre search (RotationCenterSearch/).
//
// Replaces rotationCenterSearch_ocl.cpp's rotCenterShift (:122-154),
// reconstRotCntShift_thread (:280-318) and imgFocusIndex_estimation (:185-223) over the
// kernels of rotCenterSearch.cl:
//   rotCenterShift (:37-49)            -> rot_shift_kernel: all shifts in one launch;
//   setMask (:51-97) + imgFocusIndex (:167-232)
//                                      -> focus_kernel: the mask is evaluated per pixel in
//                                         shared memory instead of being stored as an
//                                         image, and the sums are taken in double;
//   OSEM_execution with it = 1 (:307)  -> the plan's tiled OS-EM on all shifts as one batch.
//
// Per-pixel arithmetic (the resampling, the mask's dot products and comparisons, the focus
// terms) is the reference's, operation for operation; only the order of the image-wide sums
// differs (the reference sums in float per work-item, then in a local-memory tree).
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "xct_device.cuh"
#include "xct_internal.h"

namespace {

constexpr int kRcT = 32;           // focus tile: 32 x 32 pixels
constexpr int kRcThreads = 256;    // 4 pixels per thread
constexpr int kRcH = kRcT + 2;     // halo tile

// rotCenterShift: out[i][th][X] = the linear sampler at ((X + s) + 0.5, th + 0.5),
// s = start + step*(i0 + i) (rotationCenterSearch_ocl.cpp:140).  grid-stride over n*pa*px.
__global__ void rot_shift_kernel(const float *__restrict__ prj, float *__restrict__ out, int px, int pa, int n,
                                 int i0, float start, float step)
{
    const long long per = (long long)px * pa, total = per * n;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(idx / per);
        const long long r = idx - (long long)i * per;
        const int th = (int)(r / px), X = (int)(r - (long long)th * px);
        const float s = start + step * (float)(i0 + i);
        const float uu = (((float)X + s) + 0.5f) - 0.5f;
        const float fi = floorf(uu);
        const float a = uu - fi;
        const int b = (int)fi;
        const float *row = prj + (size_t)th * px;
        const float t0 = (b >= 0 && b < px) ? __ldg(row + b) : 0.0f;
        const float t1 = (b + 1 >= 0 && b + 1 < px) ? __ldg(row + b + 1) : 0.0f;
        out[idx] = (1.0f - a) * t0 + a * t1;
    }
}

__global__ void fill_kernel(float *__restrict__ p, long long n, float v)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

// setMask's test at pixel (x, y) with the shift's constants prm[13]
// (rp, rm, p1x, p1y, p2x, p2y, p3x, p3y, p4x, p4y, p_div, p_cnt.x, p_cnt.y);
// dot(a, b) = a.x*b.x + a.y*b.y, each product and the sum rounded.
__device__ __forceinline__ float mask_at(const float *prm, int x, int y)
{
    const float X = (float)x - prm[11], Y = (float)y - prm[12];
    const float rp2 = prm[0] * prm[0], rm2 = prm[1] * prm[1], pd = prm[10];
    const bool b1 = X * prm[2] + Y * prm[3] <= rp2;
    const bool b2 = X * prm[4] + Y * prm[5] <= rp2;
    const bool b3 = X * prm[6] + Y * prm[7] <= rm2;
    const bool b4 = X * prm[8] + Y * prm[9] <= rm2;
    const float d2 = X * X + Y * Y;
    const bool b5 = d2 <= rp2 && X > pd;
    const bool b6 = d2 <= rm2 && X <= pd;
    return (b1 && b2 && b3 && b4 && (b5 || b6)) ? 1.0f : 0.0f;
}

// grid: (ntx * nty, n).  Image z = imgs + z*nx*ny; red[2z], red[2z+1] += sums of
// sq_delta and mask_tot over the tile (doubles).
__global__ void __launch_bounds__(kRcThreads) focus_kernel(const float *__restrict__ imgs, int nx, int ny, int ntx,
                                                           const float *__restrict__ prms, double *__restrict__ red)
{
    __shared__ float s_img[kRcH][kRcH + 1];
    __shared__ float s_msk[kRcH][kRcH + 1];
    __shared__ float s_prm[13];
    __shared__ double s_red[2][kRcThreads / 32];
    const int z = blockIdx.y;
    const int X0 = ((int)blockIdx.x % ntx) * kRcT, Y0 = ((int)blockIdx.x / ntx) * kRcT;
    const float *img = imgs + (size_t)z * nx * ny;
    if (threadIdx.x < 13) s_prm[threadIdx.x] = prms[z * 16 + threadIdx.x];
    __syncthreads();
    for (int i = threadIdx.x; i < kRcH * kRcH; i += kRcThreads) {
        const int hy = i / kRcH, hx = i - hy * kRcH;
        const int x = X0 - 1 + hx, y = Y0 - 1 + hy;
        const bool in = x >= 0 && y >= 0 && x < nx && y < ny;  // the samplers' zero border
        s_img[hy][hx] = in ? __ldg(img + (size_t)y * nx + x) : 0.0f;
        s_msk[hy][hx] = in ? mask_at(s_prm, x, y) : 0.0f;
    }
    __syncthreads();
    // neighbours in the reference's order: u, d, r, l, ur, dr, ul, dl (u = y+1, r = x+1)
    const int dx[8] = {0, 0, 1, -1, 1, 1, -1, -1}, dy[8] = {1, -1, 0, 0, 1, -1, 1, -1};
    double acc_s = 0.0, acc_m = 0.0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int p = threadIdx.x + q * kRcThreads;
        const int ty = p / kRcT, tx = p - ty * kRcT;
        if (X0 + tx >= nx || Y0 + ty >= ny) continue;
        const int hx = tx + 1, hy = ty + 1;
        float m = s_msk[hy][hx];
#pragma unroll
        for (int k = 0; k < 8; ++k) m *= s_msk[hy + dy[k]][hx + dx[k]];
        const float a = s_img[hy][hx];
        float sq = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float d = s_img[hy + dy[k]][hx + dx[k]] - a;
            sq += (m == 1.0f) ? d * d : 0.0f;
        }
        sq = __fdiv_rn(sq, (m == 1.0f) ? a * a : 1.0f);
        acc_s += (double)sq;
        acc_m += (double)m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        acc_s += __shfl_xor_sync(0xffffffffu, acc_s, o);
        acc_m += __shfl_xor_sync(0xffffffffu, acc_m, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_red[0][threadIdx.x >> 5] = acc_s;
        s_red[1][threadIdx.x >> 5] = acc_m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kRcThreads / 32; ++w) {
            a += s_red[0][w];
            b += s_red[1][w];
        }
        atomicAdd(red + 2 * z, a);
        atomicAdd(red + 2 * z + 1, b);
    }
}

// findex[z] = sqrt(sum sq_delta / sum mask_tot) (the reference's final division and sqrt,
// rotCenterSearch.cl:229, taken in double and rounded once); clears red for the next call.
__global__ void focus_finalize_kernel(double *__restrict__ red, float *__restrict__ findex, int n)
{
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= n) return;
    findex[z] = (float)sqrt(red[2 * z] / red[2 * z + 1]);
    red[2 * z] = 0.0;
    red[2 * z + 1] = 0.0;
}

int grid_for(long long n, int sm_count)
{
    return (int)std::max(1LL, std::min((n + 255) / 256, (long long)sm_count * 16));
}

}  // namespace

// setMask's per-shift constants (rotCenterSearch.cl:58-72), computed on the host as the
// kernel computes them: angles a = ang*PI/180 and ang*PI/180 - PI/2 in double, stored to
// float; rp = min(W/2 + s, W/2), rm = max(-W/2 + s, -W/2) with W/2 an integer; p1 = rp cos(a_max),
// p2 = rp cos(a_min), p3 = rm cos(a_max), p4 = rm cos(a_min) with the float cos of each float
// component (correctly rounded); p_div = p1.x if rp^2 < rm^2 else p3.x; p_cnt = (W/2, H/2).
void xct_mask_params(int W, int H, float shift, float ang_min, float ang_max, float *prm)
{
    const double PI = 3.14159265358979323846, PI_2 = 1.57079632679489661923;
    const float amin_x = (float)((double)ang_min * PI / 180), amin_y = (float)((double)ang_min * PI / 180 - PI_2);
    const float amax_x = (float)((double)ang_max * PI / 180), amax_y = (float)((double)ang_max * PI / 180 - PI_2);
    const float rp = fminf((float)(W / 2) + shift, (float)(W / 2));
    const float rm = fmaxf((float)(-W / 2) + shift, (float)(-W / 2));
    prm[0] = rp;
    prm[1] = rm;
    prm[2] = rp * (float)cos((double)amax_x);
    prm[3] = rp * (float)cos((double)amax_y);
    prm[4] = rp * (float)cos((double)amin_x);
    prm[5] = rp * (float)cos((double)amin_y);
    prm[6] = rm * (float)cos((double)amax_x);
    prm[7] = rm * (float)cos((double)amax_y);
    prm[8] = rm * (float)cos((double)amin_x);
    prm[9] = rm * (float)cos((double)amin_y);
    prm[10] = (rp * rp < rm * rm) ? prm[2] : prm[6];
    prm[11] = (float)(W / 2);
    prm[12] = (float)(H / 2);
    for (int i = 13; i < 16; ++i) prm[i] = 0.0f;
}

float xct_shift_value(float start, float step, int i) { return start + step * (float)i; }

int launch_rot_shift(const float *prj, float *out, int px, int pa, int n, int i0, float start, float step,
                     int sm_count, cudaStream_t st)
{
    rot_shift_kernel<<<grid_for((long long)n * pa * px, sm_count), 256, 0, st>>>(prj, out, px, pa, n, i0, start,
                                                                                 step);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "rot_shift_kernel launch");
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

int launch_fill(float *p, long long n, float v, int sm_count, cudaStream_t st)
{
    fill_kernel<<<grid_for(n, sm_count), 256, 0, st>>>(p, n, v);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "fill_kernel launch");
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

// Focus index of n images [n][ny][nx] with the shifts' mask constants d_prm [n][16]; red is
// [2n] doubles, zero on entry and left zero.
int launch_focus_index(const float *imgs, int nx, int ny, int n, const float *d_prm, double *red, float *findex,
                       cudaStream_t st)
{
    const int ntx = (nx + kRcT - 1) / kRcT, nty = (ny + kRcT - 1) / kRcT;
    focus_kernel<<<dim3(ntx * nty, n), kRcThreads, 0, st>>>(imgs, nx, ny, ntx, d_prm, red);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "focus_kernel launch");
    focus_finalize_kernel<<<(n + 127) / 128, 128, 0, st>>>(red, findex, n);
    e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "focus_finalize_kernel launch");
    g_xct_launches.fetch_add(2);
    return XCT_OK;
}
