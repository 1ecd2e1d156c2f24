// xct_cs.cu -- the compressed-sensing proximal steps of the OS-EM variant
// (FISTA_OSEM_execution, CT_reconstruction/GPU.cpp:243-405): ISTA3D and FISTA3D
// (FISTA.cl:409-594) over a batch of dN slices, the batch's slices being the third axis.
//
// Per voxel: the six neighbours (x+-1, y+-1 inside the slice with a zero border; layer
// min(Z+1, dN-1); and layer 0 -- the reference takes fmin(Z-1, 0) for the lower layer,
// FISTA.cl:425,513, which this reproduces), sorted by the kernels' exchange loop, then a
// 13-candidate chain selected by 12 comparisons: the minimiser of
// (x - v)^2/2 + lambda sum_k |x - n_k|.  Element-wise, HBM-bound (7 image reads, 1-3 writes
// per voxel); the arithmetic is the reference's, so the result is bit-identical for the same
// input.
#include <math.h>

#include <algorithm>

#include "xct_internal.h"

namespace {

__device__ __forceinline__ float texz(const float *__restrict__ vz, int nx, int ny, int X, int Y)
{
    return (X >= 0 && Y >= 0 && X < nx && Y < ny) ? __ldg(vz + (size_t)Y * nx + X) : 0.0f;
}

__device__ __forceinline__ float cs_select(const float *__restrict__ v, int nx, int ny, int dN, int X, int Y, int Z,
                                           float lambda)
{
    const size_t m = (size_t)nx * ny;
    const float *vz = v + (size_t)Z * m;
    float nb[6];
    nb[0] = texz(vz, nx, ny, X + 1, Y);
    nb[1] = texz(vz, nx, ny, X - 1, Y);
    nb[2] = texz(vz, nx, ny, X, Y + 1);
    nb[3] = texz(vz, nx, ny, X, Y - 1);
    nb[4] = __ldg(v + (size_t)min(Z + 1, dN - 1) * m + (size_t)Y * nx + X);
    nb[5] = __ldg(v + (size_t)Y * nx + X);
    const float vi = __ldg(vz + (size_t)Y * nx + X);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const float img1 = nb[i];
        float img2 = img1;
        int bigger = i;
#pragma unroll
        for (int j = i + 1; j < 6; ++j) {
            bigger = (nb[j] > img2) ? j : bigger;
            img2 = (nb[j] > img2) ? nb[j] : img2;
        }
        // nb[i] = img2; nb[bigger] = img1 (bigger >= i), unrolled to keep nb in registers
#pragma unroll
        for (int j = i; j < 6; ++j) nb[j] = (j == i) ? img2 : ((j == bigger) ? img1 : nb[j]);
    }
    const float l2 = 2.0f * lambda, l4 = 4.0f * lambda, l6 = 6.0f * lambda;
    const float cnd[13] = {vi - l6, nb[0], vi - l4, nb[1], vi - l2, nb[2], vi,
                           nb[3],   vi + l2, nb[4], vi + l4, nb[5], vi + l6};
    const float rng[12] = {nb[0] + l6, nb[0] + l4, nb[1] + l4, nb[1] + l2, nb[2] + l2, nb[2],
                           nb[3],      nb[3] - l2, nb[4] - l2, nb[4] - l4, nb[5] - l4, nb[5] - l6};
    float x = cnd[0];
#pragma unroll
    for (int i = 0; i < 12; ++i) x = (vi < rng[i]) ? cnd[i + 1] : x;
    return x;
}

// grid-stride over dN*ny*nx voxels.
__global__ void ista3d_kernel(const float *__restrict__ v, float *__restrict__ x_new, int nx, int ny, int dN,
                              float lambda)
{
    const long long total = (long long)nx * ny * dN;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(i % nx);
        const long long r = i / nx;
        const int Y = (int)(r % ny), Z = (int)(r / ny);
        float x = cs_select(v, nx, ny, dN, X, Y, Z, lambda);
        x = fmaxf(1.0e-6f, x);
        x_new[i] = (x != x) ? 1.0e-6f : x;
    }
}

// x_in (the image x_t), w and beta are read and written at the voxel's own index only, so
// x_in may be w itself (FISTA_OSEM_execution passes w as x_t); x_new may be null (not stored).
__global__ void fista3d_kernel(const float *x_in, float *w, const float *__restrict__ v, float *__restrict__ beta,
                               float *__restrict__ x_new, int nx, int ny, int dN, float lambda)
{
    const long long total = (long long)nx * ny * dN;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(i % nx);
        const long long r = i / nx;
        const int Y = (int)(r % ny), Z = (int)(r / ny);
        const float xi = x_in[i], b = beta[i];
        const float x = cs_select(v, nx, ny, dN, X, Y, Z, lambda);
        if (x_new) x_new[i] = x;
        float bn = b * b * 4.0f + 1.0f;
        bn = (sqrtf(bn) + 1.0f) * 0.5f;
        const float g = __fdiv_rn(b - 1.0f, bn);
        beta[i] = bn;
        const float wn = g * x + (1.0f - g) * xi;
        w[i] = (wn != wn) ? 1.0e-6f : wn;
    }
}

// The same steps over the stacks of a batch plan (block row blockIdx.y = stack): ISTA3D of the
// stack's images into xn, FISTA3D with x = w = the stack's w (FISTA_OSEM_execution's binding),
// v = the images, and the copies around them.
__global__ void ista3d_stacks_kernel(const XctStackDev *__restrict__ stacks, float lambda)
{
    const XctStackDev &S = stacks[blockIdx.y];
    const long long total = (long long)S.nx * S.ny * S.dN;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(i % S.nx);
        const long long r = i / S.nx;
        const int Y = (int)(r % S.ny), Z = (int)(r / S.ny);
        float x = cs_select(S.img, S.nx, S.ny, S.dN, X, Y, Z, lambda);
        x = fmaxf(1.0e-6f, x);
        S.xn[i] = (x != x) ? 1.0e-6f : x;
    }
}

__global__ void fista3d_stacks_kernel(const XctStackDev *__restrict__ stacks, float lambda)
{
    const XctStackDev &S = stacks[blockIdx.y];
    const long long total = (long long)S.nx * S.ny * S.dN;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int X = (int)(i % S.nx);
        const long long r = i / S.nx;
        const int Y = (int)(r % S.ny), Z = (int)(r / S.ny);
        const float xi = S.w[i], b = S.beta[i];
        const float x = cs_select(S.img, S.nx, S.ny, S.dN, X, Y, Z, lambda);
        S.xn[i] = x;
        float bn = b * b * 4.0f + 1.0f;
        bn = (sqrtf(bn) + 1.0f) * 0.5f;
        const float g = __fdiv_rn(b - 1.0f, bn);
        S.beta[i] = bn;
        const float wn = g * x + (1.0f - g) * xi;
        S.w[i] = (wn != wn) ? 1.0e-6f : wn;
    }
}

// what: 0 img <- xn; 1 w <- img and beta <- 0
__global__ void stack_copy_kernel(const XctStackDev *__restrict__ stacks, int what)
{
    const XctStackDev &S = stacks[blockIdx.y];
    const long long total = (long long)S.nx * S.ny * S.dN;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        if (what == 0) {
            S.img[i] = S.xn[i];
        } else {
            S.w[i] = S.img[i];
            S.beta[i] = 0.0f;
        }
    }
}

int cs_grid(long long n, int sm_count)
{
    return (int)std::max(1LL, std::min((n + 255) / 256, (long long)sm_count * 16));
}

}  // namespace

int launch_ista3d(const float *v, float *x_new, int nx, int ny, int dN, float lambda, int sm_count, cudaStream_t st)
{
    ista3d_kernel<<<cs_grid((long long)nx * ny * dN, sm_count), 256, 0, st>>>(v, x_new, nx, ny, dN, lambda);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "ista3d_kernel launch");
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

int launch_fista3d(const float *x_in, float *w, const float *v, float *beta, float *x_new, int nx, int ny, int dN,
                   float lambda, int sm_count, cudaStream_t st)
{
    fista3d_kernel<<<cs_grid((long long)nx * ny * dN, sm_count), 256, 0, st>>>(x_in, w, v, beta, x_new, nx, ny, dN,
                                                                                lambda);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "fista3d_kernel launch");
    g_xct_launches.fetch_add(1);
    return XCT_OK;
}

// The stack launchers run only inside a batch plan's graph capture; xct_batch_run counts the
// launches of each replay.
static int stacks_grid(int nstacks, long long max_vox, int sm_count, dim3 &grid)
{
    if (nstacks <= 0 || nstacks > 65535) return xct_fail(XCT_E_INVALID, "stack count out of range");
    const long long per = std::max(1LL, (long long)sm_count * 16 / nstacks);
    grid = dim3((unsigned)std::max(1LL, std::min((max_vox + 255) / 256, per)), (unsigned)nstacks);
    return XCT_OK;
}

int launch_ista3d_stacks(const XctStackDev *stacks, int nstacks, long long max_vox, float lambda, int sm_count,
                         cudaStream_t st)
{
    dim3 grid;
    int rc = stacks_grid(nstacks, max_vox, sm_count, grid);
    if (rc) return rc;
    ista3d_stacks_kernel<<<grid, 256, 0, st>>>(stacks, lambda);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "ista3d_stacks_kernel launch");
    return XCT_OK;
}

int launch_fista3d_stacks(const XctStackDev *stacks, int nstacks, long long max_vox, float lambda, int sm_count,
                          cudaStream_t st)
{
    dim3 grid;
    int rc = stacks_grid(nstacks, max_vox, sm_count, grid);
    if (rc) return rc;
    fista3d_stacks_kernel<<<grid, 256, 0, st>>>(stacks, lambda);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "fista3d_stacks_kernel launch");
    return XCT_OK;
}

int launch_stack_copy(const XctStackDev *stacks, int nstacks, long long max_vox, int what, int sm_count,
                      cudaStream_t st)
{
    dim3 grid;
    int rc = stacks_grid(nstacks, max_vox, sm_count, grid);
    if (rc) return rc;
    stack_copy_kernel<<<grid, 256, 0, st>>>(stacks, what);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return xct_cuda_fail(e, "stack_copy_kernel launch");
    return XCT_OK;
}
