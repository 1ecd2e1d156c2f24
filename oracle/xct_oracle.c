/*
 * xct_oracle.c -- CPU oracle for the OS-EM path (TEST INFRASTRUCTURE ONLY).
 *
 * This is the checker, not the product: only tests/, the smoke check and the benchmark's
 * CPU-baseline leg load it.  The product path (the CUDA library) never links or calls it
 * and fails loudly when its own extension is missing.
 *
 * It restates, in plain C, the reference algorithm of NozomuIshiguro/CT-XAFS_analysis:
 *   - per-angle geometry: angle_pr = angle[th]*PI/180.0f with a double PI, stored to float,
 *     then float cos/sin (CT_reconstruction/OSEM.cl:57, :94)            -> xo_trig_*
 *   - subset order, bit reversal for power-of-two ss (GPU.cpp:564-582)  -> xo_subset_order
 *   - OSEM1 (OSEM.cl:38-68), OSEM2 (OSEM.cl:71-105), projection and backProjection
 *     (reconstShare.cl:213-275), AART1 (AART.cl:38-70), FISTAbackProjection
 *     (FISTA.cl:211-246), backProjectionFBP (FBP.cl:164-188)           -> xct_oracle_body.h
 *   - the subset/iteration loop of OSEM_execution (GPU.cpp:125-240)    -> xo_osem_run_*
 *   - the FBP ramp filter chain of FBP_execution (GPU.cpp:745-806 over FBP.cl:34-160)
 *                                                                       -> xo_fbp_filter_*
 *   - the hybrid base-up (GPU.cpp:1538-1566, reconstShare.cl:87-177)   -> xo_base_up_f32
 *   - the rotation-centre search's rotCenterShift, setMask and imgFocusIndex
 *     (RotationCenterSearch/rotCenterSearch.cl:37-232)                  -> xo_rot_center_*,
 *                                                    xo_mask_*, xo_set_mask_f32, xo_focus_index
 *   - reslice and denoiseSinogram (Reslice/reslice.cl:52-71, 223-248) -> xo_reslice_f32,
 *                                                    xo_denoise_sinogram_f32
 *   - the compressed-sensing proximal steps ISTA3D / FISTA3D (FISTA.cl:409-594)
 *                                                 -> xo_ista3d_f32, xo_fista3d_f32
 *
 * Parity pin: the reference ships no tests, fixtures or golden vectors, and its OpenCL
 * runtime is not available, so the pin is oracle/_ref: the reference's own kernel bodies --
 * CT_reconstruction/OSEM.cl, FISTA.cl, reconstShare.cl, FBP.cl,
 * RotationCenterSearch/rotCenterSearch.cl and Reslice/reslice.cl -- compiled with g++
 * against an OpenCL-C shim (recipe: oracle/build_ref.py), driven by host loops that restate
 * the reference's executors.  The literal evaluation order of this oracle matches that build
 * to the last bit on the committed fixtures (tests/).
 * Where oracle/_ref cannot be built (no reference sources present), parity rests on the
 * committed golden fixtures generated here.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off -shared -fPIC (no contraction, so that the
 * literal order really is evaluated as written; FMAs are explicit calls).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xct_oracle.h"

#define XO_PI 3.14159265358979323846

/* ---------------------------------------------------------------- float instantiation */
#define REAL float
#define SFX _f32
#define XO_FMA(a, b, c) fmaf((a), (b), (c))
#define XO_FLOOR(a) floorf(a)
#define XO_SQRT(a) sqrtf(a)
#define XO_FABS(a) fabsf(a)
#include "xct_oracle_body.h"
#undef REAL
#undef SFX
#undef XO_FMA
#undef XO_FLOOR
#undef XO_SQRT
#undef XO_FABS

/* --------------------------------------------------------------- double instantiation */
#define REAL double
#define SFX _f64
#define XO_FMA(a, b, c) fma((a), (b), (c))
#define XO_FLOOR(a) floor(a)
#define XO_SQRT(a) sqrt(a)
#define XO_FABS(a) fabs(a)
#include "xct_oracle_body.h"
#undef REAL
#undef SFX
#undef XO_FMA
#undef XO_FLOOR
#undef XO_SQRT
#undef XO_FABS

/* Per-angle (cos, sin), interleaved.  angle_pr = (float)((double)angle * PI / 180.0)
 * (OSEM.cl:57: float * double-literal PI, stored to a float), then the float cos/sin of
 * that float, taken here as the correctly rounded value (float)cos((double)angle_pr). */
void xo_trig_f32(const float *ang_deg, int pa, float *cs)
{
    for (int th = 0; th < pa; ++th) {
        const float phi = (float)(((double)ang_deg[th] * XO_PI) / 180.0);
        cs[2 * th] = (float)cos((double)phi);
        cs[2 * th + 1] = (float)sin((double)phi);
    }
}

/* FP64 companion: the same angles without any float rounding. */
void xo_trig_f64(const float *ang_deg, int pa, double *cs)
{
    for (int th = 0; th < pa; ++th) {
        const double phi = ((double)ang_deg[th] * XO_PI) / 180.0;
        cs[2 * th] = cos(phi);
        cs[2 * th + 1] = sin(phi);
    }
}

/* Subset order of OSEM_ocl (GPU.cpp:564-582): when ss is a power of two the order is
 * the bit-reversal permutation of 0..ss-1 (0, ss/2, ss/4, 3ss/4, ...); otherwise the
 * identity.  Returns 0. */
int xo_subset_order(int ss, int *sub)
{
    if (ss <= 0) return 0;
    if ((ss & (ss - 1)) == 0) {
        int bits = 0;
        while ((1 << bits) < ss) ++bits;
        for (int j = 0; j < ss; ++j) {
            int r = 0;
            for (int b = 0; b < bits; ++b)
                if (j & (1 << b)) r |= 1 << (bits - 1 - b);
            sub[j] = r;
        }
    } else {
        for (int j = 0; j < ss; ++j) sub[j] = j;
    }
    return 0;
}

int xo_abi_version(void) { return XO_ABI_VERSION; }

/* ---------------------------------------------------------------- FBP ramp filter
 * FBP_execution (GPU.cpp:745-806) runs, per sinogram row th:
 *   spinFactor  W[m] = (cos(d*m), cos(d*m + PI/2)) with d = 2*PI/ZP_SIZE stored to a float
 *               (FBP.cl:34-40): d*m is a float product, d*m + PI_2 a double sum stored to
 *               the float2 component, cos the float cos of that float;
 *   zeroPadding bin X goes to Xswap = (X - px/2) mod zp, imaginary part 0 (FBP.cl:44-57);
 *   bitReverse  xc2[rev(X)] = xc1[X], rev over log2(zp) bits (FBP.cl:60-79);
 *   butterfly   passes i = 1..log2(zp), radix-2 decimation in time with twiddle W[l],
 *               l = (zp >> i) * (X & (2^(i-1) - 1)) (FBP.cl:83-120);
 *   filtering   xc[k] *= (k < zp/2 ? k : zp - k) * h, h = PI/zp stored to a float
 *               (FBP.cl:125-134);
 *   the inverse transform: bitReverse + butterflies with flag 0x80000000, which flips the
 *               sign of W.y (FBP.cl:111), then normalization xc /= zp (FBP.cl:138-145);
 *   outputImage fprj[X] = xc[Xswap].x (FBP.cl:149-160). */
#define XO_PI_2 1.57079632679489661923

static unsigned xo_bitrev(unsigned x, int bits)
{
    unsigned r = 0;
    for (int b = 0; b < 32; ++b)
        if (x & (1u << b)) r |= 1u << (31 - b);
    return bits > 0 ? r >> (32 - bits) : 0u;
}

static int xo_log2(int n)
{
    int b = 0;
    while ((1 << b) < n) ++b;
    return b;
}

typedef struct { float x, y; } xo_c32;
typedef struct { double x, y; } xo_c64;

/* one radix-2 pass (FBP.cl:83-120) over xc[zp]; neg_wy: the inverse transform's flag */
static void xo_butterfly_f32(xo_c32 *xc, const xo_c32 *W, int zp, int it, int neg_wy)
{
    const unsigned size = 1u << (it - 1), dist = 1u << it, num = (unsigned)zp >> it;
    for (unsigned X = 0; X < (unsigned)zp / 2; ++X) {
        const unsigned base = (X >> (it - 1)) * dist, off = X & (size - 1);
        const unsigned a = base + off, b = a + size, l = num * off;
        const xo_c32 xa = xc[a], xb = xc[b];
        xo_c32 wab = W[l];
        if (neg_wy) wab.y = -wab.y;
        const xo_c32 wayx = {-wab.y, wab.x}, wbyx = {wab.y, -wab.x};
        xo_c32 ra, rb;
        ra.x = (xa.x + xb.x * wab.x) + xb.y * wayx.x;
        ra.y = (xa.y + xb.x * wab.y) + xb.y * wayx.y;
        rb.x = (xa.x - xb.x * wab.x) + xb.y * wbyx.x;
        rb.y = (xa.y - xb.x * wab.y) + xb.y * wbyx.y;
        xc[a] = ra;
        xc[b] = rb;
    }
}

void xo_fbp_filter_f32(const float *prj, int px, int nrows, int zp, float *out)
{
    const int bits = xo_log2(zp);
    xo_c32 *W = (xo_c32 *)malloc(sizeof(xo_c32) * (size_t)zp);
    const float d = (float)(2.0 * XO_PI / zp);
    for (int m = 0; m < zp; ++m) {
        const float dm = d * (float)m;
        const float q = (float)((double)dm + XO_PI_2);
        W[m].x = (float)cos((double)dm);
        W[m].y = (float)cos((double)q);
    }
    const float h = (float)(XO_PI / zp);
#pragma omp parallel
    {
        xo_c32 *x1 = (xo_c32 *)malloc(sizeof(xo_c32) * (size_t)zp);
        xo_c32 *x2 = (xo_c32 *)malloc(sizeof(xo_c32) * (size_t)zp);
#pragma omp for schedule(static)
        for (int th = 0; th < nrows; ++th) {
            memset(x1, 0, sizeof(xo_c32) * (size_t)zp);
            for (int X = 0; X < px; ++X) {
                const int xs = (X - px / 2 + zp / 2 < zp / 2) ? X - px / 2 + zp : X - px / 2;
                x1[xs].x = prj[(size_t)th * px + X];
                x1[xs].y = 0.0f;
            }
            for (int X = 0; X < zp; ++X) x2[xo_bitrev((unsigned)X, bits)] = x1[X];
            for (int i = 1; i <= bits; ++i) xo_butterfly_f32(x2, W, zp, i, 0);
            for (int k = 0; k < zp; ++k) {
                const float f = (k < zp / 2) ? (float)k * h : (float)(zp - k) * h;
                x2[k].x *= f;
                x2[k].y *= f;
            }
            for (int X = 0; X < zp; ++X) x1[xo_bitrev((unsigned)X, bits)] = x2[X];
            for (int i = 1; i <= bits; ++i) xo_butterfly_f32(x1, W, zp, i, 1);
            for (int k = 0; k < zp; ++k) {
                x1[k].x /= (float)zp;
                x1[k].y /= (float)zp;
            }
            for (int X = 0; X < px; ++X) {
                const int xs = (X - px / 2 + zp / 2 < zp / 2) ? X - px / 2 + zp : X - px / 2;
                out[(size_t)th * px + X] = x1[xs].x;
            }
        }
        free(x1);
        free(x2);
    }
    free(W);
}

/* The same chain in double with W[m] = exp(-2 pi i m / zp) taken exactly. */
void xo_fbp_filter_f64(const double *prj, int px, int nrows, int zp, double *out)
{
    const int bits = xo_log2(zp);
    xo_c64 *W = (xo_c64 *)malloc(sizeof(xo_c64) * (size_t)zp);
    for (int m = 0; m < zp; ++m) {
        W[m].x = cos(2.0 * XO_PI * m / zp);
        W[m].y = -sin(2.0 * XO_PI * m / zp);
    }
#pragma omp parallel
    {
        xo_c64 *x1 = (xo_c64 *)malloc(sizeof(xo_c64) * (size_t)zp);
        xo_c64 *x2 = (xo_c64 *)malloc(sizeof(xo_c64) * (size_t)zp);
#pragma omp for schedule(static)
        for (int th = 0; th < nrows; ++th) {
            memset(x1, 0, sizeof(xo_c64) * (size_t)zp);
            for (int X = 0; X < px; ++X) {
                const int xs = (X - px / 2 + zp / 2 < zp / 2) ? X - px / 2 + zp : X - px / 2;
                x1[xs].x = prj[(size_t)th * px + X];
            }
            for (int X = 0; X < zp; ++X) x2[xo_bitrev((unsigned)X, bits)] = x1[X];
            for (int pass = 0; pass < 2; ++pass) {
                xo_c64 *xc = pass == 0 ? x2 : x1;
                const double sgn = pass == 0 ? 1.0 : -1.0;
                for (int it = 1; it <= bits; ++it) {
                    const unsigned size = 1u << (it - 1), dist = 1u << it, num = (unsigned)zp >> it;
                    for (unsigned X = 0; X < (unsigned)zp / 2; ++X) {
                        const unsigned a = (X >> (it - 1)) * dist + (X & (size - 1)), b = a + size;
                        const double wx = W[num * (X & (size - 1))].x, wy = sgn * W[num * (X & (size - 1))].y;
                        const double tx = xc[b].x * wx - xc[b].y * wy, ty = xc[b].x * wy + xc[b].y * wx;
                        const xo_c64 xa = xc[a];
                        xc[a].x = xa.x + tx;
                        xc[a].y = xa.y + ty;
                        xc[b].x = xa.x - tx;
                        xc[b].y = xa.y - ty;
                    }
                }
                if (pass == 0) {
                    for (int k = 0; k < zp; ++k) {
                        const double f = (k < zp / 2 ? k : zp - k) * (XO_PI / zp);
                        x2[k].x *= f;
                        x2[k].y *= f;
                    }
                    for (int X = 0; X < zp; ++X) x1[xo_bitrev((unsigned)X, bits)] = x2[X];
                }
            }
            for (int X = 0; X < px; ++X) {
                const int xs = (X - px / 2 + zp / 2 < zp / 2) ? X - px / 2 + zp : X - px / 2;
                out[(size_t)th * px + X] = x1[xs].x / zp;
            }
        }
        free(x1);
        free(x2);
    }
    free(W);
}

/* Hybrid base-up (hybrid_thread, GPU.cpp:1538-1566, FBPcorrection = 1): a = the slice
 * minimum (findMinimumX/Y, reconstShare.cl:111-177), then per pixel (baseUp,
 * reconstShare.cl:87-109) b1 = (v - a)/a (0 when a == 0), g = sum_{i=1..order}
 * (-1)^(i+1) b1^i / i accumulated in float, v -= a * exp(g) with the float exp of g
 * (taken correctly rounded). */
void xo_base_up_f32(float *img, long long n, int order, float *min_out)
{
    float a = INFINITY;
    for (long long i = 0; i < n; ++i) a = fminf(a, img[i]);
    if (min_out) *min_out = a;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
        const float v = img[i];
        float g = 0.0f;
        const float b1 = (a != 0.0f) ? (v - a) / a : 0.0f;
        float b2 = 1.0f, flag = -1.0f;
        for (int k = 1; k <= order; ++k) {
            b2 *= b1;
            flag *= -1.0f;
            g += flag * b2 / (float)k;
        }
        img[i] = v - a * (float)exp((double)g);
    }
}


/* ------------------------------------------------------------- rotation-centre search
 * rotCenterShift (rotCenterSearch.cl:37-49): out[th][X] = the linear sampler at
 * ((X + shift) + 0.5, th + 0.5) of the sinogram, zero beyond its edges:
 * u = ((float)X + shift) + 0.5; i = floor(u - 0.5); a = (u - 0.5) - i;
 * (1 - a) t[i] + a t[i+1]. */
void xo_rot_center_shift_f32(const float *prj, int px, int pa, float shift, float *out)
{
#pragma omp parallel for schedule(static)
    for (int th = 0; th < pa; ++th)
        for (int X = 0; X < px; ++X) {
            const float u = ((float)X + shift) + 0.5f;
            const float uu = u - 0.5f;
            const float fi = floorf(uu);
            const float a = uu - fi;
            const int i = (int)fi;
            const float t0 = (i >= 0 && i < px) ? prj[(size_t)th * px + i] : 0.0f;
            const float t1 = (i + 1 >= 0 && i + 1 < px) ? prj[(size_t)th * px + i + 1] : 0.0f;
            out[(size_t)th * px + X] = (1.0f - a) * t0 + a * t1;
        }
}

/* setMask's constants (rotCenterSearch.cl:58-72): a = ang*PI/180 and ang*PI/180 - PI/2 in
 * double stored to float; p_cnt = (W/2, H/2) in integers; rp = min(W/2 + shift, W/2),
 * rm = max(-W/2 + shift, -W/2); p1 = rp cos(a_max), p2 = rp cos(a_min), p3 = rm cos(a_max),
 * p4 = rm cos(a_min) (float cos of the float components); p_div = p1.x if rp^2 < rm^2
 * else p3.x. */
void xo_mask_params_f32(int W, int H, float shift, float ang_min, float ang_max, float *prm)
{
    const float amin_x = (float)((double)ang_min * XO_PI / 180), amin_y = (float)((double)ang_min * XO_PI / 180 - XO_PI_2);
    const float amax_x = (float)((double)ang_max * XO_PI / 180), amax_y = (float)((double)ang_max * XO_PI / 180 - XO_PI_2);
    const float rp = fminf((float)(W / 2) + shift, (float)(W / 2));
    const float rm = fmaxf((float)(-W / 2) + shift, (float)(-W / 2));
    const float p1x = rp * (float)cos((double)amax_x), p1y = rp * (float)cos((double)amax_y);
    const float p2x = rp * (float)cos((double)amin_x), p2y = rp * (float)cos((double)amin_y);
    const float p3x = rm * (float)cos((double)amax_x), p3y = rm * (float)cos((double)amax_y);
    const float p4x = rm * (float)cos((double)amin_x), p4y = rm * (float)cos((double)amin_y);
    prm[0] = rp;
    prm[1] = rm;
    prm[2] = p1x;
    prm[3] = p1y;
    prm[4] = p2x;
    prm[5] = p2y;
    prm[6] = p3x;
    prm[7] = p3y;
    prm[8] = p4x;
    prm[9] = p4y;
    prm[10] = (rp * rp < rm * rm) ? p1x : p3x;
    prm[11] = (float)(W / 2);
    prm[12] = (float)(H / 2);
}

/* setMask's per-pixel test (rotCenterSearch.cl:79-95); dot(a, b) = a.x*b.x + a.y*b.y. */
static int xo_mask_at(const float *prm, int x, int y)
{
    const float X = (float)x - prm[11], Y = (float)y - prm[12];
    const float rp = prm[0], rm = prm[1], pd = prm[10];
    const int b1 = X * prm[2] + Y * prm[3] <= rp * rp;
    const int b2 = X * prm[4] + Y * prm[5] <= rp * rp;
    const int b3 = X * prm[6] + Y * prm[7] <= rm * rm;
    const int b4 = X * prm[8] + Y * prm[9] <= rm * rm;
    const float d2 = X * X + Y * Y;
    const int b5 = d2 <= rp * rp && X > pd;
    const int b6 = d2 <= rm * rm && X <= pd;
    return b1 && b2 && b3 && b4 && (b5 || b6);
}

void xo_set_mask_f32(int W, int H, int w_visit, const float *prm, float *mask)
{
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) mask[(size_t)y * W + x] = (x < w_visit && xo_mask_at(prm, x, y)) ? 1.0f : 0.0f;
}

static float xo_tex2(const float *im, int W, int H, int x, int y)
{
    return (x >= 0 && y >= 0 && x < W && y < H) ? im[(size_t)y * W + x] : 0.0f;
}

/* imgFocusIndex's per-pixel terms (rotCenterSearch.cl:178-224): the product of the nine
 * masks of the 3x3 neighbourhood, and the squared differences to the neighbours u, d, r, l,
 * ur, dr, ul, dl (u = y+1, r = x+1) summed in that order, divided by a*a, where the
 * product is 1. */
static void xo_focus_terms(const float *img, const float *mask, int W, int H, int x, int y, float *sq, float *mt)
{
    static const int dx[8] = {0, 0, 1, -1, 1, 1, -1, -1}, dy[8] = {1, -1, 0, 0, 1, -1, 1, -1};
    float m = xo_tex2(mask, W, H, x, y);
    for (int k = 0; k < 8; ++k) m *= xo_tex2(mask, W, H, x + dx[k], y + dy[k]);
    const float a = xo_tex2(img, W, H, x, y);
    float s = 0.0f;
    for (int k = 0; k < 8; ++k) {
        const float d = xo_tex2(img, W, H, x + dx[k], y + dy[k]) - a;
        s += (m == 1.0f) ? d * d : 0.0f;
    }
    s /= (m == 1.0f) ? a * a : 1.0f;
    *sq = s;
    *mt = m;
}

double xo_focus_index(const float *img, const float *mask, int W, int H, int L)
{
    if (L <= 0) {
        double s = 0.0, m = 0.0;
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                float a, b;
                xo_focus_terms(img, mask, W, H, x, y, &a, &b);
                s += a;
                m += b;
            }
        return sqrt(s / m);
    }
    /* work-item lid sums pixels x = lid + i*L (i < W/L) row by row in float; then the
     * local-memory tree: loc[id] += loc[id + s] for s = L/2, L/4, ..., 1 */
    float *ls = (float *)calloc((size_t)L, sizeof(float)), *lm = (float *)calloc((size_t)L, sizeof(float));
    for (int lid = 0; lid < L; ++lid)
        for (int y = 0; y < H; ++y)
            for (int i = 0; i < W / L; ++i) {
                float a, b;
                xo_focus_terms(img, mask, W, H, lid + i * L, y, &a, &b);
                ls[lid] += a;
                lm[lid] += b;
            }
    for (int st = L / 2; st > 0; st >>= 1)
        for (int id = 0; id < st; ++id) {
            ls[id] += ls[id + st];
            lm[id] += lm[id + st];
        }
    const float r = sqrtf(ls[0] / lm[0]);
    free(ls);
    free(lm);
    return r;
}


/* ------------------------------------------------------------------------ reslice
 * reslice (reslice.cl:52-71): prj[Y][th][X] = the linear sampler (zero border) of
 * projection th at ((X + xs[th]) + 0.5, (Y + ys[th]) + 0.5), plus baseup; with
 * correction, times cos(asin(theta)), theta = 2|X - W/2.0|/W (float cos/asin, taken
 * correctly rounded).  The sampler's sum is evaluated as written in the OpenCL 1.2
 * filtering formula: (1-a)(1-b) T00 + a(1-b) T10 + (1-a) b T01 + a b T11. */
void xo_reslice_f32(const float *mt, int W, int H, int A, const float *xs, const float *ys, float baseup,
                    int correction, float *prj)
{
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < H; ++Y)
        for (int th = 0; th < A; ++th) {
            const float *im = mt + (size_t)th * H * W;
            const float sx = xs ? xs[th] : 0.0f, sy = ys ? ys[th] : 0.0f;
            for (int X = 0; X < W; ++X) {
                const float uu = (((float)X + sx) + 0.5f) - 0.5f, vv = (((float)Y + sy) + 0.5f) - 0.5f;
                const float fi = floorf(uu), fj = floorf(vv);
                const float a = uu - fi, b = vv - fj;
                const int i = (int)fi, j = (int)fj;
                float t = (1.0f - a) * (1.0f - b) * xo_tex2(im, W, H, i, j) + a * (1.0f - b) * xo_tex2(im, W, H, i + 1, j) +
                          (1.0f - a) * b * xo_tex2(im, W, H, i, j + 1) + a * b * xo_tex2(im, W, H, i + 1, j + 1);
                t += baseup;
                if (correction == 1) {
                    const float theta = 2.0f * fabsf((float)X - (float)W / 2.0f) / (float)W;
                    t *= (float)cos((double)(float)asin((double)theta));
                }
                prj[((size_t)Y * A + th) * W + X] = t;
            }
        }
}

/* denoiseSinogram (reslice.cl:223-248): f1 = s[th], f2 = s[th+1], f3 = s[th-1] with the
 * angle index clamped to the edge; where the row is a one-angle spike (f2 - f1 and f1 - f3
 * both beyond the threshold, with opposite signs) it becomes (f2 + f3)/2. */
void xo_denoise_sinogram_f32(const float *src, int W, int A, int H, float threshold, float *dst)
{
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < H; ++Y)
        for (int th = 0; th < A; ++th) {
            const float *r1 = src + ((size_t)Y * A + th) * W;
            const float *r2 = src + ((size_t)Y * A + (th + 1 < A ? th + 1 : A - 1)) * W;
            const float *r3 = src + ((size_t)Y * A + (th > 0 ? th - 1 : 0)) * W;
            for (int X = 0; X < W; ++X) {
                const float f1 = r1[X], f2 = r2[X], f3 = r3[X];
                const float d1 = f2 - f1, d2 = f1 - f3;
                const float c = (f2 + f3) / 2.0f;
                dst[((size_t)Y * A + th) * W + X] =
                    ((d1 > threshold && d2 < -threshold) || (d1 < -threshold && d2 > threshold)) ? c : f1;
            }
        }
}


/* ------------------------------------------------- compressed sensing (ISTA3D / FISTA3D)
 * Per voxel (FISTA.cl:409-494): the six neighbours of v -- x+1, x-1, y+1, y-1 (zero outside
 * the slice), layer min(Z+1, dN-1), and layer 0 (the kernels take fmin(Z-1, 0), :425) --
 * sorted in descending order by the kernel's exchange loop; then the candidate chain
 * x = v - 6l, n0, v - 4l, n1, v - 2l, n2, v, n3, v + 2l, n4, v + 4l, n5, v + 6l selected by
 * v < n0 + 6l, n0 + 4l, n1 + 4l, n1 + 2l, n2 + 2l, n2, n3, n3 - 2l, n4 - 2l, n4 - 4l,
 * n5 - 4l, n5 - 6l (the last true comparison wins): the minimiser of
 * (x - v)^2/2 + l sum_k |x - n_k| (the l1 distance to the neighbours).  ISTA3D then floors
 * at 1e-6 (NaN -> 1e-6). */
static float xo_cs_select(const float *v, int nx, int ny, int dN, int X, int Y, int Z, float lambda)
{
    const size_t m = (size_t)nx * ny;
    const float *vz = v + (size_t)Z * m;
    float nb[6];
    nb[0] = xo_tex2(vz, nx, ny, X + 1, Y);
    nb[1] = xo_tex2(vz, nx, ny, X - 1, Y);
    nb[2] = xo_tex2(vz, nx, ny, X, Y + 1);
    nb[3] = xo_tex2(vz, nx, ny, X, Y - 1);
    const int zp = Z + 1 < dN - 1 ? Z + 1 : dN - 1;
    nb[4] = v[(size_t)zp * m + (size_t)Y * nx + X];
    nb[5] = v[(size_t)Y * nx + X];
    const float vi = vz[(size_t)Y * nx + X];
    for (int i = 0; i < 6; ++i) {
        const float img1 = nb[i];
        float img2 = img1;
        int bigger = i;
        for (int j = i + 1; j < 6; ++j) {
            bigger = (nb[j] > img2) ? j : bigger;
            img2 = (nb[j] > img2) ? nb[j] : img2;
        }
        nb[i] = img2;
        nb[bigger] = img1;
    }
    const float l2 = 2.0f * lambda, l4 = 4.0f * lambda, l6 = 6.0f * lambda;
    const float cnd[13] = {vi - l6, nb[0], vi - l4, nb[1], vi - l2, nb[2], vi,
                           nb[3],   vi + l2, nb[4], vi + l4, nb[5], vi + l6};
    const float rng[12] = {nb[0] + l6, nb[0] + l4, nb[1] + l4, nb[1] + l2, nb[2] + l2, nb[2],
                           nb[3],      nb[3] - l2, nb[4] - l2, nb[4] - l4, nb[5] - l4, nb[5] - l6};
    float x = cnd[0];
    for (int i = 0; i < 12; ++i) x = (vi < rng[i]) ? cnd[i + 1] : x;
    return x;
}

void xo_ista3d_f32(const float *v, int nx, int ny, int dN, float lambda, float *x_new)
{
#pragma omp parallel for collapse(2) schedule(static)
    for (int Z = 0; Z < dN; ++Z)
        for (int Y = 0; Y < ny; ++Y)
            for (int X = 0; X < nx; ++X) {
                float x = xo_cs_select(v, nx, ny, dN, X, Y, Z, lambda);
                x = fmaxf(1.0e-6f, x);
                x = (x != x) ? 1.0e-6f : x;
                x_new[((size_t)Z * ny + Y) * nx + X] = x;
            }
}

/* FISTA3D (FISTA.cl:497-594): the same selection on v (no floor), then
 * beta' = (sqrt(4 beta^2 + 1) + 1)/2, gamma = (beta - 1)/beta',
 * w' = gamma x' + (1 - gamma) x_in (NaN -> 1e-6), all in float as written. */
void xo_fista3d_f32(const float *x_in, const float *v, const float *beta, int nx, int ny, int dN, float lambda,
                    float *w_new, float *x_new, float *beta_new)
{
#pragma omp parallel for collapse(2) schedule(static)
    for (int Z = 0; Z < dN; ++Z)
        for (int Y = 0; Y < ny; ++Y)
            for (int X = 0; X < nx; ++X) {
                const size_t i = ((size_t)Z * ny + Y) * nx + X;
                const float xi = x_in[i], b = beta[i];
                const float x = xo_cs_select(v, nx, ny, dN, X, Y, Z, lambda);
                x_new[i] = x;
                float bn = b * b * 4.0f + 1.0f;
                bn = (sqrtf(bn) + 1.0f) * 0.5f;
                const float g = (b - 1.0f) / bn;
                beta_new[i] = bn;
                float w = g * x + (1.0f - g) * xi;
                w_new[i] = (w != w) ? 1.0e-6f : w;
            }
}

/* ------------------------------------------------------------ FISTA with compressed sensing
 * The Lipschitz estimate of the subset operators (powerIteration, GPU.cpp:2079-2188, over
 * the kernels powerIter1/2/3, imageL2AbsX/Y of FISTA.cl:50-208) and FISTA_execution
 * (GPU.cpp:1755-1924), float, in the kernels' literal order. */

/* Bilinear read with the linear sampler at unnormalised (u, v) on one [h][w] image, zero
 * border: texel coordinates (u - 0.5, v - 0.5), weights as the OpenCL 1.2 specification
 * writes them. */
static float xo_linear_(const float *img, int w, int h, float u, float v)
{
    const float uu = u - 0.5f, vv = v - 0.5f;
    const float fi = floorf(uu), fj = floorf(vv);
    const float a = uu - fi, b = vv - fj;
    const int i = (int)fi, j = (int)fj;
    const float t00 = xo_tex__f32(img, w, h, i, j), t10 = xo_tex__f32(img, w, h, i + 1, j);
    const float t01 = xo_tex__f32(img, w, h, i, j + 1), t11 = xo_tex__f32(img, w, h, i + 1, j + 1);
    return (1.0f - a) * (1.0f - b) * t00 + a * (1.0f - b) * t10 + (1.0f - a) * b * t01 + a * b * t11;
}

/* A linear-sampler read at INTEGER coordinates (undefined in OpenCL 1.2): the exact texel
 * (fetch_mode 0) or the 2x2 average of texels (X-1..X, Y-1..Y) (fetch_mode 1). */
static float xo_int_linear_(const float *img, int w, int h, int X, int Y, int fetch_mode)
{
    if (fetch_mode == 0) return xo_tex__f32(img, w, h, X, Y);
    return 0.25f * (((xo_tex__f32(img, w, h, X - 1, Y - 1) + xo_tex__f32(img, w, h, X, Y - 1)) +
                     xo_tex__f32(img, w, h, X - 1, Y)) +
                    xo_tex__f32(img, w, h, X, Y));
}

/* imageL2AbsX then imageL2AbsY of one [ny][nx] image with work-groups of wg items: each item
 * sums the squares at X = lid + i*wg, i < nx/wg (then Y likewise), then the tree
 * loc[lid] += loc[lid + s] for s = wg/2, wg/4, ..., 1 (FISTA.cl:133-208). */
static float xo_l2_wg_(const float *img, int nx, int ny, int wg)
{
    float *loc = (float *)malloc(sizeof(float) * (size_t)wg);
    float *rows = (float *)malloc(sizeof(float) * (size_t)ny);
    if (!loc || !rows) {
        free(loc);
        free(rows);
        return NAN;
    }
    for (int Y = 0; Y < ny; ++Y) {
        for (int l = 0; l < wg; ++l) {
            loc[l] = 0.0f;
            for (int i = 0; i < nx / wg; ++i) {
                const float v = img[(size_t)Y * nx + l + i * wg];
                loc[l] += v * v;
            }
        }
        for (int s = wg / 2; s > 0; s >>= 1)
            for (int l = 0; l < s; ++l) loc[l] += loc[l + s];
        rows[Y] = loc[0];
    }
    for (int l = 0; l < wg; ++l) {
        loc[l] = 0.0f;
        for (int i = 0; i < ny / wg; ++i) loc[l] += rows[l + i * wg];
    }
    for (int s = wg / 2; s > 0; s >>= 1)
        for (int l = 0; l < s; ++l) loc[l] += loc[l + s];
    const float r = loc[0];
    free(loc);
    free(rows);
    return r;
}

/* layer_mode: powerIter1 declares its sampling coordinate without setting the layer
 * (FISTA.cl:60, `float4 xyz;` and xyz.z never written), so which layer it projects is
 * undefined; 0 reads layer 0 for every subset (a zero-initialised coordinate, as the OpenCL-C
 * shim and a cleared register give), 1 reads the subset's own layer (the evident intent). */
void xo_power_iteration_f32(const float *cs, const xo_geom *g, int trials, int work_group, int layer_mode, float *L)
{
    const int nx = g->nx, ny = g->ny, px = g->px, pa = g->pa, ss = g->ss, D = g->depth;
    const int wg = work_group < nx ? work_group : nx; /* min(CL_DEVICE_MAX_WORK_GROUP_SIZE, g_ox) */
    const int rows = pa / ss;
    const size_t nimg = (size_t)nx * ny;
    float *img = (float *)malloc(sizeof(float) * nimg * ss);
    float *cnd = (float *)malloc(sizeof(float) * nimg * ss);
    float *prj = (float *)malloc(sizeof(float) * (size_t)px * (rows > 0 ? rows : 1) * ss);
    float *l2 = (float *)calloc((size_t)ss, sizeof(float));
    if (!img || !cnd || !prj || !l2) goto done;
    for (size_t i = 0; i < nimg * ss; ++i) img[i] = 1.0f; /* the fill of GPU.cpp:2122 */
    {
        const float scale = ((float)ss / (float)pa) / (float)D;
        for (int trial = 0; trial < trials; ++trial) {
            /* powerIter1 over (px, pa/ss, ss): ray sums of subset z's rows of the read layer,
             * integer half sizes, no +0.5 */
#pragma omp parallel for collapse(3) schedule(static)
            for (int z = 0; z < ss; ++z)
                for (int k = 0; k < rows; ++k)
                    for (int X = 0; X < px; ++X) {
                        const int th = z + k * ss;
                        const float c = cs[2 * th], s = cs[2 * th + 1];
                        const float *im = img + (layer_mode ? (size_t)z * nimg : 0);
                        float acc = 0.0f;
                        for (int Y = 0; Y < D; ++Y) {
                            const float u = ((float)(X - px / 2) * c + (float)(Y - D / 2) * s) + (float)(nx / 2);
                            const float v = ((float)(-(X - px / 2)) * s + (float)(Y - D / 2) * c) + (float)(ny / 2);
                            acc += xo_linear_(im, nx, ny, u, v);
                        }
                        prj[((size_t)z * rows + k) * px + X] = acc;
                    }
            /* powerIter2 over (nx, ny, ss): nearest-bin backprojection, floor rule, * ss/pa/D */
#pragma omp parallel for collapse(2) schedule(static)
            for (int z = 0; z < ss; ++z)
                for (int Y = 0; Y < ny; ++Y)
                    for (int X = 0; X < nx; ++X) {
                        float b = 0.0f;
                        for (int k = 0; k < rows; ++k) {
                            const int th = z + k * ss;
                            const float c = cs[2 * th], s = cs[2 * th + 1];
                            const float t = ((float)(X - nx / 2) * c - (float)(Y - ny / 2) * s) + (float)(px / 2);
                            const int bin = (int)floorf(t);
                            b += (bin >= 0 && bin < px) ? prj[((size_t)z * rows + k) * px + bin] : 0.0f;
                        }
                        cnd[(size_t)z * nimg + (size_t)Y * nx + X] = b * scale;
                    }
            for (int z = 0; z < ss; ++z) l2[z] = xo_l2_wg_(cnd + (size_t)z * nimg, nx, ny, wg);
            /* powerIter3: normalise (the candidate read at integer coordinates, linear sampler) */
#pragma omp parallel for collapse(2) schedule(static)
            for (int z = 0; z < ss; ++z)
                for (int Y = 0; Y < ny; ++Y)
                    for (int X = 0; X < nx; ++X)
                        img[(size_t)z * nimg + (size_t)Y * nx + X] =
                            xo_int_linear_(cnd + (size_t)z * nimg, nx, ny, X, Y, g->fetch_mode) / sqrtf(l2[z]);
        }
        for (int z = 0; z < ss; ++z) L[z] = l2[z];
    }
done:
    free(img);
    free(cnd);
    free(prj);
    free(l2);
}

/* FISTA_execution for dN slices: imgs [dN][ny][nx] (out), meas [dN][pa][px] the sinograms the
 * kernels read (already corrected when correctionMode > 0), res0 [dN][pa][px] the initial
 * content of the residual image (the uncorrected sinograms with a correction -- GPU.cpp:1812
 * copies them there -- else zeros: rows AART1 never writes keep it), L [ss] from the power
 * iteration, lambda_d the -D LAMBDA_FISTA value.  flags bit 1: store each FISTA3D x_{t+1} as
 * the next image (the reference binds that output to the beta image, GPU.cpp:1867-1868, so
 * its image is the first cycle's ISTA3D result). */
void xo_fista_run_f32(float *imgs, const float *meas, const float *res0, const float *cs, const xo_geom *g, int dN,
                      const int *sub, int it, float alpha, const float *L, double lambda_d, int flags)
{
    const int nx = g->nx, ny = g->ny, px = g->px, pa = g->pa, ss = g->ss;
    const size_t nimg = (size_t)nx * ny, nprj = (size_t)px * pa, all = nimg * dN;
    float *x = imgs;
    float *dest = (float *)malloc(sizeof(float) * all), *v = (float *)malloc(sizeof(float) * all);
    float *w = (float *)malloc(sizeof(float) * all), *beta = (float *)calloc(all, sizeof(float));
    float *tw = (float *)malloc(sizeof(float) * all), *tx = (float *)malloc(sizeof(float) * all);
    float *tb = (float *)malloc(sizeof(float) * all), *res = (float *)malloc(sizeof(float) * nprj * dN);
    if (!dest || !v || !w || !beta || !tw || !tx || !tb || !res) goto done;
    memcpy(res, res0, sizeof(float) * nprj * dN);
    for (int z = 0; z < dN; ++z) xo_backprojection_f32(meas + z * nprj, cs, g, sub[0], dest + z * nimg);
    memcpy(x, dest, sizeof(float) * all);
    memcpy(w, x, sizeof(float) * all);
    {
        const float *X = x;
        int first = 1;
        for (int i = 0; i < it; ++i)
            for (int k = 0; k < ss; ++k) {
                const int s = sub[k];
                for (int z = 0; z < dN; ++z) {
                    xo_aart1_f32(X + z * nimg, meas + z * nprj, cs, g, s, pa / ss, res + z * nprj);
                    xo_fista_bp_f32(X + z * nimg, v + z * nimg, res + z * nprj, cs, g, s, alpha, L[s]);
                }
                const float lam = (float)(lambda_d / (double)L[s] * 0.5);
                if (first) {
                    xo_ista3d_f32(v, nx, ny, dN, lam, dest);
                    X = w;
                    first = 0;
                } else {
                    xo_fista3d_f32(x, v, beta, nx, ny, dN, lam, tw, tx, tb);
                    memcpy(w, tw, sizeof(float) * all);
                    memcpy(beta, tb, sizeof(float) * all);
                    if (flags & 1) memcpy(dest, tx, sizeof(float) * all);
                }
                memcpy(x, dest, sizeof(float) * all);
            }
    }
done:
    free(dest);
    free(v);
    free(w);
    free(beta);
    free(tw);
    free(tx);
    free(tb);
    free(res);
}
