/*
 * xct_oracle_body.h -- type-generic body of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Included twice by xct_oracle.c, once with REAL=float (suffix _f32) and once with
 * REAL=double (suffix _f64).  Nothing in the product links this code: only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it, as the
 * checker.
 *
 * Every function restates one piece of the reference OS-EM path of
 * NozomuIshiguro/CT-XAFS_analysis (CT_reconstruction/).  The OpenCL image-sampler
 * semantics that the reference kernels rely on (reconstShare.cl:32-33) are written out
 * explicitly, following the OpenCL 1.2 specification:
 *   - unnormalised coordinates, CLK_ADDRESS_CLAMP: texels outside the image read as the
 *     border colour, whose .x is 0 for a CL_R image;
 *   - CLK_FILTER_LINEAR: i0 = floor(u - 0.5), a = frac(u - 0.5), same for v, and
 *     T = (1-a)(1-b)T00 + a(1-b)T10 + (1-a)b T01 + ab T11;
 *   - CLK_FILTER_NEAREST: i = floor(u).
 *
 * Two evaluation orders are provided, separately for the forward projector and the
 * backprojector (OpenCL leaves FP contraction to the compiler, so the reference's own
 * rounding at the last bit is implementation-defined):
 *   literal   (XO_ORDER_FWD_LITERAL / XO_ORDER_BP_LITERAL bits set): the expressions
 *             exactly as written in the .cl source, evaluated left to right with no
 *             contraction, and the specification's four-product bilinear formula;
 *   canonical (bit clear): the fused multiply-add order (coordinates as two FMAs from
 *             per-ray bases, bilinear as three FMA lerps; bin coordinate as two FMAs).
 * XO_ORDER_GPU (canonical forward, literal backprojector) is what the CUDA kernels
 * compute: every forward sample and every backprojection bin index agree bit for bit.
 * The forward order changes results by ~1e-7 relative; the backprojector's nearest-bin
 * rule is discontinuous, so its bin arithmetic is kept literal.
 */

#ifndef REAL
#error "define REAL and SFX before including xct_oracle_body.h"
#endif

#define XO_CAT2(a, b) a##b
#define XO_CAT(a, b) XO_CAT2(a, b)
#define FN(name) XO_CAT(name, SFX)

/* Texel fetch with CLK_ADDRESS_CLAMP and a zero border (CL_R border colour .x == 0). */
static inline REAL FN(xo_tex_)(const REAL *img, int w, int h, int i, int j)
{
    if (i < 0 || j < 0 || i >= w || j >= h) return (REAL)0;
    return img[(size_t)j * (size_t)w + (size_t)i];
}

/* One ray sum: the Y loop of OSEM1 / projection / AART1
 * (CT_reconstruction/OSEM.cl:56-62, reconstShare.cl:232-238, AART.cl:56-62).
 * Samples are summed sequentially in Y order, as the reference work-item does. */
static REAL FN(xo_raysum_)(const REAL *img, const xo_geom *g, REAL c, REAL s, int X)
{
    const int D = g->depth;
    const REAL hx = (REAL)g->nx * (REAL)0.5;
    const REAL hy = (REAL)g->ny * (REAL)0.5;
    const REAL hd = (REAL)D * (REAL)0.5;
    const REAL Xc = (REAL)X - (REAL)g->cx;
    REAL acc = (REAL)0;
    if (!(g->order & XO_ORDER_FWD_LITERAL)) {
        const REAL ax = XO_FMA(Xc, c, hx);
        const REAL ay = XO_FMA(Xc, -s, hy);
        for (int Y = 0; Y < D; ++Y) {
            const REAL Yc = (REAL)Y - hd;
            const REAL x = XO_FMA(Yc, s, ax);
            const REAL y = XO_FMA(Yc, c, ay);
            const REAL fi = XO_FLOOR(x), fj = XO_FLOOR(y);
            const REAL a = x - fi, b = y - fj;
            const int i = (int)fi, j = (int)fj;
            const REAL t00 = FN(xo_tex_)(img, g->nx, g->ny, i, j);
            const REAL t10 = FN(xo_tex_)(img, g->nx, g->ny, i + 1, j);
            const REAL t01 = FN(xo_tex_)(img, g->nx, g->ny, i, j + 1);
            const REAL t11 = FN(xo_tex_)(img, g->nx, g->ny, i + 1, j + 1);
            const REAL r0 = XO_FMA(a, t10 - t00, t00);
            const REAL r1 = XO_FMA(a, t11 - t01, t01);
            acc += XO_FMA(b, r1 - r0, r0);
        }
    } else {
        for (int Y = 0; Y < D; ++Y) {
            const REAL Yc = (REAL)Y - hd;
            /* xyz.x/xyz.y of OSEM.cl:58-59, left to right, then the sampler's -0.5 */
            const REAL u = (((Xc * c) + (Yc * s)) + hx) + (REAL)0.5;
            const REAL v = ((((-Xc) * s) + (Yc * c)) + hy) + (REAL)0.5;
            const REAL uu = u - (REAL)0.5, vv = v - (REAL)0.5;
            const REAL fi = XO_FLOOR(uu), fj = XO_FLOOR(vv);
            const REAL a = uu - fi, b = vv - fj;
            const int i = (int)fi, j = (int)fj;
            const REAL t00 = FN(xo_tex_)(img, g->nx, g->ny, i, j);
            const REAL t10 = FN(xo_tex_)(img, g->nx, g->ny, i + 1, j);
            const REAL t01 = FN(xo_tex_)(img, g->nx, g->ny, i, j + 1);
            const REAL t11 = FN(xo_tex_)(img, g->nx, g->ny, i + 1, j + 1);
            const REAL one = (REAL)1;
            acc += (one - a) * (one - b) * t00 + a * (one - b) * t10 + (one - a) * b * t01 + a * b * t11;
        }
    }
    return acc;
}

/* Detector bin hit by pixel (X, Y) at angle (c, s): the XthZ.x expression of
 * OSEM2 (OSEM.cl:95) under the nearest sampler (floor). */
static inline int FN(xo_bin_)(const xo_geom *g, REAL c, REAL s, int X, int Y)
{
    const REAL Xc = (REAL)X - (REAL)g->nx * (REAL)0.5;
    const REAL Yc = (REAL)Y - (REAL)g->ny * (REAL)0.5;
    REAL t;
    if (!(g->order & XO_ORDER_BP_LITERAL)) {
        const REAL bt = XO_FMA(Yc, -s, (REAL)g->cx + (REAL)0.5);
        t = XO_FMA(Xc, c, bt);
    } else {
        t = (((Xc * c) - (Yc * s)) + (REAL)g->cx) + (REAL)0.5;
    }
    return (int)XO_FLOOR(t);
}

/* Measured value y_i as OSEM1 reads it (OSEM.cl:64): read_imagef with a LINEAR sampler
 * at INTEGER coordinates, which OpenCL 1.2 leaves undefined.  fetch_mode 0 takes the
 * exact texel; fetch_mode 1 emulates "int -> float then linear", i.e. the average of
 * texels (X-1..X, th-1..th) with the zero border. */
static inline REAL FN(xo_measured_)(const REAL *meas, const xo_geom *g, int X, int th)
{
    if (g->fetch_mode == 0) return meas[(size_t)th * g->px + X];
    const REAL q = (REAL)0.25;
    return q * (FN(xo_tex_)(meas, g->px, g->pa, X - 1, th - 1) + FN(xo_tex_)(meas, g->px, g->pa, X, th - 1) +
                FN(xo_tex_)(meas, g->px, g->pa, X - 1, th) + FN(xo_tex_)(meas, g->px, g->pa, X, th));
}

/* projection (reconstShare.cl:213-241): rows th = sub + k*ss, k < nrows.
 * cs holds (cos, sin) per angle, interleaved. */
void FN(xo_projection)(const REAL *img, const REAL *cs, const xo_geom *g, int sub, int ss, int nrows, REAL *prj)
{
    const int px = g->px;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nrows; ++k)
        for (int X = 0; X < px; ++X) {
            const int th = sub + k * ss;
            prj[(size_t)th * px + X] = FN(xo_raysum_)(img, g, cs[2 * th], cs[2 * th + 1], X);
        }
}

/* Exact adjoint A^T of xo_projection over all angles (no counterpart in the reference,
 * whose backprojectors are pixel-driven nearest/linear rules): every sample of every ray
 * scatters sino[th][X] with its bilinear weights (1-a)(1-b), a(1-b), (1-a)b, ab onto its
 * 2x2 footprint (texels outside the image dropped).  Sequential, single thread. */
void FN(xo_adjoint)(const REAL *sino, const REAL *cs, const xo_geom *g, REAL *img)
{
    const int D = g->depth, nx = g->nx, ny = g->ny;
    const REAL hx = (REAL)nx * (REAL)0.5, hy = (REAL)ny * (REAL)0.5, hd = (REAL)D * (REAL)0.5;
    memset(img, 0, sizeof(REAL) * (size_t)nx * ny);
    for (int th = 0; th < g->pa; ++th) {
        const REAL c = cs[2 * th], s = cs[2 * th + 1];
        for (int X = 0; X < g->px; ++X) {
            const REAL v = sino[(size_t)th * g->px + X];
            if (v == (REAL)0) continue;
            const REAL Xc = (REAL)X - (REAL)g->cx;
            const REAL ax = XO_FMA(Xc, c, hx), ay = XO_FMA(Xc, -s, hy);
            for (int Y = 0; Y < D; ++Y) {
                const REAL Yc = (REAL)Y - hd;
                const REAL x = XO_FMA(Yc, s, ax), y = XO_FMA(Yc, c, ay);
                const REAL fi = XO_FLOOR(x), fj = XO_FLOOR(y);
                const REAL a = x - fi, b = y - fj;
                const int i = (int)fi, j = (int)fj;
                const REAL w[4] = {((REAL)1 - a) * ((REAL)1 - b), a * ((REAL)1 - b), ((REAL)1 - a) * b, a * b};
                const int ii[4] = {i, i + 1, i, i + 1}, jj[4] = {j, j, j + 1, j + 1};
                for (int q = 0; q < 4; ++q)
                    if (ii[q] >= 0 && jj[q] >= 0 && ii[q] < nx && jj[q] < ny)
                        img[(size_t)jj[q] * nx + ii[q]] += w[q] * v;
            }
        }
    }
}

/* OSEM1 (OSEM.cl:38-68): forward-project subset rows and write the measured/estimated
 * ratio r = (prj < 1e-4) ? m : m / prj with m = max(1e-6, y), NaN -> 1e-6. */
void FN(xo_osem1)(const REAL *img, const REAL *meas, const REAL *cs, const xo_geom *g, int sub, int nrows,
                  REAL *ratio)
{
    const int px = g->px, ss = g->ss;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nrows; ++k)
        for (int X = 0; X < px; ++X) {
            const int th = sub + k * ss;
            const REAL p = FN(xo_raysum_)(img, g, cs[2 * th], cs[2 * th + 1], X);
            const REAL y = FN(xo_measured_)(meas, g, X, th);
            /* max(1e-6, y) followed by the isnan guard: NaN and anything below 1e-6
             * become 1e-6 */
            const REAL m = (y > (REAL)1.0e-6f) ? y : (REAL)1.0e-6f;
            ratio[(size_t)th * px + X] = (p < (REAL)0.0001f) ? m : m / p;
        }
}

/* OSEM2 (OSEM.cl:71-105): nearest-bin backprojection of the ratio over th = sub;
 * th < pa; th += ss (summed in that order), then x <- ((x * b) * ss) / pa, NaN -> 1e-6.
 * Writes dst; src and dst may be the same buffer (each pixel only reads itself). */
void FN(xo_osem2)(const REAL *src, REAL *dst, const REAL *ratio, const REAL *cs, const xo_geom *g, int sub)
{
    const int nx = g->nx, ny = g->ny, px = g->px, pa = g->pa, ss = g->ss;
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < ny; ++Y)
        for (int X = 0; X < nx; ++X) {
            REAL b = (REAL)0;
            for (int th = sub; th < pa; th += ss) {
                const int bin = FN(xo_bin_)(g, cs[2 * th], cs[2 * th + 1], X, Y);
                b += (bin >= 0 && bin < px) ? ratio[(size_t)th * px + bin] : (REAL)0;
            }
            REAL v = src[(size_t)Y * nx + X] * b;
            v = v * (REAL)ss;
            v = v / (REAL)pa;
            dst[(size_t)Y * nx + X] = (v != v) ? (REAL)1.0e-6f : v;
        }
}

/* backProjection (reconstShare.cl:245-275): plain nearest backprojection over the
 * subset, NaN samples -> 0, scaled by ss / pa / depth.  Note the INTEGER halves
 * IMAGESIZE_X/2, IMAGESIZE_Y/2, PRJ_IMAGESIZE/2 of :265 (they truncate for odd sizes). */
void FN(xo_backprojection)(const REAL *prj, const REAL *cs, const xo_geom *g, int sub, REAL *dst)
{
    const int nx = g->nx, ny = g->ny, px = g->px, pa = g->pa, ss = g->ss;
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < ny; ++Y)
        for (int X = 0; X < nx; ++X) {
            REAL b = (REAL)0;
            const REAL Xc = (REAL)(X - nx / 2), Yc = (REAL)(Y - ny / 2);
            for (int th = sub; th < pa; th += ss) {
                const REAL c = cs[2 * th], s = cs[2 * th + 1];
                REAL t;
                if (!(g->order & XO_ORDER_BP_LITERAL)) {
                    t = XO_FMA(Xc, c, XO_FMA(Yc, -s, (REAL)(px / 2) + (REAL)0.5));
                } else {
                    t = (((Xc * c) - (Yc * s)) + (REAL)(px / 2)) + (REAL)0.5;
                }
                const int bin = (int)XO_FLOOR(t);
                REAL p = (bin >= 0 && bin < px) ? prj[(size_t)th * px + bin] : (REAL)0;
                p = (p != p) ? (REAL)0 : p;
                b += p;
            }
            REAL v = b * (REAL)ss;
            v = v / (REAL)pa;
            v = v / (REAL)g->depth;
            dst[(size_t)Y * nx + X] = v;
        }
}

/* AART1 (AART.cl:38-70): residual d = y - A x for the subset rows, NaN measured -> 0.
 * Used by the reference-FISTA gradient of the differentiable-pair checks. */
void FN(xo_aart1)(const REAL *img, const REAL *meas, const REAL *cs, const xo_geom *g, int sub, int nrows,
                  REAL *dprj)
{
    const int px = g->px, ss = g->ss;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nrows; ++k)
        for (int X = 0; X < px; ++X) {
            const int th = sub + k * ss;
            const REAL p = FN(xo_raysum_)(img, g, cs[2 * th], cs[2 * th + 1], X);
            REAL y = FN(xo_measured_)(meas, g, X, th);
            y = (y != y) ? (REAL)0 : y;
            dprj[(size_t)th * px + X] = y - p;
        }
}

/* FISTAbackProjection (FISTA.cl:211-246): gradient-style backprojection with the FLOOR
 * bin rule (no +0.5, FISTA.cl:237), x + b*alpha*ss/pa/depth/L*0.5. */
void FN(xo_fista_bp)(const REAL *src, REAL *dst, const REAL *dprj, const REAL *cs, const xo_geom *g, int sub,
                     REAL alpha, REAL L)
{
    const int nx = g->nx, ny = g->ny, px = g->px, pa = g->pa, ss = g->ss;
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < ny; ++Y)
        for (int X = 0; X < nx; ++X) {
            const REAL Xc = (REAL)X - (REAL)nx * (REAL)0.5;
            const REAL Yc = (REAL)Y - (REAL)ny * (REAL)0.5;
            REAL b = (REAL)0;
            for (int th = sub; th < pa; th += ss) {
                const REAL c = cs[2 * th], s = cs[2 * th + 1];
                const REAL t = ((Xc * c) - (Yc * s)) + (REAL)px * (REAL)0.5;
                const int bin = (int)XO_FLOOR(t);
                b += (bin >= 0 && bin < px) ? dprj[(size_t)th * px + bin] : (REAL)0;
            }
            REAL v = b * alpha;
            v = v * (REAL)ss;
            v = v / (REAL)pa;
            v = v / (REAL)g->depth;
            v = v / L;
            v = v * (REAL)0.5;
            dst[(size_t)Y * nx + X] = src[(size_t)Y * nx + X] + v;
        }
}

/* backProjectionFBP (FBP.cl:164-188): linear-interpolated pixel-driven backprojection
 * over ALL angles with the field-of-view mask r < nx/2, divided by 2*pa. */
void FN(xo_bp_fbp)(const REAL *fprj, const REAL *cs, const xo_geom *g, REAL *dst)
{
    const int nx = g->nx, ny = g->ny, px = g->px, pa = g->pa;
#pragma omp parallel for schedule(static)
    for (int Y = 0; Y < ny; ++Y)
        for (int X = 0; X < nx; ++X) {
            const REAL Xc = (REAL)X - (REAL)nx * (REAL)0.5;
            const REAL Yc = (REAL)Y - (REAL)ny * (REAL)0.5;
            const REAL radius = XO_SQRT(Xc * Xc + Yc * Yc);
            REAL b = (REAL)0;
            if (radius < (REAL)nx * (REAL)0.5) {
                for (int th = 0; th < pa; ++th) {
                    const REAL c = cs[2 * th], s = cs[2 * th + 1];
                    const REAL u = (((Xc * c) - (Yc * s)) + (REAL)g->cx) + (REAL)0.5;
                    /* linear sampler along X at row th (v = th + 0.5 -> exact row) */
                    const REAL uu = u - (REAL)0.5;
                    const REAL fi = XO_FLOOR(uu);
                    const REAL a = uu - fi;
                    const int i = (int)fi;
                    const REAL t0 = FN(xo_tex_)(fprj, px, pa, i, th);
                    const REAL t1 = FN(xo_tex_)(fprj, px, pa, i + 1, th);
                    b += ((REAL)1 - a) * t0 + a * t1;
                }
            }
            dst[(size_t)Y * nx + X] = b / ((REAL)pa * (REAL)2);
        }
}

/* sinogramCorrection (reconstShare.cl:35-70), applied by OSEM_execution before the
 * subset loop when correctionMode > 0 (GPU.cpp:175-186) with a = b = 0.5 (:182-183).
 * angle_pr = angle/180*PI here (float division first, then the double PI). */
void FN(xo_sino_correction)(const REAL *src, REAL *dst, const float *ang_deg, const xo_geom *g, int mode)
{
    const int px = g->px, pa = g->pa;
    for (int th = 0; th < pa; ++th) {
        REAL apr, ca, sf;
        if (sizeof(REAL) == sizeof(float)) {
            const float q = ang_deg[th] / 180.0f;
            apr = (REAL)(float)((double)q * XO_PI);
            ca = (REAL)(float)cos((double)apr);
        } else {
            apr = (REAL)(((double)ang_deg[th] / 180.0) * XO_PI);
            ca = (REAL)cos((double)apr);
        }
        sf = (REAL)0.5 + (REAL)0.5 * ca;
        for (int X = 0; X < px; ++X) {
            REAL v = src[(size_t)th * px + X];
            const REAL theta = (REAL)2 * XO_FABS((REAL)X - (REAL)px / (REAL)2) / (REAL)px;
            REAL cb;
            if (sizeof(REAL) == sizeof(float)) cb = (REAL)(float)cos((double)(float)asin((double)theta));
            else cb = (REAL)cos(asin((double)theta));
            switch (mode) {
            case 4: v = (theta * theta < sf * sf) ? v : (REAL)0; break;
            case 3: v = v * (cb * ca); break;
            case 2: v = v * ca; break;
            case 1: v = v * cb; break;
            default: break;
            }
            dst[(size_t)th * px + X] = v;
        }
    }
}

/* The OS-EM host loop of OSEM_execution (GPU.cpp:125-240) for ONE slice, with the
 * ratio image zero-initialised (rows OSEM1 never writes read as 0: "ref" mode) or, with
 * cover != 0, with OSEM1 run over every row OSEM2 reads.  img is updated in place. */
void FN(xo_osem_run)(REAL *img, const REAL *meas, const REAL *cs, const xo_geom *g, const int *sub_order, int it,
                     int cover)
{
    const size_t nimg = (size_t)g->nx * g->ny, nprj = (size_t)g->px * g->pa;
    REAL *ratio = (REAL *)calloc(nprj, sizeof(REAL));
    REAL *dst = (REAL *)malloc(nimg * sizeof(REAL));
    if (!ratio || !dst) {
        free(ratio);
        free(dst);
        return;
    }
    for (int i = 0; i < it; ++i)
        for (int k = 0; k < g->ss; ++k) {
            const int sub = sub_order[k];
            const int nrows = cover ? (g->pa - sub + g->ss - 1) / g->ss : g->pa / g->ss;
            FN(xo_osem1)(img, meas, cs, g, sub, nrows, ratio);
            FN(xo_osem2)(img, dst, ratio, cs, g, sub);
            memcpy(img, dst, nimg * sizeof(REAL));
        }
    free(ratio);
    free(dst);
}

#undef FN
#undef XO_CAT
#undef XO_CAT2
