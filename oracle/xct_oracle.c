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
 *
 * Parity pin: the reference ships no tests, fixtures or golden vectors, and its OpenCL
 * runtime is not available, so the pin is oracle/_ref: the reference's own OSEM.cl and
 * reconstShare.cl kernel bodies compiled with g++ against an OpenCL-C shim (recipe:
 * oracle/build_ref.py), driven by the same host loop.  The literal evaluation order of
 * this oracle matches that build to the last bit on the committed fixtures (tests/).
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
