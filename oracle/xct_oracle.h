/*
 * xct_oracle.h -- declarations of the CPU oracle (TEST INFRASTRUCTURE ONLY; see
 * xct_oracle.c).  Layouts follow the reference: a sinogram is float [pa][px] (px
 * fastest), an image is float [ny][nx] (x fastest); cs is (cos, sin) per angle.
 */
#ifndef XCT_ORACLE_H
#define XCT_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define XO_ABI_VERSION 1

enum {
    XO_ORDER_CANONICAL = 0,
    XO_ORDER_FWD_LITERAL = 1,
    XO_ORDER_BP_LITERAL = 2,
    XO_ORDER_LITERAL = 3,  /* both stages exactly as written in the reference   */
    XO_ORDER_GPU = 2       /* canonical forward + literal backprojection: CUDA's */
};

typedef struct {
    int nx, ny;     /* reconstruction size (IMAGESIZE_X/Y)                        */
    int px, pa;     /* detector bins, projection angles (PRJ_IMAGESIZE/ANGLESIZE) */
    int ss;         /* subsets (SS)                                               */
    int depth;      /* samples per ray, max(nx, ny) (DEPTHSIZE, GPU.cpp:542)     */
    double cx;      /* detector centre in bins, px/2 in the reference             */
    int order;      /* XO_ORDER_*                                                 */
    int fetch_mode; /* measured read at integer coords: 0 exact texel, 1 2x2 avg  */
} xo_geom;

void xo_trig_f32(const float *ang_deg, int pa, float *cs);
void xo_trig_f64(const float *ang_deg, int pa, double *cs);
int xo_subset_order(int ss, int *sub);
int xo_abi_version(void);

/* FBP ramp filter of nrows sinogram rows [nrows][px] -> [nrows][px], zero padding zp
 * (a power of two >= px).  _f32 follows FBP.cl's float evaluation literally; _f64 is the
 * same transform in double with exact twiddles (the accuracy yardstick). */
void xo_fbp_filter_f32(const float *prj, int px, int nrows, int zp, float *out);
void xo_fbp_filter_f64(const double *prj, int px, int nrows, int zp, double *out);
/* hybrid base-up on n pixels of one slice (reconstShare.cl:87-109 with the slice minimum);
 * returns the minimum in *min_out when not NULL. */
void xo_base_up_f32(float *img, long long n, int order, float *min_out);

/* Rotation-centre search (RotationCenterSearch/rotCenterSearch.cl).  Images are [H][W]. */
void xo_rot_center_shift_f32(const float *prj, int px, int pa, float shift, float *out);
/* setMask's per-shift constants: rp, rm, p1..p4 (x, y), p_div, p_cnt (x, y) -> prm[13] */
void xo_mask_params_f32(int W, int H, float shift, float ang_min, float ang_max, float *prm);
/* setMask over columns x < w_visit (others 0) */
void xo_set_mask_f32(int W, int H, int w_visit, const float *prm, float *mask);
/* imgFocusIndex: per-pixel (sq_delta, mask_tot) summed in the reference's order for a
 * work-group of L items (literal, float) or in double over every pixel (L = 0). */
double xo_focus_index(const float *img, const float *mask, int W, int H, int L);

/* Reslice (Reslice/reslice.cl): projections mt [A][H][W] -> sinograms prj [H][A][W] with
 * per-angle shifts (xs, ys may be NULL: 0), baseup and the optional cosine correction;
 * denoiseSinogram on sinograms [H][A][W]. */
void xo_reslice_f32(const float *mt, int W, int H, int A, const float *xs, const float *ys, float baseup,
                    int correction, float *prj);
void xo_denoise_sinogram_f32(const float *src, int W, int A, int H, float threshold, float *dst);

/* Compressed-sensing OS-EM (FISTA_OSEM_execution): ISTA3D and FISTA3D (FISTA.cl:409-594) on
 * a batch of dN images [dN][ny][nx]; lambda is the kernels' float lambda. */
void xo_ista3d_f32(const float *v, int nx, int ny, int dN, float lambda, float *x_new);
void xo_fista3d_f32(const float *x_in, const float *v, const float *beta, int nx, int ny, int dN, float lambda,
                    float *w_new, float *x_new, float *beta_new);

/* FISTA with compressed sensing (FISTA_ocl): the power iteration's Lipschitz estimates L [ss]
 * (work_group: the reference's min(CL_DEVICE_MAX_WORK_GROUP_SIZE, ox) reduction width;
 * layer_mode: which layer powerIter1 reads, see xct_oracle.c) and FISTA_execution on dN slices
 * (see xct_oracle.c for the arguments). */
void xo_power_iteration_f32(const float *cs, const xo_geom *g, int trials, int work_group, int layer_mode,
                            float *L);
void xo_fista_run_f32(float *imgs, const float *meas, const float *res0, const float *cs, const xo_geom *g, int dN,
                      const int *sub, int it, float alpha, const float *L, double lambda_d, int flags);

#define XO_DECL(T, S)                                                                                   \
    void xo_projection##S(const T *img, const T *cs, const xo_geom *g, int sub, int ss, int nrows, T *prj); \
    void xo_osem1##S(const T *img, const T *meas, const T *cs, const xo_geom *g, int sub, int nrows,      \
                     T *ratio);                                                                         \
    void xo_osem2##S(const T *src, T *dst, const T *ratio, const T *cs, const xo_geom *g, int sub);       \
    void xo_backprojection##S(const T *prj, const T *cs, const xo_geom *g, int sub, T *dst);               \
    void xo_aart1##S(const T *img, const T *meas, const T *cs, const xo_geom *g, int sub, int nrows,      \
                     T *dprj);                                                                          \
    void xo_fista_bp##S(const T *src, T *dst, const T *dprj, const T *cs, const xo_geom *g, int sub,      \
                        T alpha, T L);                                                                  \
    void xo_bp_fbp##S(const T *fprj, const T *cs, const xo_geom *g, T *dst);                               \
    void xo_sino_correction##S(const T *src, T *dst, const float *ang_deg, const xo_geom *g, int mode);    \
    void xo_adjoint##S(const T *sino, const T *cs, const xo_geom *g, T *img);                               \
    void xo_osem_run##S(T *img, const T *meas, const T *cs, const xo_geom *g, const int *sub_order, int it, \
                        int cover);

XO_DECL(float, _f32)
XO_DECL(double, _f64)
#undef XO_DECL

#ifdef __cplusplus
}
#endif
#endif
