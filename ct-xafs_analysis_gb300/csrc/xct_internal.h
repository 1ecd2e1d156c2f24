// xct_internal.h -- internal declarations shared by the libxct translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <functional>
#include <string>
#include <vector>

#include "../../include/xct.h"

// Geometry as the kernels see it (passed by value).  Half sizes are precomputed exactly
// as the reference's expressions produce them (IMAGESIZE_X*0.5f etc., OSEM.cl:58-59,95).
struct KGeom {
    int nx, ny;      // image
    int px, pa;      // sinogram
    int ss;          // subsets
    int depth;       // samples per ray, max(nx, ny)
    float hx, hy;    // nx*0.5f, ny*0.5f
    float hd;        // depth*0.5f
    float cx;        // detector centre (px*0.5f in the reference)
    int fetch;       // XCT_FETCH_*
    int fwd_T;       // tiled forward projector: tile side (44, 60, 76, 92)
    int fwd_chunk;   // tiled forward projector: subset angles per CTA (1..128)
    int ms_chunk = 0;  // slice-interleaved forward projector: subset angles per CTA (1..128);
                       // 0 = off (groups of eight slices then use the per-slice kernel)
};

// One slice of a batched launch (device-side descriptor).
struct XctItemDev {
    KGeom g;
    const float *sino;   // measured sinogram [pa][px] the OS-EM steps read (corrected if corr_mode)
    float *img;          // image [ny][nx], updated in place
    float *ratio;        // ratio image [pa][px] (rows never written stay 0)
    double *acc;         // ray-sum accumulator [ceil(pa/ss)][px] (kept zeroed between subsets)
    const float2 *trig;  // (cos, sin) [pa]
    int cover;           // XCT_SUBSETS_COVER
    int fwd_ntx, fwd_nty, bp_ntx;
    int corr_mode;            // sinogramCorrection mode 1..4, 0 none
    const float *sino_in;     // the caller's measured sinogram (the correction's input)
    float *corr;              // corrected sinogram [pa][px] (corr_mode > 0; then sino == corr)
    const float *corr_ang;    // [pa] x 2 per-angle correction factors
    const float *corr_bin;    // [px] per-bin correction factors
};

// A stack of consecutive slices of one shape in a batch plan with compressed sensing: its
// images form one [dN][ny][nx] array (the proximal step's third axis), with its own w, beta
// and x' buffers of the same size.
struct XctStackDev {
    float *img, *w, *beta, *xn;
    int nx, ny, dN;
};

struct xct_ctx {
    int device;
    int sm_count;
    int max_smem_optin;
    char name[256];
};

struct xct_plan {
    xct_ctx *ctx;
    xct_geom g;
    KGeom kg;
    std::vector<float> angles;
    std::vector<int> sub_default;
    float2 *d_trig = nullptr;    // [pa] (cos, sin) of the float angle (see trig table)
    float *d_sino = nullptr;     // [max_batch][pa][px] staging for host-buffer runs
    float *d_img = nullptr;      // [max_batch][ny][nx] staging for host-buffer runs
    float *d_ratio = nullptr;    // [max_batch][pa][px] ratio image (never-written rows stay 0)
    float *d_corr = nullptr;     // [max_batch][pa][px] corrected sinogram (correction_mode > 0)
    float *d_corr_ang = nullptr; // [pa] x 2 per-angle correction factors
    float *d_corr_bin = nullptr; // [px] per-bin correction factors
    double *d_acc = nullptr;     // tiled forward: ray-sum accumulator [max_batch][acc_rows][px]
    int *d_min_keys = nullptr;   // [max_batch] per-slice image minimum (FBP + OS-EM hybrid)
    double *d_red = nullptr;     // [2*max_batch] focus-index sums (rotation-centre search)
    float *d_rc_prm = nullptr;   // [max_batch][16] mask constants per shift
    float *d_fi = nullptr;       // [max_batch] focus indices
    float *d_cs = nullptr;       // compressed-sensing OS-EM: w, beta, x' [3][max_batch][ny][nx],
                                 // allocated by the first such run
    float *d_fista = nullptr;    // FISTA: v, w, beta, dest [4][max_batch][ny][nx] (first FISTA run)
    float *d_pi = nullptr;       // power iteration: layer images, candidate, projection (first use)
    double *d_pi_l2 = nullptr;   // power iteration: squared norms of the candidates [ss]
    int pi_layers = 0;           // layer images d_pi holds
    std::vector<float> lip;      // Lipschitz estimates L[ss] of the subset operators (empty: none)
    float *d_sino2 = nullptr;    // volume streaming: the second staging set (first volume run)
    float *d_img2 = nullptr;
    cudaStream_t s_h2d = nullptr, s_d2h = nullptr;
    int acc_rows = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // OS-EM of a batch runs its two halves on the caller's stream and on s_aux (fork/join by
    // events), so one half's kernels fill the SMs the other half's last waves leave idle
    cudaStream_t s_aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    float last_ms = 0.0f;
};

// ---- error handling (per-thread last error) ----
int xct_fail(int code, const std::string &msg);
int xct_cuda_fail(cudaError_t e, const char *what);
#define XCT_CUDA_TRY(expr)                                          \
    do {                                                            \
        cudaError_t e_ = (expr);                                    \
        if (e_ != cudaSuccess) return xct_cuda_fail(e_, #expr);     \
    } while (0)

extern std::atomic<long long> g_xct_launches;

// ---- host-side tables (identical to the oracle's) ----
void xct_trig_table(const float *ang_deg, int pa, std::vector<float2> &cs);
void xct_subset_order_host(int ss, int *sub);
int xct_subset_at(int ss, int k);  // entry k of that order

// ---- kernel launchers (xct_plain.cu / xct_tiled.cu / xct_misc.cu) ----
// Forward projection of rows th = sub + k*step, k < nrows, for dN slices.
//   ratio mode (meas != nullptr): OSEM1 ratio (OSEM.cl:38-68) into out;
//   raw mode   (meas == nullptr): projection sums (reconstShare.cl:213-241) into out.
int launch_fwd_plain(const KGeom &g, const float2 *trig, const float *img, const float *meas, float *out, int dN,
                     int sub, int step, int nrows, cudaStream_t st);
// OSEM2 backprojection + multiplicative update, in place on img (OSEM.cl:71-105).
int launch_bp_update_plain(const KGeom &g, const float2 *trig, float *img, const float *ratio, int dN, int sub,
                           cudaStream_t st);
// backProjection (reconstShare.cl:245-275) with subset (sub, step): img = B prj.
int launch_bp_ref_plain(const KGeom &g, const float2 *trig, const float *prj, float *img, int dN, int sub, int step,
                        cudaStream_t st);
// Tiled forward projector (xct_tiled.cu): same contract as launch_fwd_plain; acc is a
// zeroed [dN][nrows][px] double accumulator (left zeroed on return); nrows <= rows cap.
int fwd_tiled_rows_cap();
int launch_fwd_tiled(const KGeom &g, const float2 *trig, const float *img, const float *meas, float *out,
                     double *acc, int dN, int sub, int step, int nrows, cudaStream_t st);
// The two halves of launch_fwd_tiled (timed separately by xct_osem_profile).
int launch_fwd_tiled_main(const KGeom &g, const float2 *trig, const float *img, double *acc, int dN, int sub, int step,
                          int nrows, cudaStream_t st);
// The slice-interleaved forward projector alone over groups x 8 slices (part of
// launch_fwd_tiled_main when g.ms_chunk > 0); its slice group size and tile side.
int launch_fwd_ms(const KGeom &g, const float2 *trig, const float *img, double *acc, int groups, int sub, int step,
                  int nrows, int chunk, cudaStream_t st);
int fwd_ms_slices();
int fwd_ms_tile();
int launch_fwd_finalize(const KGeom &g, const float *meas, float *out, double *acc, int dN, int sub, int step,
                        int nrows, cudaStream_t st);
// Tiled OSEM2 backprojection + update, in place (same contract as the plain one).
int launch_bp_update_tiled(const KGeom &g, const float2 *trig, float *img, const float *ratio, int dN, int sub,
                           cudaStream_t st);
// Batched launches (xct_tiled.cu): work units of one slice, persistent grid sizes, and one
// subset step (forward, finalize, backprojection) over all slices; bases is [3][n+1]
// prefix sums of the units of each kernel, queues 3 zeroed counters.
void xct_batched_units(const KGeom &g, int &fwd_ntx, int &fwd_nty, int &fwd_units, int &fin_units, int &bp_ntx,
                       int &bp_units);
int xct_batched_grids(int device, int sm_count, int fwd_T, int grids[3]);
int launch_osem_step_batched(const XctItemDev *items, const int *bases, int n, int sub, int *queues,
                             const int grids[3], int fwd_T, cudaStream_t st);
bool xct_fwd_tile_valid(int T);
int launch_fwd_batched(const XctItemDev *items, const int *bases, int n, int sub, int *queue, int grid, int fwd_T,
                       cudaStream_t st);
int xct_check_geom(const xct_geom *g);
// Exact adjoint of the forward projector over all angles: img = A^T sino (overwrites img).
int launch_adj_tiled(const KGeom &g, const float2 *trig, const float *sino, float *img, int dN, cudaStream_t st);
// FBP (xct_fbp.cu).  zp: the zero-padded transform length (0 -> smallest power of two
// >= 2 px); checked and resolved by xct_fbp_check_zp.
int xct_fbp_check_zp(int px, int &zp);
// Ramp filter of dN sinograms [pa][px] -> [pa][px] (FBP.cl:34-160).
int launch_fbp_filter(const KGeom &g, const float *sino, float *out, int dN, int zp, cudaStream_t st);
// backProjectionFBP (FBP.cl:164-188) of dN filtered sinograms; min_keys (optional, [dN])
// receives each slice's minimum as an ordered integer key.
int launch_fbp_bp(const KGeom &g, const float2 *trig, const float *fprj, float *img, int dN, int *min_keys,
                  cudaStream_t st);
// baseUp (reconstShare.cl:87-109) with the slice minima of launch_fbp_bp, in place.
int launch_base_up(const KGeom &g, float *img, int dN, int order, const int *min_keys, int sm_count,
                   cudaStream_t st);
// Forward-projector tile autotuning (xct_tune.cu).
struct TuneChoice {
    int T, chunk;
    float ms;
    int ms_chunk = 0;  // slice-interleaved forward projector's angle chunk; 0 = off
};
std::string xct_tune_key(const char *device, int nx, int ny, int px, int pa, int ss, int dN);
bool xct_tune_lookup(const std::string &key, const char *path, TuneChoice &c);
int xct_tune_store(const std::string &key, const char *path, const TuneChoice &c);
TuneChoice xct_tune_default(int sm_count, const std::function<long long(int, int)> &ctas);
std::vector<TuneChoice> xct_tune_candidates(int max_rows);
const char *xct_tune_env_path();
void xct_plan_default_tuning(xct_plan *p);
// Compressed-sensing proximal steps (xct_cs.cu): ISTA3D, FISTA3D over dN slices.
int launch_ista3d(const float *v, float *x_new, int nx, int ny, int dN, float lambda, int sm_count, cudaStream_t st);
// FISTA3D with x_t read from x_in (may equal w) and x_{t+1} stored to x_new (may be null).
int launch_fista3d(const float *x_in, float *w, const float *v, float *beta, float *x_new, int nx, int ny, int dN,
                   float lambda, int sm_count, cudaStream_t st);
// FISTA with compressed sensing (xct_fista.cu): the power iteration's backprojection (powerIter2,
// rows th = sub + k*step, k < nrows, of prj [pa][px]) into cnd, the squared L2 norm of cnd over
// columns [0, nxe) and rows [0, nye) into *out (double), the normalisation powerIter3; the AART1
// residual in place on the subset rows of the forward projection `out`; FISTAbackProjection.
int launch_pi_bp(const KGeom &g, const float2 *trig, const float *prj, float *cnd, int sub, int step, int nrows,
                 float scale, cudaStream_t st);
int launch_pi_l2(const float *cnd, int nx, int nxe, int nye, double *out, int sm_count, cudaStream_t st);
int launch_pi_norm(const float *cnd, float *img, int nx, int ny, const double *l2, int fetch, cudaStream_t st);
int launch_residual(const KGeom &g, const float *meas, float *out, int dN, int sub, int step, int nrows,
                    cudaStream_t st);
int launch_fista_bp(const KGeom &g, const float2 *trig, const float *x, float *v, const float *res, int dN, int sub,
                    float alpha, float L, cudaStream_t st);
// The exact adjoint over the angles th = sub + k*step, k < nang (all angles: 0, 1, pa); with
// base non-null the result is base + scale * A^T sino.
int launch_adj_subset(const KGeom &g, const float2 *trig, const float *sino, float *img, int dN, int sub, int step,
                      int nang, const float *base, float scale, cudaStream_t st);
// Rotation-centre search (xct_rcs.cu).
void xct_mask_params(int W, int H, float shift, float ang_min, float ang_max, float *prm16);
float xct_shift_value(float start, float step, int i);
int launch_rot_shift(const float *prj, float *out, int px, int pa, int n, int i0, float start, float step,
                     int sm_count, cudaStream_t st);
int launch_fill(float *p, long long n, float v, int sm_count, cudaStream_t st);
int launch_focus_index(const float *imgs, int nx, int ny, int n, const float *d_prm, double *red, float *findex,
                       cudaStream_t st);
// sinogramCorrection (reconstShare.cl:35-70), modes 1..4, src -> dst.
// The ISTA3D/FISTA3D kernels' lambda for CSlambda (L fixed at 0.5, the compressed-sensing OS-EM).
float xct_cs_kernel_lambda(float cs_lambda);
// sinogramCorrection factor tables of one geometry (angle factors [2*pa], bin factors [px]).
void xct_corr_tables(const float *ang_deg, int pa, int px, std::vector<float> &af, std::vector<float> &bf);
// sinogramCorrection of every item of a batch with corr_mode > 0 (sino_in -> corr); the grid
// covers the largest (px, pa) of the batch.
int launch_sino_correction_batched(const XctItemDev *items, int n, int max_px, int max_pa, cudaStream_t st);
// Batched compressed-sensing steps over stacks (xct_cs.cu): ISTA3D (img -> xn), FISTA3D(x = img,
// w, v = img, beta -> w, beta, xn), copies img <- xn and w <- img, beta <- 0.
int launch_ista3d_stacks(const XctStackDev *stacks, int nstacks, long long max_vox, float lambda, int sm_count,
                         cudaStream_t st);
int launch_fista3d_stacks(const XctStackDev *stacks, int nstacks, long long max_vox, float lambda, int sm_count,
                          cudaStream_t st);
int launch_stack_copy(const XctStackDev *stacks, int nstacks, long long max_vox, int what, int sm_count,
                      cudaStream_t st);
int launch_sino_correction(const KGeom &g, const float *src, float *dst, const float *ang_fac, const float *bin_fac,
                           int mode, int dN, cudaStream_t st);

// ---- bounds-checked build (xct_check.cuh) ------------------------------------------------
struct XctCheckWord {
    unsigned long long count;  // accesses skipped since the last reset
    int site;                  // XCT_SITE_* of the first
    int pad;
    long long value, lo, hi;   // its index and the bounds it missed
};
enum {
    XCT_SITE_FWD_TAP = 1,   // forward tile: footprint loads (byte address in the tile)
    XCT_SITE_FWD_ACC = 2,   // forward tile: accumulator row and bin
    XCT_SITE_ADJ = 3,       // adjoint tile: shared accumulator element
    XCT_SITE_BP_WIN = 4,    // OS-EM backprojector: bin-window load (byte address)
    XCT_SITE_FBP_WIN = 5,   // FBP backprojector: bin-window load pair (byte address)
    XCT_SITE_FWD_MS_TAP = 6,  // slice-interleaved forward tile: footprint load (byte address)
};
#ifdef XCT_CHECKED
int xct_check_read_tiled(XctCheckWord *out, bool reset);
int xct_check_read_fbp(XctCheckWord *out, bool reset);
#endif

// SM count of the current device (cached per device).
int device_sm_count();

// ---- timeline ranges -----------------------------------------------------------------------
// An NVTX range over a scope: the library's calls appear by name on an Nsight Systems or
// Nsight Compute timeline.  NVTX v3 is header-only; without a tool attached a range costs a
// pointer test.
#include <nvtx3/nvToolsExt.h>
struct XctRange {
    explicit XctRange(const char *name) { nvtxRangePushA(name); }
    ~XctRange() { nvtxRangePop(); }
    XctRange(const XctRange &) = delete;
    XctRange &operator=(const XctRange &) = delete;
};
#define XCT_RANGE(name) XctRange xct_range_guard_(name)
