/*
 * xct.h -- C ABI of the GB300 OS-EM library (libxct.so).
 *
 * Drop-in replacement for the OpenCL platform/queue layer and the OS-EM executors of
 * NozomuIshiguro/CT-XAFS_analysis (CT_reconstruction).  Plain C types only: no CUDA,
 * torch or C++ types cross this boundary.  Every call returns an int status (XCT_OK = 0,
 * negative XCT_E_* on failure; the message is in xct_last_error(), per thread).
 *
 * Layouts are the reference's: a sinogram is float32 [pa][px] (bins fastest,
 * CT_reconstruction/fileIO.cpp:25-33, image (px, pa, layer) in GPU.cpp:423); an image is
 * float32 [ny][nx] (x fastest, GPU.cpp:434-443, fileIO.cpp:35-43).  A batch of dN slices
 * is dN such arrays back to back (the reference's image2d_array layers, GPU.cpp:139-140).
 * Angles are degrees, one per projection (fileIO.cpp:11-23).
 */
#ifndef XCT_H
#define XCT_H

#ifdef __cplusplus
extern "C" {
#endif

#define XCT_ABI_VERSION 1

enum {
    XCT_OK = 0,
    XCT_E_INVALID = -1,     /* bad argument / shape                                   */
    XCT_E_CUDA = -2,        /* CUDA runtime error                                     */
    XCT_E_NOMEM = -3,       /* device or host allocation failed                       */
    XCT_E_UNSUPPORTED = -4, /* device is not sm_103, or feature not built             */
    XCT_E_TIMEOUT = -5,     /* a bounded device-side wait gave up                     */
    XCT_E_IO = -6           /* file read/write error (host helpers)                    */
};

/* How OSEM1's read of the measured sinogram at integer coordinates with a LINEAR sampler
 * (OSEM.cl:64, undefined in OpenCL 1.2) is interpreted. */
enum { XCT_FETCH_EXACT = 0, XCT_FETCH_AVG2X2 = 1 };

/* Rows of the ratio image that OSEM1 never writes when pa % ss != 0 (OSEM2 still reads
 * them): XCT_SUBSETS_REF reads them as 0 (the reference's launch shape, GPU.cpp:169);
 * XCT_SUBSETS_COVER forward-projects every row OSEM2 reads. */
enum { XCT_SUBSETS_REF = 0, XCT_SUBSETS_COVER = 1 };

/* Kernel family used by a plan: the optimised tiled kernels (default) or the plain
 * one-thread-per-ray / one-thread-per-pixel kernels (the reference's launch shape). */
enum { XCT_KERNELS_TILED = 0, XCT_KERNELS_PLAIN = 1 };

typedef struct xct_ctx xct_ctx;
typedef struct xct_plan xct_plan;

/* Problem geometry of one OS-EM plan (the -D macros of OSEM_programBuild,
 * GPU.cpp:538-548, plus the globals g_it, g_ss of main.cpp:29,35). */
typedef struct {
    int nx, ny;                /* reconstruction size (IMAGESIZE_X, IMAGESIZE_Y)              */
    int ox, oy;                /* output ROI; must equal nx, ny (the reference's ROI < full
                                  path writes the top-left corner but reads and saves a centred
                                  window, GPU.cpp:152-153,170; only the full image is defined) */
    int px, pa;                /* detector bins (PRJ_IMAGESIZE), angles (PRJ_ANGLESIZE)       */
    int ss;                    /* subsets (SS)                                                 */
    int it;                    /* iterations (g_it)                                            */
    const float *angles_deg;   /* [pa], copied at plan creation                                */
    float center_bin;          /* rotation centre in bins; < 0 selects px/2 (the reference)    */
    int measured_fetch_mode;   /* XCT_FETCH_*                                                  */
    int subset_mode;           /* XCT_SUBSETS_*                                                */
    int correction_mode;       /* sinogramCorrection mode 0..4 (reconstShare.cl:35-70); 0 none */
    int max_batch;             /* largest dN passed to the run calls (numParallel, main.cpp:41)*/
    int kernels;               /* XCT_KERNELS_*                                                */
} xct_geom;

/* ---- context: replaces OCL_platform_device (share source/OpenCL_analysis.hpp:126-147) */
int xct_ctx_create(int device, xct_ctx **out);
int xct_ctx_destroy(xct_ctx *ctx);
/* Number of CUDA devices and the name of one (OpenCL_Device_Info equivalent). */
int xct_device_count(int *count);
int xct_device_name(int device, char *buf, int buflen);

/* ---- plan: replaces OSEM_programBuild (GPU.cpp:513-559) -- no JIT, shapes are runtime */
int xct_osem_plan_create(xct_ctx *ctx, const xct_geom *geom, xct_plan **out);
int xct_osem_plan_destroy(xct_plan *plan);

/* Subset order of OSEM_ocl (GPU.cpp:564-582): bit reversal for power-of-two ss. */
int xct_subset_order(int ss, int *sub);

/* ---- OS-EM: replaces OSEM_execution (GPU.cpp:125-240) + the host<->device image copies
 * of OSEM_thread (GPU.cpp:440-445, 460-463).  sino_host[i] is slice i's [pa][px]
 * sinogram, img_host[i] its [ny][nx] image (initial image in, reconstruction out).
 * Blocking.  sub may be NULL (the plan's subset order).  it < 0 uses the plan's it.  A batch
 * of two or more slices runs as two halves, each with its own copies on its own stream, so
 * one half's uploads and downloads overlap the other half's kernels (page-locked host
 * buffers overlap fully; pageable ones as far as their synchronous copies allow). */
int xct_osem_run(xct_plan *plan, int dN, const float *const *sino_host, float *const *img_host, const int *sub,
                 int it);

/* Same on device memory: d_sino [dN][pa][px], d_img [dN][ny][nx] (in/out), enqueued on
 * `stream` (a cudaStream_t; NULL is the legacy default stream, as everywhere in CUDA).
 * Asynchronous; stream-ordered with the caller's own work on that stream.  A batch of two or
 * more slices runs as two halves, the second on a stream of the plan that waits for `stream`
 * and that `stream` waits for in turn, so the call is still ordered as one unit on `stream`;
 * a plan serves one call at a time.  The call can be captured into a CUDA graph (stream
 * capture of `stream` takes in the second stream through the fork) and replayed; replay
 * saves the launch overhead that dominates for small slices. */
int xct_osem_run_device(xct_plan *plan, int dN, const float *d_sino, float *d_img, const int *sub, int it,
                        void *stream);

/* ---- a whole volume from host memory -------------------------------------------------
 * OS-EM of n slices (sino_host[i] [pa][px] in, img_host[i] [ny][nx] initial image in and
 * reconstruction out) in device batches of max_batch slices: while one batch computes, the
 * next batch's inputs are uploaded and the previous batch's images downloaded on their own
 * streams (two device staging sets, the second allocated on the first call), so the volume
 * needs no more HBM than two batches.  Page-locked host buffers (cudaHostAlloc /
 * cudaHostRegister) give full overlap; pageable ones are correct but copy synchronously.
 * Blocking; xct_plan_last_ms reports the whole run.  Replaces OSEM_ocl's dispatch of
 * OSEM_input_thread / OSEM_thread over the slices (GPU.cpp:629-658) for one device. */
int xct_osem_run_volume(xct_plan *plan, int n, const float *const *sino_host, float *const *img_host, const int *sub,
                        int it);

/* ---- batches of slices of different shapes (CT-XAFS stacks) -------------------------
 * The reference reconstructs dN slices of ONE shape per OSEM_execution call
 * (GPU.cpp:125-240, image2d_array layers).  A batch plan takes n slices of any shapes
 * (each its own xct_geom: size, bins, angle list, centre, modes) that share the subset
 * count; every subset step is three persistent launches whose CTAs take (slice, tile) work
 * units from a device queue, and the whole subset/iteration loop is one CUDA graph,
 * captured on the first xct_batch_run and replayed after.  d_sino[i] / d_img[i] are slice
 * i's device sinogram [pa_i][px_i] and image [ny_i][nx_i] (initial in, result out); they may
 * change from run to run.  Runs of one plan must not overlap (they share its buffers).
 * A slice whose geometry has a correction_mode is corrected once per run into a buffer of
 * the plan before the loop, as OSEM_execution does with prjCorrection set (GPU.cpp:175-186;
 * the CT-XAFS stack flow always sets it, Reslice_CTreconst_ocl.cpp:104-117, GPU.cpp:447-451).
 * xct_osem_run_batched = create, run, synchronise the stream, destroy.
 * xct_batch_plan_set_cs : compressed-sensing OS-EM (FISTA_OSEM_execution, GPU.cpp:243-405)
 *     over stacks: stack_len[s] consecutive slices of one image size form stack s (the lengths
 *     add up to n; nstacks = 0 turns it off), the third axis of the proximal step; every run
 *     then needs each stack's images consecutive in one [dN][ny][nx] array (d_img[i+1] =
 *     d_img[i] + ny*nx within a stack).  Semantics as xct_cs_osem_run_device.
 * Geometry groups: slices that share one geometry (sizes, centre, modes and angle list; in a
 * CT-XAFS stack, the slices of one width at one energy), at least XCT_MULTISLICE_SLICES of
 * them, form a group that runs through a single-shape plan of that geometry, up to 16 slices
 * per xct_osem_run_device call (the slice-interleaved kernels serve such slices faster than
 * the persistent launches): in place when a call's slices are consecutive in one pair of
 * arrays ([k][pa][px], [k][ny][nx]), else copied into a contiguous scratch pair of the plan
 * and the images copied back.  The graph serves the other slices; with compressed sensing
 * (stacks set) it serves every slice.  Results agree with the graph's to float rounding.
 * Each group holds a single-shape plan with the buffers of up to 16 slices of its geometry
 * (staging, ratio and accumulator: about 0.6 GB for 2048^2 with 1200 angles), so a stack of
 * many groups holds as many such sets; the graph's buffers cover every slice once.
 * xct_batch_plan_groups reports the number of groups and the slices they hold;
 * xct_batch_plan_set_grouping(plan, 0) turns the groups off (the graph serves every slice),
 * 1 on again (the default).  xct_batch_plan_uniform reports the slices per call when every
 * slice is in one group (0: not so). */
typedef struct xct_batch_plan xct_batch_plan;
int xct_batch_plan_create(xct_ctx *ctx, int n, const xct_geom *geoms, int it, xct_batch_plan **out);
int xct_batch_run(xct_batch_plan *plan, const float *const *d_sino, float *const *d_img, void *stream);
int xct_batch_plan_destroy(xct_batch_plan *plan);
int xct_osem_run_batched(xct_ctx *ctx, int n, const xct_geom *geoms, const float *const *d_sino,
                         float *const *d_img, int it, void *stream);
int xct_batch_plan_set_cs(xct_batch_plan *plan, float cs_lambda, int nstacks, const int *stack_len);
int xct_batch_plan_uniform(xct_batch_plan *plan, int *slices_per_call);
int xct_batch_plan_groups(xct_batch_plan *plan, int *ngroups, int *grouped_slices);
int xct_batch_plan_set_grouping(xct_batch_plan *plan, int on);

/* ---- OS-EM without any allocation ----------------------------------------------------
 * No counterpart in the reference: the reference allocates its image objects on every call.
 *
 * For callers that cannot allocate device memory -- an acquisition loop that must never
 * stall on cudaMalloc (it can synchronise the device), an application whose device memory
 * is all owned by its own pool, code running where allocation is forbidden.  Same work as
 * xct_osem_run_device with the tiled kernels, but without a plan: the caller passes the
 * geometry, its device sinograms d_sino [dN][pa][px] and images d_img [dN][ny][nx] (initial
 * image in, reconstruction out), and the function calls no cudaMalloc, cudaFree or other
 * allocating routine.  Its scratch (angle table, ratio image, ray-sum accumulator) is one
 * file-scope device array of XCT_STATIC_SCRATCH_BYTES bytes that every GPU that loads the
 * library holds until the process exits.
 *   - Limit: round256(8*pa) + round256(8*dN*ceil(pa/ss)*px) + 4*dN*pa*px bytes must fit in
 *     XCT_STATIC_SCRATCH_BYTES = 16 MiB (e.g. one 2048x2048 slice with 1500 angles and 15
 *     subsets needs 13.9 MB; round256 rounds up to a multiple of 256); larger problems get
 *     XCT_E_INVALID with the byte counts in the message.  Sinogram correction modes are not
 *     available here (XCT_E_UNSUPPORTED).
 *   - Runs on the CURRENT device.  The first call on a device looks up the array's device
 *     address (cudaGetSymbolAddress) for that device and keeps it; after a cudaDeviceReset
 *     of that device the kept address is stale, so do not use this entry point on a device
 *     that has been reset.
 *   - Cannot be captured into a CUDA graph: every call uploads its angle table from host
 *     memory on the stack, which a replay could not read.  A call on a stream that is being
 *     captured returns XCT_E_UNSUPPORTED and enqueues nothing.
 *   - Every call uses the same array and it keeps the last call's contents (each call clears
 *     what must start at zero).  Calls whose GPU work overlaps -- on different streams or
 *     host threads -- race on the array and give wrong results: serialise them.
 *   - it < 0 uses geom->it; sub may be NULL (the reference's subset order); NULL stream is
 *     the legacy default stream.  Asynchronous, like xct_osem_run_device. */
#define XCT_STATIC_SCRATCH_BYTES (16u << 20)
int xct_osem_run_static(const xct_geom *geom, int dN, const float *d_sino, float *d_img, const int *sub, int it,
                        void *stream);

/* ---- compressed-sensing OS-EM: replaces FISTA_OSEM_execution (GPU.cpp:243-405), the
 * path OSEM_thread takes when CSitBool is set (GPU.cpp:449-453) ----------------------
 * Per subset: OSEM1 and OSEM2, then the proximal step of the l1 distance to the six
 * neighbours across the dN slices of the call (ISTA3D in the first cycle, FISTA3D after,
 * FISTA.cl:409-594), with cs_lambda = CSlambda (main.cpp:46, default 1e-4).  The slices of
 * one call are the third axis of the neighbourhood, as in the reference (overlapping
 * batches of CSoverlap slices are the caller's business, GPU.cpp:642-643).  The reference's
 * own semantics are kept: the first cycle's proximal step starts from the image before that
 * subset's OS-EM update; the lower-layer neighbour is always layer 0 (FISTA.cl:425,513).
 * The plan allocates three image-sized buffers per slice on the first such call. */
int xct_cs_osem_run_device(xct_plan *plan, int dN, const float *d_sino, float *d_img, const int *sub, int it,
                           float cs_lambda, void *stream);
int xct_cs_osem_run(xct_plan *plan, int dN, const float *const *sino_host, float *const *img_host, const int *sub,
                    int it, float cs_lambda);

/* ---- FISTA with compressed sensing: replaces FISTA_ocl / FISTA_thread / FISTA_execution
 * (GPU.cpp:1755-2299), the path of GPU() modes 1 (AART, ss subsets) and 3 (ASIRT, one subset)
 * with CSitBool (GPU.cpp:37-41, 53-58) --------------------------------------------------
 * xct_fista_power_iteration : powerIteration (GPU.cpp:2079-2188, FISTA.cl:50-208): the
 *     Lipschitz estimate L[s] of every subset operator, from `trials` rounds (the reference
 *     runs 30) of forward projection (powerIter1), floor-rule backprojection (powerIter2),
 *     the squared L2 norm (imageL2AbsX/Y over the columns and rows that work-groups of
 *     min(work_group, nx) items visit; the reference's work_group is the device's
 *     CL_DEVICE_MAX_WORK_GROUP_SIZE, 1024 on NVIDIA GPUs) and normalisation (powerIter3).
 *     powerIter1 never sets the layer of its sampling coordinate (FISTA.cl:60): by default
 *     every subset projects layer 0's estimate, as a zero-initialised coordinate does;
 *     XCT_PI_OWN_LAYER projects each subset's own.  Stores L in the plan (and L_out [ss] when
 *     not NULL).  Synchronous on `stream`.
 * xct_fista_set_lipschitz : sets L [ss] directly (finite, > 0).
 * xct_fista_run_device : FISTA_execution on dN slices, d_sino [dN][pa][px] in, d_img
 *     [dN][ny][nx] out (its initial contents are not read: the first image is the plain
 *     backprojection of subset sub[0], GPU.cpp:1853-1858).  alpha is the AART factor g_wt1
 *     (main.cpp:35, default 1), cs_lambda CSlambda (main.cpp:46, default 1e-4).  Per subset:
 *     AART1's residual, FISTAbackProjection's gradient step, ISTA3D (first cycle) or FISTA3D.
 *     The reference writes FISTA3D's x_{t+1} into the beta image, where beta_{t+1} overwrites
 *     it (GPU.cpp:1867-1868), so its image stays the first cycle's ISTA3D result; that is kept
 *     by default.  flags: XCT_FISTA_UPDATE_X stores x_{t+1} as the next image;
 *     XCT_FISTA_ADJOINT replaces FISTAbackProjection's floor-rule backprojection by the exact
 *     adjoint of the forward projector (xct_adj).  A plan without L runs the power iteration
 *     (30 trials, work group 1024) first.  The slices of one call are the proximal step's
 *     third axis, as in the compressed-sensing OS-EM.  Uses the plan's ratio buffer; the plan
 *     allocates four image-sized buffers per slice on the first call.
 * xct_fista_run : the same from host buffers (FISTA_thread, GPU.cpp:1927-1979), blocking. */
#define XCT_PI_OWN_LAYER 1
#define XCT_FISTA_UPDATE_X 1
#define XCT_FISTA_ADJOINT 2
int xct_fista_power_iteration(xct_plan *plan, int trials, int work_group, int flags, float *L_out, void *stream);
int xct_fista_set_lipschitz(xct_plan *plan, const float *L);
int xct_fista_run_device(xct_plan *plan, int dN, const float *d_sino, float *d_img, const int *sub, int it,
                         float alpha, float cs_lambda, int flags, void *stream);
int xct_fista_run(xct_plan *plan, int dN, const float *const *sino_host, float *const *img_host, const int *sub,
                  int it, float alpha, float cs_lambda, int flags);

/* ---- the two OS-EM kernels as separate steps (dN slices, device memory) -------------
 * xct_osem1 : OSEM1 (OSEM.cl:38-68) for subset `sub`: forward-projects d_img and writes
 *             the measured/estimated ratio rows of the subset into d_ratio [dN][pa][px]
 *             (other rows untouched).
 * xct_osem2 : OSEM2 (OSEM.cl:71-105) for subset `sub`: backprojects d_ratio over the
 *             subset's angles and applies the multiplicative update to d_img in place. */
int xct_osem1(xct_plan *plan, int dN, int sub, const float *d_img, const float *d_sino, float *d_ratio,
              void *stream);
int xct_osem2(xct_plan *plan, int dN, int sub, float *d_img, const float *d_ratio, void *stream);

/* ---- operators on device memory (all angles, dN slices) ----------------------------
 * xct_fwd    : the reference forward projector `projection` (reconstShare.cl:213-241),
 *              bilinear ray sums, d_sino[dN][pa][px] = A d_img.
 * xct_bp_ref : the reference plain backprojector `backProjection`
 *              (reconstShare.cl:245-275) with ss = 1, sub = 0 (all angles).
 * xct_adj    : the exact adjoint A^T of xct_fwd (d_img = A^T d_sino): the same samples
 *              and bilinear weights (groups of slices: see the slice-interleaved kernels
 *              below).  One slice at a time they are scattered: per window of 8 angles,
 *              the rays within 2^6 of the window's largest |value| are summed as fixed-point
 *              integers (each contribution rounded by at most 2^-16 of its ray's value);
 *              smaller rays, and windows holding a NaN or an infinity, use float atomics.
 *              Results repeat bit for bit when every window takes the integer path only. */
int xct_fwd(xct_plan *plan, int dN, const float *d_img, float *d_sino, void *stream);
int xct_bp_ref(xct_plan *plan, int dN, const float *d_sino, float *d_img, void *stream);
int xct_adj(xct_plan *plan, int dN, const float *d_sino, float *d_img, void *stream);

/* ---- filtered backprojection and the FBP + OS-EM hybrid (methods 7 and 8 of GPU(),
 * GPU.cpp:80-90) ---------------------------------------------------------------------
 * zp is the zero-padded transform length (g_zp, main.cpp:36; default 4096): a power of two
 * with px <= zp <= 16384 and zp >= 64; 0 selects the smallest power of two >= 2*px.
 * xct_fbp_filter      : the ramp filter chain of FBP_execution (GPU.cpp:745-806 over
 *                       FBP.cl:34-160): d_fprj [dN][pa][px] = filtered d_sino.
 * xct_fbp_backproject : backProjectionFBP (FBP.cl:164-188): d_img [dN][ny][nx] =
 *                       (1/(2 pa)) sum over all angles of the linearly interpolated
 *                       d_fprj, 0 outside the circle r < nx/2.
 * xct_fbp_run_device  : FBP_execution (GPU.cpp:665-819): the plan's sinogram correction
 *                       (if any), the filter, the backprojection.  Uses the plan's ratio
 *                       buffer as scratch (calls on one plan must not overlap).
 * xct_hybrid_run_device : hybrid_thread (GPU.cpp:1458-1600): FBP as above, then the base-up
 *                       of its FBPcorrection = 1 branch (slice minimum a of findMinimumX/Y,
 *                       then baseUp, reconstShare.cl:87-177, with order baseup_order 0..64;
 *                       baseupOrder, main.cpp:44, default 4), then `it` OS-EM iterations on
 *                       the corrected sinogram (it < 0: the plan's; sub NULL: plan order).
 * xct_fbp_run / xct_hybrid_run : the same from host buffers (FBP_thread, GPU.cpp:822-893):
 *                       sinograms in, images out (the images' initial contents are not
 *                       read: the backprojection writes every pixel).  Blocking.  Both run a
 *                       batch of two or more slices as two halves, each with its own copies
 *                       on its own stream, as xct_osem_run does. */
int xct_fbp_filter(xct_plan *plan, int dN, int zp, const float *d_sino, float *d_fprj, void *stream);
int xct_fbp_backproject(xct_plan *plan, int dN, const float *d_fprj, float *d_img, void *stream);
int xct_fbp_run_device(xct_plan *plan, int dN, int zp, const float *d_sino, float *d_img, void *stream);
int xct_hybrid_run_device(xct_plan *plan, int dN, int zp, int baseup_order, const float *d_sino, float *d_img,
                          const int *sub, int it, void *stream);
int xct_fbp_run(xct_plan *plan, int dN, int zp, const float *const *sino_host, float *const *img_host);
/* The hybrid with CSitBool set (hybrid_thread, GPU.cpp:1569-1574): FBP and base-up as above,
 * then the compressed-sensing OS-EM of xct_cs_osem_run_device (FISTA_OSEM_execution) instead
 * of OSEM_execution; cs_lambda is CSlambda.  Host-buffer and device forms. */
int xct_hybrid_cs_run_device(xct_plan *plan, int dN, int zp, int baseup_order, const float *d_sino, float *d_img,
                             const int *sub, int it, float cs_lambda, void *stream);
int xct_hybrid_cs_run(xct_plan *plan, int dN, int zp, int baseup_order, const float *const *sino_host,
                      float *const *img_host, const int *sub, int it, float cs_lambda);
int xct_hybrid_run(xct_plan *plan, int dN, int zp, int baseup_order, const float *const *sino_host,
                   float *const *img_host, const int *sub, int it);

/* ---- rotation-centre search (RotationCenterSearch/rotationCenterSearch_ocl.cpp) ------
 * Shifts are s_i = shift_start + shift_step * i (float, :140), i < n; a positive shift
 * samples the sinogram at X + s (the rotation centre moves to px/2 + s).
 * xct_rot_center_shift : rotCenterShift (rotCenterSearch.cl:37-49) of one sinogram
 *                        d_sino [pa][px] for every shift -> d_shifted [n][pa][px].
 * xct_focus_index      : setMask + imgFocusIndex (rotCenterSearch.cl:51-97, 167-232) of
 *                        images d_imgs [n][ny][nx] reconstructed for shifts
 *                        shift_offset .. shift_offset + n - 1 -> d_findex [n] (device):
 *                        sqrt(sum of the relative squared 8-neighbour differences / pixels)
 *                        over the pixels whose 3x3 neighbourhood lies in the shift's mask;
 *                        ang_ini_deg / ang_fin_deg are the first and last projection angles.
 *                        The mask and the sums use the plan's nx, ny (the reference builds
 *                        these kernels without size options: 2048 x 2048).
 * xct_rot_center_search: rotationCenterSearch from the resliced sinogram on (:419-540): per
 *                        shift, the shifted sinogram, an image filled with init_value
 *                        (g_ini), ONE OS-EM iteration with the plan's subsets and sinogram
 *                        correction (:307), the focus index.  d_imgs [n][ny][nx] receives the
 *                        reconstructions, findex (HOST, [n]) the indices, *best the first
 *                        shift index with the smallest one (:505-513).  Batches of max_batch
 *                        shifts; uses the plan's staging and ratio buffers.  Blocking. */
int xct_rot_center_shift(xct_plan *plan, int n, float shift_start, float shift_step, const float *d_sino,
                         float *d_shifted, void *stream);
int xct_focus_index(xct_plan *plan, int n, int shift_offset, float shift_start, float shift_step, float ang_ini_deg,
                    float ang_fin_deg, const float *d_imgs, float *d_findex, void *stream);
int xct_rot_center_search(xct_plan *plan, int n, float shift_start, float shift_step, float ang_ini_deg,
                          float ang_fin_deg, float init_value, const float *d_sino, float *d_imgs, float *findex,
                          int *best, void *stream);

/* ---- reslice: projection stack -> sinograms on the device (Reslice/reslice_ocl.cpp) ----
 * A reslice plan holds the per-angle shifts and constants of reslice() (:153-208):
 * xshift/yshift [n_angles] (host, copied; NULL = 0; the y shift is the z-drift correction
 * of Z_Correction, :89-150), baseup (added to every value) and correction (0/1: multiply by
 * cos(asin(2|X - W/2|/W)), reslice.cl:65-67).
 * xct_reslice : reslice (reslice.cl:52-71) of projections d_proj [n][height][width] for angles
 *               first_angle .. first_angle + n - 1 into d_sino [height][n_angles][width]:
 *               d_sino[Y][th][X] = bilinear(projection th at (X + xshift[th], Y + yshift[th]),
 *               zero outside) + baseup.  Row Y of d_sino is slice Y's sinogram [n_angles][width],
 *               so d_sino + Y0*n_angles*width is a ready dN-slice input of the OS-EM/FBP calls.
 *               Widths that are a multiple of 4 with a 16-byte aligned d_proj run a kernel
 *               that stages each tile's sampler window in shared memory by tensor copies
 *               (TMA); its waits are bounded (about a second), and a tile whose copy misses the
 *               limit is computed from global memory instead, so the output is always complete.
 * xct_reslice_plan_destroy : synchronises the device; returns XCT_E_TIMEOUT if any copy of
 *               the plan's calls missed its wait limit (a fault report only).
 * xct_denoise_sinogram : denoiseSinogram (reslice.cl:223-248) on n_rows sinograms
 *               [n_angles][width]: a value that is a one-angle spike beyond +-threshold against
 *               both angle neighbours (clamped at the ends) becomes their mean.  d_src and
 *               d_dst must not overlap.  Runs on the current device. */
typedef struct xct_reslice_plan xct_reslice_plan;
int xct_reslice_plan_create(xct_ctx *ctx, int width, int height, int n_angles, const float *xshift,
                            const float *yshift, float baseup, int correction, xct_reslice_plan **out);
int xct_reslice(xct_reslice_plan *plan, int first_angle, int n, const float *d_proj, float *d_sino, void *stream);
int xct_reslice_plan_destroy(xct_reslice_plan *plan);
/* Diagnostics (no counterpart in the reference): the limit, in SM clocks, of the staged
 * kernel's waits for its tile copies (default 2^31, about a second).  A negative limit makes
 * every such wait give up at once, so a test can run the global-memory fallback and the
 * XCT_E_TIMEOUT report of xct_reslice_plan_destroy without stalling anything; the copies
 * already issued are still waited for, with the default limit, before the kernel ends. */
int xct_reslice_plan_set_wait_limit(xct_reslice_plan *plan, long long sm_clocks);
int xct_denoise_sinogram(int width, int n_angles, int n_rows, float threshold, const float *d_src, float *d_dst,
                         void *stream);

/* Bounds-checked build (no counterpart in the reference; libxct_checked.so, the same sources
 * compiled with -DXCT_CHECKED): every shared-memory access whose address follows from the
 * geometry rather than from an index test -- the forward tile's footprint loads and
 * accumulator rows, the adjoint's shared accumulator, the backprojectors' bin windows -- is
 * tested against its buffer; one outside is skipped and recorded.  xct_check_report: on the
 * context's device (synchronised first), the number of skipped accesses since the last
 * report, and the first one's site code, index and bounds; resets.  The standard library
 * returns XCT_E_UNSUPPORTED with *count = -1. */
int xct_check_report(xct_ctx *ctx, long long *count, int *site, long long *index, long long *lo, long long *hi);

/* Tracing by environment: with XCT_TRACE set to a file name (or 1 for stderr) when the
 * library is first used, every xct_osem_run_device / xct_osem_run call of a plan without a
 * sinogram correction runs with CUDA events around each launch, synchronously, and appends
 * one JSON line: shape, dN, iterations, summed milliseconds and launch counts per kernel kind,
 * and [forward, finalize, backprojection] milliseconds per subset step.
 *
 * Tracing by call: xct_osem_run_device with CUDA events around every launch.  The reference
 * enables CL_QUEUE_PROFILING_ENABLE but never reads the events
 * (share source/OCL_platform_device_class.cpp:175-178).  ms[0..3] = summed device time of
 * the forward-projection launches, of the ratio/finalize launches, of the
 * backprojection launches, and of the whole loop; launches[0..3] = their counts.
 * Synchronous. */
int xct_osem_profile(xct_plan *plan, int dN, const float *d_sino, float *d_img, const int *sub, int it,
                     void *stream, float *ms, long long *launches);

/* ---- forward-projector tiles: autotuner -------------------------------------------------
 * No counterpart in the reference (it launches one work-item per ray).  The tiled forward
 * projector has two launch-shape parameters: the tile side (44, 60, 76 or 92 texels) and the
 * subset angles one CTA serves (1..128).  A plan starts with the choice cached for its shape
 * (device name, nx, ny, px, pa, ss, max_batch) -- in this process, or in the JSON file named by
 * the environment variable XCT_TUNE_CACHE -- or else the largest tiles that still give two
 * waves of CTAs.  xct_plan_autotune times every candidate for dN slices on the plan's own
 * geometry (its staging buffers are the input; no caller data is read or written), keeps the
 * fastest, and records it in memory and in cache_path (NULL: XCT_TUNE_CACHE; no file if
 * neither).  A cached entry is reused without timing unless flags has XCT_TUNE_FORCE.
 * Synchronous.  xct_batch_plan_autotune does the same for a batch plan: each geometry
 * group's plan, and one choice for the slices its graph serves (the next xct_batch_run
 * captures its graph again).  The *_tuning calls report
 * the current choice; xct_plan_set_tuning sets one by hand. */
#define XCT_TUNE_FORCE 1
int xct_plan_autotune(xct_plan *plan, int dN, const char *cache_path, int flags, void *stream);
int xct_plan_tuning(xct_plan *plan, int *fwd_tile, int *ang_chunk);
int xct_plan_set_tuning(xct_plan *plan, int fwd_tile, int ang_chunk);
int xct_batch_plan_autotune(xct_batch_plan *plan, const char *cache_path, int flags, void *stream);
int xct_batch_plan_tuning(xct_batch_plan *plan, int *fwd_tile, int *ang_chunk);

/* ---- slice-interleaved kernels ---------------------------------------------------------
 * No counterpart in the reference (its OSEM1/OSEM2 work-items each serve one slice).  The
 * slices of one call share their geometry, so a plan can serve them in groups:
 *  - forward projection (OSEM1, xct_fwd) in groups of XCT_MULTISLICE_SLICES (eight): a CTA
 *    stages one tile of the eight slices (one 128-byte line of bilinear coefficients per
 *    texel), a quarter-warp walks two rays, and each lane reads the eight slices of its sample
 *    in a rotated order (no shared-memory bank conflict; a sample's coordinates are found once
 *    for all eight).  Results agree with the per-slice kernel to float rounding of the partial
 *    ray sums;
 *  - backprojection + update (OSEM2) in groups of eight, and a pair left over in a two-slice
 *    form: one bin expression per eight (two) gathers; bit-identical to the per-slice kernel;
 *    the FBP backprojection (xct_fbp_backproject, the FBP and hybrid runs) the same way, also
 *    bit-identical;
 *  - the exact adjoint (xct_adj and the FISTA adjoint step) in groups of ten or eight as a
 *    gather: a thread owns one base texel, finds the samples whose base texel it is with the
 *    forward projector's own arithmetic and sums their weighted ray values in registers (no
 *    atomics; float sums in an order fixed by the geometry, so repeatable bit for bit); a
 *    group of four left over in scatter form, each sample's coordinates and weights serving
 *    the four slices.  Both agree with the per-slice kernel to float rounding (the scatter
 *    form exactly where its fixed-point path applies).
 * With it on, a call's slices go in groups through these kernels and the rest through the
 * per-slice ones, and a call that runs as two halves cuts them at a multiple of eight.  The
 * value is the number of subset angles one forward CTA serves (1..128); 0 turns all three
 * off.  Plans start on (128) when max_batch >= 8 and the forward tiles of one group give at
 * least two CTAs per SM, else off (the tile cache and the autotuner leave this switch
 * alone). */
#define XCT_MULTISLICE_SLICES 8
int xct_plan_multislice(xct_plan *plan, int *ang_chunk);
int xct_plan_set_multislice(xct_plan *plan, int ang_chunk);

/* FP32 FMA throughput of a device (TFLOP/s), measured by a dependent-chain-free FMA
 * kernel: the roofline denominator for the projectors. */
int xct_fp32_peak(int device, float *tflops);

/* Synchronise the plan's stream; report the device time of the last xct_osem_run (ms). */
int xct_plan_sync(xct_plan *plan);
int xct_plan_last_ms(xct_plan *plan, float *ms);

/* Kernel launches issued by this process since load (for launch accounting). */
long long xct_launch_count(void);

/* Message of the last failing call on this thread ("" if none). */
const char *xct_last_error(void);
int xct_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
