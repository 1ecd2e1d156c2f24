// xct_batch.cu -- OS-EM over many slices of different shapes in one graph of persistent
// launches (CT-XAFS stacks: energies x slices, every slice its own width, bin count and
// angle list).
//
// The reference reconstructs a batch of dN slices of ONE shape per OSEM_execution call
// (GPU.cpp:125-240).  A batch plan instead holds n slices of any shapes that share the
// subset count; every subset step is three persistent launches -- forward projection,
// ratio, backprojection+update -- whose CTAs take (slice, tile) work units from a device
// queue, so small slices fill the GPU together with large ones.  The whole subset/iteration
// loop is captured once in a CUDA graph and replayed; the slices' buffer pointers live in a
// device descriptor table written before each replay, so one plan serves any buffers of
// the planned shapes.
//
// Slices that share one geometry (sizes, centre, modes, angle list) -- in a CT-XAFS stack the
// slices of one width at one energy -- form a group; a group of at least eight runs through
// a single-shape plan of its own (the slice-interleaved kernels, two halves of up to eight
// slices per call on two streams), its slices copied into one contiguous scratch pair when
// the caller's buffers are not already consecutive.  The graph serves the other slices.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "xct_internal.h"

struct xct_batch_plan {
    xct_ctx *ctx = nullptr;
    int n = 0, ss = 0, it = 0;
    std::vector<int> sub;             // subset order (GPU.cpp:564-582)
    std::vector<XctItemDev> host;     // descriptors (pointers filled per run)
    XctItemDev *d_items = nullptr;
    int *d_bases = nullptr;           // [3][m+1] over the graph's m slices
    int *d_queues = nullptr;          // [it*ss][3]
    float2 *d_trig = nullptr;
    float *d_ratio = nullptr;
    double *d_acc = nullptr;
    int grids[3] = {0, 0, 0};
    int fwd_T = 92, fwd_chunk = 128;  // forward tiles of every slice (autotuned, cached)
    std::vector<int> bases;           // [3][n+1] work-unit prefix sums for fwd_T, fwd_chunk
    size_t n_acc = 0;
    std::string key;                  // tune-cache key of the batch's shapes
    cudaStream_t cap = nullptr;       // capture stream
    cudaGraphExec_t exec = nullptr;
    size_t queue_bytes = 0;
    // sinogram correction: corrected sinograms and factor tables of the items that have one
    float *d_corr = nullptr;
    float *d_corr_fac = nullptr;
    int max_px = 0, max_pa = 0;
    bool any_corr = false;
    // compressed sensing over stacks of consecutive slices (empty: off)
    std::vector<int> stack_first;     // first item of each stack
    std::vector<XctStackDev> stacks;  // descriptors (images filled per run)
    XctStackDev *d_stacks = nullptr;
    float *d_cs = nullptr;            // w, beta, x' of every stack
    long long max_vox = 0;
    float cs_lambda = 0.0f;           // the kernels' lambda
    // geometry groups (at least kGroupMin slices of one geometry): a single-shape plan each,
    // `batch` slices per call; the graph serves `glist` -- every slice, or with groups in use
    // the slices of no group (`rest`)
    struct Group {
        xct_plan *plan = nullptr;
        int batch = 0;
        std::vector<int> items;
        size_t nprj = 0, nimg = 0;
    };
    std::vector<Group> groups;
    std::vector<int> rest;
    bool grouping = true;          // xct_batch_plan_set_grouping
    float *d_gscratch = nullptr;   // [batch][pa][px] sinograms then [batch][ny][nx] images
    std::vector<int> glist;        // the graph's slices, in descriptor order
    std::vector<XctItemDev> gdesc; // their descriptors
    bool glist_corr = false;       // some slice of the graph has a sinogram correction
};

static void batch_free(xct_batch_plan *p)
{
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->cap) cudaStreamDestroy(p->cap);
    cudaFree(p->d_items);
    cudaFree(p->d_bases);
    cudaFree(p->d_queues);
    cudaFree(p->d_trig);
    cudaFree(p->d_ratio);
    cudaFree(p->d_acc);
    cudaFree(p->d_corr);
    cudaFree(p->d_corr_fac);
    cudaFree(p->d_stacks);
    cudaFree(p->d_cs);
    cudaFree(p->d_gscratch);
    for (auto &G : p->groups)
        if (G.plan) xct_osem_plan_destroy(G.plan);
    delete p;
}

// Forward tiles (T, chunk) for every slice: work units, their prefix sums over the graph's
// slices (uploaded), the persistent grids; a captured graph is dropped (the next run
// captures again).
static int batch_layout(xct_batch_plan *p, int T, int chunk)
{
    std::vector<int> units(3 * p->host.size());  // forward, finalize, backprojection units
    for (size_t i = 0; i < p->host.size(); ++i) {
        XctItemDev &d = p->host[i];
        d.g.fwd_T = T;
        d.g.fwd_chunk = chunk;
        xct_batched_units(d.g, d.fwd_ntx, d.fwd_nty, units[3 * i], units[3 * i + 1], d.bp_ntx, units[3 * i + 2]);
    }
    const int m = (int)p->glist.size();
    p->bases.assign(3 * (size_t)(m + 1), 0);
    p->glist_corr = false;
    for (int j = 0; j < m; ++j) {
        const int i = p->glist[j];
        for (int q = 0; q < 3; ++q) p->bases[q * (m + 1) + j + 1] = p->bases[q * (m + 1) + j] + units[3 * i + q];
        p->glist_corr = p->glist_corr || p->host[i].corr_mode > 0;
    }
    XCT_CUDA_TRY(cudaMemcpy(p->d_bases, p->bases.data(), sizeof(int) * p->bases.size(), cudaMemcpyHostToDevice));
    int rc = xct_batched_grids(p->ctx->device, p->ctx->sm_count, T, p->grids);
    if (rc) return rc;
    // the finalize step runs one CTA per unit (ratio row) rather than a persistent grid: its
    // units are short, so a device queue's per-unit latency would dominate
    p->grids[1] = p->bases[1 * (m + 1) + m];
    p->fwd_T = T;
    p->fwd_chunk = chunk;
    if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    return XCT_OK;
}

// Two geometries describe the same reconstruction (sizes, centre, modes, angle list).
static bool same_geom(const xct_geom &a, const xct_geom &b)
{
    const float ca = a.center_bin < 0.0f ? (float)a.px * 0.5f : a.center_bin;
    const float cb = b.center_bin < 0.0f ? (float)b.px * 0.5f : b.center_bin;
    return a.nx == b.nx && a.ny == b.ny && a.px == b.px && a.pa == b.pa && a.ss == b.ss && ca == cb &&
           a.measured_fetch_mode == b.measured_fetch_mode && a.subset_mode == b.subset_mode &&
           a.correction_mode == b.correction_mode &&
           std::equal(a.angles_deg, a.angles_deg + a.pa, b.angles_deg);
}

// A geometry group needs whole slice groups of the slice-interleaved forward projector;
// its calls take two halves of up to that many slices.
static const int kGroupMin = XCT_MULTISLICE_SLICES;
static int group_batch(int n) { return std::min(n, 2 * XCT_MULTISLICE_SLICES); }

// FNV-1a over a geometry's fields and angle bits: equal geometries hash alike.
static unsigned long long geom_hash(const xct_geom &g)
{
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](unsigned v) {
        h ^= v;
        h *= 1099511628211ull;
    };
    const float c = g.center_bin < 0.0f ? (float)g.px * 0.5f : g.center_bin;
    unsigned cb;
    memcpy(&cb, &c, 4);
    const int v[9] = {g.nx, g.ny, g.px, g.pa, g.ss, g.measured_fetch_mode, g.subset_mode, g.correction_mode, (int)cb};
    for (int q = 0; q < 9; ++q) mix((unsigned)v[q]);
    for (int a = 0; a < g.pa; ++a) {
        unsigned b;
        memcpy(&b, &g.angles_deg[a], 4);
        mix(b);
    }
    return h;
}

static std::vector<int> all_items(int n)
{
    std::vector<int> v(n);
    for (int i = 0; i < n; ++i) v[i] = i;
    return v;
}

// Tune-cache key of the graph's slices (their shapes, in order).
static std::string graph_key(const xct_batch_plan *p)
{
    unsigned long long h = 1469598103934665603ull;  // FNV-1a over the shapes
    for (int i : p->glist) {
        const KGeom &g = p->host[i].g;
        const int v[6] = {g.nx, g.ny, g.px, g.pa, p->host[i].cover ? 1 : 0, 0};
        for (int q = 0; q < 6; ++q) {
            h ^= (unsigned)v[q];
            h *= 1099511628211ull;
        }
    }
    char kb[96];
    snprintf(kb, sizeof kb, "batch%d-%016llx", (int)p->glist.size(), h);
    return xct_tune_key(p->ctx->name, 0, 0, 0, 0, p->ss, (int)p->glist.size()) + "|" + kb;
}

extern "C" int xct_batch_plan_create(xct_ctx *ctx, int n, const xct_geom *geoms, int it, xct_batch_plan **out)
{
    if (!ctx || !out || !geoms || n <= 0) return xct_fail(XCT_E_INVALID, "xct_batch_plan_create: bad arguments");
    *out = nullptr;
    if (it < 0) return xct_fail(XCT_E_INVALID, "xct_batch_plan_create: iterations must be >= 0");
    const int ss = geoms[0].ss;
    for (int i = 0; i < n; ++i) {
        int rc = xct_check_geom(&geoms[i]);
        if (rc) return rc;
        if (geoms[i].ss != ss)
            return xct_fail(XCT_E_INVALID, "xct_batch_plan_create: every slice of a batch needs the same subset count");
    }
    XCT_CUDA_TRY(cudaSetDevice(ctx->device));
    xct_batch_plan *p = new (std::nothrow) xct_batch_plan();
    if (!p) return xct_fail(XCT_E_NOMEM, "xct_batch_plan_create: host allocation failed");
    p->ctx = ctx;
    p->n = n;
    p->ss = ss;
    p->it = it;
    p->sub.resize(ss);
    xct_subset_order_host(ss, p->sub.data());
    auto fail = [&](cudaError_t e, const char *what) {
        int r = xct_cuda_fail(e, what);
        batch_free(p);
        return r;
    };
    // sizes
    size_t n_trig = 0, n_ratio = 0, n_acc = 0, n_corr = 0, n_fac = 0;
    p->host.resize(n);
    for (int i = 0; i < n; ++i) {
        const xct_geom &g = geoms[i];
        XctItemDev &d = p->host[i];
        KGeom &k = d.g;
        k.nx = g.nx;
        k.ny = g.ny;
        k.px = g.px;
        k.pa = g.pa;
        k.ss = g.ss;
        k.depth = std::max(g.nx, g.ny);
        k.hx = (float)g.nx * 0.5f;
        k.hy = (float)g.ny * 0.5f;
        k.hd = (float)k.depth * 0.5f;
        k.cx = g.center_bin < 0.0f ? (float)g.px * 0.5f : g.center_bin;
        k.fetch = g.measured_fetch_mode;
        d.cover = g.subset_mode == XCT_SUBSETS_COVER;
        d.corr_mode = g.correction_mode;
        n_trig += g.pa;
        n_ratio += (size_t)g.pa * g.px;
        n_acc += (size_t)((g.pa + g.ss - 1) / g.ss) * g.px;
        p->max_px = std::max(p->max_px, g.px);
        p->max_pa = std::max(p->max_pa, g.pa);
        if (g.correction_mode > 0) {
            p->any_corr = true;
            n_corr += (size_t)g.pa * g.px;
            n_fac += 2 * (size_t)g.pa + g.px;
        }
    }
    cudaError_t e;
    if ((e = cudaMalloc(&p->d_items, sizeof(XctItemDev) * n)) != cudaSuccess) return fail(e, "cudaMalloc items");
    if ((e = cudaMalloc(&p->d_bases, sizeof(int) * 3 * (size_t)(n + 1))) != cudaSuccess)
        return fail(e, "cudaMalloc bases");
    p->n_acc = n_acc;
    p->queue_bytes = sizeof(int) * 3 * (size_t)std::max(1, it * ss);
    if ((e = cudaMalloc(&p->d_queues, p->queue_bytes)) != cudaSuccess) return fail(e, "cudaMalloc queues");
    if ((e = cudaMalloc(&p->d_trig, sizeof(float2) * n_trig)) != cudaSuccess) return fail(e, "cudaMalloc trig");
    if ((e = cudaMalloc(&p->d_ratio, sizeof(float) * n_ratio)) != cudaSuccess) return fail(e, "cudaMalloc ratio");
    if ((e = cudaMalloc(&p->d_acc, sizeof(double) * n_acc)) != cudaSuccess) return fail(e, "cudaMalloc acc");
    // ratio rows OSEM1 never writes read as 0 and stay 0; the accumulator starts at 0 and the
    // finalize kernel clears what it reads
    if ((e = cudaMemset(p->d_ratio, 0, sizeof(float) * n_ratio)) != cudaSuccess) return fail(e, "memset ratio");
    if ((e = cudaMemset(p->d_acc, 0, sizeof(double) * n_acc)) != cudaSuccess) return fail(e, "memset acc");
    if (p->any_corr) {
        if ((e = cudaMalloc(&p->d_corr, sizeof(float) * n_corr)) != cudaSuccess) return fail(e, "cudaMalloc corr");
        if ((e = cudaMalloc(&p->d_corr_fac, sizeof(float) * n_fac)) != cudaSuccess) return fail(e, "cudaMalloc fac");
    }
    size_t ot = 0, orat = 0, oacc = 0, ocorr = 0, ofac = 0;
    std::vector<float2> cs;
    std::vector<float> af, bf;
    for (int i = 0; i < n; ++i) {
        const xct_geom &g = geoms[i];
        XctItemDev &d = p->host[i];
        xct_trig_table(g.angles_deg, g.pa, cs);
        if ((e = cudaMemcpy(p->d_trig + ot, cs.data(), sizeof(float2) * g.pa, cudaMemcpyHostToDevice)) != cudaSuccess)
            return fail(e, "upload trig");
        d.trig = p->d_trig + ot;
        d.ratio = p->d_ratio + orat;
        d.acc = p->d_acc + oacc;
        d.sino = nullptr;
        d.img = nullptr;
        d.sino_in = nullptr;
        d.corr = nullptr;
        d.corr_ang = nullptr;
        d.corr_bin = nullptr;
        if (g.correction_mode > 0) {
            xct_corr_tables(g.angles_deg, g.pa, g.px, af, bf);
            if ((e = cudaMemcpy(p->d_corr_fac + ofac, af.data(), sizeof(float) * af.size(), cudaMemcpyHostToDevice)) !=
                    cudaSuccess ||
                (e = cudaMemcpy(p->d_corr_fac + ofac + af.size(), bf.data(), sizeof(float) * bf.size(),
                                cudaMemcpyHostToDevice)) != cudaSuccess)
                return fail(e, "upload correction factors");
            d.corr = p->d_corr + ocorr;
            d.corr_ang = p->d_corr_fac + ofac;
            d.corr_bin = p->d_corr_fac + ofac + af.size();
            ocorr += (size_t)g.pa * g.px;
            ofac += af.size() + bf.size();
        }
        ot += g.pa;
        orat += (size_t)g.pa * g.px;
        oacc += (size_t)((g.pa + g.ss - 1) / g.ss) * g.px;
    }
    // geometry groups: slices of one geometry, found through a hash of the geometry and
    // checked member by member
    {
        std::vector<std::pair<unsigned long long, int>> hs(n);
        for (int i = 0; i < n; ++i) hs[i] = {geom_hash(geoms[i]), i};
        std::stable_sort(hs.begin(), hs.end());
        std::vector<char> taken(n, 0);
        for (size_t a0 = 0; a0 < hs.size();) {
            size_t a1 = a0;
            while (a1 < hs.size() && hs[a1].first == hs[a0].first) ++a1;
            for (size_t u = a0; u < a1; ++u) {
                const int i = hs[u].second;
                if (taken[i]) continue;
                std::vector<int> members{i};
                taken[i] = 1;
                for (size_t v = u + 1; v < a1; ++v) {
                    const int j = hs[v].second;
                    if (!taken[j] && same_geom(geoms[i], geoms[j])) {
                        members.push_back(j);
                        taken[j] = 1;
                    }
                }
                std::sort(members.begin(), members.end());
                if ((int)members.size() >= kGroupMin) {
                    xct_batch_plan::Group G;
                    G.items = members;
                    p->groups.push_back(std::move(G));
                } else {
                    p->rest.insert(p->rest.end(), members.begin(), members.end());
                }
            }
            a0 = a1;
        }
        std::sort(p->rest.begin(), p->rest.end());
        std::sort(p->groups.begin(), p->groups.end(),
                  [](const xct_batch_plan::Group &x, const xct_batch_plan::Group &y) { return x.items[0] < y.items[0]; });
    }
    size_t scratch = 0;
    for (auto &G : p->groups) {
        xct_geom g = geoms[G.items[0]];
        g.it = it;
        g.max_batch = group_batch((int)G.items.size());
        g.kernels = XCT_KERNELS_TILED;
        int rc = xct_osem_plan_create(ctx, &g, &G.plan);
        if (rc) {
            batch_free(p);
            return rc;
        }
        G.batch = g.max_batch;
        G.nprj = (size_t)g.pa * g.px;
        G.nimg = (size_t)g.nx * g.ny;
        scratch = std::max(scratch, (size_t)G.batch * (G.nprj + G.nimg));
    }
    if (scratch > 0 && (e = cudaMalloc(&p->d_gscratch, sizeof(float) * scratch)) != cudaSuccess)
        return fail(e, "cudaMalloc group scratch");
    // the graph's slices with groups in use (every slice when all are grouped: the graph
    // then serves them only with groups off), its tiles: this list's cached choice, else the
    // default rule
    p->glist = p->rest.empty() ? all_items(n) : p->rest;
    p->key = graph_key(p);
    TuneChoice c;
    if (!xct_tune_lookup(p->key, xct_tune_env_path(), c))
        c = xct_tune_default(ctx->sm_count, [&](int T, int ch) {
            long long t = 0;
            for (int i : p->glist) {
                const int rows = (geoms[i].pa + ss - 1) / ss;
                t += (long long)((geoms[i].nx + T) / T) * ((geoms[i].ny + T) / T) * ((rows + ch - 1) / ch);
            }
            return t;
        });
    int rc = batch_layout(p, c.T, c.chunk);
    if (rc) {
        batch_free(p);
        return rc;
    }
    if ((e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking)) != cudaSuccess) return fail(e, "stream");
    *out = p;
    return XCT_OK;
}

extern "C" int xct_batch_plan_destroy(xct_batch_plan *p)
{
    if (p) cudaSetDevice(p->ctx->device);
    batch_free(p);
    return XCT_OK;
}

// Capture the whole loop: clear the queue counters, the corrections (if any), then it x ss
// subset steps -- with compressed sensing, w = x and beta = 0 first, the first subset step is
// ISTA3D of the images before any OS-EM update (FISTA_OSEM_execution passes the image before
// that subset's update to ISTA3D, GPU.cpp:335-336, so that OS-EM step is dead work and is
// skipped, as in the single-shape plans), and every later one is the OS-EM step then FISTA3D,
// each proximal result copied back into the images.
static int capture(xct_batch_plan *p)
{
    cudaGraph_t graph = nullptr;
    XCT_CUDA_TRY(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
    int rc = XCT_OK;
    const int sm = p->ctx->sm_count, ns = (int)p->stacks.size();
    const bool cs = ns > 0;
    cudaError_t e = cudaMemsetAsync(p->d_queues, 0, p->queue_bytes, p->cap);
    if (e != cudaSuccess) rc = xct_cuda_fail(e, "capture memset");
    const int m = (int)p->glist.size();
    if (rc == XCT_OK && p->glist_corr) rc = launch_sino_correction_batched(p->d_items, m, p->max_px, p->max_pa, p->cap);
    if (rc == XCT_OK && cs) rc = launch_stack_copy(p->d_stacks, ns, p->max_vox, 1, sm, p->cap);
    bool first = true;
    for (int i = 0; i < p->it && rc == XCT_OK; ++i)
        for (int k = 0; k < p->ss && rc == XCT_OK; ++k) {
            if (cs && first) {
                rc = launch_ista3d_stacks(p->d_stacks, ns, p->max_vox, p->cs_lambda, sm, p->cap);
                first = false;
            } else {
                rc = launch_osem_step_batched(p->d_items, p->d_bases, m, p->sub[k],
                                              p->d_queues + 3 * (size_t)(i * p->ss + k), p->grids, p->fwd_T, p->cap);
                if (rc == XCT_OK && cs) rc = launch_fista3d_stacks(p->d_stacks, ns, p->max_vox, p->cs_lambda, sm, p->cap);
            }
            if (rc == XCT_OK && cs) rc = launch_stack_copy(p->d_stacks, ns, p->max_vox, 0, sm, p->cap);
        }
    e = cudaStreamEndCapture(p->cap, &graph);
    if (rc == XCT_OK && e != cudaSuccess) rc = xct_cuda_fail(e, "cudaStreamEndCapture");
    if (rc == XCT_OK) {
        e = cudaGraphInstantiate(&p->exec, graph, 0);
        if (e != cudaSuccess) rc = xct_cuda_fail(e, "cudaGraphInstantiate");
    }
    if (graph) cudaGraphDestroy(graph);
    return rc;
}

extern "C" int xct_batch_run(xct_batch_plan *p, const float *const *d_sino, float *const *d_img, void *stream)
{
    XCT_RANGE("xct_batch_run");
    if (!p || !d_sino || !d_img) return xct_fail(XCT_E_INVALID, "xct_batch_run: null argument");
    for (int i = 0; i < p->n; ++i)
        if (!d_sino[i] || !d_img[i]) return xct_fail(XCT_E_INVALID, "xct_batch_run: null slice pointer");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;  // NULL: the legacy default stream
    // the groups (not with compressed sensing, whose stacks the graph serves): their calls
    // in place when a call's slices are consecutive in one pair of arrays, else through the
    // scratch pair
    const bool use_groups = p->grouping && p->stacks.empty() && !p->groups.empty();
    if (use_groups) {
        for (const auto &G : p->groups) {
            for (size_t off = 0; off < G.items.size(); off += (size_t)G.batch) {
                const int cnt = (int)std::min((size_t)G.batch, G.items.size() - off);
                const int *ix = G.items.data() + off;
                bool contiguous = true;
                for (int j = 1; j < cnt && contiguous; ++j)
                    contiguous = d_sino[ix[j]] == d_sino[ix[0]] + j * G.nprj && d_img[ix[j]] == d_img[ix[0]] + j * G.nimg;
                int rc;
                if (contiguous) {
                    rc = xct_osem_run_device(G.plan, cnt, d_sino[ix[0]], d_img[ix[0]], nullptr, p->it, stream);
                } else {
                    float *gs = p->d_gscratch, *gi = p->d_gscratch + (size_t)cnt * G.nprj;
                    for (int j = 0; j < cnt; ++j) {
                        XCT_CUDA_TRY(cudaMemcpyAsync(gs + j * G.nprj, d_sino[ix[j]], sizeof(float) * G.nprj,
                                                     cudaMemcpyDeviceToDevice, st));
                        XCT_CUDA_TRY(cudaMemcpyAsync(gi + j * G.nimg, d_img[ix[j]], sizeof(float) * G.nimg,
                                                     cudaMemcpyDeviceToDevice, st));
                    }
                    rc = xct_osem_run_device(G.plan, cnt, gs, gi, nullptr, p->it, stream);
                    for (int j = 0; j < cnt && rc == XCT_OK; ++j)
                        XCT_CUDA_TRY(cudaMemcpyAsync(d_img[ix[j]], gi + j * G.nimg, sizeof(float) * G.nimg,
                                                     cudaMemcpyDeviceToDevice, st));
                }
                if (rc) return rc;
            }
        }
        if (p->rest.empty()) return XCT_OK;
    }
    // the graph: the slices of no group, or every slice
    const std::vector<int> want = use_groups ? p->rest : all_items(p->n);
    if (want != p->glist) {
        p->glist = want;
        int rc = batch_layout(p, p->fwd_T, p->fwd_chunk);
        if (rc) return rc;
    }
    if (!p->exec) {
        int rc = capture(p);
        if (rc) return rc;
    }
    // a stack's images must be one [dN][ny][nx] array
    for (size_t s = 0; s < p->stacks.size(); ++s) {
        const int f = p->stack_first[s];
        const size_t m = (size_t)p->stacks[s].nx * p->stacks[s].ny;
        for (int j = 1; j < p->stacks[s].dN; ++j)
            if (d_img[f + j] != d_img[f] + j * m)
                return xct_fail(XCT_E_INVALID,
                                "xct_batch_run: with compressed sensing, the images of a stack must be consecutive in "
                                "one array");
        p->stacks[s].img = d_img[f];
    }
    const int m = (int)p->glist.size();
    p->gdesc.resize(m);
    for (int j = 0; j < m; ++j) {
        const int i = p->glist[j];
        p->host[i].sino_in = d_sino[i];
        p->host[i].sino = p->host[i].corr_mode > 0 ? p->host[i].corr : d_sino[i];
        p->host[i].img = d_img[i];
        p->gdesc[j] = p->host[i];
    }
    XCT_CUDA_TRY(cudaMemcpyAsync(p->d_items, p->gdesc.data(), sizeof(XctItemDev) * m, cudaMemcpyHostToDevice, st));
    if (!p->stacks.empty())
        XCT_CUDA_TRY(cudaMemcpyAsync(p->d_stacks, p->stacks.data(), sizeof(XctStackDev) * p->stacks.size(),
                                     cudaMemcpyHostToDevice, st));
    XCT_CUDA_TRY(cudaGraphLaunch(p->exec, st));
    // three per OS-EM step (the first step has none with compressed sensing), the
    // correction, and with compressed sensing the setup copy plus two per step
    const long long steps = (long long)p->it * p->ss, cs = p->stacks.empty() ? 0 : 1;
    g_xct_launches.fetch_add(3 * (steps - cs) + (p->glist_corr ? (m + 65534) / 65535 : 0) + cs * (1 + 2 * steps),
                             std::memory_order_relaxed);
    return XCT_OK;
}

// Compressed sensing over stacks: stack_len[s] consecutive items of one shape form stack s
// (the lengths add up to the batch's n); nstacks 0 turns it off.  The captured graph is
// dropped (the next run captures again).
extern "C" int xct_batch_plan_set_cs(xct_batch_plan *p, float cs_lambda, int nstacks, const int *stack_len)
{
    if (!p) return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_cs: plan is null");
    if (nstacks < 0 || (nstacks > 0 && !stack_len)) return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_cs: bad stacks");
    if (!(cs_lambda >= 0.0f && cs_lambda < 1.0e30f))
        return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_cs: cs_lambda must be finite and >= 0");
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    std::vector<int> first;
    std::vector<XctStackDev> st;
    long long total = 0, max_vox = 0;
    int at = 0;
    for (int s = 0; s < nstacks; ++s) {
        const int len = stack_len[s];
        if (len <= 0 || at + len > p->n) return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_cs: stack lengths exceed n");
        const KGeom &g0 = p->host[at].g;
        for (int j = 1; j < len; ++j)
            if (p->host[at + j].g.nx != g0.nx || p->host[at + j].g.ny != g0.ny)
                return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_cs: the slices of a stack need one image size");
        XctStackDev d = {nullptr, nullptr, nullptr, nullptr, g0.nx, g0.ny, len};
        first.push_back(at);
        st.push_back(d);
        const long long v = (long long)g0.nx * g0.ny * len;
        total += v;
        max_vox = std::max(max_vox, v);
        at += len;
    }
    if (nstacks > 0 && at != p->n) return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_cs: stack lengths must add up to n");
    cudaFree(p->d_cs);
    cudaFree(p->d_stacks);
    p->d_cs = nullptr;
    p->d_stacks = nullptr;
    p->stacks.clear();
    p->stack_first.clear();
    if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
    if (nstacks == 0) return XCT_OK;
    XCT_CUDA_TRY(cudaMalloc(&p->d_cs, sizeof(float) * 3 * (size_t)total));
    XCT_CUDA_TRY(cudaMalloc(&p->d_stacks, sizeof(XctStackDev) * nstacks));
    long long o = 0;
    for (auto &d : st) {
        const long long v = (long long)d.nx * d.ny * d.dN;
        d.w = p->d_cs + o;
        d.beta = p->d_cs + total + o;
        d.xn = p->d_cs + 2 * total + o;
        o += v;
    }
    p->stacks = st;
    p->stack_first = first;
    p->max_vox = max_vox;
    p->cs_lambda = xct_cs_kernel_lambda(cs_lambda);
    return XCT_OK;
}

extern "C" int xct_osem_run_batched(xct_ctx *ctx, int n, const xct_geom *geoms, const float *const *d_sino,
                                    float *const *d_img, int it, void *stream)
{
    xct_batch_plan *p = nullptr;
    int rc = xct_batch_plan_create(ctx, n, geoms, it, &p);
    if (rc) return rc;
    rc = xct_batch_run(p, d_sino, d_img, stream);
    if (rc == XCT_OK) {
        cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
        if (e != cudaSuccess) rc = xct_cuda_fail(e, "xct_osem_run_batched: sync");
    }
    xct_batch_plan_destroy(p);
    return rc;
}

// Slices per call when every slice is in one geometry group (0: not so).
extern "C" int xct_batch_plan_uniform(xct_batch_plan *p, int *slices_per_call)
{
    if (!p || !slices_per_call) return xct_fail(XCT_E_INVALID, "xct_batch_plan_uniform: null argument");
    const bool uni = p->groups.size() == 1 && (int)p->groups[0].items.size() == p->n;
    *slices_per_call = uni ? p->groups[0].batch : 0;
    return XCT_OK;
}

// The geometry groups: how many, and how many slices they hold.
extern "C" int xct_batch_plan_groups(xct_batch_plan *p, int *ngroups, int *grouped_slices)
{
    if (!p || !ngroups || !grouped_slices) return xct_fail(XCT_E_INVALID, "xct_batch_plan_groups: null argument");
    *ngroups = (int)p->groups.size();
    *grouped_slices = p->n - (int)p->rest.size();
    return XCT_OK;
}

// Groups on (1, the default) or off (0: the graph serves every slice).
extern "C" int xct_batch_plan_set_grouping(xct_batch_plan *p, int on)
{
    if (!p) return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_grouping: plan is null");
    if (on != 0 && on != 1) return xct_fail(XCT_E_INVALID, "xct_batch_plan_set_grouping: on must be 0 or 1");
    p->grouping = on != 0;
    return XCT_OK;
}

extern "C" int xct_batch_plan_tuning(xct_batch_plan *p, int *fwd_tile, int *ang_chunk)
{
    if (!p || !fwd_tile || !ang_chunk) return xct_fail(XCT_E_INVALID, "xct_batch_plan_tuning: null argument");
    *fwd_tile = p->fwd_T;
    *ang_chunk = p->fwd_chunk;
    return XCT_OK;
}

// Time the batched forward launch (subset 0) for every candidate (T, chunk) and keep the
// fastest; the slices read one scratch image of the largest size (the cost depends on the
// geometry only).  The choice is cached under the batch's shape key.
extern "C" int xct_batch_plan_autotune(xct_batch_plan *p, const char *cache_path, int flags, void *stream)
{
    XCT_RANGE("xct_batch_plan_autotune");
    if (!p) return xct_fail(XCT_E_INVALID, "xct_batch_plan_autotune: plan is null");
    if (!cache_path) cache_path = xct_tune_env_path();
    for (auto &G : p->groups) {  // the groups' own tiles
        int rc = xct_plan_autotune(G.plan, G.batch, cache_path, flags, stream);
        if (rc) return rc;
    }
    // the graph's tiles, for the slices it serves as the plan stands (every slice when all
    // are grouped: the graph then serves them only with groups off)
    const bool use_groups = p->grouping && p->stacks.empty() && !p->groups.empty();
    const std::vector<int> want = use_groups && !p->rest.empty() ? p->rest : all_items(p->n);
    if (want != p->glist) {
        p->glist = want;
        int rc = batch_layout(p, p->fwd_T, p->fwd_chunk);
        if (rc) return rc;
    }
    p->key = graph_key(p);
    TuneChoice best;
    if (!(flags & XCT_TUNE_FORCE) && xct_tune_lookup(p->key, cache_path, best))
        return batch_layout(p, best.T, best.chunk);
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const int m = (int)p->glist.size();
    size_t maxpix = 0;
    int max_rows = 1;
    for (int i : p->glist) {
        const XctItemDev &d = p->host[i];
        maxpix = std::max(maxpix, (size_t)d.g.nx * d.g.ny);
        max_rows = std::max(max_rows, (d.g.pa + d.g.ss - 1) / d.g.ss);
    }
    float *scratch = nullptr;
    XCT_CUDA_TRY(cudaMalloc(&scratch, sizeof(float) * maxpix));
    std::vector<XctItemDev> tmp(m);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int T0 = p->fwd_T, c0 = p->fwd_chunk;
    best = TuneChoice{T0, c0, 3.0e38f};
    int rc = cudaMemsetAsync(scratch, 0, sizeof(float) * maxpix, st) == cudaSuccess ? XCT_OK
                                                                                    : xct_fail(XCT_E_CUDA, "memset");
    for (const TuneChoice &c : xct_tune_candidates(max_rows)) {
        if (rc) break;
        if ((rc = batch_layout(p, c.T, c.chunk))) break;
        for (int j = 0; j < m; ++j) {
            tmp[j] = p->host[p->glist[j]];
            tmp[j].img = scratch;
            tmp[j].sino = nullptr;
        }
        cudaMemcpyAsync(p->d_items, tmp.data(), sizeof(XctItemDev) * m, cudaMemcpyHostToDevice, st);
        float tmin = 3.0e38f;
        for (int r = 0; r < 3 && rc == XCT_OK; ++r) {  // first run warms up
            cudaMemsetAsync(p->d_acc, 0, sizeof(double) * p->n_acc, st);
            cudaMemsetAsync(p->d_queues, 0, sizeof(int), st);
            cudaEventRecord(e0, st);
            rc = launch_fwd_batched(p->d_items, p->d_bases, m, p->sub[0], p->d_queues, p->grids[0], c.T, st);
            cudaEventRecord(e1, st);
            cudaError_t e = cudaEventSynchronize(e1);
            if (rc == XCT_OK && e != cudaSuccess) rc = xct_cuda_fail(e, "xct_batch_plan_autotune");
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0) tmin = std::min(tmin, ms);
        }
        if (rc == XCT_OK && tmin < best.ms) best = TuneChoice{c.T, c.chunk, tmin};
    }
    cudaMemsetAsync(p->d_acc, 0, sizeof(double) * p->n_acc, st);
    cudaStreamSynchronize(st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(scratch);
    if (rc) {
        batch_layout(p, T0, c0);
        return rc;
    }
    rc = batch_layout(p, best.T, best.chunk);
    if (rc) return rc;
    return xct_tune_store(p->key, cache_path, best);
}
