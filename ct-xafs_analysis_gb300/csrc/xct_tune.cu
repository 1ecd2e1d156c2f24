// xct_tune.cu -- the forward projector's tile autotuner and its cache.
//
// The tiled forward projector has two launch-shape parameters: the tile side T (44, 60, 76 or
// 92 base texels; a CTA stages one tile and serves its angles from shared memory) and the
// number of subset angles one CTA serves (the chunk, 16..128).  Large values amortise the
// staging and the per-ray interval search; small values give more CTAs, which small slices
// and small subsets need to fill 152 SMs.  Four CTAs (48 warps) fit on an SM for T <= 76 and
// three (36 warps) for T = 92, so the choice changes the occupancy, the grid's granularity and
// the per-tile overheads -- a trade-off that depends on the slice size, the angles per subset
// and the slices per call, so it is measured: xct_plan_autotune times every candidate on the plan's
// own geometry and keeps the fastest; the choice is cached per (device, shape) in memory and,
// optionally, in a JSON file that later plans (and processes) read.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "xct_internal.h"

namespace {

const int kTiles[] = {92, 76, 60, 44};
const int kChunks[] = {128, 64, 32, 16};

std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune_mem;  // this process's choices

// One entry per line inside "entries": "<key>": {"fwd_tile": T, "ang_chunk": C, "ms": t}
bool parse_line(const char *line, std::string &key, TuneChoice &c)
{
    const char *q0 = strchr(line, '"');
    if (!q0) return false;
    const char *q1 = strchr(q0 + 1, '"');
    if (!q1) return false;
    key.assign(q0 + 1, q1 - q0 - 1);
    const char *a = strstr(q1, "\"fwd_tile\":"), *b = strstr(q1, "\"ang_chunk\":"), *m = strstr(q1, "\"ms\":");
    if (!a || !b) return false;
    c.T = atoi(a + 11);
    c.chunk = atoi(b + 12);
    c.ms = m ? (float)atof(m + 5) : 0.0f;
    return xct_fwd_tile_valid(c.T) && c.chunk >= 1 && c.chunk <= fwd_tiled_rows_cap();
}

void load_file(const char *path, std::map<std::string, TuneChoice> &out)
{
    FILE *f = fopen(path, "r");
    if (!f) return;
    char line[1024];
    while (fgets(line, sizeof line, f)) {
        std::string key;
        TuneChoice c;
        if (strstr(line, "\"fwd_tile\"") && parse_line(line, key, c)) out[key] = c;
    }
    fclose(f);
}

int save_file(const char *path, const std::map<std::string, TuneChoice> &m)
{
    // a per-process temporary, so that processes saving at once never share one; the
    // rename replaces the file atomically (the last writer's entries win)
    std::string tmp = std::string(path) + ".tmp." + std::to_string((long long)getpid());
    FILE *f = fopen(tmp.c_str(), "w");
    if (!f) return xct_fail(XCT_E_IO, std::string("tune cache: cannot write ") + tmp);
    fprintf(f, "{\n  \"xct_tune_cache\": 1,\n  \"entries\": {\n");
    size_t i = 0;
    for (const auto &kv : m) {
        fprintf(f, "    \"%s\": {\"fwd_tile\": %d, \"ang_chunk\": %d, \"ms\": %.5g}%s\n", kv.first.c_str(),
                kv.second.T, kv.second.chunk, (double)kv.second.ms, ++i < m.size() ? "," : "");
    }
    fprintf(f, "  }\n}\n");
    const bool ok = fclose(f) == 0;
    if (!ok || rename(tmp.c_str(), path) != 0) return xct_fail(XCT_E_IO, std::string("tune cache: cannot replace ") + path);
    return XCT_OK;
}

}  // namespace

std::string xct_tune_key(const char *device, int nx, int ny, int px, int pa, int ss, int dN)
{
    char b[384];
    snprintf(b, sizeof b, "%s|%dx%d|%dx%d|ss%d|dN%d", device, nx, ny, px, pa, ss, dN);
    return b;
}

bool xct_tune_lookup(const std::string &key, const char *path, TuneChoice &c)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune_mem.find(key);
    if (it != g_tune_mem.end()) {
        c = it->second;
        return true;
    }
    if (path && *path) {
        std::map<std::string, TuneChoice> m;
        load_file(path, m);
        auto jt = m.find(key);
        if (jt != m.end()) {
            c = jt->second;
            g_tune_mem[key] = c;
            return true;
        }
    }
    return false;
}

int xct_tune_store(const std::string &key, const char *path, const TuneChoice &c)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_mem[key] = c;
    if (!path || !*path) return XCT_OK;
    std::map<std::string, TuneChoice> m;
    load_file(path, m);
    m[key] = c;
    return save_file(path, m);
}

// The largest tile and chunk whose grid still gives two waves of resident CTAs (3 per SM);
// ctas(T, chunk) is supplied by the caller (one shape x dN slices, or a whole batch).
TuneChoice xct_tune_default(int sm_count, const std::function<long long(int, int)> &ctas)
{
    const long long target = 2LL * 3 * sm_count;
    for (int T : kTiles)
        for (int c : kChunks)
            if (ctas(T, c) >= target) return TuneChoice{T, c, 0.0f};
    return TuneChoice{44, 16, 0.0f};
}

// Candidates worth timing: every tile side; chunks down to 16, dropping those that exceed
// the largest subset by more than a factor of two (they launch the same CTAs as a smaller one),
// plus the even splits of the largest subset, ceil(rows / m) for m <= 6 (a 100-angle subset in
// 2, 3, 4 ... equal chunks: finer steps in the grid's size, so that its last wave of resident
// CTAs can be fuller, at the cost of staging each tile once per chunk).
std::vector<TuneChoice> xct_tune_candidates(int max_rows)
{
    std::vector<int> chunks;
    for (int c : kChunks)
        if (c == 16 || c < 2 * max_rows) chunks.push_back(c);
    for (int m = 1; m <= 6; ++m) {
        const int c = (max_rows + m - 1) / m;
        if (c >= 1 && c <= fwd_tiled_rows_cap() && std::find(chunks.begin(), chunks.end(), c) == chunks.end())
            chunks.push_back(c);
    }
    std::vector<TuneChoice> v;
    for (int T : kTiles)
        for (int c : chunks) v.push_back(TuneChoice{T, c, 0.0f});
    return v;
}

const char *xct_tune_env_path()
{
    const char *p = getenv("XCT_TUNE_CACHE");
    return (p && *p) ? p : nullptr;
}

// ---------------------------------------------------------------- single-shape plans
static long long plan_ctas(const xct_plan *p, int dN, int T, int c)
{
    const int rows = (p->g.pa + p->g.ss - 1) / p->g.ss;
    return (long long)((p->g.nx + T) / T) * ((p->g.ny + T) / T) * ((rows + c - 1) / c) * dN;
}

// The slice-interleaved forward projector by default: on (all subset angles per CTA) when a
// plan's full batch holds a group of eight slices whose tiles give at least two waves of
// CTAs (one per SM); smaller problems keep the per-slice kernel, whose smaller CTAs fill
// the SMs better.
static int plan_default_ms_chunk(const xct_plan *p)
{
    const int G = fwd_ms_slices(), T = fwd_ms_tile();
    if (p->g.kernels != XCT_KERNELS_TILED || p->g.max_batch < G) return 0;
    const long long tiles = (long long)((p->g.nx + T) / T) * ((p->g.ny + T) / T);
    return tiles * (p->g.max_batch / G) >= 2LL * p->ctx->sm_count ? fwd_tiled_rows_cap() : 0;
}

void xct_plan_default_tuning(xct_plan *p)
{
    TuneChoice c;
    const std::string key = xct_tune_key(p->ctx->name, p->g.nx, p->g.ny, p->g.px, p->g.pa, p->g.ss, p->g.max_batch);
    if (!xct_tune_lookup(key, xct_tune_env_path(), c))
        c = xct_tune_default(p->ctx->sm_count, [&](int T, int ch) { return plan_ctas(p, p->g.max_batch, T, ch); });
    // the cache holds the per-slice kernel's tiles; the slice-interleaved kernels' switch
    // follows the plan's shape
    c.ms_chunk = plan_default_ms_chunk(p);
    p->kg.fwd_T = c.T;
    p->kg.fwd_chunk = c.chunk;
    p->kg.ms_chunk = c.ms_chunk;
}

extern "C" {

int xct_plan_tuning(xct_plan *p, int *fwd_tile, int *ang_chunk)
{
    if (!p || !fwd_tile || !ang_chunk) return xct_fail(XCT_E_INVALID, "xct_plan_tuning: null argument");
    *fwd_tile = p->kg.fwd_T;
    *ang_chunk = p->kg.fwd_chunk;
    return XCT_OK;
}

int xct_plan_set_tuning(xct_plan *p, int fwd_tile, int ang_chunk)
{
    if (!p) return xct_fail(XCT_E_INVALID, "xct_plan_set_tuning: plan is null");
    if (!xct_fwd_tile_valid(fwd_tile)) return xct_fail(XCT_E_INVALID, "fwd_tile must be 44, 60, 76 or 92");
    if (ang_chunk < 1 || ang_chunk > fwd_tiled_rows_cap())
        return xct_fail(XCT_E_INVALID, "ang_chunk must be in 1..128");
    p->kg.fwd_T = fwd_tile;
    p->kg.fwd_chunk = ang_chunk;
    return XCT_OK;
}

int xct_plan_multislice(xct_plan *p, int *ang_chunk)
{
    if (!p || !ang_chunk) return xct_fail(XCT_E_INVALID, "xct_plan_multislice: null argument");
    *ang_chunk = p->kg.ms_chunk;
    return XCT_OK;
}

int xct_plan_set_multislice(xct_plan *p, int ang_chunk)
{
    if (!p) return xct_fail(XCT_E_INVALID, "xct_plan_set_multislice: plan is null");
    if (ang_chunk < 0 || ang_chunk > fwd_tiled_rows_cap())
        return xct_fail(XCT_E_INVALID, "xct_plan_set_multislice: ang_chunk must be 0 (off) or in 1..128");
    if (ang_chunk > 0 && p->g.kernels != XCT_KERNELS_TILED)
        return xct_fail(XCT_E_UNSUPPORTED, "xct_plan_set_multislice: the plain kernels have no slice-interleaved form");
    p->kg.ms_chunk = ang_chunk;
    return XCT_OK;
}

int xct_plan_autotune(xct_plan *p, int dN, const char *cache_path, int flags, void *stream)
{
    XCT_RANGE("xct_plan_autotune");
    if (!p) return xct_fail(XCT_E_INVALID, "xct_plan_autotune: plan is null");
    if (p->g.kernels != XCT_KERNELS_TILED) return XCT_OK;  // the plain kernels have no tiles
    if (dN <= 0 || dN > p->g.max_batch) return xct_fail(XCT_E_INVALID, "xct_plan_autotune: dN outside [1, max_batch]");
    if (!cache_path) cache_path = xct_tune_env_path();
    const std::string key = xct_tune_key(p->ctx->name, p->g.nx, p->g.ny, p->g.px, p->g.pa, p->g.ss, dN);
    TuneChoice best;
    if (!(flags & XCT_TUNE_FORCE) && xct_tune_lookup(key, cache_path, best)) {
        p->kg.fwd_T = best.T;
        p->kg.fwd_chunk = best.chunk;
        return XCT_OK;
    }
    XCT_CUDA_TRY(cudaSetDevice(p->ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    const int rows = (p->g.pa + p->g.ss - 1) / p->g.ss;
    const int nrows = p->g.subset_mode == XCT_SUBSETS_COVER ? rows : p->g.pa / p->g.ss;
    const size_t acc_bytes = sizeof(double) * (size_t)dN * p->acc_rows * p->g.px;
    cudaEvent_t e0, e1;
    XCT_CUDA_TRY(cudaEventCreate(&e0));
    XCT_CUDA_TRY(cudaEventCreate(&e1));
    const KGeom saved = p->kg;
    best = TuneChoice{0, 0, 3.0e38f};
    int rc = XCT_OK;
    // the cost depends on the geometry only; the plan's staging image is the input
    for (const TuneChoice &c : xct_tune_candidates(rows)) {
        p->kg.fwd_T = c.T;
        p->kg.fwd_chunk = c.chunk;
        float tmin = 3.0e38f;
        for (int r = 0; r < 3 && rc == XCT_OK; ++r) {  // first run warms up
            cudaMemsetAsync(p->d_acc, 0, acc_bytes, st);
            cudaEventRecord(e0, st);
            rc = launch_fwd_tiled_main(p->kg, p->d_trig, p->d_img, p->d_acc, dN, 0, p->g.ss, nrows, st);
            cudaEventRecord(e1, st);
            cudaError_t e = cudaEventSynchronize(e1);
            if (rc == XCT_OK && e != cudaSuccess) rc = xct_cuda_fail(e, "xct_plan_autotune");
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0) tmin = std::min(tmin, ms);
        }
        if (rc) break;
        if (tmin < best.ms) best = TuneChoice{c.T, c.chunk, tmin};
    }
    cudaMemsetAsync(p->d_acc, 0, acc_bytes, st);
    cudaStreamSynchronize(st);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) {
        p->kg = saved;
        return rc;
    }
    p->kg.fwd_T = best.T;
    p->kg.fwd_chunk = best.chunk;
    return xct_tune_store(key, cache_path, best);
}

}  // extern "C"
