// osem_host.cpp -- the OS-EM driver of the drop-in CT_reconstruction on libxct.
//
// Same structure as the reference (CT_reconstruction/GPU.cpp): a mode switch (GPU(),
// :23-97) and, per device, a three-stage thread pipeline -- an input thread reads a batch of
// dN sinograms and initial images (OSEM_input_thread, :483-510), a reconstruction thread runs
// OS-EM on them (OSEM_thread, :408-476) and an output thread writes the slices (output_thread,
// :99-123) -- fed round-robin with batches [N, N+dN-1] by the dispatcher of OSEM_ocl
// (:562-663).  The OpenCL context/queue/program/image objects are replaced by one libxct
// context and plan per device; the reconstruction thread calls xct_osem_run, which does the
// host<->device copies and the whole subset/iteration loop on the device.  The FBP (FBP_ocl,
// GPU.cpp:997-1090) and FBP + OS-EM hybrid (hybrid_ocl, :1605-1700) drivers have the same
// pipeline shape; their reconstruction step is xct_fbp_run / xct_hybrid_run.
#include <sys/stat.h>
#include <time.h>

#include <atomic>
#include <iomanip>
#include <iostream>
#include <memory>
#include <thread>

#include "ct_reconstruction_gb300.hpp"

namespace {

struct DeviceSlot {
    int device = 0;
    int dN = 1;
    xct_ctx *ctx = nullptr;
    xct_plan *plan = nullptr;
    std::thread input_th, reconst_th, output_th;
};

enum Method { METHOD_OSEM, METHOD_FBP, METHOD_HYBRID, METHOD_FISTA };
Method g_method = METHOD_OSEM;
std::vector<int> g_sub;           // subset order (GPU.cpp:564-582)
std::atomic<int> g_status{0};     // first failure (the reference exits on the spot)
time_t g_t0 = 0;

void fail(int code)
{
    int expected = 0;
    g_status.compare_exchange_strong(expected, code);
}

void join(std::thread &t)
{
    if (t.joinable()) t.join();
}

// output_thread (GPU.cpp:99-123): write slices startN+offset..endN (imgs[0] is slice
// startN; the compressed-sensing batches overlap and skip their shared edge slices), report,
// free the images.
void output_thread(int startN, int endN, std::vector<float *> imgs, bool ok, int offset)
{
    const size_t n = (size_t)g_ox * g_oy;
    if (ok)
        for (int i = startN + offset; i <= endN; ++i)
            if (!write_data_output(g_d2, slice_name(g_f2, i), imgs[i - startN], n)) fail(XCT_E_IO);
    time_t t1;
    time(&t1);
    for (int i = startN + offset; i <= endN; ++i)
        std::cout << "[Layer " << std::setfill('0') << std::setw(4) << i << "/" << g_st - 1 + g_num << "] "
                  << (float)(t1 - g_t0) << " s elapsed" << (ok ? "" : " (failed)") << std::endl;
    for (float *p : imgs) delete[] p;
}

// OSEM_thread (GPU.cpp:408-476) / FBP_thread (:822-893) / hybrid_thread (:1458-1600):
// reconstruct the batch, hand the images to the output stage.
void osem_thread(DeviceSlot *d, std::vector<float *> imgs, std::vector<float *> prjs, int startN, int endN)
{
    const int dN = endN - startN + 1;
    int rc;
    if (g_method == METHOD_FBP) rc = xct_fbp_run(d->plan, dN, g_zp, prjs.data(), imgs.data());
    else if (g_method == METHOD_FISTA)  // FISTA_thread (GPU.cpp:1927-1979)
        rc = xct_fista_run(d->plan, dN, prjs.data(), imgs.data(), g_sub.data(), g_it, (float)g_wt1, CSlambda, 0);
    else if (g_method == METHOD_HYBRID && CSitBool)  // hybrid_thread's FISTA branch (GPU.cpp:1569-1571)
        rc = xct_hybrid_cs_run(d->plan, dN, g_zp, baseupOrder, prjs.data(), imgs.data(), g_sub.data(), g_it, CSlambda);
    else if (g_method == METHOD_HYBRID)
        rc = xct_hybrid_run(d->plan, dN, g_zp, baseupOrder, prjs.data(), imgs.data(), g_sub.data(), g_it);
    else if (CSitBool)  // FISTA_OSEM_execution (GPU.cpp:449-453)
        rc = xct_cs_osem_run(d->plan, dN, prjs.data(), imgs.data(), g_sub.data(), g_it, CSlambda);
    else rc = xct_osem_run(d->plan, dN, prjs.data(), imgs.data(), g_sub.data(), g_it);
    if (rc != XCT_OK) {
        std::cerr << "ERROR: " << xct_last_error() << " (" << rc << ")" << std::endl;
        fail(rc);
    }
    // compressed sensing: batches overlap by CSoverlap slices; inner batch edges are not
    // written (GPU.cpp:456-460)
    const bool cs = CSitBool && g_method != METHOD_FBP;
    const int offset = (cs && startN > g_st) ? CSoverlap : 0;
    const int out_end = (cs && endN < g_st + g_num - 1) ? endN - CSoverlap : endN;
    join(d->output_th);
    d->output_th = std::thread(output_thread, startN, out_end, std::move(imgs), rc == XCT_OK, offset);
    for (float *p : prjs) delete[] p;
}

// OSEM_input_thread (GPU.cpp:483-510): read the batch, then chain the reconstruction.
void osem_input_thread(DeviceSlot *d, int startN, int endN)
{
    std::vector<float *> prjs, imgs;
    bool ok = true;
    for (int i = startN; i <= endN; ++i) {
        prjs.push_back(new float[(size_t)g_px * g_pa]);
        imgs.push_back(new float[(size_t)g_ox * g_oy]);
        ok = ok && read_data_input(g_d1, slice_name(g_f1, i), prjs.back(), (size_t)g_px * g_pa);
        // FBP and the hybrid overwrite every pixel: no initial image to read
        // (FISTA_input_thread reads it too, though FISTA_execution then replaces it)
        if (g_method == METHOD_OSEM || g_method == METHOD_FISTA)
            ok = ok && first_image(g_f4, imgs.back(), (size_t)g_ox * g_oy);
    }
    join(d->reconst_th);
    if (!ok) {
        fail(XCT_E_IO);
        for (float *p : prjs) delete[] p;
        for (float *p : imgs) delete[] p;
        return;
    }
    d->reconst_th = std::thread(osem_thread, d, std::move(imgs), std::move(prjs), startN, endN);
}

}  // namespace

namespace {

// OSEM_ocl (GPU.cpp:562-663) on libxct: one context + plan per device, round-robin batches
// (FBP_ocl and hybrid_ocl dispatch the same way).
int run_pipeline(const std::vector<int> &devices, const std::vector<float> &ang, int ss, Method method)
{
    g_method = method;
    if (devices.empty()) {
        std::cerr << "ERROR: no usable CUDA device in the device list \"" << g_devList << "\"" << std::endl;
        return XCT_E_INVALID;
    }
    g_sub.assign(ss, 0);
    if (xct_subset_order(ss, g_sub.data()) != XCT_OK) {
        std::cerr << "ERROR: " << xct_last_error() << std::endl;
        return XCT_E_INVALID;
    }
    std::vector<std::unique_ptr<DeviceSlot>> slots;
    for (int dev : devices) {
        auto d = std::make_unique<DeviceSlot>();
        d->device = dev;
        d->dN = numParallel > 0 ? numParallel : 1;
        if (xct_ctx_create(dev, &d->ctx) != XCT_OK) {
            std::cerr << "ERROR: " << xct_last_error() << std::endl;
            return XCT_E_UNSUPPORTED;
        }
        xct_geom g = {};
        g.nx = g_nx;
        g.ny = g_ny;
        g.ox = g_ox;
        g.oy = g_oy;
        g.px = g_px;
        g.pa = g_pa;
        g.ss = ss;
        g.it = g_it;
        g.angles_deg = ang.data();
        g.center_bin = -1.0f;
        g.measured_fetch_mode = XCT_FETCH_EXACT;
        g.subset_mode = XCT_SUBSETS_REF;
        g.correction_mode = correctionMode;
        g.max_batch = d->dN;
        g.kernels = XCT_KERNELS_TILED;
        if (xct_osem_plan_create(d->ctx, &g, &d->plan) != XCT_OK) {
            std::cerr << "ERROR: " << xct_last_error() << std::endl;
            xct_ctx_destroy(d->ctx);
            return XCT_E_INVALID;
        }
        // FISTA_ocl estimates the subset operators' Lipschitz constants once per device before
        // dispatching (powerIteration on the input-thread slot, GPU.cpp:2246-2257)
        if (method == METHOD_FISTA && xct_fista_power_iteration(d->plan, 30, 1024, 0, nullptr, nullptr) != XCT_OK) {
            std::cerr << "ERROR: " << xct_last_error() << std::endl;
            xct_osem_plan_destroy(d->plan);
            xct_ctx_destroy(d->ctx);
            return XCT_E_CUDA;
        }
        char name[256] = {0};
        xct_device_name(dev, name, sizeof name);
        std::cout << "Device No. " << dev + 1 << ": " << name << ", " << d->dN << " slices per call" << std::endl;
        slots.push_back(std::move(d));
    }
    const int last = g_st + g_num - 1;
    // compressed sensing: consecutive batches overlap by 2*CSoverlap slices (GPU.cpp:636-647)
    // (OSEM_ocl and hybrid_ocl, GPU.cpp:636-647, 1718-1734; FBP_ocl never overlaps)
    const int cs_delta = (CSitBool && method != METHOD_FBP) ? CSoverlap : 0;
    for (auto &d : slots)
        if (d->dN - 2 * cs_delta <= 0) {
            std::cerr << "ERROR: " << d->dN << " slices per call cannot overlap by " << cs_delta
                      << " slices on each side (compressed sensing)" << std::endl;
            return XCT_E_INVALID;
        }
    for (int N = g_st; N <= last;) {
        for (auto &d : slots) {
            join(d->input_th);
            const int end = std::min(N + d->dN - 1, last);
            d->input_th = std::thread(osem_input_thread, d.get(), N, end);
            N += d->dN - 2 * cs_delta;  // as the reference: a batch may start inside the last one
            if (N > last) break;
        }
    }
    for (auto &d : slots) join(d->input_th);
    for (auto &d : slots) join(d->reconst_th);
    for (auto &d : slots) join(d->output_th);
    for (auto &d : slots) {
        xct_osem_plan_destroy(d->plan);
        xct_ctx_destroy(d->ctx);
    }
    return g_status.load();
}

}  // namespace

int OSEM_gpu(const std::vector<int> &devices, const std::vector<float> &ang, int ss)
{
    return run_pipeline(devices, ang, ss, METHOD_OSEM);
}

// GPU() (GPU.cpp:23-97): the OS-EM-family modes of the reference.
int GPU()
{
    if (g_ox != g_nx || g_oy != g_ny) {
        std::cerr << "ERROR: an output size smaller than the reconstruction size is not supported" << std::endl;
        return XCT_E_INVALID;
    }
    int ndev = 0;
    if (xct_device_count(&ndev) != XCT_OK) {
        std::cerr << "ERROR: " << xct_last_error() << std::endl;
        return XCT_E_CUDA;
    }
    const std::vector<int> devices = parse_device_list(g_devList, ndev);
    time(&g_t0);
    switch (g_mode) {
    case 1:
    case 3:
        // AART (1) and ASIRT (3): only their compressed-sensing form, FISTA_ocl (GPU.cpp:37-41,
        // 53-58), is built.  Mode 3 calls FISTA_ocl with one subset; the reference's kernels and
        // loop still use g_ss there (reading past its one-entry subset order when g_ss > 1), so
        // this build runs mode 3 with one subset throughout.
        if (!CSitBool) {
            std::cerr << "ERROR: reconstruction method " << g_mode
                      << " without compressed sensing (AART/ASIRT) is not part of this build; set CSitBool" << std::endl;
            return XCT_E_UNSUPPORTED;
        }
        std::cout << "Processing by " << (g_mode == 1 ? "AART" : "ASIRT") << " method with FISTA compressed sensing"
                  << std::endl << std::endl;
        return run_pipeline(devices, g_ang, g_mode == 1 ? g_ss : 1, METHOD_FISTA);
    case 2:
        std::cout << "Processing by MART method" << std::endl << std::endl;
        return OSEM_gpu(devices, g_ang, g_pa);  // OS-EM with ss = pa (GPU.cpp:51)
    case 4:
        std::cout << "Processing by MSIRT method" << std::endl << std::endl;
        return OSEM_gpu(devices, g_ang, 1);
    case 5:
        std::cout << "Processing by ML-EM method" << std::endl << std::endl;
        return OSEM_gpu(devices, g_ang, 1);
    case 6:
        std::cout << "Processing by OS-EM method" << std::endl << std::endl;
        return OSEM_gpu(devices, g_ang, g_ss);
    case 7:
        std::cout << "Processing by FBP method" << std::endl << std::endl;
        return run_pipeline(devices, g_ang, 1, METHOD_FBP);
    case 8:
        std::cout << "Processing by FBP+OS-EM hybrid method" << std::endl << std::endl;
        return run_pipeline(devices, g_ang, g_ss, METHOD_HYBRID);
    default:
        std::cerr << "ERROR: reconstruction method " << g_mode
                  << " is not part of this build (FISTA 1, 3 with CSitBool; OS-EM family 2, 4, 5, 6; FBP 7; hybrid 8)"
                  << std::endl;
        return XCT_E_UNSUPPORTED;
    }
}
