"""Benchmark of the OS-EM hot path (one JSON line on rank 0).

Workload: per-slice OS-EM at scale -- 100 independent slices of 2048x2048 float32,
1500 projections over 180 deg, 2048 detector bins, 15 subsets x 4 iterations, seeded 3-D
ellipsoid phantom (30 ellipsoids, attenuation 0.005-0.1 /px), I0 = 5e4 Poisson noise.
Synthetic data: the sinograms are made on the device with this library's own forward
projector (the reference projector model), then noised and log-converted.

A step is one OSEM_execution call on a batch of dN = 10 slices (the reference's
numParallel default, CT_reconstruction/main.cpp:41): 4 iterations x 15 subsets.  Each
step takes the next batch of the 100-slice volume (10 steps = the whole volume); one step's
inputs (10 sinograms + 10 images, ~290 MB) exceed the 129 MB L2, so no flush is needed.

Metric: slice-iterations per second (one slice through all 15 subsets once).
  value          -- device-resident inputs, CUDA-event time over the K timed steps
                    (max over ranks), tiled kernels, batched dN = 10;
  e2e            -- the same metric through the C ABI with host buffers, every step's
                    copies in and out inside the timed region: xct_osem_run_volume
                    (page-locked host sinograms/images, copies overlapped with the
                    reconstruction), and beside it one blocking xct_osem_run per step;
  per_slice      -- the plain one-slice-per-call path (plain kernels, dN = 1) and the tiled
                    kernels at dN = 1, each on a bounded sample of slices;
  ctxafs_batched -- the CT-XAFS stack at scale: 64 energies x 8 slices = 512 uneven items
                    (widths 512-2048, 360-1200 angles with drops) in one autotuned batch
                    plan, against one call per item (plain and tiled kernels) on a sample
                    scaled by work;
  ctxafs_grouped -- the CT-XAFS stack with whole energies: 4 energies x 64 slices = 256
                    items, the 16 slices of one width at one energy sharing a geometry, so
                    every item is in a geometry group (single-shape plans, slice-interleaved
                    kernels); against the same plan with groups off (the graph of
                    persistent launches) and one call per item;
  uniform_batch  -- 16 slices of the per-slice workload through one batch plan: its uniform
                    route (one geometry group) against its graph of persistent launches;
  parity         -- slice 0 of the timed region against the oracle's full 15 x 4 OS-EM of
                    the same sinogram (rel-L2 and max-abs of peak; the bar 1e-4 / 1e-3);
  small_256      -- the 256^2 workload (180 angles, 10 subsets x 5 it): the GPU at one and at
                    10 slices per call, beside the CPU oracle's full run of one slice;
  next_components-- throughput of FBP, the hybrid, the compressed-sensing OS-EM, reslice,
                    denoise and the rotation-centre search (HBM-bound ones against the
                    measured HBM peak), with the CPU oracle on bounded samples beside them;
  volume_stream  -- a sample of the full-volume workload (2048^2, 1800 angles, 20 subsets x 3
                    it, rotation centre +3.5 bins, I0 = 2e4) streamed from page-locked host
                    memory by xct_osem_run_volume, against blocking per-batch calls and the
                    plain per-slice path;
  roofline       -- the dominant kernel (the slice-interleaved forward projector, 8 slices
                    per launch) timed live with CUDA events inside this run; its algorithmic
                    FLOPs (12 per bilinear sample whose footprint meets the image) over its
                    measured time, against the FP32 FMA peak measured by xct_fp32_peak in the
                    same run;
  cpu_baseline   -- the CPU oracle (OpenMP, all host cores) on one whole slice (15 x 4).

--impl reference times the reference algorithm on the host cores (the CPU restatement of
the reference's OpenCL kernels; the OpenCL runtime the reference needs is not available
on the GPU host).
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "ct-xafs_analysis_gb300"))

import numpy as np  # noqa: E402

NX = NY = 2048
PX = 2048
PA = 1500
SS = 15
IT = 4
NSLICES = 100
DN = 10
I0 = 5e4
METRIC = "OS-EM slice-iters/s (2048^2, 1500 angles, 15 subsets x 4 it; rel-L2<=1e-4 vs ref)"
UNIT = "slice-iters/s"
WORKLOAD = "per-slice OS-EM at scale: 100 slices 2048x2048, 1500 angles/180deg, 2048 bins, 15 subsets x 4 it"


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None
        self._thr = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return
        self._thr = threading.Thread(target=self._read, daemon=True)
        self._thr.start()

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.samples.append(parts)

    def stop(self):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        if self._thr is not None:
            self._thr.join(timeout=2)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _int_range(a, sl, t0, lo_v, hi_v):
    """The integers t with lo_v <= a + sl * (t - t0) < hi_v, as [start, end) (arrays over a;
    sl != 0).  A falling coordinate turns the lower bound into an inclusive upper bound on t
    and the strict upper bound into a strict lower bound."""
    if sl > 0:
        return np.ceil((lo_v - a) / sl + t0), np.ceil((hi_v - a) / sl + t0)
    return np.floor((hi_v - a) / sl + t0) + 1, np.floor((lo_v - a) / sl + t0) + 1


def algorithmic_counts(angles, nx, ny, px, cx=None):
    """T_fwd: bilinear samples whose 2x2 footprint meets the image (base texel in
    [-1, nx-1] x [-1, ny-1]), per angle, from the exact chord of each ray; T_bp: (pixel,
    angle) pairs whose nearest bin lands on the detector, per angle."""
    cx = px * 0.5 if cx is None else cx
    D = max(nx, ny)
    phi = np.deg2rad(np.asarray(angles, np.float64))
    t_fwd = np.zeros(len(angles))
    t_bp = np.zeros(len(angles))
    Xc = np.arange(px) - cx
    Yc = np.arange(ny) - ny * 0.5
    for k, (c, s) in enumerate(zip(np.cos(phi), np.sin(phi))):
        # a direction cosine below 1e-12 (cos 90, sin 180 in float64) is exactly 0: the rays
        # are axis-aligned, and every term below uses the same snapped values
        c = 0.0 if abs(c) < 1e-12 else float(c)
        s = 0.0 if abs(s) < 1e-12 else float(s)
        # sample Y of ray X: x = (Y - D/2) s + ax, y = (Y - D/2) c + ay
        ax = Xc * c + nx * 0.5
        ay = -Xc * s + ny * 0.5
        lo = np.zeros(px)
        hi = np.full(px, float(D))
        for a, sl, n in ((ax, s, nx), (ay, c, ny)):
            if sl == 0.0:
                hi = np.where((a >= -1) & (a < n), hi, 0.0)
                continue
            l, h = _int_range(a, sl, D * 0.5, -1.0, float(n))
            lo = np.maximum(lo, l)
            hi = np.minimum(hi, h)
        t_fwd[k] = np.maximum(hi - lo, 0).sum()
        # bins of row Y are floor((X - nx/2) c + off), off = cx + 0.5 - Yc s: count X in
        # [0, nx) with 0 <= (X - nx/2) c + off < px
        off = cx + 0.5 - Yc * s
        if c == 0.0:
            t_bp[k] = nx * np.count_nonzero((off >= 0) & (off < px))
            continue
        l, h = _int_range(off, c, nx * 0.5, 0.0, float(px))
        t_bp[k] = np.maximum(np.minimum(h, nx) - np.maximum(l, 0), 0).sum()
    return t_fwd, t_bp


def make_volume(torch, dev, nslices, seed=2):
    """Sinograms [nslices][PA][PX] (noisy, log) and initial images [nslices][NY][NX] on dev."""
    import xct
    from xct import phantom
    ctx = xct.Context(dev.index if dev.index is not None else 0)
    plan = xct.OSEMPlan(ctx, NX, NY, PX, phantom.uniform_angles(PA), SS, IT, max_batch=1)
    pars = phantom.ellipsoid_params(NX, nslices, 30, seed, mu=(0.005, 0.1))
    sino = torch.empty((nslices, PA, PX), device=dev, dtype=torch.float32)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    for z in range(nslices):
        img = phantom.ellipsoid_slice(pars, z, NX, NY, torch_device=dev).reshape(1, NY, NX).contiguous()
        clean = torch.empty((1, PA, PX), device=dev, dtype=torch.float32)
        plan.fwd(img, clean)
        if not bool(torch.isfinite(clean).all()):
            raise RuntimeError("non-finite projection of phantom slice %d" % z)
        sino[z] = phantom.noisy_log_sinogram_torch(clean[0], I0, generator=gen)
    torch.cuda.synchronize()
    plan.close()
    return sino


def run_reference(args, rank):
    """Reference arm: the reference algorithm on the host cores (CPU restatement of its
    OpenCL kernels, OpenMP over all cores).  Each step is one subset of one slice."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from xct import phantom
    oracle.build()
    cores = os.cpu_count()
    ang = phantom.uniform_angles(PA)
    pars = phantom.ellipsoid_params(NX, NSLICES, 30, 2, mu=(0.005, 0.1))
    img = phantom.ellipsoid_slice(pars, NSLICES // 2, NX, NY)
    sub = oracle.subset_order(SS)
    # a measured sinogram for the sample slice (the reference projector, noised)
    meas = phantom.noisy_log_sinogram(oracle.projection(img, ang, PX, ss=SS, sub=int(sub[0])), I0, 3)
    x = np.ones((NY, NX), np.float32)
    ratio = np.zeros((PA, PX), np.float32)

    def step(i):
        s = int(sub[i % SS])
        r = oracle.osem1(x, meas, ang, SS, s, order=oracle.ORDER_LITERAL, ratio=ratio)
        return oracle.osem2(x, r, ang, SS, s, order=oracle.ORDER_LITERAL)

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        step(i)
    dt = time.perf_counter() - t0
    value = args.steps / SS / dt  # one subset = 1/15 of a slice-iteration
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "step": "one subset (OSEM1+OSEM2, 100 angles) of one slice",
                   "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d subsets of one 2048^2 slice (OSEM1+OSEM2 each), OpenMP" % args.steps},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_slice(meas, ang):
    """The oracle (OpenMP, all host cores) on one whole unit of the workload: the full OS-EM
    of one 2048^2 slice, 15 subsets x 4 iterations, in the reference's literal evaluation
    order.  Returns the baseline figure (slice-iters/s) and the reconstructed slice."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    ref = oracle.osem_run(np.ones((NY, NX), np.float32), meas, ang, SS, IT, order=oracle.ORDER_LITERAL)
    dt = time.perf_counter() - t0
    return ({"value": IT / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "s": dt,
             "sample": "one 2048^2 slice of the timed volume, full OS-EM (15 subsets x 4 it, 1500 angles), OpenMP"},
            np.asarray(ref, np.float64))


def next_cpu_baselines():
    """The CPU oracle (OpenMP, all host cores) on bounded samples of the next_components
    workloads, each scaled to the unit of its GPU figure: FBP of one 2048^2 slice with 300 of
    the 1500 angles (work is linear in the angle count), the compressed-sensing OS-EM of one
    slice for one iteration, reslice and denoise of 16 of the 64 rows, and the exact adjoint
    of one slice over 20 angles."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from xct import phantom
    oracle.build()
    rng = np.random.default_rng(11)
    ang = phantom.uniform_angles(PA)
    out = {"cores": os.cpu_count(), "kind": "port"}
    samp = ang[::5]  # 300 angles
    sino = rng.uniform(0.0, 1.0, (len(samp), PX)).astype(np.float32)
    t0 = time.perf_counter()
    oracle.fbp(sino, samp, NX, NY, 4096)
    out["fbp_slices_per_s"] = (len(samp) / PA) / (time.perf_counter() - t0)
    # positive random measurements: the oracle's work does not depend on the values
    meas = rng.uniform(0.05, 1.0, (1, PA, PX)).astype(np.float32)
    t0 = time.perf_counter()
    oracle.cs_osem_run(np.ones((1, NY, NX), np.float32), meas, ang, SS, 1)
    out["cs_osem_slice_iters_per_s"] = 1 / (time.perf_counter() - t0)
    H = 16
    mt = rng.uniform(0.5, 1.5, (PA, H, PX)).astype(np.float32)
    xs, ys = rng.uniform(-2, 2, PA).astype(np.float32), rng.uniform(-1, 1, PA).astype(np.float32)
    t0 = time.perf_counter()
    r = oracle.reslice(mt, xs, ys, 0.0, 1)
    out["reslice_gbs"] = 2 * mt.nbytes / (time.perf_counter() - t0) / 1e9
    t0 = time.perf_counter()
    oracle.denoise_sinogram(r, 0.1)
    out["denoise_gbs"] = 2 * r.nbytes / (time.perf_counter() - t0) / 1e9
    samp = ang[::75]  # 20 angles
    y = rng.uniform(0.0, 1.0, (len(samp), PX)).astype(np.float32)
    t_fwd, _ = algorithmic_counts(samp, NX, NY, PX)
    t0 = time.perf_counter()
    oracle.adjoint(y, samp, NX, NY)
    out["adj_gtaps_per_s"] = float(np.sum(t_fwd)) / (time.perf_counter() - t0) / 1e9
    out["samples"] = ("FBP: one 2048^2 slice, 300 of 1500 angles, zp 4096; CS OS-EM: one slice, 15 subsets x 1 "
                      "it; reslice/denoise: 1500 x 16 x 2048; adjoint: one slice, 20 angles")
    return out


def small_case_256(ctx, reps=5):
    """The 256^2 workload (180 angles over 180 degrees, 256 bins, 10 subsets x 5 iterations; 10
    seeded ellipses, Poisson I0 = 1e5): the GPU with the sinogram resident in device memory at
    one slice per call and at 10 slices per call, beside the oracle's full run of one slice
    (OpenMP, all host cores).  Slice-iters/s."""
    import torch
    import xct
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from xct import phantom
    oracle.build()
    n, pa, ss, it = 256, 180, 10, 5
    ang = phantom.uniform_angles(pa)
    img = phantom.ellipse_phantom(n)
    meas = phantom.noisy_log_sinogram(oracle.projection(img, ang, n), 1e5, 1).astype(np.float32)
    sub = oracle.subset_order(ss)
    out = {"workload": "256^2, 180 angles, 256 bins, 10 subsets x 5 iterations"}
    for dn in (1, 10):
        plan = xct.OSEMPlan(ctx, n, n, n, ang, ss, it, max_batch=dn)
        sino = torch.from_numpy(np.repeat(meas[None], dn, axis=0)).cuda()  # C-contiguous copy
        x = torch.empty((dn, n, n), device="cuda")
        for _ in range(2):
            plan.run_device(sino, x.fill_(1.0), dN=dn)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            plan.run_device(sino, x.fill_(1.0), dN=dn)
        b.record()
        torch.cuda.synchronize()
        out["gpu_dn%d" % dn] = dn * it * reps / (a.elapsed_time(b) * 1e-3)
        plan.close()
    t0 = time.perf_counter()
    oracle.osem_run(np.ones((n, n), np.float32), meas, ang, ss, it, sub_order=sub, order=oracle.ORDER_LITERAL)
    out["cpu_oracle"] = it / (time.perf_counter() - t0)
    out["cpu_cores"] = os.cpu_count()
    out["unit"] = UNIT
    return out


def ctxafs_stack_specs(n_energy, n_slices, seed=3, widths=(512, 1024, 1536, 2048), angles=(360, 720, 900, 1200),
                       max_drop=0.10):
    """Shapes of a CT-XAFS stack of n_energy x n_slices uneven items: slice s has width w_s
    (bins = w_s; every width in `widths` equally often, seeded order), energy e has its own
    projection count from `angles` over 180 deg with 0..max_drop of them dropped at random
    (one angle list for all slices of that energy, as reslicing one projection set gives).
    Returns the widths [n_slices], the angle arrays [n_energy] and, per energy, the full
    projection count and the kept indices."""
    rng = np.random.default_rng(seed)
    ws = np.resize(np.asarray(widths), n_slices)
    rng.shuffle(ws)
    angs, grids = [], []
    for _ in range(n_energy):
        pa = int(rng.choice(angles))
        drop = int(rng.integers(0, int(max_drop * pa) + 1))
        keep = np.sort(rng.choice(pa, pa - drop, replace=False))
        angs.append((keep * (180.0 / pa)).astype(np.float32))
        grids.append((pa, keep))
    return [int(w) for w in ws], angs, grids


def ctxafs_batched(ctx, n_energy=64, n_slices=8, ss=10, it=5, sample=32, compare_graph=False):
    """The CT-XAFS stack at scale: n_energy x n_slices uneven items (widths 512-2048 with
    matching bins, 360-1200 angles with 0-10 % dropped per energy), each slice a two-spectrum
    XANES mixture at its energy, Poisson I0 = 1e5; 10 subsets x 5 iterations.  One autotuned
    batch plan reconstructs all items: the slices of one width at one energy share their
    geometry, and where eight or more do they form a geometry group (a single-shape plan,
    slice-interleaved kernels); the graph of persistent launches over a device work queue
    serves the rest.  With compare_graph the same plan also runs with groups off (the graph
    serving every item).  The per-slice paths (one call per item, plain and tiled kernels)
    run on a seeded sample of `sample` items and are scaled by the work they did (sum of
    rays x angles) to the whole stack.  Device-resident inputs, CUDA-event timing."""
    import torch
    import xct
    from xct import phantom
    widths, angs, grids = ctxafs_stack_specs(n_energy, n_slices)
    e_axis, s1, s2 = phantom.xanes_mixture(n_energy, seed=3)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    t_gen = time.perf_counter()
    fields = []
    for s_i, w in enumerate(widths):
        sup, f = phantom.xanes_fields(w, 100 + s_i)
        fields.append((torch.from_numpy(sup).cuda(), torch.from_numpy(f).cuda()))
    sinos, geoms, shapes, item_grid = [], [], [], []
    for e in range(n_energy):
        ang = angs[e]
        for s_i, w in enumerate(widths):
            item_grid.append(grids[e])
            sup, f = fields[s_i]
            img = (sup * (f * float(s1[e]) + (1.0 - f) * float(s2[e])) * 0.02).float().reshape(1, w, w).contiguous()
            p = xct.OSEMPlan(ctx, w, w, w, ang, ss, it)
            clean = torch.empty((1, len(ang), w), device="cuda")
            p.fwd(img, clean)
            p.close()
            sinos.append(phantom.noisy_log_sinogram_torch(clean[0], 1e5, generator=gen).contiguous())
            geoms.append(xct.make_geom(w, w, w, ang, ss, it))
            shapes.append((w, len(ang)))
    torch.cuda.synchronize()
    n_items = len(sinos)
    work = np.array([w * w * pa for w, pa in shapes], np.float64)  # taps ~ pixels x angles
    stream = torch.cuda.current_stream()
    res = {"items": n_items, "energies": n_energy, "slices": n_slices, "subsets": ss, "iterations": it,
           "widths": sorted(set(widths)), "angles_min": min(s[1] for s in shapes),
           "angles_max": max(s[1] for s in shapes), "generate_s": time.perf_counter() - t_gen,
           "device_bytes": int(sum(w * w + w * pa for w, pa in shapes) * 4)}

    def timed(fn, reps=1):
        fn()  # warm (captures the graph / builds plans)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    t_plan = time.perf_counter()
    bp = xct.BatchPlan(ctx, geoms, it)
    res["plan_s"] = time.perf_counter() - t_plan
    t_tune = time.perf_counter()
    res["tuning"] = dict(zip(("fwd_tile", "ang_chunk"), bp.autotune()))
    res["autotune_s"] = time.perf_counter() - t_tune
    res["groups"], res["grouped_items"] = bp.groups()
    imgs = [torch.ones((w, w), device="cuda") for w, _ in shapes]

    def run_batched():
        for x in imgs:
            x.fill_(1.0)
        bp.run(sinos, imgs, stream=stream)

    l0 = xct.launch_count()
    ms = timed(run_batched, reps=1)
    res["batched"] = {"value": n_items * it / (ms * 1e-3), "items_per_s": n_items / (ms * 1e-3), "ms": ms,
                      "launches_per_run": (xct.launch_count() - l0) // 2}
    if compare_graph:
        kept = [x.clone() for x in imgs]
        bp.set_grouping(False)
        ms_g = timed(run_batched, reps=1)
        bp.set_grouping(True)
        res["graph_only"] = {"value": n_items * it / (ms_g * 1e-3), "items_per_s": n_items / (ms_g * 1e-3),
                             "ms": ms_g}
        res["grouped_over_graph"] = ms_g / ms
        num = sum(float((a.double() - b.double()).pow(2).sum()) for a, b in zip(kept, imgs))
        den = sum(float(b.double().pow(2).sum()) for b in imgs)
        res["rel_l2_grouped_vs_graph"] = (num / den) ** 0.5
        del kept
        run_batched()  # the images as the grouped run leaves them, for the comparisons below
    rng = np.random.default_rng(7)
    samp = np.sort(rng.choice(n_items, min(sample, n_items), replace=False))
    frac = work[samp].sum() / work.sum()
    res["sample_items"] = int(len(samp))
    res["sample_work_fraction"] = float(frac)
    for name, kern in (("per_slice_tiled", xct.KERNELS_TILED), ("per_slice_plain", xct.KERNELS_PLAIN)):
        plans = [xct.OSEMPlan(ctx, shapes[k][0], shapes[k][0], shapes[k][0], geoms[k]._angles, ss, it, kernels=kern)
                 for k in samp]
        if kern == xct.KERNELS_TILED:
            for p in plans:
                p.autotune(dN=1)
        ximgs = [torch.ones((1, shapes[k][0], shapes[k][0]), device="cuda") for k in samp]

        def run_single():
            for p, k, x in zip(plans, samp, ximgs):
                x.fill_(1.0)
                p.run_device(sinos[k].reshape(1, *sinos[k].shape), x, stream=stream)

        ms_s = timed(run_single)
        ms_all = ms_s / frac  # the whole stack at the sample's rate per unit of work
        res[name] = {"value": n_items * it / (ms_all * 1e-3), "items_per_s": n_items / (ms_all * 1e-3),
                     "sample_ms": ms_s}
        for p in plans:
            p.close()
        if name == "per_slice_tiled":
            got = np.concatenate([imgs[k].cpu().numpy().ravel() for k in samp]).astype(np.float64)
            ref = np.concatenate([x.cpu().numpy().ravel() for x in ximgs]).astype(np.float64)
            res["rel_l2_batched_vs_per_slice"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    bp.close()
    res["batched_over_plain"] = res["batched"]["value"] / res["per_slice_plain"]["value"]
    if compare_graph:
        res["graph_only_over_plain"] = res["graph_only"]["value"] / res["per_slice_plain"]["value"]
    res["batched_over_tiled_per_slice"] = res["batched"]["value"] / res["per_slice_tiled"]["value"]
    # the batched run against the FP32 roofline: algorithmic FLOPs of every item (12 per
    # forward tap, 5 per backprojection gather, 4 per pixel update and subset; the per-angle
    # tap and gather counts of each width and full angle grid, summed over the kept angles)
    counts = {}
    flop = 0.0
    for (w, _), (pa_full, keep) in zip(shapes, item_grid):
        key = (w, pa_full)
        if key not in counts:
            counts[key] = algorithmic_counts((np.arange(pa_full) * (180.0 / pa_full)).astype(np.float32), w, w, w)
        t_fwd, t_bp = counts[key]
        flop += it * (12.0 * t_fwd[keep].sum() + 5.0 * t_bp[keep].sum() + 4.0 * w * w * ss)
    peak = xct.fp32_peak_tflops(0)
    res["roofline"] = {"bound": "fp32", "achieved": flop / (res["batched"]["ms"] * 1e-3) / 1e12, "peak": peak,
                       "unit": "TFLOP/s", "frac": flop / (res["batched"]["ms"] * 1e-3) / 1e12 / peak,
                       "flop_per_run": flop}
    return res


def uniform_batch(ctx, sino, n=16, reps=2):
    """A uniform batch (n slices of the per-slice workload's geometry, 2048^2, 1500 angles,
    15 x 4) through one batch plan: its slices form one geometry group, which runs through a
    single-shape plan (slice-interleaved kernels; the sinograms and images each one array);
    with groups off the same plan replays its graph of persistent launches (images in
    separate allocations).  Slice-iters/s of both, CUDA-event timing, device-resident
    inputs."""
    import torch
    import xct
    from xct import phantom
    ang = phantom.uniform_angles(PA)
    geoms = [xct.make_geom(NX, NY, PX, ang, SS, IT) for _ in range(n)]
    bp = xct.BatchPlan(ctx, geoms, IT)
    bp.autotune()
    stream = torch.cuda.current_stream()
    arr = torch.ones((n, NY, NX), device="cuda")
    sep = [torch.ones((NY, NX), device="cuda") for _ in range(n)]
    sl = [sino[z] for z in range(n)]
    out = {"slices": n, "slices_per_call": bp.uniform()}
    for name, imgs in (("uniform_route", [arr[z] for z in range(n)]), ("graph", sep)):
        bp.set_grouping(name == "uniform_route")

        def run():
            for x in imgs:
                x.fill_(1.0)
            bp.run(sl, imgs, stream=stream)
        run()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            run()
        b.record(stream)
        torch.cuda.synchronize()
        out[name] = n * IT * reps / (a.elapsed_time(b) * 1e-3)
    d = (arr - torch.stack(sep)).double()
    out["rel_l2_route_vs_graph"] = float(d.norm() / torch.stack(sep).double().norm())
    out["unit"] = UNIT
    bp.close()
    return out


def volume_stream(ctx, nslices=40, dn=10):
    """Sample of the full-volume workload: nslices of 2048^2 (a slab of the 2048-slice
    ellipsoid volume), 1800 angles, 2048 bins, centre 1024 + 3.5 (the sinograms are
    projected about it and the plan reconstructs about it), I0 = 2e4, 20 subsets x 3 it.
    Host-resident page-locked sinograms and images; xct_osem_run_volume streams them in
    batches of dn with overlapped copies.  Wall-clock slice-iters/s, the same with one
    blocking xct_osem_run per batch, and the plain per-slice path on 1 slice."""
    import torch
    import xct
    from xct import phantom
    pa, ss, it, cx, i0 = 1800, 20, 3, 1024.0 + 3.5, 2e4
    ang = phantom.uniform_angles(pa)
    pars = phantom.ellipsoid_params(NX, 2048, 30, 5, mu=(0.005, 0.1))
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    plan = xct.OSEMPlan(ctx, NX, NY, PX, ang, ss, it, center_bin=cx, max_batch=dn)
    z0 = 1024 - nslices // 2  # a slab through the middle of the volume
    h_sino, h_img = [], []
    clean = torch.empty((1, pa, PX), device="cuda")
    for z in range(nslices):
        img = phantom.ellipsoid_slice(pars, z0 + z, NX, NY, torch_device="cuda").reshape(1, NY, NX).contiguous()
        plan.fwd(img, clean)
        h_sino.append(phantom.noisy_log_sinogram_torch(clean[0], i0, generator=gen).cpu().pin_memory())
        h_img.append(torch.ones((NY, NX)).pin_memory())
    torch.cuda.synchronize()
    t_tune = time.perf_counter()
    tuning = plan.autotune(dN=dn)
    tune_s = time.perf_counter() - t_tune
    res = {"slices": nslices, "of_volume_slices": 2048, "angles": pa, "subsets": ss, "iterations": it,
           "center_bin": cx, "batch": dn, "tuning": dict(zip(("fwd_tile", "ang_chunk"), tuning)),
           "autotune_s": tune_s,
           "h2d_bytes": nslices * (pa * PX + NX * NY) * 4, "d2h_bytes": nslices * NX * NY * 4}
    plan.run_volume(h_sino[:dn], h_img[:dn])  # warm
    for x in h_img:
        x.fill_(1.0)
    t0 = time.perf_counter()
    plan.run_volume(h_sino, h_img)
    dt = time.perf_counter() - t0
    res["streamed"] = {"value": nslices * it / dt, "s": dt}
    vol0 = h_img[0].clone()
    np_s = [t.numpy() for t in h_sino]
    np_i = [t.numpy() for t in h_img]
    for x in np_i:
        x.fill(1.0)
    t0 = time.perf_counter()
    for b in range(0, nslices, dn):
        plan.run(np_s[b:b + dn], np_i[b:b + dn])
    dt = time.perf_counter() - t0
    res["per_batch_blocking"] = {"value": nslices * it / dt, "s": dt}
    plan.close()
    # plain per-slice path (the reference's launch shape), one slice
    p1 = xct.OSEMPlan(ctx, NX, NY, PX, ang, ss, it, center_bin=cx, max_batch=1, kernels=xct.KERNELS_PLAIN)
    x1 = [np.ones((NY, NX), np.float32)]
    p1.run([np_s[0]], x1, it=1)  # warm
    x1[0].fill(1.0)
    t0 = time.perf_counter()
    p1.run([np_s[0]], x1)
    dt = time.perf_counter() - t0
    p1.close()
    res["per_slice_plain"] = {"value": it / dt, "s": dt}
    v = vol0.numpy().astype(np.float64)
    res["rel_l2_streamed_vs_plain"] = float(np.linalg.norm(v - x1[0]) / np.linalg.norm(x1[0]))
    res["streamed_over_plain"] = res["streamed"]["value"] / res["per_slice_plain"]["value"]
    return res


def next_components(ctx, hbm_gbs):
    """Throughput of the components either side of the OS-EM path, on the device-resident
    per-slice workload shape (2048^2, 1500 angles, 2048 bins) unless stated, CUDA-event
    timing, 3 warm-ups then 5 timed calls each:
      fbp            -- ramp filter (zp 4096) + FBP backprojection of 10 slices (FBP.cl);
      hybrid         -- FBP + base-up + 1 OS-EM iteration (15 subsets) of 10 slices;
      cs_osem        -- compressed-sensing OS-EM (ISTA3D/FISTA3D) 1 iteration, 10 slices;
      operators      -- the forward projector and its exact adjoint over all 1500 angles of
                        10 slices (xct_fwd / xct_adj);
      reslice        -- 1500 projections of 2048 x 64 rows -> 64 sinograms, with drift shifts;
      rot_center     -- rotation-centre search: 16 shifts of one slice (1 OS-EM it each).
    HBM-bound kernels report GB/s of compulsory traffic against the measured HBM peak."""
    import torch
    import xct
    from xct import phantom
    st = torch.cuda.current_stream()
    out = {}
    ang = phantom.uniform_angles(PA)
    dn = 10

    def timed(fn, reps=5):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        for _ in range(reps):
            fn()
        b.record(st)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    plan = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, 1, max_batch=dn)
    pars = phantom.ellipsoid_params(NX, 100, 30, 2, mu=(0.005, 0.1))
    sino = torch.empty((dn, PA, PX), device="cuda")
    for z in range(dn):
        img = phantom.ellipsoid_slice(pars, 45 + z, NX, NY, torch_device="cuda").reshape(1, NY, NX).contiguous()
        plan.fwd(img, sino[z:z + 1])
    x = torch.empty((dn, NY, NX), device="cuda")
    fp = torch.empty_like(sino)
    ms_f = timed(lambda: plan.fbp_filter(sino, fp, zp=4096))
    ms_b = timed(lambda: plan.fbp_backproject(fp, x))
    ms = timed(lambda: plan.fbp(sino, x, zp=4096))
    t_fwd, t_bp = algorithmic_counts(ang, NX, NY, PX)
    # FBP backprojection: every (pixel, angle) inside the circle: the bin coordinate (5), its
    # floor and fraction (2), the two-bin lerp (4) and the accumulation (1) -- 12 flop
    bp_flop = 12.0 * math.pi * (NX / 2) ** 2 * PA * dn
    out["fbp"] = {"slices_per_s": dn / (ms * 1e-3), "ms_per_10": ms, "filter_ms": ms_f, "backproject_ms": ms_b,
                  "filter_hbm_gbs": 2 * dn * PA * PX * 4 / (ms_f * 1e-3) / 1e9, "hbm_peak_gbs": hbm_gbs,
                  "backproject_tflops": bp_flop / (ms_b * 1e-3) / 1e12}
    # the same FBP through the blocking host-buffer call (pageable arrays, as the drop-in host
    # program passes them): copies in and out included, wall time
    host_s = [sino[z].cpu().numpy() for z in range(dn)]
    host_x = [np.empty((NY, NX), np.float32) for _ in range(dn)]
    plan.fbp_run(host_s, host_x, zp=4096)
    t0 = time.perf_counter()
    for _ in range(3):
        plan.fbp_run(host_s, host_x, zp=4096)
    out["fbp"]["host_slices_per_s"] = 3 * dn / (time.perf_counter() - t0)
    ms = timed(lambda: (x.fill_(0.0), plan.hybrid(sino, x, zp=4096, it=1)), reps=3)
    out["hybrid"] = {"slices_per_s": dn / (ms * 1e-3), "ms_per_10": ms, "osem_iterations": 1}
    ms = timed(lambda: (x.fill_(1.0), plan.cs_run_device(sino, x, it=1)), reps=3)
    out["cs_osem"] = {"slice_iters_per_s": dn / (ms * 1e-3), "ms_per_10": ms}
    # the operator pair: forward projection and its exact adjoint over all angles (every
    # bilinear sample whose footprint meets the image is one tap of each)
    ms_a = timed(lambda: plan.fwd(x, sino), reps=3)
    ms_t = timed(lambda: plan.adj(sino, x), reps=3)
    out["operators"] = {"slices": dn, "fwd_ms": ms_a, "adj_ms": ms_t,
                        "fwd_gtaps_per_s": float(np.sum(t_fwd)) * dn / (ms_a * 1e-3) / 1e9,
                        "adj_gtaps_per_s": float(np.sum(t_fwd)) * dn / (ms_t * 1e-3) / 1e9}
    plan.close()
    # reslice: 1500 projections of 64 rows x 2048 -> 64 sinograms [1500][2048]
    H = 64
    mt = torch.rand((PA, H, PX), device="cuda")
    dsino = torch.empty((H, PA, PX), device="cuda")
    rng = np.random.default_rng(1)
    rp = xct.ReslicePlan(ctx, PX, H, PA, rng.uniform(-2, 2, PA), rng.uniform(-1, 1, PA), 0.0, 1)
    ms = timed(lambda: rp.reslice(mt, dsino))
    gb = 2.0 * PA * H * PX * 4 / 1e9
    out["reslice"] = {"rows": H, "projections": PA, "width": PX, "ms": ms, "hbm_gbs": gb / (ms * 1e-3),
                      "hbm_peak_gbs": hbm_gbs, "frac": gb / (ms * 1e-3) / hbm_gbs if hbm_gbs else None}
    d2 = torch.empty_like(dsino)
    ms = timed(lambda: xct.denoise_sinogram(dsino, d2, 0.1))
    out["denoise"] = {"ms": ms, "hbm_gbs": gb / (ms * 1e-3), "frac": gb / (ms * 1e-3) / hbm_gbs if hbm_gbs else None}
    rp.close()
    # rotation-centre search: 9 shifts (-4..4 bins) of one noisy 2048^2 slice whose true centre
    # is px/2, 1500 angles, 15 subsets, one OS-EM iteration per shift
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    noisy = phantom.noisy_log_sinogram_torch(sino[0], I0, generator=gen).contiguous()
    rplan = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, 1, max_batch=9)
    imgs = torch.empty((9, NY, NX), device="cuda")
    rplan.rot_center_search(noisy, imgs, -4.0, 1.0)  # warm
    t0 = time.perf_counter()
    fi, best = rplan.rot_center_search(noisy, imgs, -4.0, 1.0)
    dt = time.perf_counter() - t0
    out["rot_center"] = {"shifts": 9, "s": dt, "shifts_per_s": 9 / dt, "best_shift": -4.0 + 1.0 * best,
                         "sinogram_centre_offset": 0.0,
                         "criterion": "the reference's smallest focus index (the oracle picks the same "
                                      "shift for this phantom at 256^2 and 512^2)"}
    rplan.close()
    return out


def profile_case_next():
    """Small case for profilers, the components either side of the path, each once: FBP
    (filter, backprojection, base-up) of one 2048^2 slice with 1500 angles; one
    compressed-sensing iteration of 2 slices; the rotation-centre shift and focus index of 4
    shifts; reslice and denoise of 1500 projections x 64 rows x 2048.  ~2 GB on the device."""
    import torch
    import xct
    from xct import phantom
    ang = phantom.uniform_angles(PA)
    ctx = xct.Context(0)
    plan = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, 1, max_batch=4)
    pars = phantom.ellipsoid_params(NX, NSLICES, 30, 2, mu=(0.005, 0.1))
    img = phantom.ellipsoid_slice(pars, NSLICES // 2, NX, NY, torch_device="cuda").reshape(1, NY, NX).contiguous()
    sino = torch.empty((2, PA, PX), device="cuda")
    plan.fwd(img, sino[:1])
    sino[1].copy_(sino[0])
    x = torch.empty((2, NY, NX), device="cuda")
    plan.hybrid(sino[:1], x[:1], zp=4096, it=0)
    x.fill_(1.0)
    plan.cs_run_device(sino, x, it=1)
    sh = torch.empty((4, PA, PX), device="cuda")
    plan.rot_center_shift(sino[0], sh, -1.0, 0.5)
    fi = torch.empty(4, device="cuda")
    plan.focus_index(x[:1].expand(4, NY, NX).contiguous(), fi, -1.0, 0.5, float(ang[0]), float(ang[-1]))
    mt = torch.rand((PA, 64, PX), device="cuda")
    rng = np.random.default_rng(1)  # the benchmark's drift shifts and correction
    rp = xct.ReslicePlan(ctx, PX, 64, PA, rng.uniform(-2, 2, PA), rng.uniform(-1, 1, PA), 0.0, 1)
    d = torch.empty((64, PA, PX), device="cuda")
    rp.reslice(mt, d)
    d2 = torch.empty_like(d)
    xct.denoise_sinogram(d, d2, 0.1)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "next", "ok": bool(torch.isfinite(x).all())}))


def profile_case():
    """Small case for profilers: one 2048^2 slice of the workload, its sinogram made with the
    forward projector (15 launches), then one OS-EM iteration (15 subsets: forward, finalize,
    backprojection) with the tiled kernels.  ~150 MB on the device."""
    import torch
    import xct
    from xct import phantom
    ang = phantom.uniform_angles(PA)
    ctx = xct.Context(0)
    plan = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, 1, max_batch=1)
    pars = phantom.ellipsoid_params(NX, NSLICES, 30, 2, mu=(0.005, 0.1))
    img = phantom.ellipsoid_slice(pars, NSLICES // 2, NX, NY, torch_device="cuda").reshape(1, NY, NX).contiguous()
    sino = torch.empty((1, PA, PX), device="cuda")
    plan.fwd(img, sino)
    x = torch.ones((1, NY, NX), device="cuda")
    plan.run_device(sino, x, it=1)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "ok", "mean": float(x.mean())}))


def profile_case_operators(n=8):
    """Small case for profilers, the operator pair and FBP: the forward projection, the exact
    adjoint and the FBP of n slices of the workload over all 1500 angles, each once (the
    slice-interleaved forward projector, the gather adjoint and the eight-slice FBP
    backprojector for n = 8; for n = 10 the adjoint is one ten-slice gather).  ~0.5 GB on
    the device."""
    if not 1 <= n <= 16:
        raise SystemExit("--profile-slices must be within 1..16")
    import torch
    import xct
    from xct import phantom
    ang = phantom.uniform_angles(PA)
    ctx = xct.Context(0)
    plan = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, 1, max_batch=n)
    pars = phantom.ellipsoid_params(NX, NSLICES, 30, 2, mu=(0.005, 0.1))
    img = torch.stack([phantom.ellipsoid_slice(pars, z, NX, NY, torch_device="cuda") for z in range(n)]).contiguous()
    sino = torch.empty((n, PA, PX), device="cuda")
    plan.fwd(img, sino)
    back = torch.empty_like(img)
    plan.adj(sino, back)
    rec = torch.empty_like(img)
    plan.fbp(sino, rec, zp=4096)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "operators", "n": n, "multislice": plan.multislice(),
                      "mean": float(back.mean())}))


def profile_case_ctxafs(n_energy=16, n_slices=8):
    """Small case for profilers, the batched CT-XAFS path: a stack of n_energy x n_slices
    uneven items shaped as the benchmark's (widths 512-2048, 360-1200 angles with drops),
    one batch plan, one iteration of 10 subsets (30 persistent launches).  ~1.5 GB."""
    import torch
    import xct
    from xct import phantom
    widths, angs, _ = ctxafs_stack_specs(n_energy, n_slices)
    ctx = xct.Context(0)
    rng = np.random.default_rng(5)
    geoms, sinos, imgs = [], [], []
    for e in range(n_energy):
        for w in widths:
            geoms.append(xct.make_geom(w, w, w, angs[e], 10, 1))
            sinos.append(torch.from_numpy(rng.uniform(0.5, 1.5, (len(angs[e]), w)).astype(np.float32)).cuda())
            imgs.append(torch.ones((w, w), device="cuda"))
    bp = xct.BatchPlan(ctx, geoms, 1)
    bp.run(sinos, imgs)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "ctxafs", "items": len(geoms), "tuning": bp.tuning()}))
    bp.close()


def profile_case_slices(n=8):
    """Small case for profilers, the slice-interleaved forward projector: n slices of the
    workload (sinograms made with the per-slice forward projector, one launch per 128 angles),
    then one OS-EM iteration (15 subsets) of the n slices in one call.  ~0.3 GB on the device."""
    import torch
    import xct
    from xct import phantom
    ang = phantom.uniform_angles(PA)
    ctx = xct.Context(0)
    plan = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, 1, max_batch=n)
    pars = phantom.ellipsoid_params(NX, NSLICES, 30, 2, mu=(0.005, 0.1))
    img = torch.stack([phantom.ellipsoid_slice(pars, z, NX, NY, torch_device="cuda") for z in range(n)]).contiguous()
    sino = torch.empty((n, PA, PX), device="cuda")
    ms = plan.multislice()
    plan.set_multislice(0)
    plan.fwd(img, sino)
    plan.set_multislice(ms if ms > 0 else 128)
    x = torch.ones((n, NY, NX), device="cuda")
    plan.run_device(sino, x, it=1)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": "slices", "n": n, "multislice": plan.multislice(), "mean": float(x.mean())}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-slices", type=int, default=8,
                    help="slices of the 'operators' profiling case (8: the eight-slice kernels; 10: the "
                         "benchmark's batch, the ten-slice gather adjoint)")
    ap.add_argument("--profile-case", nargs="?", const="osem", choices=["osem", "slices", "next", "operators", "ctxafs"],
                    help="run a small profiling case and exit: osem (one slice, one OS-EM iteration), slices "
                         "(eight slices, one OS-EM iteration, slice-interleaved kernels), next (the components "
                         "either side of the path, each once), operators (forward projection, exact adjoint and FBP "
                         "of eight slices) or ctxafs (one iteration of a 128-item CT-XAFS batch plan)")
    args = ap.parse_args()
    if args.profile_case == "osem":
        profile_case()
        return
    if args.profile_case == "slices":
        profile_case_slices()
        return
    if args.profile_case == "next":
        profile_case_next()
        return
    if args.profile_case == "operators":
        profile_case_operators(args.profile_slices)
        return
    if args.profile_case == "ctxafs":
        profile_case_ctxafs()
        return

    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    import xct
    from xct import phantom

    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    args.warmup = max(args.warmup, 3)

    # each rank reconstructs its own slices (weak scaling: NSLICES per rank)
    sino = make_volume(torch, dev, NSLICES, seed=2 + rank)
    imgs = torch.ones((NSLICES, NY, NX), device=dev, dtype=torch.float32)
    ang = phantom.uniform_angles(PA)
    ctx = xct.Context(local)
    plan = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, IT, max_batch=DN, kernels=xct.KERNELS_TILED)
    tuning = plan.autotune(dN=DN)  # before the timed region; cached per shape
    stream = torch.cuda.current_stream(dev)
    nb = NSLICES // DN

    def step(i):
        b = i % nb
        x = imgs[b * DN:(b + 1) * DN]
        x.fill_(1.0)  # uniform initial image (first_image, fileIO.cpp:55-68)
        plan.run_device(sino[b * DN:(b + 1) * DN], x, dN=DN, stream=stream)

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = ClockSampler(local)
    clk.start()
    l0 = xct.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for i in range(args.steps):
        step(i)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = xct.launch_count() - l0
    clk.stop()
    ms = e0.elapsed_time(e1)
    if world > 1:
        from xct import shard
        ms = shard.max_over_ranks(ms, device=dev)
    slice_iters = args.steps * DN * IT * world
    value = slice_iters / (ms * 1e-3)

    # slice 0 as the timed region left it (the first half of batch 0, on the caller's
    # stream), checked against the oracle's full run of that slice below
    timed_slice0 = imgs[0].cpu().numpy()
    finite = bool(torch.isfinite(imgs[:DN]).all())

    # ---- end to end through the C ABI with page-locked host buffers ----
    # xct_osem_run_volume over e2e_steps batches of DN slices: every step's sinograms and
    # initial images go host -> device and its images device -> host inside the timed region,
    # overlapped with the previous/next step's compute; also one blocking xct_osem_run per step
    nprj, nimg = PA * PX, NY * NX
    e2e_steps = max(2, min(args.steps, 4))
    nh = e2e_steps * DN
    h_sino = [torch.empty((PA, PX), dtype=torch.float32).pin_memory() for _ in range(nh)]
    h_img = [torch.empty((NY, NX), dtype=torch.float32).pin_memory() for _ in range(nh)]
    for j in range(nh):
        h_sino[j].copy_(sino[j % NSLICES])
        h_img[j].fill_(1.0)
    plan.run_volume(h_sino[:DN], h_img[:DN])  # warm (allocates the second staging set)
    for j in range(nh):
        h_img[j].fill_(1.0)
    t0 = time.perf_counter()
    plan.run_volume(h_sino, h_img)
    e2e_s = time.perf_counter() - t0
    h_sino_np = [t.numpy() for t in h_sino[:DN]]
    h_img_np = [t.numpy() for t in h_img[:DN]]
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        for j in range(DN):
            h_img_np[j].fill(1.0)
        plan.run(h_sino_np, h_img_np)
    blk_s = time.perf_counter() - t0
    e2e = {"value": e2e_steps * DN * IT / e2e_s * world, "unit": UNIT,
           "h2d_bytes_per_step": DN * (nprj + nimg) * 4, "d2h_bytes_per_step": DN * nimg * 4,
           "steps": e2e_steps, "api": "xct_osem_run_volume (page-locked host buffers, copies overlapped)",
           "blocking_per_step": {"value": e2e_steps * DN * IT / blk_s * world,
                                 "api": "xct_osem_run (host buffers, one blocking call per step)"}}

    # ---- per-slice paths (bounded samples) ----
    per_slice = {}
    for name, kern, nsl in (("plain", xct.KERNELS_PLAIN, 2), ("tiled", xct.KERNELS_TILED, 4)):
        p1 = xct.OSEMPlan(ctx, NX, NY, PX, ang, SS, IT, max_batch=1, kernels=kern)
        if kern == xct.KERNELS_TILED:
            p1.autotune(dN=1)
        x = imgs[:1].clone()
        p1.run_device(sino[:1], x, dN=1, it=1, stream=stream)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for z in range(nsl):
            x.fill_(1.0)
            p1.run_device(sino[z:z + 1], x, dN=1, stream=stream)
        b.record(stream)
        torch.cuda.synchronize()
        per_slice[name] = {"value": nsl * IT / (a.elapsed_time(b) * 1e-3), "unit": UNIT, "slices": nsl}
        p1.close()

    # ---- CT-XAFS stack sample: uneven slices in one batched graph vs one call per slice ----
    try:
        batched = ctxafs_batched(ctx)
    except Exception as e:  # reported, never fatal
        batched = {"error": str(e)[:300]}

    # ---- CT-XAFS stack with whole energies: the slices of one width share a geometry ----
    try:
        grouped = ctxafs_batched(ctx, n_energy=4, n_slices=64, sample=16, compare_graph=True)
    except Exception as e:  # reported, never fatal
        grouped = {"error": str(e)[:300]}

    # ---- a uniform batch through the batch plan: one geometry group against its graph ----
    try:
        uniform = uniform_batch(ctx, sino)
    except Exception as e:  # reported, never fatal
        uniform = {"error": str(e)[:300]}

    # ---- the 256^2 workload: GPU per call and batched, beside the CPU oracle ----
    try:
        small = small_case_256(ctx)
    except Exception as e:  # reported, never fatal
        small = {"error": str(e)[:300]}

    # ---- full-volume workload sample, streamed from host memory ----
    try:
        volume = volume_stream(ctx)
    except Exception as e:  # reported, never fatal
        volume = {"error": str(e)[:300]}

    # ---- the components either side of the path ----
    try:
        hbm_peak = None
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            hbm_peak = json.load(f).get("hbm_gbs")
    except Exception:
        pass
    try:
        nxt = next_components(ctx, hbm_peak)
    except Exception as e:  # reported, never fatal
        nxt = {"error": str(e)[:300]}

    # ---- roofline of the dominant kernel (live CUDA events, same stream) ----
    # The timed batch of 10 runs as halves of 8 | 2 slices; the 8-slice half's forward
    # projection is one launch of the slice-interleaved kernel per subset (fwd_ms_kernel),
    # 82 % of the forward time of a step.  It is timed here on 8 slices: every launch of a
    # 4 x 15 profile run bracketed by CUDA events on the launch stream.
    G = xct.MULTISLICE_SLICES
    prof = plan.profile(sino[:G], imgs[:G].fill_(1.0), dN=G, stream=stream)
    t_fwd, t_bp = algorithmic_counts(ang, NX, NY, PX)
    taps_per_launch = t_fwd.sum() / SS * G  # one subset's angles, G slices
    fwd_flop_per_launch = 12.0 * taps_per_launch
    fwd_ms_avg = prof["fwd"]["ms"] / prof["fwd"]["launches"]
    bp_flop_per_launch = 5.0 * t_bp.sum() / SS * G + 4.0 * NX * NY * G
    bp_ms_avg = prof["bp"]["ms"] / prof["bp"]["launches"]
    fp32_peak = xct.fp32_peak_tflops(local)
    achieved = fwd_flop_per_launch / (fwd_ms_avg * 1e-3) / 1e12
    # HBM view of the same kernel: it reads each image once per subset and adds one double
    # per (ray, tile) -- compulsory bytes are tiny next to its arithmetic
    fwd_bytes = G * NX * NY * 4.0
    # the kernel's own bound: the L1/shared-memory data path, one 16-byte record per tap and
    # slice (the four bilinear coefficients of the footprint) against 128 B/clk/SM
    props = torch.cuda.get_device_properties(dev)
    sm_mhz = clk.summary().get("sm_mhz") or 2070.0
    l1_peak = 128.0 * props.multi_processor_count * sm_mhz * 1e6
    roofline = {
        "bound": "fp32", "kernel": "fwd_ms_kernel (OSEM1 forward projection, 8 slices per launch)",
        "l1_shared": {"achieved_tbs": taps_per_launch * 16.0 / (fwd_ms_avg * 1e-3) / 1e12,
                      "peak_tbs": l1_peak / 1e12,
                      "frac": taps_per_launch * 16.0 / (fwd_ms_avg * 1e-3) / l1_peak,
                      "note": "16 B (one float4 record) per tap and slice over 128 B/clk/SM at the sampled SM "
                              "clock"},
        "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
        "peak_source": "measured live by xct_fp32_peak (FMA-chain kernel) in this run",
        "flop_per_launch": fwd_flop_per_launch, "taps_per_launch": taps_per_launch, "ms_per_launch": fwd_ms_avg,
        "slices_per_launch": G, "traffic": None,
        "hbm": {"achieved_gbs": fwd_bytes / (fwd_ms_avg * 1e-3) / 1e9, "peak_gbs": None,
                "note": "compulsory image bytes per launch over its time"},
        "bp": {"kernel": "bp_ms_kernel (OSEM2 backprojection+update, 8 slices per launch)", "ms_per_launch": bp_ms_avg,
               "achieved_tflops": bp_flop_per_launch / (bp_ms_avg * 1e-3) / 1e12,
               "frac": bp_flop_per_launch / (bp_ms_avg * 1e-3) / 1e12 / fp32_peak,
               "gathers_per_launch": t_bp.sum() / SS * G},
        "share": {k: prof[k]["ms"] / prof["total"]["ms"] for k in ("fwd", "finalize", "bp")},
    }
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            roofline["hbm"]["peak_gbs"] = json.load(f).get("hbm_gbs")
    except Exception:
        pass
    # DRAM traffic of the forward kernel per launch from the committed ncu capture of the same
    # launch shape (8 slices of 2048^2, one subset of 100 angles)
    prof_md = os.path.join(REPO, "profiles", "fwd_ms_kernel_2048x2048_1500ang_8slices.md")
    try:
        with open(prof_md) as f:
            for line in f:
                if line.startswith("dram_bytes_per_launch:"):
                    roofline["traffic"] = float(line.split(":")[1])
                    roofline["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch, "
                                                  "profiles/fwd_ms_kernel_2048x2048_1500ang_8slices.md")
    except Exception:
        pass

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        # the CPU baseline is the oracle's full OS-EM of slice 0 (15 subsets x 4 iterations, the
        # reference's literal evaluation order); its result is the parity reference of the
        # timed region's slice 0
        try:
            cpu, ref0 = cpu_baseline_slice(sino[0].cpu().numpy(), ang)
            d = timed_slice0.astype(np.float64) - ref0
            parity = {"slice": 0, "rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref0)),
                      "max_abs_of_peak": float(np.abs(d).max() / np.abs(ref0).max()),
                      "bar": {"rel_l2": 1e-4, "max_abs_of_peak": 1e-3},
                      "reference": "oracle OS-EM of the same sinogram, 15 x 4, reference order (OSEM.cl:38-105)"}
            parity["pass"] = parity["rel_l2"] <= 1e-4 and parity["max_abs_of_peak"] <= 1e-3
        except Exception as e:  # reported, never fatal
            cpu = {"value": None, "error": str(e)[:200]}
        if isinstance(nxt, dict) and "error" not in nxt:
            try:
                nxt["cpu_oracle"] = next_cpu_baselines()
            except Exception as e:  # reported, never fatal
                nxt["cpu_oracle"] = {"error": str(e)[:200]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded ellipsoid phantom, Poisson I0=5e4)",
            "config": {"workload": WORKLOAD, "batch_slices_per_call": DN, "kernels": "tiled",
                       "fwd_tiles": dict(zip(("fwd_tile", "ang_chunk"), tuning)),
                       "l2": "inputs larger than L2 (each step a new 290 MB batch)",
                       "parallelism": "dp%d over slices" % world},
            "clocks": clk.summary(), "e2e": e2e, "gpu_launches": launches, "per_slice": per_slice,
            "ctxafs_batched": batched, "ctxafs_grouped": grouped, "uniform_batch": uniform, "small_256": small, "volume_stream": volume, "next_components": nxt,
            "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "finite": finite,
            "launches_per_step": launches / max(args.steps, 1),
            # library launches before the timed region: the skip count that makes an ncu launch
            # list (-s) start at the first timed step
            "launches_before_timed": l0,
        }
        print(json.dumps(line), flush=True)
    plan.close()
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
