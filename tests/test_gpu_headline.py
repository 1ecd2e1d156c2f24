"""Parity of the measured workloads against the oracle at their own sizes.

* The per-slice workload at scale (2048x2048 image, 1500 angles over 180 deg, 2048 bins,
  15 subsets x 4 iterations; the benchmark's volume, seed 2): slice 0 through the tiled
  kernels one slice per call, and slices 0 and 9 inside a batch of ten through the
  two-stream call the benchmark times (slice 0 runs in the first half on the caller's
  stream, slice 9 in the second half on the plan's own stream), each against the oracle's
  full OS-EM in the reference's literal evaluation order (OSEM.cl:38-105 driven as
  OSEM_execution, GPU.cpp:125-240).  Bar: rel-L2 <= 1e-4 and max-abs <= 1e-3 of the peak.
* The CT-XAFS stack (widths 512-2048 with matching bins, 360-1200 angles with 0-10 % of
  them dropped, 10 subsets x 5 iterations, XANES-mixture slices): one batched plan over
  slices of all four widths against the oracle, same bar.

The oracle runs on the host cores (OpenMP): about 10 s per 2048^2 slice on 16 cores.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

N, PA, SS, IT, I0 = 2048, 1500, 15, 4, 5e4
REL, MAXABS = 1e-4, 1e-3


def _check(got, ref, what):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    assert np.all(np.isfinite(got)), what
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    mx = np.abs(got - ref).max() / np.abs(ref).max()
    assert rel <= REL and mx <= MAXABS, "%s: rel-L2 %.3e, max-abs %.3e of peak" % (what, rel, mx)
    return rel, mx


@pytest.fixture(scope="module")
def volume10(gpu_ctx):
    """Slices 0..9 of the benchmark's volume: the seeded ellipsoid phantom (30 ellipsoids,
    attenuation 0.005-0.1 /px, seed 2) projected with the library's forward projector,
    Poisson noise at I0 = 5e4 from one generator seeded 2, log-converted."""
    import xct
    from xct import phantom as P
    ang = P.uniform_angles(PA)
    plan = xct.OSEMPlan(gpu_ctx, N, N, N, ang, SS, IT, max_batch=1)
    pars = P.ellipsoid_params(N, 100, 30, 2, mu=(0.005, 0.1))
    gen = torch.Generator(device="cuda")
    gen.manual_seed(2)
    sino = torch.empty((10, PA, N), device="cuda")
    for z in range(10):
        img = P.ellipsoid_slice(pars, z, N, N, torch_device="cuda").reshape(1, N, N).contiguous()
        clean = torch.empty((1, PA, N), device="cuda")
        plan.fwd(img, clean)
        sino[z] = P.noisy_log_sinogram_torch(clean[0], I0, generator=gen)
    torch.cuda.synchronize()
    plan.close()
    return ang, sino


@pytest.fixture(scope="module")
def oracle_runs(volume10, oracle_lib):
    ang, sino = volume10
    O = oracle_lib
    out = {}
    for z in (0, 9):
        meas = sino[z].cpu().numpy()
        out[z] = O.osem_run(np.ones((N, N), np.float32), meas, ang, SS, IT, order=O.ORDER_LITERAL)
    return out


def test_headline_one_slice_per_call_matches_oracle(gpu_ctx, volume10, oracle_runs):
    import xct
    ang, sino = volume10
    plan = xct.OSEMPlan(gpu_ctx, N, N, N, ang, SS, IT, max_batch=1)
    plan.autotune(dN=1)  # the tiles the benchmark's one-slice path uses
    x = torch.ones((1, N, N), device="cuda")
    plan.run_device(sino[:1], x)
    torch.cuda.synchronize()
    _check(x[0].cpu().numpy(), oracle_runs[0], "2048^2 one slice per call")
    plan.close()


def test_headline_batch_of_ten_two_streams_matches_oracle(gpu_ctx, volume10, oracle_runs):
    import xct
    ang, sino = volume10
    plan = xct.OSEMPlan(gpu_ctx, N, N, N, ang, SS, IT, max_batch=10)
    plan.autotune(dN=10)  # as the benchmark's timed region
    x = torch.ones((10, N, N), device="cuda")
    plan.run_device(sino, x, dN=10, stream=torch.cuda.current_stream())
    torch.cuda.synchronize()
    for z in (0, 9):
        _check(x[z].cpu().numpy(), oracle_runs[z], "2048^2 batch of 10, slice %d" % z)
    plan.close()


def test_ctxafs_stack_widths_batched_matches_oracle(gpu_ctx, oracle_lib):
    """One batched plan over CT-XAFS slices of widths 512, 1024, 1536 and 2048 (bins = width),
    360-1200 angles with some dropped, XANES mixtures at one energy, 10 subsets x 5 it."""
    import xct
    from xct import phantom as P
    O = oracle_lib
    ss, it = 10, 5
    spectra = P.xanes_mixture(64, seed=3)
    rng = np.random.default_rng(5)
    specs = []
    for w, pa, drop in ((512, 360, 0.05), (1024, 720, 0.10), (1536, 900, 0.07), (2048, 1200, 0.03),
                        (512, 1200, 0.10), (1024, 360, 0.0)):
        nd = int(round(drop * pa))
        keep = np.sort(rng.choice(pa, pa - nd, replace=False))
        specs.append((w, (keep * (180.0 / pa)).astype(np.float32)))
    geoms, sinos, refs = [], [], []
    gen = torch.Generator(device="cuda")
    gen.manual_seed(3)
    for k, (w, ang) in enumerate(specs):
        p = xct.OSEMPlan(gpu_ctx, w, w, w, ang, ss, it)
        img = P.xanes_slice(w, 40, 100 + k, spectra, torch_device="cuda").reshape(1, w, w).contiguous()
        clean = torch.empty((1, len(ang), w), device="cuda")
        p.fwd(img, clean)
        s = P.noisy_log_sinogram_torch(clean[0], 1e5, generator=gen).contiguous()
        p.close()
        sinos.append(s)
        geoms.append(xct.make_geom(w, w, w, ang, ss, it))
        refs.append(O.osem_run(np.ones((w, w), np.float32), s.cpu().numpy(), ang, ss, it, order=O.ORDER_LITERAL))
    bp = xct.BatchPlan(gpu_ctx, geoms, it)
    bp.autotune()
    imgs = [torch.ones((w, w), device="cuda") for w, _ in specs]
    bp.run(sinos, imgs)
    torch.cuda.synchronize()
    for (w, ang), x, ref in zip(specs, imgs, refs):
        _check(x.cpu().numpy(), ref, "CT-XAFS item %dx%d, %d angles" % (w, w, len(ang)))
    bp.close()
